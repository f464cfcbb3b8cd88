// Host-side mesh layer of the GB300 DG path: element blocks, adjacency reconstruction and periodic
// pairing.  Replaces the reference's gmsh-driven Mesh<SC> setup:
//   element blocks   src/Mesh/Element.cpp:31-70 (elements in file order per type)
//   adjacency        src/Mesh/Adjacency.cpp:37-183, 330-495 (face map keyed by the face's vertex set;
//                    first visitor = left parent, second = right parent; 3D right rotation = position
//                    of the left face's first vertex in the right face's vertex list)
//   periodic pairing src/Mesh/Adjacency.cpp:185-328 (here: a master-node map folds periodic slaves
//                    onto their masters before the face keys are formed)
//   boundary faces   src/Mesh/Adjacency.cpp:370-430 (matched to boundary elements by vertex set; in 3D a
//                    boundary element is a quadrangle, or a triangle whose fourth index is -1)
//   1D periodic      src/Mesh/Adjacency.cpp:185-211 (without a node map the two periodic boundary points
//                    are joined: the first one in boundary-element order is the left side)
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/sdg_gpu.h"

namespace sdg {

inline int typeDim(int t) {
  return t == SDG_ELEMENT_LINE ? 1 : (t == SDG_ELEMENT_HEXAHEDRON || t == SDG_ELEMENT_TETRAHEDRON ? 3 : 2);
}
inline int typeFaces(int t) {
  return t == SDG_ELEMENT_LINE ? 2
         : (t == SDG_ELEMENT_TRIANGLE ? 3 : (t == SDG_ELEMENT_QUADRANGLE || t == SDG_ELEMENT_TETRAHEDRON ? 4 : 6));
}
inline int typeVertices(int t) {
  return t == SDG_ELEMENT_LINE ? 2
         : (t == SDG_ELEMENT_TRIANGLE ? 3 : (t == SDG_ELEMENT_QUADRANGLE || t == SDG_ELEMENT_TETRAHEDRON ? 4 : 8));
}
inline int typeFaceVertices(int t) {
  return t == SDG_ELEMENT_LINE ? 1 : (t == SDG_ELEMENT_HEXAHEDRON ? 4 : (t == SDG_ELEMENT_TETRAHEDRON ? 3 : 2));
}

// Face vertex lists in gmsh order (src/Solver/SimulationControl.cpp:170-216).
const int* faceVertexList(int t);

struct FaceSide {
  int block = -1;        // element block index
  int element = -1;      // element index within the block
  int face = -1;         // local face
};

struct InteriorFace {
  FaceSide left, right;
  int rotation = 0;      // 3D only: position of the left face's first vertex in the right face's list
};

struct BoundaryFace {
  FaceSide left;
  int physical = 0;      // 1-based physical group
  int condition = 0;     // sdg_boundary_condition
};

struct Block {
  int type = 0;
  int64_t count = 0;
  const int32_t* vertex = nullptr;    // [count][typeVertices]
  const int32_t* geometry = nullptr;  // curved meshes: [count][gmsh node count of order geometryOrder]
  int geometryOrder = 1;
};

struct Adjacency {
  std::vector<InteriorFace> interior;
  std::vector<BoundaryFace> boundary;
};

// Builds interior/boundary faces; throws std::runtime_error on inconsistent meshes.
Adjacency buildAdjacency(const sdg_mesh& mesh, const std::vector<Block>& blocks);

}  // namespace sdg
