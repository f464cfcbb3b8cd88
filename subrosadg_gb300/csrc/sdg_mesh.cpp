// Mesh layer: adjacency reconstruction, structured generators and an MSH 4.1 reader.
// See sdg_mesh.hpp for the reference functions each part replaces.
#include "sdg_geometry.hpp"
#include "sdg_mesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <random>
#include <sstream>
#include <stdexcept>
#include <unordered_map>

namespace sdg {

const int* faceVertexList(int t) {
  static const int line[] = {0, 1};
  static const int tri[] = {0, 1, 1, 2, 2, 0};
  static const int quad[] = {0, 1, 1, 2, 2, 3, 3, 0};
  static const int hex[] = {0, 3, 2, 1, 0, 1, 5, 4, 0, 4, 7, 3, 1, 2, 6, 5, 2, 3, 7, 6, 4, 5, 6, 7};
  static const int tet[] = {0, 2, 1, 0, 1, 3, 0, 3, 2, 3, 1, 2};
  if (t == SDG_ELEMENT_TETRAHEDRON) return tet;
  return t == SDG_ELEMENT_LINE ? line : (t == SDG_ELEMENT_TRIANGLE ? tri : (t == SDG_ELEMENT_QUADRANGLE ? quad : hex));
}

namespace {

struct FaceKey {
  std::array<int32_t, 4> v{{-1, -1, -1, -1}};
  bool operator==(const FaceKey& o) const { return v == o.v; }
};
struct FaceKeyHash {
  size_t operator()(const FaceKey& k) const {
    uint64_t h = 1469598103934665603ull;
    for (int32_t x : k.v) { h ^= uint64_t(uint32_t(x)); h *= 1099511628211ull; }
    return size_t(h);
  }
};
struct Visit {
  FaceSide side;
  std::array<int32_t, 4> mapped{{-1, -1, -1, -1}};
  int count = 0;
  FaceSide second;
  int rotation = 0;
};

}  // namespace

Adjacency buildAdjacency(const sdg_mesh& mesh, const std::vector<Block>& blocks) {
  const auto master = [&](int32_t v) { return mesh.periodic_master ? mesh.periodic_master[v] : v; };
  std::unordered_map<FaceKey, Visit, FaceKeyHash> faces;
  size_t expected = 0;
  for (const Block& b : blocks) expected += size_t(b.count) * typeFaces(b.type);
  faces.reserve(expected / 2 + 16);
  std::vector<FaceKey> order;  // first-visit order, for a deterministic face enumeration
  order.reserve(expected / 2 + 16);
  for (int bi = 0; bi < int(blocks.size()); ++bi) {
    const Block& b = blocks[bi];
    const int nf = typeFaces(b.type), nfv = typeFaceVertices(b.type), nv = typeVertices(b.type);
    const int* fl = faceVertexList(b.type);
    for (int64_t e = 0; e < b.count; ++e) {
      for (int f = 0; f < nf; ++f) {
        std::array<int32_t, 4> mapped{{-1, -1, -1, -1}};
        for (int k = 0; k < nfv; ++k) {
          const int32_t v = b.vertex[e * nv + fl[f * nfv + k]];
          if (v < 0 || v >= mesh.node_count) throw std::runtime_error("element vertex index out of range");
          mapped[k] = master(v);
        }
        FaceKey key; key.v = mapped;
        std::sort(key.v.begin(), key.v.begin() + nfv);
        auto it = faces.find(key);
        if (it == faces.end()) {
          Visit vis; vis.side = {bi, int(e), f}; vis.mapped = mapped; vis.count = 1;
          faces.emplace(key, vis);
          order.push_back(key);
        } else {
          Visit& vis = it->second;
          if (vis.count >= 2) throw std::runtime_error("a face is shared by more than two elements (a periodic direction needs at least three elements)");
          vis.second = {bi, int(e), f};
          vis.count = 2;
          if (nfv >= 3) {
            int r = -1;
            for (int k = 0; k < nfv; ++k) if (mapped[k] == vis.mapped[0]) r = k;
            if (r < 0) throw std::runtime_error("inconsistent shared face");
            vis.rotation = r;
          }
        }
      }
    }
  }
  // Boundary elements keyed the same way.
  std::unordered_map<FaceKey, int64_t, FaceKeyHash> bmap;
  const int nbv = mesh.dimension == 1 ? 1 : (mesh.dimension == 2 ? 2 : 4);
  bmap.reserve(size_t(mesh.boundary_count) + 16);
  for (int64_t i = 0; i < mesh.boundary_count; ++i) {
    FaceKey key;
    // 3D: a triangle's fourth index is -1
    const int nk = (nbv == 4 && mesh.boundary_node[i * nbv + 3] == -1) ? 3 : nbv;
    for (int k = 0; k < nk; ++k) {
      const int32_t v = mesh.boundary_node[i * nbv + k];
      if (v < 0 || v >= mesh.node_count) throw std::runtime_error("boundary vertex index out of range");
      key.v[k] = master(v);
    }
    std::sort(key.v.begin(), key.v.begin() + nk);
    bmap[key] = i;
  }
  Adjacency adj;
  adj.interior.reserve(order.size());
  std::vector<std::pair<int64_t, FaceSide>> periodicPoints;  // 1D periodic ends without a node map
  for (const FaceKey& key : order) {
    const Visit& vis = faces.at(key);
    if (vis.count == 2) {
      InteriorFace f; f.left = vis.side; f.right = vis.second; f.rotation = vis.rotation;
      adj.interior.push_back(f);
    } else {
      const auto it = bmap.find(key);
      if (it == bmap.end()) throw std::runtime_error("boundary face has no boundary element (check physical groups)");
      BoundaryFace f; f.left = vis.side;
      f.physical = mesh.boundary_physical ? mesh.boundary_physical[it->second] : 0;
      if (f.physical < 1 || f.physical > mesh.physical_count) throw std::runtime_error("boundary physical index out of range");
      f.condition = mesh.physical_boundary_condition[f.physical - 1];
      if (f.condition == SDG_BC_PERIODIC && mesh.dimension == 1 && !mesh.periodic_master) {
        periodicPoints.push_back({it->second, vis.side});
        continue;
      }
      if (f.condition == SDG_BC_PERIODIC) throw std::runtime_error("periodic boundary face without a periodic partner");
      if (f.condition < 0 || f.condition > SDG_BC_PERIODIC) throw std::runtime_error("unknown boundary condition");
      adj.boundary.push_back(f);
    }
  }
  if (!periodicPoints.empty()) {
    // the reference joins the first two point elements: the first one's parent is the left side
    if (periodicPoints.size() != 2) throw std::runtime_error("a 1D periodic mesh needs exactly two periodic end points");
    std::sort(periodicPoints.begin(), periodicPoints.end(),
              [](const auto& a, const auto& b) { return a.first < b.first; });
    InteriorFace f; f.left = periodicPoints[0].second; f.right = periodicPoints[1].second;
    adj.interior.push_back(f);
  }
  return adj;
}

}  // namespace sdg

// ---- generators and reader (C ABI) -----------------------------------------------------------------

namespace {

struct MeshStorage {
  std::vector<double> node;
  std::vector<int32_t> periodic, line, tri, quad, hex, tet, bnode, bphys, bc;
  int geometryOrder = 1;
  std::vector<int32_t> triGeo, quadGeo, hexGeo;  // curved meshes: gmsh-ordered geometry nodes per element
};

void publish(MeshStorage* s, int dim, sdg_generated_mesh* out) {
  sdg_mesh& m = out->mesh;
  std::memset(&m, 0, sizeof(m));
  m.dimension = dim;
  m.node_count = int64_t(s->node.size() / 3);
  m.node_coordinate = s->node.data();
  m.periodic_master = s->periodic.empty() ? nullptr : s->periodic.data();
  m.triangle_count = int64_t(s->tri.size() / 3); m.triangle_node = s->tri.empty() ? nullptr : s->tri.data();
  m.quadrangle_count = int64_t(s->quad.size() / 4); m.quadrangle_node = s->quad.empty() ? nullptr : s->quad.data();
  m.hexahedron_count = int64_t(s->hex.size() / 8); m.hexahedron_node = s->hex.empty() ? nullptr : s->hex.data();
  m.line_count = int64_t(s->line.size() / 2); m.line_node = s->line.empty() ? nullptr : s->line.data();
  m.tetrahedron_count = int64_t(s->tet.size() / 4); m.tetrahedron_node = s->tet.empty() ? nullptr : s->tet.data();
  m.boundary_count = int64_t(s->bphys.size()); m.boundary_node = s->bnode.empty() ? nullptr : s->bnode.data();
  m.boundary_physical = s->bphys.empty() ? nullptr : s->bphys.data();
  m.physical_count = int32_t(s->bc.size()); m.physical_boundary_condition = s->bc.data();
  if (s->geometryOrder > 1) {
    m.geometry_order = s->geometryOrder;
    m.triangle_geometry_node = s->triGeo.empty() ? nullptr : s->triGeo.data();
    m.quadrangle_geometry_node = s->quadGeo.empty() ? nullptr : s->quadGeo.data();
    m.hexahedron_geometry_node = s->hexGeo.empty() ? nullptr : s->hexGeo.data();
  }
  out->storage = s;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

int sdg_mesh_generate_2d(double x0, double y0, double lx, double ly, int32_t nx, int32_t ny, double jitter,
                         double split_fraction, uint64_t seed, int32_t periodic, const int32_t* boundary_condition,
                         sdg_generated_mesh* out) {
  if (!out || nx < 1 || ny < 1 || !(lx > 0) || !(ly > 0) || jitter < 0 || jitter >= 0.5 || split_fraction < 0 ||
      split_fraction > 1 || (!periodic && !boundary_condition))
    return SDG_ERR_INVALID_ARGUMENT;
  auto* s = new MeshStorage();
  const int px = nx + 1, py = ny + 1;
  const double hx = lx / nx, hy = ly / ny;
  std::mt19937_64 rng(seed);
  // Portable uniform draws from the raw 64-bit engine output (no implementation-defined distributions).
  const auto unit = [](std::mt19937_64& g) { return double(g() >> 11) * (1.0 / 9007199254740992.0); };
  const auto uni = [&](std::mt19937_64& g) { return 2.0 * unit(g) - 1.0; };
  s->node.resize(size_t(px) * py * 3);
  for (int j = 0; j < py; ++j)
    for (int i = 0; i < px; ++i) {
      const size_t n = size_t(j) * px + i;
      s->node[n * 3 + 0] = x0 + i * hx; s->node[n * 3 + 1] = y0 + j * hy; s->node[n * 3 + 2] = 0.0;
    }
  if (jitter > 0) {
    // Jitter interior nodes; for periodic meshes also the boundary nodes of the master sides so that
    // slave copies stay exact translates.
    for (int j = 0; j < py; ++j)
      for (int i = 0; i < px; ++i) {
        const double dx = uni(rng) * jitter * hx, dy = uni(rng) * jitter * hy;
        const bool ix = i > 0 && i < nx, iy = j > 0 && j < ny;  // interior node
        const size_t n = size_t(j) * px + i;
        if (periodic) {
          if (i == nx || j == ny) continue;  // slaves copied below
          s->node[n * 3 + 0] += (i == 0 ? 0.0 : dx);
          s->node[n * 3 + 1] += (j == 0 ? 0.0 : dy);
        } else if (ix && iy) {
          s->node[n * 3 + 0] += dx; s->node[n * 3 + 1] += dy;
        }
      }
    if (periodic) {
      for (int j = 0; j < py; ++j)
        for (int i = 0; i < px; ++i) {
          if (i != nx && j != ny) continue;
          const int mi = i == nx ? 0 : i, mj = j == ny ? 0 : j;
          const size_t n = size_t(j) * px + i, mn = size_t(mj) * px + mi;
          s->node[n * 3 + 0] = s->node[mn * 3 + 0] + (i == nx ? lx : 0.0);
          s->node[n * 3 + 1] = s->node[mn * 3 + 1] + (j == ny ? ly : 0.0);
        }
    }
  }
  if (periodic) {
    s->periodic.resize(size_t(px) * py);
    for (int j = 0; j < py; ++j)
      for (int i = 0; i < px; ++i) {
        const int mi = i == nx ? 0 : i, mj = j == ny ? 0 : j;
        s->periodic[size_t(j) * px + i] = int32_t(size_t(mj) * px + mi);
      }
  }
  std::mt19937_64 rsplit(seed ^ 0x9e3779b97f4a7c15ull);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int32_t a = j * px + i, b = a + 1, c = a + px + 1, d = a + px;  // counter-clockwise
      if (split_fraction > 0 && unit(rsplit) < split_fraction) {
        s->tri.insert(s->tri.end(), {a, b, c});
        s->tri.insert(s->tri.end(), {a, c, d});
      } else {
        s->quad.insert(s->quad.end(), {a, b, c, d});
      }
    }
  // Boundary lines: bottom(1) right(2) top(3) left(4), or one periodic group.
  for (int i = 0; i < nx; ++i) { s->bnode.insert(s->bnode.end(), {i, i + 1}); s->bphys.push_back(periodic ? 1 : 1); }
  for (int j = 0; j < ny; ++j) { s->bnode.insert(s->bnode.end(), {j * px + nx, (j + 1) * px + nx}); s->bphys.push_back(periodic ? 1 : 2); }
  for (int i = 0; i < nx; ++i) { s->bnode.insert(s->bnode.end(), {ny * px + i + 1, ny * px + i}); s->bphys.push_back(periodic ? 1 : 3); }
  for (int j = 0; j < ny; ++j) { s->bnode.insert(s->bnode.end(), {(j + 1) * px, j * px}); s->bphys.push_back(periodic ? 1 : 4); }
  if (periodic) s->bc = {SDG_BC_PERIODIC};
  else s->bc.assign(boundary_condition, boundary_condition + 4);
  publish(s, 2, out);
  return SDG_OK;
}

int sdg_mesh_generate_annulus(double inner_radius, double outer_radius, int32_t nr, int32_t ntheta,
                              int32_t geometry_order, double split_fraction, uint64_t seed,
                              const int32_t* boundary_condition, sdg_generated_mesh* out) {
  if (!out || !boundary_condition || nr < 1 || ntheta < 3 || !(inner_radius > 0) || !(outer_radius > inner_radius) ||
      geometry_order < 1 || geometry_order > 5 || split_fraction < 0 || split_fraction > 1)
    return SDG_ERR_INVALID_ARGUMENT;
  auto* s = new MeshStorage();
  const int q = geometry_order;
  const int64_t fr = int64_t(q) * nr + 1, ft = int64_t(q) * ntheta;  // the fine node lattice (theta periodic)
  const auto id = [&](int64_t I, int64_t J) { return int32_t(I * ft + ((J % ft) + ft) % ft); };
  s->node.resize(size_t(fr * ft) * 3);
  const double twoPi = 6.283185307179586476925286766559;
  for (int64_t I = 0; I < fr; ++I)
    for (int64_t J = 0; J < ft; ++J) {
      const double r = inner_radius + (outer_radius - inner_radius) * double(I) / double(fr - 1);
      const double t = twoPi * double(J) / double(ft);
      const size_t n = size_t(id(I, J));
      s->node[n * 3 + 0] = r * std::cos(t); s->node[n * 3 + 1] = r * std::sin(t); s->node[n * 3 + 2] = 0.0;
    }
  const std::vector<std::array<int, 3>> quadLat = sdg::gmshLattice(SDG_ELEMENT_QUADRANGLE, q);
  const std::vector<std::array<int, 3>> triLat = sdg::gmshLattice(SDG_ELEMENT_TRIANGLE, q);
  std::mt19937_64 rsplit(seed);
  const auto unit = [](std::mt19937_64& g) { return double(g() >> 11) * (1.0 / 9007199254740992.0); };
  for (int64_t i = 0; i < nr; ++i)
    for (int64_t j = 0; j < ntheta; ++j) {
      const int64_t I0 = q * i, J0 = q * j;
      // vertices counter-clockwise: (r, theta) -> (r + dr, theta) -> (r + dr, theta + dt) -> (r, theta + dt)
      const int32_t a = id(I0, J0), b = id(I0 + q, J0), c = id(I0 + q, J0 + q), d = id(I0, J0 + q);
      if (split_fraction > 0 && unit(rsplit) < split_fraction) {
        // triangles (a, b, c) and (a, c, d): their order-q nodes are points of the element's lattice
        s->tri.insert(s->tri.end(), {a, b, c});
        s->tri.insert(s->tri.end(), {a, c, d});
        if (q > 1) {
          for (const auto& l : triLat) s->triGeo.push_back(id(I0 + l[0] + l[1], J0 + l[1]));
          for (const auto& l : triLat) s->triGeo.push_back(id(I0 + l[0], J0 + l[0] + l[1]));
        }
      } else {
        s->quad.insert(s->quad.end(), {a, b, c, d});
        if (q > 1)
          for (const auto& l : quadLat) s->quadGeo.push_back(id(I0 + l[0], J0 + l[1]));
      }
    }
  // boundary lines: the inner circle (group 1) and the outer circle (group 2), in the direction of the elements'
  // own edges
  for (int64_t j = 0; j < ntheta; ++j) {
    s->bnode.insert(s->bnode.end(), {id(0, q * (j + 1)), id(0, q * j)});
    s->bphys.push_back(1);
  }
  for (int64_t j = 0; j < ntheta; ++j) {
    s->bnode.insert(s->bnode.end(), {id(fr - 1, q * j), id(fr - 1, q * (j + 1))});
    s->bphys.push_back(2);
  }
  s->bc.assign(boundary_condition, boundary_condition + 2);
  s->geometryOrder = q;
  publish(s, 2, out);
  return SDG_OK;
}

int sdg_mesh_generate_1d(double x0, double lx, int32_t nx, int32_t periodic, const int32_t* boundary_condition,
                         sdg_generated_mesh* out) {
  if (!out || nx < 1 || !(lx > 0) || (!periodic && !boundary_condition)) return SDG_ERR_INVALID_ARGUMENT;
  if (periodic && nx < 3) return SDG_ERR_INVALID_ARGUMENT;  // the two ends of one element would coincide
  auto* s = new MeshStorage();
  s->node.resize(size_t(nx + 1) * 3, 0.0);
  for (int i = 0; i <= nx; ++i) s->node[size_t(i) * 3] = x0 + lx * double(i) / nx;
  for (int i = 0; i < nx; ++i) s->line.insert(s->line.end(), {i, i + 1});
  if (periodic) {
    s->periodic.resize(size_t(nx + 1));
    for (int i = 0; i <= nx; ++i) s->periodic[size_t(i)] = i == nx ? 0 : i;
  }
  // boundary points: the x0 end (group 1) and the x0 + lx end (group 2), or one periodic group
  s->bnode = {0, nx};
  s->bphys = {1, periodic ? 1 : 2};
  if (periodic) s->bc = {SDG_BC_PERIODIC};
  else s->bc.assign(boundary_condition, boundary_condition + 2);
  publish(s, 1, out);
  return SDG_OK;
}

int sdg_mesh_generate_3d(double x0, double y0, double z0, double lx, double ly, double lz, int32_t nx, int32_t ny,
                         int32_t nz, int32_t periodic, const int32_t* boundary_condition, sdg_generated_mesh* out) {
  if (!out || nx < 1 || ny < 1 || nz < 1 || !(lx > 0) || !(ly > 0) || !(lz > 0) || (!periodic && !boundary_condition))
    return SDG_ERR_INVALID_ARGUMENT;
  const int64_t px = nx + 1, py = ny + 1, pz = nz + 1;
  if (px * py * pz >= (int64_t(1) << 31)) return SDG_ERR_INVALID_ARGUMENT;
  auto* s = new MeshStorage();
  s->node.resize(size_t(px * py * pz) * 3);
  const auto id = [&](int64_t i, int64_t j, int64_t k) { return int32_t((k * py + j) * px + i); };
  for (int64_t k = 0; k < pz; ++k)
    for (int64_t j = 0; j < py; ++j)
      for (int64_t i = 0; i < px; ++i) {
        const size_t n = size_t(id(i, j, k));
        s->node[n * 3 + 0] = x0 + lx * double(i) / nx;
        s->node[n * 3 + 1] = y0 + ly * double(j) / ny;
        s->node[n * 3 + 2] = z0 + lz * double(k) / nz;
      }
  if (periodic) {
    s->periodic.resize(size_t(px * py * pz));
    for (int64_t k = 0; k < pz; ++k)
      for (int64_t j = 0; j < py; ++j)
        for (int64_t i = 0; i < px; ++i)
          s->periodic[size_t(id(i, j, k))] = id(i == nx ? 0 : i, j == ny ? 0 : j, k == nz ? 0 : k);
  }
  s->hex.reserve(size_t(nx) * ny * nz * 8);
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t i = 0; i < nx; ++i) {
        s->hex.insert(s->hex.end(), {id(i, j, k), id(i + 1, j, k), id(i + 1, j + 1, k), id(i, j + 1, k),
                                     id(i, j, k + 1), id(i + 1, j, k + 1), id(i + 1, j + 1, k + 1), id(i, j + 1, k + 1)});
      }
  // Boundary quads with outward orientation: x-(1) x+(2) y-(3) y+(4) z-(5) z+(6).
  const auto addQ = [&](int32_t a, int32_t b, int32_t c, int32_t d, int g) {
    s->bnode.insert(s->bnode.end(), {a, b, c, d}); s->bphys.push_back(periodic ? 1 : g);
  };
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j) {
      addQ(id(0, j, k), id(0, j, k + 1), id(0, j + 1, k + 1), id(0, j + 1, k), 1);
      addQ(id(nx, j, k), id(nx, j + 1, k), id(nx, j + 1, k + 1), id(nx, j, k + 1), 2);
    }
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t i = 0; i < nx; ++i) {
      addQ(id(i, 0, k), id(i + 1, 0, k), id(i + 1, 0, k + 1), id(i, 0, k + 1), 3);
      addQ(id(i, ny, k), id(i, ny, k + 1), id(i + 1, ny, k + 1), id(i + 1, ny, k), 4);
    }
  for (int64_t j = 0; j < ny; ++j)
    for (int64_t i = 0; i < nx; ++i) {
      addQ(id(i, j, 0), id(i, j + 1, 0), id(i + 1, j + 1, 0), id(i + 1, j, 0), 5);
      addQ(id(i, j, nz), id(i + 1, j, nz), id(i + 1, j + 1, nz), id(i, j + 1, nz), 6);
    }
  if (periodic) s->bc = {SDG_BC_PERIODIC};
  else s->bc.assign(boundary_condition, boundary_condition + 6);
  publish(s, 3, out);
  return SDG_OK;
}

// Structured tetrahedral box: the hexahedral box of sdg_mesh_generate_3d with every cube split into the six
// tetrahedra around its diagonal from the lowest to the highest corner (Kuhn's subdivision, conforming
// between cubes and across periodic sides), vertices ordered for a positive Jacobian.  Boundary elements are
// the tetrahedron faces on the box sides, triangles with a fourth index of -1, in the same groups.
int sdg_mesh_generate_3d_tetrahedra(double x0, double y0, double z0, double lx, double ly, double lz, int32_t nx,
                                    int32_t ny, int32_t nz, int32_t periodic, const int32_t* boundary_condition,
                                    sdg_generated_mesh* out) {
  const int rc = sdg_mesh_generate_3d(x0, y0, z0, lx, ly, lz, nx, ny, nz, periodic, boundary_condition, out);
  if (rc != SDG_OK) return rc;
  auto* s = static_cast<MeshStorage*>(out->storage);
  const int64_t px = nx + 1, py = ny + 1;
  const auto node = [&](int32_t n, int d) { return s->node[size_t(n) * 3 + d]; };
  const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  s->tet.reserve(s->hex.size() / 8 * 24);
  for (size_t h = 0; h < s->hex.size(); h += 8) {
    // hexahedron corner of offset (dx, dy, dz): vertex list 0..7 of sdg_mesh_generate_3d
    const auto corner = [&](int dx, int dy, int dz) {
      static const int at[2][2][2] = {{{0, 4}, {3, 7}}, {{1, 5}, {2, 6}}};
      return s->hex[h + at[dx][dy][dz]];
    };
    for (const auto& pm : perms) {
      int c[3] = {0, 0, 0};
      int32_t v[4];
      v[0] = corner(0, 0, 0);
      for (int k = 0; k < 3; ++k) { c[pm[k]] = 1; v[k + 1] = corner(c[0], c[1], c[2]); }
      double a[3][3];
      for (int k = 0; k < 3; ++k)
        for (int d = 0; d < 3; ++d) a[k][d] = node(v[k + 1], d) - node(v[0], d);
      const double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
                         a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
      if (det < 0) std::swap(v[2], v[3]);
      s->tet.insert(s->tet.end(), {v[0], v[1], v[2], v[3]});
    }
  }
  s->hex.clear();
  // boundary triangles: tetrahedron faces whose three vertices lie on one side of the box
  s->bnode.clear(); s->bphys.clear();
  const int* fl = sdg::faceVertexList(SDG_ELEMENT_TETRAHEDRON);
  const auto side = [&](int32_t n) {
    const int64_t i = n % px, j = (n / px) % py, k = n / (px * py);
    int m = 0;
    if (i == 0) m |= 1; if (i == nx) m |= 2; if (j == 0) m |= 4;
    if (j == ny) m |= 8; if (k == 0) m |= 16; if (k == nz) m |= 32;
    return m;
  };
  for (size_t t = 0; t < s->tet.size(); t += 4)
    for (int f = 0; f < 4; ++f) {
      const int32_t a = s->tet[t + fl[f * 3]], b = s->tet[t + fl[f * 3 + 1]], c = s->tet[t + fl[f * 3 + 2]];
      const int common = side(a) & side(b) & side(c);
      if (!common) continue;
      int g = 0;
      while (!(common & (1 << g))) ++g;
      s->bnode.insert(s->bnode.end(), {a, b, c, -1});
      s->bphys.push_back(periodic ? 1 : g + 1);
    }
  publish(s, 3, out);
  return SDG_OK;
}

// MSH 4.1 ASCII reader: $PhysicalNames (optional), $Entities (physical tags of entities),
// $Nodes, $Elements, $Periodic (node pairs).  Element types 1/8/26-28 (lines), 2/9/21/23/25 (triangles),
// 3/10/36-38 (quadrangles), 4/11/29-31 (tetrahedra), 5/12/92-94 (hexahedra).  The primary vertices form the
// element lists; a 2D mesh of order q > 1 also keeps every element's full node list as its curved geometry
// (geometry_order q; 3D and 1D meshes are read by their vertices).  A 3D mesh holds tetrahedra or hexahedra;
// its triangular boundary elements get a fourth index of -1.
int sdg_mesh_read_msh(const char* path, sdg_generated_mesh* out) {
  if (!path || !out) return SDG_ERR_INVALID_ARGUMENT;
  std::ifstream in(path);
  if (!in) return SDG_ERR_INVALID_ARGUMENT;
  auto* s = new MeshStorage();
  std::map<std::pair<int, int>, std::vector<int>> entityPhysical;  // (dim, tag) -> physical tags
  std::unordered_map<int64_t, int32_t> nodeIndex;
  std::vector<std::pair<int64_t, int64_t>> periodicPairs;
  struct BEl { std::vector<int64_t> v; int phys; };
  std::vector<BEl> bels;
  std::vector<std::vector<int64_t>> tris, quads, hexes;
  int maxDim = 0;
  std::map<int, int> physOrder;
  const auto typeInfo = [](int t, int& dim, int& nn, int& nprim) {
    switch (t) {
      case 1: dim = 1; nn = 2; nprim = 2; return true;
      case 8: dim = 1; nn = 3; nprim = 2; return true;
      case 26: dim = 1; nn = 4; nprim = 2; return true;
      case 27: dim = 1; nn = 5; nprim = 2; return true;
      case 28: dim = 1; nn = 6; nprim = 2; return true;
      case 2: dim = 2; nn = 3; nprim = 3; return true;
      case 9: dim = 2; nn = 6; nprim = 3; return true;
      case 21: dim = 2; nn = 10; nprim = 3; return true;
      case 23: dim = 2; nn = 15; nprim = 3; return true;
      case 25: dim = 2; nn = 21; nprim = 3; return true;
      case 3: dim = 2; nn = 4; nprim = 4; return true;
      case 10: dim = 2; nn = 9; nprim = 4; return true;
      case 36: dim = 2; nn = 16; nprim = 4; return true;
      case 37: dim = 2; nn = 25; nprim = 4; return true;
      case 38: dim = 2; nn = 36; nprim = 4; return true;
      case 4: dim = 3; nn = 4; nprim = 4; return true;
      case 11: dim = 3; nn = 10; nprim = 4; return true;
      case 29: dim = 3; nn = 20; nprim = 4; return true;
      case 30: dim = 3; nn = 35; nprim = 4; return true;
      case 31: dim = 3; nn = 56; nprim = 4; return true;
      case 5: dim = 3; nn = 8; nprim = 8; return true;
      case 12: dim = 3; nn = 27; nprim = 8; return true;
      case 92: dim = 3; nn = 64; nprim = 8; return true;
      case 93: dim = 3; nn = 125; nprim = 8; return true;
      case 94: dim = 3; nn = 216; nprim = 8; return true;
      case 15: dim = 0; nn = 1; nprim = 1; return true;
      default: return false;
    }
  };
  struct RawEl { int type; int edim; int etag; std::vector<int64_t> v, all; };
  std::vector<RawEl> raw;
  std::string line;
  try {
    while (std::getline(in, line)) {
      if (line.rfind("$MeshFormat", 0) == 0) {
        std::getline(in, line);
        if (line.rfind("4.1", 0) != 0) throw std::runtime_error("only MSH 4.1 ASCII is supported");
      } else if (line.rfind("$Entities", 0) == 0) {
        int64_t np, nc, ns, nv; in >> np >> nc >> ns >> nv;
        const int64_t cnt[4] = {np, nc, ns, nv};
        for (int d = 0; d < 4; ++d)
          for (int64_t i = 0; i < cnt[d]; ++i) {
            int tag; in >> tag;
            double bb; for (int k = 0; k < (d == 0 ? 3 : 6); ++k) in >> bb;
            int nphys; in >> nphys;
            std::vector<int> ph(nphys); for (int& p : ph) in >> p;
            entityPhysical[{d, tag}] = ph;
            if (d > 0) { int nb; in >> nb; for (int k = 0; k < nb; ++k) { int t; in >> t; } }
          }
      } else if (line.rfind("$Nodes", 0) == 0) {
        int64_t nblocks, nnodes, mn, mx; in >> nblocks >> nnodes >> mn >> mx;
        s->node.reserve(size_t(nnodes) * 3);
        for (int64_t b = 0; b < nblocks; ++b) {
          int ed, et, param; int64_t n; in >> ed >> et >> param >> n;
          std::vector<int64_t> tags(n); for (auto& t : tags) in >> t;
          for (int64_t i = 0; i < n; ++i) {
            double x, y, z; in >> x >> y >> z;
            if (param) { double u; for (int k = 0; k < ed; ++k) in >> u; }
            nodeIndex[tags[i]] = int32_t(s->node.size() / 3);
            s->node.insert(s->node.end(), {x, y, z});
          }
        }
      } else if (line.rfind("$Elements", 0) == 0) {
        int64_t nblocks, nel, mn, mx; in >> nblocks >> nel >> mn >> mx;
        for (int64_t b = 0; b < nblocks; ++b) {
          int ed, et, type; int64_t n; in >> ed >> et >> type >> n;
          int dim = 0, nn = 0, nprim = 0;
          if (!typeInfo(type, dim, nn, nprim)) throw std::runtime_error("unsupported element type " + std::to_string(type));
          for (int64_t i = 0; i < n; ++i) {
            int64_t tag; in >> tag;
            RawEl r; r.type = type; r.edim = ed; r.etag = et; r.v.resize(nprim); r.all.resize(nn);
            for (int k = 0; k < nn; ++k) { int64_t v; in >> v; r.all[k] = v; if (k < nprim) r.v[k] = v; }
            maxDim = std::max(maxDim, dim);
            raw.push_back(std::move(r));
          }
        }
      } else if (line.rfind("$Periodic", 0) == 0) {
        int64_t nlinks; in >> nlinks;
        for (int64_t l = 0; l < nlinks; ++l) {
          int ed, tag, mtag; in >> ed >> tag >> mtag;
          int64_t naff; in >> naff; double a; for (int64_t k = 0; k < naff; ++k) in >> a;
          int64_t nn; in >> nn;
          for (int64_t k = 0; k < nn; ++k) { int64_t sl, ma; in >> sl >> ma; periodicPairs.push_back({sl, ma}); }
        }
      }
    }
    if (maxDim < 1) throw std::runtime_error("no line, surface or volume elements in the mesh");
    const auto idx = [&](int64_t tag) {
      const auto it = nodeIndex.find(tag);
      if (it == nodeIndex.end()) throw std::runtime_error("element references an unknown node");
      return it->second;
    };
    // 2D meshes and hexahedra of order q > 1 (the drivers' setOrder(P)): every element's full node list in
    // gmsh order is kept as its curved geometry (ReadControl.cpp:243-256); lines and tetrahedra keep their
    // vertices only
    int order2d = 0;
    for (const RawEl& r : raw) {
      int dim = 0, nn = 0, nprim = 0; typeInfo(r.type, dim, nn, nprim);
      if (dim != maxDim || (dim != 2 && !(dim == 3 && nprim == 8))) continue;
      const int et = dim == 3 ? SDG_ELEMENT_HEXAHEDRON : (nprim == 3 ? SDG_ELEMENT_TRIANGLE : SDG_ELEMENT_QUADRANGLE);
      int q = 1;
      while (sdg::gmshNodeCount(et, q) < nn) ++q;
      if (order2d && q != order2d) throw std::runtime_error("elements of different geometry orders");
      order2d = q;
    }
    for (const RawEl& r : raw) {
      int dim = 0, nn = 0, nprim = 0; typeInfo(r.type, dim, nn, nprim);
      if (dim == maxDim) {
        std::vector<int32_t>* dst = maxDim == 1 ? &s->line
                                    : maxDim == 2 ? (nprim == 3 ? &s->tri : &s->quad)
                                                  : (nprim == 4 ? &s->tet : &s->hex);
        for (int64_t v : r.v) dst->push_back(idx(v));
        if (maxDim == 2 && order2d > 1)
          for (int64_t v : r.all) (nprim == 3 ? s->triGeo : s->quadGeo).push_back(idx(v));
        if (maxDim == 3 && nprim == 8 && order2d > 1)
          for (int64_t v : r.all) s->hexGeo.push_back(idx(v));
      } else if (dim == maxDim - 1) {
        const auto it = entityPhysical.find({r.edim, r.etag});
        if (it == entityPhysical.end() || it->second.empty()) continue;
        const int phys = it->second[0];
        if (!physOrder.count(phys)) { const int k = int(physOrder.size()) + 1; physOrder[phys] = k; }
        BEl bel; bel.v.assign(r.v.begin(), r.v.end()); bel.phys = phys;
        bels.push_back(std::move(bel));
      }
    }
    // Physical groups are numbered 1..n in the order of their first boundary element; the file's own
    // tags are remapped so that boundary_physical indexes physical_boundary_condition.
    std::map<int, int> remap;
    {
      std::vector<int> tags; for (auto& kv : physOrder) tags.push_back(kv.first);
      std::sort(tags.begin(), tags.end());
      for (size_t i = 0; i < tags.size(); ++i) remap[tags[i]] = int(i) + 1;
    }
    if (order2d > 1) s->geometryOrder = order2d;
    if (!s->tet.empty() && !s->hex.empty())
      throw std::runtime_error("a 3D mesh of tetrahedra and hexahedra needs pyramids, which are not supported");
    for (const BEl& b : bels) {
      for (int64_t v : b.v) s->bnode.push_back(idx(v));
      if (maxDim == 3 && b.v.size() == 3) s->bnode.push_back(-1);
      s->bphys.push_back(remap[b.phys]);
    }
    s->bc.assign(remap.size(), SDG_BC_PERIODIC);
    if (!periodicPairs.empty()) {
      s->periodic.resize(s->node.size() / 3);
      for (size_t i = 0; i < s->periodic.size(); ++i) s->periodic[i] = int32_t(i);
      for (auto& pr : periodicPairs) s->periodic[idx(pr.first)] = idx(pr.second);
      // Resolve chains (corner nodes slave to slaves).
      for (size_t i = 0; i < s->periodic.size(); ++i) {
        int32_t m = s->periodic[i];
        for (int g = 0; g < 8 && s->periodic[m] != m; ++g) m = s->periodic[m];
        s->periodic[i] = m;
      }
    }
  } catch (const std::exception&) {
    delete s;
    return SDG_ERR_MESH;
  }
  publish(s, maxDim, out);
  return SDG_OK;
}

int sdg_mesh_free(sdg_generated_mesh* m) {
  if (!m) return SDG_ERR_INVALID_ARGUMENT;
  delete static_cast<MeshStorage*>(m->storage);
  m->storage = nullptr;
  std::memset(&m->mesh, 0, sizeof(m->mesh));
  return SDG_OK;
}

}  // extern "C"
#pragma GCC visibility pop
