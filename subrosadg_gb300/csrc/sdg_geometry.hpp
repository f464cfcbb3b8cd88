// High-order (curved) element geometry: the order-q Lagrange map through an element's geometry nodes in gmsh's
// node order, as gmsh evaluates it for the reference's Jacobians and normals (src/Mesh/Geometry.cpp:44-86,
// 102-169; the nodes come from src/Mesh/ReadControl.cpp:243-256 after the drivers' setOrder(P)).
//
// gmsh's order of the nodes of a Lagrange element of order q (equispaced):
//   line        the two end points, then the interior points from the first end to the second;
//   quadrangle  ([-1,1]^2) the 4 corners, the q-1 interior points of each edge 0-1, 1-2, 2-3, 3-0 in edge
//               direction, then the interior nodes as a quadrangle of order q-2 on the inner lattice (recursively;
//               order 0 is the single centre node);
//   triangle    ((0,0), (1,0), (0,1)) the 3 corners, the q-1 interior points of edges 0-1, 1-2, 2-0 in edge
//               direction, then the interior nodes as a triangle of order q-3 on the inner lattice (recursively);
//   hexahedron  ([-1,1]^3, corners (-1,-1,-1), (1,-1,-1), (1,1,-1), (-1,1,-1), then the same at z = +1) the 8
//               corners, the q-1 interior points of each edge in the edge order 0-1, 0-3, 0-4, 1-2, 1-5, 2-3, 2-6,
//               3-7, 4-5, 4-7, 5-6, 6-7 (in edge direction), the interior nodes of each face in the face order
//               (0,3,2,1), (0,1,5,4), (0,4,7,3), (1,2,6,5), (2,3,7,6), (4,5,6,7) as a quadrangle of order q-2
//               whose corners follow the face's vertex list, then the interior nodes as a hexahedron of order
//               q-2 on the inner lattice (recursively).
// Lattice index (i, j, k): quadrangles and hexahedra x = -1 + 2i/q, y = -1 + 2j/q, z = -1 + 2k/q; triangles
// x = i/q, y = j/q.
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "../../include/sdg_gpu.h"

namespace sdg {

// Lattice indices (i, j, k) of the nodes of an order-q element in gmsh order (k = 0 below 3D).
inline std::vector<std::array<int, 3>> gmshLattice(int type, int q) {
  std::vector<std::array<int, 3>> out;
  if (type == SDG_ELEMENT_LINE) {
    out.push_back({0, 0, 0});
    if (q >= 1) out.push_back({q, 0, 0});
    for (int k = 1; k < q; ++k) out.push_back({k, 0, 0});
    return out;
  }
  if (type == SDG_ELEMENT_QUADRANGLE) {
    // rings from the outside in: ring of order r on the lattice offset o
    for (int r = q, o = 0; r >= 0; r -= 2, ++o) {
      if (r == 0) { out.push_back({o, o, 0}); break; }
      const int a = o, b = o + r;
      out.push_back({a, a, 0}); out.push_back({b, a, 0}); out.push_back({b, b, 0}); out.push_back({a, b, 0});
      for (int k = 1; k < r; ++k) out.push_back({a + k, a, 0});
      for (int k = 1; k < r; ++k) out.push_back({b, a + k, 0});
      for (int k = 1; k < r; ++k) out.push_back({b - k, b, 0});
      for (int k = 1; k < r; ++k) out.push_back({a, b - k, 0});
    }
    return out;
  }
  if (type == SDG_ELEMENT_TRIANGLE) {
    for (int r = q, o = 0; r >= 0; r -= 3, ++o) {
      if (r == 0) { out.push_back({o, o, 0}); break; }
      out.push_back({o, o, 0}); out.push_back({o + r, o, 0}); out.push_back({o, o + r, 0});
      for (int k = 1; k < r; ++k) out.push_back({o + k, o, 0});
      for (int k = 1; k < r; ++k) out.push_back({o + r - k, o + k, 0});
      for (int k = 1; k < r; ++k) out.push_back({o, o + r - k, 0});
    }
    return out;
  }
  if (type == SDG_ELEMENT_HEXAHEDRON) {
    static const int edge[12][2] = {{0, 1}, {0, 3}, {0, 4}, {1, 2}, {1, 5}, {2, 3},
                                    {2, 6}, {3, 7}, {4, 5}, {4, 7}, {5, 6}, {6, 7}};
    static const int face[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {0, 4, 7, 3}, {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};
    for (int r = q, o = 0; r >= 0; r -= 2, ++o) {
      if (r == 0) { out.push_back({o, o, o}); break; }
      const int a = o, b = o + r;
      const std::array<int, 3> V[8] = {{a, a, a}, {b, a, a}, {b, b, a}, {a, b, a},
                                       {a, a, b}, {b, a, b}, {b, b, b}, {a, b, b}};
      // unit lattice step from corner u towards corner v (their coordinates differ by r along one axis per step)
      const auto step = [&](int u, int v) {
        return std::array<int, 3>{(V[v][0] - V[u][0]) / r, (V[v][1] - V[u][1]) / r, (V[v][2] - V[u][2]) / r};
      };
      for (const auto& c : V) out.push_back(c);
      for (const auto& e : edge) {
        const auto d = step(e[0], e[1]);
        for (int k = 1; k < r; ++k) out.push_back({V[e[0]][0] + k * d[0], V[e[0]][1] + k * d[1], V[e[0]][2] + k * d[2]});
      }
      if (r >= 2) {
        const auto inner = gmshLattice(SDG_ELEMENT_QUADRANGLE, r - 2);
        for (const auto& f : face) {
          const auto d1 = step(f[0], f[1]), d2 = step(f[0], f[3]);
          for (const auto& l : inner) {
            const int s1 = l[0] + 1, s2 = l[1] + 1;
            out.push_back({V[f[0]][0] + s1 * d1[0] + s2 * d2[0], V[f[0]][1] + s1 * d1[1] + s2 * d2[1],
                           V[f[0]][2] + s1 * d1[2] + s2 * d2[2]});
          }
        }
      }
    }
    return out;
  }
  throw std::runtime_error("high-order geometry: unsupported element type");
}

inline int gmshNodeCount(int type, int q) {
  if (type == SDG_ELEMENT_LINE) return q + 1;
  if (type == SDG_ELEMENT_QUADRANGLE) return (q + 1) * (q + 1);
  if (type == SDG_ELEMENT_TRIANGLE) return (q + 1) * (q + 2) / 2;
  if (type == SDG_ELEMENT_HEXAHEDRON) return (q + 1) * (q + 1) * (q + 1);
  return 0;
}

// Reference coordinates of lattice node l of an order-q element.
inline void gmshLatticePoint(int type, int q, const std::array<int, 3>& l, double* X) {
  for (int d = 0; d < 3; ++d) X[d] = 0.0;
  const int dim = type == SDG_ELEMENT_HEXAHEDRON ? 3 : 2;
  for (int d = 0; d < dim; ++d) X[d] = type == SDG_ELEMENT_TRIANGLE ? double(l[d]) / q : -1.0 + 2.0 * l[d] / q;
}

// 1D Lagrange basis on the equispaced points t_k = -1 + 2k/q: value and derivative of basis k at t.
inline void lagrange1d(int q, int k, double t, double& v, double& d) {
  v = 1.0;
  d = 0.0;
  const double tk = -1.0 + 2.0 * k / q;
  for (int m = 0; m <= q; ++m) {
    if (m == k) continue;
    const double tm = -1.0 + 2.0 * m / q;
    const double f = (t - tm) / (tk - tm);
    d = d * f + v / (tk - tm);
    v *= f;
  }
}

// P_m(l) = prod_{a<m} (q l - a) / (a + 1) (the equispaced simplex Lagrange factor) and its derivative in l.
inline void simplexFactor(int q, int m, double l, double& v, double& d) {
  v = 1.0;
  d = 0.0;
  for (int a = 0; a < m; ++a) {
    const double f = (q * l - a) / (a + 1);
    d = d * f + v * q / (a + 1);
    v *= f;
  }
}

// Values N[n] and reference gradients G[n][3] of the gmsh-ordered order-q basis of a quadrangle, triangle or
// hexahedron at the reference point X.
inline void gmshBasis(int type, int q, const std::vector<std::array<int, 3>>& lat, const double* X, double* N,
                      double (*G)[3]) {
  for (size_t n = 0; n < lat.size(); ++n) {
    const int i = lat[n][0], j = lat[n][1];
    G[n][2] = 0.0;
    if (type == SDG_ELEMENT_QUADRANGLE || type == SDG_ELEMENT_HEXAHEDRON) {
      double vx, dx, vy, dy, vz = 1.0, dz = 0.0;
      lagrange1d(q, i, X[0], vx, dx);
      lagrange1d(q, j, X[1], vy, dy);
      if (type == SDG_ELEMENT_HEXAHEDRON) lagrange1d(q, lat[n][2], X[2], vz, dz);
      N[n] = vx * vy * vz;
      G[n][0] = dx * vy * vz;
      G[n][1] = vx * dy * vz;
      if (type == SDG_ELEMENT_HEXAHEDRON) G[n][2] = vx * vy * dz;
    } else {
      const int k = q - i - j;
      double a, da, b, db, c, dc;
      simplexFactor(q, i, X[0], a, da);
      simplexFactor(q, j, X[1], b, db);
      simplexFactor(q, k, 1.0 - X[0] - X[1], c, dc);
      N[n] = a * b * c;
      G[n][0] = da * b * c - a * b * dc;
      G[n][1] = a * db * c - a * b * dc;
    }
  }
}

// The order-q map of an element through its gmsh-ordered geometry nodes: x(X) and J[l][k] = dx_l/dX_k.
struct CurvedMap {
  int type = 0, q = 1, dim = 2;
  std::vector<std::array<int, 3>> lattice;
  void init(int t, int order) {
    type = t;
    q = order;
    dim = t == SDG_ELEMENT_HEXAHEDRON ? 3 : 2;
    lattice = gmshLattice(t, order);
  }
  void eval(const double* coords, const int32_t* idx, const double* X, double J[3][3], double* x) const {
    const size_t nn = lattice.size();
    std::vector<double> N(nn);
    std::vector<std::array<double, 3>> G(nn);
    gmshBasis(type, q, lattice, X, N.data(), reinterpret_cast<double(*)[3]>(G.data()));
    for (int l = 0; l < 3; ++l) { x[l] = 0.0; for (int k = 0; k < 3; ++k) J[l][k] = 0.0; }
    for (size_t n = 0; n < nn; ++n) {
      const double* c = &coords[size_t(idx[n]) * 3];
      for (int l = 0; l < 3; ++l) x[l] += N[n] * c[l];
      for (int l = 0; l < dim; ++l)
        for (int k = 0; k < dim; ++k) J[l][k] += G[n][k] * c[l];
    }
  }
};

}  // namespace sdg
