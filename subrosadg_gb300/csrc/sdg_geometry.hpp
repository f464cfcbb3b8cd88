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
//               direction, then the interior nodes as a triangle of order q-3 on the inner lattice (recursively).
// Lattice index (i, j): quadrangles x = -1 + 2i/q, y = -1 + 2j/q; triangles x = i/q, y = j/q.
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "../../include/sdg_gpu.h"

namespace sdg {

// Lattice indices (i, j) of the nodes of an order-q element in gmsh order.
inline std::vector<std::array<int, 2>> gmshLattice(int type, int q) {
  std::vector<std::array<int, 2>> out;
  if (type == SDG_ELEMENT_LINE) {
    out.push_back({0, 0});
    if (q >= 1) out.push_back({q, 0});
    for (int k = 1; k < q; ++k) out.push_back({k, 0});
    return out;
  }
  if (type == SDG_ELEMENT_QUADRANGLE) {
    // rings from the outside in: ring of order r on the lattice offset o
    for (int r = q, o = 0; r >= 0; r -= 2, ++o) {
      if (r == 0) { out.push_back({o, o}); break; }
      const int a = o, b = o + r;
      out.push_back({a, a}); out.push_back({b, a}); out.push_back({b, b}); out.push_back({a, b});
      for (int k = 1; k < r; ++k) out.push_back({a + k, a});
      for (int k = 1; k < r; ++k) out.push_back({b, a + k});
      for (int k = 1; k < r; ++k) out.push_back({b - k, b});
      for (int k = 1; k < r; ++k) out.push_back({a, b - k});
    }
    return out;
  }
  if (type == SDG_ELEMENT_TRIANGLE) {
    for (int r = q, o = 0; r >= 0; r -= 3, ++o) {
      if (r == 0) { out.push_back({o, o}); break; }
      out.push_back({o, o}); out.push_back({o + r, o}); out.push_back({o, o + r});
      for (int k = 1; k < r; ++k) out.push_back({o + k, o});
      for (int k = 1; k < r; ++k) out.push_back({o + r - k, o + k});
      for (int k = 1; k < r; ++k) out.push_back({o, o + r - k});
    }
    return out;
  }
  throw std::runtime_error("high-order geometry: unsupported element type");
}

inline int gmshNodeCount(int type, int q) {
  if (type == SDG_ELEMENT_LINE) return q + 1;
  if (type == SDG_ELEMENT_QUADRANGLE) return (q + 1) * (q + 1);
  if (type == SDG_ELEMENT_TRIANGLE) return (q + 1) * (q + 2) / 2;
  return 0;
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

// Values N[n] and reference gradients G[n][2] of the gmsh-ordered order-q basis of a quadrangle or triangle at
// the reference point X.
inline void gmshBasis(int type, int q, const std::vector<std::array<int, 2>>& lat, const double* X, double* N,
                      double (*G)[2]) {
  for (size_t n = 0; n < lat.size(); ++n) {
    const int i = lat[n][0], j = lat[n][1];
    if (type == SDG_ELEMENT_QUADRANGLE) {
      double vx, dx, vy, dy;
      lagrange1d(q, i, X[0], vx, dx);
      lagrange1d(q, j, X[1], vy, dy);
      N[n] = vx * vy;
      G[n][0] = dx * vy;
      G[n][1] = vx * dy;
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

// The order-q map of a 2D element through its gmsh-ordered geometry nodes: x(X) and J[l][k] = dx_l/dX_k.
struct CurvedMap2d {
  int type = 0, q = 1;
  std::vector<std::array<int, 2>> lattice;
  void init(int t, int order) {
    type = t;
    q = order;
    lattice = gmshLattice(t, order);
  }
  void eval(const double* coords, const int32_t* idx, const double* X, double J[3][3], double* x) const {
    const size_t nn = lattice.size();
    std::vector<double> N(nn);
    std::vector<std::array<double, 2>> G(nn);
    gmshBasis(type, q, lattice, X, N.data(), reinterpret_cast<double(*)[2]>(G.data()));
    for (int l = 0; l < 3; ++l) { x[l] = 0.0; for (int k = 0; k < 3; ++k) J[l][k] = 0.0; }
    for (size_t n = 0; n < nn; ++n) {
      const double* c = &coords[size_t(idx[n]) * 3];
      for (int l = 0; l < 3; ++l) x[l] += N[n] * c[l];
      for (int l = 0; l < 2; ++l)
        for (int k = 0; k < 2; ++k) J[l][k] += G[n][k] * c[l];
    }
  }
};

}  // namespace sdg
