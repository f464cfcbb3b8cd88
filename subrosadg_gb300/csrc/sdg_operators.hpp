// Reference-element operators of the GB300 DG path (host side, built once per problem).
//
// Quadrature follows the reference's orders (src/Solver/SimulationControl.cpp:268-283: volume rule of
// order 2P, face rule of order 2P+1); gmsh's tensor Gauss-Legendre rules are used for quadrangles with
// P >= 2 and for hexahedra, so on those elements the volume rule has (P+1)^d points and coincides with a
// nodal Lagrange basis collocated at the Gauss points.  In that basis the quadrature mass matrix the
// reference inverts per element (src/Mesh/Geometry.cpp:88-100) is exactly diagonal, the volume term of
// src/Solver/SpatialDiscrete.cpp:194-266,1016-1032 becomes a sum-factorised 1D derivative per direction,
// and face traces/lifts (src/Solver/VariableConvertor.cpp:432-485) are 1D end-point interpolations.
// Triangles, first-order quadrangles (7-point rule) and tetrahedra keep a dense modal formulation.
//
// The modal basis -- used for the dense blocks, for the modal state exchange and for the relative error
// of src/Solver/TimeIntegration.cpp:279-324 (which depends on the basis) -- is the hierarchic H1 basis
// of Solin (Lobatto shape functions): the same family gmsh's "H1Legendre" provides the reference
// (src/Mesh/BasisFunction.cpp:45-74).
#pragma once
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sdg_gpu.h"
#include "tetrahedron_rules.h"
#include "triangle_rules.h"

namespace sdg {

constexpr int kMaxN = 6;  // points per direction (P <= 5)

// Legendre polynomial and derivative by recurrence.
inline void legendreP(int n, double x, double* p, double* dp) {
  double a = 1.0, b = x, da = 0.0, db = 1.0;
  if (n == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    const double c = ((2 * k - 1) * x * b - (k - 1) * a) / k;
    const double dc = da + (2 * k - 1) * b;
    a = b; b = c; da = db; db = dc;
  }
  *p = b; *dp = db;
}

// n-point Gauss-Legendre nodes (ascending) and weights: Newton iteration on P_n from the Chebyshev-like
// initial guess cos(pi (i + 3/4)/(n + 1/2)).
inline void gaussRule(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = -std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 64; ++it) {
      double p, dp; legendreP(n, z, &p, &dp);
      const double step = p / dp;
      z -= step;
      if (std::fabs(step) <= 1e-17) break;
    }
    double p, dp; legendreP(n, z, &p, &dp);
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// 1D Lagrange basis on nodes x[0..n): value and derivative of l_i at t.
inline void lagrange1d(int n, const double* x, int i, double t, double* v, double* d) {
  double val = 1.0, der = 0.0;
  for (int j = 0; j < n; ++j) {
    if (j == i) continue;
    const double f = (t - x[j]) / (x[i] - x[j]);
    der = der * f + val / (x[i] - x[j]);
    val *= f;
  }
  *v = val; *d = der;
}

// 1D Lobatto shape functions: l0=(1-x)/2, l1=(1+x)/2, lk=(P_k - P_{k-2})/sqrt(2(2k-1)).
inline double lobatto1d(int k, double x) {
  if (k == 0) return 0.5 * (1.0 - x);
  if (k == 1) return 0.5 * (1.0 + x);
  double pk, d, pk2;
  legendreP(k, x, &pk, &d);
  legendreP(k - 2, x, &pk2, &d);
  return (pk - pk2) / std::sqrt(2.0 * (2.0 * k - 1.0));
}

// Collocation operators of a tensor block with n = P+1 Gauss points per direction.
struct TensorOps {
  int n = 0;
  double x[kMaxN], w[kMaxN];
  double dhat[kMaxN][kMaxN];   // dhat[a][i] = l_i'(x_a) w_a / w_i  (weak derivative, mass-scaled)
  double endm[kMaxN], endp[kMaxN];   // l_i(-1), l_i(+1)       (traces)
  double liftm[kMaxN], liftp[kMaxN]; // l_i(-1)/w_i, l_i(+1)/w_i (lifts)
  double b1[kMaxN][kMaxN];     // sum_k lob_k(x_a) lob_k(x_b)     (relative-error transform)
  double phi1[kMaxN][kMaxN];   // phi1[i][m] = lob_m(x_i)         (modal -> nodal)
  double phi1inv[kMaxN][kMaxN];

  void build(int np) {
    n = np;
    gaussRule(n, x, w);
    for (int i = 0; i < n; ++i) {
      double v, d;
      for (int a = 0; a < n; ++a) { lagrange1d(n, x, i, x[a], &v, &d); dhat[a][i] = d * w[a] / w[i]; }
      lagrange1d(n, x, i, -1.0, &v, &d); endm[i] = v; liftm[i] = v / w[i];
      lagrange1d(n, x, i, 1.0, &v, &d); endp[i] = v; liftp[i] = v / w[i];
      for (int m = 0; m < n; ++m) phi1[i][m] = lobatto1d(m, x[i]);
    }
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        double s = 0; for (int k = 0; k < n; ++k) s += lobatto1d(k, x[a]) * lobatto1d(k, x[b]);
        b1[a][b] = s;
      }
    // invert phi1 (Gauss-Jordan)
    double m[kMaxN][2 * kMaxN];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < 2 * n; ++j) m[i][j] = j < n ? phi1[i][j] : (j - n == i ? 1.0 : 0.0);
    for (int c = 0; c < n; ++c) {
      int piv = c;
      for (int r = c + 1; r < n; ++r) if (std::fabs(m[r][c]) > std::fabs(m[piv][c])) piv = r;
      for (int j = 0; j < 2 * n; ++j) std::swap(m[c][j], m[piv][j]);
      const double inv = 1.0 / m[c][c];
      for (int j = 0; j < 2 * n; ++j) m[c][j] *= inv;
      for (int r = 0; r < n; ++r) {
        if (r == c) continue;
        const double f = m[r][c];
        for (int j = 0; j < 2 * n; ++j) m[r][j] -= f * m[c][j];
      }
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) phi1inv[i][j] = m[i][n + j];
  }
};

// ---- dense (modal) blocks ------------------------------------------------------------------------
struct Dual2 { double v, x, y; };
inline Dual2 dadd(Dual2 a, Dual2 b) { return {a.v + b.v, a.x + b.x, a.y + b.y}; }
inline Dual2 dsub(Dual2 a, Dual2 b) { return {a.v - b.v, a.x - b.x, a.y - b.y}; }
inline Dual2 dmul(Dual2 a, Dual2 b) { return {a.v * b.v, a.x * b.v + a.v * b.x, a.y * b.v + a.v * b.y}; }
inline Dual2 dlegendre(int n, Dual2 t) { double p, dp; legendreP(n, t.v, &p, &dp); return {p, dp * t.x, dp * t.y}; }
// Solin kernel function phi_{k-2}(t) = -4 sqrt((2k-1)/2) / ((k-1)k) * P'_{k-1}(t), with P'_m written as
// sum_{j = m-1, m-3, ...} (2j+1) P_j(t).
inline Dual2 dkernel(int k, Dual2 t) {
  const int m = k - 1;
  double s = 0.0, ds = 0.0;
  for (int j = m - 1; j >= 0; j -= 2) { double p, dp; legendreP(j, t.v, &p, &dp); s += (2 * j + 1) * p; ds += (2 * j + 1) * dp; }
  const double c = -4.0 * std::sqrt((2.0 * k - 1.0) / 2.0) / ((k - 1.0) * k);
  return {c * s, c * ds * t.x, c * ds * t.y};
}

// Three-variable forward-mode dual (tetrahedron basis gradients).
struct Dual3 { double v, g[3]; };
inline Dual3 d3add(Dual3 a, Dual3 b) { return {a.v + b.v, {a.g[0] + b.g[0], a.g[1] + b.g[1], a.g[2] + b.g[2]}}; }
inline Dual3 d3sub(Dual3 a, Dual3 b) { return {a.v - b.v, {a.g[0] - b.g[0], a.g[1] - b.g[1], a.g[2] - b.g[2]}}; }
inline Dual3 d3mul(Dual3 a, Dual3 b) {
  return {a.v * b.v, {a.g[0] * b.v + a.v * b.g[0], a.g[1] * b.v + a.v * b.g[1], a.g[2] * b.v + a.v * b.g[2]}};
}
inline Dual3 d3chain(Dual3 t, double f, double df) { return {f, {df * t.g[0], df * t.g[1], df * t.g[2]}}; }
inline Dual3 d3legendre(int n, Dual3 t) { double p, dp; legendreP(n, t.v, &p, &dp); return d3chain(t, p, dp); }
inline Dual3 d3kernel(int k, Dual3 t) {
  const Dual2 r = dkernel(k, {t.v, 1.0, 0.0});
  return d3chain(t, r.v, r.x);
}

inline int modalCount(int type, int p) {
  if (type == SDG_ELEMENT_LINE) return p + 1;
  if (type == SDG_ELEMENT_TRIANGLE) return (p + 1) * (p + 2) / 2;
  if (type == SDG_ELEMENT_TETRAHEDRON) return (p + 1) * (p + 2) * (p + 3) / 6;
  if (type == SDG_ELEMENT_QUADRANGLE) return (p + 1) * (p + 1);
  return (p + 1) * (p + 1) * (p + 1);
}

// Modal basis values and reference gradients at (xi, eta[, zeta]).
//   line: index a -> l_a(xi); quadrangle: index a*(P+1)+b -> l_a(xi) l_b(eta); hexahedron: (a*(P+1)+b)*(P+1)+c.
//   triangle  : lambda_0..2; edge functions lambda_a lambda_b phi_{k-2}(lambda_b - lambda_a) on edges
//               (0,1),(1,2),(2,0), k = 2..P; bubbles lambda_0 lambda_1 lambda_2 P_i(l2-l1) P_j(l1-l0), i+j <= P-3.
//   tetrahedron: lambda_0..3; edge functions on gmsh's edges (0,1),(1,2),(2,0),(3,0),(3,2),(3,1), k = 2..P;
//               face bubbles l_a l_b l_c P_i(l_c-l_b) P_j(l_b-l_a), i+j <= P-3, on the faces (a,b,c) of the
//               face vertex list; interior bubbles l0 l1 l2 l3 P_i(l1-l0) P_j(l2-l1) P_k(l3-l2), i+j+k <= P-4.
inline void modalBasisTetrahedron(int p, const double* X, double* val, double* grad) {
  const Dual3 lam[4] = {{1.0 - X[0] - X[1] - X[2], {-1.0, -1.0, -1.0}}, {X[0], {1.0, 0.0, 0.0}},
                        {X[1], {0.0, 1.0, 0.0}}, {X[2], {0.0, 0.0, 1.0}}};
  std::vector<Dual3> f(lam, lam + 4);
  const int edge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 2}, {3, 1}};
  for (const auto& e : edge)
    for (int k = 2; k <= p; ++k) f.push_back(d3mul(d3mul(lam[e[0]], lam[e[1]]), d3kernel(k, d3sub(lam[e[1]], lam[e[0]]))));
  const int face[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};
  for (const auto& t : face) {
    const Dual3 a = lam[t[0]], b = lam[t[1]], c = lam[t[2]], bub = d3mul(d3mul(a, b), c);
    for (int s = 0; s <= p - 3; ++s)
      for (int i = 0; i <= s; ++i)
        f.push_back(d3mul(d3mul(bub, d3legendre(i, d3sub(c, b))), d3legendre(s - i, d3sub(b, a))));
  }
  const Dual3 inner = d3mul(d3mul(lam[0], lam[1]), d3mul(lam[2], lam[3]));
  for (int s = 0; s <= p - 4; ++s)
    for (int i = 0; i <= s; ++i)
      for (int j = 0; j <= s - i; ++j)
        f.push_back(d3mul(d3mul(inner, d3legendre(i, d3sub(lam[1], lam[0]))),
                          d3mul(d3legendre(j, d3sub(lam[2], lam[1])), d3legendre(s - i - j, d3sub(lam[3], lam[2])))));
  for (size_t i = 0; i < f.size(); ++i) {
    val[i] = f[i].v;
    for (int d = 0; d < 3; ++d) grad[i * 3 + d] = f[i].g[d];
  }
}

inline void modalBasis(int type, int p, const double* X, double* val, double* grad /* [nb][3] */) {
  if (type == SDG_ELEMENT_TETRAHEDRON) { modalBasisTetrahedron(p, X, val, grad); return; }
  if (type != SDG_ELEMENT_TRIANGLE) {
    const int m = p + 1, dim = type == SDG_ELEMENT_HEXAHEDRON ? 3 : (type == SDG_ELEMENT_LINE ? 1 : 2);
    double lv[3][kMaxN], ld[3][kMaxN];
    for (int d = 0; d < dim; ++d)
      for (int k = 0; k < m; ++k) {
        lv[d][k] = lobatto1d(k, X[d]);
        if (k == 0) ld[d][k] = -0.5;
        else if (k == 1) ld[d][k] = 0.5;
        else { double pk1, dd; legendreP(k - 1, X[d], &pk1, &dd); ld[d][k] = std::sqrt((2.0 * k - 1.0) / 2.0) * pk1; }
      }
    int idx = 0;
    if (dim == 1) {
      for (int a = 0; a < m; ++a, ++idx) { val[idx] = lv[0][a]; grad[idx * 3] = ld[0][a]; grad[idx * 3 + 1] = grad[idx * 3 + 2] = 0; }
    } else if (dim == 2) {
      for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b, ++idx) {
          val[idx] = lv[0][a] * lv[1][b];
          grad[idx * 3] = ld[0][a] * lv[1][b]; grad[idx * 3 + 1] = lv[0][a] * ld[1][b]; grad[idx * 3 + 2] = 0;
        }
    } else {
      for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b)
          for (int c = 0; c < m; ++c, ++idx) {
            val[idx] = lv[0][a] * lv[1][b] * lv[2][c];
            grad[idx * 3] = ld[0][a] * lv[1][b] * lv[2][c];
            grad[idx * 3 + 1] = lv[0][a] * ld[1][b] * lv[2][c];
            grad[idx * 3 + 2] = lv[0][a] * lv[1][b] * ld[2][c];
          }
    }
    return;
  }
  const Dual2 l0{1.0 - X[0] - X[1], -1.0, -1.0}, l1{X[0], 1.0, 0.0}, l2{X[1], 0.0, 1.0};
  const Dual2 lam[3] = {l0, l1, l2};
  std::vector<Dual2> f = {l0, l1, l2};
  const int edge[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  for (int e = 0; e < 3; ++e) {
    const Dual2 a = lam[edge[e][0]], b = lam[edge[e][1]];
    for (int k = 2; k <= p; ++k) f.push_back(dmul(dmul(a, b), dkernel(k, dsub(b, a))));
  }
  const Dual2 bubble = dmul(dmul(l0, l1), l2);
  for (int s = 0; s <= p - 3; ++s)
    for (int i = 0; i <= s; ++i)
      f.push_back(dmul(dmul(bubble, dlegendre(i, dsub(l2, l1))), dlegendre(s - i, dsub(l1, l0))));
  for (size_t i = 0; i < f.size(); ++i) { val[i] = f[i].v; grad[i * 3] = f[i].x; grad[i * 3 + 1] = f[i].y; grad[i * 3 + 2] = 0; }
}

struct PointRule {
  int n = 0;
  std::vector<double> x, w;  // x: [n][3]
};

// Volume rule of order 2P (kTriangle/kQuadrangle/kTetrahedron/kHexahedronQuadratureNumber,
// SimulationControl.cpp:268-273).
inline PointRule volumeRule(int type, int p) {
  PointRule r;
  const int order = 2 * p;
  if (type == SDG_ELEMENT_TETRAHEDRON) {
    for (const auto& t : sdg_tables::kTetrahedronRules)
      if (t.degree == order) {
        r.n = t.count;
        for (int i = 0; i < t.count; ++i) { r.x.insert(r.x.end(), {t.xi[i], t.eta[i], t.zeta[i]}); r.w.push_back(t.weight[i]); }
        return r;
      }
    throw std::runtime_error("no tetrahedron rule of order " + std::to_string(order));
  }
  if (type == SDG_ELEMENT_TRIANGLE) {
    for (const auto& t : sdg_tables::kTriangleRules)
      if (t.degree == order) {
        r.n = t.count;
        for (int i = 0; i < t.count; ++i) { r.x.insert(r.x.end(), {t.xi[i], t.eta[i], 0.0}); r.w.push_back(t.weight[i]); }
        return r;
      }
    throw std::runtime_error("no triangle rule of order " + std::to_string(order));
  }
  if (type == SDG_ELEMENT_QUADRANGLE && p == 1) {  // 7 points (Radon's degree-5 formula)
    const double a = std::sqrt(14.0 / 15.0), b = std::sqrt(0.6), c = std::sqrt(1.0 / 3.0);
    const double pts[7][2] = {{0, 0}, {0, a}, {0, -a}, {b, c}, {-b, c}, {b, -c}, {-b, -c}};
    const double wts[7] = {8.0 / 7.0, 20.0 / 63.0, 20.0 / 63.0, 5.0 / 9.0, 5.0 / 9.0, 5.0 / 9.0, 5.0 / 9.0};
    r.n = 7;
    for (int i = 0; i < 7; ++i) { r.x.insert(r.x.end(), {pts[i][0], pts[i][1], 0.0}); r.w.push_back(wts[i]); }
    return r;
  }
  const int n = p + 1;
  double g[kMaxN], gw[kMaxN];
  gaussRule(n, g, gw);
  if (type == SDG_ELEMENT_LINE) {  // kLineQuadratureNumber[2P] = P + 1 Gauss points
    for (int i = 0; i < n; ++i) { r.x.insert(r.x.end(), {g[i], 0.0, 0.0}); r.w.push_back(gw[i]); }
  } else if (type == SDG_ELEMENT_QUADRANGLE) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) { r.x.insert(r.x.end(), {g[i], g[j], 0.0}); r.w.push_back(gw[i] * gw[j]); }
  } else {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) { r.x.insert(r.x.end(), {g[i], g[j], g[k]}); r.w.push_back(gw[i] * gw[j] * gw[k]); }
  }
  r.n = int(r.w.size());
  return r;
}

// Face rule of order 2P+1 in face coordinates: P+1 Gauss points per face direction (the point faces of a
// line: one point of weight 1).
inline PointRule faceRule(int type, int p) {
  PointRule r;
  if (type == SDG_ELEMENT_LINE) { r.n = 1; r.x = {0.0, 0.0, 0.0}; r.w = {1.0}; return r; }
  if (type == SDG_ELEMENT_TETRAHEDRON) {  // triangular faces: the rule of order 2P+1 on (0,0),(1,0),(0,1)
    for (const auto& t : sdg_tables::kFaceTriangleRules)
      if (t.degree == 2 * p + 1) {
        r.n = t.count;
        for (int i = 0; i < t.count; ++i) { r.x.insert(r.x.end(), {t.xi[i], t.eta[i], 0.0}); r.w.push_back(t.weight[i]); }
        return r;
      }
    throw std::runtime_error("no triangle face rule of order " + std::to_string(2 * p + 1));
  }
  const int n = p + 1;
  double g[kMaxN], gw[kMaxN];
  gaussRule(n, g, gw);
  if (type != SDG_ELEMENT_HEXAHEDRON) {
    for (int i = 0; i < n; ++i) { r.x.insert(r.x.end(), {g[i], 0.0, 0.0}); r.w.push_back(gw[i]); }
  } else {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) { r.x.insert(r.x.end(), {g[i], g[j], 0.0}); r.w.push_back(gw[i] * gw[j]); }
  }
  r.n = int(r.w.size());
  return r;
}

inline void referenceVertex(int type, int v, double* X) {
  static const double line[2][3] = {{-1, 0, 0}, {1, 0, 0}};
  static const double tri[3][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}};
  static const double quad[4][3] = {{-1, -1, 0}, {1, -1, 0}, {1, 1, 0}, {-1, 1, 0}};
  static const double hex[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                   {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  static const double tet[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  if (type == SDG_ELEMENT_TETRAHEDRON) { X[0] = tet[v][0]; X[1] = tet[v][1]; X[2] = tet[v][2]; return; }
  const double* s = type == SDG_ELEMENT_LINE ? line[v]
                    : (type == SDG_ELEMENT_TRIANGLE ? tri[v] : (type == SDG_ELEMENT_QUADRANGLE ? quad[v] : hex[v]));
  X[0] = s[0]; X[1] = s[1]; X[2] = s[2];
}

// Parent reference coordinates of face point fx on local face f (P1 map of the face vertex list,
// src/Mesh/BasisFunction.cpp:76-111).
void facePointInParent(int type, int f, const double* fx, double* X);

}  // namespace sdg
