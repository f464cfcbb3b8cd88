// Oracle -- test infrastructure only (the checker, never the product).
// Reference elements, quadrature and the modal basis, restated from the reference's gmsh calls:
//   quadrature  : src/Mesh/Quadrature.cpp:27-51 (gmsh "Gauss{order}"), orders from
//                 src/Solver/SimulationControl.cpp:268-283 (volume 2P, face 2P+1)
//   modal basis : src/Mesh/BasisFunction.cpp:45-74 (gmsh "H1Legendre{P}" = hierarchic Lobatto)
//   face traces : src/Mesh/BasisFunction.cpp:76-111,149-197 (P1 map of face points into the parent)
//   face tables : src/Solver/SimulationControl.cpp:170-216 (face vertex lists),
//                 src/Solver/SimulationControl.cpp:381-523 (face point permutation by rotation)
// gmsh 4.13.1 is not vendored under the reference tree, so its Lobatto normalisation, point orderings
// and triangle tables are restated from the published definitions (parity for these is unpinned
// against gmsh itself; the DG solution does not depend on the basis choice).  Tetrahedra use Keast's
// volume rules and Dunavant's odd-degree face rules (tetrahedron_rules.h, shared with the GPU host layer),
// whose point counts are the reference's kTetrahedron/kTriangleQuadratureNumber for P1..P3.
#pragma once
#include <array>
#include <limits>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "../subrosadg_gb300/csrc/tetrahedron_rules.h"
#include "../subrosadg_gb300/csrc/triangle_rules.h"

namespace orc {

#ifndef ORC_REAL
#define ORC_REAL double
#endif
// Arithmetic type of the oracle: double (the reference's Real, src/Utils/BasicDataType.cpp:35-39) or
// long double for an extended-precision truth (build flag -DORC_REAL="long double").
using Real = ORC_REAL;

enum ElemType { kLine = 1, kTri = 2, kQuad = 3, kTet = 4, kHex = 5 };

inline int elemDim(int t) { return t == kLine ? 1 : (t == kHex || t == kTet ? 3 : 2); }
inline int elemFaces(int t) { return t == kLine ? 2 : (t == kTri ? 3 : (t == kQuad || t == kTet ? 4 : 6)); }
inline int elemVerts(int t) { return t == kLine ? 2 : (t == kTri ? 3 : (t == kQuad || t == kTet ? 4 : 8)); }
inline int faceVerts(int t) { return t == kLine ? 1 : (t == kHex ? 4 : (t == kTet ? 3 : 2)); }

// Face vertex lists of each element type (SimulationControl.cpp:170-216).
inline const int* faceVertexTable(int t) {
  static const int line[] = {0, 1};
  static const int tri[] = {0, 1, 1, 2, 2, 0};
  static const int quad[] = {0, 1, 1, 2, 2, 3, 3, 0};
  static const int hex[] = {0, 3, 2, 1, 0, 1, 5, 4, 0, 4, 7, 3, 1, 2, 6, 5, 2, 3, 7, 6, 4, 5, 6, 7};
  static const int tet[] = {0, 2, 1, 0, 1, 3, 0, 3, 2, 3, 1, 2};
  return t == kLine ? line : (t == kTri ? tri : (t == kQuad ? quad : (t == kTet ? tet : hex)));
}

// Reference-element vertex coordinates (gmsh conventions).
inline std::array<Real, 3> refVertex(int t, int v) {
  static const Real line[2][3] = {{-1, 0, 0}, {1, 0, 0}};
  static const Real tri[3][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}};
  static const Real quad[4][3] = {{-1, -1, 0}, {1, -1, 0}, {1, 1, 0}, {-1, 1, 0}};
  static const Real hex[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                   {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  static const Real tet[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const Real* p = t == kLine ? line[v] : (t == kTri ? tri[v] : (t == kQuad ? quad[v] : (t == kTet ? tet[v] : hex[v])));
  return {p[0], p[1], p[2]};
}

// Legendre P_n and P'_n by the three-term recurrence.
inline void legendre(int n, Real x, Real& p, Real& dp) {
  Real p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (n == 0) { p = 1.0; dp = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    const Real p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    const Real d2 = d0 + (2.0 * k - 1.0) * p1;
    p0 = p1; p1 = p2; d0 = d1; d1 = d2;
  }
  p = p1; dp = d1;
}

// n-point Gauss-Legendre rule on [-1,1], points ascending (Newton on P_n).
inline void gaussLegendre(int n, std::vector<Real>& x, std::vector<Real>& w) {
  x.assign(n, 0.0); w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    Real z = -std::cos(Real(M_PI) * (i + Real(0.75)) / (n + Real(0.5)));
    for (int it = 0; it < 100; ++it) {
      Real p, dp; legendre(n, z, p, dp);
      const Real dz = p / dp; z -= dz;
      if (std::fabs(dz) <= 4 * std::numeric_limits<Real>::epsilon()) break;
    }
    Real p, dp; legendre(n, z, p, dp);
    x[i] = z; w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Line rule for a polynomial order (Gauss, ceil((order+1)/2) points; counts match
// kLineQuadratureNumber, SimulationControl.cpp:268).
inline int linePoints(int order) { return order / 2 + 1; }

struct Quadrature {
  int dim = 0, n = 0;
  std::vector<Real> x;  // n * 3 reference coordinates
  std::vector<Real> w;  // n
};

// Element quadrature of the given order for each element type.
inline Quadrature elementQuadrature(int t, int order) {
  Quadrature q; q.dim = elemDim(t);
  if (t == kTet) {  // Keast's symmetric rules of degree 2, 4, 6 (4 / 11 / 24 points, kTetrahedronQuadratureNumber)
    for (const auto& r : sdg_tables::kTetrahedronRules) {
      if (r.degree == order) {
        q.n = r.count;
        for (int i = 0; i < r.count; ++i) { q.x.insert(q.x.end(), {r.xi[i], r.eta[i], r.zeta[i]}); q.w.push_back(r.weight[i]); }
        return q;
      }
    }
    throw std::runtime_error("no tetrahedron rule of order " + std::to_string(order));
  }
  if (t == kTri) {
    for (const auto& r : sdg_tables::kTriangleRules) {
      if (r.degree == order) {
        q.n = r.count;
        for (int i = 0; i < r.count; ++i) { q.x.insert(q.x.end(), {r.xi[i], r.eta[i], 0.0}); q.w.push_back(r.weight[i]); }
        return q;
      }
    }
    throw std::runtime_error("no triangle rule of order " + std::to_string(order));
  }
  if (t == kQuad && order == 2) {
    // 7-point degree-5 rule (kQuadrangleQuadratureNumber[2] = 7): Radon's symmetric formula.
    const Real a = std::sqrt(14.0 / 15.0), b = std::sqrt(3.0 / 5.0), c = std::sqrt(1.0 / 3.0);
    const Real pts[7][2] = {{0, 0}, {0, a}, {0, -a}, {b, c}, {-b, c}, {b, -c}, {-b, -c}};
    const Real wts[7] = {8.0 / 7.0, 20.0 / 63.0, 20.0 / 63.0, 5.0 / 9.0, 5.0 / 9.0, 5.0 / 9.0, 5.0 / 9.0};
    q.n = 7;
    for (int i = 0; i < 7; ++i) { q.x.insert(q.x.end(), {pts[i][0], pts[i][1], 0.0}); q.w.push_back(wts[i]); }
    return q;
  }
  const int m = linePoints(order);
  std::vector<Real> gx, gw; gaussLegendre(m, gx, gw);
  if (t == kLine) {
    q.n = m;
    for (int i = 0; i < m; ++i) { q.x.insert(q.x.end(), {gx[i], 0.0, 0.0}); q.w.push_back(gw[i]); }
  } else if (t == kQuad) {  // index = i*m + j with (xi=x_i, eta=x_j)
    q.n = m * m;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) { q.x.insert(q.x.end(), {gx[i], gx[j], 0.0}); q.w.push_back(gw[i] * gw[j]); }
  } else {  // hex: index = (i*m + j)*m + k
    q.n = m * m * m;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j)
        for (int k = 0; k < m; ++k) {
          q.x.insert(q.x.end(), {gx[i], gx[j], gx[k]});
          q.w.push_back(gw[i] * gw[j] * gw[k]);
        }
  }
  return q;
}

// Face rule (face reference coordinates: line xi in [-1,1]; quad face (xi,eta) in [-1,1]^2,
// index i*m + j with (xi=x_i, eta=x_j)).
inline Quadrature faceQuadrature(int t, int order) {
  Quadrature q; q.dim = elemDim(t) - 1;
  if (t == kLine) {  // point faces: one point of weight 1 (kPoint rules, SimulationControl.cpp:287-289)
    q.n = 1; q.x = {0.0, 0.0, 0.0}; q.w = {1.0};
    return q;
  }
  if (t == kTet) {  // triangular faces: Dunavant's odd-degree rules on (0,0),(1,0),(0,1)
    for (const auto& r : sdg_tables::kFaceTriangleRules) {
      if (r.degree == order) {
        q.n = r.count;
        for (int i = 0; i < r.count; ++i) { q.x.insert(q.x.end(), {r.xi[i], r.eta[i], 0.0}); q.w.push_back(r.weight[i]); }
        return q;
      }
    }
    throw std::runtime_error("no triangle face rule of order " + std::to_string(order));
  }
  const int m = linePoints(order);
  std::vector<Real> gx, gw; gaussLegendre(m, gx, gw);
  if (t != kHex) {
    q.n = m;
    for (int i = 0; i < m; ++i) { q.x.insert(q.x.end(), {gx[i], 0.0, 0.0}); q.w.push_back(gw[i]); }
  } else {
    q.n = m * m;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) { q.x.insert(q.x.end(), {gx[i], gx[j], 0.0}); q.w.push_back(gw[i] * gw[j]); }
  }
  return q;
}

// P1 shape functions of the face reference element (BasisFunction.cpp:76-111 uses gmsh Lagrange1).
inline void faceShape(int t, const Real* fx, Real* n) {
  if (t == kLine) { n[0] = 1.0; return; }
  if (t == kTet) { n[0] = 1 - fx[0] - fx[1]; n[1] = fx[0]; n[2] = fx[1]; return; }
  if (t != kHex) { n[0] = 0.5 * (1.0 - fx[0]); n[1] = 0.5 * (1.0 + fx[0]); return; }
  const Real x = fx[0], y = fx[1];
  n[0] = 0.25 * (1 - x) * (1 - y); n[1] = 0.25 * (1 + x) * (1 - y);
  n[2] = 0.25 * (1 + x) * (1 + y); n[3] = 0.25 * (1 - x) * (1 + y);
}
inline void faceShapeGrad(int t, const Real* fx, Real* dxi, Real* deta) {
  if (t == kLine) { dxi[0] = 0.0; return; }
  if (t == kTet) { dxi[0] = -1; dxi[1] = 1; dxi[2] = 0; deta[0] = -1; deta[1] = 0; deta[2] = 1; return; }
  if (t != kHex) { dxi[0] = -0.5; dxi[1] = 0.5; return; }
  const Real x = fx[0], y = fx[1];
  dxi[0] = -0.25 * (1 - y); dxi[1] = 0.25 * (1 - y); dxi[2] = 0.25 * (1 + y); dxi[3] = -0.25 * (1 + y);
  deta[0] = -0.25 * (1 - x); deta[1] = -0.25 * (1 + x); deta[2] = 0.25 * (1 + x); deta[3] = 0.25 * (1 - x);
}

// P1 element shape functions and reference gradients (geometry map of straight-sided elements).
inline void elemShape(int t, const Real* X, Real* n, Real* g /* nv*3 */) {
  if (t == kLine) {
    n[0] = 0.5 * (1 - X[0]); n[1] = 0.5 * (1 + X[0]);
    const Real gg[6] = {-0.5, 0, 0, 0.5, 0, 0};
    for (int i = 0; i < 6; ++i) g[i] = gg[i];
    return;
  }
  if (t == kTri) {
    n[0] = 1 - X[0] - X[1]; n[1] = X[0]; n[2] = X[1];
    const Real gg[9] = {-1, -1, 0, 1, 0, 0, 0, 1, 0};
    for (int i = 0; i < 9; ++i) g[i] = gg[i];
    return;
  }
  if (t == kTet) {
    n[0] = 1 - X[0] - X[1] - X[2]; n[1] = X[0]; n[2] = X[1]; n[3] = X[2];
    const Real gg[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < 12; ++i) g[i] = gg[i];
    return;
  }
  const int nv = elemVerts(t);
  for (int v = 0; v < nv; ++v) {
    const auto r = refVertex(t, v);
    const Real a = 1 + r[0] * X[0], b = 1 + r[1] * X[1];
    if (t == kQuad) {
      n[v] = 0.25 * a * b; g[v * 3 + 0] = 0.25 * r[0] * b; g[v * 3 + 1] = 0.25 * a * r[1]; g[v * 3 + 2] = 0;
    } else {
      const Real c = 1 + r[2] * X[2];
      n[v] = 0.125 * a * b * c;
      g[v * 3 + 0] = 0.125 * r[0] * b * c; g[v * 3 + 1] = 0.125 * a * r[1] * c; g[v * 3 + 2] = 0.125 * a * b * r[2];
    }
  }
}

// 1D Lobatto shape functions (Solin): l0=(1-x)/2, l1=(1+x)/2, lk=(P_k-P_{k-2})/sqrt(2(2k-1)).
inline void lobatto(int k, Real x, Real& v, Real& d) {
  if (k == 0) { v = 0.5 * (1 - x); d = -0.5; return; }
  if (k == 1) { v = 0.5 * (1 + x); d = 0.5; return; }
  Real pk, dpk, pk2, dpk2, pk1, dpk1;
  legendre(k, x, pk, dpk); legendre(k - 2, x, pk2, dpk2); legendre(k - 1, x, pk1, dpk1);
  const Real s = std::sqrt(2.0 * (2.0 * k - 1.0));
  v = (pk - pk2) / s;
  d = std::sqrt((2.0 * k - 1.0) / 2.0) * pk1;
}

// Tiny forward-mode dual number in two variables (for triangle basis gradients).
struct Dual { Real v, dx, dy; };
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.dx + b.dx, a.dy + b.dy}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.dx - b.dx, a.dy - b.dy}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.dx * b.v + a.v * b.dx, a.dy * b.v + a.v * b.dy}; }
inline Dual scale(Dual a, Real s) { return {a.v * s, a.dx * s, a.dy * s}; }
inline Dual legendreD(int n, Dual x) {  // P_n(x) as a dual
  Real p, dp; legendre(n, x.v, p, dp);
  return {p, dp * x.dx, dp * x.dy};
}
// Solin kernel function phi_{k-2}(x) = 4 l_k(x)/(1-x^2) = -4 sqrt((2k-1)/2)/((k-1)k) P'_{k-1}(x).
inline Dual kernelD(int k, Dual x) {
  // P'_{k-1}(x) and its derivative P''_{k-1}(x) via (1-x^2)P'' = 2xP' - n(n+1)P is singular at
  // |x|=1; use the sum form P'_{n} = sum_{j=n-1,n-3,..} (2j+1) P_j instead.
  const int n = k - 1;
  Real dpn = 0.0, ddpn = 0.0;
  for (int j = n - 1; j >= 0; j -= 2) {
    Real pj, dpj; legendre(j, x.v, pj, dpj);
    dpn += (2.0 * j + 1.0) * pj; ddpn += (2.0 * j + 1.0) * dpj;
  }
  const Real c = -4.0 * std::sqrt((2.0 * k - 1.0) / 2.0) / ((k - 1.0) * k);
  return {c * dpn, c * ddpn * x.dx, c * ddpn * x.dy};
}

// Forward-mode dual in three variables (tetrahedron basis gradients).
struct Dual3 { Real v, d[3]; };
inline Dual3 operator+(Dual3 a, Dual3 b) { return {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}}; }
inline Dual3 operator-(Dual3 a, Dual3 b) { return {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}}; }
inline Dual3 operator*(Dual3 a, Dual3 b) {
  Dual3 r{a.v * b.v, {0, 0, 0}};
  for (int k = 0; k < 3; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
// f(x) for a scalar function with value fv and derivative fd at x.v
inline Dual3 lift3(Dual3 x, Real fv, Real fd) { return {fv, {fd * x.d[0], fd * x.d[1], fd * x.d[2]}}; }
inline Dual3 legendre3(int n, Dual3 x) { Real p, dp; legendre(n, x.v, p, dp); return lift3(x, p, dp); }
inline Dual3 kernel3(int k, Dual3 x) { const Dual r = kernelD(k, Dual{x.v, 1, 0}); return lift3(x, r.v, r.dx); }

inline int basisCount(int t, int p) {
  if (t == kLine) return p + 1;
  if (t == kTri) return (p + 1) * (p + 2) / 2;
  if (t == kTet) return (p + 1) * (p + 2) * (p + 3) / 6;
  if (t == kQuad) return (p + 1) * (p + 1);
  return (p + 1) * (p + 1) * (p + 1);
}

// Modal (hierarchic H1) basis: values [nb] and reference gradients [nb][3] at X.
//   line: index a -> l_a(xi); quad: index a*(P+1)+b -> l_a(xi) l_b(eta); hex: index (a*(P+1)+b)*(P+1)+c.
//   tri : vertices lambda_i; edges (0,1),(1,2),(2,0) with l_a l_b phi_{k-2}(l_b-l_a), k=2..P;
//         bubbles l0 l1 l2 P_i(l2-l1) P_j(l1-l0), i+j<=P-3.
//   tet : vertices lambda_i; edges (0,1),(1,2),(2,0),(3,0),(3,2),(3,1) (gmsh's edge order) with
//         l_a l_b phi_{k-2}(l_b-l_a); face bubbles l_a l_b l_c P_i(l_c-l_b) P_j(l_b-l_a), i+j<=P-3, on the faces
//         (a,b,c) of the face vertex table; interior l0 l1 l2 l3 P_i(l1-l0) P_j(l2-l1) P_k(l3-l2), i+j+k<=P-4.
inline void modalBasis(int t, int p, const Real* X, Real* val, Real* grad) {
  if (t == kTet) {
    const Dual3 l[4] = {{1 - X[0] - X[1] - X[2], {-1, -1, -1}}, {X[0], {1, 0, 0}}, {X[1], {0, 1, 0}}, {X[2], {0, 0, 1}}};
    std::vector<Dual3> f(l, l + 4);
    const int edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 2}, {3, 1}};
    for (const auto& e : edges)
      for (int k = 2; k <= p; ++k) f.push_back(l[e[0]] * l[e[1]] * kernel3(k, l[e[1]] - l[e[0]]));
    const int* fv = faceVertexTable(kTet);
    for (int fc = 0; fc < 4; ++fc) {
      const Dual3 a = l[fv[fc * 3]], b = l[fv[fc * 3 + 1]], c = l[fv[fc * 3 + 2]];
      for (int s = 0; s <= p - 3; ++s)
        for (int i = 0; i <= s; ++i) f.push_back(a * b * c * legendre3(i, c - b) * legendre3(s - i, b - a));
    }
    for (int s = 0; s <= p - 4; ++s)
      for (int i = 0; i <= s; ++i)
        for (int j = 0; j <= s - i; ++j)
          f.push_back(l[0] * l[1] * l[2] * l[3] * legendre3(i, l[1] - l[0]) * legendre3(j, l[2] - l[1]) *
                      legendre3(s - i - j, l[3] - l[2]));
    for (size_t i = 0; i < f.size(); ++i) { val[i] = f[i].v; for (int k = 0; k < 3; ++k) grad[i * 3 + k] = f[i].d[k]; }
    return;
  }
  if (t == kLine) {
    for (int a = 0; a <= p; ++a) {
      Real v, d; lobatto(a, X[0], v, d);
      val[a] = v; grad[a * 3 + 0] = d; grad[a * 3 + 1] = 0; grad[a * 3 + 2] = 0;
    }
    return;
  }
  if (t == kQuad || t == kHex) {
    const int m = p + 1;
    Real lv[3][6], ld[3][6];
    for (int dd = 0; dd < elemDim(t); ++dd)
      for (int k = 0; k < m; ++k) lobatto(k, X[dd], lv[dd][k], ld[dd][k]);
    int idx = 0;
    if (t == kQuad) {
      for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b, ++idx) {
          val[idx] = lv[0][a] * lv[1][b];
          grad[idx * 3 + 0] = ld[0][a] * lv[1][b]; grad[idx * 3 + 1] = lv[0][a] * ld[1][b]; grad[idx * 3 + 2] = 0;
        }
    } else {
      for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b)
          for (int c = 0; c < m; ++c, ++idx) {
            val[idx] = lv[0][a] * lv[1][b] * lv[2][c];
            grad[idx * 3 + 0] = ld[0][a] * lv[1][b] * lv[2][c];
            grad[idx * 3 + 1] = lv[0][a] * ld[1][b] * lv[2][c];
            grad[idx * 3 + 2] = lv[0][a] * lv[1][b] * ld[2][c];
          }
    }
    return;
  }
  const Dual l0{1 - X[0] - X[1], -1, -1}, l1{X[0], 1, 0}, l2{X[1], 0, 1};
  const Dual lam[3] = {l0, l1, l2};
  std::vector<Dual> f;
  f.push_back(l0); f.push_back(l1); f.push_back(l2);
  const int edges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  for (int e = 0; e < 3; ++e) {
    const Dual a = lam[edges[e][0]], b = lam[edges[e][1]];
    for (int k = 2; k <= p; ++k) f.push_back(a * b * kernelD(k, b - a));
  }
  const Dual bub = l0 * l1 * l2;
  for (int s = 0; s <= p - 3; ++s)
    for (int i = 0; i <= s; ++i) {
      const int j = s - i;
      f.push_back(bub * legendreD(i, l2 - l1) * legendreD(j, l1 - l0));
    }
  for (size_t i = 0; i < f.size(); ++i) { val[i] = f[i].v; grad[i * 3 + 0] = f[i].dx; grad[i * 3 + 1] = f[i].dy; grad[i * 3 + 2] = 0; }
}

// Face point permutation for a right element with the given rotation
// (reproduces the tables of SimulationControl.cpp:381-523 from the orientation rule:
//  line faces are traversed in reverse; quadrangle faces map (xi,eta) of the left face to
//  rotation 0:(eta,xi) 1:(-xi,eta) 2:(-eta,-xi) 3:(xi,-eta) on the right face).
//  Triangular faces: the right face lists the shared vertices in the opposite orientation with the left
//  face's first vertex at position `rotation`; in barycentric terms left (xi,eta) is right
//  0:(eta,xi) 1:(1-xi-eta,eta) 2:(xi,1-xi-eta), matched against the face rule's own points.
inline std::vector<int> facePermutation(int t, int m, int rotation) {
  std::vector<int> perm;
  if (t == kTet) {
    const Quadrature fq = faceQuadrature(kTet, m);
    for (int j = 0; j < fq.n; ++j) {
      const Real x = fq.x[j * 3], y = fq.x[j * 3 + 1];
      const Real X = rotation == 0 ? y : (rotation == 1 ? 1 - x - y : x);
      const Real Y = rotation == 0 ? x : (rotation == 1 ? y : 1 - x - y);
      int hit = -1;
      for (int k = 0; k < fq.n; ++k)
        if (std::fabs(fq.x[k * 3] - X) < 1e-12 && std::fabs(fq.x[k * 3 + 1] - Y) < 1e-12) hit = k;
      if (hit < 0) throw std::runtime_error("asymmetric triangle face rule");
      perm.push_back(hit);
    }
    return perm;
  }
  if (t != kHex) { for (int j = 0; j < m; ++j) perm.push_back(m - 1 - j); return perm; }
  for (int i = 0; i < m; ++i)
    for (int k = 0; k < m; ++k) {
      int ii = 0, kk = 0;
      switch (rotation) {
        case 0: ii = k; kk = i; break;
        case 1: ii = m - 1 - i; kk = k; break;
        case 2: ii = m - 1 - k; kk = m - 1 - i; break;
        default: ii = i; kk = m - 1 - k; break;
      }
      perm.push_back(ii * m + kk);
    }
  return perm;
}

// Dense square inverse by Gauss-Jordan with partial pivoting (Eigen's inverse() in the reference).
inline void invert(int n, const Real* a, Real* inv) {
  std::vector<Real> m(a, a + n * n);
  for (int i = 0; i < n * n; ++i) inv[i] = 0.0;
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c; Real best = std::fabs(m[c * n + c]);
    for (int r = c + 1; r < n; ++r) if (std::fabs(m[r * n + c]) > best) { best = std::fabs(m[r * n + c]); piv = r; }
    if (best == 0.0) throw std::runtime_error("singular matrix");
    if (piv != c) for (int k = 0; k < n; ++k) { std::swap(m[c * n + k], m[piv * n + k]); std::swap(inv[c * n + k], inv[piv * n + k]); }
    const Real d = 1.0 / m[c * n + c];
    for (int k = 0; k < n; ++k) { m[c * n + k] *= d; inv[c * n + k] *= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const Real f = m[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) { m[r * n + k] -= f * m[c * n + k]; inv[r * n + k] -= f * inv[c * n + k]; }
    }
  }
}

// ---- curved (high-order) 2D geometry ------------------------------------------------------------------
// gmsh's node order of an order-q Lagrange triangle or quadrangle, restated from its convention: the corners,
// then the q-1 interior points of each edge (corner k to corner k+1), then the interior nodes as the element of
// order q-2 (quadrangle) or q-3 (triangle) whose corners sit one lattice step inside each corner, recursively.
// Reference positions are built ring by ring from the corners (not from lattice indices).
inline std::vector<std::array<Real, 2>> gmshNodePositions(int t, int q) {
  std::vector<std::array<Real, 2>> out;
  std::vector<std::array<Real, 2>> c;
  if (t == kQuad) c = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  else c = {{0, 0}, {1, 0}, {0, 1}};
  const int nc = int(c.size()), shrink = t == kQuad ? 2 : 3;
  int r = q;
  while (r >= 0) {
    if (r == 0) {  // a single node: the centre of the remaining ring
      std::array<Real, 2> m = {0, 0};
      for (const auto& p : c) { m[0] += p[0] / nc; m[1] += p[1] / nc; }
      out.push_back(m);
      break;
    }
    for (const auto& p : c) out.push_back(p);
    for (int k = 0; k < nc; ++k) {
      const auto& a = c[k];
      const auto& b = c[(k + 1) % nc];
      for (int i = 1; i < r; ++i) out.push_back({a[0] + (b[0] - a[0]) * i / r, a[1] + (b[1] - a[1]) * i / r});
    }
    if (r - shrink < 0) break;
    // inner corners: one lattice step along both edges adjacent to each corner
    std::vector<std::array<Real, 2>> inner(c.size());
    const Real f = Real(1) / Real(r);
    for (int k = 0; k < nc; ++k) {
      const auto& p = c[k];
      const auto& nx = c[(k + 1) % nc];
      const auto& pv = c[(k + nc - 1) % nc];
      inner[k] = {p[0] + (nx[0] - p[0]) * f + (pv[0] - p[0]) * f, p[1] + (nx[1] - p[1]) * f + (pv[1] - p[1]) * f};
    }
    c = inner;
    r -= shrink;
  }
  return out;
}

// Hexahedron ([-1,1]^3, gmsh corner order: z = -1 counter-clockwise from (-1,-1), then z = +1): the 8 corners,
// the q-1 interior points of each edge of gmsh's edge table in edge direction, each face's interior nodes in
// gmsh's face order as the quadrangle construction above on the face's inner corners (one lattice step in
// from each face corner along the face's two edges), then the interior as a hexahedron on the inner corners
// (one lattice step along each of a corner's three edges), recursively.  Positions are built from corner
// points, not lattice indices.
inline std::vector<std::array<Real, 3>> gmshHexNodePositions(int q) {
  static const int edges[12][2] = {{0, 1}, {0, 3}, {0, 4}, {1, 2}, {1, 5}, {2, 3},
                                   {2, 6}, {3, 7}, {4, 5}, {4, 7}, {5, 6}, {6, 7}};
  static const int faces[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {0, 4, 7, 3}, {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};
  static const int nbr[8][3] = {{1, 3, 4}, {0, 2, 5}, {1, 3, 6}, {0, 2, 7}, {0, 5, 7}, {1, 4, 6}, {2, 5, 7}, {3, 4, 6}};
  using P3 = std::array<Real, 3>;
  const auto lerp = [](const P3& a, const P3& b, Real t) {
    return P3{a[0] + (b[0] - a[0]) * t, a[1] + (b[1] - a[1]) * t, a[2] + (b[2] - a[2]) * t};
  };
  // the quadrangle construction on four 3D corners (the order of gmshNodePositions for kQuad)
  const auto quad = [&](std::array<P3, 4> c, int r, std::vector<P3>& out) {
    while (r >= 0) {
      if (r == 0) {
        P3 m = {0, 0, 0};
        for (const auto& p : c) for (int d = 0; d < 3; ++d) m[d] += p[d] / 4;
        out.push_back(m);
        return;
      }
      for (const auto& p : c) out.push_back(p);
      for (int k = 0; k < 4; ++k)
        for (int i = 1; i < r; ++i) out.push_back(lerp(c[k], c[(k + 1) % 4], Real(i) / Real(r)));
      if (r - 2 < 0) return;
      std::array<P3, 4> in;
      for (int k = 0; k < 4; ++k) {
        const P3& p = c[k];
        const P3& nx = c[(k + 1) % 4];
        const P3& pv = c[(k + 3) % 4];
        for (int d = 0; d < 3; ++d) in[k][d] = p[d] + (nx[d] - p[d]) / r + (pv[d] - p[d]) / r;
      }
      c = in;
      r -= 2;
    }
  };
  std::vector<P3> out;
  std::array<P3, 8> c = {P3{-1, -1, -1}, P3{1, -1, -1}, P3{1, 1, -1}, P3{-1, 1, -1},
                         P3{-1, -1, 1},  P3{1, -1, 1},  P3{1, 1, 1},  P3{-1, 1, 1}};
  int r = q;
  while (r >= 0) {
    if (r == 0) {
      P3 m = {0, 0, 0};
      for (const auto& p : c) for (int d = 0; d < 3; ++d) m[d] += p[d] / 8;
      out.push_back(m);
      break;
    }
    for (const auto& p : c) out.push_back(p);
    for (const auto& e : edges)
      for (int i = 1; i < r; ++i) out.push_back(lerp(c[e[0]], c[e[1]], Real(i) / Real(r)));
    if (r - 2 < 0) break;
    for (const auto& f : faces) {
      std::array<P3, 4> fc;
      for (int k = 0; k < 4; ++k) {
        const P3& p = c[f[k]];
        const P3& nx = c[f[(k + 1) % 4]];
        const P3& pv = c[f[(k + 3) % 4]];
        for (int d = 0; d < 3; ++d) fc[k][d] = p[d] + (nx[d] - p[d]) / r + (pv[d] - p[d]) / r;
      }
      quad(fc, r - 2, out);
    }
    std::array<P3, 8> in;
    for (int k = 0; k < 8; ++k)
      for (int d = 0; d < 3; ++d) {
        Real v = c[k][d];
        for (int a = 0; a < 3; ++a) v += (c[nbr[k][a]][d] - c[k][d]) / r;
        in[k][d] = v;
      }
    c = in;
    r -= 2;
  }
  return out;
}

// Lagrange basis through the gmsh-ordered nodes.  Quadrangles and triangles: the inverse Vandermonde matrix of
// the monomials x^a y^b (a, b <= q on quadrangles, a + b <= q on triangles): N_n(X) = sum_m C[m][n] mono_m(X).
// Hexahedra: products L_i(x) L_j(y) L_k(z) of the 1D Lagrange polynomials through the q+1 equispaced
// coordinates (each from the inverse 1D Vandermonde matrix), (i, j, k) the node's coordinate indices.
struct CurvedBasis {
  int t = 0, q = 1, nn = 0;
  std::vector<std::array<int, 3>> mono;  // monomial exponents (2D), or the node's coordinate indices (hexahedra)
  std::vector<Real> C;  // 2D: [nn][nn], C[m * nn + n]; hexahedra: the 1D [q+1][q+1], C1[a * (q+1) + i]
  void init(int type, int order) {
    t = type; q = order;
    mono.clear();
    if (type == kHex) {
      const auto pos = gmshHexNodePositions(order);
      nn = int(pos.size());
      for (const auto& p : pos) {
        std::array<int, 3> ijk;
        for (int d = 0; d < 3; ++d) ijk[d] = int(std::lround(double((p[d] + 1) * q / 2)));
        mono.push_back(ijk);
      }
      std::vector<Real> V(size_t(q + 1) * (q + 1));
      for (int i = 0; i <= q; ++i)
        for (int a = 0; a <= q; ++a) V[size_t(i) * (q + 1) + a] = ipow(Real(-1) + Real(2 * i) / Real(q), a);
      C.assign(size_t(q + 1) * (q + 1), 0);
      invert(q + 1, V.data(), C.data());
      return;
    }
    const auto pos = gmshNodePositions(type, order);
    nn = int(pos.size());
    for (int a = 0; a <= q; ++a)
      for (int b = 0; b <= q; ++b)
        if (type == kQuad || a + b <= q) mono.push_back({a, b, 0});
    std::vector<Real> V(size_t(nn) * nn);
    for (int n = 0; n < nn; ++n)
      for (int m = 0; m < nn; ++m) V[size_t(n) * nn + m] = ipow(pos[n][0], mono[m][0]) * ipow(pos[n][1], mono[m][1]);
    C.assign(size_t(nn) * nn, 0);
    invert(nn, V.data(), C.data());
  }
  static Real ipow(Real x, int k) { Real r = 1; for (int i = 0; i < k; ++i) r *= x; return r; }
  // the 1D Lagrange polynomial i at x and its derivative (hexahedra)
  void lagrange(int i, Real x, Real& v, Real& d) const {
    v = 0; d = 0;
    for (int a = 0; a <= q; ++a) {
      const Real c = C[size_t(a) * (q + 1) + i];
      v += c * ipow(x, a);
      if (a) d += c * a * ipow(x, a - 1);
    }
  }
  // N[n], G[n][3] at X
  void eval(const Real* X, Real* N, Real* G) const {
    if (t == kHex) {
      for (int n = 0; n < nn; ++n) {
        Real v[3], d[3];
        for (int k = 0; k < 3; ++k) lagrange(mono[n][k], X[k], v[k], d[k]);
        N[n] = v[0] * v[1] * v[2];
        G[n * 3] = d[0] * v[1] * v[2]; G[n * 3 + 1] = v[0] * d[1] * v[2]; G[n * 3 + 2] = v[0] * v[1] * d[2];
      }
      return;
    }
    std::vector<Real> mv(nn), mx(nn), my(nn);
    for (int m = 0; m < nn; ++m) {
      const int a = mono[m][0], b = mono[m][1];
      mv[m] = ipow(X[0], a) * ipow(X[1], b);
      mx[m] = a ? a * ipow(X[0], a - 1) * ipow(X[1], b) : 0;
      my[m] = b ? b * ipow(X[0], a) * ipow(X[1], b - 1) : 0;
    }
    for (int n = 0; n < nn; ++n) {
      Real v = 0, gx = 0, gy = 0;
      for (int m = 0; m < nn; ++m) {
        const Real cc = C[size_t(m) * nn + n];
        v += cc * mv[m]; gx += cc * mx[m]; gy += cc * my[m];
      }
      N[n] = v; G[n * 3] = gx; G[n * 3 + 1] = gy; G[n * 3 + 2] = 0;
    }
  }
};

// Reference-element operator tables for one (type, P) (ElementBasisFunction, BasisFunction.cpp:136-230).
struct RefElement {
  int type = 0, dim = 0, p = 0, nb = 0, nq = 0, nface = 0, nfq = 0;
  Quadrature vq, fq;
  std::vector<Real> phi;    // [nq][nb]        modal_value_
  std::vector<Real> dphi;   // [nq*dim][nb]    modal_gradient_value_ (row q*dim+k)
  std::vector<Real> phif;   // [nface*nfq][nb] modal_adjacency_value_
  std::vector<Real> lsqInv; // [nb][nb]        modal_least_squares_inverse_
  std::vector<Real> ptp;    // [nb][nb]        Phi^T Phi
  std::vector<std::vector<int>> perm;  // rotation -> face point permutation
  // artificial viscosity: first-order nodal basis at the volume and face points (BasisFunction.cpp:138-140,
  // 177,205: nodal_value_, nodal_adjacency_value_) and the modes of degree P (the sensor's high-order part)
  int nvert = 0;
  std::vector<Real> nodal;   // [nq][nvert]
  std::vector<Real> nodalf;  // [nface*nfq][nvert]
  std::vector<int> high;     // [nb] 1 for the modes of degree P

  void build(int t, int order) {
    type = t; dim = elemDim(t); p = order; nb = basisCount(t, order); nface = elemFaces(t);
    vq = elementQuadrature(t, 2 * order);
    fq = faceQuadrature(t, 2 * order + 1);
    nq = vq.n; nfq = fq.n;
    phi.assign(size_t(nq) * nb, 0); dphi.assign(size_t(nq) * dim * nb, 0);
    std::vector<Real> v(nb), g(nb * 3);
    for (int q = 0; q < nq; ++q) {
      modalBasis(t, order, &vq.x[q * 3], v.data(), g.data());
      for (int b = 0; b < nb; ++b) {
        phi[size_t(q) * nb + b] = v[b];
        for (int k = 0; k < dim; ++k) dphi[(size_t(q) * dim + k) * nb + b] = g[b * 3 + k];
      }
    }
    phif.assign(size_t(nface) * nfq * nb, 0);
    const int* fv = faceVertexTable(t);
    const int nfv = faceVerts(t);
    for (int f = 0; f < nface; ++f)
      for (int j = 0; j < nfq; ++j) {
        Real sh[4]; faceShape(t, &fq.x[j * 3], sh);
        Real X[3] = {0, 0, 0};
        for (int k = 0; k < nfv; ++k) {
          const auto r = refVertex(t, fv[f * nfv + k]);
          for (int d = 0; d < 3; ++d) X[d] += sh[k] * r[d];
        }
        modalBasis(t, order, X, v.data(), g.data());
        for (int b = 0; b < nb; ++b) phif[(size_t(f) * nfq + j) * nb + b] = v[b];
        Real sh8[8], g8[24];
        elemShape(t, X, sh8, g8);
        nodalf.resize(size_t(nface) * nfq * elemVerts(t));
        for (int k = 0; k < elemVerts(t); ++k) nodalf[(size_t(f) * nfq + j) * elemVerts(t) + k] = sh8[k];
      }
    nvert = elemVerts(t);
    nodal.assign(size_t(nq) * nvert, 0);
    for (int q = 0; q < nq; ++q) {
      Real sh8[8], g8[24];
      elemShape(t, &vq.x[q * 3], sh8, g8);
      for (int k = 0; k < nvert; ++k) nodal[size_t(q) * nvert + k] = sh8[k];
    }
    // degree of each mode: tensor blocks max(a, b[, c]) of the Lobatto indices (l_0, l_1 linear, l_k of
    // degree k); triangles: vertices 1, edge modes k, bubbles i + j + 3
    high.assign(nb, 0);
    for (int b = 0; b < nb; ++b) {
      int deg = 0;
      if (t == kLine || t == kQuad || t == kHex) {
        int r = b;
        for (int dd = 0; dd < dim; ++dd) { deg = std::max(deg, std::max(1, r % (order + 1))); r /= order + 1; }
      } else if (t == kTet) {  // vertices, then 6 edges x (P-1), 4 faces x (P-1)(P-2)/2, then the interior
        const int ne = 6 * (order - 1), nfm = (order - 1) * (order - 2) / 2;
        if (b < 4) {
          deg = 1;
        } else if (b < 4 + ne) {
          deg = 2 + (b - 4) % (order - 1);
        } else if (b < 4 + ne + 4 * nfm) {
          int idx = (b - 4 - ne) % nfm, sdeg = 0;
          while (idx > sdeg) { idx -= sdeg + 1; ++sdeg; }
          deg = sdeg + 3;
        } else {
          int idx = b - 4 - ne - 4 * nfm, sdeg = 0;
          while (idx >= (sdeg + 1) * (sdeg + 2) / 2) { idx -= (sdeg + 1) * (sdeg + 2) / 2; ++sdeg; }
          deg = sdeg + 4;
        }
      } else if (b < 3) {
        deg = 1;
      } else if (b < 3 + 3 * (order - 1)) {
        deg = 2 + (b - 3) % (order - 1);
      } else {
        int idx = b - 3 - 3 * (order - 1), sdeg = 0;
        while (idx > sdeg) { idx -= sdeg + 1; ++sdeg; }
        deg = sdeg + 3;
      }
      high[b] = order == 1 || deg == order ? 1 : 0;  // P1: the whole density (SpatialDiscrete.cpp:51-52)
    }
    ptp.assign(size_t(nb) * nb, 0.0);
    for (int a = 0; a < nb; ++a)
      for (int b = 0; b < nb; ++b) {
        Real s = 0; for (int q = 0; q < nq; ++q) s += phi[size_t(q) * nb + a] * phi[size_t(q) * nb + b];
        ptp[size_t(a) * nb + b] = s;
      }
    lsqInv.assign(size_t(nb) * nb, 0.0);
    invert(nb, ptp.data(), lsqInv.data());
    const int m = t == kLine ? 1 : (t == kTet ? 2 * order + 1 : linePoints(2 * order + 1));
    perm.clear();
    for (int r = 0; r < (t == kHex ? 4 : (t == kTet ? 3 : 1)); ++r) perm.push_back(facePermutation(t, m, r));
  }
};

}  // namespace orc
