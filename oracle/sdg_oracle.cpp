// Oracle -- TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU path is compared against
// and the timed CPU baseline; nothing in the product links, imports or calls it.
//
// A CPU restatement, in plain C++17 + OpenMP, of SubrosaDG's explicit DG residual-and-update path
// with the reference's own data flow: modal (hierarchic Lobatto) basis, per-element dense mass-matrix
// inverse, per-element AoS blocks, and the stage sequence of Solver::stepSolver
// (src/Solver/TimeIntegration.cpp:326-350), including -- when `faithful` is set -- the gradient pass
// that the reference runs even for Euler and never reads.
//
// Followed reference code:
//   adjacency / periodic pairing   src/Mesh/Adjacency.cpp:37-495
//   geometry                       src/Mesh/Geometry.cpp:29-169
//   initial condition (LSQ)        src/Solver/InitialCondition.cpp:85-149
//   volume / face quadrature       src/Solver/SpatialDiscrete.cpp:194-322, 633-968
//   residual assembly              src/Solver/SpatialDiscrete.cpp:1016-1068
//   RK update, dt, relative error  src/Solver/TimeIntegration.cpp:45-324
//   source term (Boussinesq)       src/Solver/SpatialDiscrete.cpp:254-262,1026-1029, SourceTerm.cpp:29-58
//   artificial viscosity           src/Solver/SpatialDiscrete.cpp:37-192 (sensor, vertex max), :204-250 (volume),
//                                  :528-631,685-734 (faces), :785-834 (boundary), ViscousFlux.cpp:105-200
// Periodic pairing uses a node map (master node per slave node) in place of gmsh's periodic entity
// queries; the right rotation of a periodic face is taken from the parents' face vertex order, the
// same rule as for ordinary interior faces.
#include <omp.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../include/sdg_gpu.h"
#include "orc_basis.hpp"
#include "orc_physics.hpp"

namespace orc {

struct Block {
  int type = 0;
  RefElement ref;
  int64_t ne = 0;
  std::vector<int> verts;       // ne * nvert
  std::vector<Real> qcoord;   // ne * nq * 3
  std::vector<Real> jw;       // ne * nq        |J| w
  std::vector<Real> jtiw;     // ne * nq * d*d  J^-T |J| w, column-major d x d per point
  std::vector<Real> minv;     // ne * nb*nb     local mass matrix inverse
  // curved geometry: the order-q map through each element's gmsh-ordered geometry nodes
  bool curved = false;
  int geoOrder = 1;
  std::vector<int> geo;       // ne * (nodes of the order-q element)
  CurvedBasis cb;
  // element-sample mode (orc_create_sampled): what each element is needed for -- 0 its residual, 1 its
  // gradient (a neighbour of a sampled element, gradient pass on), 2 its coefficients only (traces), 3 nothing;
  // and the slot of its dense M^-1 (and M) in minv / mass (-1: none).  Empty: every element at level 0.
  std::vector<signed char> level;
  std::vector<int32_t> slot;
  // shared-inverse (lean) mode on a block of affine elements: M_e^-1 = M_ref^-1 / |J|_e
  bool sharedInverse = false;
  std::vector<Real> minvRef;  // nb*nb         inverse of the reference mass matrix sum_q phi_a phi_b w_q
  std::vector<Real> detJ;     // ne            constant Jacobian determinant of each element
  std::vector<Real> mass;     // ne * nb*nb     local mass matrix (kept when refining solves)
  std::vector<Real> minEdge;  // ne
  std::vector<Real> innerRadius;  // ne (artificial viscosity length scale)
  std::vector<Real> epsV;     // ne * nvert  artificial viscosity at the element's vertices
  // state (column-major nv x nb per element: index b*nv + v)
  std::vector<Real> coef, last, res;
  std::vector<Real> qvol;     // ne * nv x (nq*d)
  std::vector<Real> qface;    // ne * nv x (nface*nfq)
  std::vector<Real> qsrc;     // ne * nv x nq  source |J| w (Boussinesq only)
  // gradient blocks, rows (v*d + k)
  std::vector<Real> qvg, qfvg, qfig, rvg, rig, vgc, igc, gc;
};

struct Face {
  int bl = 0, el = 0, fl = 0, br = -1, er = -1, fr = -1, rot = 0;
  int physical = 0, bc = -1;
  std::vector<Real> normal;  // nfq * 3
  std::vector<Real> fjw;     // nfq
  std::vector<Real> coord;   // nfq * 3
};

struct Problem {
  int dim = 2, nv = 4, p = 1;
  int eq = 0, flux = 0, visc = 0, rk = 2;
  bool faithful = true;
  // Refine each M^-1 product / least-squares solve with one residual-correction step.  The reference
  // multiplies by the explicit inverse (TimeIntegration.cpp:196); refinement removes the
  // condition-number round-off of the hierarchic basis at high order so the checker stays accurate to
  // ~1e-15.  Off for the timed CPU baseline, which mirrors the reference's arithmetic exactly.
  bool refine = true;
  // Lean CPU-baseline mode: a block whose elements are all affine multiplies by one shared reference inverse
  // scaled by 1/|J| (M = |J| M_ref exactly for a constant Jacobian) instead of reading a dense inverse per element.
  bool lean = false;
  Physics ph;
  std::vector<Block> blocks;
  std::vector<Face> interior, boundary;
  std::vector<PointVar> dummy;  // boundary dummy variables, [boundary][nfq]
  std::vector<Real> relErr;
  int64_t totalElements = 0;
  bool hasState = false;
  std::string err;

  // artificial viscosity (ShockCapturingEnum::ArtificialViscosity): empirical tolerance and factor
  bool av = false;
  Real avTol = 0, avFactor = 1;
  std::vector<Real> nodeAV;   // per mesh node, the max over its elements
  bool ns() const { return eq == 1 || eq == 3; }  // compressible or incompressible Navier-Stokes
  bool gradientPass() const { return ns() || faithful || av; }
  int nfq() const { return blocks[0].ref.nfq; }
  bool sampled = false;
};

// Is element e of block B needed at `lvl` (0 residual, 1 gradient, 2 coefficients)?  Always outside sample mode.
static inline bool needed(const Block& B, int64_t e, int lvl) { return B.level.empty() || B.level[size_t(e)] <= lvl; }
// A face is evaluated at `lvl` when either parent is needed there.
static inline bool faceNeeded(const Problem& P, const Face& F, int lvl) {
  return needed(P.blocks[F.bl], F.el, lvl) || (F.br >= 0 && needed(P.blocks[F.br], F.er, lvl));
}
// Slot of element e's dense inverse.
static inline size_t minvSlot(const Block& B, int64_t e) { return B.slot.empty() ? size_t(e) : size_t(B.slot[size_t(e)]); }

// ---- setup ----------------------------------------------------------------------------------------

// Inner radius (gmsh quality "innerRadius", the artificial-viscosity length, Geometry.cpp:31-41; gmsh 4.13.1 is
// not vendored): the inscribed radius 2A/perimeter of a triangle, the same tangential-polygon formula for a
// quadrangle (A from its diagonals), and 3V/S for a hexahedron (V by 2x2x2 Gauss quadrature of the trilinear map,
// S from each face's diagonals) -- exact for squares and cubes.
static Real innerRadiusOf(int type, const double* nodes, const int* vv) {
  auto X = [&](int k, int d) { return Real(nodes[size_t(vv[k]) * 3 + d]); };
  if (type == kLine) return std::fabs(X(1, 0) - X(0, 0)) / 2.0;  // gmsh MLine: half the length
  auto sub = [&](int a, int b, Real* o) { for (int d = 0; d < 3; ++d) o[d] = X(a, d) - X(b, d); };
  auto norm = [](const Real* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); };
  auto crossNorm = [&](const Real* a, const Real* b) {
    const Real c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    return norm(c);
  };
  if (type == kTri || type == kQuad) {
    const int nv = type == kTri ? 3 : 4;
    Real per = 0, e[3];
    for (int i = 0; i < nv; ++i) { sub((i + 1) % nv, i, e); per += norm(e); }
    Real d1[3], d2[3];
    if (type == kTri) { sub(1, 0, d1); sub(2, 0, d2); }
    else { sub(2, 0, d1); sub(3, 1, d2); }
    return crossNorm(d1, d2) / per;  // 2 (|d1 x d2| / 2) / perimeter
  }
  if (type == kTet) {  // 3V/S
    Real a[3], b[3], c[3];
    sub(1, 0, a); sub(2, 0, b); sub(3, 0, c);
    const Real vol = std::fabs(a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                               a[2] * (b[0] * c[1] - b[1] * c[0])) / 6.0;
    static const int tf[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};
    Real area = 0;
    for (const auto& f : tf) { Real d1[3], d2[3]; sub(f[1], f[0], d1); sub(f[2], f[0], d2); area += crossNorm(d1, d2) / 2.0; }
    return 3.0 * vol / area;
  }
  static const int faces[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {0, 4, 7, 3}, {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};
  Real area = 0;
  for (const auto& f : faces) {
    Real d1[3], d2[3];
    sub(f[2], f[0], d1); sub(f[3], f[1], d2);
    area += crossNorm(d1, d2) / 2.0;
  }
  const Real g = 1.0 / std::sqrt(3.0);
  Real vol = 0;
  for (int q = 0; q < 8; ++q) {
    const Real xi[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, (q & 4) ? g : -g};
    Real sh[8], gr[24], J[3][3] = {{0}};
    elemShape(kHex, xi, sh, gr);
    for (int k = 0; k < 8; ++k)
      for (int l = 0; l < 3; ++l)
        for (int m = 0; m < 3; ++m) J[l][m] += gr[k * 3 + m] * X(k, l);
    vol += J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  }
  return 3.0 * vol / area;
}

// Reference vertices of the element types with curved geometry (quadrangles, triangles, hexahedra).
static void refVertexCurved(int type, int v, Real* X) {
  static const Real quad[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  static const Real tri[3][2] = {{0, 0}, {1, 0}, {0, 1}};
  if (type == kHex) {
    X[0] = (v == 1 || v == 2 || v == 5 || v == 6) ? 1 : -1;
    X[1] = (v == 2 || v == 3 || v == 6 || v == 7) ? 1 : -1;
    X[2] = v >= 4 ? 1 : -1;
    return;
  }
  X[0] = type == kQuad ? quad[v][0] : tri[v][0];
  X[1] = type == kQuad ? quad[v][1] : tri[v][1];
  X[2] = 0;
}

// The curved map of element e: x(X) and J[l][k] = dx_l/dX_k (the gmsh Jacobian of Geometry.cpp:44-67 for
// high-order elements).
static void curvedMap(const Block& B, int64_t e, const double* nodes, const Real* X, Real J[3][3], Real* x) {
  const int nn = B.cb.nn, d = B.type == kHex ? 3 : 2;
  std::vector<Real> N(nn), G(size_t(nn) * 3);
  B.cb.eval(X, N.data(), G.data());
  for (int l = 0; l < 3; ++l) { x[l] = 0; for (int k = 0; k < 3; ++k) J[l][k] = 0; }
  for (int n = 0; n < nn; ++n) {
    const double* c = &nodes[size_t(B.geo[size_t(e) * nn + n]) * 3];
    for (int l = 0; l < 3; ++l) x[l] += N[n] * c[l];
    for (int l = 0; l < d; ++l)
      for (int k = 0; k < d; ++k) J[l][k] += G[n * 3 + k] * c[l];
  }
}

static void buildGeometry(Problem& P, Block& B, const double* nodes) {
  const RefElement& R = B.ref;
  const int d = P.dim, nq = R.nq, nb = R.nb, nvert = elemVerts(B.type);
  B.qcoord.assign(size_t(B.ne) * nq * 3, 0.0);
  B.jw.assign(size_t(B.ne) * nq, 0.0);
  B.jtiw.assign(size_t(B.ne) * nq * d * d, 0.0);
  B.detJ.assign(size_t(B.ne), 0.0);
  std::vector<char> affine(size_t(B.ne), 1);
  B.minEdge.assign(size_t(B.ne), 0.0);
  B.innerRadius.assign(size_t(B.ne), 0.0);
  std::string failure;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < B.ne; ++e) {
    if (!needed(B, e, 2)) continue;
    const int* vv = &B.verts[size_t(e) * nvert];
    for (int q = 0; q < nq; ++q) {
      Real sh[8], g[24];
      Real J[3][3] = {{0}};  // J[l][k] = d x_l / d xi_k
      Real x[3] = {0, 0, 0};
      if (B.curved) {
        curvedMap(B, e, nodes, &R.vq.x[q * 3], J, x);
      } else {
        elemShape(B.type, &R.vq.x[q * 3], sh, g);
        for (int v = 0; v < nvert; ++v) {
          const double* c = &nodes[size_t(vv[v]) * 3];
          for (int l = 0; l < 3; ++l) x[l] += sh[v] * c[l];
          for (int l = 0; l < d; ++l)
            for (int k = 0; k < d; ++k) J[l][k] += g[v * 3 + k] * c[l];
        }
      }
      for (int l = 0; l < 3; ++l) B.qcoord[(size_t(e) * nq + q) * 3 + l] = x[l];
      Real det, inv[3][3];
      if (d == 1) {
        det = J[0][0];
        inv[0][0] = 1.0 / det;
      } else if (d == 2) {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        inv[0][0] = J[1][1] / det; inv[0][1] = -J[0][1] / det; inv[1][0] = -J[1][0] / det; inv[1][1] = J[0][0] / det;
      } else {
        det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
              J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
      }
      if (!(det > 0.0)) {
#pragma omp critical
        failure = "inverted or degenerate element";
      }
      const Real jw = det * R.vq.w[q];
      B.jw[size_t(e) * nq + q] = jw;
      if (q == 0) B.detJ[e] = det;
      else if (std::fabs(det - B.detJ[e]) > 1e-13 * std::fabs(B.detJ[e])) affine[e] = 0;
      // M(a,b) = (J^-T)(a,b) |J| w = (J^-1)(b,a) |J| w, stored column-major at [a + b*d].
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) B.jtiw[(size_t(e) * nq + q) * d * d + a + b * d] = inv[b][a] * jw;
    }
    // minEdge quality: shortest straight edge between vertices.
    static const int lineE[1][2] = {{0, 1}};
    static const int triE[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    static const int quadE[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
    static const int hexE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                    {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    static const int tetE[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 2}, {3, 1}};
    const int(*E)[2] = B.type == kLine ? lineE
                       : (B.type == kTri ? triE : (B.type == kQuad ? quadE : (B.type == kTet ? tetE : hexE)));
    const int nE = B.type == kLine ? 1 : (B.type == kTri ? 3 : (B.type == kQuad ? 4 : (B.type == kTet ? 6 : 12)));
    Real me = 1e300;
    for (int i = 0; i < nE; ++i) {
      const double* a = &nodes[size_t(vv[E[i][0]]) * 3];
      const double* b = &nodes[size_t(vv[E[i][1]]) * 3];
      const Real l = std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
      me = std::min(me, l);
    }
    B.minEdge[e] = me;
    B.innerRadius[e] = innerRadiusOf(B.type, nodes, vv);
  }
  if (!failure.empty()) throw std::runtime_error(failure);
  B.sharedInverse = P.lean && !P.refine && std::all_of(affine.begin(), affine.end(), [](char a) { return a != 0; });
  if (B.sharedInverse) {
    std::vector<Real> m(size_t(nb) * nb, 0.0);
    for (int a = 0; a < nb; ++a)
      for (int b = 0; b < nb; ++b) {
        Real s = 0;
        for (int q = 0; q < nq; ++q) s += R.phi[size_t(q) * nb + a] * R.phi[size_t(q) * nb + b] * R.vq.w[q];
        m[size_t(a) * nb + b] = s;
      }
    B.minvRef.assign(size_t(nb) * nb, 0.0);
    invert(nb, m.data(), B.minvRef.data());
    return;
  }
  // sample mode: inverses only where a residual or gradient is evaluated, in compact slots
  const int minvLevel = P.gradientPass() ? 1 : 0;
  int64_t slots = B.ne;
  if (P.sampled) {
    B.slot.assign(size_t(B.ne), -1);
    slots = 0;
    for (int64_t e = 0; e < B.ne; ++e)
      if (needed(B, e, minvLevel)) B.slot[size_t(e)] = int32_t(slots++);
  }
  B.minv.assign(size_t(slots) * nb * nb, 0.0);
  if (P.refine) B.mass.assign(size_t(slots) * nb * nb, 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < B.ne; ++e) {
    if (!needed(B, e, minvLevel)) continue;
    // Local mass matrix inverse (Geometry.cpp:88-100).
    std::vector<Real> m(size_t(nb) * nb, 0.0);
    for (int a = 0; a < nb; ++a)
      for (int b = 0; b < nb; ++b) {
        Real s = 0;
        for (int q = 0; q < nq; ++q) s += R.phi[size_t(q) * nb + a] * R.phi[size_t(q) * nb + b] * B.jw[size_t(e) * nq + q];
        m[size_t(a) * nb + b] = s;
      }
    invert(nb, m.data(), &B.minv[minvSlot(B, e) * nb * nb]);
    if (P.refine) std::copy(m.begin(), m.end(), &B.mass[minvSlot(B, e) * nb * nb]);
  }
}

static void faceGeometry(Problem& P, Face& F, const double* nodes) {
  const Block& B = P.blocks[F.bl];
  const RefElement& R = B.ref;
  const int nfv = faceVerts(B.type), nfq = R.nfq;
  const int* ft = faceVertexTable(B.type);
  const int* vv = &B.verts[size_t(F.el) * elemVerts(B.type)];
  F.normal.assign(size_t(nfq) * 3, 0.0); F.fjw.assign(nfq, 0.0); F.coord.assign(size_t(nfq) * 3, 0.0);
  for (int j = 0; j < nfq; ++j) {
    Real sh[4], dxi[4], deta[4];
    faceShape(B.type, &R.fq.x[j * 3], sh);
    faceShapeGrad(B.type, &R.fq.x[j * 3], dxi, deta);
    Real x[3] = {0, 0, 0}, tx[3] = {0, 0, 0}, ty[3] = {0, 0, 0};
    if (B.curved) {  // the face point and the face tangents through the parent's curved map
      Real X[3] = {0, 0, 0}, dX[3] = {0, 0, 0}, dY[3] = {0, 0, 0}, V[3], J[3][3];
      for (int k = 0; k < nfv; ++k) {
        refVertexCurved(B.type, ft[F.fl * nfv + k], V);
        for (int l = 0; l < 3; ++l) { X[l] += sh[k] * V[l]; dX[l] += dxi[k] * V[l]; if (nfv >= 3) dY[l] += deta[k] * V[l]; }
      }
      curvedMap(B, F.el, nodes, X, J, x);
      for (int l = 0; l < 3; ++l) {
        tx[l] = J[l][0] * dX[0] + J[l][1] * dX[1] + J[l][2] * dX[2];
        ty[l] = J[l][0] * dY[0] + J[l][1] * dY[1] + J[l][2] * dY[2];
      }
    } else {
      for (int k = 0; k < nfv; ++k) {
        const double* c = &nodes[size_t(vv[ft[F.fl * nfv + k]]) * 3];
        for (int l = 0; l < 3; ++l) { x[l] += sh[k] * c[l]; tx[l] += dxi[k] * c[l]; if (nfv >= 3) ty[l] += deta[k] * c[l]; }
      }
    }
    for (int l = 0; l < 3; ++l) F.coord[j * 3 + l] = x[l];
    Real n[3], det;
    if (P.dim == 1) {  // Geometry.cpp:102-112: -1 at local face 0, +1 at local face 1; a point's measure is 1
      det = 1.0;
      n[0] = F.fl == 0 ? -1.0 : 1.0; n[1] = 0; n[2] = 0;
    } else if (P.dim == 2) {  // Geometry.cpp:115-127
      det = std::sqrt(tx[0] * tx[0] + tx[1] * tx[1]);
      n[0] = tx[1] / det; n[1] = -tx[0] / det; n[2] = 0;
    } else {           // Geometry.cpp:130-147
      const Real cx = tx[1] * ty[2] - tx[2] * ty[1], cy = tx[2] * ty[0] - tx[0] * ty[2], cz = tx[0] * ty[1] - tx[1] * ty[0];
      det = std::sqrt(cx * cx + cy * cy + cz * cz);
      n[0] = cx / det; n[1] = cy / det; n[2] = cz / det;
    }
    for (int l = 0; l < 3; ++l) F.normal[j * 3 + l] = n[l];
    F.fjw[j] = det * R.fq.w[j];
  }
}

static void buildAdjacency(Problem& P, const sdg_mesh& m) {
  struct Visit { int b, e, f; std::vector<int> mapped; };
  struct Entry { Visit left; Visit right; int count = 0; };
  std::map<std::vector<int>, Entry> faces;
  auto master = [&](int v) { return m.periodic_master ? m.periodic_master[v] : v; };
  for (int b = 0; b < int(P.blocks.size()); ++b) {
    const Block& B = P.blocks[b];
    const int nfv = faceVerts(B.type), nf = elemFaces(B.type), nvert = elemVerts(B.type);
    const int* ft = faceVertexTable(B.type);
    for (int64_t e = 0; e < B.ne; ++e)
      for (int f = 0; f < nf; ++f) {
        Visit v{b, int(e), f, {}};
        for (int k = 0; k < nfv; ++k) v.mapped.push_back(master(B.verts[size_t(e) * nvert + ft[f * nfv + k]]));
        std::vector<int> key = v.mapped; std::sort(key.begin(), key.end());
        Entry& en = faces[key];
        if (en.count == 0) en.left = v;
        else if (en.count == 1) en.right = v;
        else throw std::runtime_error("a face is recorded more than twice");
        en.count++;
      }
  }
  std::map<std::vector<int>, int> bmap;
  const int nbv = P.dim == 1 ? 1 : (P.dim == 2 ? 2 : 4);
  for (int64_t i = 0; i < m.boundary_count; ++i) {
    std::vector<int> key;
    for (int k = 0; k < nbv; ++k) {
      if (nbv == 4 && k == 3 && m.boundary_node[i * nbv + k] == -1) break;  // a triangle in 3D
      key.push_back(master(m.boundary_node[i * nbv + k]));
    }
    std::sort(key.begin(), key.end());
    bmap[key] = int(i);
  }
  std::vector<std::pair<int, Face>> periodicEnds;
  for (auto& kv : faces) {
    Entry& en = kv.second;
    Face F;
    F.bl = en.left.b; F.el = en.left.e; F.fl = en.left.f;
    if (en.count == 2) {
      F.br = en.right.b; F.er = en.right.e; F.fr = en.right.f;
      if (P.dim == 3) {
        const auto it = std::find(en.right.mapped.begin(), en.right.mapped.end(), en.left.mapped[0]);
        F.rot = int(it - en.right.mapped.begin());
      }
      P.interior.push_back(F);
    } else {
      const auto it = bmap.find(kv.first);
      if (it == bmap.end()) throw std::runtime_error("boundary face without a boundary element");
      F.physical = m.boundary_physical[it->second];
      if (F.physical < 1 || F.physical > m.physical_count) throw std::runtime_error("bad physical index");
      F.bc = m.physical_boundary_condition[F.physical - 1];
      if (F.bc == SDG_BC_PERIODIC && P.dim == 1 && !m.periodic_master) {
        periodicEnds.push_back({it->second, F});
        continue;
      }
      if (F.bc == SDG_BC_PERIODIC) throw std::runtime_error("unpaired periodic face");
      P.boundary.push_back(F);
    }
  }
  // 1D periodic without a node map (Adjacency.cpp:185-211): the first two point elements are joined, the
  // first one's parent on the left
  if (!periodicEnds.empty()) {
    if (periodicEnds.size() != 2) throw std::runtime_error("a 1D periodic mesh needs two periodic end points");
    std::sort(periodicEnds.begin(), periodicEnds.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    Face F;
    F.bl = periodicEnds[0].second.bl; F.el = periodicEnds[0].second.el; F.fl = periodicEnds[0].second.fl;
    F.br = periodicEnds[1].second.bl; F.er = periodicEnds[1].second.el; F.fr = periodicEnds[1].second.fl;
    P.interior.push_back(F);
  }
}

// ---- point evaluation helpers ---------------------------------------------------------------------

// vals[q][v] = sum_b coef(v,b) phi[q][b] for rows q of a phi table.
static inline void interp(int nv, int nb, int nrow, const Real* coef, const Real* phi, Real* vals) {
  for (int q = 0; q < nrow; ++q) {
    Real* out = vals + size_t(q) * nv;
    for (int v = 0; v < nv; ++v) out[v] = 0;
    const Real* ph = phi + size_t(q) * nb;
    for (int b = 0; b < nb; ++b) {
      const Real w = ph[b];
      const Real* c = coef + size_t(b) * nv;
      for (int v = 0; v < nv; ++v) out[v] += c[v] * w;
    }
  }
}

// out(r, b) (+)= sum_c in(r, c) * tab(c, b): column-major (nr x nc) times row-major (nc x nb) table.
static inline void gemmAcc(int nr, int nc, int nb, const Real* in, const Real* tab, Real* out, Real sign) {
  for (int c = 0; c < nc; ++c) {
    const Real* col = in + size_t(c) * nr;
    const Real* row = tab + size_t(c) * nb;
    for (int b = 0; b < nb; ++b) {
      const Real w = sign * row[b];
      Real* o = out + size_t(b) * nr;
      for (int r = 0; r < nr; ++r) o[r] += col[r] * w;
    }
  }
}

// Element-face trace (AdjacencyElementVariable::compute, VariableConvertor.cpp:434-451).
static void trace(const Problem& P, int b, int e, int f, PointVar* out) {
  const Block& B = P.blocks[b];
  const int nv = P.nv, nb = B.ref.nb, nfq = B.ref.nfq;
  Real vals[64 * kMaxVar];
  interp(nv, nb, nfq, &B.coef[size_t(e) * nv * nb], &B.ref.phif[size_t(f) * nfq * nb], vals);
  for (int j = 0; j < nfq; ++j) {
    for (int v = 0; v < nv; ++v) out[j].cons[v] = vals[j * nv + v];
    computationalFromConserved(P.ph, out[j]);
  }
}

// Gradient trace on face f: BR1 -> gc; BR2 -> vgc + igc[f]; conserved gradient rows (v*d+k).
static void gradientTrace(const Problem& P, int b, int e, int f, Real* out /* nfq * nv*d */) {
  const Block& B = P.blocks[b];
  const int nr = P.nv * P.dim, nb = B.ref.nb, nfq = B.ref.nfq;
  std::vector<Real> c(size_t(nr) * nb);
  if (P.visc == 1) {
    std::copy_n(&B.gc[size_t(e) * nr * nb], nr * nb, c.data());
  } else {
    const Real* a = &B.vgc[size_t(e) * nr * nb];
    const Real* g = &B.igc[(size_t(e) * B.ref.nface + f) * nr * nb];
    for (int i = 0; i < nr * nb; ++i) c[i] = a[i] + g[i];
  }
  interp(nr, nb, nfq, c.data(), &B.ref.phif[size_t(f) * nfq * nb], out);
}

// x = R M^-1 for an (nr x nb, column-major) block R (TimeIntegration.cpp:196,205-225), optionally refined:
// x += (R - x M) M^-1.
static void applyMinv(const Problem& P, const Block& B, int64_t e, int nr, const Real* R, Real* x) {
  const int nb = B.ref.nb;
  for (int i = 0; i < nr * nb; ++i) x[i] = 0;
  if (B.sharedInverse) {  // lean mode, affine block: M^-1 = M_ref^-1 / |J|
    gemmAcc(nr, nb, nb, R, B.minvRef.data(), x, 1);
    const Real s = 1.0 / B.detJ[e];
    for (int i = 0; i < nr * nb; ++i) x[i] *= s;
    return;
  }
  const Real* Mi = &B.minv[minvSlot(B, e) * nb * nb];
  gemmAcc(nr, nb, nb, R, Mi, x, 1);
  if (!P.refine) return;
  const Real* M = &B.mass[minvSlot(B, e) * nb * nb];
  std::vector<Real> res(R, R + size_t(nr) * nb);
  gemmAcc(nr, nb, nb, x, M, res.data(), -1);
  gemmAcc(nr, nb, nb, res.data(), Mi, x, 1);
}

// ---- the stage kernels ----------------------------------------------------------------------------

static void gradientQuadratureAndResidual(Problem& P) {
  const int d = P.dim, nv = P.nv, nr = nv * d;
  // volume part (SpatialDiscrete.cpp:294-322)
  for (Block& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      if (!needed(B, e, 1)) continue;
      Real vals[216 * kMaxVar];
      interp(nv, nb, nq, &B.coef[size_t(e) * nv * nb], B.ref.phi.data(), vals);
      Real* Q = &B.qvg[size_t(e) * nr * nq * d];
      for (int q = 0; q < nq; ++q) {
        const Real* M = &B.jtiw[(size_t(e) * nq + q) * d * d];
        for (int v = 0; v < nv; ++v)
          for (int a = 0; a < d; ++a)
            for (int bb = 0; bb < d; ++bb) Q[size_t(q * d + bb) * nr + v * d + a] = vals[q * nv + v] * M[a + bb * d];
      }
    }
  }
  // interior faces (SpatialDiscrete.cpp:844-911)
  const int nfq = P.nfq();
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(P.interior.size()); ++i) {
    const Face& F = P.interior[i];
    if (!faceNeeded(P, F, 1)) continue;
    PointVar L[64], R[64];
    trace(P, F.bl, F.el, F.fl, L); trace(P, F.br, F.er, F.fr, R);
    Block& BL = P.blocks[F.bl]; Block& BR = P.blocks[F.br];
    const std::vector<int>& perm = BR.ref.perm[F.rot];
    const int nfl = BL.ref.nface * nfq, nfr = BR.ref.nface * nfq;
    Real* QL = &BL.qfvg[size_t(F.el) * nr * nfl];
    Real* QR = &BR.qfvg[size_t(F.er) * nr * nfr];
    for (int j = 0; j < nfq; ++j) {
      const int jr = perm[j];
      const Real* n = &F.normal[j * 3];
      for (int v = 0; v < nv; ++v)
        for (int k = 0; k < d; ++k) {
          const Real t = n[k] * (L[j].cons[v] + R[jr].cons[v]) / 2.0 * F.fjw[j];
          QL[size_t(F.fl * nfq + j) * nr + v * d + k] = t;
          QR[size_t(F.fr * nfq + jr) * nr + v * d + k] = -t;
        }
      if (P.ns()) {
        Real* IL = &BL.qfig[size_t(F.el) * nr * nfl];
        Real* IR = &BR.qfig[size_t(F.er) * nr * nfr];
        for (int v = 0; v < nv; ++v)
          for (int k = 0; k < d; ++k) {
            const Real t = n[k] * (R[jr].cons[v] - L[j].cons[v]) / 2.0 * F.fjw[j];
            IL[size_t(F.fl * nfq + j) * nr + v * d + k] = t;
            IR[size_t(F.fr * nfq + jr) * nr + v * d + k] = t;
          }
      }
    }
  }
  // boundary faces (SpatialDiscrete.cpp:913-968)
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(P.boundary.size()); ++i) {
    const Face& F = P.boundary[i];
    if (!faceNeeded(P, F, 1)) continue;
    PointVar L[64];
    trace(P, F.bl, F.el, F.fl, L);
    Block& BL = P.blocks[F.bl];
    const int nfl = BL.ref.nface * nfq;
    for (int j = 0; j < nfq; ++j) {
      Real vol[kMaxVar], itf[kMaxVar];
      boundaryGradientState(P.ph, F.bc, &F.normal[j * 3], L[j], P.dummy[size_t(i) * nfq + j], vol, itf);
      const Real* n = &F.normal[j * 3];
      for (int v = 0; v < nv; ++v)
        for (int k = 0; k < d; ++k) {
          BL.qfvg[size_t(F.el) * nr * nfl + size_t(F.fl * nfq + j) * nr + v * d + k] = n[k] * vol[v] * F.fjw[j];
          if (P.ns()) BL.qfig[size_t(F.el) * nr * nfl + size_t(F.fl * nfq + j) * nr + v * d + k] = n[k] * itf[v] * F.fjw[j];
        }
    }
  }
  // gradient residual and coefficients (SpatialDiscrete.cpp:1034-1068, TimeIntegration.cpp:200-228)
  for (Block& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb, nf = B.ref.nface, nfl = nf * nfq;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      if (!needed(B, e, 1)) continue;
      const Real* QF = &B.qfvg[size_t(e) * nr * nfl];
      const Real* QV = &B.qvg[size_t(e) * nr * nq * d];
      Real* RV = &B.rvg[size_t(e) * nr * nb];
      for (int i = 0; i < nr * nb; ++i) RV[i] = 0;
      gemmAcc(nr, nfl, nb, QF, B.ref.phif.data(), RV, 1);
      gemmAcc(nr, nq * d, nb, QV, B.ref.dphi.data(), RV, -1);
      Real* VG = &B.vgc[size_t(e) * nr * nb];
      applyMinv(P, B, e, nr, RV, VG);
      if (!P.ns()) continue;
      Real* G = &B.gc[size_t(e) * nr * nb];
      std::copy_n(VG, nr * nb, G);
      const Real* QI = &B.qfig[size_t(e) * nr * nfl];
      const int nblk = P.visc == 1 ? 1 : nf;
      for (int blk = 0; blk < nblk; ++blk) {
        const int c0 = P.visc == 1 ? 0 : blk * nfq, c1 = P.visc == 1 ? nfl : (blk + 1) * nfq;
        Real* RI = &B.rig[(size_t(e) * nblk + blk) * nr * nb];
        for (int k = 0; k < nr * nb; ++k) RI[k] = 0;
        gemmAcc(nr, c1 - c0, nb, QI + size_t(c0) * nr, B.ref.phif.data() + size_t(c0) * nb, RI, 1);
        Real* IG = &B.igc[(size_t(e) * nblk + blk) * nr * nb];
        applyMinv(P, B, e, nr, RI, IG);
        for (int i = 0; i < nr * nb; ++i) G[i] += IG[i];
      }
    }
  }
}

// Artificial viscosity of every element (SpatialDiscrete.cpp:37-89): the Persson-Peraire sensor
// s = log10(int rho_h^2 / int rho^2) with rho_h the degree-P modes of the density (the whole density for P1);
// eps = 0 below s0 - kappa, eps0 h/P above s0 + kappa, and the sine ramp between; then the max over the
// elements sharing each mesh node (:91-109) and the elements' vertex values from their nodes (:111-124).
// s0 per order (SimulationControl.cpp:892-893).
static const Real kAvTolerance[5] = {0.0, -1.20411998266, -1.90848501888, -2.40823996531, -2.79588001734};
static const Real kWeakPressureAddition = 0.01;  // PhysicalModel.cpp:63-66
static const Real kBoussinesqGravity = 1.0;      // SourceTerm.cpp:31
static const Real kPiReal = Real(3.141592653589793238462643383279502884L);

static void artificialViscosity(Problem& P) {
  const Real s0 = kAvTolerance[P.p - 1];
  std::fill(P.nodeAV.begin(), P.nodeAV.end(), Real(0));
  for (Block& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb, nv = P.nv, nvert = B.ref.nvert;
    std::vector<Real> eps(size_t(B.ne));
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      const Real* c = &B.coef[size_t(e) * nv * nb];
      Real num = 0, den = 0;
      for (int q = 0; q < nq; ++q) {
        Real all = 0, hi = 0;
        for (int b = 0; b < nb; ++b) {
          const Real t = B.ref.phi[size_t(q) * nb + b] * c[b * nv];
          all += t;
          if (B.ref.high[b]) hi += t;
        }
        const Real w = B.jw[size_t(e) * nq + q];
        num += hi * (hi * w);
        den += all * (all * w);
      }
      const Real sc = std::log10(num / den);
      const Real full = P.avFactor * (B.innerRadius[e] / Real(P.p));
      if (sc < s0 - P.avTol) eps[e] = 0;
      else if (sc > s0 + P.avTol) eps[e] = full;
      else eps[e] = full * (1.0 + std::sin(kPiReal * (sc - s0) / (2.0 * P.avTol))) / 2.0;
    }
    for (int64_t e = 0; e < B.ne; ++e)
      for (int k = 0; k < nvert; ++k) {
        Real& n = P.nodeAV[size_t(B.verts[size_t(e) * nvert + k])];
        n = std::max(n, eps[e]);
      }
  }
  for (Block& B : P.blocks) {
    const int nvert = B.ref.nvert;
    for (int64_t e = 0; e < B.ne; ++e)
      for (int k = 0; k < nvert; ++k)
        B.epsV[size_t(e) * nvert + k] = P.nodeAV[size_t(B.verts[size_t(e) * nvert + k])];
  }
}

// Volume-gradient trace on face f (the artificial viscosity's gradient, ViscousFluxEnum::None:
// variable_volume_gradient_basis_function_coefficient_), conserved rows (v*d+k).
static void volumeGradientTrace(const Problem& P, int b, int e, int f, Real* out /* nfq * nv*d */) {
  const Block& B = P.blocks[b];
  const int nr = P.nv * P.dim, nb = B.ref.nb, nfq = B.ref.nfq;
  interp(nr, nb, nfq, &B.vgc[size_t(e) * nr * nb], &B.ref.phif[size_t(f) * nfq * nb], out);
}

// Artificial viscosity at face f's points of element e (nodal_adjacency_value_ x vertex values).
static void faceViscosity(const Problem& P, int b, int e, int f, Real* out /* nfq */) {
  const Block& B = P.blocks[b];
  const int nvert = B.ref.nvert, nfq = B.ref.nfq;
  for (int j = 0; j < nfq; ++j) {
    Real s = 0;
    for (int k = 0; k < nvert; ++k) s += B.ref.nodalf[(size_t(f) * nfq + j) * nvert + k] * B.epsV[size_t(e) * nvert + k];
    out[j] = s;
  }
}

static void quadratureAndResidual(Problem& P) {
  const int d = P.dim, nv = P.nv, nr = nv * d;
  // volume (SpatialDiscrete.cpp:194-266)
  for (Block& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      if (!needed(B, e, 0)) continue;
      Real vals[216 * kMaxVar];
      std::vector<Real> gvals;
      interp(nv, nb, nq, &B.coef[size_t(e) * nv * nb], B.ref.phi.data(), vals);
      if (P.ns()) { gvals.resize(size_t(nq) * nr); interp(nr, nb, nq, &B.gc[size_t(e) * nr * nb], B.ref.phi.data(), gvals.data()); }
      std::vector<Real> avg;
      if (P.av) { avg.resize(size_t(nq) * nr); interp(nr, nb, nq, &B.vgc[size_t(e) * nr * nb], B.ref.phi.data(), avg.data()); }
      Real* Q = &B.qvol[size_t(e) * nv * nq * d];
      for (int q = 0; q < nq; ++q) {
        PointVar v; for (int i = 0; i < nv; ++i) v.cons[i] = vals[q * nv + i];
        computationalFromConserved(P.ph, v);
        Real F[3][kMaxVar]; rawFlux(P.ph, v, F);
        if (P.ns()) {
          Real pg[15]; primitiveGradient(P.ph, v, &gvals[size_t(q) * nr], pg);
          for (int k = 0; k < d; ++k) {
            Real nk[3] = {0, 0, 0}; nk[k] = 1.0;
            Real fv[kMaxVar]; viscousNormalFlux(P.ph, nk, v, pg, fv);
            for (int i = 0; i < nv; ++i) F[k][i] -= fv[i];
          }
        }
        if (P.av) {  // eps(x_q) times the volume gradient (ViscousFlux.cpp:105-113)
          Real eq = 0;
          for (int k = 0; k < B.ref.nvert; ++k) eq += B.ref.nodal[size_t(q) * B.ref.nvert + k] * B.epsV[size_t(e) * B.ref.nvert + k];
          for (int k = 0; k < d; ++k)
            for (int i = 0; i < nv; ++i) F[k][i] -= eq * avg[size_t(q) * nr + i * d + k];
        }
        const Real* M = &B.jtiw[(size_t(e) * nq + q) * d * d];
        for (int i = 0; i < nv; ++i)
          for (int bb = 0; bb < d; ++bb) {
            Real s = 0; for (int a = 0; a < d; ++a) s += F[a][i] * M[a + bb * d];
            Q[size_t(q * d + bb) * nv + i] = s;
          }
        if (P.ph.source) {  // rho beta (T - Tref) g on the last momentum component, times |J| w
          Real* S = &B.qsrc[(size_t(e) * nq + q) * nv];
          for (int i = 0; i < nv; ++i) S[i] = 0.0;
          S[d] = v.rho * P.ph.beta * (P.ph.temperatureFromInternalEnergy(v.e) - P.ph.tref) * kBoussinesqGravity *
                 B.jw[size_t(e) * nq + q];
        }
      }
    }
  }
  const int nfq = P.nfq();
  // interior faces (SpatialDiscrete.cpp:633-748)
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(P.interior.size()); ++i) {
    const Face& F = P.interior[i];
    if (!faceNeeded(P, F, 0)) continue;
    PointVar L[64], R[64];
    trace(P, F.bl, F.el, F.fl, L); trace(P, F.br, F.er, F.fr, R);
    Block& BL = P.blocks[F.bl]; Block& BR = P.blocks[F.br];
    const std::vector<int>& perm = BR.ref.perm[F.rot];
    std::vector<Real> gl, gr;
    if (P.ns()) {
      gl.resize(size_t(nfq) * nr); gr.resize(size_t(nfq) * nr);
      gradientTrace(P, F.bl, F.el, F.fl, gl.data()); gradientTrace(P, F.br, F.er, F.fr, gr.data());
    }
    std::vector<Real> al, ar, el_, er_;
    if (P.av) {
      al.resize(size_t(nfq) * nr); ar.resize(size_t(nfq) * nr); el_.resize(nfq); er_.resize(nfq);
      volumeGradientTrace(P, F.bl, F.el, F.fl, al.data()); volumeGradientTrace(P, F.br, F.er, F.fr, ar.data());
      faceViscosity(P, F.bl, F.el, F.fl, el_.data()); faceViscosity(P, F.br, F.er, F.fr, er_.data());
    }
    Real* QL = &BL.qface[size_t(F.el) * nv * BL.ref.nface * nfq];
    Real* QR = &BR.qface[size_t(F.er) * nv * BR.ref.nface * nfq];
    for (int j = 0; j < nfq; ++j) {
      const int jr = perm[j];
      const Real* n = &F.normal[j * 3];
      Real h[kMaxVar]; convectiveFlux(P.ph, P.flux, n, L[j], R[jr], h);
      if (P.ns()) {
        Real pl[15], pr[15], fl[kMaxVar], fr[kMaxVar];
        primitiveGradient(P.ph, L[j], &gl[size_t(j) * nr], pl);
        primitiveGradient(P.ph, R[jr], &gr[size_t(jr) * nr], pr);
        viscousNormalFlux(P.ph, n, L[j], pl, fl); viscousNormalFlux(P.ph, n, R[jr], pr, fr);
        for (int v = 0; v < nv; ++v) h[v] -= (fl[v] + fr[v]) / 2.0;
      }
      if (P.av) {  // central artificial viscous flux (ViscousFlux.cpp:183-197)
        for (int v = 0; v < nv; ++v) {
          Real sl = 0, sr = 0;
          for (int k = 0; k < d; ++k) {
            sl += el_[j] * al[size_t(j) * nr + v * d + k] * n[k];
            sr += er_[jr] * ar[size_t(jr) * nr + v * d + k] * n[k];
          }
          h[v] -= (sl + sr) / 2.0;
        }
      }
      for (int v = 0; v < nv; ++v) {
        const Real t = h[v] * F.fjw[j];
        QL[size_t(F.fl * nfq + j) * nv + v] = t;
        QR[size_t(F.fr * nfq + jr) * nv + v] = -t;
      }
    }
  }
  // boundary faces (SpatialDiscrete.cpp:750-842)
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(P.boundary.size()); ++i) {
    const Face& F = P.boundary[i];
    if (!faceNeeded(P, F, 0)) continue;
    PointVar L[64];
    trace(P, F.bl, F.el, F.fl, L);
    Block& BL = P.blocks[F.bl];
    std::vector<Real> gl;
    if (P.ns()) { gl.resize(size_t(nfq) * nr); gradientTrace(P, F.bl, F.el, F.fl, gl.data()); }
    std::vector<Real> al, el_;
    if (P.av) {
      al.resize(size_t(nfq) * nr); el_.resize(nfq);
      volumeGradientTrace(P, F.bl, F.el, F.fl, al.data()); faceViscosity(P, F.bl, F.el, F.fl, el_.data());
    }
    Real* QL = &BL.qface[size_t(F.el) * nv * BL.ref.nface * nfq];
    for (int j = 0; j < nfq; ++j) {
      const Real* n = &F.normal[j * 3];
      PointVar b{};
      boundaryState(P.ph, F.bc, n, L[j], P.dummy[size_t(i) * nfq + j], b);
      Real h[kMaxVar]; normalFlux(P.ph, n, b, h);
      if (P.ns()) {
        Real pl[15]; primitiveGradient(P.ph, L[j], &gl[size_t(j) * nr], pl);
        Real pb[15]; std::copy_n(pl, nr, pb);
        PointVar lm = L[j];
        if (F.bc >= 3) { lm.rho = b.rho; for (int k = 0; k < 3; ++k) lm.u[k] = b.u[k]; lm.e = b.e; lm.p = b.p; }
        if (F.bc >= 4) for (int k = 0; k < d; ++k) pb[(d + 1) * d + k] = 0.0;
        Real fl[kMaxVar], fb[kMaxVar];
        viscousNormalFlux(P.ph, n, lm, pl, fl); viscousNormalFlux(P.ph, n, b, pb, fb);
        for (int v = 0; v < nv; ++v) h[v] -= (fl[v] + fb[v]) / 2.0;
      }
      if (P.av)  // the interior side's artificial viscous flux only (SpatialDiscrete.cpp:815-834)
        for (int v = 0; v < nv; ++v) {
          Real s = 0;
          for (int k = 0; k < d; ++k) s += el_[j] * al[size_t(j) * nr + v * d + k] * n[k];
          h[v] -= s;
        }
      for (int v = 0; v < nv; ++v) QL[size_t(F.fl * nfq + j) * nv + v] = h[v] * F.fjw[j];
    }
  }
  // residual (SpatialDiscrete.cpp:1016-1032)
  for (Block& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb, nfl = B.ref.nface * nfq;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      if (!needed(B, e, 0)) continue;
      const Real* QV = &B.qvol[size_t(e) * nv * nq * d];
      const Real* QF = &B.qface[size_t(e) * nv * nfl];
      Real* Rr = &B.res[size_t(e) * nv * nb];
      for (int i = 0; i < nv * nb; ++i) Rr[i] = 0;
      gemmAcc(nv, nq * d, nb, QV, B.ref.dphi.data(), Rr, 1);
      gemmAcc(nv, nfl, nb, QF, B.ref.phif.data(), Rr, -1);
      if (P.ph.source) gemmAcc(nv, nq, nb, &B.qsrc[size_t(e) * nv * nq], B.ref.phi.data(), Rr, 1);
    }
  }
}

static const Real kRk[3][3][3] = {
    {{1.0, 0.0, 1.0}, {0, 0, 0}, {0, 0, 0}},
    {{1.0, 0.0, 1.0}, {0.5, 0.5, 0.5}, {0, 0, 0}},
    {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}}};  // TimeIntegration.cpp:45-65

static void update(Problem& P, int stage, Real dt) {
  const int nv = P.nv;
  const Real* c = kRk[P.rk][stage];
  for (Block& B : P.blocks) {
    const int nb = B.ref.nb;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      Real* U = &B.coef[size_t(e) * nv * nb];
      const Real* L = &B.last[size_t(e) * nv * nb];
      const Real* Rr = &B.res[size_t(e) * nv * nb];
      std::vector<Real> du(size_t(nv) * nb);
      applyMinv(P, B, e, nv, Rr, du.data());
      for (int i = 0; i < nv * nb; ++i) U[i] *= c[1];
      for (int i = 0; i < nv * nb; ++i) U[i] += c[0] * L[i];
      for (int i = 0; i < nv * nb; ++i) U[i] += c[2] * dt * du[i];
    }
  }
}

static void relativeError(Problem& P) {
  const int nv = P.nv;
  std::vector<Real> acc(nv, 0.0);
  for (Block& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb;
    std::vector<Real> part(size_t(omp_get_max_threads()) * nv, 0.0);
#pragma omp parallel
    {
      Real* my = &part[size_t(omp_get_thread_num()) * nv];
#pragma omp for schedule(static)
      for (int64_t e = 0; e < B.ne; ++e) {
        Real vals[216 * kMaxVar];
        interp(nv, nb, nq, &B.res[size_t(e) * nv * nb], B.ref.phi.data(), vals);
        for (int v = 0; v < nv; ++v) {
          Real s = 0; for (int q = 0; q < nq; ++q) s += std::fabs(vals[q * nv + v]);
          my[v] += s / nq;
        }
      }
    }
    for (size_t t = 0; t < part.size() / nv; ++t)
      for (int v = 0; v < nv; ++v) acc[v] += part[t * nv + v];
  }
  for (int v = 0; v < nv; ++v) P.relErr[v] = acc[v] / Real(P.totalElements);
}

// One RK stage s of Solver::stepSolver (TimeIntegration.cpp:339-347); stage 0 first saves U^n
// (TimeIntegration.cpp:70-102) and evaluates the once-per-step artificial viscosity (:336-338).
static void stage(Problem& P, int s, Real dt) {
  if (s == 0) {
    for (Block& B : P.blocks) B.last = B.coef;
    if (P.av) artificialViscosity(P);
  }
  if (P.gradientPass()) gradientQuadratureAndResidual(P);
  quadratureAndResidual(P);
  update(P, s, dt);
}

static void step(Problem& P, Real dt) {
  const int nstage = P.rk + 1;
  for (int s = 0; s < nstage; ++s) stage(P, s, dt);
  relativeError(P);
}

// LSQ projection of point values (InitialCondition.cpp:91-104): coef = U_q Phi (Phi^T Phi)^-1.
static void project(Problem& P, const Real* cons) {
  const int nv = P.nv;
  size_t off = 0;
  for (Block& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      if (!needed(B, e, 2)) continue;
      const Real* u = &cons[(off + size_t(e) * nq) * nv];
      std::vector<Real> t(size_t(nv) * nb, 0.0);
      for (int b = 0; b < nb; ++b)
        for (int v = 0; v < nv; ++v) {
          Real s = 0; for (int q = 0; q < nq; ++q) s += u[q * nv + v] * B.ref.phi[size_t(q) * nb + b];
          t[b * nv + v] = s;
        }
      Real* U = &B.coef[size_t(e) * nv * nb];
      for (int b = 0; b < nb; ++b)
        for (int v = 0; v < nv; ++v) {
          Real s = 0; for (int k = 0; k < nb; ++k) s += t[k * nv + v] * B.ref.lsqInv[size_t(k) * nb + b];
          U[b * nv + v] = s;
        }
      if (P.refine) {  // one correction step of the normal equations (Phi^T Phi) c = Phi^T u
        std::vector<Real> r(size_t(nv) * nb);
        for (int b = 0; b < nb; ++b)
          for (int v = 0; v < nv; ++v) {
            Real s = t[b * nv + v];
            for (int k = 0; k < nb; ++k) s -= U[k * nv + v] * B.ref.ptp[size_t(k) * nb + b];
            r[b * nv + v] = s;
          }
        for (int b = 0; b < nb; ++b)
          for (int v = 0; v < nv; ++v) {
            Real s = 0; for (int k = 0; k < nb; ++k) s += r[k * nv + v] * B.ref.lsqInv[size_t(k) * nb + b];
            U[b * nv + v] += s;
          }
      }
    }
    off += size_t(B.ne) * nq;
  }
  P.hasState = true;
}

// Levels of the element-sample mode: the sampled elements (0), their face neighbours (1: their gradients when
// the gradient pass runs, else their coefficients only) and, with the gradient pass, the neighbours of those (2).
static void sampleLevels(Problem& P, int64_t count, const int64_t* sample) {
  for (Block& B : P.blocks) B.level.assign(size_t(B.ne), 3);
  std::vector<int64_t> first(P.blocks.size() + 1, 0);
  for (size_t b = 0; b < P.blocks.size(); ++b) first[b + 1] = first[b] + P.blocks[b].ne;
  for (int64_t i = 0; i < count; ++i) {
    const int64_t g = sample[i];
    if (g < 0 || g >= first.back()) throw std::runtime_error("sampled element index out of range");
    const size_t b = size_t(std::upper_bound(first.begin(), first.end(), g) - first.begin()) - 1;
    P.blocks[b].level[size_t(g - first[b])] = 0;
  }
  const int rings = P.gradientPass() ? 2 : 1;
  for (int ring = 1; ring <= rings; ++ring) {
    const int lvl = ring == rings ? 2 : 1;
    std::vector<std::pair<int, int>> mark;
    for (const Face& F : P.interior) {
      const signed char l = P.blocks[F.bl].level[F.el], r = P.blocks[F.br].level[F.er];
      if (l < ring && r > lvl) mark.push_back({F.br, F.er});
      if (r < ring && l > lvl) mark.push_back({F.bl, F.el});
    }
    for (const auto& [b, e] : mark) P.blocks[b].level[size_t(e)] = std::min<signed char>(P.blocks[b].level[size_t(e)], lvl);
  }
}

static Problem* create(const sdg_mesh* m, const sdg_config* c, int flags, int64_t sampleCount = 0,
                       const int64_t* sample = nullptr) {
  auto P = std::make_unique<Problem>();
  const int faithful = flags & 1;
  P->refine = (flags & 2) == 0;
  P->lean = (flags & 4) != 0;
  P->dim = m->dimension; P->nv = P->dim + 2; P->p = c->polynomial_order;
  P->eq = c->equation; P->flux = c->convective_flux; P->visc = c->viscous_flux; P->rk = c->time_integration;
  P->faithful = faithful != 0;
  P->ph.dim = P->dim; P->ph.gamma = c->specific_heat_ratio; P->ph.cp = c->specific_heat_constant_pressure;
  P->ph.cv = c->specific_heat_constant_volume; P->ph.mu = c->dynamic_viscosity; P->ph.pr = c->prandtl_number;
  P->ph.transport = c->transport_model;
  P->ph.kappa = P->ph.cp * P->ph.mu / P->ph.pr;  // PhysicalModel.cpp:149-153
  P->ph.incomp = c->equation == SDG_INCOMPRESSIBLE_EULER || c->equation == SDG_INCOMPRESSIBLE_NS;
  if (P->ph.incomp) {  // PhysicalModel.cpp:57-78
    P->ph.c0 = c->reference_sound_speed; P->ph.rho0 = c->reference_density;
    P->ph.padd = kWeakPressureAddition * P->ph.rho0 * P->ph.c0 * P->ph.c0;
    if (P->flux == SDG_FLUX_HLLC || P->flux == SDG_FLUX_ROE) throw std::runtime_error("HLLC/Roe need the ideal gas");
  } else if (P->flux == SDG_FLUX_EXACT) {
    throw std::runtime_error("the Exact flux belongs to the incompressible models");
  }
  P->av = c->shock_capturing == SDG_SHOCK_ARTIFICIAL_VISCOSITY;  // SystemControl.cpp:105-108
  P->avTol = c->empirical_tolerance; P->avFactor = c->artificial_viscosity_factor;
  if (P->av && !(P->avTol > 0)) throw std::runtime_error("artificial viscosity needs empirical_tolerance > 0");
  P->ph.source = c->source_term;
  P->ph.beta = c->thermal_expansion_coefficient; P->ph.tref = c->reference_temperature;
  if (P->ns() && P->visc == 0) throw std::runtime_error("NS needs BR1 or BR2");
  struct Src { int type; int64_t n; const int32_t* v; };
  std::vector<Src> src;
  if (P->dim == 1) src.push_back({kLine, m->line_count, m->line_node});
  else if (P->dim == 2) { src.push_back({kTri, m->triangle_count, m->triangle_node}); src.push_back({kQuad, m->quadrangle_count, m->quadrangle_node}); }
  else { src.push_back({kTet, m->tetrahedron_count, m->tetrahedron_node}); src.push_back({kHex, m->hexahedron_count, m->hexahedron_node}); }
  for (const Src& s : src) {
    if (s.n <= 0) continue;
    Block B; B.type = s.type; B.ne = s.n;
    B.ref.build(s.type, P->p);
    B.verts.assign(s.v, s.v + size_t(s.n) * elemVerts(s.type));
    const int32_t* g = s.type == kTri ? m->triangle_geometry_node
                       : s.type == kQuad ? m->quadrangle_geometry_node
                       : s.type == kHex ? m->hexahedron_geometry_node : nullptr;
    if (m->geometry_order > 1 && g) {  // curved geometry (ReadControl.cpp:243-256)
      B.curved = true;
      B.geoOrder = m->geometry_order;
      B.cb.init(s.type, B.geoOrder);
      B.geo.assign(g, g + size_t(s.n) * B.cb.nn);
    }
    P->blocks.push_back(std::move(B));
  }
  if (P->blocks.empty()) throw std::runtime_error("mesh has no elements");
  buildAdjacency(*P, *m);
  if (sample) {
    if (P->lean || P->av) throw std::runtime_error("the element-sample mode has no lean or artificial-viscosity form");
    P->sampled = true;
    sampleLevels(*P, sampleCount, sample);
  }
  for (Block& B : P->blocks) {
    buildGeometry(*P, B, m->node_coordinate);
    P->totalElements += B.ne;
    const int nv = P->nv, nb = B.ref.nb, nq = B.ref.nq, d = P->dim, nr = nv * d, nfl = B.ref.nface * B.ref.nfq;
    B.coef.assign(size_t(B.ne) * nv * nb, 0.0); B.last = B.coef; B.res = B.coef;
    B.qvol.assign(size_t(B.ne) * nv * nq * d, 0.0);
    B.qface.assign(size_t(B.ne) * nv * nfl, 0.0);
    if (P->ph.source) B.qsrc.assign(size_t(B.ne) * nv * nq, 0.0);
    if (P->av) B.epsV.assign(size_t(B.ne) * B.ref.nvert, 0.0);
    if (P->gradientPass()) {
      B.qvg.assign(size_t(B.ne) * nr * nq * d, 0.0);
      B.qfvg.assign(size_t(B.ne) * nr * nfl, 0.0);
      B.rvg.assign(size_t(B.ne) * nr * nb, 0.0);
      B.vgc.assign(size_t(B.ne) * nr * nb, 0.0);
    }
    if (P->ns()) {
      const int nblk = P->visc == 1 ? 1 : B.ref.nface;
      B.qfig.assign(size_t(B.ne) * nr * nfl, 0.0);
      B.rig.assign(size_t(B.ne) * nblk * nr * nb, 0.0);
      B.igc.assign(size_t(B.ne) * nblk * nr * nb, 0.0);
      B.gc.assign(size_t(B.ne) * nr * nb, 0.0);
    }
  }
  if (P->av) P->nodeAV.assign(size_t(m->node_count), 0.0);
  const int faceLevel = P->gradientPass() ? 1 : 0;
  for (Face& F : P->interior)
    if (faceNeeded(*P, F, faceLevel)) faceGeometry(*P, F, m->node_coordinate);
  for (Face& F : P->boundary)
    if (faceNeeded(*P, F, faceLevel)) faceGeometry(*P, F, m->node_coordinate);
  P->dummy.assign(P->boundary.size() * size_t(P->nfq()), PointVar{});
  P->relErr.assign(P->nv, 0.0);
  return P.release();
}

}  // namespace orc

// ---- C interface for the tests and the CPU baseline ------------------------------------------------
// Only these symbols are exported (the library is built with -fvisibility=hidden), so the double and
// long-double builds can be loaded into one process without their C++ internals interposing.
#pragma GCC visibility push(default)
extern "C" {

struct orc_handle { orc::Problem* p; };

static thread_local std::string g_orc_error;

const char* orc_last_error() { return g_orc_error.c_str(); }

// flags: bit 0 = run the gradient pass also for Euler (as the reference does); bit 1 = multiply by the
// plain explicit inverses (no refinement), i.e. the reference's arithmetic; bit 2 (with bit 1) = lean: blocks
// of affine elements use one shared reference inverse scaled by 1/|J| instead of a dense inverse per element.
// The timed CPU baselines use 3 (reference-faithful) and 6 (lean: no Euler gradient pass, shared inverse);
// the parity checker uses 0.
void* orc_create(const sdg_mesh* mesh, const sdg_config* config, int flags) {
  try {
    return orc::create(mesh, config, flags);
  } catch (const std::exception& e) {
    g_orc_error = e.what();
    return nullptr;
  }
}

// Element-sample mode (test infrastructure for meshes too large for the long-double build): only the residual
// of the `count` elements listed (global indices in block order) is evaluated, with exactly the arithmetic of
// the full evaluation -- a residual is local to an element and its face neighbours, so on the sampled elements
// it equals the full evaluation's.  Geometry, inverses and the projection of the initial state are computed
// only where that residual needs them.  Supports the initial state, the boundary state and orc_residual_point
// (zeros outside the sample); stepping, dt and relative errors are refused.
void* orc_create_sampled(const sdg_mesh* mesh, const sdg_config* config, int flags, int64_t count,
                         const int64_t* elements) {
  try {
    if (!elements || count <= 0) throw std::runtime_error("empty element sample");
    return orc::create(mesh, config, flags, count, elements);
  } catch (const std::exception& e) {
    g_orc_error = e.what();
    return nullptr;
  }
}

void orc_destroy(void* h) { delete static_cast<orc::Problem*>(h); }

void orc_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }
int orc_max_threads() { return omp_get_max_threads(); }

// Constants of the restated model, for the checks against the reference's own tables.
double orc_constant(const char* name) {
  const std::string n(name ? name : "");
  if (n == "weak_pressure_addition") return double(orc::kWeakPressureAddition);
  if (n == "boussinesq_gravity") return double(orc::kBoussinesqGravity);
  for (int p = 1; p <= 5; ++p)
    if (n == "artificial_viscosity_tolerance_" + std::to_string(p)) return double(orc::kAvTolerance[p - 1]);
  return std::numeric_limits<double>::quiet_NaN();
}
int orc_real_digits() { return std::numeric_limits<orc::Real>::digits; }

// counts: [element_count, volume_point_count, interior_faces, boundary_faces, nfq, dof]
void orc_counts(void* h, int64_t* out) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  int64_t vp = 0, dof = 0;
  for (const auto& B : P.blocks) { vp += B.ne * B.ref.nq; dof += B.ne * B.ref.nb * P.nv; }
  out[0] = P.totalElements; out[1] = vp; out[2] = int64_t(P.interior.size()); out[3] = int64_t(P.boundary.size());
  out[4] = P.nfq(); out[5] = dof;
}

void orc_volume_point_coordinate(void* h, double* out) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  size_t off = 0;
  for (const auto& B : P.blocks) { std::copy(B.qcoord.begin(), B.qcoord.end(), out + off); off += B.qcoord.size(); }
}

void orc_boundary_point_coordinate(void* h, double* out, int32_t* physical) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  const int nfq = P.nfq();
  for (size_t i = 0; i < P.boundary.size(); ++i) {
    std::copy(P.boundary[i].coord.begin(), P.boundary[i].coord.end(), out + i * nfq * 3);
    if (physical) physical[i] = P.boundary[i].physical;
  }
}

int orc_set_initial_primitive(void* h, const double* prim) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  int64_t c[6]; orc_counts(h, c);
  std::vector<orc::Real> cons(size_t(c[1]) * P.nv);
  for (int64_t q = 0; q < c[1]; ++q) {
    orc::Real pr[orc::kMaxVar];
    for (int i = 0; i < P.nv; ++i) pr[i] = prim[q * P.nv + i];
    orc::PointVar v; orc::fromPrimitive(P.ph, pr, v);
    for (int i = 0; i < P.nv; ++i) cons[q * P.nv + i] = v.cons[i];
  }
  orc::project(P, cons.data());
  return 0;
}

int orc_set_state_point(void* h, const double* cons) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  int64_t c[6]; orc_counts(h, c);
  std::vector<orc::Real> v(cons, cons + size_t(c[1]) * P.nv);
  orc::project(P, v.data());
  return 0;
}

int orc_set_boundary_primitive(void* h, const double* prim) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  for (size_t i = 0; i < P.dummy.size(); ++i) {
    orc::Real pr[orc::kMaxVar];
    for (int k = 0; k < P.nv; ++k) pr[k] = prim[i * P.nv + k];
    orc::fromPrimitive(P.ph, pr, P.dummy[i]);
  }
  return 0;
}

int orc_get_state_point(void* h, double* out) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  size_t off = 0;
  for (const auto& B : P.blocks) {
    std::vector<orc::Real> tmp(size_t(B.ref.nq) * P.nv);
    for (int64_t e = 0; e < B.ne; ++e) {
      orc::interp(P.nv, B.ref.nb, B.ref.nq, &B.coef[size_t(e) * P.nv * B.ref.nb], B.ref.phi.data(), tmp.data());
      std::copy(tmp.begin(), tmp.end(), out + (off + size_t(e) * B.ref.nq) * P.nv);
    }
    off += size_t(B.ne) * B.ref.nq;
  }
  return 0;
}

int orc_get_state_modal(void* h, double* out) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  size_t off = 0;
  for (const auto& B : P.blocks) { std::copy(B.coef.begin(), B.coef.end(), out + off); off += B.coef.size(); }
  return 0;
}

int orc_calculate_delta_time(void* h, double cfl, double* dt) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  if (P.sampled) return 1;
  orc::Real best = 1.79769313486231570e308;
  for (const auto& B : P.blocks) {
    const int nq = B.ref.nq, nb = B.ref.nb;
    for (int64_t e = 0; e < B.ne; ++e) {
      orc::Real vals[216 * orc::kMaxVar];
      orc::interp(P.nv, nb, nq, &B.coef[size_t(e) * P.nv * nb], B.ref.phi.data(), vals);
      for (int q = 0; q < nq; ++q) {
        orc::PointVar v; for (int i = 0; i < P.nv; ++i) v.cons[i] = vals[q * P.nv + i];
        orc::computationalFromConserved(P.ph, v);
        const orc::Real c = P.ph.soundSpeed(v.rho, v.p);
        const orc::Real sr = std::sqrt(v.u2(P.dim)) + c;
        const orc::Real t = orc::Real(cfl) * B.minEdge[e] / (sr * (P.p + 1.0) * (P.p + 1.0));  // TimeIntegration.cpp:119-125
        best = std::min(best, t);
      }
    }
  }
  *dt = best;
  return 0;
}

int orc_step(void* h, int n, double dt) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  if (P.sampled) return 1;
  for (int i = 0; i < n; ++i) orc::step(P, orc::Real(dt));
  return 0;
}

// One RK stage (0 .. stages-1) of a step; the last stage also evaluates the step's relative error.
int orc_stage(void* h, int s, double dt) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  if (s < 0 || s > P.rk || P.sampled) return 1;
  orc::stage(P, s, orc::Real(dt));
  if (s == P.rk) orc::relativeError(P);
  return 0;
}

int orc_relative_error(void* h, double* out) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  std::copy(P.relErr.begin(), P.relErr.end(), out);
  return 0;
}

// du/dt at the volume points for the current state (one residual evaluation, no update).
int orc_residual_point(void* h, double* out) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  if (P.av) orc::artificialViscosity(P);
  if (P.gradientPass()) orc::gradientQuadratureAndResidual(P);
  orc::quadratureAndResidual(P);
  size_t off = 0;
  for (auto& B : P.blocks) {
    const int nb = B.ref.nb, nq = B.ref.nq, nv = P.nv;
    for (int64_t e = 0; e < B.ne; ++e) {
      if (!orc::needed(B, e, 0)) {
        std::fill(out + (off + size_t(e) * nq) * nv, out + (off + size_t(e + 1) * nq) * nv, 0.0);
        continue;
      }
      std::vector<orc::Real> du(size_t(nv) * nb), tmp(size_t(nq) * nv);
      orc::applyMinv(P, B, e, nv, &B.res[size_t(e) * nv * nb], du.data());
      orc::interp(nv, nb, nq, du.data(), B.ref.phi.data(), tmp.data());
      std::copy(tmp.begin(), tmp.end(), out + (off + size_t(e) * nq) * nv);
    }
    off += size_t(B.ne) * nq;
  }
  return 0;
}

// Artificial viscosity of the current state at every mesh node (zeros without shock capturing).
int orc_node_artificial_viscosity(void* h, double* out) {
  orc::Problem& P = *static_cast<orc::Problem*>(h);
  if (!P.av) return 0;
  orc::artificialViscosity(P);
  for (size_t i = 0; i < P.nodeAV.size(); ++i) out[i] = double(P.nodeAV[i]);
  return 0;
}

// Canonical adjacency tuples, sorted (same definition as sdg_adjacency).
int orc_adjacency(void* h, int32_t* interior, int32_t* boundary) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  std::vector<std::array<int32_t, 7>> in;
  for (const auto& F : P.interior)
    in.push_back({P.blocks[F.bl].type, F.el, F.fl, P.blocks[F.br].type, F.er, F.fr, F.rot});
  std::sort(in.begin(), in.end());
  for (size_t i = 0; i < in.size(); ++i) std::copy(in[i].begin(), in[i].end(), interior + i * 7);
  std::vector<std::array<int32_t, 5>> bd;
  for (const auto& F : P.boundary) bd.push_back({P.blocks[F.bl].type, F.el, F.fl, F.physical, F.bc});
  std::sort(bd.begin(), bd.end());
  for (size_t i = 0; i < bd.size(); ++i) std::copy(bd[i].begin(), bd[i].end(), boundary + i * 5);
  return 0;
}

// The gradient records of the reference's raw-binary file for Navier-Stokes (src/View/RawBinary.cpp:75-154): per
// element its gradient coefficients (element_out, block order, column-major (d+2)d x Nb), per boundary face in the
// sorted order of orc_adjacency the record of its parent -- BR1: the element's gradient; BR2: the volume gradient
// plus the lift of that face (boundary_out) -- of the last stage input, as the reference holds them after a step.
int orc_raw_gradient(void* h, double* element_out, double* boundary_out) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  if (!P.ns()) return 1;
  const int nr = P.nv * P.dim;
  size_t off = 0;
  for (const auto& B : P.blocks) {
    const size_t n = size_t(B.ne) * nr * B.ref.nb;
    for (size_t i = 0; i < n; ++i) element_out[off + i] = double(B.gc[i]);
    off += n;
  }
  std::vector<std::pair<std::array<int32_t, 5>, const orc::Face*>> bd;
  for (const auto& F : P.boundary) bd.push_back({{P.blocks[F.bl].type, F.el, F.fl, F.physical, F.bc}, &F});
  std::sort(bd.begin(), bd.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  size_t boff = 0;
  for (const auto& kv : bd) {
    const orc::Face& F = *kv.second;
    const auto& B = P.blocks[F.bl];
    const int nb = B.ref.nb, nblk = P.visc == 1 ? 1 : B.ref.nface;
    for (int i = 0; i < nr * nb; ++i) {
      const orc::Real g = P.visc == 1 ? B.gc[size_t(F.el) * nr * nb + i]
                                      : B.vgc[size_t(F.el) * nr * nb + i] +
                                            B.igc[(size_t(F.el) * nblk + F.fl) * nr * nb + i];
      boundary_out[boff + i] = double(g);
    }
    boff += size_t(nr) * nb;
  }
  return 0;
}

// Face normals and |J_f| w of every interior face point, in the sorted order of orc_adjacency
// (for geometry parity checks): [interior][nfq][4] = (nx, ny, nz, |J_f| w).
int orc_interior_face_geometry(void* h, double* out) {
  const orc::Problem& P = *static_cast<orc::Problem*>(h);
  std::vector<std::pair<std::array<int32_t, 7>, size_t>> in;
  for (size_t i = 0; i < P.interior.size(); ++i) {
    const auto& F = P.interior[i];
    in.push_back({{P.blocks[F.bl].type, F.el, F.fl, P.blocks[F.br].type, F.er, F.fr, F.rot}, i});
  }
  std::sort(in.begin(), in.end());
  const int nfq = P.nfq();
  for (size_t i = 0; i < in.size(); ++i) {
    const auto& F = P.interior[in[i].second];
    for (int j = 0; j < nfq; ++j) {
      for (int k = 0; k < 3; ++k) out[(i * nfq + j) * 4 + k] = F.normal[j * 3 + k];
      out[(i * nfq + j) * 4 + 3] = F.fjw[j];
    }
  }
  return 0;
}

}  // extern "C"
#pragma GCC visibility pop
