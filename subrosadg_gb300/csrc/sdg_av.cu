// Artificial-viscosity shock capturing of the GB300 DG path (ShockCapturingEnum::ArtificialViscosity):
// the per-step Persson-Peraire density sensor, the max over the elements sharing each mesh node, and the
// elements' vertex values (src/Solver/SpatialDiscrete.cpp:37-192), run once per step before the stages
// (src/Solver/TimeIntegration.cpp:336-338).  The stage, gradient and face kernels then add the artificial
// viscous flux eps grad U of the volume gradient (ViscousFlux.cpp:105-200).
//
// Sensor of element e (SpatialDiscrete.cpp:46-88):
//   s = log10( int rho_h^2 / int rho^2 ),  rho_h = the degree-P modes of the density (P1: the density),
//   eps = 0 for s < s0 - kappa, eps0 h/P for s > s0 + kappa, eps0 h/P (1 + sin(pi (s - s0)/(2 kappa)))/2 between,
// with s0 per order (SimulationControl.cpp:892-893), h the element's inner radius, kappa the empirical
// tolerance and eps0 the factor of System::setArtificialViscosity.  Integrals use the volume rule (|J| w).
// Tensor blocks hold nodal values at the Gauss points: the modal coefficients are (Phi1^-1)^{(x)d} rho, the
// degree-P modes those with a Lobatto index equal to P along some axis.
//
// The node field is a max over elements: a non-negative double orders like its bit pattern, so the max is
// an integer atomicMax on the 64-bit representation.
#include <cmath>
#include <cstring>
#include <vector>

#include "sdg_internal.hpp"
#include "sdg_kernels_dense.cuh"

namespace sdg {
namespace {

constexpr int kAvThreads = 128;
constexpr int kAvMaxNb = 216;

__device__ double avTensorSensor(const AvArgs& a, int64_t e) {
  const int n = a.n, nb = a.nb, dim = a.dim;
  const double* w = a.tab + n;
  const double* phi1 = a.tab + 2 * n;
  const double* phi1inv = phi1 + n * n;
  double rho[kAvMaxNb], c[kAvMaxNb], t[kAvMaxNb];
  const double* u = a.u + e * a.ustride;
  for (int i = 0; i < nb; ++i) { rho[i] = u[i]; c[i] = u[i]; }
  const int strides[3] = {dim == 1 ? 1 : (dim == 2 ? n : n * n), dim == 2 ? 1 : n, 1};
  // nodal -> modal along each axis
  for (int ax = 0; ax < dim; ++ax) {
    const int st = strides[ax];
    for (int b = 0; b < nb; ++b) {
      const int ib = (b / st) % n, base = b - ib * st;
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = fma(phi1inv[ib * n + k], c[base + k * st], s);
      t[b] = s;
    }
    for (int b = 0; b < nb; ++b) c[b] = t[b];
  }
  // keep the degree-P modes
  for (int b = 0; b < nb; ++b) {
    int top = 0;
    for (int ax = 0; ax < dim; ++ax) top = max(top, (b / strides[ax]) % n);
    if (a.p > 1 && top != a.p) c[b] = 0.0;  // P1: the whole density (SpatialDiscrete.cpp:51-52)
  }
  // back to the nodes
  for (int ax = 0; ax < dim; ++ax) {
    const int st = strides[ax];
    for (int b = 0; b < nb; ++b) {
      const int ib = (b / st) % n, base = b - ib * st;
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = fma(phi1[ib * n + k], c[base + k * st], s);
      t[b] = s;
    }
    for (int b = 0; b < nb; ++b) c[b] = t[b];
  }
  const int gs = dim * dim + 1;
  double num = 0.0, den = 0.0;
  for (int b = 0; b < nb; ++b) {
    double wb = 1.0;
    for (int ax = 0; ax < dim; ++ax) wb *= w[(b / strides[ax]) % n];
    const double jinv = a.affine ? a.geom[e * gs + dim * dim] : a.geom[(e * nb + b) * gs + dim * dim];
    const double jw = wb / jinv;
    num = fma(c[b], c[b] * jw, num);
    den = fma(rho[b], rho[b] * jw, den);
  }
  return num / den;
}

__device__ double avDenseSensor(const AvArgs& a, int64_t e) {
  const int nb = a.nb, nq = a.nq;
  const double* phi = a.tab;
  const double* high = phi + nq * nb;
  const double* w = high + nb;
  const double* c = a.u + e * a.ustride;  // density: the first nb modal coefficients
  const int gs = a.dim * a.dim + 1, gstride = a.affine ? gs : nq * gs + nb * nb;
  double num = 0.0, den = 0.0;
  for (int q = 0; q < nq; ++q) {
    double all = 0.0, hi = 0.0;
    for (int b = 0; b < nb; ++b) {
      const double x = phi[q * nb + b] * c[b];
      all += x;
      hi += high[b] * x;
    }
    const double jinv = a.affine ? a.geom[e * gstride + gs - 1] : a.geom[e * gstride + q * gs + gs - 1];
    const double jw = w[q] / jinv;
    num = fma(hi, hi * jw, num);
    den = fma(all, all * jw, den);
  }
  return num / den;
}

// One CTA-sized chunk `block` of a pass (thread t = block * blockDim + threadIdx).
__device__ __forceinline__ void avBody(const AvArgs& a, int64_t block) {
  const int64_t t = block * blockDim.x + threadIdx.x;
  if (a.kind == 0) {
    if (t < a.nodes) a.nodeAV[t] = 0.0;
    return;
  }
  if (a.kind == 3) {
    if (t < a.ne * a.nvert) a.epsV[t] = a.nodeAV[a.vert[t]];
    return;
  }
  if (t >= a.ne) return;
  const double ratio = a.kind == 1 ? avTensorSensor(a, t) : avDenseSensor(a, t);
  const double sc = log10(ratio);
  const double full = a.factor * (a.inner[t] / double(a.p));
  double eps;
  if (sc < a.s0 - a.kappa) eps = 0.0;
  else if (sc > a.s0 + a.kappa) eps = full;
  else eps = full * (1.0 + sin(3.141592653589793 * (sc - a.s0) / (2.0 * a.kappa))) / 2.0;
  eps = fmax(eps, 0.0);  // +0 for the integer max (NaN propagates)
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(eps));
  for (int v = 0; v < a.nvert; ++v)
    atomicMax(reinterpret_cast<unsigned long long*>(a.nodeAV + a.vert[t * a.nvert + v]), bits);
}

__global__ void __launch_bounds__(kAvThreads) avKernel(AvArgs a) { avBody(a, blockIdx.x); }

// Batched: CTA c runs work items c, c + gridDim.x, ... of (argument set, chunk) pairs over many instances (the
// instances' node fields are disjoint, so one level of a batch runs every instance's pass at once).
__global__ void __launch_bounds__(kAvThreads)
    avBatchKernel(const AvArgs* __restrict__ args, const int2* __restrict__ items, int nitems) {
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const int2 it = items[w];
    avBody(args[it.x], it.y);
  }
}

// s0 per order (SimulationControl.cpp:892-893)
const double kAvTolerance[5] = {0.0, -1.20411998266, -1.90848501888, -2.40823996531, -2.79588001734};

double norm3(const double* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
double crossNorm(const double* a, const double* b) {
  const double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  return norm3(c);
}

Rec avRec(int kind, int64_t count) {
  Rec r;
  r.kind = kRecAv; r.cls = 4;
  r.fn = reinterpret_cast<const void*>(&avKernel); r.bfn = reinterpret_cast<const void*>(&avBatchKernel);
  r.threads = kAvThreads; r.epb = 1; r.smem = 0;
  r.units = (count + kAvThreads - 1) / kAvThreads;
  std::memset(&r.av, 0, sizeof(r.av));
  r.av.kind = kind;
  return r;
}

}  // namespace

// Inner radius (gmsh quality "innerRadius", Geometry.cpp:31-41; gmsh 4.13.1 is not vendored): half the length of
// a line (gmsh MLine), 2A/perimeter for
// triangles and quadrangles (A of a quadrangle from its diagonals), 3V/S for tetrahedra and hexahedra (hexahedra:
// V by 2x2x2 Gauss quadrature of the trilinear map, each face's area from its diagonals); exact for squares and
// cubes.
double innerRadiusOf(int type, const double* nodes, const int32_t* vv) {
  auto sub = [&](int a, int b, double* o) {
    for (int d = 0; d < 3; ++d) o[d] = nodes[size_t(vv[a]) * 3 + d] - nodes[size_t(vv[b]) * 3 + d];
  };
  if (type == SDG_ELEMENT_LINE) {  // gmsh's MLine inner radius: half the length
    double e[3]; sub(1, 0, e);
    return norm3(e) / 2.0;
  }
  if (type == SDG_ELEMENT_TRIANGLE || type == SDG_ELEMENT_QUADRANGLE) {
    const int nv = type == SDG_ELEMENT_TRIANGLE ? 3 : 4;
    double per = 0, e[3];
    for (int i = 0; i < nv; ++i) { sub((i + 1) % nv, i, e); per += norm3(e); }
    double d1[3], d2[3];
    if (type == SDG_ELEMENT_TRIANGLE) { sub(1, 0, d1); sub(2, 0, d2); }
    else { sub(2, 0, d1); sub(3, 1, d2); }
    return crossNorm(d1, d2) / per;
  }
  if (type == SDG_ELEMENT_TETRAHEDRON) {
    double a[3], b[3], c[3];
    sub(1, 0, a); sub(2, 0, b); sub(3, 0, c);
    const double vol = std::fabs(a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                                 a[2] * (b[0] * c[1] - b[1] * c[0])) / 6.0;
    const int* fl = faceVertexList(type);
    double area = 0;
    for (int f = 0; f < 4; ++f) {
      double d1[3], d2[3];
      sub(fl[f * 3 + 1], fl[f * 3], d1); sub(fl[f * 3 + 2], fl[f * 3], d2);
      area += crossNorm(d1, d2) / 2.0;
    }
    return 3.0 * vol / area;
  }
  static const int faces[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {0, 4, 7, 3}, {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};
  double area = 0;
  for (const auto& f : faces) {
    double d1[3], d2[3];
    sub(f[2], f[0], d1); sub(f[3], f[1], d2);
    area += crossNorm(d1, d2) / 2.0;
  }
  static const double sgn[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                   {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const double g = 1.0 / std::sqrt(3.0);
  double vol = 0;
  for (int q = 0; q < 8; ++q) {
    const double xi[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, (q & 4) ? g : -g};
    double J[3][3] = {{0}};
    for (int k = 0; k < 8; ++k) {
      const double a = 1 + sgn[k][0] * xi[0], b = 1 + sgn[k][1] * xi[1], c = 1 + sgn[k][2] * xi[2];
      const double gr[3] = {0.125 * sgn[k][0] * b * c, 0.125 * a * sgn[k][1] * c, 0.125 * a * b * sgn[k][2]};
      for (int l = 0; l < 3; ++l)
        for (int m = 0; m < 3; ++m) J[l][m] += gr[m] * nodes[size_t(vv[k]) * 3 + l];
    }
    vol += J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  }
  return 3.0 * vol / area;
}

// Host tables of block B for the artificial viscosity (avTableLayout in sdg_kernels.cuh).
void buildAvTables(DevBlock& B) {
  std::vector<double>& t = B.avTabHost;
  t.clear();
  if (B.kind == kTensor) {
    const TensorOps& o = B.ops;
    const int n = o.n;
    for (int i = 0; i < n; ++i) t.push_back(o.x[i]);
    for (int i = 0; i < n; ++i) t.push_back(o.w[i]);
    for (int i = 0; i < n; ++i)
      for (int m = 0; m < n; ++m) t.push_back(o.phi1[i][m]);
    for (int i = 0; i < n; ++i)
      for (int m = 0; m < n; ++m) t.push_back(o.phi1inv[i][m]);
    return;
  }
  const PointRule vr = volumeRule(B.type, B.p), fr = faceRule(B.type, B.p);
  const int nb = B.nb, nq = vr.n, nvert = typeVertices(B.type);
  t.insert(t.end(), B.phi.begin(), B.phi.end());  // [nq][nb]
  // degrees of the modes (modalBasis order): vertices 1; triangle edge modes k = 2..P edge by edge, bubbles
  // i + j + 3 by increasing i + j; tetrahedra: six edges of modes k = 2..P, four faces of bubbles s + 3
  // (s = 0..P-3, s + 1 modes each), interior bubbles s + 4; quadrangles (P1 only here) are all degree 1 --
  // P1 takes the whole density
  std::vector<int> tetDegree;
  if (B.type == SDG_ELEMENT_TETRAHEDRON) {
    tetDegree.assign(4, 1);
    for (int e = 0; e < 6; ++e)
      for (int k = 2; k <= B.p; ++k) tetDegree.push_back(k);
    for (int f = 0; f < 4; ++f)
      for (int s = 0; s <= B.p - 3; ++s)
        for (int i = 0; i <= s; ++i) tetDegree.push_back(s + 3);
    for (int s = 0; s <= B.p - 4; ++s)
      for (int i = 0; i < (s + 1) * (s + 2) / 2; ++i) tetDegree.push_back(s + 4);
    if (int(tetDegree.size()) != nb) throw Failure(SDG_ERR_INVALID_ARGUMENT, "tetrahedron mode count");
  }
  for (int b = 0; b < nb; ++b) {
    int deg = B.type == SDG_ELEMENT_TETRAHEDRON ? tetDegree[b] : 1;
    if (B.type == SDG_ELEMENT_TRIANGLE && b >= 3) {
      if (b < 3 + 3 * (B.p - 1)) {
        deg = 2 + (b - 3) % (B.p - 1);
      } else {
        int idx = b - 3 - 3 * (B.p - 1), s = 0;
        while (idx > s) { idx -= s + 1; ++s; }
        deg = s + 3;
      }
    }
    t.push_back(B.p == 1 || deg == B.p ? 1.0 : 0.0);
  }
  for (int q = 0; q < nq; ++q) t.push_back(vr.w[q]);
  const auto shape = [&](const double* X, double* sh) {
    if (B.type == SDG_ELEMENT_TRIANGLE) { sh[0] = 1.0 - X[0] - X[1]; sh[1] = X[0]; sh[2] = X[1]; return; }
    if (B.type == SDG_ELEMENT_TETRAHEDRON) {
      sh[0] = 1.0 - X[0] - X[1] - X[2]; sh[1] = X[0]; sh[2] = X[1]; sh[3] = X[2];
      return;
    }
    sh[0] = 0.25 * (1 - X[0]) * (1 - X[1]); sh[1] = 0.25 * (1 + X[0]) * (1 - X[1]);
    sh[2] = 0.25 * (1 + X[0]) * (1 + X[1]); sh[3] = 0.25 * (1 - X[0]) * (1 + X[1]);
  };
  double sh[4];
  for (int q = 0; q < nq; ++q) { shape(&vr.x[q * 3], sh); t.insert(t.end(), sh, sh + nvert); }
  for (int f = 0; f < B.nface; ++f)
    for (int j = 0; j < fr.n; ++j) {
      double X[3];
      facePointInParent(B.type, f, &fr.x[j * 3], X);
      shape(X, sh);
      t.insert(t.end(), sh, sh + nvert);
    }
}

// Records of the per-step artificial viscosity: zero the node field, sensor per block, vertex gather.
void emitArtificialViscosity(sdg_handle* h, int seq, std::vector<Rec>& out) {
  {
    Rec r = avRec(0, h->nodeCount);
    r.av.nodeAV = h->nodeAV; r.av.nodes = h->nodeCount;
    r.seq = seq;
    out.push_back(r);
  }
  for (int pass = 1; pass <= 2; ++pass)
    for (DevBlock& B : h->blocks) {
      const int nvert = typeVertices(B.type);
      Rec r = avRec(pass == 1 ? (B.kind == kTensor ? 1 : 2) : 3, pass == 1 ? B.ne : B.ne * nvert);
      AvArgs& a = r.av;
      a.u = h->state[0] + B.stateOffset; a.geom = B.geom; a.vert = B.vertDev; a.inner = B.innerDev;
      a.tab = B.avTab; a.nodeAV = h->nodeAV; a.epsV = B.epsV;
      a.ne = B.ne; a.nodes = h->nodeCount;
      a.dim = B.dim; a.n = B.n; a.nb = B.nb; a.nq = B.nq; a.nvert = nvert; a.ustride = B.ustride;
      a.affine = B.affine; a.p = B.p;
      a.s0 = kAvTolerance[B.p - 1];
      a.kappa = h->cfg.empirical_tolerance; a.factor = h->cfg.artificial_viscosity_factor;
      r.seq = seq + pass;
      out.push_back(r);
    }
}

}  // namespace sdg

using namespace sdg;

#pragma GCC visibility push(default)
extern "C" {

int sdg_get_node_artificial_viscosity(sdg_handle* h, double* out) {
  if (!h || !out) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  try {
    if (!h->hasState) throw Failure(SDG_ERR_STATE, "no state");
    SDG_CUDA(cudaSetDevice(h->device));
    if (!h->av) {
      for (int64_t i = 0; i < h->nodeCount; ++i) out[i] = 0.0;
      return SDG_OK;
    }
    std::vector<Rec> recs;
    emitArtificialViscosity(h, 0, recs);
    runRecs(h, recs, h->stream);
    SDG_CUDA(cudaMemcpyAsync(out, h->nodeAV, size_t(h->nodeCount) * 8, cudaMemcpyDeviceToHost, h->stream));
    SDG_CUDA(cudaStreamSynchronize(h->stream));
  } catch (const Failure& f) {
    h->err = f.what();
    return f.code;
  }
  return SDG_OK;
}

}  // extern "C"
#pragma GCC visibility pop
