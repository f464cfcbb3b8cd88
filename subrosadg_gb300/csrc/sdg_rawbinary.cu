// Raw-binary solution files compatible with the reference's writer and restart reader
// (src/View/RawBinary.cpp:42-191, src/Solver/InitialCondition.cpp:40-80, src/Utils/SystemControl.cpp:146-156).
//
// File: a little-endian u64 holding ZSTD_compressBound(payload size) (the reference writes the bound, and its
// reader sizes the decompression buffer with it), then one zstd frame of the payload at level 1.
// Payload, all FP64, in the reference's block order (2D: triangles, quadrangles; 3D: hexahedra):
//   per element: the modal coefficients, column-major (d+2) x Nb; for Navier-Stokes then the gradient
//                coefficients, column-major (d+2)*d x Nb (row v*d + k)
//   per boundary face: the parent element's coefficients (and gradient -- BR1: the element's; BR2: its volume
//                gradient plus the lift of that face), in the caller's boundary-face order
//                (sdg_set_boundary_face_order: the reference's own adjacency order, Adjacency.cpp:466-485) or,
//                without one, in this library's
//   per mesh node: the artificial viscosity of the current state (zero without shock capturing)
// libzstd is loaded at run time (libzstd.so.1, its public C API); without it the calls return
// SDG_ERR_UNSUPPORTED.
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <array>
#include <cstring>
#include <map>
#include <memory>
#include <fstream>
#include <iterator>
#include <mutex>
#include <string>
#include <vector>

#include "sdg_internal.hpp"

using namespace sdg;

namespace {

struct Zstd {
  size_t (*compressBound)(size_t) = nullptr;
  size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
  size_t (*decompress)(void*, size_t, const void*, size_t) = nullptr;
  unsigned (*isError)(size_t) = nullptr;
  const char* (*errorName)(size_t) = nullptr;
  bool ok = false;
};

const Zstd& zstd() {
  static Zstd z;
  static std::once_flag once;
  std::call_once(once, [] {
    void* lib = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!lib) lib = dlopen("libzstd.so", RTLD_NOW | RTLD_LOCAL);
    if (!lib) return;
    z.compressBound = reinterpret_cast<size_t (*)(size_t)>(dlsym(lib, "ZSTD_compressBound"));
    z.compress = reinterpret_cast<size_t (*)(void*, size_t, const void*, size_t, int)>(dlsym(lib, "ZSTD_compress"));
    z.decompress = reinterpret_cast<size_t (*)(void*, size_t, const void*, size_t)>(dlsym(lib, "ZSTD_decompress"));
    z.isError = reinterpret_cast<unsigned (*)(size_t)>(dlsym(lib, "ZSTD_isError"));
    z.errorName = reinterpret_cast<const char* (*)(size_t)>(dlsym(lib, "ZSTD_getErrorName"));
    z.ok = z.compressBound && z.compress && z.decompress && z.isError;
  });
  return z;
}

// Tensor blocks store nodal values; the file holds modal (hierarchic Lobatto) coefficients: apply
// Phi1^-1 along each axis of every (element, component) vector of nb values.
void nodalToModal(const DevBlock& B, double* v /* [nb] */, std::vector<double>& t) {
  const int n = B.n, nb = B.nb;
  const int strides[3] = {B.dim == 1 ? 1 : (B.dim == 2 ? n : n * n), B.dim == 2 ? 1 : n, 1};
  t.assign(nb, 0.0);
  for (int ax = 0; ax < B.dim; ++ax) {
    const int st = strides[ax];
    for (int b = 0; b < nb; ++b) {
      const int ib = (b / st) % n;
      const int base = b - ib * st;
      double s = 0;
      for (int k = 0; k < n; ++k) s += B.ops.phi1inv[ib][k] * v[base + k * st];
      t[b] = s;
    }
    std::copy(t.begin(), t.end(), v);
  }
}

// Device-layout gradient block of one element (nr rows of nb values) -> its file record (column-major nr x Nb,
// modal; tensor blocks convert their nodal values with Phi1^-1 along each axis).
void gradientRecord(const DevBlock& B, int nr, const double* g, double* out) {
  std::vector<double> v(B.nb), t;
  for (int c = 0; c < nr; ++c) {
    std::copy(g + size_t(c) * B.nb, g + size_t(c + 1) * B.nb, v.begin());
    if (B.kind == kTensor) nodalToModal(B, v.data(), t);
    for (int b = 0; b < B.nb; ++b) out[size_t(b) * nr + c] = v[b];
  }
}

template <class T>
std::vector<T> download(sdg_handle* h, const T* src, size_t count) {
  std::vector<T> out(count);
  if (count) SDG_CUDA(cudaMemcpyAsync(out.data(), src, count * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  return out;
}

// BR2 boundary-face gradient records (RawBinary.cpp:98-112): the parent's volume gradient plus the lift of
// that face.  The gradient pass keeps the total gradient G = G_vol + sum_f r_f (the gradient of the volume
// term), so the record is G - sum_{f' != f} r_{f'}, each lift rebuilt from the jump 1/2 (U+ - U-) at face f'
// in the last gradient pass:
//   U+ (neighbour traces): the faceOther buffer;
//   U- (own traces): on interior faces the neighbour's copy of it in faceOther (the exchange writes each
//      side's trace into the other's slot); on farfield, inflow and outflow faces U+ itself (their gradient
//      state is the interior state: no jump); on walls the trace of the pass's input state (the last stage
//      input, kept in the stage buffer by two- and three-stage schemes; forward Euler updates in place, so
//      its wall faces are refused).
// Lifts, with the gradient kernels' arithmetic:
//   tensor blocks, node i, face f' (axis b, end s): r(i) = lift_s[i_b] nF_f'(j) 1/2[U](j) / |J|_i, j the face
//      point on the line through i;
//   dense blocks: r = c M^-1 sum_j phifw_j nF_f'(j) 1/2[U](j) (c = 1/|J| with the reference M^-1 on affine
//      elements; 1 with the element's own M^-1 otherwise).
class Br2Records {
 public:
  explicit Br2Records(sdg_handle* h) : h_(h), nv_(h->nv), nfq_(h->nfq), nr_(h->nv * h->dim) {
    other_ = download(h, h->faceOther, h->faceCount);
    const int64_t slots = int64_t(h->faceCount / (size_t(nv_) * nfq_));
    side_.assign(size_t(slots), {-1, 0});
    const std::vector<int> fc = download(h, h->fconn, size_t(h->nInterior) * 3);
    const std::vector<int> bc = download(h, h->bconn, size_t(h->nBoundary) * 3);
    for (int64_t i = 0; i < h->nInterior; ++i) {
      side_[size_t(fc[i * 3])] = {i, 0};
      side_[size_t(fc[i * 3 + 1])] = {i, 1};
    }
    for (int64_t i = 0; i < h->nBoundary; ++i) side_[size_t(bc[i * 3])] = {i, 2 + bc[i * 3 + 1]};
    fconn_ = fc;
    if (h->n1d < 0) perm_ = triangleFacePermutation(h->blocks[0].type, h->p);
  }

  // File record of boundary face k (library order) with the parent's device-layout total gradient g.
  void record(int64_t k, const double* g, double* out) {
    const int32_t* r = &h_->boundaryParent[size_t(k) * 3];
    const DevBlock& B = h_->blocks[r[0]];
    const int64_t e = r[1];
    const int f = r[2], nb = B.nb;
    std::vector<double> acc(g, g + size_t(nr_) * nb), lift(size_t(nr_) * nb);
    for (int fo = 0; fo < B.nface; ++fo) {
      if (fo == f) continue;
      faceLift(B, e, fo, lift.data());
      for (size_t i = 0; i < acc.size(); ++i) acc[i] -= lift[i];
    }
    gradientRecord(B, nr_, acc.data(), out);
  }

 private:
  sdg_handle* h_;
  int nv_, nfq_, nr_;
  std::vector<double> other_, input_;
  std::vector<std::pair<int64_t, int>> side_;  // per slot: (face, 0 left / 1 right / 2 + condition boundary)
  std::vector<int> fconn_, perm_;

  int paired(int j, int rot) const {
    if (h_->dim == 1) return 0;
    if (h_->dim == 2) return rightPoint<2>(j, rot, h_->n1d);
    return h_->n1d < 0 ? perm_[size_t(rot) * nfq_ + j] : rightPoint<3>(j, rot, h_->n1d);
  }

  // 1/2 (U+ - U-) of slot `slot` (block B, element e, local face f): [v][j]
  void jump(const DevBlock& B, int64_t e, int f, double* out) {
    const int64_t slot = B.faceBase + e * B.nface + f;
    const double* o = &other_[size_t(slot) * nv_ * nfq_];
    std::vector<double> own(size_t(nv_) * nfq_);
    const auto [face, kind] = side_[size_t(slot)];
    if (kind == 0 || kind == 1) {  // the neighbour's slot holds this side's trace at the paired points
      const int sl = fconn_[size_t(face) * 3], sr = fconn_[size_t(face) * 3 + 1], rot = fconn_[size_t(face) * 3 + 2];
      const double* mo = &other_[size_t(kind == 0 ? sr : sl) * nv_ * nfq_];
      for (int j = 0; j < nfq_; ++j) {
        const int jr = paired(j, rot);
        for (int v = 0; v < nv_; ++v) {
          if (kind == 0) own[size_t(v) * nfq_ + j] = mo[size_t(v) * nfq_ + jr];
          else own[size_t(v) * nfq_ + jr] = mo[size_t(v) * nfq_ + j];
        }
      }
    } else if (kind - 2 <= SDG_BC_PRESSURE_OUTFLOW) {
      std::copy(o, o + size_t(nv_) * nfq_, own.begin());
    } else {
      stageTrace(B, e, f, own.data());
    }
    for (size_t i = 0; i < own.size(); ++i) out[i] = 0.5 * (o[i] - own[i]);
  }

  // Trace at face f of element e of the gradient pass's input state: [v][j]
  void stageTrace(const DevBlock& B, int64_t e, int f, double* out) {
    if (!h_->gradInput)
      throw Failure(SDG_ERR_UNSUPPORTED, "BR2 gradient records of wall-face parents need the last gradient pass's input "
                                         "state, which forward Euler does not keep (and other calls since the last step "
                                         "may have replaced)");
    if (input_.empty()) input_ = download(h_, h_->gradInput, h_->stateCount);
    const double* u = &input_[B.stateOffset + size_t(e) * B.ustride];
    if (B.kind == kTensor) {
      TensorTables T;
      std::memcpy(&T, B.tablesHost.data(), sizeof(T));
      const int axis = T.faceAxis[f];
      const double* end = T.faceEnd[f] ? B.ops.endp : B.ops.endm;
      int st = 1;
      for (int a = axis + 1; a < B.dim; ++a) st *= B.n;
      for (int j = 0; j < nfq_; ++j)
        for (int v = 0; v < nv_; ++v) {
          double s = 0.0;
          for (int a = 0; a < B.n; ++a) s += end[a] * u[size_t(v) * B.nb + T.faceBase[f][j] + a * st];
          out[size_t(v) * nfq_ + j] = s;
        }
    } else {
      const double* phif = B.tablesHost.data() + size_t(B.nq) * B.nb * (1 + B.dim);
      for (int j = 0; j < nfq_; ++j)
        for (int v = 0; v < nv_; ++v) {
          double s = 0.0;
          for (int b = 0; b < B.nb; ++b) s += phif[size_t(f * nfq_ + j) * B.nb + b] * u[size_t(v) * B.nb + b];
          out[size_t(v) * nfq_ + j] = s;
        }
    }
  }

  // n|J_f| of face f of element e at face point j
  void faceMetric(const DevBlock& B, int64_t e, int f, int j, double* nF) const {
    const int d = B.dim;
    if (B.kind == kTensor && B.affine) {
      TensorTables T;
      std::memcpy(&T, B.tablesHost.data(), sizeof(T));
      const double* g = &B.geomHost[size_t(e) * B.geomStride];
      const double sg = T.faceEnd[f] ? 1.0 : -1.0;
      for (int k = 0; k < d; ++k) nF[k] = sg * g[T.faceAxis[f] * d + k];
    } else if (B.facePoint) {
      for (int k = 0; k < d; ++k) nF[k] = B.fmetricHost[((size_t(e) * B.nface + f) * nfq_ + j) * d + k];
    } else {
      for (int k = 0; k < d; ++k) nF[k] = B.fmetricHost[(size_t(e) * B.nface + f) * d + k];
    }
  }

  // Lift of face f of element e in the device layout [v*d+k][i]
  void faceLift(const DevBlock& B, int64_t e, int f, double* out) {
    const int d = B.dim, nb = B.nb, gs = d * d + 1;
    std::vector<double> J(size_t(nv_) * nfq_), nF(size_t(nfq_) * d);
    jump(B, e, f, J.data());
    for (int j = 0; j < nfq_; ++j) faceMetric(B, e, f, j, &nF[size_t(j) * d]);
    if (B.kind == kTensor) {
      TensorTables T;
      std::memcpy(&T, B.tablesHost.data(), sizeof(T));
      const int axis = T.faceAxis[f], s = T.faceEnd[f];
      int st = 1;
      for (int a = axis + 1; a < d; ++a) st *= B.n;
      for (int i = 0; i < nb; ++i) {
        const int j = T.nodeFacePoint[axis][s][i];
        const double lift = (s ? B.ops.liftp : B.ops.liftm)[(i / st) % B.n];
        const double jinv = B.geomHost[size_t(e) * B.geomStride + (B.affine ? 0 : size_t(i) * gs) + d * d];
        for (int v = 0; v < nv_; ++v)
          for (int k = 0; k < d; ++k)
            out[size_t(v * d + k) * nb + i] = lift * nF[size_t(j) * d + k] * J[size_t(v) * nfq_ + j] * jinv;
      }
    } else {
      const size_t nfp = size_t(B.nface) * nfq_;
      const double* phifw = B.tablesHost.data() + size_t(B.nq) * nb * (1 + d) + nfp * nb;
      const double* mref = phifw + nfp * nb;
      const double* g = &B.geomHost[size_t(e) * B.geomStride];
      const double* minv = B.affine ? mref : g + size_t(B.nq) * gs;
      const double sc = B.affine ? g[d * d] : 1.0;
      std::vector<double> t(nb);
      for (int v = 0; v < nv_; ++v)
        for (int k = 0; k < d; ++k) {
          for (int m = 0; m < nb; ++m) {
            double s = 0.0;
            for (int j = 0; j < nfq_; ++j)
              s += phifw[size_t(f * nfq_ + j) * nb + m] * nF[size_t(j) * d + k] * J[size_t(v) * nfq_ + j];
            t[m] = s;
          }
          for (int i = 0; i < nb; ++i) {
            double s = 0.0;
            for (int m = 0; m < nb; ++m) s += minv[size_t(i) * nb + m] * t[m];
            out[size_t(v * d + k) * nb + i] = sc * s;
          }
        }
    }
  }
};

int rawFail(sdg_handle* h, int code, const std::string& m) {
  h->err = m;
  return code;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

int sdg_write_raw_binary(sdg_handle* h, const char* path) {
  if (!h || !path) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) return rawFail(h, SDG_ERR_STATE, "host-only handle (created with device < 0)");
  if (!h->hasState) return rawFail(h, SDG_ERR_STATE, "no state");
  const Zstd& z = zstd();
  if (!z.ok) return rawFail(h, SDG_ERR_UNSUPPORTED, "libzstd.so.1 is not available");
  try {
    std::vector<double> modal(size_t(h->dof));
    const int rc = sdg_get_state_modal(h, modal.data());
    if (rc != SDG_OK) return rc;
    std::vector<double> grad;  // device layout: per element nr rows of nb values
    if (h->ns) grad = download(h, h->grad, h->gradCount);
    const int nv = h->nv, nr = h->nv * h->dim;
    std::vector<double> rec;
    std::vector<double> payload;
    payload.reserve(size_t(h->dof) * (h->ns ? 1 + h->dim : 1) + size_t(h->nBoundary) * 64);
    std::vector<size_t> modalOffset;
    size_t moff = 0;
    for (const DevBlock& B : h->blocks) {
      modalOffset.push_back(moff);
      for (int64_t e = 0; e < B.ne; ++e) {
        const double* c = &modal[moff + size_t(e) * nv * B.nb];
        payload.insert(payload.end(), c, c + size_t(nv) * B.nb);
        if (h->ns) {
          rec.resize(size_t(nr) * B.nb);
          gradientRecord(B, nr, &grad[B.gradOffset + size_t(e) * B.nb * nr], rec.data());
          payload.insert(payload.end(), rec.begin(), rec.end());
        }
      }
      moff += size_t(B.ne) * nv * B.nb;
    }
    // boundary faces: the parent's coefficients (and gradient), in the caller's boundary-face order when one
    // was given (sdg_set_boundary_face_order), else in this library's
    std::unique_ptr<Br2Records> br2;
    if (h->ns && h->cfg.viscous_flux == SDG_VISCOUS_BR2 && h->nBoundary > 0) br2 = std::make_unique<Br2Records>(h);
    for (int64_t k = 0; k < h->nBoundary; ++k) {
      const int64_t i = h->boundaryOrder.empty() ? k : h->boundaryOrder[size_t(k)];
      const int32_t* r = &h->boundaryParent[size_t(i) * 3];
      const DevBlock& B = h->blocks[r[0]];
      const double* c = &modal[modalOffset[r[0]] + size_t(r[1]) * nv * B.nb];
      payload.insert(payload.end(), c, c + size_t(nv) * B.nb);
      if (h->ns) {
        rec.resize(size_t(nr) * B.nb);
        const double* g = &grad[B.gradOffset + size_t(r[1]) * B.nb * nr];
        if (br2) br2->record(i, g, rec.data());  // BR2: volume gradient + this face's lift
        else gradientRecord(B, nr, g, rec.data());
        payload.insert(payload.end(), rec.begin(), rec.end());
      }
    }
    // node artificial viscosity (the current state's; zeros without shock capturing)
    const size_t nodeStart = payload.size();
    payload.insert(payload.end(), size_t(h->nodeCount), 0.0);
    if (h->av) {
      const int rc2 = sdg_get_node_artificial_viscosity(h, payload.data() + nodeStart);
      if (rc2 != SDG_OK) return rc2;
    }
    const size_t raw = payload.size() * sizeof(double);
    const size_t bound = z.compressBound(raw);
    std::vector<char> packed(bound);
    const size_t n = z.compress(packed.data(), bound, payload.data(), raw, 1);
    if (z.isError(n)) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, std::string("zstd: ") + (z.errorName ? z.errorName(n) : "error"));
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    const uint64_t header = bound;
    f.write(reinterpret_cast<const char*>(&header), sizeof(header));
    f.write(packed.data(), std::streamsize(n));
    if (!f) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
  } catch (const Failure& e) {
    return rawFail(h, e.code, e.what());
  }
  return SDG_OK;
}

int sdg_set_boundary_face_order(sdg_handle* h, int64_t count, const int32_t* faces) {
  if (!h || count != h->nBoundary || (count > 0 && !faces)) {
    if (h) h->err = "the order must list every boundary face once";
    return SDG_ERR_INVALID_ARGUMENT;
  }
  std::map<std::array<int32_t, 3>, int64_t> index;  // (element type, element, local face) -> library face
  for (int64_t i = 0; i < h->nBoundary; ++i) {
    const int32_t* r = &h->boundaryParent[size_t(i) * 3];
    index[{h->blocks[r[0]].type, r[1], r[2]}] = i;
  }
  std::vector<int64_t> order(static_cast<size_t>(count));
  std::vector<char> seen(static_cast<size_t>(count), 0);
  for (int64_t k = 0; k < count; ++k) {
    const auto it = index.find({faces[k * 3], faces[k * 3 + 1], faces[k * 3 + 2]});
    if (it == index.end() || seen[size_t(it->second)]) {
      h->err = "boundary face " + std::to_string(k) + " of the order is not a boundary face or is listed twice";
      return SDG_ERR_INVALID_ARGUMENT;
    }
    seen[size_t(it->second)] = 1;
    order[size_t(k)] = it->second;
  }
  h->boundaryOrder = std::move(order);
  return SDG_OK;
}

int sdg_read_raw_binary(sdg_handle* h, const char* path, int32_t lower_order) {
  if (!h || !path || (lower_order != 0 && lower_order != 1)) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) return rawFail(h, SDG_ERR_STATE, "host-only handle (created with device < 0)");
  const Zstd& z = zstd();
  if (!z.ok) return rawFail(h, SDG_ERR_UNSUPPORTED, "libzstd.so.1 is not available");
  std::ifstream f(path, std::ios::binary);
  if (!f) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  uint64_t header = 0;
  f.read(reinterpret_cast<char*>(&header), sizeof(header));
  std::vector<char> packed((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (!f.eof() && f.fail()) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, "short file");
  if (header == 0 || header > (uint64_t(1) << 40)) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, "bad raw-binary header");
  std::vector<char> raw(header);
  const size_t got = z.decompress(raw.data(), raw.size(), packed.data(), packed.size());
  if (z.isError(got)) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, std::string("zstd: ") + (z.errorName ? z.errorName(got) : "error"));
  // LastStep: the same order; SpecificFile: order P-1 coefficients, zero-padded (InitialCondition.cpp:58-80)
  const int nv = h->nv;
  std::vector<double> modal(size_t(h->dof), 0.0);
  size_t pos = 0, moff = 0;
  const auto take = [&](double* dst, size_t count) {
    if ((pos + count) * sizeof(double) > got) return false;
    std::memcpy(dst, raw.data() + pos * sizeof(double), count * sizeof(double));
    pos += count;
    return true;
  };
  for (const DevBlock& B : h->blocks) {
    const int nbf = lower_order ? (h->p > 1 ? modalCount(B.type, h->p - 1) : 0) : B.nb;
    if (lower_order && nbf == 0) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, "no lower order below P1");
    std::vector<double> c(size_t(nv) * nbf), g(size_t(nv) * h->dim * nbf);
    for (int64_t e = 0; e < B.ne; ++e) {
      if (!take(c.data(), c.size())) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, "raw-binary payload too short");
      if (h->ns && !take(g.data(), g.size())) return rawFail(h, SDG_ERR_INVALID_ARGUMENT, "raw-binary payload too short");
      double* dst = &modal[moff + size_t(e) * nv * B.nb];
      std::copy(c.begin(), c.end(), dst);  // leading Nb(P-1) columns, the rest stays zero
    }
    moff += size_t(B.ne) * nv * B.nb;
  }
  return sdg_set_state_modal(h, modal.data());
}

}  // extern "C"
#pragma GCC visibility pop
