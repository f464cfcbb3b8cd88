// Raw-binary solution files compatible with the reference's writer and restart reader
// (src/View/RawBinary.cpp:42-191, src/Solver/InitialCondition.cpp:40-80, src/Utils/SystemControl.cpp:146-156).
//
// File: a little-endian u64 holding ZSTD_compressBound(payload size) (the reference writes the bound, and its
// reader sizes the decompression buffer with it), then one zstd frame of the payload at level 1.
// Payload, all FP64, in the reference's block order (2D: triangles, quadrangles; 3D: hexahedra):
//   per element: the modal coefficients, column-major (d+2) x Nb; for Navier-Stokes then the gradient
//                coefficients, column-major (d+2)*d x Nb (row v*d + k)
//   per boundary face: the parent element's coefficients (and gradient), in the caller's boundary-face order
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

// Modal gradient coefficients of every element, [block][e][b][(d+2)*d] (column-major (d+2)d x Nb).
std::vector<double> gradientCoefficients(sdg_handle* h) {
  std::vector<double> dev(h->gradCount);
  SDG_CUDA(cudaMemcpyAsync(dev.data(), h->grad, h->gradCount * 8, cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  std::vector<double> out(h->gradCount);
  const int nr = h->nv * h->dim;
  for (const DevBlock& B : h->blocks) {
    const int nb = B.nb;
    std::vector<double> v(nb), t;
    for (int64_t e = 0; e < B.ne; ++e)
      for (int c = 0; c < nr; ++c) {
        const double* src = &dev[B.gradOffset + (size_t(e) * nr + c) * nb];
        std::copy(src, src + nb, v.begin());
        if (B.kind == kTensor) nodalToModal(B, v.data(), t);
        for (int b = 0; b < nb; ++b) out[B.gradOffset + (size_t(e) * nb + b) * nr + c] = v[b];
      }
  }
  return out;
}

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
    std::vector<double> grad;
    if (h->ns) grad = gradientCoefficients(h);
    const int nv = h->nv, nr = h->nv * h->dim;
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
          const double* g = &grad[B.gradOffset + size_t(e) * B.nb * nr];
          payload.insert(payload.end(), g, g + size_t(nr) * B.nb);
        }
      }
      moff += size_t(B.ne) * nv * B.nb;
    }
    // boundary faces: the parent's coefficients (and gradient), in the caller's boundary-face order when one
    // was given (sdg_set_boundary_face_order), else in this library's
    for (int64_t k = 0; k < h->nBoundary; ++k) {
      const int64_t i = h->boundaryOrder.empty() ? k : h->boundaryOrder[size_t(k)];
      const int32_t* r = &h->boundaryParent[size_t(i) * 3];
      const DevBlock& B = h->blocks[r[0]];
      const double* c = &modal[modalOffset[r[0]] + size_t(r[1]) * nv * B.nb];
      payload.insert(payload.end(), c, c + size_t(nv) * B.nb);
      if (h->ns) {
        const double* g = &grad[B.gradOffset + size_t(r[1]) * B.nb * nr];
        payload.insert(payload.end(), g, g + size_t(nr) * B.nb);
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
