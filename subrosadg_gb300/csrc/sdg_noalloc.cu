// Allocation-free CFL time step (sdg_delta_time_noalloc, include/sdg_gpu.h).
//
// Some callers cannot call cudaMalloc at the point where they need a time step: code running inside a
// memory-pool-managed framework that forbids raw device allocations, real-time loops that must not
// allocate, or hosts that record work into a stream and do not own any device memory of their own.
// This entry point computes the same dt as sdg_calculate_delta_time for one element block (one call per
// block of a hybrid mesh; the caller takes the minimum) from device arrays the caller already holds, and
// keeps its only scratch -- one partial minimum per CTA -- in the file-scope __device__ array below, so it
// allocates nothing.
//
// Scratch: kMaxPartials doubles (1 MiB) held by every GPU that loads the library until the process
// exits.  Every call shares it and it keeps the last call's contents; each CTA overwrites its own slot
// before the final reduction reads it, so nothing has to start at zero.  Calls that overlap on the GPU
// (two streams, or two threads) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/sdg_gpu.h"

namespace sdg {
void setCreateError(const std::string& message);  // text returned by sdg_last_error(NULL) (sdg_gpu.cu)
}

namespace sdg_noalloc {

constexpr int kThreads = 256;
constexpr int64_t kMaxPartials = 131072;                 // 1 MiB of doubles
constexpr int64_t kMaxPoints = kMaxPartials * kThreads;  // 33,554,432 volume points per call
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_partial[kMaxPartials];

// Per-CTA minimum of CFL * minEdge / ((|u| + c) (P+1)^2) over one volume point per thread
// (Solver::calculateDeltaTime, src/Solver/TimeIntegration.cpp:104-131).
// The sound speed is sqrt(gamma p / rho) for the ideal gas, or the constant c0 of the incompressible models
// (weakly compressible fluid, PhysicalModel.cpp:57-78) when c0 > 0.
__global__ void __launch_bounds__(kThreads) partialKernel(const double* __restrict__ pts,
                                                          const double* __restrict__ minEdge, int64_t n, int nq,
                                                          int dim, double cfl, double p1sq, double gamma, double c0,
                                                          double* __restrict__ part) {
  __shared__ double sh[kThreads];
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double dt = 1.79769313486231570e308;
  if (t < n) {
    const double* p = pts + t * (dim + 2);
    const double rho = p[0];
    double u2 = 0.0;
    for (int k = 0; k < dim; ++k) { const double u = p[1 + k] / rho; u2 += u * u; }
    const double e = p[dim + 1] / rho - u2 / 2.0;
    const double pr = (gamma - 1.0) * rho * e;
    const double c = c0 > 0.0 ? c0 : sqrt(gamma * pr / rho);
    dt = cfl * minEdge[t / nq] / ((sqrt(u2) + c) * p1sq);
  }
  sh[threadIdx.x] = dt;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Minimum of the first `count` partials into *out (one CTA, fixed order).
__global__ void __launch_bounds__(kThreads) finalKernel(const double* __restrict__ part, int64_t count,
                                                        double* __restrict__ out) {
  __shared__ double sh[kThreads];
  double m = 1.79769313486231570e308;
  for (int64_t i = threadIdx.x; i < count; i += blockDim.x) m = fmin(m, part[i]);
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// The device address of g_partial, per device, together with the CUDA context it was resolved in.  The
// address belongs to the module loaded in that context: after a cudaDeviceReset (a new primary context) or
// under another current context the module is loaded again elsewhere, so the cached address is looked up
// anew whenever the current context differs from the recorded one.
struct Scratch {
  void* context = nullptr;
  double* address = nullptr;
};
std::mutex g_mutex;
Scratch g_scratch[kMaxDevices];
using CtxGetCurrent = int (*)(void**);  // cuCtxGetCurrent(CUcontext*), fetched from the runtime: no -lcuda
CtxGetCurrent g_ctxGetCurrent = nullptr;

// With the device current: resolve the device address of the static scratch array (once per device and
// context).  In host code `g_partial` names a host-side stand-in, not device memory.
int scratchFor(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_ctxGetCurrent) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      sdg::setCreateError("sdg_delta_time_noalloc: cuCtxGetCurrent is not available");
      return SDG_ERR_CUDA;
    }
    g_ctxGetCurrent = reinterpret_cast<CtxGetCurrent>(fn);
  }
  void* ctx = nullptr;
  if (g_ctxGetCurrent(&ctx) != 0 || !ctx) {
    sdg::setCreateError("sdg_delta_time_noalloc: no current CUDA context");
    return SDG_ERR_CUDA;
  }
  Scratch& S = g_scratch[device];
  if (!S.address || S.context != ctx) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_partial);
    if (e != cudaSuccess) {
      sdg::setCreateError(std::string("sdg_delta_time_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return SDG_ERR_CUDA;
    }
    S.context = ctx;
    S.address = static_cast<double*>(p);
  }
  *out = S.address;
  return SDG_OK;
}

}  // namespace sdg_noalloc

#pragma GCC visibility push(default)
extern "C" {

int sdg_delta_time_noalloc(const double* state_point, const double* minimum_edge, int64_t point_count,
                           int32_t points_per_element, int32_t dimension, int32_t polynomial_order,
                           double specific_heat_ratio, double reference_sound_speed,
                           double courant_friedrichs_lewy_number, double* delta_time, void* stream) {
  using namespace sdg_noalloc;
  if (!state_point || !minimum_edge || !delta_time || point_count <= 0 || points_per_element <= 0 ||
      dimension < 1 || dimension > 3 || polynomial_order < 1 || polynomial_order > 5 ||
      !(reference_sound_speed >= 0.0) || (reference_sound_speed == 0.0 && !(specific_heat_ratio > 1.0)) ||
      !(courant_friedrichs_lewy_number > 0.0)) {
    sdg::setCreateError("sdg_delta_time_noalloc: invalid argument");
    return SDG_ERR_INVALID_ARGUMENT;
  }
  if (point_count % points_per_element != 0) {
    sdg::setCreateError("sdg_delta_time_noalloc: point_count is not a multiple of points_per_element");
    return SDG_ERR_INVALID_ARGUMENT;
  }
  if (point_count > kMaxPoints) {
    sdg::setCreateError("sdg_delta_time_noalloc: " + std::to_string(point_count) +
                        " volume points exceed the maximum of " + std::to_string(kMaxPoints) +
                        " (1 MiB of static scratch); use sdg_calculate_delta_time");
    return SDG_ERR_INVALID_ARGUMENT;
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess || device < 0 || device >= kMaxDevices) {
    sdg::setCreateError("sdg_delta_time_noalloc: no current CUDA device");
    return SDG_ERR_CUDA;
  }
  double* part = nullptr;
  const int rc = scratchFor(device, &part);
  if (rc != SDG_OK) return rc;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t blocks = (point_count + kThreads - 1) / kThreads;
  const double p1 = double(polynomial_order) + 1.0;
  partialKernel<<<unsigned(blocks), kThreads, 0, s>>>(state_point, minimum_edge, point_count, points_per_element,
                                                      dimension, courant_friedrichs_lewy_number, p1 * p1,
                                                      specific_heat_ratio, reference_sound_speed, part);
  finalKernel<<<1, kThreads, 0, s>>>(part, blocks, delta_time);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    sdg::setCreateError(std::string("sdg_delta_time_noalloc: ") + cudaGetErrorString(e));
    return SDG_ERR_CUDA;
  }
  return SDG_OK;
}

}  // extern "C"
#pragma GCC visibility pop
