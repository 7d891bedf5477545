// Allocation-free PageRank PEval.
//
// Some callers cannot allocate device memory: a process whose device memory
// belongs to another framework's pool, or a latency-bound loop where the
// implicit synchronisation of cudaMalloc / cudaFree is not allowed.  For
// them this file provides sg_pr_peval_noalloc: the caller passes the graph
// and the output buffers in device memory, and the only scratch the
// computation needs (one push value per vertex plus a few control words)
// lives in file-scope __device__ arrays of a fixed maximum size.  Every GPU
// that loads the library holds those arrays until the process exits.
//
// The computation is the delta-accumulative PageRank of sg_pr_peval on a
// plain packed CSR: rounds of (activate |delta| > threshold / N, push
// d * delta / outdeg along out-edges with atomicAdd) until the L1 residual
// sum|delta| is below the threshold.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/suminc_gb300.h"
#include "dev.cuh"

namespace sg {
namespace {

constexpr uint32_t kMaxVertices = SG_PR_NOALLOC_MAX_VERTICES;
constexpr int kMaxDevices = 64;

// Scratch shared by every call on a device: push values and control words
// (residual accumulator, active-vertex counter).  Calls whose work overlaps
// on the GPU race on these arrays.
static __device__ __align__(256) float g_noalloc_pv[kMaxVertices];
static __device__ __align__(256) double g_noalloc_ctl[4];

struct DevicePtrs {
  float* pv = nullptr;
  double* ctl = nullptr;
  bool ready = false;
};
DevicePtrs g_dev[kMaxDevices];
std::mutex g_mu;

// Host code cannot use the arrays' names as device addresses; their device
// addresses are looked up once per device with that device current.
cudaError_t device_ptrs(int dev, DevicePtrs* out) {
  std::lock_guard<std::mutex> lock(g_mu);
  DevicePtrs& d = g_dev[dev];
  if (!d.ready) {
    cudaError_t e = cudaGetSymbolAddress((void**)&d.pv, g_noalloc_pv);
    if (e != cudaSuccess) return e;
    e = cudaGetSymbolAddress((void**)&d.ctl, g_noalloc_ctl);
    if (e != cudaSuccess) return e;
    d.ready = true;
  }
  *out = d;
  return cudaSuccess;
}

__global__ void k_na_init(uint32_t n, float init_c, float* x, float* delta) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    x[v] = 0.f;
    delta[v] = init_c;
  }
}

// activate: |delta| > thr_v moves delta into x and publishes the push value
__global__ void k_na_vertex(uint32_t n, const uint64_t* __restrict__ rp, float damping,
                            float thr_v, float* __restrict__ x, float* __restrict__ delta,
                            float* __restrict__ pv, double* __restrict__ ctl) {
  unsigned long long active = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const float dl = delta[v];
    float p = 0.f;
    if (fabsf(dl) > thr_v) {
      x[v] += dl;
      delta[v] = 0.f;
      const uint64_t deg = rp[v + 1] - rp[v];
      if (deg > 0) p = damping * dl / (float)deg;
      active++;
    }
    pv[v] = p;
  }
  if (active) atomicAdd(&ctl[1], (double)active);
}

// push: warp-cooperative over the vertices with a non-zero push value
__global__ void k_na_push(uint32_t n, const uint64_t* __restrict__ rp,
                          const uint32_t* __restrict__ col, const float* __restrict__ pv,
                          float* __restrict__ delta) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nn = ((n + 31u) / 32u) * 32u;
  for (uint32_t v0 = blockIdx.x * blockDim.x + threadIdx.x; v0 < nn; v0 += gridDim.x * blockDim.x) {
    const float p = v0 < n ? pv[v0] : 0.f;
    uint32_t mask = __ballot_sync(0xffffffffu, p != 0.f);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const uint32_t u = (v0 & ~31u) + src;
      const float val = __shfl_sync(0xffffffffu, p, src);
      for (uint64_t e = rp[u] + lane; e < rp[u + 1]; e += 32) atomicAdd(&delta[col[e]], val);
    }
  }
}

// residual sum|delta| into ctl[0]
__global__ void k_na_residual(uint32_t n, const float* __restrict__ delta, double* __restrict__ ctl) {
  __shared__ double s_red[8];
  double r = 0.0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    r += fabs((double)delta[v]);
  const double b = block_sum<256>(r, s_red);
  if (threadIdx.x == 0) atomicAdd(&ctl[0], b);
}

}  // namespace
}  // namespace sg

extern "C" sg_status sg_pr_peval_noalloc(uint32_t n, uint64_t m, const uint64_t* d_row_ptr,
                                         const uint32_t* d_col, double damping, double threshold,
                                         int32_t max_rounds, void* stream, float* d_values,
                                         float* d_deltas, int32_t* rounds_out,
                                         double* residual_out) {
  using namespace sg;
  if (n == 0 || !d_row_ptr || (!d_col && m > 0) || !d_values || !d_deltas)
    return SG_ERR_INVALID;
  if (n > kMaxVertices) return SG_ERR_TOO_LARGE;
  if (!(damping > 0.0 && damping < 1.0) || !(threshold > 0.0)) return SG_ERR_INVALID;
  // an error the caller has not collected yet is left in place for the
  // caller, and nothing is launched on top of it; every error seen below is
  // then this call's own
  if (cudaPeekAtLastError() != cudaSuccess) return SG_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return SG_ERR_CUDA;
  }
  DevicePtrs P;
  if (device_ptrs(dev, &P) != cudaSuccess) {
    cudaGetLastError();
    return SG_ERR_CUDA;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const float d = (float)damping;
  const float thr_v = (float)(threshold / (double)n);
  const int cap = max_rounds > 0 ? max_rounds : 1000;
  const unsigned blocks = grid_for(n, 256);
  k_na_init<<<blocks, 256, 0, st>>>(n, (float)((1.0 - damping) / (double)n), d_values, d_deltas);
  int round = 0;
  double res = 0.0;
  bool converged = false, cuda_err = false;
  while (round < cap) {
    ++round;
    if (cudaMemsetAsync(P.ctl, 0, 4 * sizeof(double), st) != cudaSuccess) {
      cuda_err = true;
      break;
    }
    k_na_vertex<<<blocks, 256, 0, st>>>(n, d_row_ptr, d, thr_v, d_values, d_deltas, P.pv, P.ctl);
    k_na_push<<<blocks, 256, 0, st>>>(n, d_row_ptr, d_col, P.pv, d_deltas);
    k_na_residual<<<blocks, 256, 0, st>>>(n, d_deltas, P.ctl);
    double ctl[2] = {0.0, 0.0};
    if (cudaMemcpyAsync(ctl, P.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cuda_err = true;
      break;
    }
    res = ctl[0];
    if (res < threshold || ctl[1] == 0.0) {
      converged = true;
      break;
    }
  }
  if (cuda_err || cudaGetLastError() != cudaSuccess) {
    cudaGetLastError();
    return SG_ERR_CUDA;
  }
  if (rounds_out) *rounds_out = round;
  if (residual_out) *residual_out = res;
  return converged ? SG_OK : SG_ERR_NOT_CONVERGED;
}
