// Device-side helpers shared by the kernels: launch sizing, warp utilities,
// ordered-bits atomics for non-negative doubles and the edge-balanced owner
// search used by the pull / push kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ctx.h"

namespace sg {

// 4-edge quads per tile of the warp-level pull (one quad per lane)
constexpr uint32_t kWarpTileQuads = 32;

// Blocks for a grid-stride loop over n items: at most 16 resident CTAs per
// SM of the 152-SM part (the loop covers the rest).
inline unsigned grid_for(uint64_t n, int threads, int max_blocks = 152 * 16) {
  uint64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (uint64_t)max_blocks) b = max_blocks;
  return (unsigned)b;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Appends `pred` items to a queue with one atomic per warp.  All lanes of the
// warp must call it (pred may differ).  Returns the slot for this lane (only
// meaningful when pred is true).
__device__ __forceinline__ uint32_t warp_append(bool pred, uint32_t* tail) {
  const uint32_t mask = __ballot_sync(0xffffffffu, pred);
  uint32_t base = 0;
  const uint32_t leader = mask ? (__ffs(mask) - 1) : 0;
  if (mask && lane_id() == leader) base = atomicAdd(tail, (uint32_t)__popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  return base + __popc(mask & lanemask_lt());
}

// Non-negative IEEE doubles order like their bit patterns read as unsigned
// integers, so atomicMin on the bits is an exact min of the doubles.
__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double bitsd(unsigned long long b) {
  return __longlong_as_double((long long)b);
}
constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;

// Largest index i in [lo, hi) with q[i] <= t (q non-decreasing, q[lo] <= t).
template <typename Q>
__device__ __forceinline__ uint32_t upper_owner(const Q* q, uint32_t lo, uint32_t hi,
                                                uint64_t t) {
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if ((uint64_t)q[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// L2 eviction-priority policies (createpolicy, sm_80+): streamed data that is
// read once per pass goes evict-first so that it does not push out data that
// is gathered many times (the push values).
__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ uint4 ld_u4_hint(const uint32_t* ptr, unsigned long long pol) {
  uint4 r;
  asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(ptr), "l"(pol));
  return r;
}

__device__ __forceinline__ float4 ld_f4_hint(const float* ptr, unsigned long long pol) {
  float4 r;
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(ptr), "l"(pol));
  return r;
}

// Block-wide sum of a double; result valid in thread 0.
template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double* smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) smem[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < THREADS / 32 ? smem[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

// CUB wrappers (instantiated in graph.cu)
sg_status cub_exclusive_sum_u64(sg_ctx* ctx, const uint64_t* in, uint64_t* out, uint64_t n);
sg_status cub_select_flagged_u32(sg_ctx* ctx, const uint32_t* in, const uint8_t* flags,
                                 uint32_t* out, uint64_t* d_count, uint64_t n);
sg_status cub_sort_pairs_u64_u32(sg_ctx* ctx, const uint64_t* kin, uint64_t* kout,
                                 const uint32_t* vin, uint32_t* vout, uint64_t n);

}  // namespace sg
