// Delta-accumulative PageRank (Ingress form) on the device.
//
// State per vertex: x (values_), delta (deltas_) and a push value
// pv = d * delta / outdeg published by each activation (g_function,
// pagerank_ingress.h:50-72).  A vertex is active when |delta| > threshold / N
// (isChange, sum_sync_iter_worker.h:2914-2925); activation moves delta into
// x.  The L1 residual sum|delta| after every round is the reference's
// termCheck (sum_sync_iter_worker.h:2873-2912), accumulated in FP64.
//
// Round structure:
//   k_pr_vertex   first round of every run: activation of every vertex from
//                 the current delta (PEval init or the amended IncEval state)
//   k_pr_pull_warp  dense pull over the in-CSR, edge-balanced in warp tiles
//                 of 32 4-edge quads (one 128-bit neighbour load and four
//                 push-value gathers per lane, owners found by popc over the
//                 tile's segment starts, segmented shuffle sums).  A vertex
//                 whose quads all lie in the tile is updated by its owner
//                 lane (incoming sum, residual, activation, next push
//                 value); a vertex spanning tiles gets its partial sums by
//                 atomicAdd.  With the hub cache (the default on graphs
//                 with enough high out-degree vertices) push values are
//                 indexed by out-degree rank, each CTA first copies the
//                 lowest ranks' push values into shared memory, and the pull
//                 reads an encoded column copy that holds ranks
//   k_pr_fixup    updates the tile-spanning vertices; its last block makes
//                 the termination decision on the device
// Push values are double-buffered by pull index.  When the residual passes
// the test, one more pull distributes the last activations without
// activating anything (drain) and the run ends.
#include <algorithm>
#include <cmath>

#include "ctx.h"
#include "dev.cuh"

namespace sg {

enum {
  M_DONE = 0,
  M_PENDING = 1,   // residual test passed: next pull drains
  M_BLOCKS = 2,    // last-block counter of the fix-up kernel
  M_ROUNDS = 3,
  M_NOTCONV = 4,
  M_WORDS = 8
};
enum { C_EDGES = 0, C_VISITS = 1, C_WORDS = 4 };
enum { R_ACC = 0, R_LAST = 1, R_ZERO_IN = 2, R_WORDS = 4 };

constexpr int VT = 256;

struct PrArgs {
  uint32_t n;
  float damping;
  float thr_v;      // threshold / N
  double tau;       // threshold
  int max_rounds;
  uint64_t live_edges;
  const uint32_t* scale_deg;  // push value d*delta/deg (PageRank); null: d*delta,
                              // the edge weights are applied in the gather
  const uint32_t* pull_deg;   // live degree of the pulled direction
  float* x;
  float* delta;
  float* pv0;       // push values of the first round
  float* pvb[2];    // push values of later rounds, by pull parity
  const uint32_t* rank;  // push values are indexed by rank[v] (the pull's
                         // vertex order); null: by v
  uint32_t* misc;
  double* res;
  unsigned long long* cnt;
};

// activation of one vertex with its new delta; returns 1 when active.  Each
// thread sums its vertices' |delta| in FP32; the block, grid and the
// termination test take those partial sums in FP64 (per-vertex FP64 adds
// would load GB300's FP64 pipe, which issues at a small fraction of the
// FP32 rate, once per vertex and round).
__device__ __forceinline__ uint32_t activate(const PrArgs& A, uint32_t v, float dl, float* pv_next,
                                             float& res) {
  res += fabsf(dl);
  const uint32_t r = A.rank ? A.rank[v] : v;
  if (fabsf(dl) > A.thr_v) {
    A.x[v] += dl;
    A.delta[v] = 0.f;
    if (A.scale_deg) {
      const uint32_t od = A.scale_deg[v];
      pv_next[r] = od > 0 ? A.damping * dl / (float)od : 0.f;
    } else {
      pv_next[r] = A.damping * dl;
    }
    return 1;
  }
  A.delta[v] = dl;
  pv_next[r] = 0.f;
  return 0;
}

__global__ void __launch_bounds__(VT) k_pr_vertex(PrArgs A) {
  __shared__ double s_red[VT / 32];
  __shared__ double s_red2[VT / 32];
  float res = 0.f, res0 = 0.f;
  unsigned long long visits = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < A.n; v += gridDim.x * blockDim.x) {
    visits += activate(A, v, A.delta[v], A.pv0, res);
    // vertices without in-edges never change again: their leftover delta is
    // a constant part of every later residual
    if (A.pull_deg[v] == 0) res0 += fabsf(A.delta[v]);
    A.pvb[0][v] = 0.f;
    A.pvb[1][v] = 0.f;
  }
  const double b = block_sum<VT>((double)res, s_red);
  const double b0 = block_sum<VT>((double)res0, s_red2);
  if (threadIdx.x == 0) {
    atomicAdd(&A.res[R_LAST], b);
    atomicAdd(&A.res[R_ZERO_IN], b0);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) visits += __shfl_down_sync(0xffffffffu, visits, o);
  if ((threadIdx.x & 31) == 0 && visits) atomicAdd(&A.cnt[C_VISITS], visits);
}

constexpr int PT_THREADS = 256;

// Warp-level pull: a warp takes a tile of kWarpTileQuads quads, one quad per
// lane.  The up-to-32 owners of the tile are loaded one per lane (first
// quad, segment offset and degree from nz-ordered copies, so a lane's
// neighbour load depends on one load only; the owner's delta and degree
// for the epilogue are fetched alongside, off the gather's critical path).
// A lane finds its owner from the mask of segment starts (popc), gathers its
// four push values, and a segmented shuffle reduction leaves each owner's
// sum in the first lane of its segment.  Owners whose quads all lie in the
// tile are finished there (no shared memory, no block barrier); the others
// add their partial sums to delta by atomicAdd and are finished by
// k_pr_fixup.  The next tile's first owner is prefetched.
struct WarpPullArgs {
  const uint32_t* nz;
  const uint64_t* qoff;
  const uint64_t* off_nz;   // segment offset of nz[i]
  const uint32_t* deg_nz;   // live degree of nz[i]
  const uint32_t* wtile_v0;
  uint32_t nz_count;
  uint64_t quads;
  uint64_t ntiles;
  const uint32_t* col;
  const float* w;
  uint32_t nhub;            // hub cache: ranks below nhub (HUB kernels)
};

// Hub cache and vertex order: the pull gathers the push value of every
// in-neighbour, and the vertices with the highest out-degree take a large
// share of those gathers (R-MAT scale 24: the top 13,312 of 16.8 M vertices
// take 27 %).  The HUB kernels index push values by rank (vertices sorted by
// out-degree, highest first) and read an encoded column copy that holds the
// ranks of the in-neighbours.  A CTA copies the push values of the lowest
// ranks (the hubs) into shared memory once per launch; the next ranks are
// contiguous in memory, so the L1 and L2 lines they occupy hold hot values
// only (in vertex-id order a line of 32 push values holds one or two).
// 1024 threads, two CTAs per SM.  Shared memory comes out of the same array
// as L1, which the other gathers need: at scale 24 the pull takes 1.12 ms
// without the cache, 1.05 ms with 2,048 hubs, 0.995 ms with 12,288 (48 KB per
// CTA), 1.00 ms with 16,384 and 2.36 ms with 26,624 (104 KB per CTA).
constexpr uint32_t kHubAuto = 12288;
constexpr uint32_t kHubMax = 16384;
constexpr uint32_t kHubMin = 1024;  // fewer hubs than this: no cache
constexpr int kHubThreads = 1024;

// Without the hub cache: 8 CTAs of 256 threads per SM, 32 registers per
// thread, full occupancy (measured faster than 6 CTAs without spills).  With
// it: 2 CTAs of 1024 threads per SM, the same 32 registers, and the hubs'
// push values in dynamic shared memory.
template <bool W, bool HUB>
__global__ void __launch_bounds__(HUB ? kHubThreads : PT_THREADS, HUB ? 2 : 8)
    k_pr_pull_warp(PrArgs A, WarpPullArgs P, int p) {
  constexpr int NT = HUB ? kHubThreads : PT_THREADS;
  // neighbour ids and weights are streamed once per pull: evict-first in L2,
  // so the gathered push values stay resident (2.6 % faster at scale 24)
  const unsigned long long l2_stream = l2_evict_first_policy();
  extern __shared__ float s_hub[];
  __shared__ double s_red[NT / 32];
  if (A.misc[M_DONE]) return;
  const bool drain = A.misc[M_PENDING] != 0;
  const float* __restrict__ pv = p == 0 ? A.pv0 : ((p & 1) ? A.pvb[1] : A.pvb[0]);
  float* pv_next = (p & 1) ? A.pvb[0] : A.pvb[1];
  if (HUB) {
    for (uint32_t h = threadIdx.x; h < P.nhub; h += NT) s_hub[h] = pv[h];
    __syncthreads();
  }
  // a column is a vertex id, or with the hub cache a rank
  auto gather = [&](uint32_t c) -> float {
    if (HUB && c < P.nhub) return s_hub[c];
    return pv[c];
  };
  const uint32_t lane = threadIdx.x & 31;
  // tiles are 32 quads, so tile indices fit 32 bits for any graph in HBM
  const uint32_t nwarps = (gridDim.x * NT) >> 5;
  const uint32_t ntiles = (uint32_t)P.ntiles;
  float res = 0.f;
  uint32_t visits = 0;
  uint32_t t = (blockIdx.x * NT + threadIdx.x) >> 5;
  uint32_t i0 = t < ntiles ? P.wtile_v0[t] : 0u;
  for (; t < ntiles; t += nwarps) {
    const uint64_t base = (uint64_t)t * kWarpTileQuads;
    const uint64_t q = base + lane;
    const bool valid = q < P.quads;
    // owner candidate i0 + lane
    const uint32_t ic = min(i0 + lane, P.nz_count);
    const bool real = ic < P.nz_count;
    const uint64_t qb_c = P.qoff[ic];
    const uint64_t qe_c = P.qoff[min(ic + 1, P.nz_count)];
    const uint64_t off_c = real ? P.off_nz[ic] : 0ull;
    const uint32_t deg_c = real ? P.deg_nz[ic] : 0u;
    const uint32_t v_c = real ? P.nz[ic] : 0u;
    // prefetch the next tile's first owner
    const uint32_t tn = t + nwarps;
    const uint32_t i0_next = tn < ntiles && tn > t ? P.wtile_v0[tn] : 0u;
    const bool starts = lane > 0 && real && qb_c < base + kWarpTileQuads;
    const unsigned heads = __reduce_or_sync(0xffffffffu, starts ? 1u << (uint32_t)(qb_c - base) : 0u);
    const uint32_t k = __popc(heads & (0xffffffffu >> (31 - lane)));
    // Per owner, two shuffled operands: the edge index of quad 0 of the
    // address space (segment offset - 4 x first quad, so a lane's first edge
    // is that + 4q) and the owner's edge count from the tile's first edge,
    // clamped (only whether a lane's quad is partial matters).
    const uint64_t ebase_c = off_c - 4ull * qb_c;
    const int64_t eend_raw = 4ll * (int64_t)(qb_c - base) + (int64_t)deg_c;
    const int eend_c = (int)(eend_raw < 4ll * kWarpTileQuads + 8 ? eend_raw : 4ll * kWarpTileQuads + 8);
    const uint64_t ebase = __shfl_sync(0xffffffffu, ebase_c, k);
    const int rem = __shfl_sync(0xffffffffu, eend_c, k) - 4 * (int)lane;
    // epilogue operands of the candidate owners, loaded before the gathers
    const bool cand_used = real && (lane == 0 || starts);
    const float dl_c = cand_used ? A.delta[v_c] : 0.f;
    const bool interior = qb_c >= base && qe_c <= base + kWarpTileQuads;
    const uint32_t run0 = lane == 0 ? 0u : (uint32_t)(qb_c - base) & 31u;
    float sum = 0.f;
    if (valid) {
      const uint4 c4 = ld_u4_hint(P.col + ebase + 4ull * q, l2_stream);
      if (W) {
        const float4 w4 = ld_f4_hint(P.w + ebase + 4ull * q, l2_stream);
        sum = gather(c4.x) * w4.x;  // the last quad of a vertex may be partial
        if (rem > 1) sum += gather(c4.y) * w4.y;
        if (rem > 2) sum += gather(c4.z) * w4.z;
        if (rem > 3) sum += gather(c4.w) * w4.w;
      } else {
        sum = gather(c4.x);
        if (rem > 1) sum += gather(c4.y);
        if (rem > 2) sum += gather(c4.z);
        if (rem > 3) sum += gather(c4.w);
      }
    }
    // segmented suffix sums: the first lane of each owner's run gets its
    // total; a lane adds lane + o while no segment starts in (lane, lane + o]
    const unsigned above = heads & ~(0xffffffffu >> (31 - lane));
    const uint32_t seg_end = above ? (uint32_t)__ffs(above) - 1u : 32u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float ts = __shfl_down_sync(0xffffffffu, sum, o);
      if (lane + o < seg_end) sum += ts;
    }
    // each candidate owner takes its total from its run's first lane and
    // finishes itself
    const float tot = __shfl_sync(0xffffffffu, sum, run0);
    if (cand_used) {
      if (interior) {
        const float dl = dl_c + tot;
        if (drain) {
          A.delta[v_c] = dl;
          res += fabsf(dl);
        } else {
          visits += activate(A, v_c, dl, pv_next, res);
        }
      } else if (tot != 0.f) {
        atomicAdd(&A.delta[v_c], tot);
      }
    }
    i0 = i0_next;
  }
  const double b = block_sum<NT>((double)res, s_red);
  if (threadIdx.x == 0 && b != 0.0) atomicAdd(&A.res[R_ACC], b);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) visits += __shfl_down_sync(0xffffffffu, visits, o);
  if ((threadIdx.x & 31) == 0 && visits) atomicAdd(&A.cnt[C_VISITS], (unsigned long long)visits);
}

// ---------------------------------------------------------- hub cache set-up

__global__ void k_count_deg_ge(const uint32_t* __restrict__ deg, uint32_t n, uint32_t d,
                               unsigned long long* cnt) {
  uint32_t c = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    c += deg[v] >= d;
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, (unsigned long long)c);
}

// sort keys: out-degree descending (complemented), values: vertex ids
__global__ void k_rank_keys(const uint32_t* __restrict__ deg, uint32_t n, uint32_t* __restrict__ key,
                            uint32_t* __restrict__ iota) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    key[v] = ~deg[v];
    iota[v] = v;
  }
}

__global__ void k_rank_scatter(const uint32_t* __restrict__ order, uint32_t n, uint32_t* __restrict__ rank) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    rank[order[i]] = i;
}

// encoded column copy: every live id replaced by its rank
__global__ void k_hub_encode(const uint32_t* __restrict__ col, uint64_t cap,
                             const uint32_t* __restrict__ rank, uint32_t n,
                             uint32_t* __restrict__ out) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < cap;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = col[e];
    out[e] = c < n ? rank[c] : c;
  }
}

// the live entries of the given rows only (block per row: in-rows of hubs
// hold up to millions of entries)
__global__ void __launch_bounds__(256) k_hub_encode_rows(const uint64_t* __restrict__ off,
                                                         const uint32_t* __restrict__ deg,
                                                         const uint32_t* __restrict__ col,
                                                         const uint32_t* __restrict__ rank, uint32_t n,
                                                         const uint32_t* __restrict__ rows,
                                                         uint64_t nrows, uint32_t* __restrict__ out) {
  for (uint64_t r = blockIdx.x; r < nrows; r += gridDim.x) {
    const uint32_t v = rows[r];
    const uint64_t b = off[v], e = b + deg[v];
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
      const uint32_t c = col[i];
      out[i] = c < n ? rank[c] : c;
    }
  }
}

sg_status cub_sort_pairs_u32_u32(sg_ctx* ctx, const uint32_t* kin, uint32_t* kout, const uint32_t* vin,
                                 uint32_t* vout, uint64_t n);

sg_status pr_hub_after_apply(sg_ctx* ctx, const uint32_t* rows, uint64_t nrows, bool patched) {
  DevGraph& g = ctx->g;
  HubView& H = g.hub;
  if (patched && H.col && H.gen + 1 == g.gen && H.layout == g.in.layout && H.cap == g.in.pool_cap) {
    H.gen = g.gen;
    return SG_OK;
  }
  // only a copy that reflected the adjacency right before this batch (one
  // generation back) in the same layout can be patched; others stay stale
  // and are re-encoded in full by the next pull
  if (!H.col || H.k == 0 || H.gen + 1 != g.gen || H.layout != g.in.layout ||
      H.cap != g.in.pool_cap)
    return SG_OK;
  if (nrows)
    k_hub_encode_rows<<<(unsigned)std::min<uint64_t>(nrows, (uint64_t)ctx->num_sms * 16), 256, 0,
                        ctx->stream>>>(g.in.off, g.in.deg, g.in.col, H.rank, g.n, rows, nrows,
                                       H.col);
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  H.gen = g.gen;
  return SG_OK;
}

// Chooses the vertex order and the hubs: ranks by out-degree, highest first
// (ties by id); the hubs are the lowest min(kmax, vertices of out-degree >= 2)
// ranks.  The order is kept while the graph takes batches (any order is
// correct; this one is chosen for locality).
static sg_status hub_choose(sg_ctx* ctx, HubView& H, const uint32_t* hot_deg, uint32_t kmax) {
  DevGraph& g = ctx->g;
  cudaStream_t st = ctx->stream;
  dfree(H.rank);
  dfree(H.col);
  H = HubView();
  H.chosen = true;
  H.kmax = kmax;
  if (kmax < kHubMin || g.n < 4 * kHubMin) return SG_OK;
  unsigned long long* d_cnt = nullptr;
  SG_TRY(dalloc(ctx, &d_cnt, 1));
  unsigned long long c = 0;
  SG_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, 8, st));
  k_count_deg_ge<<<grid_for(g.n, 256), 256, 0, st>>>(hot_deg, g.n, 2, d_cnt);
  SG_CUDA(ctx, cudaMemcpyAsync(&c, d_cnt, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  dfree(d_cnt);
  const uint32_t k = (uint32_t)std::min<unsigned long long>(c, kmax);
  if (k < kHubMin) return SG_OK;
  uint32_t *key = nullptr, *key2 = nullptr, *iota = nullptr, *order = nullptr;
  SG_TRY(dalloc(ctx, &key, g.n));
  SG_TRY(dalloc(ctx, &key2, g.n));
  SG_TRY(dalloc(ctx, &iota, g.n));
  SG_TRY(dalloc(ctx, &order, g.n));
  SG_TRY(dalloc(ctx, &H.rank, g.n));
  k_rank_keys<<<grid_for(g.n, 256), 256, 0, st>>>(hot_deg, g.n, key, iota);
  SG_TRY(cub_sort_pairs_u32_u32(ctx, key, key2, iota, order, g.n));
  k_rank_scatter<<<grid_for(g.n, 256), 256, 0, st>>>(order, g.n, H.rank);
  count_launch(ctx, 4);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  dfree(key);
  dfree(key2);
  dfree(iota);
  dfree(order);
  H.k = k;
  return SG_OK;
}

// The hub view for the current in-CSR: order and hubs chosen once per graph
// (or when the cap changes), the encoded column copy refreshed when the
// adjacency has changed since.  Returns null when the cache is off or too
// small.
static sg_status hub_view(sg_ctx* ctx, HubView& H, const DevCSR& c, const uint32_t* hot_deg,
                          const HubView** out) {
  DevGraph& g = ctx->g;
  *out = nullptr;
  const int opt = ctx->opt.pull_hubs;
  const uint32_t kmax = opt < 0 ? 0u : (opt == 0 ? kHubAuto : std::min<uint32_t>((uint32_t)opt, kHubMax));
  if (!H.chosen || H.kmax != kmax) SG_TRY(hub_choose(ctx, H, hot_deg, kmax));
  if (H.k == 0) return SG_OK;
  if (H.gen != g.gen || H.cap != c.pool_cap || !H.col) {
    if (H.cap != c.pool_cap || !H.col) {
      dfree(H.col);
      H.col = nullptr;
      H.cap = 0;
      // the copy is an optimisation: without room for it the pull runs
      // uncached (the cudaMalloc error is cleared by dalloc)
      if (dalloc(ctx, &H.col, std::max<uint64_t>(c.pool_cap, 1)) != SG_OK) {
        H.col = nullptr;
        return SG_OK;
      }
      H.cap = c.pool_cap;
    }
    k_hub_encode<<<grid_for(H.cap, 256), 256, 0, ctx->stream>>>(c.col, H.cap, H.rank, g.n,
                                                                  H.col);
    count_launch(ctx);
    SG_CUDA(ctx, cudaGetLastError());
    H.gen = g.gen;
    H.layout = c.layout;
  }
  static bool s_attr[64] = {};
  if (ctx->device >= 0 && ctx->device < 64 && !s_attr[ctx->device]) {
    SG_CUDA(ctx, cudaFuncSetAttribute(k_pr_pull_warp<false, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(kHubMax * sizeof(float))));
    SG_CUDA(ctx, cudaFuncSetAttribute(k_pr_pull_warp<true, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(kHubMax * sizeof(float))));
    s_attr[ctx->device] = true;
  }
  *out = &H;
  return SG_OK;
}

// Tile-spanning vertices, then the round's termination decision.
__global__ void __launch_bounds__(VT) k_pr_fixup(PrArgs A, const uint32_t* __restrict__ bnd,
                                                 uint32_t nb, int p) {
  __shared__ double s_red[VT / 32];
  __shared__ bool s_last;
  if (A.misc[M_DONE]) return;
  const bool drain = A.misc[M_PENDING] != 0;
  float* pv_next = (p & 1) ? A.pvb[0] : A.pvb[1];
  float res = 0.f;
  unsigned long long visits = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
    const uint32_t v = bnd[i];
    const float dl = A.delta[v];
    if (drain) res += fabsf(dl);
    else visits += activate(A, v, dl, pv_next, res);
  }
  const double b = block_sum<VT>((double)res, s_red);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) visits += __shfl_down_sync(0xffffffffu, visits, o);
  if ((threadIdx.x & 31) == 0 && visits) atomicAdd(&A.cnt[C_VISITS], visits);
  if (threadIdx.x == 0) {
    if (b != 0.0) atomicAdd(&A.res[R_ACC], b);
    __threadfence();
    s_last = atomicAdd(&A.misc[M_BLOCKS], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    const double R = atomicAdd(&A.res[R_ACC], 0.0) + A.res[R_ZERO_IN];
    A.res[R_ACC] = 0.0;
    A.res[R_LAST] = R;
    A.misc[M_BLOCKS] = 0;
    A.cnt[C_EDGES] += A.live_edges;
    if (drain) {
      A.misc[M_DONE] = 1;
      return;
    }
    const uint32_t rounds = A.misc[M_ROUNDS] + 1;
    A.misc[M_ROUNDS] = rounds;
    if (R < A.tau) A.misc[M_PENDING] = 1;
    if ((int)rounds >= A.max_rounds && !(R < A.tau)) {
      A.misc[M_PENDING] = 1;
      A.misc[M_NOTCONV] = 1;
    }
  }
}

__global__ void k_pr_init(uint32_t n, float* x, float* delta, float init_c) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    x[v] = 0.f;         // init_v (pagerank_ingress.h:32)
    delta[v] = init_c;  // init_c = (1-d)/N (pagerank_ingress.h:27-30)
  }
}

__global__ void __launch_bounds__(VT) k_pr_residual(uint32_t n, const float* delta, double* res) {
  __shared__ double s_red[VT / 32];
  double r = 0.0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    r += fabs((double)delta[v]);
  const double b = block_sum<VT>(r, s_red);
  if (threadIdx.x == 0) atomicAdd(&res[R_ACC], b);
}

__global__ void k_pr_seed(const uint32_t* __restrict__ seeds, uint32_t cnt, float* delta,
                          float mass) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    atomicAdd(delta + seeds[i], mass);
}

sg_status pr_free(sg_ctx* ctx) {
  PrState& s = ctx->pr;
  dfree(s.x); dfree(s.delta); dfree(s.acc); dfree(s.pv);
  dfree(s.d_misc); dfree(s.d_res); dfree(s.d_cnt);
  s = PrState();
  return SG_OK;
}

sg_status pr_alloc(sg_ctx* ctx) {
  PrState& s = ctx->pr;
  const uint32_t n = std::max(ctx->g.n, summary_rows(ctx));  // mirror rows too
  if (s.x && s.n_alloc == n) {  // same size: keep the buffers
    s.valid = false;
    return SG_OK;
  }
  pr_free(ctx);
  SG_TRY(dalloc(ctx, &s.x, n));
  SG_TRY(dalloc(ctx, &s.delta, n));
  SG_TRY(dalloc(ctx, &s.acc, n));       // pv0
  SG_TRY(dalloc(ctx, &s.pv, 2ull * n)); // pvb[0], pvb[1]
  SG_TRY(dalloc(ctx, &s.d_misc, M_WORDS));
  SG_TRY(dalloc(ctx, &s.d_res, R_WORDS));
  SG_TRY(dalloc(ctx, &s.d_cnt, C_WORDS));
  s.n_alloc = n;
  return SG_OK;
}

PrAmendArgs pr_amend_args(sg_ctx* ctx) {
  PrAmendArgs a{};
  a.active = ctx->pr.valid;
  a.x = ctx->pr.x;
  a.delta = ctx->pr.delta;
  a.damping = (float)ctx->opt.damping;
  return a;
}

static sg_status pr_rounds(sg_ctx* ctx);

// Runs rounds until the residual test passes (or the round cap).  inc=false
// starts from init_v / init_c; inc=true continues from the amended state.
sg_status pr_run(sg_ctx* ctx, bool inc) {
  DevGraph& g = ctx->g;
  PrState& s = ctx->pr;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  cudaStream_t st = ctx->stream;
  if (!inc) {
    if (!s.x) SG_TRY(pr_alloc(ctx));
    const float init_c = (float)((1.0 - ctx->opt.damping) / (double)g.n);
    k_pr_init<<<grid_for(g.n, 256), 256, 0, st>>>(g.n, s.x, s.delta, init_c);
    count_launch(ctx);
  } else if (!s.valid) {
    return fail(ctx, SG_ERR_STATE, "PageRank IncEval before PEval");
  }
  return pr_rounds(ctx);
}

// Personalized PageRank (ppr/ppr.h's teleport to a seed set): x = 0, delta =
// (1-d)/|seeds| on the seeds, then the same rounds.
sg_status pr_run_personalized(sg_ctx* ctx, const uint32_t* d_seeds, uint32_t n_seeds) {
  DevGraph& g = ctx->g;
  PrState& s = ctx->pr;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  if (n_seeds == 0) return fail(ctx, SG_ERR_INVALID, "personalized PageRank needs seeds");
  cudaStream_t st = ctx->stream;
  if (!s.x) SG_TRY(pr_alloc(ctx));
  k_pr_init<<<grid_for(g.n, 256), 256, 0, st>>>(g.n, s.x, s.delta, 0.f);
  k_pr_seed<<<grid_for(n_seeds, 256), 256, 0, st>>>(
      d_seeds, n_seeds, s.delta, (float)((1.0 - ctx->opt.damping) / (double)n_seeds));
  count_launch(ctx, 2);
  return pr_rounds(ctx);
}

sg_status pr_rounds_ex(sg_ctx* ctx, const PrRunSpec& R) {
  DevGraph& g = ctx->g;
  cudaStream_t st = ctx->stream;
  if (R.lists == &g.in_wl) SG_TRY(graph_in_worklists(ctx));
  const PrBufs& s = R.buf;
  const PullLists& L = *R.lists;
  SG_CUDA(ctx, cudaMemsetAsync(s.misc, 0, sizeof(uint32_t) * M_WORDS, st));
  SG_CUDA(ctx, cudaMemsetAsync(s.res, 0, sizeof(double) * R_WORDS, st));
  SG_CUDA(ctx, cudaMemsetAsync(s.cnt, 0, sizeof(unsigned long long) * C_WORDS, st));

  PrArgs A;
  A.n = g.n;
  A.damping = (float)ctx->opt.damping;
  A.thr_v = (float)(R.tau / (double)g.n);
  A.tau = R.tau;
  A.max_rounds = ctx->opt.max_rounds > 0 ? ctx->opt.max_rounds : 1000;
  A.live_edges = g.m;
  A.scale_deg = R.scale_deg;
  A.pull_deg = R.csr->deg;
  A.x = s.x;
  A.delta = s.delta;
  A.pv0 = s.pv0;
  A.pvb[0] = s.pvb;
  A.pvb[1] = s.pvb + g.n;
  A.misc = s.misc;
  A.res = s.res;
  A.cnt = s.cnt;
  A.rank = nullptr;

  WarpPullArgs WP;
  WP.nz = L.nz;
  WP.qoff = L.qoff;
  WP.off_nz = L.off_nz;
  WP.deg_nz = L.deg_nz;
  WP.wtile_v0 = L.wtile_v0;
  WP.nz_count = L.nz_count;
  WP.quads = L.quads;
  WP.ntiles = L.nwtiles;
  WP.col = R.csr->col;
  WP.w = R.weighted ? R.csr->w : nullptr;
  WP.nhub = 0;
  const uint32_t* bnd = L.wbnd;
  const uint32_t nbnd = L.wbnd_count;

  SG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  // the hub cache serves pulls over the in-CSR (its encoded column copy)
  const HubView* hub = nullptr;
  // pulls over the in-CSR gather the push values of in-neighbours (hot:
  // high out-degree), the adjoint's pulls over the out-CSR those of
  // out-neighbours (hot: high in-degree); each direction has its own view
  if (R.csr == &g.in && L.quads > 0) SG_TRY(hub_view(ctx, g.hub, g.in, g.out.deg, &hub));
  else if (R.csr == &g.out && L.quads > 0)
    SG_TRY(hub_view(ctx, g.hub_out, g.out, g.in.deg, &hub));
  if (hub) {
    WP.col = hub->col;
    WP.nhub = hub->k;
    A.rank = hub->rank;  // push values in the pull's vertex order
  }
  const int pt = hub ? kHubThreads : PT_THREADS;
  const size_t hub_smem = hub ? (size_t)hub->k * sizeof(float) : 0;
  const unsigned vblocks = grid_for(g.n, VT, ctx->num_sms * 8);
  const unsigned wblocks = (unsigned)std::min<uint64_t>(
      std::max<uint64_t>((L.nwtiles + pt / 32 - 1) / (pt / 32), 1),
      (uint64_t)ctx->num_sms * (hub ? 2 : 8));
  const unsigned fblocks = grid_for(std::max<uint32_t>(nbnd, 1), VT, ctx->num_sms * 2);
  const int kpull = R.kclass;

  kprof_begin(ctx);
  k_pr_vertex<<<vblocks, VT, 0, st>>>(A);
  kprof_end(ctx, SG_K_PR_VERTEX);
  uint32_t h_misc[M_WORDS] = {0};
  int pull = 0;
  if (L.quads > 0) {
    // the first pull distributes the first round's activations
    const int chunk = 4;
    for (;;) {
      for (int r = 0; r < chunk; ++r, ++pull) {
        kprof_begin(ctx);
        if (hub) {
          if (R.weighted) k_pr_pull_warp<true, true><<<wblocks, pt, hub_smem, st>>>(A, WP, pull);
          else k_pr_pull_warp<false, true><<<wblocks, pt, hub_smem, st>>>(A, WP, pull);
        } else {
          if (R.weighted) k_pr_pull_warp<true, false><<<wblocks, pt, 0, st>>>(A, WP, pull);
          else k_pr_pull_warp<false, false><<<wblocks, pt, 0, st>>>(A, WP, pull);
        }
        kprof_end(ctx, kpull);
        kprof_begin(ctx);
        k_pr_fixup<<<fblocks, VT, 0, st>>>(A, bnd, nbnd, pull);
        kprof_end(ctx, SG_K_PR_VERTEX);
      }
      SG_CUDA(ctx, cudaGetLastError());
      SG_CUDA(ctx, cudaMemcpyAsync(h_misc, s.misc, sizeof(h_misc), cudaMemcpyDeviceToHost, st));
      SG_CUDA(ctx, cudaStreamSynchronize(st));
      if (h_misc[M_DONE]) break;
      if (pull > 2 * A.max_rounds + 64) break;  // host-side guard
    }
  }
  // final residual over every vertex
  SG_CUDA(ctx, cudaMemsetAsync(s.res, 0, sizeof(double), st));
  k_pr_residual<<<vblocks, VT, 0, st>>>(g.n, s.delta, s.res);
  count_launch(ctx);
  SG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  double h_res[R_WORDS];
  unsigned long long h_cnt[C_WORDS];
  SG_CUDA(ctx, cudaMemcpyAsync(h_res, s.res, sizeof(h_res), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(h_cnt, s.cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(h_misc, s.misc, sizeof(h_misc), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.rounds = (int32_t)h_misc[M_ROUNDS] + 1;
  ctx->stats.converged = h_misc[M_NOTCONV] ? 0 : 1;
  ctx->stats.residual = h_res[R_ACC];
  ctx->stats.edges_relaxed = h_cnt[C_EDGES];
  ctx->stats.edges_pull = h_cnt[C_EDGES];
  ctx->stats.edges_push = 0;
  ctx->stats.vertex_visits = h_cnt[C_VISITS];
  ctx->stats.elapsed_ms = ms;
  ctx->stats.live_edges = g.m;
  if (h_misc[M_NOTCONV])
    return fail(ctx, SG_ERR_NOT_CONVERGED, "PageRank reached the round cap");
  return SG_OK;
}

static sg_status pr_rounds(sg_ctx* ctx) {
  DevGraph& g = ctx->g;
  PrState& s = ctx->pr;
  PrRunSpec R;
  R.buf.x = s.x;
  R.buf.delta = s.delta;
  R.buf.pv0 = s.acc;
  R.buf.pvb = s.pv;
  R.buf.misc = s.d_misc;
  R.buf.res = s.d_res;
  R.buf.cnt = (unsigned long long*)s.d_cnt;
  R.lists = &g.in_wl;
  R.csr = &g.in;
  R.weighted = false;
  R.scale_deg = g.out.deg;
  R.tau = ctx->opt.termcheck_threshold;
  R.kclass = SG_K_PR_PULL;
  const sg_status st = pr_rounds_ex(ctx, R);
  if (st == SG_OK || st == SG_ERR_NOT_CONVERGED) s.valid = true;
  return st;
}

}  // namespace sg
