// Weighted SSSP with FP64 distances: delta-stepping (near / far queues) in
// one cooperative persistent kernel, plus the incremental path.
//
// Distances are stored as the bit patterns of non-negative doubles, so an
// unsigned 64-bit atomicMin is an exact min (integer weights give exact FP64
// sums below 2^53; results are bit-identical to Dijkstra).  This replaces
// SSSPIngress's DependencyData::SetIfLessThanAtomic CAS loop
// (grape/utils/dependency_data.h:21-34) and the reference's bitmap-frontier
// rounds (sum_sync_traversal_worker.h:1037-1300).
//
// Every wait in the persistent kernel is a grid barrier with a bounded spin;
// on expiry the kernel records an error word and every block returns.
#include <algorithm>
#include <cmath>

#include "ctx.h"
#include "dev.cuh"

namespace sg {

enum {
  S_Q0 = 0, S_Q1 = 1, S_Q2 = 2,      // near queue counts (rotating slots)
  S_F0 = 3, S_F1 = 4,                // far queue counts (rotating by split)
  S_BAR_COUNT = 5, S_BAR_GEN = 6,
  S_ERR = 7,
  S_ITERS = 8,
  S_SPLITS = 9,
  S_H0 = 10, S_H1 = 11, S_H2 = 12,   // deferred long-row counts (slots as near)
  S_WORDS = 16
};
enum { SC_EDGES = 0, SC_IMPROVE = 1, SC_VISITS = 2, SC_MIN = 3, SC_WORDS = 4 };

// Rows (in- or out-adjacency) longer than kHeavyRow are left by the warp
// kernels to a second kernel in which every CTA scans a share of each such
// row: a hub's row on one warp would be the tail of the launch.  A deferred
// row keeps its vertex and a 64-bit result (a distance key or a vertex id,
// reduced by atomicMin).
constexpr uint32_t kHeavyRow = 4096;

struct HeavyRows {
  uint32_t* list;
  unsigned long long* best;
  uint32_t* cnt;
  uint32_t cap;
};

// called by one lane; false when the list is full (the warp then scans the
// row itself)
__device__ __forceinline__ bool defer_heavy(const HeavyRows& H, uint32_t v, unsigned long long init) {
  const uint32_t s = atomicAdd(H.cnt, 1u);
  if (s >= H.cap) return false;
  H.list[s] = v;
  H.best[s] = init;
  return true;
}

__device__ __forceinline__ uint32_t heavy_count(const HeavyRows& H) { return min(*H.cnt, H.cap); }

// warp-uniform: whether lane 0 deferred the row
__device__ __forceinline__ bool warp_defer(const HeavyRows& H, uint32_t v, unsigned long long init) {
  const bool ok = (threadIdx.x & 31) == 0 ? defer_heavy(H, v, init) : false;
  return __shfl_sync(0xffffffffu, ok, 0);
}

struct SsspArgs {
  uint32_t n;
  const uint64_t* off;
  const uint32_t* deg;
  const uint32_t* col;
  const float* w;
  unsigned long long* dist;
  uint32_t* stamp;       // near de-duplication: last iteration a vertex was queued
  uint32_t* fstamp;      // far de-duplication: last split epoch
  uint32_t* nq[3];       // near queues
  uint32_t* fq[2];       // far queues
  uint32_t* ctl;
  unsigned long long* cnt;
  double delta;
  uint32_t iter_base;    // stamps start above this value
  uint64_t fcap;         // far queue capacity
  long long spin_limit;
  // IncEval only (null in PEval): every vertex whose distance improves is
  // listed once (tag chg_tag) for the parent refresh
  uint32_t* chg_mark;
  uint32_t* chg_list;
  uint32_t* chg_cnt;
  uint32_t chg_tag;
  // vertices of a near queue with out-rows longer than kHeavyRow are
  // deferred to the next iteration, in which every warp relaxes a share of
  // each (null: relaxed by one warp); three slots of hcap, rotating as the
  // near queues
  uint32_t* hq[3];
  uint32_t hcap;
};

__device__ __forceinline__ void note_change(const SsspArgs& A, uint32_t x) {
  if (A.chg_mark && atomicExch(A.chg_mark + x, A.chg_tag) != A.chg_tag)
    A.chg_list[atomicAdd(A.chg_cnt, 1u)] = x;
}

__device__ __forceinline__ bool grid_sync(const SsspArgs& A) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = A.ctl + S_BAR_GEN;
    const uint32_t g = *gen;
    __threadfence();
    if (atomicAdd(A.ctl + S_BAR_COUNT, 1u) == gridDim.x - 1) {
      A.ctl[S_BAR_COUNT] = 0;
      __threadfence();
      atomicAdd(A.ctl + S_BAR_GEN, 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > A.spin_limit) {
          atomicExch(A.ctl + S_ERR, 1u);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile uint32_t*)(A.ctl + S_ERR) == 0;
}

// Failure detection of the grid barrier above: a few CTAs meet at it; with
// `skip` the last CTA leaves without arriving, so the others' bounded waits
// run out and set the error word instead of hanging the GPU.
__global__ void k_barrier_probe(SsspArgs A, int skip) {
  if (skip && blockIdx.x == gridDim.x - 1) return;
  grid_sync(A);
}

// Relaxes one 128-edge chunk (4-edge quad per lane, 128-bit loads of
// neighbour and weight arrays) of vertex v's out-row; improved vertices go
// to the next near queue (inside the window) or the far queue.
__device__ __forceinline__ void relax_chunk(const SsspArgs& A, uint64_t base, uint32_t d, uint32_t kb,
                                            double dv, double thr, uint32_t* nq_next,
                                            uint32_t* nq_cnt, uint32_t* fq, uint32_t* fq_cnt,
                                            uint32_t tag, unsigned long long& improve) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t k = kb + lane * 4;
  uint32_t cc[4] = {kInvalidVid, kInvalidVid, kInvalidVid, kInvalidVid};
  float ww[4] = {0.f, 0.f, 0.f, 0.f};
  if (k < d) {
    const uint4 c4 = *reinterpret_cast<const uint4*>(A.col + base + k);
    const float4 w4 = *reinterpret_cast<const float4*>(A.w + base + k);
    cc[0] = c4.x; cc[1] = k + 1 < d ? c4.y : kInvalidVid;
    cc[2] = k + 2 < d ? c4.z : kInvalidVid; cc[3] = k + 3 < d ? c4.w : kInvalidVid;
    ww[0] = w4.x; ww[1] = w4.y; ww[2] = w4.z; ww[3] = w4.w;
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    bool to_near = false, to_far = false;
    const uint32_t x = cc[t];
    if (x != kInvalidVid) {
      const double nd = dv + (double)ww[t];
      const unsigned long long nb = dbits(nd);
      if (nb < A.dist[x]) {
        const unsigned long long old = atomicMin(A.dist + x, nb);
        if (nb < old) {
          improve++;
          note_change(A, x);
          if (nd < thr) {
            to_near = atomicExch(A.stamp + x, tag) != tag;
          } else {
            to_far = true;
          }
        }
      }
    }
    const uint32_t sn = warp_append(to_near, nq_cnt);
    if (to_near) nq_next[sn] = x;
    const uint32_t sf = warp_append(to_far, fq_cnt);
    if (to_far) {
      if (sf < A.fcap) fq[sf] = x; else atomicExch(A.ctl + S_ERR, 2u);
    }
  }
}

// Relaxes the out-edges of every vertex in `q` (warp per vertex) and a
// share of every long row deferred by the previous iteration (`hq`, `hn`:
// all warps of the grid split each); long rows of `q` are deferred to
// `hq_next` when the heavy slots are in use.
__device__ __forceinline__ void relax_queue(const SsspArgs& A, const uint32_t* q, uint32_t qn,
                                            const uint32_t* hq, uint32_t hn, uint32_t* hq_next,
                                            uint32_t* hq_cnt, double thr, uint32_t* nq_next,
                                            uint32_t* nq_cnt, uint32_t* fq, uint32_t* fq_cnt,
                                            uint32_t tag, unsigned long long& edges,
                                            unsigned long long& improve) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (uint32_t i = wid; i < qn; i += nwarps) {
    const uint32_t v = __ldcg(q + i);
    const uint32_t d = A.deg[v];
    if (d > kHeavyRow && hq_next) {
      bool deferred = false;
      if (lane == 0) {
        const uint32_t s = atomicAdd(hq_cnt, 1u);
        deferred = s < A.hcap;
        if (deferred) hq_next[s] = v;
      }
      if (__shfl_sync(0xffffffffu, deferred, 0)) continue;
    }
    const double dv = bitsd(__ldcg(A.dist + v));
    const uint64_t base = A.off[v];
    if (lane == 0) edges += d;
    for (uint32_t kb = 0; kb < d; kb += 128)
      relax_chunk(A, base, d, kb, dv, thr, nq_next, nq_cnt, fq, fq_cnt, tag, improve);
  }
  for (uint32_t h = 0; h < hn; ++h) {
    const uint32_t v = __ldcg(hq + h);
    const uint32_t d = A.deg[v];
    const double dv = bitsd(__ldcg(A.dist + v));
    const uint64_t base = A.off[v];
    if (wid == 0 && lane == 0) edges += d;
    for (uint64_t kb = (uint64_t)wid * 128; kb < d; kb += (uint64_t)nwarps * 128)
      relax_chunk(A, base, d, (uint32_t)kb, dv, thr, nq_next, nq_cnt, fq, fq_cnt, tag, improve);
  }
}

__global__ void __launch_bounds__(256) k_sssp_persistent(SsspArgs A) {
  __shared__ unsigned long long s_red[8];
  unsigned long long edges = 0, improve = 0;
  uint32_t it = 0;       // near iterations
  uint32_t seq = 0;      // phases so far: every phase gets a fresh queue tag
  uint32_t fslot = 0;    // current far queue
  double thr = 0.0;      // current window end

  // iteration `it` reads near slot it % 3, appends to (it+1) % 3 and clears
  // (it+2) % 3; the host seeds slot 0 or the far queue.
  bool ok = true;
  for (;;) {
    const uint32_t rs = it % 3, ws = (it + 1) % 3, cs = (it + 2) % 3;
    const uint32_t qn = *(volatile uint32_t*)(A.ctl + S_Q0 + rs);
    const uint32_t hn = A.hq[0] ? min(*(volatile uint32_t*)(A.ctl + S_H0 + rs), A.hcap) : 0u;
    if (qn == 0 && hn == 0) {
      // bucket advance: smallest far distance decides the next window
      const uint32_t fn = *(volatile uint32_t*)(A.ctl + S_F0 + fslot);
      if (fn == 0) break;
      if (blockIdx.x == 0 && threadIdx.x == 0) A.cnt[SC_MIN] = kInfBits;
      if (!(ok = grid_sync(A))) break;
      // smallest distance among far entries not already settled: entries of
      // vertices finished in an earlier window are stale and ignored
      const unsigned long long settled_b = dbits(thr);
      unsigned long long mn = kInfBits;
      for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < fn; i += gridDim.x * blockDim.x) {
        const unsigned long long dx = __ldcg(A.dist + __ldcg(A.fq[fslot] + i));
        if (dx >= settled_b && dx < mn) mn = dx;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xffffffffu, mn, o);
        mn = t < mn ? t : mn;
      }
      if ((threadIdx.x & 31) == 0 && mn != kInfBits) atomicMin(A.cnt + SC_MIN, mn);
      if (!(ok = grid_sync(A))) break;
      const unsigned long long mnb = *(volatile unsigned long long*)(A.cnt + SC_MIN);
      const uint32_t nf = fslot ^ 1u;
      if (mnb >= kInfBits) {
        // nothing reachable left in the far queue
        if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl[S_F0 + fslot] = 0;
        if (!(ok = grid_sync(A))) break;
        continue;
      }
      const double mind = bitsd(mnb);
      const double settled = thr;  // everything below the old window is final
      thr = (floor(mind / A.delta) + 1.0) * A.delta;
      const uint32_t tag = A.iter_base + (++seq);
      const uint32_t epoch = tag;
      if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl[S_F0 + nf] = 0;
      if (!(ok = grid_sync(A))) break;
      const uint32_t fn_full = ((fn + 31u) / 32u) * 32u;
      for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < fn_full; i += gridDim.x * blockDim.x) {
        bool to_near = false, to_far = false;
        uint32_t x = 0;
        if (i < fn) {
          x = __ldcg(A.fq[fslot] + i);
          const double dx = bitsd(__ldcg(A.dist + x));
          if (dx < settled) {
            // stale entry of a vertex finished in an earlier window
          } else if (dx < thr) {
            to_near = atomicExch(A.stamp + x, tag) != tag;
          } else {
            to_far = atomicExch(A.fstamp + x, epoch) != epoch;
          }
        }
        const uint32_t sn = warp_append(to_near, A.ctl + S_Q0 + rs);
        if (to_near) A.nq[rs][sn] = x;
        const uint32_t sf = warp_append(to_far, A.ctl + S_F0 + nf);
        if (to_far) A.fq[nf][sf] = x;
      }
      fslot = nf;
      if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl[S_SPLITS] = seq;
      if (!(ok = grid_sync(A))) break;
      continue;
    }
    // relax the near queue.  Slot cs was read in the previous iteration and
    // is appended to in the next one; nobody touches it in this one.  The
    // read slot rs keeps its count until it becomes cs again.
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      A.ctl[S_Q0 + cs] = 0;
      A.ctl[S_H0 + cs] = 0;
      A.ctl[S_ITERS] = it + 1;
      A.ctl[S_SPLITS] = seq + 1;
    }
    relax_queue(A, A.nq[rs], qn, A.hq[rs], hn, A.hq[ws], A.ctl + S_H0 + ws, thr, A.nq[ws],
                A.ctl + S_Q0 + ws, A.fq[fslot], A.ctl + S_F0 + fslot, A.iter_base + (++seq),
                edges, improve);
    if (!(ok = grid_sync(A))) break;
    ++it;
  }
  // counters
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    edges += __shfl_down_sync(0xffffffffu, edges, o);
    improve += __shfl_down_sync(0xffffffffu, improve, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (edges) atomicAdd(A.cnt + SC_EDGES, edges);
    if (improve) atomicAdd(A.cnt + SC_IMPROVE, improve);
  }
  (void)s_red;
  (void)ok;
}

// parent[v] = smallest in-neighbour u with dist[u] + w(u,v) == dist[v]
__global__ void k_sssp_parents(uint32_t n, uint32_t source, const uint64_t* __restrict__ off,
                               const uint32_t* __restrict__ deg, const uint32_t* __restrict__ col,
                               const float* __restrict__ w,
                               const unsigned long long* __restrict__ dist,
                               uint32_t* __restrict__ parent) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nwarps) {
    const unsigned long long dvb = dist[v];
    uint32_t best = kInvalidVid;
    if (v != source && dvb < kInfBits) {
      const uint32_t d = deg[v];
      const uint64_t base = off[v];
      for (uint32_t k = lane; k < d; k += 32) {
        const uint32_t u = col[base + k];
        const unsigned long long dub = dist[u];
        if (dub < kInfBits && dbits(bitsd(dub) + (double)w[base + k]) == dvb && u < best) best = u;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_down_sync(0xffffffffu, best, o));
    }
    if (lane == 0) parent[v] = best;
  }
}

// The same over a list of vertices (IncEval: only vertices whose parent can
// have changed).
__global__ void k_sssp_parents_list(const uint32_t* __restrict__ list, const uint32_t* cnt_dev,
                                    uint32_t source, const uint64_t* __restrict__ off,
                                    const uint32_t* __restrict__ deg,
                                    const uint32_t* __restrict__ col, const float* __restrict__ w,
                                    const unsigned long long* __restrict__ dist,
                                    uint32_t* __restrict__ parent, HeavyRows H) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t cnt = *cnt_dev;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nwarps) {
    const uint32_t v = list[i];
    const unsigned long long dvb = dist[v];
    uint32_t best = kInvalidVid;
    if (v != source && dvb < kInfBits) {
      const uint32_t d = deg[v];
      const uint64_t base = off[v];
      if (d > kHeavyRow && warp_defer(H, v, kInvalidVid)) continue;
      for (uint32_t k = lane; k < d; k += 32) {
        const uint32_t u = col[base + k];
        const unsigned long long dub = dist[u];
        if (dub < kInfBits && dbits(bitsd(dub) + (double)w[base + k]) == dvb && u < best) best = u;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_down_sync(0xffffffffu, best, o));
    }
    if (lane == 0) parent[v] = best;
  }
}

// The parent of every vertex is its smallest tight in-neighbour.  After an
// IncEval it can change only for (a) vertices whose distance changed (reset
// or improved), (b) heads of inserted or re-weighted edges, and (c) vertices
// that gain a smaller tight in-neighbour among the changed vertices: a
// vertex whose distance is unchanged keeps a tight parent, since that parent
// is unchanged too (a parent that got shorter would shorten the child; one
// that got longer was reset with its subtree).  (a) and (b) are recomputed
// in full over the in-row, (c) by a push over the changed vertices'
// out-edges.

// the vertices of (a) and (b), each once by the parent marks
__global__ void k_parent_list(const uint32_t* __restrict__ chg, uint32_t nchg,
                              const uint32_t* __restrict__ heads, uint32_t nheads,
                              uint32_t* __restrict__ mark, uint32_t tag, uint32_t* __restrict__ out,
                              uint32_t* __restrict__ cnt) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nchg + nheads;
       i += gridDim.x * blockDim.x) {
    const uint32_t u = i < nchg ? chg[i] : heads[i - nchg];
    if (atomicExch(mark + u, tag) != tag) out[atomicAdd(cnt, 1u)] = u;
  }
}

// every CTA: its share of each deferred in-row, smallest tight in-neighbour
__global__ void __launch_bounds__(256) k_heavy_parent_scan(HeavyRows H, uint32_t source,
                                                           const uint64_t* __restrict__ off,
                                                           const uint32_t* __restrict__ deg,
                                                           const uint32_t* __restrict__ col,
                                                           const float* __restrict__ w,
                                                           const unsigned long long* __restrict__ dist) {
  const uint32_t nh = heavy_count(H);
  for (uint32_t h = 0; h < nh; ++h) {
    const uint32_t v = H.list[h];
    const unsigned long long dvb = dist[v];
    if (v == source || dvb >= kInfBits) continue;
    const uint32_t d = deg[v];
    const uint64_t base = off[v];
    uint32_t best = kInvalidVid;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < d; k += gridDim.x * blockDim.x) {
      const uint32_t u = col[base + k];
      const unsigned long long dub = dist[u];
      if (dub < kInfBits && dbits(bitsd(dub) + (double)w[base + k]) == dvb && u < best) best = u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_down_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best != kInvalidVid)
      atomicMin(H.best + h, (unsigned long long)best);
  }
}

__global__ void k_heavy_parent_apply(HeavyRows H, uint32_t* __restrict__ parent) {
  const uint32_t nh = heavy_count(H);
  for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x)
    parent[H.list[h]] = (uint32_t)H.best[h];
}

// (c): a changed vertex u lowers the parent of an unchanged out-neighbour v
// when the edge is tight (warp per changed vertex; long out-rows deferred)
__device__ __forceinline__ void push_parent(uint32_t u, unsigned long long dub, uint32_t v, float wv,
                                            uint32_t source, const unsigned long long* dist,
                                            const uint32_t* chg_mark, uint32_t tag,
                                            uint32_t* parent) {
  if (v == source || chg_mark[v] == tag) return;
  if (dbits(bitsd(dub) + (double)wv) == dist[v]) atomicMin(parent + v, u);
}

__global__ void k_parent_push(const uint32_t* __restrict__ chg, uint32_t nchg, uint32_t source,
                              const uint64_t* __restrict__ off, const uint32_t* __restrict__ deg,
                              const uint32_t* __restrict__ col, const float* __restrict__ w,
                              const unsigned long long* __restrict__ dist,
                              const uint32_t* __restrict__ chg_mark, uint32_t tag,
                              uint32_t* __restrict__ parent, HeavyRows H) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nchg; i += nwarps) {
    const uint32_t u = chg[i];
    const unsigned long long dub = dist[u];
    if (dub >= kInfBits) continue;
    const uint32_t d = deg[u];
    if (d > kHeavyRow && warp_defer(H, u, 0ull)) continue;
    const uint64_t base = off[u];
    for (uint32_t k = lane; k < d; k += 32)
      push_parent(u, dub, col[base + k], w[base + k], source, dist, chg_mark, tag, parent);
  }
}

__global__ void __launch_bounds__(256) k_heavy_parent_push(HeavyRows H, uint32_t source,
                                                           const uint64_t* __restrict__ off,
                                                           const uint32_t* __restrict__ deg,
                                                           const uint32_t* __restrict__ col,
                                                           const float* __restrict__ w,
                                                           const unsigned long long* __restrict__ dist,
                                                           const uint32_t* __restrict__ chg_mark,
                                                           uint32_t tag, uint32_t* __restrict__ parent) {
  const uint32_t nh = heavy_count(H);
  for (uint32_t h = 0; h < nh; ++h) {
    const uint32_t u = H.list[h];
    const unsigned long long dub = dist[u];
    const uint32_t d = deg[u];
    const uint64_t base = off[u];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < d; k += gridDim.x * blockDim.x)
      push_parent(u, dub, col[base + k], w[base + k], source, dist, chg_mark, tag, parent);
  }
}

// Reset BFS over the shortest-path tree in one cooperative launch: level by
// level, children whose parent is a reset vertex join the list (deltaCompute,
// sum_sync_traversal_worker.h:183-226); then the whole list is reset and
// recorded as changed.  ctl: [0] bar count, [1] bar gen, [2] err, [3] next.
struct ResetArgs {
  const uint32_t* seed_cnt;
  uint32_t* list;
  uint32_t cap;
  const uint64_t* off;
  const uint32_t* deg;
  const uint32_t* col;
  uint32_t* parent;
  uint32_t* reset;
  unsigned long long* dist;
  uint32_t* ctl;
  uint32_t* chg_mark;
  uint32_t* chg_list;
  uint32_t* chg_cnt;
  uint32_t chg_tag;
  long long spin_limit;
  uint32_t* hv;       // two halves of hv_half entries: long rows deferred by a level
  uint32_t hv_half;
};

__device__ __forceinline__ bool reset_sync(const ResetArgs& A) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = A.ctl + 1;
    const uint32_t g = *gen;
    __threadfence();
    if (atomicAdd(A.ctl + 0, 1u) == gridDim.x - 1) {
      A.ctl[0] = 0;
      __threadfence();
      atomicAdd(A.ctl + 1, 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > A.spin_limit) {
          atomicExch(A.ctl + 2, 1u);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile uint32_t*)(A.ctl + 2) == 0;
}

// children of x whose parent is x join the list (warp w of nw scans the
// row's 32-entry chunks w, w + nw, ...)
__device__ __forceinline__ void reset_scan_row(const ResetArgs& A, uint32_t x, uint32_t w,
                                               uint32_t nw) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t d = A.deg[x];
  const uint64_t base = A.off[x];
  for (uint64_t kb = (uint64_t)w * 32; kb < d; kb += (uint64_t)nw * 32) {
    const uint64_t k = kb + lane;
    bool take = false;
    uint32_t y = 0;
    if (k < d) {
      y = A.col[base + k];
      take = __ldcg(A.parent + y) == x && y != x && atomicExch(A.reset + y, 1u) == 0u;
    }
    const uint32_t s0 = warp_append(take, A.ctl + 3);
    if (take) {
      if (s0 < A.cap) A.list[s0] = y;
      else atomicExch(A.ctl + 2, 2u);
    }
  }
}

// Each level: warps scan the short out-rows of the level's vertices, and
// every warp of the grid scans a share of each long row deferred by the
// previous level (a hub's row on one warp would hold the level's barrier).
// Children found from a deferred row join one level late, which the
// closure does not mind.  ctl [6], [7]: deferred counts by level parity.
__global__ void __launch_bounds__(256) k_sssp_reset_all(ResetArgs A) {
  __shared__ uint32_t s_end, s_hv;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t begin = 0;
  uint32_t end = min(*(volatile const uint32_t*)A.seed_cnt, A.cap);
  uint32_t hv_prev = 0;
  for (uint32_t lvl = 0; end > begin || hv_prev > 0; ++lvl) {
    const uint32_t cur = lvl & 1;
    uint32_t* hv_cur = A.hv + (size_t)cur * A.hv_half;
    const uint32_t* hv_old = A.hv + (size_t)(cur ^ 1) * A.hv_half;
    for (uint32_t i = begin + wid; i < end; i += nwarps) {
      const uint32_t x = __ldcg(A.list + i);
      if (A.deg[x] > kHeavyRow) {
        bool deferred = false;
        if (lane == 0) {
          const uint32_t s = atomicAdd(A.ctl + 6 + cur, 1u);
          deferred = s < A.hv_half;
          if (deferred) hv_cur[s] = x;
        }
        if (__shfl_sync(0xffffffffu, deferred, 0)) continue;
      }
      reset_scan_row(A, x, 0, 1);
    }
    for (uint32_t h = 0; h < hv_prev; ++h) reset_scan_row(A, __ldcg(hv_old + h), wid, nwarps);
    if (!reset_sync(A)) return;
    if (threadIdx.x == 0) {
      s_end = min(*(volatile uint32_t*)(A.ctl + 3), A.cap);
      s_hv = min(*(volatile uint32_t*)(A.ctl + 6 + cur), A.hv_half);
    }
    __syncthreads();
    begin = end;
    end = s_end;
    hv_prev = s_hv;
    // the previous level's deferred list is consumed: its counter serves
    // the next level
    if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl[6 + (cur ^ 1)] = 0;
    if (!reset_sync(A)) return;
  }
  // reset the whole list (the BFS above read the old parents)
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
    const uint32_t v = A.list[i];
    A.dist[v] = kInfBits;
    A.parent[v] = kInvalidVid;
    if (atomicExch(A.chg_mark + v, A.chg_tag) != A.chg_tag) A.chg_list[atomicAdd(A.chg_cnt, 1u)] = v;
  }
}

// every CTA: its share of each deferred in-row, min over the in-neighbours
// of dist[u] + w (as distance bits)
__global__ void __launch_bounds__(256) k_heavy_reseed_scan(HeavyRows H, const uint64_t* __restrict__ off,
                                                           const uint32_t* __restrict__ deg,
                                                           const uint32_t* __restrict__ col,
                                                           const float* __restrict__ w,
                                                           const unsigned long long* __restrict__ dist) {
  const uint32_t nh = heavy_count(H);
  for (uint32_t h = 0; h < nh; ++h) {
    const uint32_t v = H.list[h];
    const uint32_t d = deg[v];
    const uint64_t base = off[v];
    unsigned long long best = kInfBits;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < d; k += gridDim.x * blockDim.x) {
      const unsigned long long du = dist[col[base + k]];
      if (du < kInfBits) {
        const unsigned long long nb = dbits(bitsd(du) + (double)w[base + k]);
        best = nb < best ? nb : best;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_down_sync(0xffffffffu, best, o);
      best = t < best ? t : best;
    }
    if ((threadIdx.x & 31) == 0 && best < kInfBits) atomicMin(H.best + h, best);
  }
}

__global__ void k_heavy_reseed_apply(HeavyRows H, unsigned long long* __restrict__ dist,
                                     uint32_t* __restrict__ fq, uint32_t* __restrict__ fq_cnt,
                                     uint32_t* chg_mark, uint32_t* chg_list, uint32_t* chg_cnt,
                                     uint32_t chg_tag) {
  const uint32_t nh = heavy_count(H);
  for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) {
    const uint32_t v = H.list[h];
    const unsigned long long best = H.best[h];
    if (best >= kInfBits) continue;
    const unsigned long long old = atomicMin(dist + v, best);
    if (best < old) {
      fq[atomicAdd(fq_cnt, 1u)] = v;
      if (chg_mark && atomicExch(chg_mark + v, chg_tag) != chg_tag)
        chg_list[atomicAdd(chg_cnt, 1u)] = v;
    }
  }
}

// Re-seed reset vertices from their in-neighbours (pull) and queue them.
__global__ void k_sssp_reseed(const uint32_t* __restrict__ list, uint32_t cnt,
                              const uint64_t* __restrict__ off, const uint32_t* __restrict__ deg,
                              const uint32_t* __restrict__ col, const float* __restrict__ w,
                              unsigned long long* __restrict__ dist, uint32_t* __restrict__ fq,
                              uint32_t* __restrict__ fq_cnt, uint32_t* chg_mark, uint32_t* chg_list,
                              uint32_t* chg_cnt, uint32_t chg_tag, HeavyRows H,
                              uint32_t* __restrict__ seen, uint32_t seen_tag) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nwarps) {
    const uint32_t v = list[i];
    // a head listed more than once (several new edges into it) is pulled once
    const bool dup = lane == 0 && atomicExch(seen + v, seen_tag) == seen_tag;
    if (__shfl_sync(0xffffffffu, dup, 0)) continue;
    const uint32_t d = deg[v];
    const uint64_t base = off[v];
    if (d > kHeavyRow && warp_defer(H, v, kInfBits)) continue;
    unsigned long long best = kInfBits;
    for (uint32_t k = lane; k < d; k += 32) {
      const unsigned long long du = dist[col[base + k]];
      if (du < kInfBits) {
        const unsigned long long nb = dbits(bitsd(du) + (double)w[base + k]);
        best = nb < best ? nb : best;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_down_sync(0xffffffffu, best, o);
      best = t < best ? t : best;
    }
    if (lane == 0 && best < kInfBits) {
      const unsigned long long old = atomicMin(dist + v, best);
      if (best < old) {
        fq[atomicAdd(fq_cnt, 1u)] = v;
        if (chg_mark && atomicExch(chg_mark + v, chg_tag) != chg_tag)
          chg_list[atomicAdd(chg_cnt, 1u)] = v;
      }
    }
  }
}

// One batch since the last run: relax its new edges from their tails'
// current distances.
__global__ void k_sssp_relax_adds(const uint32_t* __restrict__ ps, const uint32_t* __restrict__ pd,
                                  const float* __restrict__ pw, uint32_t cnt,
                                  unsigned long long* __restrict__ dist, uint32_t* __restrict__ fq,
                                  uint32_t* __restrict__ fq_cnt, uint32_t* chg_mark, uint32_t* chg_list,
                                  uint32_t* chg_cnt, uint32_t chg_tag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const unsigned long long du = dist[ps[i]];
    if (du >= kInfBits) continue;
    const uint32_t v = pd[i];
    const unsigned long long nb = dbits(bitsd(du) + (double)pw[i]);
    const unsigned long long old = atomicMin(dist + v, nb);
    if (nb < old) {
      fq[atomicAdd(fq_cnt, 1u)] = v;
      if (chg_mark && atomicExch(chg_mark + v, chg_tag) != chg_tag)
        chg_list[atomicAdd(chg_cnt, 1u)] = v;
    }
  }
}

// One batch since the last run: a new edge lowers the parent of its head
// when the head's distance did not change and the edge is tight.
__global__ void k_parent_adds(const uint32_t* __restrict__ ps, const uint32_t* __restrict__ pd,
                              const float* __restrict__ pw, uint32_t cnt, uint32_t source,
                              const unsigned long long* __restrict__ dist,
                              const uint32_t* __restrict__ chg_mark, uint32_t tag,
                              uint32_t* __restrict__ parent) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const uint32_t u = ps[i], v = pd[i];
    const unsigned long long du = dist[u];
    if (du >= kInfBits || v == source || chg_mark[v] == tag) continue;
    if (dbits(bitsd(du) + (double)pw[i]) == dist[v]) atomicMin(parent + v, u);
  }
}

__global__ void k_sssp_init(uint32_t n, unsigned long long* dist, uint32_t* stamp,
                            uint32_t* fstamp, uint32_t* reset) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    dist[v] = kInfBits;
    stamp[v] = 0;
    fstamp[v] = 0;
    reset[v] = 0;
  }
}

__global__ void k_clear_marks(const uint32_t* list, uint32_t cnt, uint32_t* reset) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    reset[list[i]] = 0;
}

__global__ void k_dist_to_double(uint32_t n, const unsigned long long* dist, double* out) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    out[v] = bitsd(dist[v]);
}

// ------------------------------------------------------------ host side

sg_status sssp_free(sg_ctx* ctx) {
  SsspState& s = ctx->sp;
  dfree(s.dist); dfree(s.parent); dfree(s.stamp);
  dfree(s.q[0]); dfree(s.q[1]); dfree(s.q[2]); dfree(s.far2); dfree(s.reset);
  dfree(s.d_ctl); dfree(s.d_cnt);
  dfree(s.fstamp); dfree(s.seeds); dfree(s.seed_cnt); dfree(s.far);
  dfree(s.out);
  dfree(s.padd_dst);
  dfree(s.padd_src);
  dfree(s.padd_w);
  dfree(s.chg_mark); dfree(s.chg_list); dfree(s.par_mark); dfree(s.par_list); dfree(s.inc_ctl);
  dfree(s.hv_list); dfree(s.hv_best); dfree(s.hv_cnt); dfree(s.seed_mark);
  s = SsspState();
  return SG_OK;
}

static sg_status sssp_alloc(sg_ctx* ctx) {
  SsspState& s = ctx->sp;
  const uint32_t n = ctx->g.n;
  if (s.dist && s.n_alloc == n && s.far_cap >= ctx->g.m + (uint64_t)n + 1024) {
    // same graph size: keep the buffers, drop the result
    s.valid = false;
    s.has_pending = false;
    s.padd_bound = 0;
    return SG_OK;
  }
  sssp_free(ctx);
  SG_TRY(dalloc(ctx, &s.dist, n));
  SG_TRY(dalloc(ctx, &s.parent, n));
  SG_TRY(dalloc(ctx, &s.stamp, n));
  SG_TRY(dalloc(ctx, &s.fstamp, n));
  SG_TRY(dalloc(ctx, &s.reset, n));
  // queues: a vertex is queued at most once per near iteration, but the far
  // queue may hold a vertex once per improvement; bound it by edges + n.
  SG_TRY(dalloc(ctx, &s.q[0], n));
  SG_TRY(dalloc(ctx, &s.q[1], n));
  SG_TRY(dalloc(ctx, &s.q[2], n));
  const uint64_t fcap = ctx->g.m + (uint64_t)n + 1024;
  SG_TRY(dalloc(ctx, &s.far, fcap));
  SG_TRY(dalloc(ctx, &s.far2, fcap));
  s.far_cap = fcap;
  SG_TRY(dalloc(ctx, &s.seeds, n));
  SG_TRY(dalloc(ctx, &s.seed_cnt, 4));
  SG_TRY(dalloc(ctx, &s.d_ctl, S_WORDS));
  SG_TRY(dalloc(ctx, &s.d_cnt, SC_WORDS));
  SG_TRY(dalloc(ctx, &s.chg_mark, n));
  SG_TRY(dalloc(ctx, &s.chg_list, n));
  SG_TRY(dalloc(ctx, &s.par_mark, n));
  SG_TRY(dalloc(ctx, &s.par_list, n));
  SG_TRY(dalloc(ctx, &s.inc_ctl, 8));
  SG_TRY(dalloc(ctx, &s.hv_list, n));
  SG_TRY(dalloc(ctx, &s.hv_best, n));
  SG_TRY(dalloc(ctx, &s.hv_cnt, 4));
  SG_TRY(dalloc(ctx, &s.seed_mark, n));
  SG_CUDA(ctx, cudaMemsetAsync(s.seed_mark, 0, 4ull * n, ctx->stream));
  s.seed_tag = 0;
  SG_CUDA(ctx, cudaMemsetAsync(s.chg_mark, 0, 4ull * n, ctx->stream));
  SG_CUDA(ctx, cudaMemsetAsync(s.par_mark, 0, 4ull * n, ctx->stream));
  s.chg_tag = 0;
  s.n_alloc = n;
  return SG_OK;
}

SsspAmendArgs sssp_amend_args(sg_ctx* ctx) {
  SsspAmendArgs a{};
  SsspState& s = ctx->sp;
  a.active = s.valid;
  a.parent = s.parent;
  a.seeds = s.seeds;
  a.seed_count = s.seed_cnt;
  a.reset = s.reset;
  if (s.valid && !s.has_pending) {
    // first batch since the last run: empty seed list and pending adds
    cudaMemsetAsync(s.seed_cnt, 0, 4 * sizeof(uint32_t), ctx->stream);
    s.padd_bound = 0;
    s.pending_batches = 0;
  }
  if (s.valid) {
    s.has_pending = true;
    s.pending_batches++;
  }
  return a;
}

__global__ void k_collect_adds(const uint32_t* __restrict__ a_src, const uint32_t* __restrict__ a_dst,
                               const float* __restrict__ a_w, const uint32_t* __restrict__ a_kind,
                               uint64_t n_act, uint32_t* __restrict__ ps, uint32_t* __restrict__ pd,
                               float* __restrict__ pw, uint32_t* __restrict__ cnt) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_act;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (!(a_kind[i] & 2u)) continue;
    const uint32_t s = atomicAdd(cnt, 1u);
    ps[s] = a_src[i];
    pd[s] = a_dst[i];
    pw[s] = a_w[i];
  }
}

// Called by the applier after the batch's actions are known: remembers the
// added (or re-weighted) edges for the next IncEval.  The reference re-sends
// from every finite vertex after the reset (sum_sync_traversal_worker.h:
// 323-332); only these edges' heads and the reset vertices can get a
// shorter distance.  When one batch separates the IncEval from the last
// run, the recorded edges are exactly the graph's new edges and IncEval
// relaxes them (after the reset, so a tail reset by the same batch lends no
// stale distance); after several batches a later one may have deleted or
// re-weighted a recorded edge, so IncEval re-seeds the heads by a pull over
// their in-edges in the graph as it is then.
sg_status sssp_collect_adds(sg_ctx* ctx) {
  SsspState& s = ctx->sp;
  const DevBatch& B = ctx->batch;
  if (!s.valid || B.n_act == 0) return SG_OK;
  const uint64_t need = s.padd_bound + B.n_act;
  if (need > s.padd_cap) {
    // grow, keeping the pending entries
    const uint64_t ncap = std::max<uint64_t>(need * 2, 4096);
    uint32_t *nd = nullptr, *ns = nullptr;
    float* nw = nullptr;
    SG_TRY(dalloc(ctx, &nd, ncap));
    SG_TRY(dalloc(ctx, &ns, ncap));
    SG_TRY(dalloc(ctx, &nw, ncap));
    if (s.padd_bound) {
      SG_CUDA(ctx, cudaMemcpyAsync(nd, s.padd_dst, 4 * s.padd_bound, cudaMemcpyDeviceToDevice, ctx->stream));
      SG_CUDA(ctx, cudaMemcpyAsync(ns, s.padd_src, 4 * s.padd_bound, cudaMemcpyDeviceToDevice, ctx->stream));
      SG_CUDA(ctx, cudaMemcpyAsync(nw, s.padd_w, 4 * s.padd_bound, cudaMemcpyDeviceToDevice, ctx->stream));
      SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    dfree(s.padd_dst);
    dfree(s.padd_src);
    dfree(s.padd_w);
    s.padd_dst = nd;
    s.padd_src = ns;
    s.padd_w = nw;
    s.padd_cap = ncap;
  }
  k_collect_adds<<<grid_for(B.n_act, 256), 256, 0, ctx->stream>>>(
      B.a_src, B.a_dst, B.a_w, B.a_kind, B.n_act, s.padd_src, s.padd_dst, s.padd_w, s.seed_cnt + 2);
  SG_CUDA(ctx, cudaGetLastError());
  s.padd_bound = need;
  return SG_OK;
}

static double auto_delta(sg_ctx* ctx) {
  if (ctx->opt.sssp_delta > 0) return ctx->opt.sssp_delta;
  return 32.0;
}

// Launches the persistent kernel (cooperative) for the given arguments and
// reads its control words back.
static sg_status sssp_launch_args(sg_ctx* ctx, SsspArgs& A, uint32_t* h_ctl) {
  int bps = 0;
  SG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_sssp_persistent, 256, 0));
  if (bps < 1) return fail(ctx, SG_ERR_CUDA, "persistent SSSP kernel cannot be resident");
  bps = std::min(bps, 4);
  const unsigned blocks = (unsigned)(bps * ctx->num_sms);
  void* args[] = {&A};
  kprof_begin(ctx);
  SG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_sssp_persistent, dim3(blocks), dim3(256), args,
                                           0, ctx->stream));
  kprof_end(ctx, SG_K_SSSP);
  SG_CUDA(ctx, cudaMemcpyAsync(h_ctl, A.ctl, sizeof(uint32_t) * S_WORDS, cudaMemcpyDeviceToHost,
                               ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h_ctl[S_ERR] == 2u) return fail(ctx, SG_ERR_OOM, "SSSP far queue overflow");
  if (h_ctl[S_ERR]) return fail(ctx, SG_ERR_TIMEOUT, "SSSP grid barrier wait expired");
  return SG_OK;
}

// Runs the persistent kernel from the current ctl / queues; `track` lists
// every improved vertex (IncEval).
static sg_status sssp_launch(sg_ctx* ctx, bool track) {
  SsspState& s = ctx->sp;
  DevGraph& g = ctx->g;
  SsspArgs A;
  A.n = g.n;
  A.off = g.out.off; A.deg = g.out.deg; A.col = g.out.col; A.w = g.out.w;
  A.dist = s.dist; A.stamp = s.stamp; A.fstamp = s.fstamp;
  A.nq[0] = s.q[0]; A.nq[1] = s.q[1]; A.nq[2] = s.q[2];
  A.fq[0] = s.far; A.fq[1] = s.far2;
  A.ctl = s.d_ctl;
  A.cnt = s.d_cnt;
  A.delta = s.delta_width;
  A.iter_base = s.iter_base;
  A.fcap = s.far_cap;
  A.spin_limit = 40ll * 1000 * 1000;  // ~2-4 s of polling
  // deferred long rows: three slots of the long-row buffer (free while the
  // persistent kernel runs)
  A.hcap = g.n / 3;
  for (int i = 0; i < 3; ++i) A.hq[i] = A.hcap ? s.hv_list + (size_t)i * A.hcap : nullptr;
  A.chg_mark = track ? s.chg_mark : nullptr;
  A.chg_list = s.chg_list;
  A.chg_cnt = s.inc_ctl + 4;
  A.chg_tag = s.chg_tag;
  uint32_t h_ctl[S_WORDS];
  SG_TRY(sssp_launch_args(ctx, A, h_ctl));
  // stamps must keep growing across launches
  s.iter_base += h_ctl[S_ITERS] + h_ctl[S_SPLITS] + 4;
  return SG_OK;
}

__global__ void k_sssp_seed_list(const uint32_t* __restrict__ v, const double* __restrict__ d,
                                 uint32_t cnt, unsigned long long* dist, uint32_t* far) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    atomicMin(dist + v[i], dbits(d[i]));
    far[i] = v[i];
  }
}

// Delta-stepping over a caller-given padded CSR view (segments 16-byte
// aligned, readable in quads) from a list of seeds with start distances.
// Temporary queues are allocated for the call.  dist: device [G.n].
void sssp_view_scratch_free(SsspViewScratch& v) {
  dfree(v.stamp); dfree(v.fstamp); dfree(v.reset);
  dfree(v.q[0]); dfree(v.q[1]); dfree(v.q[2]);
  dfree(v.far); dfree(v.far2); dfree(v.ctl); dfree(v.cnt); dfree(v.sv); dfree(v.sd);
  v = SsspViewScratch();
}

// grows the scratch to n rows, a far capacity of fcap and nseeds seeds
static sg_status view_scratch(sg_ctx* ctx, SsspViewScratch& V, uint64_t n, uint64_t fcap,
                              uint64_t nseeds) {
  if (V.n_cap < n) {
    dfree(V.stamp); dfree(V.fstamp); dfree(V.reset);
    dfree(V.q[0]); dfree(V.q[1]); dfree(V.q[2]);
    V.n_cap = 0;
    const uint64_t c = n + n / 8;
    SG_TRY(dalloc(ctx, &V.stamp, c));
    SG_TRY(dalloc(ctx, &V.fstamp, c));
    SG_TRY(dalloc(ctx, &V.reset, c));
    for (int i = 0; i < 3; ++i) SG_TRY(dalloc(ctx, &V.q[i], c));
    V.n_cap = c;
  }
  if (V.f_cap < fcap) {
    dfree(V.far); dfree(V.far2);
    V.f_cap = 0;
    const uint64_t c = fcap + fcap / 8;
    SG_TRY(dalloc(ctx, &V.far, c));
    SG_TRY(dalloc(ctx, &V.far2, c));
    V.f_cap = c;
  }
  if (V.s_cap < std::max<uint64_t>(nseeds, 1)) {
    dfree(V.sv); dfree(V.sd);
    V.s_cap = 0;
    const uint64_t c = std::max<uint64_t>(nseeds, 1) * 2;
    SG_TRY(dalloc(ctx, &V.sv, c));
    SG_TRY(dalloc(ctx, &V.sd, c));
    V.s_cap = c;
  }
  if (!V.ctl) SG_TRY(dalloc(ctx, &V.ctl, S_WORDS));
  if (!V.cnt) SG_TRY(dalloc(ctx, &V.cnt, SC_WORDS));
  return SG_OK;
}

sg_status sssp_run_view(sg_ctx* ctx, const SsspView& G, const uint32_t* h_seeds,
                        const double* h_seed_dist, uint32_t nseeds, unsigned long long* dist,
                        unsigned long long* h_cnt, SsspViewScratch& V) {
  cudaStream_t st = ctx->stream;
  const uint32_t n = G.n;
  const uint64_t fcap = G.m + (uint64_t)n + nseeds + 1024;
  SG_TRY(view_scratch(ctx, V, n, fcap, nseeds));
  uint32_t *stamp = V.stamp, *fstamp = V.fstamp, *reset = V.reset, *q0 = V.q[0], *q1 = V.q[1],
           *q2 = V.q[2], *far = V.far, *far2 = V.far2, *ctl = V.ctl, *sv = V.sv;
  unsigned long long* cnt = V.cnt;
  double* sd = V.sd;
  k_sssp_init<<<grid_for(n, 256), 256, 0, st>>>(n, dist, stamp, fstamp, reset);
  SG_CUDA(ctx, cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * S_WORDS, st));
  SG_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * SC_WORDS, st));
  if (nseeds) {
    SG_CUDA(ctx, cudaMemcpyAsync(sv, h_seeds, 4ull * nseeds, cudaMemcpyHostToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(sd, h_seed_dist, 8ull * nseeds, cudaMemcpyHostToDevice, st));
    k_sssp_seed_list<<<grid_for(nseeds, 256), 256, 0, st>>>(sv, sd, nseeds, dist, far);
    SG_CUDA(ctx, cudaMemcpyAsync(ctl + S_F0, &nseeds, 4, cudaMemcpyHostToDevice, st));
  }
  count_launch(ctx, 2);
  SsspArgs A;
  A.n = n;
  A.off = G.off; A.deg = G.deg; A.col = G.col; A.w = G.w;
  A.dist = dist; A.stamp = stamp; A.fstamp = fstamp;
  A.nq[0] = q0; A.nq[1] = q1; A.nq[2] = q2;
  A.fq[0] = far; A.fq[1] = far2;
  A.ctl = ctl;
  A.cnt = cnt;
  A.delta = auto_delta(ctx);
  A.iter_base = 1;
  A.fcap = fcap;
  A.spin_limit = 40ll * 1000 * 1000;
  A.hq[0] = A.hq[1] = A.hq[2] = nullptr;  // one warp per row on this view
  A.hcap = 0;
  A.chg_mark = nullptr;
  A.chg_list = nullptr;
  A.chg_cnt = nullptr;
  A.chg_tag = 0;
  uint32_t h_ctl[S_WORDS];
  sg_status rs = sssp_launch_args(ctx, A, h_ctl);
  if (rs == SG_OK && h_cnt)
    SG_CUDA(ctx, cudaMemcpy(h_cnt, cnt, sizeof(unsigned long long) * SC_WORDS, cudaMemcpyDeviceToHost));
  return rs;
}

sg_status sssp_compute_parents(sg_ctx* ctx) {
  SsspState& s = ctx->sp;
  DevGraph& g = ctx->g;
  k_sssp_parents<<<grid_for((uint64_t)g.n * 32, 256), 256, 0, ctx->stream>>>(
      g.n, s.source, g.in.off, g.in.deg, g.in.col, g.in.w, s.dist, s.parent);
  SG_CUDA(ctx, cudaGetLastError());
  return SG_OK;
}

static void fill_stats(sg_ctx* ctx, const unsigned long long* cnt) {
  ctx->stats.edges_relaxed = cnt[SC_EDGES];
  ctx->stats.improvements = cnt[SC_IMPROVE];
  ctx->stats.live_edges = ctx->g.m;
}

sg_status sssp_run_peval(sg_ctx* ctx, uint32_t source) {
  DevGraph& g = ctx->g;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  if (!g.weighted) return fail(ctx, SG_ERR_INVALID, "SSSP needs a weighted graph");
  if (source >= g.n) return fail(ctx, SG_ERR_INVALID, "source >= n");
  SG_TRY(sssp_alloc(ctx));
  SsspState& s = ctx->sp;
  s.source = source;
  s.delta_width = auto_delta(ctx);
  s.iter_base = 1;
  cudaStream_t st = ctx->stream;
  SG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  k_sssp_init<<<grid_for(g.n, 256), 256, 0, st>>>(g.n, s.dist, s.stamp, s.fstamp, s.reset);
  SG_CUDA(ctx, cudaMemsetAsync(s.d_ctl, 0, sizeof(uint32_t) * S_WORDS, st));
  SG_CUDA(ctx, cudaMemsetAsync(s.d_cnt, 0, sizeof(unsigned long long) * SC_WORDS, st));
  // seed: dist[source] = 0 in the far queue; the first split opens its bucket
  const unsigned long long zero = 0ull;
  const uint32_t one = 1;
  SG_CUDA(ctx, cudaMemcpyAsync(s.dist + source, &zero, 8, cudaMemcpyHostToDevice, st));
  SG_CUDA(ctx, cudaMemcpyAsync(s.far, &source, 4, cudaMemcpyHostToDevice, st));
  SG_CUDA(ctx, cudaMemcpyAsync(s.d_ctl + S_F0, &one, 4, cudaMemcpyHostToDevice, st));
  SG_TRY(sssp_launch(ctx, false));
  SG_TRY(sssp_compute_parents(ctx));
  SG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  unsigned long long h_cnt[SC_WORDS];
  SG_CUDA(ctx, cudaMemcpyAsync(h_cnt, s.d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  fill_stats(ctx, h_cnt);
  ctx->stats.elapsed_ms = ms;
  ctx->stats.rounds = 0;
  ctx->stats.converged = 1;
  ctx->stats.reset_vertices = 0;
  s.valid = true;
  s.has_pending = false;
  return SG_OK;
}

// A PEval whose distances are computed elsewhere (the summarized graph):
// buffers and tags as sssp_run_peval sets them, distances left to the caller.
sg_status sssp_prepare_external(sg_ctx* ctx, uint32_t source) {
  DevGraph& g = ctx->g;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  if (!g.weighted) return fail(ctx, SG_ERR_INVALID, "SSSP needs a weighted graph");
  if (source >= g.n) return fail(ctx, SG_ERR_INVALID, "source >= n");
  SG_TRY(sssp_alloc(ctx));
  SsspState& s = ctx->sp;
  s.source = source;
  s.delta_width = auto_delta(ctx);
  s.iter_base = 1;
  k_sssp_init<<<grid_for(g.n, 256), 256, 0, ctx->stream>>>(g.n, s.dist, s.stamp, s.fstamp, s.reset);
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  return SG_OK;
}

sg_status sssp_finish_external(sg_ctx* ctx, const unsigned long long* h_cnt, float ms) {
  SsspState& s = ctx->sp;
  SG_TRY(sssp_compute_parents(ctx));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h_cnt) fill_stats(ctx, h_cnt);
  ctx->stats.elapsed_ms = ms;
  ctx->stats.rounds = 0;
  ctx->stats.converged = 1;
  ctx->stats.reset_vertices = 0;
  s.valid = true;
  s.has_pending = false;
  return SG_OK;
}

__global__ void k_inc_start(const uint32_t* seed_cnt, uint32_t* inc_ctl) {
  inc_ctl[0] = 0;
  inc_ctl[1] = 0;
  inc_ctl[2] = 0;
  inc_ctl[3] = seed_cnt[0];
  inc_ctl[4] = 0;
  inc_ctl[5] = 0;
  inc_ctl[6] = 0;
  inc_ctl[7] = 0;
}

// Steps 1 and 2 of the incremental stage (deltaCompute and the re-seed of
// sum_sync_traversal_worker.h:113-352): the reset BFS over the shortest-path
// tree, the pulls that give every reset vertex its best distance from the
// vertices that kept theirs, and the relaxation of the batch's new edges.
// The far queue holds the improved vertices.  Shared by the plain IncEval and
// the IncEval over the summary.
static sg_status inc_reset_seed(sg_ctx* ctx, SsspIncInfo* info) {
  DevGraph& g = ctx->g;
  SsspState& s = ctx->sp;
  cudaStream_t st = ctx->stream;
  if (!s.has_pending) SG_CUDA(ctx, cudaMemsetAsync(s.seed_cnt, 0, 4 * sizeof(uint32_t), st));
  if (++s.chg_tag == 0) {  // tags wrapped: clear the marks
    SG_CUDA(ctx, cudaMemsetAsync(s.chg_mark, 0, 4ull * g.n, st));
    SG_CUDA(ctx, cudaMemsetAsync(s.par_mark, 0, 4ull * g.n, st));
    s.chg_tag = 1;
  }
  // 1. reset BFS over the tree from the applier's seeds, in one launch; the
  //    list grows in place behind the seeds
  k_inc_start<<<1, 1, 0, st>>>(s.seed_cnt, s.inc_ctl);
  {
    ResetArgs R;
    R.seed_cnt = s.seed_cnt;
    R.list = s.seeds;
    R.cap = g.n;
    R.off = g.out.off; R.deg = g.out.deg; R.col = g.out.col;
    R.parent = s.parent;
    R.reset = s.reset;
    R.dist = s.dist;
    R.ctl = s.inc_ctl;
    R.chg_mark = s.chg_mark;
    R.chg_list = s.chg_list;
    R.chg_cnt = s.inc_ctl + 4;
    R.chg_tag = s.chg_tag;
    R.spin_limit = 40ll * 1000 * 1000;
    R.hv = s.hv_list;
    R.hv_half = g.n / 2;
    int bps = 0;
    SG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_sssp_reset_all, 256, 0));
    if (bps < 1) return fail(ctx, SG_ERR_CUDA, "reset kernel cannot be resident");
    bps = std::min(bps, 2);
    void* args[] = {&R};
    SG_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_sssp_reset_all, dim3(bps * ctx->num_sms),
                                             dim3(256), args, 0, st));
    count_launch(ctx, 2);
  }
  uint32_t h_inc[8], h_seed[4];
  SG_CUDA(ctx, cudaMemcpyAsync(h_inc, s.inc_ctl, sizeof(h_inc), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(h_seed, s.seed_cnt, sizeof(h_seed), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  if (h_inc[2] == 1u) return fail(ctx, SG_ERR_TIMEOUT, "reset BFS grid barrier wait expired");
  if (h_inc[2] == 2u) return fail(ctx, SG_ERR_INVALID, "reset list overflow");
  const uint32_t total = h_inc[3];
  const uint32_t nadd = s.has_pending ? h_seed[2] : 0u;
  // 2. far queue <- re-seeded reset vertices and heads of added edges
  const uint64_t need_far = (uint64_t)total + nadd + g.n + 1024;
  if (need_far > s.far_cap) {
    dfree(s.far);
    dfree(s.far2);
    const uint64_t ncap = std::max<uint64_t>(need_far, g.m + g.n + 1024);
    SG_TRY(dalloc(ctx, &s.far, ncap));
    SG_TRY(dalloc(ctx, &s.far2, ncap));
    s.far_cap = ncap;
  }
  SG_CUDA(ctx, cudaMemsetAsync(s.d_ctl, 0, sizeof(uint32_t) * S_WORDS, st));
  SG_CUDA(ctx, cudaMemsetAsync(s.d_cnt, 0, sizeof(unsigned long long) * SC_WORDS, st));
  const HeavyRows H{s.hv_list, s.hv_best, s.hv_cnt, g.n};
  if (++s.seed_tag == 0) {  // tags wrapped: clear the marks
    SG_CUDA(ctx, cudaMemsetAsync(s.seed_mark, 0, 4ull * g.n, st));
    s.seed_tag = 1;
  }
  const unsigned heavy_grid = ctx->num_sms * 4;
  // re-seed a list: warps pull the short in-rows, every CTA a share of the
  // long ones, then the long rows' results are applied
  auto reseed = [&](const uint32_t* list, uint32_t cnt) -> sg_status {
    SG_CUDA(ctx, cudaMemsetAsync(s.hv_cnt, 0, 4, st));
    k_sssp_reseed<<<grid_for((uint64_t)cnt * 32, 256), 256, 0, st>>>(
        list, cnt, g.in.off, g.in.deg, g.in.col, g.in.w, s.dist, s.far, s.d_ctl + S_F0,
        s.chg_mark, s.chg_list, s.inc_ctl + 4, s.chg_tag, H, s.seed_mark, s.seed_tag);
    k_heavy_reseed_scan<<<heavy_grid, 256, 0, st>>>(H, g.in.off, g.in.deg, g.in.col, g.in.w, s.dist);
    k_heavy_reseed_apply<<<4, 256, 0, st>>>(H, s.dist, s.far, s.d_ctl + S_F0, s.chg_mark,
                                            s.chg_list, s.inc_ctl + 4, s.chg_tag);
    count_launch(ctx, 3);
    return SG_OK;
  };
  // one batch: relax its new edges; several: pull their heads' in-rows
  const bool one_batch = s.pending_batches == 1;
  if (total > 0) SG_TRY(reseed(s.seeds, total));
  if (nadd > 0 && one_batch) {
    k_sssp_relax_adds<<<grid_for(nadd, 256), 256, 0, st>>>(
        s.padd_src, s.padd_dst, s.padd_w, nadd, s.dist, s.far, s.d_ctl + S_F0, s.chg_mark,
        s.chg_list, s.inc_ctl + 4, s.chg_tag);
    count_launch(ctx);
  } else if (nadd > 0) {
    SG_TRY(reseed(s.padd_dst, nadd));
  }
  SG_CUDA(ctx, cudaGetLastError());
  info->total = total;
  info->nadd = nadd;
  info->one_batch = one_batch;
  return SG_OK;
}

sg_status sssp_inc_prepare(sg_ctx* ctx, SsspIncInfo* info) {
  if (!ctx->sp.valid) return fail(ctx, SG_ERR_STATE, "SSSP IncEval before PEval");
  return inc_reset_seed(ctx, info);
}

sg_status sssp_run_inceval(sg_ctx* ctx) {
  DevGraph& g = ctx->g;
  SsspState& s = ctx->sp;
  if (!s.valid) return fail(ctx, SG_ERR_STATE, "SSSP IncEval before PEval");
  cudaStream_t st = ctx->stream;
  SG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  SsspIncInfo info;
  SG_TRY(inc_reset_seed(ctx, &info));
  const uint32_t total = info.total, nadd = info.nadd;
  const bool one_batch = info.one_batch;
  const HeavyRows H{s.hv_list, s.hv_best, s.hv_cnt, g.n};
  const unsigned heavy_grid = ctx->num_sms * 4;
  // 3. delta-stepping from the seeds, listing every improved vertex
  SG_TRY(sssp_launch(ctx, true));
  if (total > 0) k_clear_marks<<<grid_for(total, 256), 256, 0, st>>>(s.seeds, total, s.reset);
  // 4. parents of the vertices whose smallest tight in-neighbour can change
  uint32_t nchg = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&nchg, s.inc_ctl + 4, 4, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  if (nchg + nadd > 0) {
    // (a) + (b) in full, long in-rows by every CTA; then (c) by a push
    SG_CUDA(ctx, cudaMemsetAsync(s.inc_ctl + 5, 0, 4, st));
    SG_CUDA(ctx, cudaMemsetAsync(s.hv_cnt, 0, 4, st));
    // heads of new edges in full only after several batches (with one, the
    // new edges themselves are checked below)
    const uint32_t nheads = one_batch ? 0u : nadd;
    k_parent_list<<<grid_for(nchg + nheads, 256), 256, 0, st>>>(s.chg_list, nchg, s.padd_dst,
                                                                nheads, s.par_mark, s.chg_tag,
                                                                s.par_list, s.inc_ctl + 5);
    k_sssp_parents_list<<<ctx->num_sms * 8, 256, 0, st>>>(s.par_list, s.inc_ctl + 5, s.source,
                                                          g.in.off, g.in.deg, g.in.col, g.in.w,
                                                          s.dist, s.parent, H);
    k_heavy_parent_scan<<<heavy_grid, 256, 0, st>>>(H, s.source, g.in.off, g.in.deg, g.in.col,
                                                    g.in.w, s.dist);
    k_heavy_parent_apply<<<4, 256, 0, st>>>(H, s.parent);
    count_launch(ctx, 4);
    if (nchg > 0) {
      SG_CUDA(ctx, cudaMemsetAsync(s.hv_cnt, 0, 4, st));
      k_parent_push<<<grid_for((uint64_t)nchg * 32, 256), 256, 0, st>>>(
          s.chg_list, nchg, s.source, g.out.off, g.out.deg, g.out.col, g.out.w, s.dist, s.chg_mark,
          s.chg_tag, s.parent, H);
      k_heavy_parent_push<<<heavy_grid, 256, 0, st>>>(H, s.source, g.out.off, g.out.deg, g.out.col,
                                                      g.out.w, s.dist, s.chg_mark, s.chg_tag,
                                                      s.parent);
      count_launch(ctx, 2);
    }
    if (one_batch && nadd > 0) {
      k_parent_adds<<<grid_for(nadd, 256), 256, 0, st>>>(s.padd_src, s.padd_dst, s.padd_w, nadd,
                                                         s.source, s.dist, s.chg_mark, s.chg_tag,
                                                         s.parent);
      count_launch(ctx);
    }
  }
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  unsigned long long h_cnt[SC_WORDS];
  SG_CUDA(ctx, cudaMemcpyAsync(h_cnt, s.d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  fill_stats(ctx, h_cnt);
  ctx->stats.elapsed_ms = ms;
  ctx->stats.converged = 1;
  ctx->stats.reset_vertices = total;
  s.has_pending = false;
  return SG_OK;
}

// The end of an IncEval whose distances were finished elsewhere (over the
// summary): the reset marks cleared, every parent recomputed over the
// in-rows, the counters of the traversal.
sg_status sssp_inc_finish_external(sg_ctx* ctx, const SsspIncInfo& info,
                                   const unsigned long long* h_cnt, float ms) {
  SsspState& s = ctx->sp;
  cudaStream_t st = ctx->stream;
  if (info.total > 0) {
    k_clear_marks<<<grid_for(info.total, 256), 256, 0, st>>>(s.seeds, info.total, s.reset);
    count_launch(ctx);
  }
  SG_TRY(sssp_compute_parents(ctx));
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  if (h_cnt) fill_stats(ctx, h_cnt);
  ctx->stats.elapsed_ms = ms;
  ctx->stats.converged = 1;
  ctx->stats.reset_vertices = info.total;
  s.has_pending = false;
  return SG_OK;
}

// Delta-stepping over a view from a warm state: `dist` (device [G.n]) holds
// valid upper bounds, final for every vertex whose distance cannot change,
// and the device list `d_seeds` holds the vertices whose out-rows must be
// relaxed again.  Temporary queues are allocated for the call.
sg_status sssp_run_view_warm(sg_ctx* ctx, const SsspView& G, const uint32_t* d_seeds,
                             uint32_t nseeds, unsigned long long* dist, unsigned long long* h_cnt,
                             SsspViewScratch& V) {
  cudaStream_t st = ctx->stream;
  const uint32_t n = G.n;
  const uint64_t fcap = G.m + (uint64_t)n + nseeds + 1024;
  SG_TRY(view_scratch(ctx, V, n, fcap, 0));
  uint32_t *stamp = V.stamp, *fstamp = V.fstamp, *q0 = V.q[0], *q1 = V.q[1], *q2 = V.q[2],
           *far = V.far, *far2 = V.far2, *ctl = V.ctl;
  unsigned long long* cnt = V.cnt;
  SG_CUDA(ctx, cudaMemsetAsync(stamp, 0, 4ull * n, st));
  SG_CUDA(ctx, cudaMemsetAsync(fstamp, 0, 4ull * n, st));
  SG_CUDA(ctx, cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * S_WORDS, st));
  SG_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * SC_WORDS, st));
  if (nseeds) {
    SG_CUDA(ctx, cudaMemcpyAsync(far, d_seeds, 4ull * nseeds, cudaMemcpyDeviceToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(ctl + S_F0, &nseeds, 4, cudaMemcpyHostToDevice, st));
  }
  SsspArgs A;
  A.n = n;
  A.off = G.off; A.deg = G.deg; A.col = G.col; A.w = G.w;
  A.dist = dist; A.stamp = stamp; A.fstamp = fstamp;
  A.nq[0] = q0; A.nq[1] = q1; A.nq[2] = q2;
  A.fq[0] = far; A.fq[1] = far2;
  A.ctl = ctl;
  A.cnt = cnt;
  A.delta = auto_delta(ctx);
  A.iter_base = 1;
  A.fcap = fcap;
  A.spin_limit = 40ll * 1000 * 1000;
  A.hq[0] = A.hq[1] = A.hq[2] = nullptr;  // one warp per row on this view
  A.hcap = 0;
  A.chg_mark = nullptr;
  A.chg_list = nullptr;
  A.chg_cnt = nullptr;
  A.chg_tag = 0;
  uint32_t h_ctl[S_WORDS];
  sg_status rs = sssp_launch_args(ctx, A, h_ctl);
  if (rs == SG_OK && h_cnt)
    SG_CUDA(ctx, cudaMemcpy(h_cnt, cnt, sizeof(unsigned long long) * SC_WORDS, cudaMemcpyDeviceToHost));
  return rs;
}

sg_status sssp_download(sg_ctx* ctx, double* out) {
  SsspState& s = ctx->sp;
  if (!s.valid) return fail(ctx, SG_ERR_STATE, "no SSSP result");
  const uint32_t n = ctx->g.n;
  if (!s.out) SG_TRY(dalloc(ctx, &s.out, n));
  k_dist_to_double<<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, s.dist, s.out);
  SG_CUDA(ctx, cudaMemcpyAsync(out, s.out, 8ull * n, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

sg_status sssp_barrier_probe(sg_ctx* ctx, int skip) {
  uint32_t* ctl = nullptr;
  SG_TRY(dalloc(ctx, &ctl, S_WORDS));
  SG_CUDA(ctx, cudaMemsetAsync(ctl, 0, 4 * S_WORDS, ctx->stream));
  SsspArgs A{};
  A.ctl = ctl;
  A.spin_limit = 100000;  // about 10 ms of polling
  k_barrier_probe<<<4, 128, 0, ctx->stream>>>(A, skip ? 1 : 0);
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  uint32_t err = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&err, ctl + S_ERR, 4, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(ctl);
  if (err) return fail(ctx, SG_ERR_TIMEOUT, "grid barrier wait expired (probe)");
  return SG_OK;
}

}  // namespace sg
