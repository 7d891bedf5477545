// PageRank with message_type = pull (SumSyncIterWorkerPull,
// grape/worker/sum_sync_iter_worker_pull.h; pull functions
// pagerank_ingress.h:210-310): synchronous rounds in which every vertex
// gathers from its in-neighbours the values they published the round
// before, so no round writes another vertex's state and no atomics are
// needed.
//
//   init             last_values = x; with a summary, per vertex class (out
//                    node: x += delta; exit / inner: delta parked for the
//                    correction; entry: delta handed to its supernode)
//                    (:510-535, :1343-1360)
//   summarized round out nodes gather along all in-edges, entries along
//                    in-edges from other clusters into their supernode's
//                    index value, exits gather the entries' index values
//                    through the shortcut weights (:757-980)
//   correction       parked deltas return, inner vertices take their value
//                    and delta shares of the accumulated entry mass
//                    (:1045-1131)
//   plain round      every vertex gathers along all in-edges (:600-630):
//                    the same round as the library's dense pull rounds
//                    (pagerank.cu: gather the published d*delta/outdeg, add
//                    the sum to x, stop when the gathered sum |delta| is
//                    below termcheck_threshold), which therefore run this
//                    stage, and all of compress = 0
//   stop test        summarized stage: sum |last_values - x| <
//                    termcheck_threshold, or the step counter passes 200
//                    (:1044, termCheck :1430-1462), where the mass that
//                    reached the entries this round counts too (below); the
//                    plain stage stops as the dense pull rounds do (its sum
//                    |last_values - x| is the gathered sum |delta|), within
//                    max_rounds
//
// The summarized stage is a two-round pipeline (entries gather from exits,
// exits gather from the entries' index values of the round before), and an
// entry's arrivals change no value until the correction.  The reference's
// test on values alone therefore passes in the round after the exits last
// moved while the entries hold mass in flight; the correction never hands
// the exits their share of it, and that mass is lost (on a graph of 64
// planted communities the reference stops after 2 summarized rounds and
// ends 1.5e-3 in L1 from the fixed point).  Counting the entries' arrivals
// keeps the stage running until they are below the threshold too.
//
// The summarized rounds visit the vertices of classes 0-3 only (inner
// members neither gather nor publish until the correction), one lane per
// vertex, except rows longer than a warp (a hub's in-edges), which take a
// warp each (summarized rounds and correction per IncEval at 5.2 M vertices
// of planted communities: 4.0 ms with 8 lanes per vertex, 2.6 ms with 4,
// 1.9 ms with 2, 1.35 ms with 1); the published values of a round live in two buffers
// used by round parity (last_deltas_ / last_index_values_).  The
// residual is summed in FP64 per block and by the last block to finish, which
// also takes the stop decision; kernels of a chunk launched after the
// decision return at once, so the host reads the control words once per
// chunk.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.h"
#include "dev.cuh"

namespace sg {

namespace {

constexpr int kPT = 256;         // threads per block
constexpr int kStepCap = 200;    // `step > 200` (sum_sync_iter_worker_pull.h:1044)
constexpr int kChunk = 8;        // rounds launched per host check

// control words: [0] stop, [1] blocks finished, [2] rounds of the stage,
// [3] residual test passed
enum { P_STOP = 0, P_DONE_BLOCKS = 1, P_ROUNDS = 2, P_PASSED = 3, P_WORDS = 4 };

struct PullState {
  uint32_t n_alloc = 0;
  float* ld = nullptr;     // published d*delta/outdeg, 2n (round parity)
  float* li = nullptr;     // published supernode index values, 2n
  float* lastx = nullptr;  // last_values
  float* spd = nullptr;    // spnode_datas
  float* bsave = nullptr;  // bound_deltas
  double* part = nullptr;  // per-block residual sums
  double* res = nullptr;   // last residual
  uint32_t* ctl = nullptr;
  uint32_t nblocks = 0;
};

PullState* pstate(sg_ctx* ctx) { return (PullState*)ctx->pull_state; }

void pfree_arrays(PullState& P) {
  dfree(P.ld); dfree(P.li); dfree(P.lastx); dfree(P.spd); dfree(P.bsave);
  dfree(P.part); dfree(P.res); dfree(P.ctl);
}

struct PullArgs {
  uint32_t n;
  float d;
  double tau;
  const uint64_t* in_off;  // graph in-CSR segments
  const uint32_t* in_deg;
  const uint32_t* in_col;
  const uint32_t* outdeg;
  PullView V;              // summary in-indexes (cls null: no summary)
  float* x;
  float* delta;
  float* ld;
  float* li;
  float* lastx;
  float* spd;
  float* bsave;
  double* part;
  double* res;
  uint32_t* ctl;
};

__device__ __forceinline__ float publish(float dl, uint32_t od, float d) {
  return od ? dl * d / (float)od : 0.f;
}

// Block sum of `r`, then the last block to finish sums the block partials in
// a fixed order and decides whether the stage stops.
__device__ void residual_and_decide(const PullArgs& A, double r) {
  __shared__ double s_w[kPT / 32];
  __shared__ bool s_last;
#pragma unroll
  for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < kPT / 32; ++i) t += s_w[i];
    A.part[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(&A.ctl[P_DONE_BLOCKS], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double t = 0;
  for (uint32_t i = threadIdx.x; i < gridDim.x; i += kPT) t += ((volatile double*)A.part)[i];
#pragma unroll
  for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0;
    for (int i = 0; i < kPT / 32; ++i) tot += s_w[i];
    const uint32_t step = A.ctl[P_ROUNDS] + 1;
    A.ctl[P_ROUNDS] = step;
    *A.res = tot;
    const bool passed = tot < A.tau;
    A.ctl[P_PASSED] = passed ? 1u : 0u;
    if (passed || step > (uint32_t)kStepCap) A.ctl[P_STOP] = 1u;
    A.ctl[P_DONE_BLOCKS] = 0u;
  }
}

// init: last_values = x, then the class rules; both parities of the
// published buffers start defined (inner members never write theirs).
__global__ void __launch_bounds__(kPT) k_pull_init(PullArgs A) {
  for (uint32_t v = blockIdx.x * kPT + threadIdx.x; v < A.n; v += gridDim.x * kPT) {
    float x = A.x[v], dl = A.delta[v];
    A.lastx[v] = x;
    const uint32_t t = A.V.cls[v];
    float nd = 0.f, nl = 0.f;
    if (t == 0) {
      x += dl;
      nd = dl;
    } else if (t == 1 || t == 4) {
      A.bsave[v] = dl;
      dl = 0.f;
    } else {  // 2, 3: the delta becomes the supernode's index value
      nl = dl;
      dl = 0.f;
    }
    A.x[v] = x;
    A.delta[v] = dl;
    A.ld[v] = publish(nd, A.outdeg[v], A.d);
    A.ld[A.n + v] = 0.f;
    A.li[v] = nl;
    A.li[A.n + v] = 0.f;
    A.spd[v] = nl;
  }
}

// One summarized round over the vertices of classes 0-3: rows longer than
// a warp (listed first) take a warp each, the others a lane each.
struct RowSums {
  float a, b;
};

__device__ __forceinline__ void round_finish(const PullArgs& A, uint32_t v, uint32_t t, float a,
                                             float b, float* ldo, float* lio, double& r) {
  float x = A.x[v];
  float nd = 0.f, nl = 0.f;
  if (t == 0) {
    x += a;
    A.delta[v] = a;
    nd = a;
  } else if (t == 1) {
    x += b;
    A.delta[v] = b;
    nd = b;
  } else {  // 2, 3
    A.spd[v] += a;
    nl = a;
    r += fabs((double)a);
    if (t == 3) {
      x += b;
      A.delta[v] = b;
      nd = b;
    }
  }
  ldo[v] = publish(nd, A.outdeg[v], A.d);
  lio[v] = nl;
  A.x[v] = x;
  r += fabs((double)A.lastx[v] - (double)x);
  A.lastx[v] = x;
}

// Sums of vertex v's rows over entries lane0, lane0 + step, ...
__device__ __forceinline__ RowSums row_sums(const PullArgs& A, uint32_t v, uint32_t t,
                                            const float* ldi, const float* lii, uint32_t lane0,
                                            uint32_t step) {
  float a = 0.f, b = 0.f;
  if (t == 0) {
    const uint64_t o = A.in_off[v];
    const uint32_t dg = A.in_deg[v];
    for (uint32_t e = lane0; e < dg; e += step) a += ldi[A.in_col[o + e]];
  } else if (t == 2 || t == 3) {
    for (uint64_t e = A.V.ie_off[v] + lane0; e < A.V.ie_off[v + 1]; e += step)
      a += ldi[A.V.ie_nbr[e]];
  }
  if (t == 1 || t == 3) {
    for (uint64_t e = A.V.bd_off[v] + lane0; e < A.V.bd_off[v + 1]; e += step)
      b += lii[A.V.bd_src[e]] * A.V.bd_w[e];
  }
  return {a, b};
}

__global__ void __launch_bounds__(kPT) k_pull_round(PullArgs A, int parity) {
  if (((volatile uint32_t*)A.ctl)[P_STOP]) return;
  const float* __restrict__ ldi = A.ld + (size_t)parity * A.n;
  float* __restrict__ ldo = A.ld + (size_t)(parity ^ 1) * A.n;
  const float* __restrict__ lii = A.li + (size_t)parity * A.n;
  float* __restrict__ lio = A.li + (size_t)(parity ^ 1) * A.n;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gtid = (uint64_t)blockIdx.x * kPT + threadIdx.x;
  const uint64_t warp = gtid >> 5;
  const uint64_t nwarps = (uint64_t)gridDim.x * (kPT / 32);
  const uint32_t cnt = A.V.n_act, nlong = A.V.n_long;
  double r = 0;
  // long rows: one warp per vertex (warp-uniform trip count)
  for (uint64_t i = warp; i < nlong; i += nwarps) {
    const uint32_t v = A.V.act[i];
    const uint32_t t = A.V.cls[v];
    RowSums s = row_sums(A, v, t, ldi, lii, lane, 32);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      s.a += __shfl_xor_sync(0xffffffffu, s.a, o);
      s.b += __shfl_xor_sync(0xffffffffu, s.b, o);
    }
    if (lane == 0) round_finish(A, v, t, s.a, s.b, ldo, lio, r);
  }
  // the other rows: one lane per vertex
  for (uint64_t i = nlong + gtid; i < cnt; i += nwarps * 32) {
    const uint32_t v = A.V.act[i];
    const uint32_t t = A.V.cls[v];
    const RowSums s = row_sums(A, v, t, ldi, lii, 0, 1);
    round_finish(A, v, t, s.a, s.b, ldo, lio, r);
  }
  residual_and_decide(A, r);
}

// Correction after the summarized rounds (:1045-1131), written in the
// library's convention (x without the pending delta): exits and inner
// members take back their parked delta, out nodes and exits with a delta
// from the last round keep it pending; then every entry's accumulated mass
// spreads through its supernode's inner_value (into x) and inner_delta
// (into delta) lists.  The reference gathers the same products per target.
__global__ void __launch_bounds__(kPT) k_pull_settle(PullArgs A) {
  for (uint32_t v = blockIdx.x * kPT + threadIdx.x; v < A.n; v += gridDim.x * kPT) {
    const uint32_t t = A.V.cls[v];
    if (t == 1 || t == 4) {
      A.delta[v] = A.bsave[v];
    } else if (t == 0 || t == 3) {
      A.x[v] -= A.delta[v];
    }
  }
}

__global__ void __launch_bounds__(kPT) k_pull_spread(PullArgs A) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t i = (blockIdx.x * kPT + threadIdx.x) >> 5; i < A.V.n_ent;
       i += (gridDim.x * kPT) >> 5) {
    const uint32_t u = A.V.ent[i];
    const float m = A.spd[u];
    if (!A.V.L.row_sp[u] || m == 0.f) continue;
    const uint64_t b = A.V.L.slot[u];
    for (uint64_t e = b + lane; e < b + A.V.L.iv_cnt[u]; e += 32)
      atomicAdd(&A.x[A.V.L.iv_nbr[e]], m * A.V.L.iv_w[e]);
    for (uint64_t e = b + lane; e < b + A.V.L.id_cnt[u]; e += 32)
      atomicAdd(&A.delta[A.V.L.id_nbr[e]], m * A.V.L.id_w[e]);
  }
}

__global__ void k_pull_start(uint32_t n, float* x, float* delta, float init_c) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    x[v] = 0.f;
    delta[v] = init_c;
  }
}

// The worker adds a gathered delta to x on arrival; the library's state
// keeps x without the pending delta (the convention of the dense pull
// rounds, AmendValue and IncEval), to which the correction converts.

sg_status preserve(sg_ctx* ctx, uint32_t n) {
  if (!ctx->pull_state) ctx->pull_state = new PullState();
  PullState& P = *pstate(ctx);
  if (P.n_alloc == n && P.ld) return SG_OK;
  pfree_arrays(P);
  P = PullState();
  P.nblocks = (uint32_t)ctx->num_sms * 8;
  SG_TRY(dalloc(ctx, &P.ld, 2ull * n));
  SG_TRY(dalloc(ctx, &P.li, 2ull * n));
  SG_TRY(dalloc(ctx, &P.lastx, n));
  SG_TRY(dalloc(ctx, &P.spd, n));
  SG_TRY(dalloc(ctx, &P.bsave, n));
  SG_TRY(dalloc(ctx, &P.part, P.nblocks));
  SG_TRY(dalloc(ctx, &P.res, 1));
  SG_TRY(dalloc(ctx, &P.ctl, P_WORDS));
  P.n_alloc = n;
  return SG_OK;
}

// Summarized rounds until the stop word is set; returns the rounds run.
sg_status summarized_stage(sg_ctx* ctx, const PullArgs& A, uint32_t* rounds) {
  cudaStream_t st = ctx->stream;
  const PullState& P = *pstate(ctx);
  SG_CUDA(ctx, cudaMemsetAsync(A.ctl, 0, sizeof(uint32_t) * P_WORDS, st));
  uint32_t h[P_WORDS] = {0, 0, 0, 0};
  int launched = 0;
  const int cap = kStepCap + 2;
  // a lane per short row and a warp per long row (long rows are listed first;
  // on a hub-dominated summary the long rows get their own warps even when
  // there are fewer than a block's worth of them)
  const unsigned blocks = std::max(
      1u, std::min(P.nblocks, (A.V.n_act + kPT - 1) / kPT + (A.V.n_long + kPT / 32 - 1) / (kPT / 32)));
  while (launched < cap) {
    kprof_begin(ctx);
    int c = 0;
    for (; c < kChunk && launched < cap; ++c, ++launched)
      k_pull_round<<<blocks, kPT, 0, st>>>(A, launched & 1);
    kprof_end(ctx, SG_K_SUMMARY);
    count_launch(ctx, c);
    SG_CUDA(ctx, cudaGetLastError());
    SG_CUDA(ctx, cudaMemcpyAsync(h, A.ctl, sizeof(h), cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
    if (h[P_STOP]) break;
  }
  *rounds = h[P_ROUNDS];
  return SG_OK;
}

}  // namespace

sg_status pull_free(sg_ctx* ctx) {
  PullState* P = pstate(ctx);
  if (P) {
    pfree_arrays(*P);
    delete P;
  }
  ctx->pull_state = nullptr;
  return SG_OK;
}

// PEval (inc = false: x = 0, delta = (1-d)/N) or IncEval (the amended state)
// of the pull worker.  compress = 1: the summarized stage, the correction,
// then the plain stage (Query's batch / inc stages,
// sum_sync_iter_worker_pull.h:243-1400); compress = 0: the plain stage.
sg_status pr_pull_worker(sg_ctx* ctx, bool inc) {
  DevGraph& g = ctx->g;
  PrState& s = ctx->pr;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  if (!ctx->opt.compress || summary_no_supernodes(ctx)) return pr_run(ctx, inc);
  PullView V;
  SG_TRY(summary_pull_view(ctx, &V));
  if (inc && !s.valid) return fail(ctx, SG_ERR_STATE, "PageRank IncEval before PEval");
  if (!s.x) SG_TRY(pr_alloc(ctx));
  const uint32_t n = g.n;
  SG_TRY(preserve(ctx, n));
  PullState& P = *pstate(ctx);
  cudaStream_t st = ctx->stream;
  PullArgs A;
  A.n = n;
  A.d = (float)ctx->opt.damping;
  A.tau = ctx->opt.termcheck_threshold;
  A.in_off = g.in.off;
  A.in_deg = g.in.deg;
  A.in_col = g.in.col;
  A.outdeg = g.out.deg;
  A.V = V;
  A.x = s.x;
  A.delta = s.delta;
  A.ld = P.ld;
  A.li = P.li;
  A.lastx = P.lastx;
  A.spd = P.spd;
  A.bsave = P.bsave;
  A.part = P.part;
  A.res = P.res;
  A.ctl = P.ctl;
  SG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  const unsigned vb = grid_for(n, kPT);
  if (!inc) {
    k_pull_start<<<vb, kPT, 0, st>>>(n, s.x, s.delta,
                                     (float)((1.0 - ctx->opt.damping) / (double)n));
    count_launch(ctx);
  }
  k_pull_init<<<vb, kPT, 0, st>>>(A);
  count_launch(ctx);
  uint32_t rc = 0;
  SG_TRY(summarized_stage(ctx, A, &rc));
  kprof_begin(ctx);
  k_pull_settle<<<vb, kPT, 0, st>>>(A);
  if (V.n_ent)
    k_pull_spread<<<grid_for((uint64_t)V.n_ent * 32, kPT), kPT, 0, st>>>(A);
  kprof_end(ctx, SG_K_SUMMARY);
  count_launch(ctx, 1 + (V.n_ent > 0));
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  // the plain stage: the library's dense pull rounds from this state
  s.valid = true;
  const sg_status stt = pr_run(ctx, true);
  sg_stats& S = ctx->stats;
  S.rounds += (int32_t)rc;
  S.shortcut_edges = (uint64_t)rc * V.round_shortcuts;
  S.edges_relaxed += (uint64_t)rc * V.round_edges + V.corr_entries;
  S.edges_pull = S.edges_relaxed;
  S.vertex_visits += (uint64_t)rc * V.n_act;
  S.elapsed_ms += ms;
  return stt;
}

}  // namespace sg
