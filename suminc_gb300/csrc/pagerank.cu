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
//   k_pr_pull     dense pull over the in-CSR, edge-balanced in tiles of
//                 PT_TILE 4-edge quads (128-bit neighbour loads, gathers of
//                 pv, shared-memory sums).  A vertex whose quads all lie in
//                 the tile is updated in the tile's epilogue (incoming sum,
//                 residual, activation, next push value); a vertex spanning
//                 tiles gets its partial sums by atomicAdd
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
  uint32_t* misc;
  double* res;
  unsigned long long* cnt;
};

// activation of one vertex with its new delta; returns 1 when active
__device__ __forceinline__ uint32_t activate(const PrArgs& A, uint32_t v, float dl, float* pv_next,
                                             double& res) {
  res += fabs((double)dl);
  if (fabsf(dl) > A.thr_v) {
    A.x[v] += dl;
    A.delta[v] = 0.f;
    if (A.scale_deg) {
      const uint32_t od = A.scale_deg[v];
      pv_next[v] = od > 0 ? A.damping * dl / (float)od : 0.f;
    } else {
      pv_next[v] = A.damping * dl;
    }
    return 1;
  }
  A.delta[v] = dl;
  pv_next[v] = 0.f;
  return 0;
}

__global__ void __launch_bounds__(VT) k_pr_vertex(PrArgs A) {
  __shared__ double s_red[VT / 32];
  __shared__ double s_red2[VT / 32];
  double res = 0.0, res0 = 0.0;
  unsigned long long visits = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < A.n; v += gridDim.x * blockDim.x) {
    double r = 0.0;
    visits += activate(A, v, A.delta[v], A.pv0, r);
    res += r;
    // vertices without in-edges never change again: their leftover delta is
    // a constant part of every later residual
    if (A.pull_deg[v] == 0) res0 += fabs((double)A.delta[v]);
    A.pvb[0][v] = 0.f;
    A.pvb[1][v] = 0.f;
  }
  const double b = block_sum<VT>(res, s_red);
  const double b0 = block_sum<VT>(res0, s_red2);
  if (threadIdx.x == 0) {
    atomicAdd(&A.res[R_LAST], b);
    atomicAdd(&A.res[R_ZERO_IN], b0);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) visits += __shfl_down_sync(0xffffffffu, visits, o);
  if ((threadIdx.x & 31) == 0 && visits) atomicAdd(&A.cnt[C_VISITS], visits);
}

constexpr int PT_THREADS = 256;
constexpr int PT_QPT = kPullTileQuads / PT_THREADS;  // quads per thread, contiguous
constexpr int PT_TILE = kPullTileQuads;              // quads per tile

struct PullArgs {
  const uint32_t* nz;      // vertices with in-degree > 0, in id order
  const uint64_t* qoff;    // [nz_count + 1] quad prefix
  const uint32_t* tile_v0; // owner (nz index) of each tile's first quad
  uint32_t nz_count;
  uint64_t quads;
  uint64_t ntiles;
  const uint64_t* off;     // the pulled CSR (in-CSR for PageRank)
  const uint32_t* col;
  const float* w;          // its weights (weighted pulls only)
};

// pull number p reads pvb[p & 1] (or pv0 for p == 0) and writes the next
// push values into pvb[(p + 1) & 1].  W: multiply each gathered push value
// by the edge weight (weighted PageRank and its adjoint).
template <bool W>
__global__ void __launch_bounds__(PT_THREADS) k_pr_pull(PrArgs A, PullArgs P, int p) {
  __shared__ uint64_t sq[PT_TILE + 2];
  __shared__ uint32_t snz[PT_TILE + 1];
  __shared__ float sacc[PT_TILE + 1];
  __shared__ double s_red[PT_THREADS / 32];
  if (A.misc[M_DONE]) return;
  const bool drain = A.misc[M_PENDING] != 0;
  const float* __restrict__ pv = p == 0 ? A.pv0 : ((p & 1) ? A.pvb[1] : A.pvb[0]);
  float* pv_next = (p & 1) ? A.pvb[0] : A.pvb[1];
  double res = 0.0;
  unsigned long long visits = 0;
  for (uint64_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
    const uint64_t q0 = tile * PT_TILE;
    const uint64_t q1 = min(q0 + (uint64_t)PT_TILE, P.quads);
    const uint32_t v0 = P.tile_v0[tile];
    uint32_t v1;
    if (tile + 1 < P.ntiles) {
      const uint32_t nv = P.tile_v0[tile + 1];
      v1 = P.qoff[nv] < q1 ? nv : nv - 1;
    } else {
      v1 = P.nz_count - 1;
    }
    const uint32_t cnt = v1 - v0 + 1;
    for (uint32_t i = threadIdx.x; i <= cnt; i += PT_THREADS) {
      sq[i] = P.qoff[v0 + i];
      if (i < cnt) {
        snz[i] = P.nz[v0 + i];
        sacc[i] = 0.f;
      }
    }
    __syncthreads();
    // contiguous quads of this thread, owners walked in order
    const uint64_t qa = q0 + (uint64_t)threadIdx.x * PT_QPT;
    const uint64_t qb = min(qa + PT_QPT, q1);
    if (qa < qb) {
      uint32_t i = upper_owner(sq, 0u, cnt, qa);
      uint32_t v = snz[i];
      uint64_t base = P.off[v];
      uint64_t qbeg = sq[i], qend = sq[i + 1];
      uint32_t deg = A.pull_deg[v];
      float acc = 0.f;
      for (uint64_t q = qa; q < qb; ++q) {
        if (q >= qend) {
          if (acc != 0.f) atomicAdd(&sacc[i], acc);
          acc = 0.f;
          do {
            ++i;
          } while (q >= sq[i + 1]);
          v = snz[i];
          base = P.off[v];
          qbeg = sq[i];
          qend = sq[i + 1];
          deg = A.pull_deg[v];
        }
        const uint32_t k = (uint32_t)(q - qbeg) * 4;
        const uint4 c4 = *reinterpret_cast<const uint4*>(P.col + base + k);
        if (W) {
          const float4 w4 = *reinterpret_cast<const float4*>(P.w + base + k);
          float s = pv[c4.x] * w4.x;  // the last quad of a vertex may be partial
          if (k + 1 < deg) s += pv[c4.y] * w4.y;
          if (k + 2 < deg) s += pv[c4.z] * w4.z;
          if (k + 3 < deg) s += pv[c4.w] * w4.w;
          acc += s;
        } else {
          float s = pv[c4.x];  // the last quad of a vertex may be partial
          if (k + 1 < deg) s += pv[c4.y];
          if (k + 2 < deg) s += pv[c4.z];
          if (k + 3 < deg) s += pv[c4.w];
          acc += s;
        }
      }
      if (acc != 0.f) atomicAdd(&sacc[i], acc);
    }
    __syncthreads();
    // epilogue: vertices entirely inside the tile are final for this round
    for (uint32_t i = threadIdx.x; i < cnt; i += PT_THREADS) {
      const uint32_t v = snz[i];
      const float s = sacc[i];
      const bool interior = sq[i] >= q0 && sq[i + 1] <= q1;
      if (interior) {
        const float dl = A.delta[v] + s;
        if (drain) {
          A.delta[v] = dl;
          res += fabs((double)dl);
        } else {
          visits += activate(A, v, dl, pv_next, res);
        }
      } else if (s != 0.f) {
        atomicAdd(&A.delta[v], s);
      }
    }
    __syncthreads();
  }
  const double b = block_sum<PT_THREADS>(res, s_red);
  if (threadIdx.x == 0 && b != 0.0) atomicAdd(&A.res[R_ACC], b);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) visits += __shfl_down_sync(0xffffffffu, visits, o);
  if ((threadIdx.x & 31) == 0 && visits) atomicAdd(&A.cnt[C_VISITS], visits);
}

// Tile-spanning vertices, then the round's termination decision.
__global__ void __launch_bounds__(VT) k_pr_fixup(PrArgs A, const uint32_t* __restrict__ bnd,
                                                 uint32_t nb, int p) {
  __shared__ double s_red[VT / 32];
  __shared__ bool s_last;
  if (A.misc[M_DONE]) return;
  const bool drain = A.misc[M_PENDING] != 0;
  float* pv_next = (p & 1) ? A.pvb[0] : A.pvb[1];
  double res = 0.0;
  unsigned long long visits = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
    const uint32_t v = bnd[i];
    const float dl = A.delta[v];
    if (drain) res += fabs((double)dl);
    else visits += activate(A, v, dl, pv_next, res);
  }
  const double b = block_sum<VT>(res, s_red);
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
  dfree(s.x); dfree(s.delta); dfree(s.acc); dfree(s.pv); dfree(s.frontier);
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

  PullArgs P;
  P.nz = L.nz;
  P.qoff = L.qoff;
  P.tile_v0 = L.tile_v0;
  P.nz_count = L.nz_count;
  P.quads = L.quads;
  P.ntiles = L.ntiles;
  P.off = R.csr->off;
  P.col = R.csr->col;
  P.w = R.weighted ? R.csr->w : nullptr;

  const unsigned vblocks = grid_for(g.n, VT, ctx->num_sms * 8);
  const unsigned pblocks =
      (unsigned)std::min<uint64_t>(std::max<uint64_t>(P.ntiles, 1), (uint64_t)ctx->num_sms * 8);
  const unsigned fblocks = grid_for(std::max<uint32_t>(L.bnd_count, 1), VT, ctx->num_sms * 2);
  const int kpull = R.kclass;

  SG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
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
        if (R.weighted) k_pr_pull<true><<<pblocks, PT_THREADS, 0, st>>>(A, P, pull);
        else k_pr_pull<false><<<pblocks, PT_THREADS, 0, st>>>(A, P, pull);
        kprof_end(ctx, kpull);
        kprof_begin(ctx);
        k_pr_fixup<<<fblocks, VT, 0, st>>>(A, L.bnd, L.bnd_count, pull);
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
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
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
