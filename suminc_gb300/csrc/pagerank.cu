// Delta-accumulative PageRank (Ingress form) on the device.
//
// State per vertex: x (values_), delta (deltas_), acc (incoming sums of the
// current round), pv (this round's push value d * delta / outdeg).
//
// One round = k_pr_vertex + (k_pr_pull | k_pr_push):
//   k_pr_vertex  delta += acc; residual += |delta|; a vertex with
//                |delta| > threshold / N (isChange, sum_sync_iter_worker.h:
//                2914-2925) moves delta into x and publishes pv
//                (g_function, pagerank_ingress.h:50-72); the last block
//                picks the propagation mode for the round on the device.
//   k_pr_pull    dense rounds: acc[v] += sum of pv over in-edges, edge-balanced
//                over 4-edge quads of the in-CSR (no global atomics per edge).
//   k_pr_push    sparse rounds: frontier vertices scatter pv to out-edges.
// The residual sum|delta| is the reference's termCheck
// (sum_sync_iter_worker.h:2873-2912), accumulated in FP64.
#include <cmath>

#include "ctx.h"
#include "dev.cuh"

namespace sg {

enum {
  M_FCNT0 = 0,   // frontier counters (double-buffered by round parity)
  M_FCNT1 = 1,
  M_DONE = 2,
  M_PENDING = 3,
  M_BLOCKS = 4,
  M_MODE = 5,    // 0 pull, 1 push, 2 idle (no active vertex)
  M_ROUNDS = 6,
  M_NOTCONV = 7,
  M_WORDS = 8
};
enum { C_EDGES = 0, C_VISITS = 1, C_FEDGES = 2, C_PUSHED = 3, C_WORDS = 4 };

struct PrRoundArgs {
  uint32_t n;
  float damping;
  float thr_v;            // threshold / N
  double tau;             // termcheck threshold
  int max_rounds;
  float alpha;            // push when frontier edges * alpha < live edges
  uint64_t live_edges;
  const uint32_t* out_deg;
  float* x;
  float* delta;
  float* acc;
  float* pv;
  uint32_t* frontier;
  uint32_t* misc;
  double* res;            // [0] accumulator, [1] last residual
  unsigned long long* cnt;
};

constexpr int VT = 256;  // vertex kernel block size

__global__ void __launch_bounds__(VT) k_pr_vertex(PrRoundArgs A, int round) {
  __shared__ double s_red[VT / 32];
  __shared__ unsigned long long s_fe[VT / 32];
  __shared__ bool s_last;
  if (A.misc[M_DONE]) return;
  if (A.misc[M_PENDING]) {
    if (blockIdx.x == 0 && threadIdx.x == 0) A.misc[M_DONE] = 1;
    return;
  }
  uint32_t* fcnt = &A.misc[(round & 1) ? M_FCNT1 : M_FCNT0];
  double res = 0.0;
  unsigned long long fedges = 0, visits = 0;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t nn = ((A.n + 31u) / 32u) * 32u;  // whole warps for warp_append
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nn; v += stride) {
    bool push = false;
    uint32_t od = 0;
    if (v < A.n) {
      float dl = A.delta[v] + A.acc[v];
      A.acc[v] = 0.f;
      res += fabs((double)dl);
      float p = 0.f;
      if (fabsf(dl) > A.thr_v) {
        A.x[v] += dl;
        od = A.out_deg[v];
        if (od > 0) {
          p = A.damping * dl / (float)od;
          push = true;
          fedges += od;
        }
        visits++;
        dl = 0.f;
      }
      A.delta[v] = dl;
      A.pv[v] = p;
    }
    const uint32_t slot = warp_append(push, fcnt);
    if (push) A.frontier[slot] = v;
  }
  // block reductions
  const double bres = block_sum<VT>(res, s_red);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fedges += __shfl_down_sync(0xffffffffu, fedges, o);
    visits += __shfl_down_sync(0xffffffffu, visits, o);
  }
  if ((threadIdx.x & 31) == 0) s_fe[threadIdx.x >> 5] = fedges;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long fe = 0;
    for (int i = 0; i < VT / 32; ++i) fe += s_fe[i];
    atomicAdd(&A.res[0], bres);
    atomicAdd(&A.cnt[C_FEDGES], fe);
    __threadfence();
    const uint32_t done_blocks = atomicAdd(&A.misc[M_BLOCKS], 1u);
    s_last = (done_blocks == gridDim.x - 1);
  }
  if ((threadIdx.x & 31) == 0 && visits) atomicAdd(&A.cnt[C_VISITS], visits);
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    const double R = atomicAdd(&A.res[0], 0.0);
    const unsigned long long fe = atomicAdd(&A.cnt[C_FEDGES], 0ull);
    A.res[0] = 0.0;
    A.res[1] = R;
    A.cnt[C_FEDGES] = 0;
    A.misc[M_BLOCKS] = 0;
    A.misc[(round & 1) ? M_FCNT0 : M_FCNT1] = 0;  // next round's counter
    const uint32_t rounds = A.misc[M_ROUNDS] + 1;
    A.misc[M_ROUNDS] = rounds;
    uint32_t mode;
    if (fe == 0) mode = 2;
    else if ((double)fe * A.alpha < (double)A.live_edges) mode = 1;
    else mode = 0;
    A.misc[M_MODE] = mode;
    if (mode == 0) A.cnt[C_EDGES] += A.live_edges;
    else if (mode == 1) A.cnt[C_PUSHED] += fe;
    if (R < A.tau || fe == 0) A.misc[M_PENDING] = 1;
    if ((int)rounds >= A.max_rounds && !(R < A.tau)) {
      A.misc[M_PENDING] = 1;
      A.misc[M_NOTCONV] = 1;
    }
  }
}

// Edge-balanced pull over the in-CSR: a tile covers PT_THREADS * PT_QPT
// consecutive 4-edge quads of the concatenated in-segments of the vertices
// with in-degree > 0.
constexpr int PT_THREADS = 256;
constexpr int PT_QPT = 4;
constexpr int PT_TILE = PT_THREADS * PT_QPT;

struct PullArgs {
  const uint32_t* nz;      // vertices with in-degree > 0
  const uint64_t* qoff;    // [nz_count + 1] quad prefix
  uint32_t nz_count;
  uint64_t quads;
  const uint64_t* off;
  const uint32_t* deg;
  const uint32_t* col;
  const float* pv;
  float* acc;
  const uint32_t* misc;
};

__global__ void __launch_bounds__(PT_THREADS) k_pr_pull(PullArgs P) {
  __shared__ uint64_t sq[PT_TILE + 2];
  __shared__ float sacc[PT_TILE + 1];
  __shared__ uint32_t s_v0, s_cnt;
  if (P.misc[M_DONE] || P.misc[M_MODE] != 0) return;
  const uint64_t ntiles = (P.quads + PT_TILE - 1) / PT_TILE;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t q0 = tile * PT_TILE;
    const uint64_t q1 = min(q0 + (uint64_t)PT_TILE, P.quads);
    if (threadIdx.x == 0) {
      const uint32_t v0 = upper_owner(P.qoff, 0u, P.nz_count, q0);
      const uint32_t v1 = upper_owner(P.qoff, v0, P.nz_count, q1 - 1);
      s_v0 = v0;
      s_cnt = v1 - v0 + 1;
    }
    __syncthreads();
    const uint32_t v0 = s_v0, cnt = s_cnt;
    for (uint32_t i = threadIdx.x; i <= cnt; i += PT_THREADS) {
      sq[i] = P.qoff[v0 + i];
      sacc[i] = 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PT_QPT; ++j) {
      const uint64_t q = q0 + (uint64_t)j * PT_THREADS + threadIdx.x;
      if (q < q1) {
        const uint32_t i = upper_owner(sq, 0u, cnt, q);
        const uint32_t v = P.nz[v0 + i];
        const uint32_t kq = (uint32_t)(q - sq[i]);
        const uint32_t d = P.deg[v];
        const uint4 c4 = *reinterpret_cast<const uint4*>(P.col + P.off[v] + 4ull * kq);
        const uint32_t k = 4u * kq;
        float s = P.pv[c4.x];
        if (k + 1 < d) s += P.pv[c4.y];
        if (k + 2 < d) s += P.pv[c4.z];
        if (k + 3 < d) s += P.pv[c4.w];
        if (s != 0.f) atomicAdd(&sacc[i], s);
      }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < cnt; i += PT_THREADS) {
      const float s = sacc[i];
      if (s != 0.f) atomicAdd(&P.acc[P.nz[v0 + i]], s);
    }
    __syncthreads();
  }
}

struct PushArgs {
  const uint32_t* frontier;
  const uint32_t* misc;
  const uint64_t* off;
  const uint32_t* deg;
  const uint32_t* col;
  const float* pv;
  float* acc;
};

__global__ void __launch_bounds__(256) k_pr_push(PushArgs P, int round) {
  if (P.misc[M_DONE] || P.misc[M_MODE] != 1) return;
  const uint32_t cnt = P.misc[(round & 1) ? M_FCNT1 : M_FCNT0];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nwarps) {
    const uint32_t v = P.frontier[i];
    const float val = P.pv[v];
    const uint32_t d = P.deg[v];
    const uint32_t* seg = P.col + P.off[v];
    for (uint32_t k = lane * 4; k < d; k += 128) {
      const uint4 c4 = *reinterpret_cast<const uint4*>(seg + k);
      atomicAdd(&P.acc[c4.x], val);
      if (k + 1 < d) atomicAdd(&P.acc[c4.y], val);
      if (k + 2 < d) atomicAdd(&P.acc[c4.z], val);
      if (k + 3 < d) atomicAdd(&P.acc[c4.w], val);
    }
  }
}

// Folds the last round's incoming sums into delta and measures the final
// residual.
__global__ void __launch_bounds__(VT) k_pr_fold(uint32_t n, float* delta, float* acc,
                                                double* res) {
  __shared__ double s_red[VT / 32];
  double r = 0.0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const float d = delta[v] + acc[v];
    acc[v] = 0.f;
    delta[v] = d;
    r += fabs((double)d);
  }
  const double b = block_sum<VT>(r, s_red);
  if (threadIdx.x == 0) atomicAdd(&res[0], b);
}

__global__ void k_pr_init(uint32_t n, float* x, float* delta, float* acc, float init_c) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    x[v] = 0.f;       // init_v (pagerank_ingress.h:32)
    delta[v] = init_c;  // init_c = (1-d)/N (pagerank_ingress.h:27-30)
    acc[v] = 0.f;
  }
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
  const uint32_t n = ctx->g.n;
  pr_free(ctx);
  SG_TRY(dalloc(ctx, &s.x, n));
  SG_TRY(dalloc(ctx, &s.delta, n));
  SG_TRY(dalloc(ctx, &s.acc, n));
  SG_TRY(dalloc(ctx, &s.pv, n));
  SG_TRY(dalloc(ctx, &s.frontier, n));
  SG_TRY(dalloc(ctx, &s.d_misc, M_WORDS));
  SG_TRY(dalloc(ctx, &s.d_res, 2));
  SG_TRY(dalloc(ctx, &s.d_cnt, C_WORDS));
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
    k_pr_init<<<grid_for(g.n, 256), 256, 0, st>>>(g.n, s.x, s.delta, s.acc, init_c);
  } else if (!s.valid) {
    return fail(ctx, SG_ERR_STATE, "PageRank IncEval before PEval");
  }
  SG_CUDA(ctx, cudaMemsetAsync(s.d_misc, 0, sizeof(uint32_t) * M_WORDS, st));
  SG_CUDA(ctx, cudaMemsetAsync(s.d_res, 0, sizeof(double) * 2, st));
  SG_CUDA(ctx, cudaMemsetAsync(s.d_cnt, 0, sizeof(unsigned long long) * C_WORDS, st));

  PrRoundArgs A;
  A.n = g.n;
  A.damping = (float)ctx->opt.damping;
  A.thr_v = (float)(ctx->opt.termcheck_threshold / (double)g.n);
  A.tau = ctx->opt.termcheck_threshold;
  A.max_rounds = ctx->opt.max_rounds > 0 ? ctx->opt.max_rounds : 1000;
  A.alpha = 4.0f;
  A.live_edges = g.m;
  A.out_deg = g.out.deg;
  A.x = s.x; A.delta = s.delta; A.acc = s.acc; A.pv = s.pv;
  A.frontier = s.frontier;
  A.misc = s.d_misc;
  A.res = s.d_res;
  A.cnt = (unsigned long long*)s.d_cnt;

  PullArgs P;
  P.nz = g.in_nz; P.qoff = g.in_qoff; P.nz_count = g.in_nz_count; P.quads = g.in_quads;
  P.off = g.in.off; P.deg = g.in.deg; P.col = g.in.col; P.pv = s.pv; P.acc = s.acc;
  P.misc = s.d_misc;
  PushArgs Q;
  Q.frontier = s.frontier; Q.misc = s.d_misc; Q.off = g.out.off; Q.deg = g.out.deg;
  Q.col = g.out.col; Q.pv = s.pv; Q.acc = s.acc;

  const unsigned vblocks = grid_for(g.n, VT, ctx->num_sms * 8);
  const uint64_t ntiles = (g.in_quads + PT_TILE - 1) / PT_TILE;
  const unsigned pblocks = (unsigned)std::min<uint64_t>(std::max<uint64_t>(ntiles, 1),
                                                        (uint64_t)ctx->num_sms * 8);
  const unsigned hblocks = (unsigned)ctx->num_sms * 8;

  SG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  int round = 0;
  const int chunk = 4;
  uint32_t h_misc[M_WORDS];
  for (;;) {
    for (int r = 0; r < chunk; ++r, ++round) {
      kprof_begin(ctx);
      k_pr_vertex<<<vblocks, VT, 0, st>>>(A, round);
      kprof_end(ctx, SG_K_PR_VERTEX);
      kprof_begin(ctx);
      k_pr_pull<<<pblocks, PT_THREADS, 0, st>>>(P);
      kprof_end(ctx, SG_K_PR_PULL);
      kprof_begin(ctx);
      k_pr_push<<<hblocks, 256, 0, st>>>(Q, round);
      kprof_end(ctx, SG_K_PR_PUSH);
    }
    SG_CUDA(ctx, cudaGetLastError());
    SG_CUDA(ctx, cudaMemcpyAsync(h_misc, s.d_misc, sizeof(h_misc), cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
    if (h_misc[M_DONE] || h_misc[M_PENDING]) break;
    if (round > 4 * A.max_rounds + 64) break;  // host-side guard
  }
  SG_CUDA(ctx, cudaMemsetAsync(s.d_res, 0, sizeof(double), st));
  k_pr_fold<<<vblocks, VT, 0, st>>>(g.n, s.delta, s.acc, s.d_res);
  SG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  double h_res[2];
  unsigned long long h_cnt[C_WORDS];
  SG_CUDA(ctx, cudaMemcpyAsync(h_res, s.d_res, sizeof(h_res), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(h_cnt, s.d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(h_misc, s.d_misc, sizeof(h_misc), cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  s.valid = true;
  ctx->stats.rounds = (int32_t)h_misc[M_ROUNDS];
  ctx->stats.converged = h_misc[M_NOTCONV] ? 0 : 1;
  ctx->stats.residual = h_res[0];
  ctx->stats.edges_relaxed = h_cnt[C_EDGES] + h_cnt[C_PUSHED];
  ctx->stats.edges_pull = h_cnt[C_EDGES];
  ctx->stats.edges_push = h_cnt[C_PUSHED];
  ctx->stats.vertex_visits = h_cnt[C_VISITS];
  ctx->stats.elapsed_ms = ms;
  ctx->stats.live_edges = g.m;
  if (h_misc[M_NOTCONV])
    return fail(ctx, SG_ERR_NOT_CONVERGED, "PageRank reached the round cap");
  return SG_OK;
}

}  // namespace sg
