// PageRank with edge weights, and its hand-written adjoint.
//
// Forward (the Ingress delta rounds with weights): x = (1-d) t + d M x with
// M[v][u] = w_uv (the edge weights as given; column-normalised weights make
// M column-stochastic) and teleport vector t (uniform 1/N by default).  Delta
// rounds pull over the in-CSR, multiplying each gathered push value d*delta_u
// by w_uv.
//
// Adjoint: for a loss L(x) with g = dL/dx, lambda solves
//   lambda = g + d M^T lambda,
// the transposed delta iteration: the same rounds pulling over the out-CSR
// (lambda_u += d * sum_v w_uv * dlambda_v), FP32 with an FP64 residual.  Then
//   dL/dw_uv = d * lambda_v * x_u        (one pass over the edges)
//   dL/dt_v  = (1 - d) * lambda_v.
// Both use the partial sums plus the unpropagated remainder (x + delta,
// lambda + dlambda), the closest estimate the rounds leave.
//
// Edge gradients are written in the order of sg_graph_download_csr (rows by
// source, neighbours ascending), from a packed copy of the out-CSR kept while
// the graph is unchanged.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.h"
#include "dev.cuh"

namespace sg {

struct AdjState {
  uint32_t n_alloc = 0;
  float *x = nullptr, *delta = nullptr;    // forward values / remainder
  float *lam = nullptr, *dlam = nullptr;   // adjoint values / remainder
  float *pv0 = nullptr, *pvb = nullptr;    // push values (shared by both runs)
  uint32_t* misc = nullptr;
  double* res = nullptr;
  unsigned long long* cnt = nullptr;
  float* vec = nullptr;                    // staging: teleport / loss gradient
  float* dt = nullptr;                     // dL/dt
  float* dw = nullptr;                     // dL/dw, packed order
  uint64_t dw_cap = 0;
  uint64_t* prp = nullptr;                 // packed sorted out-CSR
  uint32_t* pcol = nullptr;
  uint32_t* psrc = nullptr;                // source of each packed entry
  float *xs = nullptr, *ls = nullptr;      // x + delta, lambda + dlambda
  uint64_t packed_gen = ~0ull, packed_cap = 0;
  bool fwd_valid = false, adj_valid = false;
  uint64_t fwd_gen = 0;
  sg_adjoint_info info{};
};

static AdjState* astate(sg_ctx* ctx) { return (AdjState*)ctx->adjoint_state; }

static void afree_arrays(AdjState& S) {
  dfree(S.x); dfree(S.delta); dfree(S.lam); dfree(S.dlam); dfree(S.pv0); dfree(S.pvb);
  dfree(S.misc); dfree(S.res); dfree(S.cnt); dfree(S.vec); dfree(S.dt); dfree(S.dw);
  dfree(S.prp); dfree(S.pcol); dfree(S.psrc); dfree(S.xs); dfree(S.ls);
}

sg_status adjoint_free(sg_ctx* ctx) {
  AdjState* S = astate(ctx);
  if (S) {
    afree_arrays(*S);
    delete S;
  }
  ctx->adjoint_state = nullptr;
  return SG_OK;
}

static sg_status areserve(sg_ctx* ctx, AdjState& S) {
  const uint32_t n = ctx->g.n;
  if (S.n_alloc == n && S.x) return SG_OK;
  afree_arrays(S);
  S = AdjState();
  SG_TRY(dalloc(ctx, &S.x, n));
  SG_TRY(dalloc(ctx, &S.delta, n));
  SG_TRY(dalloc(ctx, &S.lam, n));
  SG_TRY(dalloc(ctx, &S.dlam, n));
  SG_TRY(dalloc(ctx, &S.pv0, n));
  SG_TRY(dalloc(ctx, &S.pvb, 2ull * n));
  SG_TRY(dalloc(ctx, &S.misc, 8));
  SG_TRY(dalloc(ctx, &S.res, 4));
  SG_TRY(dalloc(ctx, &S.cnt, 4));
  SG_TRY(dalloc(ctx, &S.vec, n));
  SG_TRY(dalloc(ctx, &S.dt, n));
  S.n_alloc = n;
  return SG_OK;
}

// x = 0, delta = (1-d) t (t uniform 1/n when tele is null)
__global__ void k_adj_init(uint32_t n, float* x, float* delta, const float* tele, float one_minus_d) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    x[v] = 0.f;
    delta[v] = tele ? one_minus_d * tele[v] : one_minus_d / (float)n;
  }
}

// lambda = 0, dlambda = g; FP64 sum |g| for the residual scale
__global__ void k_adj_seed(uint32_t n, float* lam, float* dlam, const float* g, double* gsum) {
  __shared__ double s_red[8];
  double r = 0.0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    lam[v] = 0.f;
    dlam[v] = g[v];
    r += fabs((double)g[v]);
  }
  const double b = block_sum<256>(r, s_red);
  if (threadIdx.x == 0 && b != 0.0) atomicAdd(gsum, b);
}

// dL/dw_uv = d * (lambda + dlambda)_v * (x + delta)_u, a thread per packed
// entry: the source and column streams are read once and coalesced, the
// source's value is nearly coalesced (entries sorted by source), the
// column's adjoint value is the one random gather per edge (both sums
// formed once per vertex beforehand)
__global__ void k_adj_grad_w(uint64_t m, const uint32_t* __restrict__ src,
                             const uint32_t* __restrict__ col, const float* __restrict__ xs,
                             const float* __restrict__ ls, float d, float* __restrict__ dw) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
       e += (uint64_t)gridDim.x * blockDim.x)
    dw[e] = d * xs[src[e]] * ls[col[e]];
}

// the source of every packed entry (warp per row; once per packing)
__global__ void k_row_ids(uint32_t n, const uint64_t* __restrict__ rp, uint32_t* __restrict__ src) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t wv = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wv < n;
       wv += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const uint64_t a = rp[wv], b = rp[wv + 1];
    for (uint64_t e = a + lane; e < b; e += 32) src[e] = (uint32_t)wv;
  }
}

// dL/dt = (1-d) * (lambda + dlambda)
__global__ void k_adj_grad_t(uint32_t n, const float* lam, const float* dlam, float c, float* dt) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    dt[v] = c * (lam[v] + dlam[v]);
}

__global__ void k_add(uint32_t n, const float* a, const float* b, float* o) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    o[v] = a[v] + b[v];
}

sg_status pr_weighted_forward(sg_ctx* ctx, const float* tele_host, float* x_out) {
  DevGraph& g = ctx->g;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  if (!g.weighted) return fail(ctx, SG_ERR_INVALID, "weighted PageRank needs edge weights");
  if (!ctx->adjoint_state) ctx->adjoint_state = new AdjState();
  AdjState& S = *astate(ctx);
  SG_TRY(areserve(ctx, S));
  S.fwd_valid = false;
  S.adj_valid = false;
  cudaStream_t st = ctx->stream;
  const uint32_t n = g.n;
  if (tele_host)
    SG_CUDA(ctx, cudaMemcpyAsync(S.vec, tele_host, 4ull * n, cudaMemcpyHostToDevice, st));
  k_adj_init<<<grid_for(n, 256), 256, 0, st>>>(n, S.x, S.delta, tele_host ? S.vec : nullptr,
                                               (float)(1.0 - ctx->opt.damping));
  count_launch(ctx);
  PrRunSpec R;
  R.buf = {S.x, S.delta, S.pv0, S.pvb, S.misc, S.res, S.cnt};
  R.lists = &g.in_wl;
  R.csr = &g.in;
  R.weighted = true;
  R.scale_deg = nullptr;
  R.tau = ctx->opt.termcheck_threshold;
  R.kclass = SG_K_PR_PULL;
  const sg_status rs = pr_rounds_ex(ctx, R);
  if (rs != SG_OK && rs != SG_ERR_NOT_CONVERGED) return rs;
  S.info.forward_rounds = ctx->stats.rounds;
  S.info.forward_ms = ctx->stats.elapsed_ms;
  S.info.forward_residual = ctx->stats.residual;
  S.info.forward_edges = ctx->stats.edges_relaxed;
  S.fwd_valid = true;
  S.fwd_gen = g.gen;
  if (x_out) {
    SG_CUDA(ctx, cudaMemcpyAsync(x_out, S.x, 4ull * n, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
  }
  return rs;
}

sg_status pr_adjoint(sg_ctx* ctx, const float* dl_dx_host, bool on_device, float* dl_dw,
                     float* dl_dt) {
  DevGraph& g = ctx->g;
  AdjState* Sp = astate(ctx);
  if (!Sp || !Sp->fwd_valid || Sp->fwd_gen != g.gen)
    return fail(ctx, SG_ERR_STATE, "adjoint needs a weighted PageRank of the current graph");
  AdjState& S = *Sp;
  S.adj_valid = false;
  cudaStream_t st = ctx->stream;
  const uint32_t n = g.n;
  const uint64_t m = g.m;
  SG_TRY(graph_out_worklists(ctx));
  if (S.packed_gen != g.gen) {
    if (m + 1 > S.packed_cap) {
      dfree(S.pcol);
      dfree(S.psrc);
      dfree(S.dw);
      S.packed_cap = m + 1;
      SG_TRY(dalloc(ctx, &S.pcol, S.packed_cap));
      SG_TRY(dalloc(ctx, &S.psrc, S.packed_cap));
      SG_TRY(dalloc(ctx, &S.dw, S.packed_cap));
    }
    if (!S.prp) SG_TRY(dalloc(ctx, &S.prp, (uint64_t)n + 1));
    SG_TRY(packed_sorted_out(ctx, S.prp, S.pcol));
    k_row_ids<<<grid_for((uint64_t)n * 32, 256), 256, 0, st>>>(n, S.prp, S.psrc);
    count_launch(ctx);
    S.packed_gen = g.gen;
  }
  cudaEvent_t e0 = ctx->kev0, e1 = ctx->kev1;
  SG_CUDA(ctx, cudaEventRecord(e0, st));
  if (on_device) {
    SG_CUDA(ctx, cudaMemcpyAsync(S.vec, dl_dx_host, 4ull * n, cudaMemcpyDeviceToDevice, st));
  } else {
    SG_CUDA(ctx, cudaMemcpyAsync(S.vec, dl_dx_host, 4ull * n, cudaMemcpyHostToDevice, st));
  }
  // residual scale: sum |g| (FP64), read back once
  SG_CUDA(ctx, cudaMemsetAsync(S.res + 3, 0, 8, st));
  k_adj_seed<<<grid_for(n, 256, ctx->num_sms * 4), 256, 0, st>>>(n, S.lam, S.dlam, S.vec, S.res + 3);
  count_launch(ctx);
  double gsum = 0.0;
  SG_CUDA(ctx, cudaMemcpyAsync(&gsum, S.res + 3, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  sg_status rs = SG_OK;
  if (gsum > 0.0) {
    PrRunSpec R;
    R.buf = {S.lam, S.dlam, S.pv0, S.pvb, S.misc, S.res, S.cnt};
    R.lists = &g.out_wl;
    R.csr = &g.out;
    R.weighted = true;
    R.scale_deg = nullptr;
    // relative stop: the remaining adjoint mass below 1e-7 of |g| (FP32
    // resolution of the accumulated values)
    R.tau = gsum * ctx->opt.adjoint_rel_tol;
    R.kclass = SG_K_ADJOINT;
    rs = pr_rounds_ex(ctx, R);
    if (rs != SG_OK && rs != SG_ERR_NOT_CONVERGED) return rs;
    S.info.adjoint_rounds = ctx->stats.rounds;
    S.info.adjoint_residual = ctx->stats.residual;
    S.info.adjoint_edges = ctx->stats.edges_relaxed;
  } else {
    S.info.adjoint_rounds = 0;
    S.info.adjoint_residual = 0.0;
    S.info.adjoint_edges = 0;
  }
  const float d = (float)ctx->opt.damping;
  if (!S.xs) SG_TRY(dalloc(ctx, &S.xs, n));
  if (!S.ls) SG_TRY(dalloc(ctx, &S.ls, n));
  k_add<<<grid_for(n, 256), 256, 0, st>>>(n, S.x, S.delta, S.xs);
  k_add<<<grid_for(n, 256), 256, 0, st>>>(n, S.lam, S.dlam, S.ls);
  count_launch(ctx, 2);
  kprof_begin(ctx);
  k_adj_grad_w<<<grid_for(m, 256, ctx->num_sms * 16), 256, 0, st>>>(m, S.psrc, S.pcol, S.xs, S.ls,
                                                                      d, S.dw);
  kprof_end(ctx, SG_K_ADJOINT);
  k_adj_grad_t<<<grid_for(n, 256), 256, 0, st>>>(n, S.lam, S.dlam, 1.f - d, S.dt);
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaEventRecord(e1, st));
  if (dl_dw) SG_CUDA(ctx, cudaMemcpyAsync(dl_dw, S.dw, 4ull * m, cudaMemcpyDeviceToHost, st));
  if (dl_dt) SG_CUDA(ctx, cudaMemcpyAsync(dl_dt, S.dt, 4ull * n, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
  S.info.adjoint_ms = ms;
  S.info.gradient_edges = m;
  S.adj_valid = true;
  return rs;
}

sg_status adjoint_info(sg_ctx* ctx, sg_adjoint_info* out) {
  AdjState* S = astate(ctx);
  if (!S || !S->fwd_valid) return fail(ctx, SG_ERR_STATE, "no weighted PageRank has run");
  *out = S->info;
  return SG_OK;
}

sg_status adjoint_values(sg_ctx* ctx, float* x, float* lam) {
  AdjState* S = astate(ctx);
  if (!S || !S->fwd_valid) return fail(ctx, SG_ERR_STATE, "no weighted PageRank has run");
  const uint32_t n = ctx->g.n;
  cudaStream_t st = ctx->stream;
  if (x) SG_CUDA(ctx, cudaMemcpyAsync(x, S->x, 4ull * n, cudaMemcpyDeviceToHost, st));
  if (lam) {
    if (!S->adj_valid) return fail(ctx, SG_ERR_STATE, "no adjoint has run");
    k_add<<<grid_for(n, 256), 256, 0, st>>>(n, S->lam, S->dlam, S->vec);
    SG_CUDA(ctx, cudaMemcpyAsync(lam, S->vec, 4ull * n, cudaMemcpyDeviceToHost, st));
  }
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  return SG_OK;
}

}  // namespace sg
