// extern "C" surface of libsuminc_gb300: argument checks, device selection,
// error capture and the per-kernel-class profiler.  No C++ exception crosses
// this file's functions.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "ctx.h"

namespace sg {

sg_status fail(sg_ctx* ctx, sg_status st, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return st;
}

sg_status cuda_fail(sg_ctx* ctx, cudaError_t e, const char* where) {
  std::string m = std::string(cudaGetErrorName(e)) + ": " + cudaGetErrorString(e) + " at " + where;
  cudaGetLastError();
  return fail(ctx, e == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA, m);
}

// Profiling records an event pair around each launch of a kernel class and
// resolves the pairs after the API call's final synchronisation, so the
// launches stay asynchronous.  The bitmask opt.profile selects classes
// (bit k = class k; any non-zero value below 256 enables the listed ones).
void kprof_begin(sg_ctx* ctx) {
  count_launch(ctx);
  if (!ctx->opt.profile) return;
  if (ctx->kused + 2 > ctx->kpool.size()) {
    if (ctx->kpool.size() >= 8192) {
      cudaStreamSynchronize(ctx->stream);
      kprof_flush(ctx);
    } else {
      const size_t old = ctx->kpool.size();
      const size_t want = old ? old * 2 : 256;
      ctx->kpool.resize(want, nullptr);
      ctx->kclass.resize(want / 2, -1);
      for (size_t i = old; i < want; ++i) cudaEventCreate(&ctx->kpool[i]);
    }
  }
  cudaEventRecord(ctx->kpool[ctx->kused], ctx->stream);
  ctx->kopen = (int)ctx->kused;
}

void kprof_end(sg_ctx* ctx, int klass) {
  if (!ctx->opt.profile || ctx->kopen < 0) return;
  if (!(ctx->opt.profile & (1 << klass)) && ctx->opt.profile != 0xFF) {
    ctx->kopen = -1;  // class not selected: drop the begin event
    return;
  }
  cudaEventRecord(ctx->kpool[ctx->kused + 1], ctx->stream);
  ctx->kclass[ctx->kused / 2] = klass;
  ctx->kused += 2;
  ctx->kopen = -1;
}

void kprof_flush(sg_ctx* ctx) {
  for (size_t i = 0; i + 1 < ctx->kused; i += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->kpool[i], ctx->kpool[i + 1]) == cudaSuccess) {
      const int k = ctx->kclass[i / 2];
      ctx->stats.kernel_ms[k] += ms;
      ctx->stats.kernel_launches[k] += 1;
    }
  }
  cudaGetLastError();
  ctx->kused = 0;
}

}  // namespace sg

using namespace sg;

#define SG_GUARD(ctx)                                                  \
  if (!(ctx)) return SG_ERR_INVALID;                                   \
  do {                                                                 \
    cudaError_t e_ = cudaSetDevice((ctx)->device);                     \
    if (e_ != cudaSuccess) return cuda_fail((ctx), e_, "cudaSetDevice"); \
  } while (0)

#define SG_CATCH(ctx)                                                          \
  catch (const std::bad_alloc&) {                                             \
    return fail((ctx), SG_ERR_OOM, "host allocation failed");                  \
  }                                                                            \
  catch (...) {                                                                \
    return fail((ctx), SG_ERR_INVALID, "unexpected C++ exception");            \
  }

extern "C" {

sg_status sg_options_default(sg_options* o) {
  if (!o) return SG_ERR_INVALID;
  std::memset(o, 0, sizeof(*o));
  o->damping = 0.85;             // PageRankIngress::d
  o->termcheck_threshold = 1e-6; // the SumInc scripts' -termcheck_threshold
  o->max_rounds = 1000;
  o->compress = 0;
  o->max_node_num = 150;         // flags.cc:60
  o->min_node_num = 8;           // flags.cc:61
  o->mirror_k = 4;               // flags.cc:62
  o->profile = 0;
  o->compress_threshold = 1.0;   // flags.cc:67
  o->sssp_delta = 0.0;
  o->slack = 0.125;
  o->adjoint_rel_tol = 1e-7;
  return SG_OK;
}

sg_status sg_ctx_create(int device, const sg_options* opt, sg_ctx** out) {
  if (!out) return SG_ERR_INVALID;
  *out = nullptr;
  sg_ctx* ctx = nullptr;
  try {
    ctx = new sg_ctx();
  } catch (...) {
    return SG_ERR_OOM;
  }
  if (opt) ctx->opt = *opt; else sg_options_default(&ctx->opt);
  if (!(ctx->opt.damping > 0.0 && ctx->opt.damping < 1.0) || !(ctx->opt.termcheck_threshold > 0.0) ||
      (ctx->opt.message_type != SG_MSG_PUSH && ctx->opt.message_type != SG_MSG_PULL)) {
    delete ctx;
    return SG_ERR_INVALID;
  }
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  // The context's stream takes the highest priority: the summary repair
  // runs its shortcut solves on a stream of the lowest priority beside it,
  // and the table rebuilds queued here are dispatched ahead of them.
  int least = 0, greatest = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, greatest);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->kev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->kev1);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SG_ERR_CUDA;
  }
  ctx->own_stream = true;
  *out = ctx;
  return SG_OK;
}

sg_status sg_ctx_destroy(sg_ctx* ctx) {
  if (!ctx) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  pr_free(ctx);
  sssp_free(ctx);
  summary_free(ctx);
  batch_free(ctx);
  adjoint_free(ctx);
  pull_free(ctx);
  graph_free(ctx);
  DevBatch& B = ctx->batch;
  dfree(B.raw); dfree(B.key); dfree(B.key2); dfree(B.val); dfree(B.val2);
  dfree(B.a_src); dfree(B.a_dst); dfree(B.a_w); dfree(B.a_kind); dfree(B.a_found);
  dfree(B.grp_vertex); dfree(B.grp_begin); dfree(B.grp_end); dfree(B.perm);
  dfree(B.igrp_vertex); dfree(B.igrp_begin); dfree(B.igrp_end); dfree(B.d_count);
  dfree(B.a_pos_in); dfree(B.a_tmp); dfree(B.g_d0); dfree(B.g_ndel); dfree(B.g_nins);
  dfree(B.chunk_off); dfree(B.nch);
  if (ctx->cub_tmp) cudaFree(ctx->cub_tmp);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->kev0) cudaEventDestroy(ctx->kev0);
  if (ctx->kev1) cudaEventDestroy(ctx->kev1);
  for (auto e : ctx->kpool)
    if (e) cudaEventDestroy(e);
  for (auto e : ctx->user_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SG_OK;
}

const char* sg_last_error(const sg_ctx* ctx) {
  if (!ctx) return "null context";
  return ctx->err.c_str();
}

sg_status sg_ctx_set_stream(sg_ctx* ctx, void* stream) {
  SG_GUARD(ctx);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  ctx->stream = (cudaStream_t)stream;
  ctx->own_stream = false;
  return SG_OK;
}

sg_status sg_get_stats(const sg_ctx* ctx, sg_stats* out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  *out = ctx->stats;
  out->launches_total = ctx->launches;
  out->repacks = ctx->repacks;
  return SG_OK;
}

sg_status sg_ctx_record_event(sg_ctx* ctx, int slot) {
  SG_GUARD(ctx);
  if (slot < 0 || slot >= 8) return fail(ctx, SG_ERR_INVALID, "event slot out of range");
  if (!ctx->user_ev[slot]) SG_CUDA(ctx, cudaEventCreate(&ctx->user_ev[slot]));
  SG_CUDA(ctx, cudaEventRecord(ctx->user_ev[slot], ctx->stream));
  return SG_OK;
}

sg_status sg_ctx_elapsed_ms(sg_ctx* ctx, int a, int b, double* ms) {
  SG_GUARD(ctx);
  if (a < 0 || a >= 8 || b < 0 || b >= 8 || !ms || !ctx->user_ev[a] || !ctx->user_ev[b])
    return fail(ctx, SG_ERR_INVALID, "bad event slots");
  SG_CUDA(ctx, cudaEventSynchronize(ctx->user_ev[b]));
  float f = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&f, ctx->user_ev[a], ctx->user_ev[b]));
  *ms = f;
  return SG_OK;
}

sg_status sg_ctx_set_profile(sg_ctx* ctx, int32_t mask) {
  SG_GUARD(ctx);
  cudaStreamSynchronize(ctx->stream);
  kprof_flush(ctx);
  ctx->opt.profile = mask;
  return SG_OK;
}

sg_status sg_ctx_synchronize(sg_ctx* ctx) {
  SG_GUARD(ctx);
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

sg_status sg_reset_stats(sg_ctx* ctx) {
  if (!ctx) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  kprof_flush(ctx);
  std::memset(&ctx->stats, 0, sizeof(ctx->stats));
  ctx->launches = 0;
  ctx->repacks = 0;
  return SG_OK;
}

sg_status sg_graph_load_csr(sg_ctx* ctx, uint32_t n, const uint64_t* row_ptr,
                            const uint32_t* col, const float* w) {
  SG_GUARD(ctx);
  try {
    pr_free(ctx);
    sssp_free(ctx);
    summary_free(ctx);
    batch_free(ctx);
    adjoint_free(ctx);
    pull_free(ctx);
    ctx->oids.clear();
    return load_csr(ctx, n, row_ptr, col, w);
  }
  SG_CATCH(ctx)
}

sg_status sg_graph_generate_rmat(sg_ctx* ctx, int scale, uint64_t edges, double a, double b,
                                 double c, uint64_t seed, int weight_kind, double wlo,
                                 double whi) {
  SG_GUARD(ctx);
  if (!(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0)) return fail(ctx, SG_ERR_INVALID, "bad R-MAT probabilities");
  if (weight_kind < 0 || weight_kind > 2) return fail(ctx, SG_ERR_INVALID, "bad weight kind");
  if (weight_kind == 1 && !(whi >= wlo)) return fail(ctx, SG_ERR_INVALID, "bad weight range");
  try {
    pr_free(ctx);
    sssp_free(ctx);
    summary_free(ctx);
    batch_free(ctx);
    adjoint_free(ctx);
    pull_free(ctx);
    ctx->oids.clear();
    return generate_rmat(ctx, scale, edges, a, b, c, seed, weight_kind, wlo, whi);
  }
  SG_CATCH(ctx)
}

sg_status sg_graph_num_vertices(const sg_ctx* ctx, uint32_t* n) {
  if (!ctx || !n) return SG_ERR_INVALID;
  *n = ctx->g.n;
  return SG_OK;
}

sg_status sg_graph_num_edges(const sg_ctx* ctx, uint64_t* m) {
  if (!ctx || !m) return SG_ERR_INVALID;
  *m = ctx->g.m;
  return SG_OK;
}

sg_status sg_graph_download_csr(sg_ctx* ctx, uint64_t* row_ptr, uint32_t* col, float* w) {
  SG_GUARD(ctx);
  try {
    return download_csr(ctx, row_ptr, col, w);
  }
  SG_CATCH(ctx)
}

sg_status sg_apply_updates(sg_ctx* ctx, uint64_t count, const sg_update* upd) {
  SG_GUARD(ctx);
  try {
    sg_status st = apply_updates_device(ctx, count, upd, false);
    if (st == SG_OK && ctx->opt.compress) st = summary_after_apply(ctx);
    kprof_flush(ctx);
    return st;
  }
  SG_CATCH(ctx)
}

sg_status sg_apply_updates_device(sg_ctx* ctx, uint64_t count, const sg_update* dptr) {
  SG_GUARD(ctx);
  try {
    sg_status st = apply_updates_device(ctx, count, dptr, true);
    if (st == SG_OK && ctx->opt.compress) st = summary_after_apply(ctx);
    kprof_flush(ctx);
    return st;
  }
  SG_CATCH(ctx)
}

static sg_status copy_out_f32(sg_ctx* ctx, const float* d, float* h) {
  if (!h) return SG_OK;
  SG_CUDA(ctx, cudaMemcpyAsync(h, d, 4ull * ctx->g.n, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

sg_status sg_pr_peval(sg_ctx* ctx, float* out) {
  SG_GUARD(ctx);
  try {
    ctx->pr.valid = false;
    sg_status st = pr_alloc(ctx);
    if (st != SG_OK) return st;
    if (ctx->opt.message_type == SG_MSG_PULL) st = pr_pull_worker(ctx, false);
    else if (ctx->opt.compress) st = pr_summarized(ctx, false);
    else st = pr_run(ctx, false);
    kprof_flush(ctx);
    if (st != SG_OK && st != SG_ERR_NOT_CONVERGED) return st;
    sg_status c = copy_out_f32(ctx, ctx->pr.x, out);
    return c != SG_OK ? c : st;
  }
  SG_CATCH(ctx)
}

sg_status sg_pr_inceval(sg_ctx* ctx, float* out) {
  SG_GUARD(ctx);
  try {
    sg_status st = ctx->opt.message_type == SG_MSG_PULL ? pr_pull_worker(ctx, true)
                   : ctx->opt.compress                   ? pr_summarized(ctx, true)
                                                         : pr_run(ctx, true);
    kprof_flush(ctx);
    if (st != SG_OK && st != SG_ERR_NOT_CONVERGED) return st;
    sg_status c = copy_out_f32(ctx, ctx->pr.x, out);
    return c != SG_OK ? c : st;
  }
  SG_CATCH(ctx)
}

sg_status sg_pr_values(sg_ctx* ctx, float* out) {
  SG_GUARD(ctx);
  if (!ctx->pr.valid) return fail(ctx, SG_ERR_STATE, "no PageRank result");
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  return copy_out_f32(ctx, ctx->pr.x, out);
}

sg_status sg_pr_deltas(sg_ctx* ctx, float* out) {
  SG_GUARD(ctx);
  if (!ctx->pr.valid) return fail(ctx, SG_ERR_STATE, "no PageRank result");
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  return copy_out_f32(ctx, ctx->pr.delta, out);
}

sg_status sg_pr_values_device(sg_ctx* ctx, const float** dptr) {
  if (!ctx || !dptr) return SG_ERR_INVALID;
  if (!ctx->pr.valid) return fail(ctx, SG_ERR_STATE, "no PageRank result");
  *dptr = ctx->pr.x;
  return SG_OK;
}

sg_status sg_summary_build(sg_ctx* ctx, uint32_t n_clusters, const uint32_t* cluster_ptr,
                           const uint32_t* members) {
  SG_GUARD(ctx);
  if (n_clusters > 0 && (!cluster_ptr || !members))
    return fail(ctx, SG_ERR_INVALID, "null cluster arrays");
  try {
    std::vector<std::vector<uint32_t>> cl(n_clusters);
    for (uint32_t i = 0; i < n_clusters; ++i) {
      if (cluster_ptr[i + 1] < cluster_ptr[i]) return fail(ctx, SG_ERR_INVALID, "cluster_ptr not monotone");
      cl[i].assign(members + cluster_ptr[i], members + cluster_ptr[i + 1]);
      for (uint32_t v : cl[i])
        if (v >= ctx->g.n) return fail(ctx, SG_ERR_INVALID, "cluster member >= n");
    }
    pr_free(ctx);
    sg_status st = summary_build(ctx, cl);
    kprof_flush(ctx);
    return st;
  }
  SG_CATCH(ctx)
}

sg_status sg_summary_info_get(sg_ctx* ctx, sg_summary_info* out) {
  SG_GUARD(ctx);
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  return summary_info(ctx, out);
}

sg_status sg_summary_check_tables(sg_ctx* ctx, sg_summary_check* out) {
  SG_GUARD(ctx);
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  try {
    return summary_check(ctx, out);
  } catch (const std::bad_alloc&) {
    return fail(ctx, SG_ERR_OOM, "host allocation failed");
  }
}

sg_status sg_sssp_peval(sg_ctx* ctx, uint32_t source, double* out) {
  SG_GUARD(ctx);
  try {
    sg_status st = ctx->opt.compress && ctx->summary ? sssp_summarized(ctx, source)
                                                     : sssp_run_peval(ctx, source);
    kprof_flush(ctx);
    if (st != SG_OK) return st;
    if (out) return sssp_download(ctx, out);
    return SG_OK;
  }
  SG_CATCH(ctx)
}

sg_status sg_sssp_inceval(sg_ctx* ctx, double* out) {
  SG_GUARD(ctx);
  try {
    // over the summary once a summarized PEval has built its shortcut
    // distances; else (compress = 0, or a PEval on the original graph) plain
    sg_status st = ctx->opt.compress && sssp_summary_ready(ctx) ? sssp_summarized_inc(ctx)
                                                                : sssp_run_inceval(ctx);
    kprof_flush(ctx);
    if (st != SG_OK) return st;
    if (out) return sssp_download(ctx, out);
    return SG_OK;
  }
  SG_CATCH(ctx)
}

sg_status sg_sssp_distances(sg_ctx* ctx, double* out) {
  SG_GUARD(ctx);
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  try {
    return sssp_download(ctx, out);
  }
  SG_CATCH(ctx)
}

sg_status sg_debug_barrier_probe(sg_ctx* ctx, int32_t skip_one_block) {
  SG_GUARD(ctx);
  return sssp_barrier_probe(ctx, skip_one_block);
}

sg_status sg_sssp_parents(sg_ctx* ctx, uint32_t* out) {
  SG_GUARD(ctx);
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  if (!ctx->sp.valid) return fail(ctx, SG_ERR_STATE, "no SSSP result");
  SG_CUDA(ctx, cudaMemcpyAsync(out, ctx->sp.parent, 4ull * ctx->g.n, cudaMemcpyDeviceToHost,
                               ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

sg_status sg_ppr(sg_ctx* ctx, uint32_t n_seeds, const uint32_t* seeds, float* out) {
  SG_GUARD(ctx);
  try {
    if (!seeds || n_seeds == 0) return fail(ctx, SG_ERR_INVALID, "PPR needs seeds");
    if (!ctx->g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
    for (uint32_t i = 0; i < n_seeds; ++i)
      if (seeds[i] >= ctx->g.n) return fail(ctx, SG_ERR_INVALID, "seed vertex >= n");
    sg_status st = pr_alloc(ctx);
    if (st != SG_OK) return st;
    uint32_t* d_seeds = nullptr;
    st = dalloc(ctx, &d_seeds, n_seeds);
    if (st != SG_OK) return st;
    if (cudaMemcpyAsync(d_seeds, seeds, 4ull * n_seeds, cudaMemcpyHostToDevice, ctx->stream) !=
        cudaSuccess) {
      dfree(d_seeds);
      return fail(ctx, SG_ERR_CUDA, "seed upload failed");
    }
    st = pr_run_personalized(ctx, d_seeds, n_seeds);
    kprof_flush(ctx);
    cudaStreamSynchronize(ctx->stream);
    dfree(d_seeds);
    ctx->pr.valid = false;  // a personalized result is no IncEval state
    if (st != SG_OK && st != SG_ERR_NOT_CONVERGED) return st;
    sg_status c = copy_out_f32(ctx, ctx->pr.x, out);
    return c != SG_OK ? c : st;
  }
  SG_CATCH(ctx)
}

sg_status sg_batch_run(sg_ctx* ctx, const sg_batch_spec* spec, float* ppr_out, double* sssp_out) {
  SG_GUARD(ctx);
  if (!spec) return fail(ctx, SG_ERR_INVALID, "null batch spec");
  try {
    return batch_run(ctx, spec, ppr_out, sssp_out, false);
  }
  SG_CATCH(ctx)
}

sg_status sg_batch_tune_run(sg_ctx* ctx, const sg_batch_spec* spec, float* ppr_out,
                            double* sssp_out) {
  SG_GUARD(ctx);
  if (!spec) return fail(ctx, SG_ERR_INVALID, "null batch spec");
  try {
    return batch_run(ctx, spec, ppr_out, sssp_out, true);
  }
  SG_CATCH(ctx)
}

sg_status sg_batch_info_get(sg_ctx* ctx, sg_batch_info* out) {
  SG_GUARD(ctx);
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  return batch_info(ctx, out);
}

sg_status sg_batch_query_stats(sg_ctx* ctx, int32_t* rounds, double* residual) {
  SG_GUARD(ctx);
  try {
    return batch_query_stats(ctx, rounds, residual);
  }
  SG_CATCH(ctx)
}

sg_status sg_batch_outputs_device(sg_ctx* ctx, const float** ppr, const double** sssp) {
  SG_GUARD(ctx);
  return batch_device_outputs(ctx, ppr, sssp);
}

sg_status sg_graph_normalize_weights(sg_ctx* ctx) {
  SG_GUARD(ctx);
  try {
    return normalize_out_weights(ctx);
  }
  SG_CATCH(ctx)
}

sg_status sg_pr_weighted(sg_ctx* ctx, const float* tele, float* x_out) {
  SG_GUARD(ctx);
  try {
    sg_status st = pr_weighted_forward(ctx, tele, x_out);
    kprof_flush(ctx);
    return st;
  }
  SG_CATCH(ctx)
}

sg_status sg_pr_adjoint(sg_ctx* ctx, const float* dl_dx, float* dl_dw, float* dl_dtele) {
  SG_GUARD(ctx);
  if (!dl_dx) return fail(ctx, SG_ERR_INVALID, "null dL/dx");
  try {
    sg_status st = pr_adjoint(ctx, dl_dx, false, dl_dw, dl_dtele);
    kprof_flush(ctx);
    return st;
  }
  SG_CATCH(ctx)
}

sg_status sg_pr_adjoint_device(sg_ctx* ctx, const float* d_dl_dx, float* dl_dw, float* dl_dtele) {
  SG_GUARD(ctx);
  if (!d_dl_dx) return fail(ctx, SG_ERR_INVALID, "null dL/dx");
  try {
    sg_status st = pr_adjoint(ctx, d_dl_dx, true, dl_dw, dl_dtele);
    kprof_flush(ctx);
    return st;
  }
  SG_CATCH(ctx)
}

sg_status sg_adjoint_info_get(sg_ctx* ctx, sg_adjoint_info* out) {
  SG_GUARD(ctx);
  if (!out) return fail(ctx, SG_ERR_INVALID, "null output");
  return adjoint_info(ctx, out);
}

sg_status sg_adjoint_values(sg_ctx* ctx, float* x, float* lambda) {
  SG_GUARD(ctx);
  try {
    return adjoint_values(ctx, x, lambda);
  }
  SG_CATCH(ctx)
}

sg_status sg_graph_load_files(sg_ctx* ctx, const char* efile, const char* vfile, int weighted) {
  SG_GUARD(ctx);
  if (!efile) return fail(ctx, SG_ERR_INVALID, "null edge file name");
  try {
    pr_free(ctx);
    sssp_free(ctx);
    summary_free(ctx);
    batch_free(ctx);
    adjoint_free(ctx);
    pull_free(ctx);
    ctx->oids.clear();
    return load_files(ctx, efile, vfile, weighted != 0);
  }
  SG_CATCH(ctx)
}

sg_status sg_graph_vertex_oids(sg_ctx* ctx, uint64_t* oids) {
  SG_GUARD(ctx);
  if (!oids) return fail(ctx, SG_ERR_INVALID, "null output");
  if (!ctx->g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  for (uint32_t v = 0; v < ctx->g.n; ++v) oids[v] = ctx->oids.empty() ? v : ctx->oids[v];
  return SG_OK;
}

sg_status sg_graph_set_vertex_oids(sg_ctx* ctx, const uint64_t* oids) {
  SG_GUARD(ctx);
  if (!oids) return fail(ctx, SG_ERR_INVALID, "null oids");
  if (!ctx->g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  try {
    const uint32_t n = ctx->g.n;
    bool identity = true;
    for (uint32_t v = 0; v < n; ++v) {
      if (v > 0 && oids[v] <= oids[v - 1])
        return fail(ctx, SG_ERR_INVALID, "oids must be strictly increasing");
      identity = identity && oids[v] == v;
    }
    ctx->oids.clear();
    if (!identity) ctx->oids.assign(oids, oids + n);
    return SG_OK;
  }
  SG_CATCH(ctx)
}

sg_status sg_apply_update_file(sg_ctx* ctx, const char* path) {
  SG_GUARD(ctx);
  if (!path) return fail(ctx, SG_ERR_INVALID, "null update file name");
  if (!ctx->g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  try {
    std::vector<sg_update> upd;
    sg_status st = read_update_file(ctx, path, &upd);
    if (st != SG_OK) return st;
    if (upd.empty()) return SG_OK;
    return sg_apply_updates(ctx, upd.size(), upd.data());
  }
  SG_CATCH(ctx)
}

sg_status sg_summary_save(sg_ctx* ctx, const char* path) {
  SG_GUARD(ctx);
  if (!path) return fail(ctx, SG_ERR_INVALID, "null path");
  try {
    std::vector<uint8_t> blob;
    sg_status st = summary_serialized(ctx, &blob);
    if (st != SG_OK) return st;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ctx, SG_ERR_INVALID, std::string("cannot write ") + path);
    const size_t wr = std::fwrite(blob.data(), 1, blob.size(), f);
    std::fclose(f);
    if (wr != blob.size()) return fail(ctx, SG_ERR_INVALID, std::string("short write to ") + path);
    return SG_OK;
  }
  SG_CATCH(ctx)
}

sg_status sg_summary_load(sg_ctx* ctx, const char* path) {
  SG_GUARD(ctx);
  if (!path) return fail(ctx, SG_ERR_INVALID, "null path");
  if (!ctx->g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  try {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(ctx, SG_ERR_INVALID, std::string("cannot read ") + path);
    std::vector<uint8_t> blob;
    uint8_t buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) blob.insert(blob.end(), buf, buf + got);
    std::fclose(f);
    pr_free(ctx);
    sg_status st = summary_build_serialized(ctx, blob);
    kprof_flush(ctx);
    return st;
  }
  SG_CATCH(ctx)
}

sg_status sg_summary_build_file(sg_ctx* ctx, const char* path) {
  SG_GUARD(ctx);
  if (!path) return fail(ctx, SG_ERR_INVALID, "null cluster file name");
  if (!ctx->g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  try {
    std::vector<std::vector<uint32_t>> cl;
    sg_status st = read_cluster_file(ctx, path, &cl);
    if (st != SG_OK) return st;
    std::vector<uint32_t> ptr(cl.size() + 1, 0), mem;
    for (size_t i = 0; i < cl.size(); ++i) {
      ptr[i + 1] = ptr[i] + (uint32_t)cl[i].size();
      mem.insert(mem.end(), cl[i].begin(), cl[i].end());
    }
    return sg_summary_build(ctx, (uint32_t)cl.size(), ptr.data(), mem.empty() ? nullptr : mem.data());
  }
  SG_CATCH(ctx)
}

}  // extern "C"
