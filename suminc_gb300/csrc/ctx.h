// Internal context shared by the translation units of libsuminc_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/suminc_gb300.h"
#include "common.h"

namespace sg {

// One direction of adjacency.  Vertex v owns the segment
// col[off[v] .. off[v] + cap[v]); the first deg[v] slots are live.  Segment
// starts are multiples of 4 entries so a segment can be read with 128-bit
// loads.  Segments that outgrow their capacity move to the pool tail.
struct DevCSR {
  uint64_t* off = nullptr;
  uint32_t* deg = nullptr;
  uint32_t* cap = nullptr;
  uint32_t* col = nullptr;
  float* w = nullptr;           // null for unweighted graphs
  uint64_t pool_cap = 0;        // total slots allocated
  uint64_t* pool_tail = nullptr;  // device counter: first free slot
  uint64_t layout = 0;          // bumped when a repack moves every segment
};

// Edge-balanced work lists over one direction of adjacency: vertices with
// degree > 0 (with their segment offset and degree in the same order), the
// exclusive prefix of their 4-edge quads, the owner of the first quad of
// each kWarpTileQuads tile and the vertices whose quads span tiles.  Rebuilt
// when the adjacency changes.
struct PullLists {
  uint32_t* nz = nullptr;       // [n]
  uint64_t* qoff = nullptr;     // [n + 1]
  uint64_t* off_nz = nullptr;   // [n] segment offset of nz[i]
  uint32_t* deg_nz = nullptr;   // [n] live degree of nz[i]
  uint32_t nz_count = 0;
  uint64_t quads = 0;
  uint32_t* wtile_v0 = nullptr; // owner (index into nz) of each tile's first quad
  uint64_t nwtiles = 0;
  uint64_t wtile_cap = 0;
  uint32_t* wbnd = nullptr;     // vertices whose quads span tiles
  uint32_t wbnd_count = 0;
  uint32_t n_alloc = 0;
  uint64_t gen = ~0ull;         // graph generation the lists describe
};

// Vertex order and hub cache of a PageRank pull: every vertex ranked by how
// often its push value is gathered (its degree in the other direction,
// highest first) and a copy of the pulled CSR's column pool holding ranks;
// push values are indexed by rank and the lowest ranks sit in shared memory.
struct HubView {
  uint32_t* rank = nullptr;  // [n] position of each vertex in the pull's vertex
                             // order (degree descending, ties by id)
  uint32_t* col = nullptr;   // [cap] col pool with ids replaced by ranks
  uint32_t k = 0;            // hubs: ranks below k live in shared memory
  uint32_t kmax = 0;         // the cap the set was chosen under
  bool chosen = false;
  uint64_t cap = 0;
  uint64_t gen = ~0ull;      // graph generation the copy reflects
  uint64_t layout = 0;       // in-CSR layout the copy reflects
};

struct DevGraph {
  uint32_t n = 0;
  uint64_t m = 0;  // live edges (host mirror of the device count)
  bool weighted = false;
  bool valid = false;
  DevCSR out, in;
  PullLists in_wl;   // over the in-CSR (PageRank pulls); rebuilt after each update
  PullLists out_wl;  // over the out-CSR (adjoint pulls); built on demand
  HubView hub;       // hub cache of the in-CSR pull; chosen on first use
  HubView hub_out;   // the same for pulls over the out-CSR (the adjoint);
                     // re-encoded in full after a batch
  uint64_t gen = 0;  // bumped whenever the adjacency changes
};

// Normalized update batch kept on the device between apply and IncEval.
struct DevBatch {
  uint64_t cap = 0;
  sg_update* raw = nullptr;     // as uploaded
  uint64_t* key = nullptr;      // scratch keys
  uint64_t* key2 = nullptr;
  uint32_t* val = nullptr;
  uint32_t* val2 = nullptr;
  // normalized actions
  uint32_t* a_src = nullptr;
  uint32_t* a_dst = nullptr;
  float* a_w = nullptr;
  uint32_t* a_kind = nullptr;   // bit0: delete old, bit1: add
  uint32_t* a_found = nullptr;  // out-dir: slot found (kInvalidVid if none)
  uint64_t n_act = 0;
  uint32_t* grp_vertex = nullptr;  // per-vertex groups over actions
  uint32_t* grp_begin = nullptr;
  uint32_t* grp_end = nullptr;
  uint64_t n_grp = 0;
  uint32_t* perm = nullptr;        // action order sorted by (dst, src)
  uint32_t* igrp_vertex = nullptr;
  uint32_t* igrp_begin = nullptr;
  uint32_t* igrp_end = nullptr;
  uint64_t n_igrp = 0;
  uint32_t* a_pos_in = nullptr;    // in-direction slot of each action's pair
  uint32_t* a_tmp = nullptr;       // per-action scratch (hole lists)
  uint32_t* g_d0 = nullptr;        // per group (out: [0,cap), in: [cap,2cap))
  uint32_t* g_ndel = nullptr;
  uint32_t* g_nins = nullptr;
  uint32_t* chunk_off = nullptr;   // work-item prefix per direction
  uint32_t* nch = nullptr;
  uint64_t* d_count = nullptr;     // device scalars
};

struct PrState {
  bool valid = false;
  uint32_t n_alloc = 0;
  float* x = nullptr;      // values_
  float* delta = nullptr;  // deltas_
  float* acc = nullptr;    // push values of the first round (pv0)
  float* pv = nullptr;     // push values d*delta/outdeg of later rounds, 2n (by parity)
  uint32_t* d_misc = nullptr;     // round control words (pagerank.cu M_*)
  double* d_res = nullptr;        // [0] residual accumulator, [1] last residual
  uint64_t* d_cnt = nullptr;      // [0] edges relaxed, [1] vertex visits
};

struct SsspState {
  bool valid = false;
  uint32_t source = 0;
  uint32_t n_alloc = 0;
  unsigned long long* dist = nullptr;  // ordered bits of non-negative doubles
  uint32_t* parent = nullptr;
  uint32_t* stamp = nullptr;      // near-queue de-duplication tags
  uint32_t* fstamp = nullptr;     // far-queue de-duplication epochs
  uint32_t* q[3] = {nullptr, nullptr, nullptr};  // rotating near queues
  uint32_t* far = nullptr;        // two far queues
  uint32_t* far2 = nullptr;
  uint64_t far_cap = 0;
  uint32_t* reset = nullptr;      // reset marks for IncEval
  uint32_t* seeds = nullptr;      // reset seeds found by the applier; the
                                  // reset BFS appends the rest of the list
  uint32_t* seed_cnt = nullptr;   // [0] seeds, [1] BFS level counter
  uint32_t* d_ctl = nullptr;      // control words of the persistent kernel
  unsigned long long* d_cnt = nullptr;
  double* out = nullptr;          // staging for FP64 output
  uint32_t* padd_dst = nullptr;   // heads of edges added since the last run
  uint32_t* padd_src = nullptr;   // their tails and weights
  float* padd_w = nullptr;
  uint32_t pending_batches = 0;   // batches applied since the last run
  uint64_t padd_cap = 0;
  uint64_t padd_bound = 0;        // host upper bound of the pending count
  uint32_t iter_base = 1;         // queue tags grow across launches
  // IncEval: vertices with a changed distance and the parent refresh set
  uint32_t* chg_mark = nullptr;
  uint32_t* chg_list = nullptr;
  uint32_t* par_mark = nullptr;
  uint32_t* par_list = nullptr;
  uint32_t* inc_ctl = nullptr;    // [0..3] reset-BFS barrier / next, [4] changed, [5] refresh
  // rows too long for one warp, deferred to a kernel in which every CTA
  // scans a share of each: the rows, a per-row result and the count
  uint32_t* seed_mark = nullptr;  // re-seed: each head once per IncEval (tag)
  uint32_t seed_tag = 0;
  uint32_t* hv_list = nullptr;
  unsigned long long* hv_best = nullptr;
  uint32_t* hv_cnt = nullptr;
  uint32_t chg_tag = 0;
  bool has_pending = false;       // a batch was applied since the last run
  double delta_width = 0;
};

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
};

}  // namespace sg

struct sg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  sg_options opt{};
  sg::DevGraph g;
  sg::DevBatch batch;
  sg::PrState pr;
  sg::SsspState sp;
  sg_stats stats{};
  std::string err;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t kev0 = nullptr, kev1 = nullptr;
  cudaEvent_t user_ev[8] = {};  // caller-visible timing events on the stream
  // kernel-class profiler: event pairs resolved after the call's final sync
  std::vector<cudaEvent_t> kpool;
  std::vector<int> kclass;
  size_t kused = 0;
  int kopen = -1;
  uint64_t launches = 0;  // kernels launched by the library (all classes)
  uint64_t repacks = 0;   // adjacency pool repacks since the last stats reset
  void* cub_tmp = nullptr;
  size_t cub_tmp_bytes = 0;
  int num_sms = 0;
  void* summary = nullptr;  // summary.cu: summarized graph (compress = 1)
  void* batch_state = nullptr;  // batch.cu: batched PPR / SSSP queries
  void* adjoint_state = nullptr;  // adjoint.cu: weighted PageRank + adjoint
  void* pull_state = nullptr;     // pull.cu: PageRank with message_type = pull
  std::vector<uint64_t> oids;     // io.cpp: vid -> oid when loaded from files (empty: identity)
};

namespace sg {

// status helpers -----------------------------------------------------------
sg_status fail(sg_ctx* ctx, sg_status st, const std::string& msg);
sg_status cuda_fail(sg_ctx* ctx, cudaError_t e, const char* where);

#define SG_CUDA(ctx, call)                                       \
  do {                                                           \
    cudaError_t e_ = (call);                                     \
    if (e_ != cudaSuccess) return ::sg::cuda_fail(ctx, e_, #call); \
  } while (0)

#define SG_TRY(call)                    \
  do {                                  \
    sg_status s_ = (call);              \
    if (s_ != SG_OK) return s_;         \
  } while (0)

// device memory helpers
template <typename T>
sg_status dalloc(sg_ctx* ctx, T** p, uint64_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, SG_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  return SG_OK;
}
template <typename T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

sg_status ensure_cub_tmp(sg_ctx* ctx, size_t bytes);

// kernel-class timing (active when opt.profile != 0)
void kprof_begin(sg_ctx* ctx);
void kprof_end(sg_ctx* ctx, int klass);
void kprof_flush(sg_ctx* ctx);  // after a stream sync: accumulate durations
inline void count_launch(sg_ctx* ctx, uint64_t k = 1) { ctx->launches += k; }

// graph.cu
sg_status graph_free(sg_ctx* ctx);
sg_status graph_build_from_sorted_keys(sg_ctx* ctx, uint32_t n, uint64_t m,
                                       uint64_t* d_keys, float* d_w,
                                       bool weighted);
sg_status graph_rebuild_worklists(sg_ctx* ctx);
// out-CSR work lists for pulls along out-edges (built when stale)
sg_status graph_out_worklists(sg_ctx* ctx);
sg_status graph_in_worklists(sg_ctx* ctx);  // current in-CSR pull lists
void pull_lists_free(PullLists& L);
// packed out-CSR with rows sorted by neighbour (the order of
// sg_graph_download_csr), into caller-owned device arrays
sg_status packed_sorted_out(sg_ctx* ctx, uint64_t* d_rp, uint32_t* d_col);
// divide every edge weight by its source's out-weight sum (both directions)
sg_status normalize_out_weights(sg_ctx* ctx);
sg_status apply_updates_device(sg_ctx* ctx, uint64_t count,
                               const sg_update* upd, bool on_device);

// pagerank.cu
sg_status pr_free(sg_ctx* ctx);
sg_status pr_alloc(sg_ctx* ctx);
sg_status pr_run(sg_ctx* ctx, bool inc);
// failure detection: the persistent kernels' grid barrier, met by a few CTAs
// (skip: one CTA never arrives, the bounded waits run out)
sg_status sssp_barrier_probe(sg_ctx* ctx, int skip);
// after an apply (the generation already bumped): the hub view's copy is
// current again when the applier patched it (patched), else its touched
// in-rows are re-encoded when it was current before the batch
sg_status pr_hub_after_apply(sg_ctx* ctx, const uint32_t* rows, uint64_t nrows, bool patched);
// buffers and direction of one delta-PageRank run (pagerank.cu)
struct PrBufs {
  float* x;
  float* delta;
  float* pv0;      // [n]
  float* pvb;      // [2n]
  uint32_t* misc;  // 8 words
  double* res;     // 4 words
  unsigned long long* cnt;  // 4 words
};
struct PrRunSpec {
  PrBufs buf;
  const PullLists* lists;
  const DevCSR* csr;          // pulled direction
  bool weighted;              // gather push value x edge weight
  const uint32_t* scale_deg;  // push value d*delta/deg[v]; null: d*delta
  double tau;                 // residual test (sum |delta| < tau)
  int kclass;                 // profiler class of the pull kernel
};
sg_status pr_rounds_ex(sg_ctx* ctx, const PrRunSpec& R);
// personalized PageRank of one query: teleport mass (1-d) spread uniformly
// over the seeds (device array), plain rounds to the residual test
sg_status pr_run_personalized(sg_ctx* ctx, const uint32_t* d_seeds, uint32_t n_seeds);
// called by the applier for each affected source vertex group
struct PrAmendArgs {
  float* x;
  float* delta;
  float damping;
  bool active;
};
PrAmendArgs pr_amend_args(sg_ctx* ctx);

// sssp.cu
sg_status sssp_free(sg_ctx* ctx);
sg_status sssp_run_peval(sg_ctx* ctx, uint32_t source);
sg_status sssp_run_inceval(sg_ctx* ctx);
sg_status sssp_compute_parents(sg_ctx* ctx);
struct SsspAmendArgs {
  uint32_t* parent;
  uint32_t* seeds;      // reset seed list (device)
  uint32_t* seed_count; // device counter
  uint32_t* reset;      // reset marks
  bool active;
};
SsspAmendArgs sssp_amend_args(sg_ctx* ctx);
sg_status sssp_collect_adds(sg_ctx* ctx);
sg_status sssp_download(sg_ctx* ctx, double* out);
// delta-stepping over another padded CSR (the summarized graph)
struct SsspView {
  uint32_t n;
  uint64_t m;
  const uint64_t* off;
  const uint32_t* deg;
  const uint32_t* col;
  const float* w;
};
// Queues and tags of a delta-stepping run over a view, held by the caller
// and grown on demand, so repeated runs allocate nothing.
struct SsspViewScratch {
  uint32_t *stamp = nullptr, *fstamp = nullptr, *reset = nullptr;
  uint32_t* q[3] = {nullptr, nullptr, nullptr};
  uint32_t *far = nullptr, *far2 = nullptr, *ctl = nullptr, *sv = nullptr;
  unsigned long long* cnt = nullptr;
  double* sd = nullptr;
  uint64_t n_cap = 0, f_cap = 0, s_cap = 0;
};
void sssp_view_scratch_free(SsspViewScratch& v);
sg_status sssp_run_view(sg_ctx* ctx, const SsspView& G, const uint32_t* h_seeds,
                        const double* h_seed_dist, uint32_t nseeds, unsigned long long* dist,
                        unsigned long long* h_cnt, SsspViewScratch& V);
// prepares ctx->sp for a result written from outside (buffers, no run)
sg_status sssp_prepare_external(sg_ctx* ctx, uint32_t source);
sg_status sssp_finish_external(sg_ctx* ctx, const unsigned long long* h_cnt, float ms);
// IncEval over the summary: the plain reset and re-seed, then the traversal
// over the summary's view from a warm state, then the plain parents.
struct SsspIncInfo {
  uint32_t total = 0;  // reset vertices (s.seeds[0, total))
  uint32_t nadd = 0;   // heads of added edges (s.padd_dst[0, nadd))
  bool one_batch = false;
};
sg_status sssp_inc_prepare(sg_ctx* ctx, SsspIncInfo* info);
sg_status sssp_run_view_warm(sg_ctx* ctx, const SsspView& G, const uint32_t* d_seeds,
                             uint32_t nseeds, unsigned long long* dist, unsigned long long* h_cnt,
                             SsspViewScratch& V);
sg_status sssp_inc_finish_external(sg_ctx* ctx, const SsspIncInfo& info,
                                   const unsigned long long* h_cnt, float ms);

// io.cpp: the reference's text formats
sg_status load_files(sg_ctx* ctx, const char* efile, const char* vfile, bool weighted);
sg_status read_update_file(sg_ctx* ctx, const char* path, std::vector<sg_update>* out);
sg_status read_cluster_file(sg_ctx* ctx, const char* path,
                            std::vector<std::vector<uint32_t>>* clusters);

// adjoint.cu
sg_status adjoint_free(sg_ctx* ctx);
sg_status pr_weighted_forward(sg_ctx* ctx, const float* tele_host, float* x_out);
sg_status pr_adjoint(sg_ctx* ctx, const float* dl_dx, bool on_device, float* dl_dw, float* dl_dt);
sg_status adjoint_info(sg_ctx* ctx, sg_adjoint_info* out);
sg_status adjoint_values(sg_ctx* ctx, float* x, float* lam);

// batch.cu
sg_status batch_free(sg_ctx* ctx);
sg_status batch_run(sg_ctx* ctx, const sg_batch_spec* spec, float* ppr_out, double* sssp_out,
                    bool retune);
sg_status batch_info(sg_ctx* ctx, sg_batch_info* out);
sg_status batch_query_stats(sg_ctx* ctx, int32_t* rounds, double* residual);
sg_status batch_device_outputs(sg_ctx* ctx, const float** ppr, const double** sssp);

// summary.cu
sg_status summary_free(sg_ctx* ctx);
sg_status summary_build(sg_ctx* ctx, const std::vector<std::vector<uint32_t>>& clusters);
sg_status summary_after_apply(sg_ctx* ctx);
sg_status summary_check(sg_ctx* ctx, sg_summary_check* out);
// the reference's serialized cluster state (serialize_cluster layout)
sg_status summary_build_serialized(sg_ctx* ctx, const std::vector<uint8_t>& blob);
sg_status summary_serialized(sg_ctx* ctx, std::vector<uint8_t>* blob);
sg_status pr_summarized(sg_ctx* ctx, bool inc);

// SumSyncIterWorkerPull's in-indexes over the summary, on the device (built
// on first use after each summary change).  Vertex classes: 0 out node, 1
// exit only, 2 entry only, 3 entry and exit, 4 inner member.
// A summary's supernode lists on the device (the repair's slot layout):
// supernode row r keeps its shortcuts to exits (is), to inner members'
// values (inner_value) and deltas (inner_delta) at slot[r], with a count per
// row; row_sp marks supernode rows and row_inner holds their clusters'
// member counts.
struct SpLists {
  const uint64_t* slot = nullptr;
  const uint8_t* row_sp = nullptr;
  const uint32_t* row_inner = nullptr;
  const uint32_t *is_cnt = nullptr, *iv_cnt = nullptr, *id_cnt = nullptr;
  const uint32_t *is_nbr = nullptr, *iv_nbr = nullptr, *id_nbr = nullptr;
  const float *is_w = nullptr, *iv_w = nullptr, *id_w = nullptr;
  uint64_t pool = 0;  // entries of the slot arrays in use
  const uint32_t* sp_rows = nullptr;  // the supernode rows, in row order
  uint32_t n_sp = 0;
};

struct PullView {
  uint32_t n = 0;
  const uint8_t* cls = nullptr;
  const uint32_t* act = nullptr;     // vertices of classes 0-3 (the rounds' rows),
  uint32_t n_act = 0;                // those with more than 32 row entries first
  uint32_t n_long = 0;
  const uint32_t* ent = nullptr;     // vertices of classes 2-3 (the entries)
  uint32_t n_ent = 0;
  const uint64_t* ie_off = nullptr;  // per vertex: in-edges from other clusters (2, 3)
  const uint32_t* ie_nbr = nullptr;
  const uint64_t* bd_off = nullptr;  // per vertex: bound_delta shortcuts ending here (1, 3)
  const uint32_t* bd_src = nullptr;  // (the supernode's entry)
  const float* bd_w = nullptr;
  // the correction scatters each entry's supernode lists
  SpLists L;
  uint64_t round_edges = 0;      // entries one summarized round reads
  uint64_t round_shortcuts = 0;  // of which shortcut entries
  uint64_t corr_entries = 0;
};
sg_status summary_pull_view(sg_ctx* ctx, PullView* out);

// pull.cu: PageRank with message_type = pull
sg_status pr_pull_worker(sg_ctx* ctx, bool inc);
sg_status pull_free(sg_ctx* ctx);
sg_status sssp_summarized(sg_ctx* ctx, uint32_t source);
sg_status sssp_summarized_inc(sg_ctx* ctx);
bool summary_no_supernodes(sg_ctx* ctx);
bool sssp_summary_ready(sg_ctx* ctx);
uint32_t summary_rows(sg_ctx* ctx);  // rows incl. mirrors, 0 without a summary
sg_status summary_info(sg_ctx* ctx, sg_summary_info* out);

// graph.cu entry points behind the C ABI
sg_status generate_rmat(sg_ctx* ctx, int scale, uint64_t edges, double a, double b,
                        double c, uint64_t seed, int wkind, double wlo, double whi);
sg_status load_csr(sg_ctx* ctx, uint32_t n, const uint64_t* row_ptr,
                   const uint32_t* col, const float* w);
sg_status download_csr(sg_ctx* ctx, uint64_t* row_ptr, uint32_t* col, float* w);

}  // namespace sg
