// Incremental repair of the summarized graph's PageRank tables on the device,
// after each batch: the reference's inc_run (inc_compress_mirror,
// compressor_base.h:5634-5803; judge_out_bound_node, :3924-3956;
// build_subgraph_mirror's incremental form, :3859-3922; the shortcut rebuild
// of the touched supernodes, iter_compressor.h:796-896; get_nodetype_mirror,
// :4144-4182; sketch2csr_mirror, :4636-4880).
//
// Cluster membership, mirrors and the sync edges stay as the construction
// left them.  What a batch changes:
//   entries    a deleted edge from outside the cluster retires an entry whose
//              other in-edges all come from its cluster or from in-mirror
//              masters of its cluster; an added edge from outside (not from
//              an in-mirror master) makes a member an entry.  Both rules give
//              the same result in any order over the batch, so a warp per
//              action decides them.
//   exits      members of updated clusters with an out-edge that leaves the
//              cluster other than to one of its out-mirrors become exits, and
//              in-mirror masters of updated clusters stay exits; exit marks are
//              only ever set.
//   shortcuts  every supernode (entry or in-mirror) of a cluster with a
//              changed source vertex, the in-mirrors of changed source
//              vertices and the new entries are solved again on their cluster
//              from the current graph; the others keep their solve.
//   tables     node types, the entry / exit / single lists, the is and ib
//              CSRs, the correction lists and the cluster-precompute lists are
//              rebuilt from that state in count / scan / fill passes.
// A supernode's solve is a dense block: the value and the residual delta of
// every node of its cluster, in the cluster's node order (members, then
// in-mirrors, then out-mirrors).  Blocks sit in a pool in row order and move
// to a fresh layout after each batch.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cstring>

#include "ctx.h"
#include "dev.cuh"
#include "summary.h"
#include "summary_dev.h"

namespace sg {

namespace {
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint64_t kNoSlot = ~0ull;  // a row without a block
}

struct RepairDev {
  uint32_t n = 0, all_n = 0, ncl = 0;
  uint32_t max_L = 0;           // largest cluster node list
  // fixed after the construction
  uint32_t* cl_of = nullptr;    // [all_n] cluster of each vertex / mirror
  uint32_t* loc = nullptr;      // [all_n] index in its cluster's node list
  uint64_t* cn_off = nullptr;   // [ncl + 1]
  uint32_t* cn = nullptr;       // cluster nodes: members, in-mirrors, out-mirrors
  uint32_t* inner = nullptr;    // [ncl] members
  uint32_t* n_im = nullptr;     // [ncl] in-mirrors
  uint32_t* master = nullptr;   // [all_n - n] master of each mirror
  uint64_t* vim_off = nullptr;  // [n + 1] in-mirrors of each master, by cluster
  uint32_t* vim = nullptr;
  uint64_t* vom_off = nullptr;  // [n + 1] out-mirrors of each master, by cluster
  uint32_t* vom = nullptr;
  // repaired state
  int32_t* fc = nullptr;        // [n] >= 0: entry of that cluster; < 0: member
  uint8_t* ob = nullptr;        // [n] exit marks
  // marks of one batch (cleared at its end) and of the IncEval to come
  uint8_t *m_src = nullptr, *m_ret = nullptr, *m_new = nullptr;          // [n]
  uint8_t *c_src = nullptr, *c_upd = nullptr, *c_job = nullptr;          // [ncl]
  uint8_t* c_pend = nullptr;                                             // [ncl]
  uint8_t* r_job = nullptr;                                              // [all_n]
  uint8_t* f_sp = nullptr;                                               // [all_n]
  uint32_t* sp_rows = nullptr;                                           // [all_n]
  uint32_t n_sp = 0;
  uint8_t *f_entry = nullptr, *f_exit = nullptr, *f_single = nullptr;    // [n]
  uint64_t* r_size = nullptr;                                            // [all_n + 1]
  // shortcut blocks: row offsets [all_n + 1] and pools (current, next)
  struct Pool {
    double* val = nullptr;  // value of each node of the cluster
    double* del = nullptr;  // residual delta of each node
    // the row's lists (at most a cluster's node count each): shortcuts to
    // exits and out-mirrors, inner values, inner deltas
    uint32_t *is_nbr = nullptr, *iv_nbr = nullptr, *id_nbr = nullptr;
    float *is_w = nullptr, *iv_w = nullptr, *id_w = nullptr;
    uint64_t cap = 0;
  };
  uint64_t *blk = nullptr, *blk2 = nullptr;
  Pool pool, pool2;
  uint64_t pool_used = 0;       // slots handed out (the pool tail)
  uint64_t live_at_layout = 0;  // live entries at the last new layout
  uint64_t relayouts = 0;
  unsigned long long* d_tail = nullptr;  // device copy of the pool tail
  uint32_t *is_cnt = nullptr, *iv_cnt = nullptr, *id_cnt = nullptr;  // [all_n] list lengths
  uint32_t* row_inner = nullptr;  // [all_n] members of the row's cluster
  uint64_t n_members = 0;       // members over all clusters (cm layout positions)
  // SSSP over the summary (after its first query): distance blocks in the
  // layout of the PageRank blocks, the weights of the ib rows, and whether
  // the summarized CSR needs a rebuild
  bool sssp_on = false, sk_stale = true;
  double *sd = nullptr, *sd2 = nullptr;
  uint64_t sd_cap = 0, sd2_cap = 0;
  float* ib_w = nullptr;
  uint64_t ib_w_cap = 0;
  uint8_t* f_corr = nullptr;       // [all_n] rows with correction entries
  uint32_t *im_list = nullptr, *im_master = nullptr;  // every in-mirror and its master
  uint32_t n_im_total = 0;
  double* src_dist = nullptr;      // the source cluster's local distances
  uint32_t *seed_v = nullptr, *seed_n = nullptr;
  double* seed_d = nullptr;
  // scratch of the passes (grown on demand)
  uint32_t *jobs = nullptr, *tcl = nullptr, *tc_idx = nullptr, *tc_inner = nullptr;
  uint32_t *sp_cl = nullptr, *sp_src = nullptr;
  uint32_t *wjobs = nullptr, *wjobs5 = nullptr, *bjobs = nullptr, *hjobs = nullptr;
  uint8_t *j_warp = nullptr, *j_warp5 = nullptr, *j_block = nullptr, *j_half = nullptr;
  uint64_t *lp_off = nullptr, *adj_off = nullptr, *out_off = nullptr, *lin_off = nullptr;
  uint64_t* cl_lin = nullptr;
  uint32_t* adj_nbr = nullptr;
  float* adj_w = nullptr;
  uint64_t cap_adjw = 0;
  uint8_t* lin_src = nullptr;
  float* div = nullptr;
  uint64_t *cnt_a = nullptr, *cnt_b = nullptr, *cnt_c = nullptr, *cnt_d = nullptr;
  uint64_t *o_lin = nullptr, *o_lout = nullptr, *o_sub = nullptr;  // [ncl + 1]
  // the cluster-precompute lists' next build (the summary holds the current)
  struct CmCaps {
    uint64_t bl_off = 0, bound_list = 0, lin_off = 0, lin_src = 0, lout_off = 0, lout_dst = 0,
             sub_off = 0, sub_nbr = 0;
  };
  struct CmBuf {
    uint64_t *bl_off = nullptr, *lin_off = nullptr, *lout_off = nullptr, *sub_off = nullptr;
    uint32_t *bound_list = nullptr, *lout_dst = nullptr, *sub_nbr = nullptr;
    uint8_t* lin_src = nullptr;
    CmCaps cap;
  };
  CmBuf nx;
  CmCaps cur;          // capacities of the summary's current arrays (0: unknown)
  bool cm_built = false;
  // the shortcut solves run on a stream of their own, below the context
  // stream's priority, while the tables are rebuilt on the context stream
  cudaStream_t side = nullptr;
  cudaEvent_t ev_ready = nullptr, ev_solved = nullptr;
  uint32_t n_jobs = 0;      // rows solved again by the batch
  bool solving = false;     // solves launched and not joined yet
  uint32_t* d_num = nullptr;    // selected counts
  uint32_t* d_err = nullptr;
  uint64_t cap_lp = 0, cap_div = 0, cap_linoff = 0, cap_cntd = 0, cap_adj = 0, cap_lin = 0;
  // actions of the batches the host restatement has not seen yet
  uint32_t *log_src = nullptr, *log_dst = nullptr, *log_kind = nullptr, *log_found = nullptr;
  float* log_w = nullptr;
  uint64_t log_n = 0, log_cap = 0;
  std::vector<uint64_t> log_end;  // end of each batch in the log
};

namespace {

template <typename T>
sg_status grow(sg_ctx* ctx, T** p, uint64_t* cap, uint64_t need) {
  if (need <= *cap && *p) return SG_OK;
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(*p);
  const uint64_t c = std::max<uint64_t>(need + need / 8, 64);
  SG_TRY(dalloc(ctx, p, c));
  *cap = c;
  return SG_OK;
}

// a device table of SummaryDev, kept while large enough (capacities shared
// with the host uploads of summary.cu)
template <typename T>
sg_status reserve(sg_ctx* ctx, SummaryDev& D, T** d, uint64_t need) {
  need = std::max<uint64_t>(need, 1);
  auto it = D.dcap.find((const void*)d);
  if (*d && it != D.dcap.end() && it->second >= need) return SG_OK;
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(*d);
  const uint64_t cap = need + need / 8;
  SG_TRY(dalloc(ctx, d, cap));
  D.dcap[(const void*)d] = cap;
  return SG_OK;
}

template <typename T, typename A>
sg_status put(sg_ctx* ctx, T** d, const std::vector<T, A>& h) {
  dfree(*d);
  SG_TRY(dalloc(ctx, d, std::max<size_t>(h.size(), 1)));
  if (!h.empty())
    SG_CUDA(ctx, cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
  return SG_OK;
}

// exclusive prefix over n + 1 entries (the last input entry is ignored and
// the last output is the total)
sg_status scan_u64(sg_ctx* ctx, const uint64_t* in, uint64_t* out, uint64_t n1) {
  size_t bytes = 0;
  SG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int64_t)n1, ctx->stream));
  SG_TRY(ensure_cub_tmp(ctx, bytes));
  bytes = ctx->cub_tmp_bytes;
  SG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(ctx->cub_tmp, bytes, in, out, (int64_t)n1, ctx->stream));
  count_launch(ctx);
  return SG_OK;
}

// indices i < n with flag[i] != 0, in increasing order; the count lands in
// *d_num (device)
sg_status select_idx(sg_ctx* ctx, const uint8_t* flag, uint32_t* out, uint32_t* d_num, uint64_t n) {
  thrust::counting_iterator<uint32_t> it(0);
  size_t bytes = 0;
  SG_CUDA(ctx, cub::DeviceSelect::Flagged(nullptr, bytes, it, flag, out, d_num, (int64_t)n,
                                          ctx->stream));
  SG_TRY(ensure_cub_tmp(ctx, bytes));
  bytes = ctx->cub_tmp_bytes;
  SG_CUDA(ctx, cub::DeviceSelect::Flagged(ctx->cub_tmp, bytes, it, flag, out, d_num, (int64_t)n,
                                          ctx->stream));
  count_launch(ctx);
  return SG_OK;
}

sg_status read_u64(sg_ctx* ctx, const uint64_t* d, uint64_t* h) {
  SG_CUDA(ctx, cudaMemcpyAsync(h, d, 8, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

// ------------------------------------------------------------- kernels

struct RepArgs {
  uint32_t n, all_n, ncl;
  const uint32_t *cl_of, *loc, *cn, *inner, *n_im, *master;
  const uint64_t *cn_off, *vim_off, *vom_off;
  const uint32_t *vim, *vom;
  int32_t* fc;
  uint8_t* ob;
  uint8_t *m_src, *m_ret, *m_new, *c_src, *c_upd, *c_job, *c_pend, *r_job;
  uint32_t *is_cnt, *iv_cnt, *id_cnt;
  uint64_t* slot;  // block of each row (kNoSlot: none)
  const uint64_t *out_off, *in_off;  // the graph's two directions (live prefix of each row)
  const uint32_t *out_deg, *in_deg, *out_col, *in_col;
  const float* out_w;                // edge weights (null: unweighted)
};

__device__ __forceinline__ uint32_t cl_size(const RepArgs& R, uint32_t c) {
  return (uint32_t)(R.cn_off[c + 1] - R.cn_off[c]);
}

// the mirror of master x in cluster c from a list sorted by cluster
__device__ __forceinline__ uint32_t mirror_in(const RepArgs& R, const uint64_t* off,
                                              const uint32_t* list, uint32_t c, uint32_t x) {
  if (x >= R.n || c == kNone) return kNone;
  uint64_t lo = off[x], hi = off[x + 1];
  const uint64_t end = hi;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (R.cl_of[list[mid]] < c) lo = mid + 1; else hi = mid;
  }
  return lo < end && R.cl_of[list[lo]] == c ? list[lo] : kNone;
}
// x is the master of an in-mirror of cluster c
__device__ __forceinline__ bool im_of(const RepArgs& R, uint32_t c, uint32_t x) {
  return mirror_in(R, R.vim_off, R.vim, c, x) != kNone;
}
// the out-mirror of x in cluster c (kNone if none)
__device__ __forceinline__ uint32_t om_of(const RepArgs& R, uint32_t c, uint32_t x) {
  return mirror_in(R, R.vom_off, R.vom, c, x);
}

__device__ __forceinline__ bool is_sp_row(const RepArgs& R, uint32_t r, uint32_t c) {
  if (c == kNone) return false;
  return r < R.n ? R.fc[r] >= 0 : R.loc[r] < R.inner[c] + R.n_im[c];
}

// 1. per action (warp): touched sources, updated clusters, retire / new
//    entry candidates (fc is the state before the batch)
__global__ void __launch_bounds__(256) k_rp_actions(RepArgs R, const uint32_t* a_src,
                                                    const uint32_t* a_dst, const uint32_t* a_kind,
                                                    const uint32_t* a_found, uint64_t na) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < na; i += nw) {
    const uint32_t kind = a_kind[i];
    const bool found = a_found[i] != kInvalidVid;
    const bool del = (kind & 1u) && found, add = (kind & 2u) != 0;
    if (!del && !add) continue;
    const uint32_t u = a_src[i], v = a_dst[i];
    const uint32_t cu = R.cl_of[u], cv = R.cl_of[v];
    if (lane == 0 && cu != kNone) {
      R.m_src[u] = 1;
      R.c_src[cu] = 1;
      R.c_upd[cu] = 1;
    }
    if (cv == kNone) continue;
    if (del && R.fc[v] >= 0) {
      if (lane == 0) R.c_upd[cv] = 1;
      if (cv != cu) {
        bool outside = false;
        const uint64_t b = R.in_off[v];
        const uint32_t d = R.in_deg[v];
        for (uint32_t k0 = 0; k0 < d && !outside; k0 += 32) {
          bool hit = false;
          if (k0 + lane < d) {
            const uint32_t x = R.in_col[b + k0 + lane];
            hit = x != u && R.cl_of[x] != cv && !im_of(R, cv, x);
          }
          outside = __any_sync(0xffffffffu, hit);
        }
        if (!outside && lane == 0) R.m_ret[v] = 1;
      }
    }
    if (add && lane == 0) {
      R.c_upd[cv] = 1;
      if (cu != cv && !im_of(R, cv, u)) R.m_new[v] = 1;
    }
  }
}

// 2. per vertex: entry changes; in-mirrors of touched sources
__global__ void k_rp_entries(RepArgs R) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < R.n; v += gridDim.x * blockDim.x) {
    if (R.m_src[v]) {
      R.m_src[v] = 0;
      for (uint64_t k = R.vim_off[v]; k < R.vim_off[v + 1]; ++k) {
        const uint32_t m = R.vim[k];
        R.r_job[m] = 1;
        R.c_upd[R.cl_of[m]] = 1;
      }
    }
    const uint8_t ret = R.m_ret[v], nw = R.m_new[v];
    if (ret | nw) {
      const uint32_t c = R.cl_of[v];
      int32_t f = R.fc[v];
      if (ret && f >= 0) f = -(int32_t)(c + 1);
      if (nw && f < 0) {
        f = (int32_t)c;
        R.r_job[v] = 1;
      }
      R.fc[v] = f;
      R.m_ret[v] = 0;
      R.m_new[v] = 0;
    }
  }
}

// 3. per row: supernode rows and their block sizes, the solves to redo,
//    exits of updated clusters, out-degrees of all rows
__global__ void k_rp_rows(RepArgs R, uint64_t* r_size, uint8_t* f_sp, uint32_t* out_deg_all) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < R.all_n; r += gridDim.x * blockDim.x) {
    const uint32_t c = R.cl_of[r];
    const bool sp = is_sp_row(R, r, c);
    uint64_t size = 0;
    if (sp) {
      size = cl_size(R, c);
      if (R.c_src[c]) R.r_job[r] = 1;
    } else {
      R.r_job[r] = 0;
      R.is_cnt[r] = R.iv_cnt[r] = R.id_cnt[r] = 0;
      R.slot[r] = kNoSlot;  // a retired supernode's block becomes a hole
    }
    if (c != kNone && R.c_upd[c]) {
      if (r < R.n) {
        if (!R.ob[r]) {
          const uint64_t b = R.out_off[r];
          const uint32_t d = R.out_deg[r];
          for (uint32_t k = 0; k < d; ++k) {
            const uint32_t x = R.out_col[b + k];
            if (R.cl_of[x] != c && om_of(R, c, x) == kNone) {
              R.ob[r] = 1;
              break;
            }
          }
        }
      } else if (sp) {
        R.ob[R.master[r - R.n]] = 1;
      }
    }
    r_size[r] = size;
    f_sp[r] = sp;
    out_deg_all[r] = R.out_deg[r < R.n ? r : R.master[r - R.n]];
  }
}

// 4. per vertex: node type (get_nodetype_mirror) and list flags
__global__ void k_rp_types(RepArgs R, uint8_t* ntype, uint8_t* f_entry, uint8_t* f_exit,
                           uint8_t* f_single) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < R.n; v += gridDim.x * blockDim.x) {
    const int32_t f = R.fc[v];  // Summary::kFcDefault for unclustered vertices
    const bool ob = R.ob[v] != 0;
    uint8_t t = 127;
    if (f == Summary::kFcDefault) t = kSingle;
    else if (f >= 0) t = kOnlyIn;
    else if (!ob) t = kInner;
    if (ob) t = f >= 0 ? kBothOutIn : kOnlyOut;
    if (R.vim_off[v + 1] > R.vim_off[v]) {
      if (t == kOnlyOut) t = kOutMaster;
      else if (t == kBothOutIn) t = kBothOutInMaster;
    }
    ntype[v] = t;
    f_entry[v] = t == kOnlyIn || t == kBothOutIn || t == kBothOutInMaster;
    f_exit[v] = t == kOnlyOut || t == kBothOutIn || t == kOutMaster || t == kBothOutInMaster;
    f_single[v] = t == kSingle;
  }
}

// 5. per job row: its cluster marked for a local problem
__global__ void k_rp_job_clusters(RepArgs R, const uint32_t* jobs, uint32_t nj) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nj; j += gridDim.x * blockDim.x)
    R.c_job[R.cl_of[jobs[j]]] = 1;
}

// 6. per touched cluster: its index and node count
__global__ void k_rp_tcl(RepArgs R, const uint32_t* tcl, uint32_t ntc, uint32_t* tc_idx,
                         uint32_t* tc_inner, uint64_t* lp_size) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ntc; k += gridDim.x * blockDim.x) {
    const uint32_t c = tcl[k];
    tc_idx[c] = k;
    tc_inner[k] = R.inner[c];
    lp_size[k] = cl_size(R, c);
  }
}

// local out-edges of node i of cluster c: a member's edges to members and,
// redirected, to the cluster's out-mirrors (unless the member is an
// in-mirror master of the target's cluster); an in-mirror's master's edges
// into the cluster; none for out-mirrors (build_subgraph_mirror)
template <bool FILL>
__device__ __forceinline__ uint32_t local_edges(const RepArgs& R, uint32_t c, uint32_t i,
                                                uint32_t* out, float* wout = nullptr) {
  const uint32_t inner = R.inner[c];
  const uint32_t node = R.cn[R.cn_off[c] + i];
  uint32_t k = 0;
  if (i < inner) {
    const uint64_t b = R.out_off[node];
    const uint32_t d = R.out_deg[node];
    for (uint32_t e = 0; e < d; ++e) {
      const uint32_t t = R.out_col[b + e];
      const uint32_t ct = R.cl_of[t];
      uint32_t l = kNone;
      if (ct == c) {
        l = R.loc[t];
      } else {
        const uint32_t m = om_of(R, c, t);
        if (m != kNone && !im_of(R, ct, node)) l = R.loc[m];
      }
      if (l != kNone) {
        if (FILL) {
          out[k] = l;
          if (wout) wout[k] = R.out_w[b + e];
        }
        ++k;
      }
    }
  } else if (i < inner + R.n_im[c]) {
    const uint32_t u = R.master[node - R.n];
    const uint64_t b = R.out_off[u];
    const uint32_t d = R.out_deg[u];
    for (uint32_t e = 0; e < d; ++e) {
      const uint32_t t = R.out_col[b + e];
      if (R.cl_of[t] == c) {
        if (FILL) {
          out[k] = R.loc[t];
          if (wout) wout[k] = R.out_w[b + e];
        }
        ++k;
      }
    }
  }
  return k;
}

// 7. per touched cluster (warp): local edge counts per node
__global__ void __launch_bounds__(256) k_rp_lp_count(RepArgs R, const uint32_t* tcl, uint32_t ntc,
                                                     const uint64_t* lp_off, uint64_t* cnt) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < ntc; k += nw) {
    const uint32_t c = tcl[k];
    const uint32_t L = cl_size(R, c);
    for (uint32_t i = lane; i < L; i += 32) cnt[lp_off[k] + i] = local_edges<false>(R, c, i, nullptr);
  }
}

// 8. per touched cluster (warp): local edges and divisors
__global__ void __launch_bounds__(256) k_rp_lp_fill(RepArgs R, const uint32_t* tcl, uint32_t ntc,
                                                    const uint64_t* lp_off, const uint64_t* adj_off,
                                                    uint32_t* adj_nbr, float* adj_w, float* div) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < ntc; k += nw) {
    const uint32_t c = tcl[k];
    const uint32_t L = cl_size(R, c);
    for (uint32_t i = lane; i < L; i += 32) {
      const uint64_t p = lp_off[k] + i;
      local_edges<true>(R, c, i, adj_nbr + adj_off[p], adj_w ? adj_w + adj_off[p] : nullptr);
      const uint32_t node = R.cn[R.cn_off[c] + i];
      const uint32_t mst = node < R.n ? node : R.master[node - R.n];
      div[p] = (float)max(R.out_deg[mst], 1u);
    }
  }
}

// 9. per touched cluster: member-to-node edge count of clusters the warp
//    kernel stages (at most kStageCap nodes)
__global__ void k_rp_lin_count(RepArgs R, const uint32_t* tcl, uint32_t ntc, const uint64_t* lp_off,
                               const uint64_t* adj_off, uint64_t* cnt) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ntc; k += gridDim.x * blockDim.x) {
    const uint32_t c = tcl[k];
    const uint32_t L = cl_size(R, c);
    cnt[k] = L <= (uint32_t)kStageCap ? adj_off[lp_off[k] + R.inner[c]] - adj_off[lp_off[k]] : 0;
  }
}

// 10. per staged touched cluster (warp): in-edges from members per node,
//     tails as 8-bit local indices (counting sort in shared memory)
__global__ void __launch_bounds__(256) k_rp_lin_fill(RepArgs R, const uint32_t* tcl, uint32_t ntc,
                                                     const uint64_t* lp_off, const uint64_t* adj_off,
                                                     const uint32_t* adj_nbr, const uint64_t* cl_lin,
                                                     uint64_t* lin_off, uint8_t* lin_src) {
  __shared__ uint32_t s_cnt[kStageWarps][kStageCap + 1];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < ntc; k += nw) {
    const uint32_t c = tcl[k];
    const uint32_t L = cl_size(R, c);
    const uint64_t p0 = lp_off[k];
    if (L > (uint32_t)kStageCap) {
      for (uint32_t j = lane; j < L; j += 32) lin_off[p0 + j] = cl_lin[k];
      continue;
    }
    const uint32_t inner = R.inner[c];
    uint32_t* cnt = s_cnt[w];
    for (uint32_t j = lane; j <= L; j += 32) cnt[j] = 0;
    __syncwarp();
    for (uint32_t i = lane; i < inner; i += 32)
      for (uint64_t e = adj_off[p0 + i]; e < adj_off[p0 + i + 1]; ++e) atomicAdd(&cnt[adj_nbr[e] + 1], 1u);
    __syncwarp();
    if (lane == 0)
      for (uint32_t j = 0; j < L; ++j) cnt[j + 1] += cnt[j];
    __syncwarp();
    for (uint32_t j = lane; j < L; j += 32) lin_off[p0 + j] = cl_lin[k] + cnt[j];
    __syncwarp();
    for (uint32_t i = lane; i < inner; i += 32)
      for (uint64_t e = adj_off[p0 + i]; e < adj_off[p0 + i + 1]; ++e)
        lin_src[cl_lin[k] + atomicAdd(&cnt[adj_nbr[e]], 1u)] = (uint8_t)i;
    __syncwarp();
  }
}

// 11. per job: cluster index, local source, output offset, kernel choice
__global__ void k_rp_jobs(RepArgs R, const uint32_t* jobs, uint32_t nj, const uint32_t* tc_idx,
                          const uint64_t* blk, uint32_t* sp_cl, uint32_t* sp_src, uint64_t* out_off,
                          uint8_t* j_half, uint8_t* j_warp, uint8_t* j_warp5, uint8_t* j_block) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nj; j += gridDim.x * blockDim.x) {
    const uint32_t r = jobs[j];
    const uint32_t c = R.cl_of[r];
    sp_cl[j] = tc_idx[c];
    sp_src[j] = R.loc[r];
    out_off[j] = blk[r];
    const uint32_t L = cl_size(R, c);
    j_half[j] = L <= kShortcutHalfL;
    j_warp[j] = L > kShortcutHalfL && L <= kShortcutSmallL;
    j_warp5[j] = L > kShortcutSmallL && L <= (uint32_t)kStageCap;
    j_block[j] = L > (uint32_t)kStageCap;
  }
}

// 12. per supernode row (warp): blocks (and lists) of rows whose solve stays
//     move to the new layout
struct MoveArgs {
  const uint64_t *blk, *blk2;
  const double *val, *del;
  double *val2, *del2;
  const uint32_t *is_nbr, *iv_nbr, *id_nbr;  // null: blocks only
  const float *is_w, *iv_w, *id_w;
  uint32_t *is_nbr2, *iv_nbr2, *id_nbr2;
  float *is_w2, *iv_w2, *id_w2;
};

__global__ void __launch_bounds__(256) k_rp_move(RepArgs R, const uint32_t* sp_rows, uint32_t nsp,
                                                 const uint64_t* r_size, MoveArgs M, uint32_t* err) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nsp; k += nw) {
    const uint32_t r = sp_rows[k];
    const uint64_t L = r_size[r];
    if (L == 0 || R.r_job[r]) continue;
    const uint64_t s = M.blk[r], t = M.blk2[r];
    if (s == kNoSlot) {  // a kept supernode without a block
      if (lane == 0) atomicExch(err, 1u);
      continue;
    }
    for (uint64_t i = lane; i < L; i += 32) {
      M.val2[t + i] = M.val[s + i];
      M.del2[t + i] = M.del[s + i];
    }
    if (!M.is_nbr) continue;
    for (uint32_t i = lane; i < R.is_cnt[r]; i += 32) {
      M.is_nbr2[t + i] = M.is_nbr[s + i];
      M.is_w2[t + i] = M.is_w[s + i];
    }
    for (uint32_t i = lane; i < R.iv_cnt[r]; i += 32) {
      M.iv_nbr2[t + i] = M.iv_nbr[s + i];
      M.iv_w2[t + i] = M.iv_w[s + i];
    }
    for (uint32_t i = lane; i < R.id_cnt[r]; i += 32) {
      M.id_nbr2[t + i] = M.id_nbr[s + i];
      M.id_w2[t + i] = M.id_w[s + i];
    }
  }
}

// SSSP over the summary.  Rows of the summarized CSR (sketch2csr's traversal
// form): a master's 0-weight edges to its in-mirrors (clusters in order),
// then a supernode row's bound shortcuts (exits, and out-mirrors as their
// masters, at their local distance), then a row's boundary edges; rows are
// padded to quads.  Correction entries: a supernode's inner members at a
// finite distance.
struct SkArgs {
  const uint64_t* blk;
  const double* sd;
  const uint64_t* ib_off;
  const uint32_t* ib_nbr;
  const float* ib_w;
  uint32_t* deg;      // count pass
  uint64_t* pad;
  uint64_t* ccnt;
  uint8_t* fcorr;
  const uint64_t* off;  // fill pass
  uint32_t* col;
  float* w;
  const uint64_t* coff;
  uint32_t* cv;
  float* cd;
};

template <bool FILL>
__global__ void k_rp_sketch(RepArgs R, SkArgs K) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < R.all_n; r += gridDim.x * blockDim.x) {
    uint64_t k = FILL ? K.off[r] : 0, kc = FILL ? K.coff[r] : 0;
    uint32_t ne = 0, nc = 0;
    if (r < R.n)
      for (uint64_t q = R.vim_off[r]; q < R.vim_off[r + 1]; ++q, ++ne)
        if (FILL) {
          K.col[k] = R.vim[q];
          K.w[k++] = 0.f;
        }
    const uint32_t c = R.cl_of[r];
    if (is_sp_row(R, r, c)) {
      const uint32_t L = cl_size(R, c), inner = R.inner[c], om0 = inner + R.n_im[c];
      const uint64_t b = K.blk[r], n0 = R.cn_off[c];
      for (uint32_t i = 0; i < L; ++i) {
        const double d = K.sd[b + i];
        if (!isfinite(d)) continue;  // unreached inside the cluster
        const uint32_t node = R.cn[n0 + i];
        if (i < inner && !R.ob[node]) {
          if (FILL) {
            K.cv[kc] = node;
            K.cd[kc++] = (float)d;
          }
          ++nc;
        } else if (i < inner || i >= om0) {
          if (FILL) {
            K.col[k] = i < inner ? node : R.master[node - R.n];
            K.w[k++] = (float)d;
          }
          ++ne;
        }
      }
    }
    if (r < R.n)
      for (uint64_t e = K.ib_off[r]; e < K.ib_off[r + 1]; ++e, ++ne)
        if (FILL) {
          K.col[k] = K.ib_nbr[e];
          K.w[k++] = K.ib_w ? K.ib_w[e] : 1.f;
        }
    if (!FILL) {
      K.deg[r] = ne;
      K.pad[r] = (ne + 3u) & ~3u;
      K.ccnt[r] = nc;
      K.fcorr[r] = nc != 0;
    }
  }
}

__global__ void k_rp_gather_off(const uint32_t* rows, uint32_t nrows, const uint64_t* off_row,
                                uint64_t total, uint64_t* out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= nrows; k += gridDim.x * blockDim.x)
    out[k] = k < nrows ? off_row[rows[k]] : total;
}

// seeds of the source's cluster from its local distances
__global__ void k_rp_seeds(RepArgs R, uint32_t c, const double* dist, uint32_t* sv, double* sdist,
                           uint32_t* count) {
  const uint32_t L = cl_size(R, c), inner = R.inner[c], om0 = inner + R.n_im[c];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
    const double d = dist[i];
    if (!isfinite(d)) continue;
    if (i >= inner && i < om0) continue;  // in-mirrors do not seed
    const uint32_t node = R.cn[R.cn_off[c] + i];
    const uint32_t p = atomicAdd(count, 1u);
    sv[p] = i < inner ? node : R.master[node - R.n];
    sdist[p] = d;
  }
}

// slots for supernode rows that have none (new entries): at the pool tail
__global__ void k_rp_alloc(const uint32_t* jobs, uint32_t nj, const uint64_t* r_size, uint64_t* blk,
                           unsigned long long* tail) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nj; j += gridDim.x * blockDim.x) {
    const uint32_t r = jobs[j];
    if (blk[r] == kNoSlot) blk[r] = atomicAdd(tail, (unsigned long long)r_size[r]);
  }
}

// after a re-layout: rows without a block have no slot
__global__ void k_rp_unslot(const uint8_t* f_sp, uint32_t all_n, uint64_t* blk) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < all_n; r += gridDim.x * blockDim.x)
    if (!f_sp[r]) blk[r] = kNoSlot;
}

// A supernode's lists (fianl_build_iter_index_for_mirror,
// iter_compressor.h:433-491), written into its slot: members with a value go
// to bound_delta (exits) or inner_value (the rest), members with a residual
// delta to inner_delta, out-mirrors with value + delta to bound_delta.  A
// warp per row solved again (the other rows' lists moved with their blocks).
__global__ void __launch_bounds__(256) k_rp_lists(RepArgs R, const uint32_t* rows, uint32_t nrows,
                                                  const uint64_t* blk, RepairDev::Pool Q) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nrows; k += nw) {
    const uint32_t r = rows[k];
    const uint32_t c = R.cl_of[r];
    const uint32_t L = cl_size(R, c), inner = R.inner[c], om0 = inner + R.n_im[c];
    const uint64_t b = blk[r], n0 = R.cn_off[c];
    uint32_t nis = 0, niv = 0, nid = 0;
    for (uint32_t i0 = 0; i0 < L; i0 += 32) {
      const uint32_t i = i0 + lane;
      bool bis = false, biv = false, bid = false;
      float wis = 0.f, wiv = 0.f, wid = 0.f;
      uint32_t node = 0;
      if (i < L) {
        node = R.cn[n0 + i];
        const double v = Q.val[b + i], d = Q.del[b + i];
        if (i < inner) {
          if (v != 0.0) {
            if (R.ob[node]) { bis = true; wis = (float)v; }
            else { biv = true; wiv = (float)v; }
          }
          if (d != 0.0) { bid = true; wid = (float)d; }
        } else if (i >= om0) {
          const double sum = v + d;
          if (sum != 0.0) { bis = true; wis = (float)sum; }
        }
      }
      const uint32_t lt = lanemask_lt();
      const uint32_t mis = __ballot_sync(0xffffffffu, bis), miv = __ballot_sync(0xffffffffu, biv),
                     mid = __ballot_sync(0xffffffffu, bid);
      if (bis) {
        const uint64_t p = b + nis + __popc(mis & lt);
        Q.is_nbr[p] = node;
        Q.is_w[p] = wis;
      }
      if (biv) {
        const uint64_t p = b + niv + __popc(miv & lt);
        Q.iv_nbr[p] = node;
        Q.iv_w[p] = wiv;
      }
      if (bid) {
        const uint64_t p = b + nid + __popc(mid & lt);
        Q.id_nbr[p] = node;
        Q.id_w[p] = wid;
      }
      nis += __popc(mis);
      niv += __popc(miv);
      nid += __popc(mid);
    }
    if (lane == 0) {
      R.is_cnt[r] = nis;
      R.iv_cnt[r] = niv;
      R.id_cnt[r] = nid;
    }
  }
}

// boundary edge u -> x of a clustered exit (sketch2csr_mirror): it leaves the
// cluster, does not go to one of the cluster's out-mirrors, and u is not an
// in-mirror master of x's cluster
__device__ __forceinline__ bool ib_take(const RepArgs& R, uint32_t u, uint32_t x) {
  const uint32_t ids = R.cl_of[u], oid = R.cl_of[x];
  if (ids == oid) return false;
  if (om_of(R, ids, x) != kNone) return false;
  return oid == kNone || !im_of(R, oid, u);
}

__device__ __forceinline__ int ib_mode(uint8_t t) {
  if (t == kOnlyOut || t == kBothOutIn || t == kBothOutInMaster || t == kOutMaster) return 1;
  return t == kSingle ? 2 : 0;
}

// ib rows: exits keep their boundary edges, unclustered vertices all edges
// over the rows of a list (exits, unclustered vertices); the other rows'
// counts are cleared before
template <bool FILL>
__global__ void k_rp_ib(RepArgs R, const uint8_t* ntype, const uint32_t* rows, uint32_t nrows,
                        uint64_t* cnt, const uint64_t* off, uint32_t* nbr, float* wout) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nrows; q += gridDim.x * blockDim.x) {
    const uint32_t r = rows[q];
    const int mode = r < R.n ? ib_mode(ntype[r]) : 0;
    uint64_t k = FILL ? off[r] : 0;
    if (mode) {
      const uint64_t b = R.out_off[r];
      const uint32_t d = R.out_deg[r];
      for (uint32_t e = 0; e < d; ++e) {
        const uint32_t x = R.out_col[b + e];
        if (mode == 2 || ib_take(R, r, x)) {
          if (FILL) {
            nbr[k] = x;
            if (wout) wout[k] = R.out_w[b + e];
          }
          ++k;
        }
      }
    }
    if (!FILL) cnt[r] = k;
  }
}

// cluster precompute lists per member position (cm layout: members of the
// clusters in order): exits per cluster; for clusters of at most kStageCap
// members their in-edges from members (tails as local indices) and their
// edges to out-mirrors; for the others (and clusters with more than
// kStageEdges member edges) every subgraph out-edge
struct CmArgs {
  const uint64_t* cm_off;
  uint64_t *c_bl, *c_lin, *c_lout, *c_sub;        // counts per cluster (count pass)
  const uint64_t *o_bl, *o_lin, *o_lout, *o_sub;  // their prefixes (fill pass)
  uint32_t* bound_list;
  uint64_t *lin_off, *lout_off, *sub_off;         // per member position (+ total)
  uint8_t* lin_src;
  uint32_t *lout_dst, *sub_nbr;
  // clusters a batch left alone copy their lists from the previous build
  // (changed == null: every cluster is built)
  const uint8_t* changed;
  const uint64_t *old_bl_off, *old_lin_off, *old_lout_off, *old_sub_off;
  const uint32_t *old_bound_list, *old_lout_dst, *old_sub_nbr;
  const uint8_t* old_lin_src;
};

// the subgraph target of member edge v -> t in cluster c (kNone: not in the
// subgraph); *member says whether it is a member of c
__device__ __forceinline__ uint32_t sub_target(const RepArgs& R, uint32_t c, uint32_t v, uint32_t t,
                                               bool* member) {
  const uint32_t ct = R.cl_of[t];
  *member = ct == c;
  if (ct == c) return t;
  const uint32_t m = om_of(R, c, t);
  return m != kNone && !im_of(R, ct, v) ? m : kNone;
}

template <bool FILL>
__global__ void __launch_bounds__(256) k_rp_cm(RepArgs R, CmArgs A) {
  __shared__ uint32_t s_cnt[kStageWarps][kStageCap + 1];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < R.ncl; c += nw) {
    const uint32_t m = R.inner[c];
    const uint64_t n0 = R.cn_off[c], p0 = A.cm_off[c];
    const bool small = m <= (uint32_t)kStageCap;
    if (A.changed && !A.changed[c]) {
      const uint64_t p1 = p0 + m;
      if (!FILL) {
        if (lane == 0) {
          A.c_bl[c] = A.old_bl_off[c + 1] - A.old_bl_off[c];
          A.c_lin[c] = A.old_lin_off[p1] - A.old_lin_off[p0];
          A.c_lout[c] = A.old_lout_off[p1] - A.old_lout_off[p0];
          A.c_sub[c] = A.old_sub_off[p1] - A.old_sub_off[p0];
        }
        continue;
      }
      // the previous lists at their new offsets
      const uint64_t ob = A.old_bl_off[c], nb = A.o_bl[c];
      for (uint64_t i = lane; i < A.old_bl_off[c + 1] - ob; i += 32) A.bound_list[nb + i] = A.old_bound_list[ob + i];
      const uint64_t oli = A.old_lin_off[p0], nli = A.o_lin[c];
      const uint64_t olo = A.old_lout_off[p0], nlo = A.o_lout[c];
      const uint64_t osu = A.old_sub_off[p0], nsu = A.o_sub[c];
      for (uint64_t i = lane; i < A.old_lin_off[p1] - oli; i += 32) A.lin_src[nli + i] = A.old_lin_src[oli + i];
      for (uint64_t i = lane; i < A.old_lout_off[p1] - olo; i += 32) A.lout_dst[nlo + i] = A.old_lout_dst[olo + i];
      for (uint64_t i = lane; i < A.old_sub_off[p1] - osu; i += 32) A.sub_nbr[nsu + i] = A.old_sub_nbr[osu + i];
      for (uint32_t i = lane; i < m; i += 32) {
        A.lin_off[p0 + i] = A.old_lin_off[p0 + i] - oli + nli;
        A.lout_off[p0 + i] = A.old_lout_off[p0 + i] - olo + nlo;
        A.sub_off[p0 + i] = A.old_sub_off[p0 + i] - osu + nsu;
      }
      continue;
    }
    if (!FILL) {
      uint64_t nb = 0, nin = 0, nout = 0;
      for (uint32_t i = lane; i < m; i += 32) {
        const uint32_t v = R.cn[n0 + i];
        nb += R.ob[v] != 0;
        const uint64_t b = R.out_off[v];
        const uint32_t d = R.out_deg[v];
        for (uint32_t e = 0; e < d; ++e) {
          bool mem;
          if (sub_target(R, c, v, R.out_col[b + e], &mem) == kNone) continue;
          if (mem) ++nin; else ++nout;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        nb += __shfl_xor_sync(0xffffffffu, nb, o);
        nin += __shfl_xor_sync(0xffffffffu, nin, o);
        nout += __shfl_xor_sync(0xffffffffu, nout, o);
      }
      if (lane == 0) {
        const bool staged = small && nin <= (uint64_t)kStageEdges;
        A.c_bl[c] = nb;
        A.c_lin[c] = small ? nin : 0;
        A.c_lout[c] = small ? nout : 0;
        A.c_sub[c] = staged ? 0 : nin + nout;
      }
      continue;
    }
    const uint64_t lin0 = A.o_lin[c], nlin = A.o_lin[c + 1] - lin0;
    const bool staged = small && nlin <= (uint64_t)kStageEdges;
    const bool subs = A.o_sub[c + 1] > A.o_sub[c] || !staged;
    // exits in member order
    uint64_t nb = A.o_bl[c];
    for (uint32_t i0 = 0; i0 < m; i0 += 32) {
      const uint32_t i = i0 + lane;
      const bool x = i < m && R.ob[R.cn[n0 + i]];
      const uint32_t mask = __ballot_sync(0xffffffffu, x);
      if (x) A.bound_list[nb + __popc(mask & lanemask_lt())] = R.cn[n0 + i];
      nb += __popc(mask);
    }
    // per member: out-mirror edges and subgraph edges (offsets by a warp scan
    // over members in order)
    uint64_t lo = A.o_lout[c], so = A.o_sub[c];
    for (uint32_t i0 = 0; i0 < m; i0 += 32) {
      const uint32_t i = i0 + lane;
      uint32_t nout = 0, nall = 0;
      uint32_t v = 0;
      if (i < m) {
        v = R.cn[n0 + i];
        const uint64_t b = R.out_off[v];
        const uint32_t d = R.out_deg[v];
        for (uint32_t e = 0; e < d; ++e) {
          bool mem;
          if (sub_target(R, c, v, R.out_col[b + e], &mem) == kNone) continue;
          ++nall;
          nout += !mem;
        }
      }
      uint32_t xo = small ? nout : 0, xs = subs ? nall : 0;
      uint32_t io = xo, is = xs;  // inclusive scans
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t a = __shfl_up_sync(0xffffffffu, io, o), b2 = __shfl_up_sync(0xffffffffu, is, o);
        if (lane >= (uint32_t)o) {
          io += a;
          is += b2;
        }
      }
      if (i < m) {
        uint64_t po = lo + io - xo, ps = so + is - xs;
        A.lout_off[p0 + i] = po;
        A.sub_off[p0 + i] = ps;
        const uint64_t b = R.out_off[v];
        const uint32_t d = R.out_deg[v];
        for (uint32_t e = 0; e < d && (xo | xs); ++e) {
          bool mem;
          const uint32_t t = sub_target(R, c, v, R.out_col[b + e], &mem);
          if (t == kNone) continue;
          if (small && !mem) A.lout_dst[po++] = t;
          if (subs) A.sub_nbr[ps++] = t;
        }
      }
      lo += __shfl_sync(0xffffffffu, io, 31);
      so += __shfl_sync(0xffffffffu, is, 31);
    }
    // local in-edges of small clusters: counting sort by head in shared memory
    if (small) {
      uint32_t* cnt = s_cnt[w];
      for (uint32_t j = lane; j <= m; j += 32) cnt[j] = 0;
      __syncwarp();
      for (uint32_t i = lane; i < m; i += 32) {
        const uint32_t v = R.cn[n0 + i];
        const uint64_t b = R.out_off[v];
        const uint32_t d = R.out_deg[v];
        for (uint32_t e = 0; e < d; ++e) {
          const uint32_t t = R.out_col[b + e];
          if (R.cl_of[t] == c) atomicAdd(&cnt[R.loc[t] + 1], 1u);
        }
      }
      __syncwarp();
      if (lane == 0)
        for (uint32_t j = 0; j < m; ++j) cnt[j + 1] += cnt[j];
      __syncwarp();
      for (uint32_t j = lane; j < m; j += 32) A.lin_off[p0 + j] = lin0 + cnt[j];
      __syncwarp();
      for (uint32_t i = lane; i < m; i += 32) {
        const uint32_t v = R.cn[n0 + i];
        const uint64_t b = R.out_off[v];
        const uint32_t d = R.out_deg[v];
        for (uint32_t e = 0; e < d; ++e) {
          const uint32_t t = R.out_col[b + e];
          if (R.cl_of[t] == c) A.lin_src[lin0 + atomicAdd(&cnt[R.loc[t]], 1u)] = (uint8_t)i;
        }
      }
      __syncwarp();
    } else {
      for (uint32_t j = lane; j < m; j += 32) A.lin_off[p0 + j] = lin0;
    }
  }
}

// the totals behind the last member position
__global__ void k_rp_cm_tail(CmArgs A, uint32_t ncl, uint64_t npos) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    A.lin_off[npos] = A.o_lin[ncl];
    A.lout_off[npos] = A.o_lout[ncl];
    A.sub_off[npos] = A.o_sub[ncl];
  }
}

__global__ void k_rp_pending(RepArgs R) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < R.ncl; c += gridDim.x * blockDim.x) {
    if (R.c_upd[c]) R.c_pend[c] = 1;
    R.c_src[c] = 0;
    R.c_upd[c] = 0;
    R.c_job[c] = 0;
  }
}

}  // namespace

namespace {

template <typename T>
sg_status grow_keep(sg_ctx* ctx, T** p, uint64_t used, uint64_t* cap, uint64_t need) {
  if (need <= *cap && *p) return SG_OK;
  const uint64_t c = std::max<uint64_t>(need + need / 2, 1024);
  T* q = nullptr;
  SG_TRY(dalloc(ctx, &q, c));
  if (used) SG_CUDA(ctx, cudaMemcpyAsync(q, *p, sizeof(T) * used, cudaMemcpyDeviceToDevice, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(*p);
  *p = q;
  *cap = c;
  return SG_OK;
}

void free_pool(RepairDev::Pool* p) {
  dfree(p->val); dfree(p->del);
  dfree(p->is_nbr); dfree(p->iv_nbr); dfree(p->id_nbr);
  dfree(p->is_w); dfree(p->iv_w); dfree(p->id_w);
  p->cap = 0;
}

sg_status grow_pool(sg_ctx* ctx, RepairDev::Pool* p, uint64_t need) {
  if (need <= p->cap && p->val) return SG_OK;
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  free_pool(p);
  const uint64_t c = std::max<uint64_t>(need + need / 8, 64);
  SG_TRY(dalloc(ctx, &p->val, c));
  SG_TRY(dalloc(ctx, &p->del, c));
  SG_TRY(dalloc(ctx, &p->is_nbr, c));
  SG_TRY(dalloc(ctx, &p->iv_nbr, c));
  SG_TRY(dalloc(ctx, &p->id_nbr, c));
  SG_TRY(dalloc(ctx, &p->is_w, c));
  SG_TRY(dalloc(ctx, &p->iv_w, c));
  SG_TRY(dalloc(ctx, &p->id_w, c));
  p->cap = c;
  return SG_OK;
}

RepArgs rep_args(sg_ctx* ctx, RepairDev& P) {
  RepArgs R;
  R.n = P.n;
  R.all_n = P.all_n;
  R.ncl = P.ncl;
  R.cl_of = P.cl_of; R.loc = P.loc; R.cn = P.cn; R.inner = P.inner; R.n_im = P.n_im;
  R.master = P.master;
  R.cn_off = P.cn_off; R.vim_off = P.vim_off; R.vom_off = P.vom_off;
  R.vim = P.vim; R.vom = P.vom;
  R.fc = P.fc; R.ob = P.ob;
  R.m_src = P.m_src; R.m_ret = P.m_ret; R.m_new = P.m_new;
  R.c_src = P.c_src; R.c_upd = P.c_upd; R.c_job = P.c_job; R.c_pend = P.c_pend; R.r_job = P.r_job;
  R.is_cnt = P.is_cnt; R.iv_cnt = P.iv_cnt; R.id_cnt = P.id_cnt;
  R.slot = P.blk;
  const DevGraph& g = ctx->g;
  R.out_off = g.out.off; R.out_deg = g.out.deg; R.out_col = g.out.col;
  R.in_off = g.in.off; R.in_deg = g.in.deg; R.in_col = g.in.col;
  R.out_w = g.out.w;
  return R;
}

// A new layout: every supernode row packed in row order (an exclusive scan
// of the block sizes), with room for new rows; rows that keep their solve
// move there with their lists, rows solved again only get their slot.
sg_status rp_relayout(sg_ctx* ctx, RepairDev& P, const RepArgs& R) {
  cudaStream_t st = ctx->stream;
  const uint32_t all = P.all_n;
  SG_TRY(scan_u64(ctx, P.r_size, P.blk2, (uint64_t)all + 1));
  uint64_t total = 0;
  SG_TRY(read_u64(ctx, P.blk2 + all, &total));
  const uint64_t cap = total + total / 2 + 1024;
  SG_TRY(grow_pool(ctx, &P.pool2, cap));
  if (P.sssp_on) SG_TRY(grow(ctx, &P.sd2, &P.sd2_cap, P.pool2.cap));
  MoveArgs M{};
  M.blk = P.blk;
  M.blk2 = P.blk2;
  M.val = P.pool.val; M.del = P.pool.del; M.val2 = P.pool2.val; M.del2 = P.pool2.del;
  M.is_nbr = P.pool.is_nbr; M.iv_nbr = P.pool.iv_nbr; M.id_nbr = P.pool.id_nbr;
  M.is_w = P.pool.is_w; M.iv_w = P.pool.iv_w; M.id_w = P.pool.id_w;
  M.is_nbr2 = P.pool2.is_nbr; M.iv_nbr2 = P.pool2.iv_nbr; M.id_nbr2 = P.pool2.id_nbr;
  M.is_w2 = P.pool2.is_w; M.iv_w2 = P.pool2.iv_w; M.id_w2 = P.pool2.id_w;
  k_rp_move<<<grid_for((uint64_t)P.n_sp * 32, 256), 256, 0, st>>>(R, P.sp_rows, P.n_sp, P.r_size, M,
                                                                  P.d_err);
  if (P.sssp_on && P.sd) {
    MoveArgs Ms{};
    Ms.blk = P.blk;
    Ms.blk2 = P.blk2;
    Ms.val = Ms.del = P.sd;
    Ms.val2 = Ms.del2 = P.sd2;
    k_rp_move<<<grid_for((uint64_t)P.n_sp * 32, 256), 256, 0, st>>>(R, P.sp_rows, P.n_sp, P.r_size,
                                                                    Ms, P.d_err);
  }
  std::swap(P.blk, P.blk2);
  std::swap(P.pool, P.pool2);
  std::swap(P.sd, P.sd2);
  std::swap(P.sd_cap, P.sd2_cap);
  k_rp_unslot<<<grid_for(all, 256), 256, 0, st>>>(P.f_sp, all, P.blk);
  SG_CUDA(ctx, cudaMemcpyAsync(P.d_tail, &total, 8, cudaMemcpyHostToDevice, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  count_launch(ctx, 3 + (P.sssp_on ? 1 : 0));
  SG_CUDA(ctx, cudaGetLastError());
  P.pool_used = total;
  P.live_at_layout = total;
  P.relayouts++;
  return SG_OK;
}

// Solves again the supernode rows marked in r_job (r_size holds every row's
// block size) into the next pool layout and moves the other blocks there.
// Local problems of the ntc clusters listed in P.tcl: their node ranges
// (lp_off), local edges (adj_off / adj_nbr, with weights when the graph has
// them), divisors, and for the clusters of at most kStageCap nodes the
// in-edges from members (lin_off / lin_src).
sg_status rp_local_problems(sg_ctx* ctx, RepairDev& P, const RepArgs& R, uint32_t ntc,
                            uint64_t* npos_out) {
  cudaStream_t st = ctx->stream;
  k_rp_tcl<<<grid_for(ntc, 256), 256, 0, st>>>(R, P.tcl, ntc, P.tc_idx, P.tc_inner, P.cnt_a);
  SG_TRY(scan_u64(ctx, P.cnt_a, P.lp_off, (uint64_t)ntc + 1));
  uint64_t npos = 0;
  SG_TRY(read_u64(ctx, P.lp_off + ntc, &npos));
  SG_TRY(grow(ctx, &P.adj_off, &P.cap_lp, npos + 1));
  SG_TRY(grow(ctx, &P.div, &P.cap_div, npos + 1));
  SG_TRY(grow(ctx, &P.lin_off, &P.cap_linoff, npos + 1));
  SG_TRY(grow(ctx, &P.cnt_d, &P.cap_cntd, npos + 1));
  const unsigned wg = grid_for((uint64_t)ntc * 32, 256);
  k_rp_lp_count<<<wg, 256, 0, st>>>(R, P.tcl, ntc, P.lp_off, P.cnt_d);
  SG_TRY(scan_u64(ctx, P.cnt_d, P.adj_off, npos + 1));
  uint64_t nadj = 0;
  SG_TRY(read_u64(ctx, P.adj_off + npos, &nadj));
  SG_TRY(grow(ctx, &P.adj_nbr, &P.cap_adj, nadj));
  if (R.out_w) SG_TRY(grow(ctx, &P.adj_w, &P.cap_adjw, nadj));
  k_rp_lp_fill<<<wg, 256, 0, st>>>(R, P.tcl, ntc, P.lp_off, P.adj_off, P.adj_nbr,
                                   R.out_w ? P.adj_w : nullptr, P.div);
  k_rp_lin_count<<<grid_for(ntc, 256), 256, 0, st>>>(R, P.tcl, ntc, P.lp_off, P.adj_off, P.cnt_a);
  SG_TRY(scan_u64(ctx, P.cnt_a, P.cl_lin, (uint64_t)ntc + 1));
  uint64_t nlin = 0;
  SG_TRY(read_u64(ctx, P.cl_lin + ntc, &nlin));
  SG_TRY(grow(ctx, &P.lin_src, &P.cap_lin, nlin));
  k_rp_lin_fill<<<wg, 256, 0, st>>>(R, P.tcl, ntc, P.lp_off, P.adj_off, P.adj_nbr, P.cl_lin,
                                    P.lin_off, P.lin_src);
  SG_CUDA(ctx, cudaMemcpyAsync(P.lin_off + npos, P.cl_lin + ntc, 8, cudaMemcpyDeviceToDevice, st));
  count_launch(ctx, 9);
  *npos_out = npos;
  return SG_OK;
}

// SSSP distances inside the listed jobs' clusters (Bellman-Ford in shared
// memory, a CTA per job) into out at the jobs' offsets
sg_status rp_sssp_solve(sg_ctx* ctx, RepairDev& P, uint32_t nj, const uint64_t* out_off, double* out,
                        cudaStream_t st) {
  const size_t smem = (size_t)P.max_L * sizeof(unsigned long long);
  if (smem > 48 * 1024)
    SG_CUDA(ctx, cudaFuncSetAttribute(k_sssp_shortcuts, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  k_sssp_shortcuts<<<nj, 128, smem, st>>>(P.sp_cl, P.sp_src, P.lp_off, P.adj_off, P.adj_nbr, P.adj_w,
                                          out_off, out, nj);
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  return SG_OK;
}

// Launches the solves of the supernode rows marked in r_job (r_size holds
// every row's block size) into their slots (the SSSP distance blocks too,
// once SSSP over the summary has run) on the side stream; rp_join waits for
// them and writes the rows' lists.
sg_status rp_shortcuts(sg_ctx* ctx, SummaryDev& D, RepairDev& P, const RepArgs& R, PhaseTrace& T) {
  cudaStream_t st = ctx->stream;
  const uint32_t all = P.all_n;
  // distance blocks once SSSP over the summary starts (every row is solved
  // again then, so nothing to keep)
  if (P.sssp_on && P.sd_cap < P.pool.cap) SG_TRY(grow(ctx, &P.sd, &P.sd_cap, P.pool.cap));
  SG_TRY(select_idx(ctx, P.r_job, P.jobs, P.d_num, all));
  SG_TRY(select_idx(ctx, P.f_sp, P.sp_rows, P.d_num + 1, all));
  uint32_t nj_sp[2] = {0, 0};
  SG_CUDA(ctx, cudaMemcpyAsync(nj_sp, P.d_num, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  const uint32_t nj = nj_sp[0];
  P.n_sp = nj_sp[1];
  // Rows keep their blocks; new rows take slots at the pool tail.  A new
  // layout (every row packed in row order, blocks moved) when the tail could
  // outgrow the pool or the holes of retired rows reach the live size.
  if (P.pool_used + (uint64_t)nj * P.max_L > P.pool.cap || P.pool_used > 2 * P.live_at_layout + 1024) {
    SG_TRY(rp_relayout(ctx, P, R));
  } else if (nj) {
    k_rp_alloc<<<grid_for(nj, 256), 256, 0, st>>>(P.jobs, nj, P.r_size, P.blk, P.d_tail);
    SG_TRY(read_u64(ctx, (const uint64_t*)P.d_tail, &P.pool_used));
    count_launch(ctx);
  }
  T.mark("layout and jobs");
  if (nj) {
    k_rp_job_clusters<<<grid_for(nj, 256), 256, 0, st>>>(R, P.jobs, nj);
    SG_TRY(select_idx(ctx, P.c_job, P.tcl, P.d_num, P.ncl));
    uint32_t ntc = 0;
    SG_CUDA(ctx, cudaMemcpyAsync(&ntc, P.d_num, 4, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
    uint64_t npos = 0;
    SG_TRY(rp_local_problems(ctx, P, R, ntc, &npos));
    k_rp_jobs<<<grid_for(nj, 256), 256, 0, st>>>(R, P.jobs, nj, P.tc_idx, P.blk, P.sp_cl, P.sp_src,
                                                 P.out_off, P.j_half, P.j_warp, P.j_warp5, P.j_block);
    SG_TRY(select_idx(ctx, P.j_warp, P.wjobs, P.d_num, nj));
    SG_TRY(select_idx(ctx, P.j_block, P.bjobs, P.d_num + 1, nj));
    SG_TRY(select_idx(ctx, P.j_warp5, P.wjobs5, P.d_num + 2, nj));
    SG_TRY(select_idx(ctx, P.j_half, P.hjobs, P.d_num + 3, nj));
    uint32_t nwb[4] = {0, 0, 0, 0};
    SG_CUDA(ctx, cudaMemcpyAsync(nwb, P.d_num, 16, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
    T.mark("local problems");
    ShortcutArgs A;
    A.n_sp = nj;
    A.sp_cluster = P.sp_cl;
    A.sp_src = P.sp_src;
    A.cl_off = P.lp_off;
    A.cl_inner = P.tc_inner;  // members per touched cluster, by its index
    A.adj_off = P.adj_off;
    A.adj_nbr = P.adj_nbr;
    A.div = P.div;
    A.out_off = P.out_off;
    A.out_value = P.pool.val;
    A.out_delta = P.pool.del;
    A.damping = (float)ctx->opt.damping;
    A.thr_per_node = ctx->opt.termcheck_threshold / (double)P.n;
    A.lin_off = P.lin_off;
    A.lin_src = P.lin_src;
    // The side stream starts after the work queued so far; the kernel-class
    // profiler brackets kernels on the context stream, so the solves stay
    // there while it is on.
    cudaStream_t ss = ctx->opt.profile ? st : P.side;
    if (ss != st) {
      SG_CUDA(ctx, cudaEventRecord(P.ev_ready, st));
      SG_CUDA(ctx, cudaStreamWaitEvent(ss, P.ev_ready, 0));
    }
    kprof_begin(ctx);
    if (nwb[3]) {
      A.jobs = P.hjobs;
      launch_shortcuts_warp(3, A, nwb[3], ss);
    }
    if (nwb[0]) {
      A.jobs = P.wjobs;
      launch_shortcuts_warp(2, A, nwb[0], ss);
    }
    if (nwb[2]) {
      A.jobs = P.wjobs5;
      launch_shortcuts_warp(5, A, nwb[2], ss);
    }
    if (nwb[1]) {
      const size_t smem = shortcut_smem(P.max_L);
      if (smem > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_shortcuts, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
      A.jobs = P.bjobs;
      k_shortcuts<<<nwb[1], 128, smem, ss>>>(A, nwb[1]);
    }
    kprof_end(ctx, SG_K_SUMMARY);
    count_launch(ctx, 4);
    SG_CUDA(ctx, cudaGetLastError());
    if (P.sssp_on) SG_TRY(rp_sssp_solve(ctx, P, nj, P.out_off, P.sd, ss));
    if (ss != st) {
      SG_CUDA(ctx, cudaEventRecord(P.ev_solved, ss));
      P.solving = true;
    }
  }
  P.n_jobs = nj;
  P.sk_stale = true;
  (void)D;
  return SG_OK;
}

// The context stream waits for the solves launched by rp_shortcuts, then
// the lists of the rows solved again are written into their slots.
sg_status rp_join(sg_ctx* ctx, RepairDev& P, const RepArgs& R, PhaseTrace& T) {
  cudaStream_t st = ctx->stream;
  if (P.solving) {
    P.solving = false;
    SG_CUDA(ctx, cudaStreamWaitEvent(st, P.ev_solved, 0));
  }
  const uint32_t nj = P.n_jobs;
  if (!nj) return SG_OK;
  T.mark("shortcut solves (the rest after the tables)", st);
  k_rp_lists<<<grid_for((uint64_t)nj * 32, 256), 256, 0, st>>>(R, P.jobs, nj, P.blk, P.pool);
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  T.mark("lists", st);
  return SG_OK;
}

// Rebuilds the PageRank tables of the summary from the repaired state.
sg_status rp_tables(sg_ctx* ctx, SummaryDev& D, RepairDev& P, const RepArgs& R, PhaseTrace& PT) {
  cudaStream_t st = ctx->stream;
  const uint32_t n = P.n, all = P.all_n, ncl = P.ncl;
  SG_TRY(reserve(ctx, D, &D.ntype, n));
  SG_TRY(reserve(ctx, D, &D.l_entry, n));
  SG_TRY(reserve(ctx, D, &D.l_exit, n));
  SG_TRY(reserve(ctx, D, &D.l_single, n));
  SG_TRY(reserve(ctx, D, &D.ib_off, (uint64_t)all + 1));
  k_rp_types<<<grid_for(n, 256), 256, 0, st>>>(R, D.ntype, P.f_entry, P.f_exit, P.f_single);
  SG_TRY(select_idx(ctx, P.f_entry, D.l_entry, P.d_num, n));
  SG_TRY(select_idx(ctx, P.f_exit, D.l_exit, P.d_num + 1, n));
  SG_TRY(select_idx(ctx, P.f_single, D.l_single, P.d_num + 2, n));
  uint32_t nl[3] = {0, 0, 0};
  SG_CUDA(ctx, cudaMemcpyAsync(nl, P.d_num, 12, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.cnt_d, 0, 8ull * (all + 1), st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  D.n_entry = nl[0];
  D.n_exit = nl[1];
  D.n_single = nl[2];
  PT.mark("node types and lists", st);
  // boundary rows of exits and unclustered vertices
  if (D.n_exit)
    k_rp_ib<false><<<grid_for(D.n_exit, 256), 256, 0, st>>>(R, D.ntype, D.l_exit, D.n_exit, P.cnt_d,
                                                            nullptr, nullptr, nullptr);
  if (D.n_single)
    k_rp_ib<false><<<grid_for(D.n_single, 256), 256, 0, st>>>(R, D.ntype, D.l_single, D.n_single,
                                                              P.cnt_d, nullptr, nullptr, nullptr);
  SG_TRY(scan_u64(ctx, P.cnt_d, D.ib_off, (uint64_t)all + 1));
  uint64_t nib = 0;
  SG_TRY(read_u64(ctx, D.ib_off + all, &nib));
  D.n_ib = nib;
  SG_TRY(reserve(ctx, D, &D.ib_nbr, nib));
  float* ibw = nullptr;
  if (R.out_w) {
    SG_TRY(grow(ctx, &P.ib_w, &P.ib_w_cap, nib));
    ibw = P.ib_w;
  }
  if (D.n_exit)
    k_rp_ib<true><<<grid_for(D.n_exit, 256), 256, 0, st>>>(R, D.ntype, D.l_exit, D.n_exit, nullptr,
                                                           D.ib_off, D.ib_nbr, ibw);
  if (D.n_single)
    k_rp_ib<true><<<grid_for(D.n_single, 256), 256, 0, st>>>(R, D.ntype, D.l_single, D.n_single,
                                                             nullptr, D.ib_off, D.ib_nbr, ibw);
  PT.mark("ib rows", st);
  // cluster precompute lists: clusters the batch updated are built again,
  // the others copy theirs into the new layout (double-buffered: the
  // summary's arrays are the current build, P.nx the next)
  CmArgs C{};
  C.cm_off = D.cm_off;
  C.c_bl = P.cnt_a;
  C.c_lin = P.cnt_b;
  C.c_lout = P.cnt_c;
  C.c_sub = P.cnt_d;
  C.changed = P.cm_built ? P.c_upd : nullptr;
  C.old_bl_off = D.bl_off;
  C.old_lin_off = D.lin_off;
  C.old_lout_off = D.lout_off;
  C.old_sub_off = D.sub_off;
  C.old_bound_list = D.bound_list;
  C.old_lin_src = D.lin_src;
  C.old_lout_dst = D.lout_dst;
  C.old_sub_nbr = D.sub_nbr;
  const unsigned cg = grid_for((uint64_t)ncl * 32, 256);
  k_rp_cm<false><<<cg, 256, 0, st>>>(R, C);
  RepairDev::CmBuf& X = P.nx;
  SG_TRY(grow(ctx, &X.bl_off, &X.cap.bl_off, (uint64_t)ncl + 1));
  SG_TRY(scan_u64(ctx, P.cnt_a, X.bl_off, (uint64_t)ncl + 1));
  SG_TRY(scan_u64(ctx, P.cnt_b, P.o_lin, (uint64_t)ncl + 1));
  SG_TRY(scan_u64(ctx, P.cnt_c, P.o_lout, (uint64_t)ncl + 1));
  SG_TRY(scan_u64(ctx, P.cnt_d, P.o_sub, (uint64_t)ncl + 1));
  uint64_t ct[4] = {0, 0, 0, 0};
  SG_CUDA(ctx, cudaMemcpyAsync(&ct[0], X.bl_off + ncl, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(&ct[1], P.o_lin + ncl, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(&ct[2], P.o_lout + ncl, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(&ct[3], P.o_sub + ncl, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  const uint64_t npos = P.n_members;
  SG_TRY(grow(ctx, &X.bound_list, &X.cap.bound_list, ct[0]));
  SG_TRY(grow(ctx, &X.lin_src, &X.cap.lin_src, ct[1]));
  SG_TRY(grow(ctx, &X.lout_dst, &X.cap.lout_dst, ct[2]));
  SG_TRY(grow(ctx, &X.sub_nbr, &X.cap.sub_nbr, ct[3]));
  SG_TRY(grow(ctx, &X.lin_off, &X.cap.lin_off, npos + 1));
  SG_TRY(grow(ctx, &X.lout_off, &X.cap.lout_off, npos + 1));
  SG_TRY(grow(ctx, &X.sub_off, &X.cap.sub_off, npos + 1));
  C.o_bl = X.bl_off;
  C.o_lin = P.o_lin;
  C.o_lout = P.o_lout;
  C.o_sub = P.o_sub;
  C.bound_list = X.bound_list;
  C.lin_off = X.lin_off;
  C.lout_off = X.lout_off;
  C.sub_off = X.sub_off;
  C.lin_src = X.lin_src;
  C.lout_dst = X.lout_dst;
  C.sub_nbr = X.sub_nbr;
  k_rp_cm<true><<<cg, 256, 0, st>>>(R, C);
  k_rp_cm_tail<<<1, 32, 0, st>>>(C, ncl, npos);
  // the new build becomes the summary's (and the old one the next buffer)
  std::swap(D.bl_off, X.bl_off);
  std::swap(D.bound_list, X.bound_list);
  std::swap(D.lin_off, X.lin_off);
  std::swap(D.lin_src, X.lin_src);
  std::swap(D.lout_off, X.lout_off);
  std::swap(D.lout_dst, X.lout_dst);
  std::swap(D.sub_off, X.sub_off);
  std::swap(D.sub_nbr, X.sub_nbr);
  std::swap(P.cur, X.cap);
  P.cm_built = true;
  PT.mark("cluster lists", st);
  count_launch(ctx, 8);
  SG_CUDA(ctx, cudaGetLastError());
  return SG_OK;
}

sg_status rp_finish(sg_ctx* ctx, RepairDev& P, const RepArgs& R) {
  cudaStream_t st = ctx->stream;
  k_rp_pending<<<grid_for(P.ncl, 256), 256, 0, st>>>(R);
  SG_CUDA(ctx, cudaMemsetAsync(P.r_job, 0, P.all_n, st));
  uint32_t err = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&err, P.d_err, 4, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  count_launch(ctx);
  if (err) return fail(ctx, SG_ERR_STATE, "summary repair: a kept supernode lost its shortcut block");
  return SG_OK;
}

// The shortcut solves (side stream) beside the table rebuild (context
// stream), then the solved rows' lists and the end of the batch; the solves
// are waited for on every path, so no work of this batch outlives the call.
sg_status rp_rebuild(sg_ctx* ctx, SummaryDev& D, RepairDev& P, const RepArgs& R, PhaseTrace& T) {
  sg_status s = rp_shortcuts(ctx, D, P, R, T);
  if (s == SG_OK) s = rp_tables(ctx, D, P, R, T);
  const sg_status j = rp_join(ctx, P, R, T);
  if (s != SG_OK) return s;
  if (j != SG_OK) return j;
  return rp_finish(ctx, P, R);
}

}  // namespace

void repair_free(SummaryDev& D) {
  RepairDev* P = D.rep;
  if (!P) return;
  if (P->side) {
    cudaStreamSynchronize(P->side);
    cudaStreamDestroy(P->side);
  }
  if (P->ev_ready) cudaEventDestroy(P->ev_ready);
  if (P->ev_solved) cudaEventDestroy(P->ev_solved);
  dfree(P->cl_of); dfree(P->loc); dfree(P->cn_off); dfree(P->cn); dfree(P->inner); dfree(P->n_im);
  dfree(P->master); dfree(P->vim_off); dfree(P->vim); dfree(P->vom_off); dfree(P->vom);
  dfree(P->fc); dfree(P->ob);
  dfree(P->m_src); dfree(P->m_ret); dfree(P->m_new);
  dfree(P->c_src); dfree(P->c_upd); dfree(P->c_job); dfree(P->c_pend); dfree(P->r_job);
  dfree(P->f_entry); dfree(P->f_exit); dfree(P->f_single); dfree(P->r_size);
  dfree(P->f_sp); dfree(P->sp_rows);
  dfree(P->blk); dfree(P->blk2); dfree(P->sd); dfree(P->sd2); dfree(P->ib_w); dfree(P->adj_w);
  dfree(P->f_corr); dfree(P->im_list); dfree(P->im_master); dfree(P->src_dist);
  dfree(P->seed_v); dfree(P->seed_n); dfree(P->seed_d);
  free_pool(&P->pool); free_pool(&P->pool2);
  dfree(P->is_cnt); dfree(P->iv_cnt); dfree(P->id_cnt); dfree(P->row_inner); dfree(P->d_tail);
  dfree(P->jobs); dfree(P->tcl); dfree(P->tc_idx); dfree(P->tc_inner); dfree(P->sp_cl);
  dfree(P->sp_src); dfree(P->wjobs); dfree(P->bjobs); dfree(P->j_warp); dfree(P->j_block);
  dfree(P->wjobs5); dfree(P->j_warp5); dfree(P->hjobs); dfree(P->j_half);
  dfree(P->lp_off); dfree(P->adj_off); dfree(P->out_off); dfree(P->lin_off); dfree(P->cl_lin);
  dfree(P->adj_nbr); dfree(P->lin_src); dfree(P->div);
  dfree(P->cnt_a); dfree(P->cnt_b); dfree(P->cnt_c); dfree(P->cnt_d);
  dfree(P->o_lin); dfree(P->o_lout); dfree(P->o_sub);
  dfree(P->nx.bl_off); dfree(P->nx.lin_off); dfree(P->nx.lout_off); dfree(P->nx.sub_off);
  dfree(P->nx.bound_list); dfree(P->nx.lout_dst); dfree(P->nx.sub_nbr); dfree(P->nx.lin_src);
  dfree(P->d_num); dfree(P->d_err);
  dfree(P->log_src); dfree(P->log_dst); dfree(P->log_kind); dfree(P->log_found); dfree(P->log_w);
  delete P;
  D.rep = nullptr;
}

sg_status repair_init(sg_ctx* ctx, SummaryDev& D) {
  repair_free(D);
  const Summary& S = D.S;
  if (S.supernode_ids.empty()) return SG_OK;  // no supernode: the plain path runs
  RepairDev* Pp = new RepairDev();
  D.rep = Pp;
  RepairDev& P = *Pp;
  cudaStream_t st = ctx->stream;
  {
    int least = 0, greatest = 0;
    SG_CUDA(ctx, cudaDeviceGetStreamPriorityRange(&least, &greatest));
    SG_CUDA(ctx, cudaStreamCreateWithPriority(&P.side, cudaStreamNonBlocking, least));
    SG_CUDA(ctx, cudaEventCreateWithFlags(&P.ev_ready, cudaEventDisableTiming));
    SG_CUDA(ctx, cudaEventCreateWithFlags(&P.ev_solved, cudaEventDisableTiming));
  }
  const uint32_t n = S.old_n, all = S.all_n, ncl = (uint32_t)S.supernode_ids.size();
  P.n = n;
  P.all_n = all;
  P.ncl = ncl;
  // cluster node lists: members, then in-mirrors, then out-mirrors
  std::vector<uint32_t> loc(all, kNone), inner(ncl), nim(ncl), cn;
  std::vector<uint64_t> cn_off(ncl + 1, 0);
  for (uint32_t c = 0; c < ncl; ++c) {
    const auto& nodes = S.cluster_ids[c];
    const auto& mem = S.supernode_ids[c];
    const auto& im = S.cluster_in_mirror_ids[c];
    const auto& om = S.cluster_out_mirror_ids[c];
    if (nodes.size() != mem.size() + im.size() + om.size())
      return fail(ctx, SG_ERR_STATE, "summary repair: unexpected cluster node list");
    for (size_t i = 0; i < nodes.size(); ++i) {
      const uint32_t x = nodes[i];
      const bool ok = i < mem.size() ? x == mem[i]
                      : i < mem.size() + im.size() ? x == im[i - mem.size()]
                                                   : x == om[i - mem.size() - im.size()];
      if (!ok || x >= all) return fail(ctx, SG_ERR_STATE, "summary repair: unexpected cluster node order");
      loc[x] = (uint32_t)i;
      cn.push_back(x);
    }
    cn_off[c + 1] = cn.size();
    inner[c] = (uint32_t)mem.size();
    nim[c] = (uint32_t)im.size();
    P.max_L = std::max<uint32_t>(P.max_L, (uint32_t)nodes.size());
    P.n_members += mem.size();
  }
  if (shortcut_smem(P.max_L) > 200 * 1024)
    return fail(ctx, SG_ERR_UNSUPPORTED, "cluster too large for the shortcut kernel");
  // in-mirrors and out-mirrors of each master, by cluster
  std::vector<std::vector<uint32_t>> byv_i(n), byv_o(n);
  for (uint32_t c = 0; c < ncl; ++c) {
    for (uint32_t m : S.cluster_in_mirror_ids[c]) byv_i[S.mirror_master(m)].push_back(m);
    for (uint32_t m : S.cluster_out_mirror_ids[c]) byv_o[S.mirror_master(m)].push_back(m);
  }
  std::vector<uint64_t> vim_off(n + 1, 0), vom_off(n + 1, 0);
  std::vector<uint32_t> vim, vom;
  for (uint32_t v = 0; v < n; ++v) {
    // clusters are visited in order, so each list is sorted by cluster
    vim.insert(vim.end(), byv_i[v].begin(), byv_i[v].end());
    vom.insert(vom.end(), byv_o[v].begin(), byv_o[v].end());
    vim_off[v + 1] = vim.size();
    vom_off[v + 1] = vom.size();
  }
  std::vector<uint32_t> master(S.mirrorid2vid.begin(), S.mirrorid2vid.end());
  std::vector<int32_t> fc(S.Fc.begin(), S.Fc.end());
  std::vector<uint8_t> ob(n);
  for (uint32_t v = 0; v < n; ++v) ob[v] = S.out_bound[v] != 0;
  std::vector<uint32_t> cl_of(S.id2spids.begin(), S.id2spids.end());
  cl_of.resize(all, kNone);
  SG_TRY(put(ctx, &P.cl_of, cl_of));
  SG_TRY(put(ctx, &P.loc, loc));
  SG_TRY(put(ctx, &P.cn_off, cn_off));
  SG_TRY(put(ctx, &P.cn, cn));
  SG_TRY(put(ctx, &P.inner, inner));
  SG_TRY(put(ctx, &P.n_im, nim));
  SG_TRY(put(ctx, &P.master, master));
  SG_TRY(put(ctx, &P.vim_off, vim_off));
  SG_TRY(put(ctx, &P.vim, vim));
  SG_TRY(put(ctx, &P.vom_off, vom_off));
  SG_TRY(put(ctx, &P.vom, vom));
  SG_TRY(put(ctx, &P.fc, fc));
  SG_TRY(put(ctx, &P.ob, ob));
  {
    std::vector<uint32_t> iml, imm;
    for (uint32_t c = 0; c < ncl; ++c)
      for (uint32_t m : S.cluster_in_mirror_ids[c]) {
        iml.push_back(m);
        imm.push_back(S.mirror_master(m));
      }
    P.n_im_total = (uint32_t)iml.size();
    SG_TRY(put(ctx, &P.im_list, iml));
    SG_TRY(put(ctx, &P.im_master, imm));
  }
  // marks and fixed-size scratch
  SG_TRY(dalloc(ctx, &P.m_src, n));
  SG_TRY(dalloc(ctx, &P.m_ret, n));
  SG_TRY(dalloc(ctx, &P.m_new, n));
  SG_TRY(dalloc(ctx, &P.f_entry, n));
  SG_TRY(dalloc(ctx, &P.f_exit, n));
  SG_TRY(dalloc(ctx, &P.f_single, n));
  SG_TRY(dalloc(ctx, &P.c_src, ncl));
  SG_TRY(dalloc(ctx, &P.c_upd, ncl));
  SG_TRY(dalloc(ctx, &P.c_job, ncl));
  SG_TRY(dalloc(ctx, &P.c_pend, ncl));
  SG_TRY(dalloc(ctx, &P.r_job, all));
  SG_TRY(dalloc(ctx, &P.f_sp, all));
  SG_TRY(dalloc(ctx, &P.is_cnt, all));
  SG_TRY(dalloc(ctx, &P.iv_cnt, all));
  SG_TRY(dalloc(ctx, &P.id_cnt, all));
  {
    std::vector<uint32_t> ri(all, 0);
    for (uint32_t r = 0; r < all; ++r)
      if (cl_of[r] != kNone) ri[r] = inner[cl_of[r]];
    SG_TRY(put(ctx, &P.row_inner, ri));
  }
  SG_TRY(dalloc(ctx, &P.f_corr, all));
  SG_TRY(dalloc(ctx, &P.src_dist, std::max<uint32_t>(P.max_L, 1)));
  SG_TRY(dalloc(ctx, &P.seed_v, std::max<uint32_t>(P.max_L, 1)));
  SG_TRY(dalloc(ctx, &P.seed_d, std::max<uint32_t>(P.max_L, 1)));
  SG_TRY(dalloc(ctx, &P.seed_n, 1));
  SG_TRY(dalloc(ctx, &P.sp_rows, all));
  SG_TRY(dalloc(ctx, &P.r_size, (uint64_t)all + 1));
  SG_TRY(dalloc(ctx, &P.blk, (uint64_t)all + 1));
  SG_TRY(dalloc(ctx, &P.blk2, (uint64_t)all + 1));
  SG_TRY(dalloc(ctx, &P.jobs, all));
  SG_TRY(dalloc(ctx, &P.sp_cl, all));
  SG_TRY(dalloc(ctx, &P.sp_src, all));
  SG_TRY(dalloc(ctx, &P.out_off, all));
  SG_TRY(dalloc(ctx, &P.wjobs, all));
  SG_TRY(dalloc(ctx, &P.bjobs, all));
  SG_TRY(dalloc(ctx, &P.j_warp, all));
  SG_TRY(dalloc(ctx, &P.j_warp5, all));
  SG_TRY(dalloc(ctx, &P.j_half, all));
  SG_TRY(dalloc(ctx, &P.hjobs, all));
  SG_TRY(dalloc(ctx, &P.wjobs5, all));
  SG_TRY(dalloc(ctx, &P.j_block, all));
  SG_TRY(dalloc(ctx, &P.tcl, ncl));
  SG_TRY(dalloc(ctx, &P.tc_idx, ncl));
  SG_TRY(dalloc(ctx, &P.tc_inner, ncl));
  SG_TRY(dalloc(ctx, &P.lp_off, (uint64_t)ncl + 1));
  SG_TRY(dalloc(ctx, &P.cl_lin, (uint64_t)ncl + 1));
  SG_TRY(dalloc(ctx, &P.o_lin, (uint64_t)ncl + 1));
  SG_TRY(dalloc(ctx, &P.o_lout, (uint64_t)ncl + 1));
  SG_TRY(dalloc(ctx, &P.o_sub, (uint64_t)ncl + 1));
  const uint64_t nc = std::max<uint64_t>(all, ncl) + 1;
  SG_TRY(dalloc(ctx, &P.cnt_a, nc));
  SG_TRY(dalloc(ctx, &P.cnt_b, nc));
  SG_TRY(dalloc(ctx, &P.cnt_c, nc));
  // cnt_d also holds the local edge count of each touched cluster node
  SG_TRY(dalloc(ctx, &P.cnt_d, nc));
  P.cap_cntd = nc;
  SG_TRY(dalloc(ctx, &P.d_num, 4));
  SG_TRY(dalloc(ctx, &P.d_err, 1));
  SG_TRY(dalloc(ctx, &P.d_tail, 1));
  SG_CUDA(ctx, cudaMemsetAsync(P.m_src, 0, n, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.m_ret, 0, n, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.m_new, 0, n, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.c_upd, 0, ncl, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.c_job, 0, ncl, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.c_pend, 0, ncl, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.r_job, 0, all, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.is_cnt, 0, 4ull * all, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.iv_cnt, 0, 4ull * all, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.id_cnt, 0, 4ull * all, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.blk, 0xFF, 8ull * (all + 1), st));  // no row has a slot yet
  SG_CUDA(ctx, cudaMemsetAsync(P.cnt_a, 0, 8ull * nc, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.cnt_b, 0, 8ull * nc, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.cnt_c, 0, 8ull * nc, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.cnt_d, 0, 8ull * nc, st));
  SG_CUDA(ctx, cudaMemsetAsync(P.d_err, 0, 4, st));
  // every supernode solved once (every cluster a changed source), then the
  // tables built from that state
  SG_CUDA(ctx, cudaMemsetAsync(P.c_src, 1, ncl, st));
  const RepArgs R = rep_args(ctx, P);
  SG_TRY(reserve(ctx, D, &D.out_deg_all, all));
  k_rp_rows<<<grid_for(all, 256), 256, 0, st>>>(R, P.r_size, P.f_sp, D.out_deg_all);
  count_launch(ctx);
  PhaseTrace T("device summary build");
  return rp_rebuild(ctx, D, P, R, T);
}

sg_status repair_after_apply(sg_ctx* ctx, SummaryDev& D) {
  RepairDev* Pp = D.rep;
  if (!Pp) return SG_OK;
  RepairDev& P = *Pp;
  cudaStream_t st = ctx->stream;
  const DevBatch& B = ctx->batch;
  const uint64_t na = B.n_act;
  PhaseTrace T("device repair");
  // the actions, kept for the host restatement
  if (na) {
    const uint64_t need = P.log_n + na;
    uint64_t c1 = P.log_cap, c2 = P.log_cap, c3 = P.log_cap, c4 = P.log_cap, c5 = P.log_cap;
    SG_TRY(grow_keep(ctx, &P.log_src, P.log_n, &c1, need));
    SG_TRY(grow_keep(ctx, &P.log_dst, P.log_n, &c2, need));
    SG_TRY(grow_keep(ctx, &P.log_kind, P.log_n, &c3, need));
    SG_TRY(grow_keep(ctx, &P.log_found, P.log_n, &c4, need));
    SG_TRY(grow_keep(ctx, &P.log_w, P.log_n, &c5, need));
    P.log_cap = c1;
    SG_CUDA(ctx, cudaMemcpyAsync(P.log_src + P.log_n, B.a_src, 4 * na, cudaMemcpyDeviceToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(P.log_dst + P.log_n, B.a_dst, 4 * na, cudaMemcpyDeviceToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(P.log_kind + P.log_n, B.a_kind, 4 * na, cudaMemcpyDeviceToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(P.log_found + P.log_n, B.a_found, 4 * na, cudaMemcpyDeviceToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(P.log_w + P.log_n, B.a_w, 4 * na, cudaMemcpyDeviceToDevice, st));
    P.log_n = need;
  }
  P.log_end.push_back(P.log_n);
  T.mark("action log", st);
  const RepArgs R = rep_args(ctx, P);
  if (na)
    k_rp_actions<<<grid_for(na * 32, 256), 256, 0, st>>>(R, B.a_src, B.a_dst, B.a_kind, B.a_found, na);
  k_rp_entries<<<grid_for(P.n, 256), 256, 0, st>>>(R);
  SG_TRY(reserve(ctx, D, &D.out_deg_all, P.all_n));
  k_rp_rows<<<grid_for(P.all_n, 256), 256, 0, st>>>(R, P.r_size, P.f_sp, D.out_deg_all);
  count_launch(ctx, 3);
  T.mark("entries, exits, rows", st);
  const sg_status fs = rp_rebuild(ctx, D, P, R, T);
  T.mark("finish");
  return fs;
}

sg_status repair_pending_clusters(sg_ctx* ctx, SummaryDev& D, const uint32_t** list, uint32_t* count) {
  RepairDev* P = D.rep;
  *list = nullptr;
  *count = 0;
  if (!P) return SG_OK;
  SG_TRY(select_idx(ctx, P->c_pend, P->tcl, P->d_num, P->ncl));
  SG_CUDA(ctx, cudaMemcpyAsync(count, P->d_num, 4, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaMemsetAsync(P->c_pend, 0, P->ncl, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *list = P->tcl;
  return SG_OK;
}


bool repair_active(const SummaryDev& D) { return D.rep != nullptr; }

SpLists repair_lists(const SummaryDev& D) {
  SpLists L;
  const RepairDev* P = D.rep;
  if (!P) return L;
  L.slot = P->blk;
  L.row_sp = P->f_sp;
  L.row_inner = P->row_inner;
  L.is_cnt = P->is_cnt;
  L.iv_cnt = P->iv_cnt;
  L.id_cnt = P->id_cnt;
  L.is_nbr = P->pool.is_nbr;
  L.iv_nbr = P->pool.iv_nbr;
  L.id_nbr = P->pool.id_nbr;
  L.is_w = P->pool.is_w;
  L.iv_w = P->pool.iv_w;
  L.id_w = P->pool.id_w;
  L.pool = P->pool_used;
  L.sp_rows = P->sp_rows;
  L.n_sp = P->n_sp;
  return L;
}

namespace {

// the summarized CSR and correction lists from the SSSP distance blocks
sg_status rp_sketch(sg_ctx* ctx, SummaryDev& D, RepairDev& P, const RepArgs& R) {
  cudaStream_t st = ctx->stream;
  const uint32_t all = P.all_n;
  SG_TRY(reserve(ctx, D, &D.sk_deg, all));
  SG_TRY(reserve(ctx, D, &D.sk_off, (uint64_t)all + 1));
  SkArgs K{};
  K.blk = P.blk;
  K.sd = P.sd;
  K.ib_off = D.ib_off;
  K.ib_nbr = D.ib_nbr;
  K.ib_w = P.ib_w;
  K.deg = D.sk_deg;
  K.pad = P.cnt_a;
  K.ccnt = P.cnt_b;
  K.fcorr = P.f_corr;
  k_rp_sketch<false><<<grid_for(all, 256), 256, 0, st>>>(R, K);
  SG_TRY(scan_u64(ctx, P.cnt_a, D.sk_off, (uint64_t)all + 1));
  SG_TRY(scan_u64(ctx, P.cnt_b, P.cnt_c, (uint64_t)all + 1));
  SG_TRY(reserve(ctx, D, &D.sk_crow, all));
  SG_TRY(select_idx(ctx, P.f_corr, D.sk_crow, P.d_num, all));
  uint64_t tot[2] = {0, 0};
  uint32_t ncorr = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&tot[0], D.sk_off + all, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(&tot[1], P.cnt_c + all, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaMemcpyAsync(&ncorr, P.d_num, 4, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  SG_TRY(reserve(ctx, D, &D.sk_col, tot[0] + 4));
  SG_TRY(reserve(ctx, D, &D.sk_w, tot[0] + 4));
  SG_TRY(reserve(ctx, D, &D.sk_cv, tot[1]));
  SG_TRY(reserve(ctx, D, &D.sk_cd, tot[1]));
  SG_TRY(reserve(ctx, D, &D.sk_coff, (uint64_t)ncorr + 1));
  SG_CUDA(ctx, cudaMemsetAsync(D.sk_col, 0, 4 * (tot[0] + 4), st));
  SG_CUDA(ctx, cudaMemsetAsync(D.sk_w, 0, 4 * (tot[0] + 4), st));
  K.off = D.sk_off;
  K.col = D.sk_col;
  K.w = D.sk_w;
  K.coff = P.cnt_c;
  K.cv = D.sk_cv;
  K.cd = D.sk_cd;
  k_rp_sketch<true><<<grid_for(all, 256), 256, 0, st>>>(R, K);
  k_rp_gather_off<<<grid_for((uint64_t)ncorr + 1, 256), 256, 0, st>>>(D.sk_crow, ncorr, P.cnt_c, tot[1],
                                                                     D.sk_coff);
  SG_TRY(reserve(ctx, D, &D.sk_spid, std::max<uint32_t>(P.n_sp, 1)));
  if (P.n_sp)
    SG_CUDA(ctx, cudaMemcpyAsync(D.sk_spid, P.sp_rows, 4ull * P.n_sp, cudaMemcpyDeviceToDevice, st));
  SG_TRY(reserve(ctx, D, &D.sk_imir, std::max<uint32_t>(P.n_im_total, 1)));
  SG_TRY(reserve(ctx, D, &D.sk_imaster, std::max<uint32_t>(P.n_im_total, 1)));
  if (P.n_im_total) {
    SG_CUDA(ctx, cudaMemcpyAsync(D.sk_imir, P.im_list, 4ull * P.n_im_total, cudaMemcpyDeviceToDevice,
                                 st));
    SG_CUDA(ctx, cudaMemcpyAsync(D.sk_imaster, P.im_master, 4ull * P.n_im_total,
                                 cudaMemcpyDeviceToDevice, st));
  }
  count_launch(ctx, 6);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  D.sk_m = tot[0];
  D.sk_ncorr = ncorr;
  D.sk_nspid = P.n_sp;
  D.sk_nimir = P.n_im_total;
  P.sk_stale = false;
  return SG_OK;
}

}  // namespace

sg_status repair_sssp_refresh(sg_ctx* ctx, SummaryDev& D) {
  RepairDev* Pp = D.rep;
  if (!Pp) return fail(ctx, SG_ERR_STATE, "no device summary");
  RepairDev& P = *Pp;
  cudaStream_t st = ctx->stream;
  PhaseTrace T("device SSSP summary");
  const RepArgs R = rep_args(ctx, P);
  if (!P.sssp_on) {
    // every supernode's distances (and its PageRank solve again) once
    P.sssp_on = true;
    SG_CUDA(ctx, cudaMemsetAsync(P.c_src, 1, P.ncl, st));
    SG_TRY(reserve(ctx, D, &D.out_deg_all, P.all_n));
    k_rp_rows<<<grid_for(P.all_n, 256), 256, 0, st>>>(R, P.r_size, P.f_sp, D.out_deg_all);
    count_launch(ctx);
    SG_TRY(rp_rebuild(ctx, D, P, R, T));
  }
  if (P.sk_stale) SG_TRY(rp_sketch(ctx, D, P, R));
  T.mark("summarized CSR", st);
  D.sssp_ready = true;
  return SG_OK;
}

sg_status repair_source_seeds(sg_ctx* ctx, SummaryDev& D, uint32_t source, const uint32_t** v,
                              const double** d, uint32_t* count) {
  RepairDev* Pp = D.rep;
  *count = 0;
  *v = nullptr;
  *d = nullptr;
  if (!Pp) return SG_OK;
  RepairDev& P = *Pp;
  const Summary& S = D.S;  // membership and local indices are fixed after the build
  if (source >= S.old_n) return SG_OK;
  const uint32_t c = S.id2spids[source];
  if (c == Summary::kIdDefault || c >= P.ncl) return SG_OK;
  const auto& nodes = S.cluster_ids[c];
  uint32_t loc = 0;
  while (loc < nodes.size() && nodes[loc] != source) ++loc;
  if (loc == nodes.size()) return fail(ctx, SG_ERR_STATE, "source missing from its cluster");
  cudaStream_t st = ctx->stream;
  const RepArgs R = rep_args(ctx, P);
  SG_CUDA(ctx, cudaMemcpyAsync(P.tcl, &c, 4, cudaMemcpyHostToDevice, st));
  uint64_t npos = 0;
  SG_TRY(rp_local_problems(ctx, P, R, 1, &npos));
  const uint32_t zero = 0;
  const uint64_t zero64 = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(P.sp_cl, &zero, 4, cudaMemcpyHostToDevice, st));
  SG_CUDA(ctx, cudaMemcpyAsync(P.sp_src, &loc, 4, cudaMemcpyHostToDevice, st));
  SG_CUDA(ctx, cudaMemcpyAsync(P.out_off, &zero64, 8, cudaMemcpyHostToDevice, st));
  SG_TRY(rp_sssp_solve(ctx, P, 1, P.out_off, P.src_dist, ctx->stream));
  SG_CUDA(ctx, cudaMemsetAsync(P.seed_n, 0, 4, st));
  k_rp_seeds<<<1, 256, 0, st>>>(R, c, P.src_dist, P.seed_v, P.seed_d, P.seed_n);
  count_launch(ctx);
  SG_CUDA(ctx, cudaMemcpyAsync(count, P.seed_n, 4, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  SG_CUDA(ctx, cudaGetLastError());
  *v = P.seed_v;
  *d = P.seed_d;
  return SG_OK;
}

uint64_t repair_logged_actions(const SummaryDev& D) { return D.rep ? D.rep->log_n : 0; }

uint64_t repair_logged_batches(const SummaryDev& D) { return D.rep ? D.rep->log_end.size() : 0; }

sg_status repair_take_log(sg_ctx* ctx, SummaryDev& D, std::vector<uint32_t>* src,
                          std::vector<uint32_t>* dst, std::vector<uint32_t>* kind,
                          std::vector<uint32_t>* found, std::vector<float>* w,
                          std::vector<uint64_t>* batch_end) {
  RepairDev* P = D.rep;
  batch_end->clear();
  if (!P) return SG_OK;
  const uint64_t na = P->log_n;
  src->resize(na);
  dst->resize(na);
  kind->resize(na);
  found->resize(na);
  w->resize(na);
  cudaStream_t st = ctx->stream;
  if (na) {
    SG_CUDA(ctx, cudaMemcpyAsync(src->data(), P->log_src, 4 * na, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaMemcpyAsync(dst->data(), P->log_dst, 4 * na, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaMemcpyAsync(kind->data(), P->log_kind, 4 * na, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaMemcpyAsync(found->data(), P->log_found, 4 * na, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaMemcpyAsync(w->data(), P->log_w, 4 * na, cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
  }
  *batch_end = P->log_end;
  P->log_n = 0;
  P->log_end.clear();
  return SG_OK;
}

}  // namespace sg
