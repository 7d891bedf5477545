// Summarized-graph PageRank on the device (the reference's SumInc PR path).
//
//   shortcut precompute   one CTA per supernode runs the cluster-local
//                         delta iteration from its entry (delta = 1 at the
//                         entry) in shared memory with FP64 accumulation and
//                         returns the converged values / residual deltas
//                         (build_iter_index_mirror, iter_compressor.h:318-491)
//   cluster precompute    one CTA per cluster converges the current deltas
//                         inside the cluster; exits then push the mass that
//                         passed through them out of the cluster
//                         (first_step + precompute_spnode_one/two,
//                         sum_sync_iter_worker.h:348-438,
//                         iter_compressor.h:534-785)
//   summarized rounds     entries push deltas along shortcuts into exit
//                         buffers, exits push along boundary edges (and
//                         masters through their in-mirrors' shortcuts),
//                         unclustered vertices push along all their edges,
//                         out-mirrors hand their buffer to the master
//                         (sum_sync_iter_worker.h:949-1127)
//   correction            accumulated entry mass flows to the inner vertices
//                         through inner_delta / inner_value
//                         (sum_sync_iter_worker.h:1385-1492)
// after which the plain rounds of pagerank.cu finish the residual.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <unordered_map>

#include "ctx.h"
#include "dev.cuh"
#include "summary.h"
#include "summary_dev.h"

namespace sg {

void host_transpose(const HostAdj& out, HostAdj& in);
void host_adj_from_csr(uint32_t n, const uint64_t* rp, const uint32_t* col, const float* w,
                       HostAdj& out);

static SummaryDev* sdev(sg_ctx* ctx) { return (SummaryDev*)ctx->summary; }

static void sfree(SummaryDev& D) {
  dfree(D.ib_off); dfree(D.sync_off);
  dfree(D.ib_nbr); dfree(D.sync_nbr);
  dfree(D.out_deg_all);
  dfree(D.l_entry); dfree(D.l_exit); dfree(D.l_single); dfree(D.l_omirror);
  dfree(D.omirror_master); dfree(D.ntype);
  dfree(D.cm_off); dfree(D.sub_off); dfree(D.cm_v); dfree(D.sub_nbr);
  dfree(D.lin_off); dfree(D.lin_src); dfree(D.lout_off); dfree(D.lout_dst);
  dfree(D.bound_list); dfree(D.bl_off);
  dfree(D.bound); dfree(D.spnode); dfree(D.old_x); dfree(D.d_res); dfree(D.sctl);
  dfree(D.sk_off); dfree(D.sk_coff); dfree(D.sk_deg); dfree(D.sk_col); dfree(D.sk_crow);
  dfree(D.sk_cv); dfree(D.sk_w); dfree(D.sk_cd);
  dfree(D.sk_spid); dfree(D.sk_imir); dfree(D.sk_imaster);
  dfree(D.p_cls); dfree(D.p_ie_off); dfree(D.p_bd_off);
  dfree(D.p_ie_nbr); dfree(D.p_bd_src); dfree(D.p_act); dfree(D.p_ent); dfree(D.p_bd_w);
  for (auto& st : D.stage) {
    dfree(st.p);
    st = SummaryDev::Stage();
  }
  sssp_view_scratch_free(D.view);
  repair_free(D);
  D.dcap.clear();
}

sg_status summary_free(sg_ctx* ctx) {
  SummaryDev* D = sdev(ctx);
  if (!D) return SG_OK;
  sfree(*D);
  delete D;
  ctx->summary = nullptr;
  return SG_OK;
}

// Host staging vectors that skip value-initialisation: the large per-batch
// tables are written in full before they are uploaded, so zero-filling them
// first only costs time.
template <typename T>
struct NoInitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() noexcept = default;
  template <typename U>
  NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
  template <typename U>
  void construct(U* p) noexcept {
    ::new ((void*)p) U;
  }
  template <typename U, typename... Args>
  void construct(U* p, Args&&... args) {
    ::new ((void*)p) U(std::forward<Args>(args)...);
  }
};
template <typename T>
using hvec = std::vector<T, NoInitAlloc<T>>;

template <typename T, typename A>
static sg_status upload(sg_ctx* ctx, T** d, const std::vector<T, A>& h) {
  dfree(*d);
  SG_TRY(dalloc(ctx, d, std::max<size_t>(h.size(), 1)));
  if (!h.empty())
    SG_CUDA(ctx, cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
  return SG_OK;
}

// The same for the tables rebuilt after every batch: the device array is
// kept while it is large enough (capacities in D.dcap, with 1/8 slack), so
// a batch costs a copy instead of a free, an allocation and a copy.
template <typename T, typename A>
static sg_status reupload(sg_ctx* ctx, SummaryDev& D, T** d, const std::vector<T, A>& h) {
  const uint64_t need = std::max<size_t>(h.size(), 1);
  auto it = D.dcap.find((const void*)d);
  if (!*d || it == D.dcap.end() || it->second < need) {
    dfree(*d);
    const uint64_t cap = need + need / 8;
    SG_TRY(dalloc(ctx, d, cap));
    D.dcap[(const void*)d] = cap;
  }
  if (!h.empty())
    SG_CUDA(ctx, cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
  return SG_OK;
}

// Staging slots: the device buffer of a slot is kept and grown (1/8 slack)
// across calls.  Callers synchronise before returning, so a slot is free
// again at the next call.
enum StageSlot {
  ST_HJOBS, ST_WJOBS, ST_WJOBS5, ST_BJOBS, ST_LINOFF, ST_LINSRC, ST_SPC, ST_SRC, ST_INNER, ST_ADJ, ST_CLOFF,
  ST_ADJOFF, ST_OUTOFF, ST_DIV, ST_VAL, ST_DEL,
  SI_DALL, SI_SEEDS, SI_S2, SP_DIST, ST_SLOTS
};
static_assert(ST_SLOTS <= 32, "staging slots");

template <typename T>
static sg_status stage_alloc(sg_ctx* ctx, SummaryDev& D, int slot, uint64_t count, T** out) {
  SummaryDev::Stage& s = D.stage[slot];
  const size_t need = (size_t)std::max<uint64_t>(count, 1) * sizeof(T);
  if (s.cap < need) {
    dfree(s.p);
    s.p = nullptr;
    s.cap = 0;
    char* p = nullptr;
    SG_TRY(dalloc(ctx, &p, need + need / 8));
    s.p = p;
    s.cap = need + need / 8;
  }
  *out = (T*)s.p;
  return SG_OK;
}

template <typename T, typename A>
static sg_status stage_up(sg_ctx* ctx, SummaryDev& D, int slot, const std::vector<T, A>& h,
                          T** out) {
  SG_TRY(stage_alloc(ctx, D, slot, h.size(), out));
  if (!h.empty())
    SG_CUDA(ctx, cudaMemcpyAsync(*out, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
  return SG_OK;
}

// ------------------------------------------------------ shortcut kernel


// Both kernels iterate like the reference's local sweep
// (inc_run_to_convergence_mirror, iter_compressor.h:350-430): deltas, the
// values pushed along edges (the reference's value_t for PageRank: delta
// times d / out_degree) and the delta mass of a step (its float Diff) in
// FP32.  The shortcut value of every node accumulates in FP64: each node
// sums its deltas of eight steps in FP32 and adds that partial sum to its
// FP64 value (GB300 issues a warp's FP64 add at a small fraction of the FP32
// rate, and one per node and step held the kernel at the FP64 pipe's limit).
constexpr int kShortcutFlush = 8;

// One CTA per supernode job (clusters of any size).
__global__ void __launch_bounds__(128) k_shortcuts(ShortcutArgs A, uint32_t njobs) {
  extern __shared__ double sm[];
  if (blockIdx.x >= njobs) return;
  const uint32_t s = A.jobs ? A.jobs[blockIdx.x] : blockIdx.x;
  if (s >= A.n_sp) return;
  const uint32_t c = A.sp_cluster[s];
  const uint64_t l0 = A.cl_off[c];
  const uint32_t L = (uint32_t)(A.cl_off[c + 1] - l0);
  const uint32_t inner = A.cl_inner[c];
  const uint32_t src = A.sp_src[s];
  const float d = A.damping;
  double* value = sm;                    // [L]
  float* delta = (float*)(sm + L);       // [L]
  float* next = delta + L;               // [L]
  float* part = next + L;                // [L] partial sums of the current eight steps
  __shared__ float s_diff;
  for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) {
    value[i] = 0.0;
    delta[i] = (i == src) ? 1.f : 0.f;
    part[i] = 0.f;
  }
  __syncthreads();
  // an in-mirror entry first sends its unit along its edges into the cluster
  if (src >= inner) {
    const uint64_t e0 = A.adj_off[l0 + src], e1 = A.adj_off[l0 + src + 1];
    const float outv = d / A.div[l0 + src];
    for (uint64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) atomicAdd(&delta[A.adj_nbr[e]], outv);
    __syncthreads();
    if (threadIdx.x == 0) {
      value[src] += 1.0;
      delta[src] = 0.f;
    }
    __syncthreads();
  }
  const float thr = f32_at_most(A.thr_per_node * (double)inner);
  for (int step = 1;; ++step) {
    if (threadIdx.x == 0) s_diff = 0.f;
    for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) next[i] = i < inner ? 0.f : delta[i];
    __syncthreads();
    float diff = 0.f;
    const bool flush = step % kShortcutFlush == 0;
    for (uint32_t i = threadIdx.x; i < inner; i += blockDim.x) {
      const float ts = delta[i];
      const float p = part[i] + ts;
      if (flush) {
        value[i] += widen_f32(p);
        part[i] = 0.f;
      } else {
        part[i] = p;
      }
      if (ts == 0.f) continue;
      diff += fabsf(ts);
      const float outv = ts * (d / A.div[l0 + i]);
      for (uint64_t e = A.adj_off[l0 + i]; e < A.adj_off[l0 + i + 1]; ++e)
        atomicAdd(&next[A.adj_nbr[e]], outv);
    }
    if (diff != 0.f) atomicAdd(&s_diff, diff);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) delta[i] = next[i];
    __syncthreads();
    const float d_all = s_diff;
    __syncthreads();
    if (d_all <= thr || step > 100) break;
  }
  const uint64_t o = A.out_off[s];
  for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) {
    A.out_value[o + i] = i < inner ? value[i] + widen_f32(part[i]) : value[i];
    A.out_delta[o + i] = (double)delta[i];
  }
}

// G lanes per supernode job (a warp, or half a warp for two jobs) for
// clusters of at most G x NPL local nodes: the same iteration as
// k_shortcuts (a unit of delta at the entry, Jacobi steps until the
// members' delta mass is at most thr x members or 101 steps) in two phases
// per step without atomics: members take their delta and publish
// delta * d / div, then every node sums the published values of its
// in-edges from members (mirrors keep what they hold).  Lane l of a group
// owns nodes l, l + G, ..., and keeps their delta, partial sum, FP64 value,
// d / div and in-edge range in registers; only the published values go
// through shared memory.  The two jobs of a warp step together until both
// have stopped; a stopped job's state no longer changes.
template <int NPL, int G>
__global__ void __launch_bounds__(256) k_shortcuts_warp(ShortcutArgs A, uint32_t njobs) {
  constexpr uint32_t JPW = 32 / G;  // jobs per warp
  __shared__ float s_pv[kStageWarps][32 * NPL];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t h = lane / G, sl = lane % G;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const float d = A.damping;
  float* pv = s_pv[w] + h * G * NPL;
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * JPW; base < njobs;
       base += nwarps * JPW) {
    const uint32_t jj = base + h;
    const bool valid = jj < njobs;
    uint32_t s = 0, L = 0, inner = 0, src = 0;
    uint64_t l0 = 0, e_base = 0;
    if (valid) {
      s = A.jobs[jj];
      const uint32_t c = A.sp_cluster[s];
      l0 = A.cl_off[c];
      L = (uint32_t)(A.cl_off[c + 1] - l0);
      inner = A.cl_inner[c];
      src = A.sp_src[s];
      e_base = A.lin_off[l0];
    }
    float del[NPL], part[NPL], f[NPL];
    double val[NPL];
    uint32_t e0[NPL], e1[NPL];
#pragma unroll
    for (int t = 0; t < NPL; ++t) {
      const uint32_t j = sl + G * t;
      val[t] = 0.0;
      part[t] = 0.f;
      del[t] = 0.f;
      f[t] = 0.f;
      e0[t] = e1[t] = 0;
      if (j < L) {
        f[t] = d / A.div[l0 + j];
        e0[t] = (uint32_t)(A.lin_off[l0 + j] - e_base);
        e1[t] = (uint32_t)(A.lin_off[l0 + j + 1] - e_base);
        del[t] = j == src ? 1.f : 0.f;
      }
    }
    // an in-mirror entry first sends its unit along its edges into the
    // cluster (through shared memory: its targets belong to other lanes)
    const bool mirror_src = valid && src >= inner;
    if (__any_sync(0xffffffffu, mirror_src)) {
#pragma unroll
      for (int t = 0; t < NPL; ++t)
        if (sl + G * t < L) pv[sl + G * t] = 0.f;
      __syncwarp();
      if (sl == 0 && mirror_src) {
        const float outv = d / A.div[l0 + src];
        for (uint64_t e = A.adj_off[l0 + src]; e < A.adj_off[l0 + src + 1]; ++e)
          pv[A.adj_nbr[e]] += outv;
      }
      __syncwarp();
      if (mirror_src) {
#pragma unroll
        for (int t = 0; t < NPL; ++t) {
          const uint32_t j = sl + G * t;
          if (j < L) {
            if (j == src) {
              val[t] = 1.0;
              del[t] = 0.f;
            } else {
              del[t] = pv[j];
            }
          }
        }
      }
      __syncwarp();
    }
    const float thr = valid ? f32_at_most(A.thr_per_node * (double)inner) : 0.f;
    const uint8_t* ls = A.lin_src + e_base;
    bool active = valid;
    for (int step = 1;; ++step) {
      float diff = 0.f;
      const bool flush = step % kShortcutFlush == 0;
      if (active) {
#pragma unroll
        for (int t = 0; t < NPL; ++t) {
          const uint32_t j = sl + G * t;
          if (j < inner) {
            const float ts = del[t];
            const float p = part[t] + ts;
            if (flush) {
              val[t] += widen_f32(p);
              part[t] = 0.f;
            } else {
              part[t] = p;
            }
            diff += fabsf(ts);
            pv[j] = ts * f[t];
          }
        }
      }
      __syncwarp();
      if (active) {
#pragma unroll
        for (int t = 0; t < NPL; ++t) {
          const uint32_t j = sl + G * t;
          if (j < L) {
            float acc = 0.f;
            for (uint32_t e = e0[t]; e < e1[t]; ++e) acc += pv[ls[e]];
            del[t] = (j < inner ? 0.f : del[t]) + acc;
          }
        }
      }
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) diff += __shfl_xor_sync(0xffffffffu, diff, o);
      __syncwarp();
      if (active && (diff <= thr || step > 100)) active = false;
      if (!__any_sync(0xffffffffu, active)) break;
    }
    if (valid) {
      const uint64_t o = A.out_off[s];
#pragma unroll
      for (int t = 0; t < NPL; ++t) {
        const uint32_t j = sl + G * t;
        if (j < L) {
          A.out_value[o + j] = j < inner ? val[t] + widen_f32(part[t]) : val[t];
          A.out_delta[o + j] = (double)del[t];
        }
      }
    }
    __syncwarp();
  }
}
// One block per batch of jobs (no grid cap): blocks live for one solve, so
// SM slots free up all along the launch for kernels queued beside it.
void launch_shortcuts_warp(int npl, ShortcutArgs A, uint32_t njobs, cudaStream_t st) {
  constexpr int kNoCap = 1 << 30;
  if (npl == 3) {
    k_shortcuts_warp<3, 16><<<grid_for((uint64_t)njobs * 16, 32 * kStageWarps, kNoCap), 32 * kStageWarps,
                              0, st>>>(A, njobs);
    return;
  }
  const unsigned grid = grid_for((uint64_t)njobs * 32, 32 * kStageWarps, kNoCap);
  if (npl == 2) k_shortcuts_warp<2, 32><<<grid, 32 * kStageWarps, 0, st>>>(A, njobs);
  else k_shortcuts_warp<5, 32><<<grid, 32 * kStageWarps, 0, st>>>(A, njobs);
}

// Builds the local problems of the given supernodes, runs the kernel and
// writes inner_value / inner_delta / bound_delta back into the summary.
static sg_status compute_shortcuts(sg_ctx* ctx, SummaryDev& D, const std::vector<uint32_t>& spids) {
  Summary& S = D.S;
  if (spids.empty()) return SG_OK;
  // clusters involved
  std::unordered_map<uint32_t, uint32_t> cl_index;
  std::vector<uint32_t> cls;
  for (uint32_t sp : spids) {
    const uint32_t c = S.supernodes[sp].ids;
    if (cl_index.emplace(c, (uint32_t)cls.size()).second) cls.push_back(c);
  }
  // local problems, one per cluster: nodes (members, then mirrors), the
  // divisor of each, and the subgraph edges as local indices; built in two
  // parallel passes (sizes, then fills at prefix offsets).  A node's local
  // index is kept in local_of; nodes of different clusters are distinct.
  const size_t ncl = cls.size();
  std::vector<uint64_t> cl_off(ncl + 1, 0), cl_adj(ncl + 1, 0);
  std::vector<uint32_t> cl_inner(ncl);
  std::vector<uint32_t> local_of(S.all_n, 0xFFFFFFFFu);
  size_t maxL = 1;
  for (size_t k = 0; k < ncl; ++k) {
    const auto& nodes = S.cluster_ids[cls[k]];  // members first, then mirror ids
    cl_off[k + 1] = cl_off[k] + nodes.size();
    maxL = std::max(maxL, nodes.size());
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (long long k = 0; k < (long long)ncl; ++k) {
    const auto& nodes = S.cluster_ids[cls[k]];
    uint64_t ne = 0;
    for (uint32_t i = 0; i < nodes.size(); ++i) {
      local_of[nodes[i]] = i;
      ne += S.subgraph[nodes[i]].size();
    }
    cl_adj[k + 1] = ne;
    cl_inner[k] = (uint32_t)S.supernode_ids[cls[k]].size();
  }
  for (size_t k = 0; k < ncl; ++k) cl_adj[k + 1] += cl_adj[k];
  std::vector<uint64_t> adj_off(cl_off[ncl] + 1);
  std::vector<uint32_t> adj_nbr(cl_adj[ncl]);
  std::vector<float> div(cl_off[ncl]);
  bool foreign = false;
#pragma omp parallel for schedule(dynamic, 256) reduction(|| : foreign)
  for (long long k = 0; k < (long long)ncl; ++k) {
    const auto& nodes = S.cluster_ids[cls[k]];
    uint64_t e = cl_adj[k];
    for (uint32_t i = 0; i < nodes.size(); ++i) {
      const uint32_t v = nodes[i];
      const uint32_t master = v < S.old_n ? v : S.mirror_master(v);
      div[cl_off[k] + i] = (float)std::max<uint64_t>(D.out.deg(master), 1);
      adj_off[cl_off[k] + i] = e;
      for (uint32_t t : S.subgraph[v]) {
        const uint32_t l = local_of[t];
        // every subgraph edge stays inside its cluster's nodes
        if (l >= nodes.size() || nodes[l] != t) foreign = true;
        adj_nbr[e++] = l < nodes.size() ? l : 0u;
      }
    }
  }
  adj_off[cl_off[ncl]] = cl_adj[ncl];
  if (foreign) return fail(ctx, SG_ERR_STATE, "subgraph edge leaves its cluster");
  std::vector<uint32_t> sp_cluster(spids.size()), sp_src(spids.size());
  std::vector<uint64_t> out_off(spids.size() + 1, 0);
  for (size_t j = 0; j < spids.size(); ++j) {
    const Supernode& sp = S.supernodes[spids[j]];
    const uint32_t k = cl_index[sp.ids];
    sp_cluster[j] = k;
    const auto& nodes = S.cluster_ids[sp.ids];
    const uint32_t l = local_of[sp.id];
    sp_src[j] = (l < nodes.size() && nodes[l] == sp.id) ? l : 0u;
    out_off[j + 1] = out_off[j] + (cl_off[k + 1] - cl_off[k]);
  }
  // in-edges from members per local node of clusters with at most
  // kStageCap nodes (warp kernel), in two parallel passes
  std::vector<uint64_t> cl_lin(ncl + 1, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (long long k = 0; k < (long long)ncl; ++k) {
    const uint64_t L = cl_off[k + 1] - cl_off[k];
    if (L > (uint64_t)kStageCap) continue;
    uint64_t c = 0;
    for (uint32_t i = 0; i < cl_inner[k]; ++i)
      c += adj_off[cl_off[k] + i + 1] - adj_off[cl_off[k] + i];
    cl_lin[k + 1] = c;
  }
  for (size_t k = 0; k < ncl; ++k) cl_lin[k + 1] += cl_lin[k];
  std::vector<uint64_t> lin_off(cl_off[ncl] + 1);
  std::vector<uint8_t> lin_src(cl_lin[ncl]);
#pragma omp parallel for schedule(dynamic, 256)
  for (long long k = 0; k < (long long)ncl; ++k) {
    const uint64_t b = cl_off[k];
    const uint32_t L = (uint32_t)(cl_off[k + 1] - b);
    if (L > (uint32_t)kStageCap) {
      for (uint32_t j = 0; j < L; ++j) lin_off[b + j] = cl_lin[k];
      continue;
    }
    uint32_t cnt[kStageCap + 1];
    for (uint32_t j = 0; j <= L; ++j) cnt[j] = 0;
    for (uint32_t i = 0; i < cl_inner[k]; ++i)
      for (uint64_t e = adj_off[b + i]; e < adj_off[b + i + 1]; ++e) ++cnt[adj_nbr[e] + 1];
    for (uint32_t j = 0; j < L; ++j) cnt[j + 1] += cnt[j];
    for (uint32_t j = 0; j < L; ++j) lin_off[b + j] = cl_lin[k] + cnt[j];
    for (uint32_t i = 0; i < cl_inner[k]; ++i)
      for (uint64_t e = adj_off[b + i]; e < adj_off[b + i + 1]; ++e)
        lin_src[cl_lin[k] + cnt[adj_nbr[e]]++] = (uint8_t)i;
  }
  lin_off[cl_off[ncl]] = cl_lin[ncl];
  std::vector<uint32_t> half_jobs, warp_jobs, warp_jobs5, block_jobs;
  size_t maxL_block = 1;
  for (size_t j = 0; j < spids.size(); ++j) {
    const uint32_t k = sp_cluster[j];
    const uint64_t L = cl_off[k + 1] - cl_off[k];
    if (L <= (uint64_t)kShortcutHalfL) {
      half_jobs.push_back((uint32_t)j);
    } else if (L <= (uint64_t)kShortcutSmallL) {
      warp_jobs.push_back((uint32_t)j);
    } else if (L <= (uint64_t)kStageCap) {
      warp_jobs5.push_back((uint32_t)j);
    } else {
      block_jobs.push_back((uint32_t)j);
      maxL_block = std::max<size_t>(maxL_block, L);
    }
  }
  (void)maxL;
  const size_t smem = shortcut_smem(maxL_block);
  if (smem > 200 * 1024) return fail(ctx, SG_ERR_UNSUPPORTED, "cluster too large for the shortcut kernel");
  uint32_t *d_spc = nullptr, *d_src = nullptr, *d_inner = nullptr, *d_adj = nullptr;
  uint64_t *d_cloff = nullptr, *d_adjoff = nullptr, *d_outoff = nullptr;
  float* d_div = nullptr;
  double *d_val = nullptr, *d_del = nullptr;
  uint32_t *d_wjobs = nullptr, *d_bjobs = nullptr;
  uint64_t* d_linoff = nullptr;
  uint8_t* d_linsrc = nullptr;
  uint32_t *d_wjobs5 = nullptr, *d_hjobs = nullptr;
  SG_TRY(stage_up(ctx, D, ST_HJOBS, half_jobs, &d_hjobs));
  SG_TRY(stage_up(ctx, D, ST_WJOBS, warp_jobs, &d_wjobs));
  SG_TRY(stage_up(ctx, D, ST_WJOBS5, warp_jobs5, &d_wjobs5));
  SG_TRY(stage_up(ctx, D, ST_BJOBS, block_jobs, &d_bjobs));
  SG_TRY(stage_up(ctx, D, ST_LINOFF, lin_off, &d_linoff));
  SG_TRY(stage_up(ctx, D, ST_LINSRC, lin_src, &d_linsrc));
  SG_TRY(stage_up(ctx, D, ST_SPC, sp_cluster, &d_spc));
  SG_TRY(stage_up(ctx, D, ST_SRC, sp_src, &d_src));
  SG_TRY(stage_up(ctx, D, ST_INNER, cl_inner, &d_inner));
  SG_TRY(stage_up(ctx, D, ST_ADJ, adj_nbr, &d_adj));
  SG_TRY(stage_up(ctx, D, ST_CLOFF, cl_off, &d_cloff));
  SG_TRY(stage_up(ctx, D, ST_ADJOFF, adj_off, &d_adjoff));
  SG_TRY(stage_up(ctx, D, ST_OUTOFF, out_off, &d_outoff));
  SG_TRY(stage_up(ctx, D, ST_DIV, div, &d_div));
  SG_TRY(stage_alloc(ctx, D, ST_VAL, out_off.back(), &d_val));
  SG_TRY(stage_alloc(ctx, D, ST_DEL, out_off.back(), &d_del));
  ShortcutArgs A;
  A.n_sp = (uint32_t)spids.size();
  A.sp_cluster = d_spc;
  A.sp_src = d_src;
  A.cl_off = d_cloff;
  A.cl_inner = d_inner;
  A.adj_off = d_adjoff;
  A.adj_nbr = d_adj;
  A.div = d_div;
  A.out_off = d_outoff;
  A.out_value = d_val;
  A.out_delta = d_del;
  A.damping = (float)ctx->opt.damping;
  A.thr_per_node = ctx->opt.termcheck_threshold / (double)S.old_n;
  A.lin_off = d_linoff;
  A.lin_src = d_linsrc;
  if (smem > 48 * 1024)
    SG_CUDA(ctx, cudaFuncSetAttribute(k_shortcuts, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  kprof_begin(ctx);
  if (!half_jobs.empty()) {
    A.jobs = d_hjobs;
    launch_shortcuts_warp(3, A, (uint32_t)half_jobs.size(), ctx->stream);
  }
  if (!warp_jobs.empty()) {
    A.jobs = d_wjobs;
    launch_shortcuts_warp(2, A, (uint32_t)warp_jobs.size(), ctx->stream);
  }
  if (!warp_jobs5.empty()) {
    A.jobs = d_wjobs5;
    launch_shortcuts_warp(5, A, (uint32_t)warp_jobs5.size(), ctx->stream);
  }
  if (!block_jobs.empty()) {
    A.jobs = d_bjobs;
    k_shortcuts<<<(unsigned)block_jobs.size(), 128, smem, ctx->stream>>>(A, (uint32_t)block_jobs.size());
  }
  kprof_end(ctx, SG_K_SUMMARY);
  SG_CUDA(ctx, cudaGetLastError());
  hvec<double> val(out_off.back()), del(out_off.back());
  SG_CUDA(ctx, cudaMemcpyAsync(val.data(), d_val, 8 * val.size(), cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaMemcpyAsync(del.data(), d_del, 8 * del.size(), cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  // fianl_build_iter_index_for_mirror (iter_compressor.h:433-491); each
  // supernode writes only its own lists
#pragma omp parallel for schedule(dynamic, 256)
  for (long long j = 0; j < (long long)spids.size(); ++j) {
    Supernode& sp = S.supernodes[spids[j]];
    const uint32_t c = sp.ids;
    const auto& nodes = S.cluster_ids[c];
    const uint32_t inner = (uint32_t)S.supernode_ids[c].size();
    const uint64_t o = out_off[j];
    sp.inner_value.clear();
    sp.inner_delta.clear();
    sp.bound_delta.clear();
    sp.status = true;
    for (uint32_t i = 0; i < inner; ++i) {
      const uint32_t v = nodes[i];
      if (val[o + i] != 0.0) {
        if (S.out_bound[v]) sp.bound_delta.push_back({v, val[o + i]});
        else sp.inner_value.push_back({v, val[o + i]});
      }
      if (del[o + i] != 0.0) sp.inner_delta.push_back({v, del[o + i]});
    }
    const auto& om = S.cluster_out_mirror_ids[c];
    for (uint32_t m : om) {
      const uint32_t i = local_of[m];
      if (i >= nodes.size() || nodes[i] != m) continue;
      const double v = val[o + i] + del[o + i];
      if (v != 0.0) sp.bound_delta.push_back({m, v});
    }
  }
  return SG_OK;
}

// ------------------------------------------------------ device sketch upload

static sg_status upload_sketch(sg_ctx* ctx, SummaryDev& D) {
  Summary& S = D.S;
  const uint32_t all = S.all_n, n = S.old_n;
  SG_TRY(reupload(ctx, D, &D.ib_off, S.ib_off));
  SG_TRY(reupload(ctx, D, &D.ib_nbr, S.ib_nbr));
  SG_TRY(reupload(ctx, D, &D.sync_off, S.sync_off));
  SG_TRY(reupload(ctx, D, &D.sync_nbr, S.sync_nbr));
  std::vector<uint32_t> odeg(all);
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)all; ++v)
    odeg[v] = (uint32_t)D.out.deg(v < n ? (uint32_t)v : S.mirror_master((uint32_t)v));
  SG_TRY(reupload(ctx, D, &D.out_deg_all, odeg));
  std::vector<uint32_t> le, lx, ls;
  std::vector<uint8_t> nt(n);
  for (uint32_t v = 0; v < n; ++v) {
    const char t = S.node_type[v];
    nt[v] = (uint8_t)t;
    if (t == kOnlyIn || t == kBothOutIn || t == kBothOutInMaster) le.push_back(v);
    if (t == kOnlyOut || t == kBothOutIn || t == kOutMaster || t == kBothOutInMaster) lx.push_back(v);
    if (t == kSingle) ls.push_back(v);
  }
  SG_TRY(reupload(ctx, D, &D.ntype, nt));
  SG_TRY(reupload(ctx, D, &D.l_entry, le));
  SG_TRY(reupload(ctx, D, &D.l_exit, lx));
  SG_TRY(reupload(ctx, D, &D.l_single, ls));
  D.n_entry = (uint32_t)le.size();
  D.n_exit = (uint32_t)lx.size();
  D.n_single = (uint32_t)ls.size();
  std::vector<uint32_t> om, omm;
  for (uint32_t m : S.all_out_mirror) {
    om.push_back(m);
    omm.push_back(S.mirror_master(m));
  }
  SG_TRY(reupload(ctx, D, &D.l_omirror, om));
  SG_TRY(reupload(ctx, D, &D.omirror_master, omm));
  D.n_omirror = (uint32_t)om.size();
  // the supernode lists (shortcuts and correction) live in the device
  // repair's slots (repair_init)
  // Cluster members, exits and the precompute lists, all per member
  // position of the cm layout, built in two parallel passes (counts, then
  // fills at prefix offsets).  Clusters of at most kStageCap members get
  // their local in-edges (tails as 8-bit local indices) and their edges to
  // out-mirrors; clusters that are not staged (more members, or more local
  // edges than kStageEdges) get their subgraph out-edges instead.
  const size_t ncl = S.supernode_ids.size();
  std::vector<uint64_t> cmo(ncl + 1, 0), blo(ncl + 1, 0), c_lin(ncl + 1, 0), c_lout(ncl + 1, 0),
      c_sub(ncl + 1, 0);
  std::vector<uint8_t> slot(n, 0);
  // a head inside a small cluster c (members carry their local slot)
  auto is_local = [&](uint32_t t, size_t c, const std::vector<uint32_t>& M) {
    return t < n && S.id2spids[t] == (uint32_t)c && slot[t] < M.size() && M[slot[t]] == t;
  };
#pragma omp parallel for schedule(dynamic, 512)
  for (long long c = 0; c < (long long)ncl; ++c) {
    const auto& M = S.supernode_ids[c];
    const size_t m = M.size();
    uint64_t nb = 0, nin = 0, nout = 0, nall = 0;
    for (size_t j = 0; j < m; ++j) {
      if (m <= (size_t)kStageCap) slot[M[j]] = (uint8_t)j;
      nb += S.out_bound[M[j]] != 0;
    }
    for (size_t i = 0; i < m; ++i) {
      nall += S.subgraph[M[i]].size();
      if (m <= (size_t)kStageCap)
        for (uint32_t t : S.subgraph[M[i]]) {
          if (is_local(t, c, M)) ++nin; else ++nout;
        }
    }
    cmo[c + 1] = m;
    blo[c + 1] = nb;
    const bool staged = m <= (size_t)kStageCap && nin <= (uint64_t)kStageEdges;
    c_lin[c + 1] = m <= (size_t)kStageCap ? nin : 0;
    c_lout[c + 1] = m <= (size_t)kStageCap ? nout : 0;
    c_sub[c + 1] = staged ? 0 : nall;
  }
  for (size_t c = 0; c < ncl; ++c) {
    cmo[c + 1] += cmo[c];
    blo[c + 1] += blo[c];
    c_lin[c + 1] += c_lin[c];
    c_lout[c + 1] += c_lout[c];
    c_sub[c + 1] += c_sub[c];
  }
  const uint64_t npos = cmo[ncl];
  hvec<uint32_t> cmv(npos), bl(blo[ncl]), loutd(c_lout[ncl]), subn(c_sub[ncl]);
  hvec<uint8_t> lins(c_lin[ncl]);
  hvec<uint64_t> lino(npos + 1), louto(npos + 1), subo(npos + 1);
#pragma omp parallel for schedule(dynamic, 512)
  for (long long c = 0; c < (long long)ncl; ++c) {
    const auto& M = S.supernode_ids[c];
    const size_t m = M.size();
    const uint64_t p0 = cmo[c];
    uint64_t nb = blo[c];
    for (size_t j = 0; j < m; ++j) {
      cmv[p0 + j] = M[j];
      if (S.out_bound[M[j]]) bl[nb++] = M[j];
    }
    const bool small = m <= (size_t)kStageCap;
    const bool staged = small && c_lin[c + 1] - c_lin[c] <= (uint64_t)kStageEdges;
    // local in-edges: counts per head, then tails in increasing local order
    uint32_t cnt[kStageCap + 1];
    if (small) {
      for (size_t j = 0; j <= m; ++j) cnt[j] = 0;
      for (size_t i = 0; i < m; ++i)
        for (uint32_t t : S.subgraph[M[i]])
          if (is_local(t, c, M)) ++cnt[slot[t] + 1];
      for (size_t j = 0; j < m; ++j) cnt[j + 1] += cnt[j];
      for (size_t j = 0; j < m; ++j) lino[p0 + j] = c_lin[c] + cnt[j];
      for (size_t i = 0; i < m; ++i)
        for (uint32_t t : S.subgraph[M[i]])
          if (is_local(t, c, M)) lins[c_lin[c] + cnt[slot[t]]++] = (uint8_t)i;
    } else {
      for (size_t j = 0; j < m; ++j) lino[p0 + j] = c_lin[c];
    }
    uint64_t no = c_lout[c], ns = c_sub[c];
    for (size_t i = 0; i < m; ++i) {
      louto[p0 + i] = no;
      subo[p0 + i] = ns;
      for (uint32_t t : S.subgraph[M[i]]) {
        if (small && !is_local(t, c, M)) loutd[no++] = t;
        if (!staged) subn[ns++] = t;
      }
    }
  }
  lino[npos] = c_lin[ncl];
  louto[npos] = c_lout[ncl];
  subo[npos] = c_sub[ncl];
  SG_TRY(reupload(ctx, D, &D.cm_off, cmo));
  SG_TRY(reupload(ctx, D, &D.cm_v, cmv));
  SG_TRY(reupload(ctx, D, &D.sub_off, subo));
  SG_TRY(reupload(ctx, D, &D.sub_nbr, subn));
  SG_TRY(reupload(ctx, D, &D.lin_off, lino));
  SG_TRY(reupload(ctx, D, &D.lin_src, lins));
  SG_TRY(reupload(ctx, D, &D.lout_off, louto));
  SG_TRY(reupload(ctx, D, &D.lout_dst, loutd));
  SG_TRY(reupload(ctx, D, &D.bl_off, blo));
  SG_TRY(reupload(ctx, D, &D.bound_list, bl));
  if (!D.bound) {
    SG_TRY(dalloc(ctx, &D.bound, all));
    SG_TRY(dalloc(ctx, &D.spnode, all));
    SG_TRY(dalloc(ctx, &D.old_x, n));
    SG_TRY(dalloc(ctx, &D.d_res, 2));
    SG_TRY(dalloc(ctx, &D.sctl, 4));
  }
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}


// ------------------------------------------------------ build entry point

// Shared tail of both builds: host graph copy, then `first_half` fills the
// state between the construction's halves (from a clustering or a file).
template <typename FIRST>
static sg_status summary_build_with(sg_ctx* ctx, FIRST first_half) {
  if (!ctx->g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  summary_free(ctx);
  SummaryDev* D = new SummaryDev();
  ctx->summary = D;
  // host copy of the graph (rows sorted, as the reference fragment keeps them)
  const uint32_t n = ctx->g.n;
  const uint64_t m = ctx->g.m;
  std::vector<uint64_t> rp(n + 1);
  std::vector<uint32_t> col(m);
  std::vector<float> w(ctx->g.weighted ? m : 0);
  SG_TRY(download_csr(ctx, rp.data(), col.data(), ctx->g.weighted ? w.data() : nullptr));
  host_adj_from_csr(n, rp.data(), col.data(), ctx->g.weighted ? w.data() : nullptr, D->out);
  host_transpose(D->out, D->in);
  Summary& S = D->S;
  uint64_t init_mirrors = 0;
  SG_TRY(first_half(*D, &init_mirrors));
  D->init_blob = summary_serialize_init(S, init_mirrors);
  summary_final_build(S, D->in, init_mirrors);
  summary_judge_out_bound(S, D->out, nullptr);
  summary_build_subgraph(S, D->out, D->in, nullptr);
  std::vector<uint32_t> all_sp(S.supernodes.size());
  for (uint32_t i = 0; i < all_sp.size(); ++i) all_sp[i] = i;
  SG_TRY(compute_shortcuts(ctx, *D, all_sp));
  summary_node_types(S);
  summary_sketch_csr(S, D->out);
  D->old_n = S.old_n;
  D->all_n = S.all_n;
  SG_TRY(upload_sketch(ctx, *D));
  SG_TRY(repair_init(ctx, *D));
  D->valid = true;
  return SG_OK;
}

sg_status summary_build(sg_ctx* ctx, const std::vector<std::vector<uint32_t>>& clusters) {
  return summary_build_with(ctx, [&](SummaryDev& D, uint64_t* im) {
    *im = summary_init_by_clusters(D.S, D.out, D.in, clusters, ctx->opt.min_node_num,
                                   ctx->opt.mirror_k, ctx->opt.compress_threshold);
    return SG_OK;
  });
}

sg_status summary_build_serialized(sg_ctx* ctx, const std::vector<uint8_t>& blob) {
  return summary_build_with(ctx, [&](SummaryDev& D, uint64_t* im) {
    if (!summary_deserialize_init(D.S, ctx->g.n, blob, im))
      return fail(ctx, SG_ERR_INVALID, "serialized summary does not fit this graph");
    return SG_OK;
  });
}

sg_status summary_serialized(sg_ctx* ctx, std::vector<uint8_t>* blob) {
  SummaryDev* D = sdev(ctx);
  if (!D || !D->valid) return fail(ctx, SG_ERR_STATE, "no summary built");
  *blob = D->init_blob;
  return SG_OK;
}

// ------------------------------------------------------ PageRank kernels

struct SumArgs {
  float damping;
  float thr_v;
  uint32_t old_n;
  float* x;
  float* delta;
  float* bound;
  float* spnode;
  const uint64_t *ib_off, *sync_off;
  const uint32_t *ib_nbr, *sync_nbr;
  SpLists L;  // supernode lists (slot layout)
  const uint32_t* out_deg_all;
  const uint8_t* ntype;
  unsigned long long* cnt;  // [0] edges, [1] shortcut edges
  // on-device termination of the summarized rounds: sctl [0] done, [1] blocks
  // finished in the residual pass, [2] rounds run; sres [0] running sum,
  // [1] the last round's residual
  uint32_t* sctl;
  double* sres;
  double tau;
};

__device__ __forceinline__ bool rounds_done(const SumArgs& A) {
  return *(volatile uint32_t*)A.sctl != 0u;
}

// mass a (mirror) entry receives goes along its shortcuts into exit buffers
// The round kernels give each listed row a group of G lanes (G divides 32):
// a supernode's shortcut list and an exit's boundary edges hold a few
// entries each, so several rows per warp keep more of their dependent
// loads and atomics in flight than one row per warp.
template <uint32_t G>
__device__ __forceinline__ unsigned group_mask() {
  if (G == 32) return 0xffffffffu;
  return ((1u << (G & 31)) - 1u) << ((threadIdx.x & 31) & ~(G - 1));
}

template <uint32_t G>
__device__ __forceinline__ void entry_push(const SumArgs& A, uint32_t u, float d, uint32_t gl,
                                           unsigned long long& sc) {
  const uint64_t b = A.L.slot[u], e1 = b + A.L.is_cnt[u];
  for (uint64_t e = b + gl; e < e1; e += G) atomicAdd(&A.bound[A.L.is_nbr[e]], A.L.is_w[e] * d);
  if (gl == 0) {
    atomicAdd(&A.spnode[u], d);
    sc += e1 - b;
  }
}

// the warp's sum of v into *dst (every lane of the warp calls it)
__device__ __forceinline__ void warp_add_to(unsigned long long* dst, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

template <uint32_t G>
__global__ void __launch_bounds__(256) k_sum_entries(SumArgs A, const uint32_t* list, uint32_t cnt) {
  if (rounds_done(A)) return;
  const uint32_t gl = threadIdx.x & (G - 1);
  const unsigned gm = group_mask<G>();
  unsigned long long sc = 0;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) / G; i < cnt;
       i += (gridDim.x * blockDim.x) / G) {
    const uint32_t u = list[i];
    float d = 0.f;
    if (gl == 0) {
      d = A.delta[u];
      d = fabsf(d) > A.thr_v ? atomicExch(&A.delta[u], 0.f) : 0.f;
    }
    d = __shfl_sync(gm, d, 0, G);
    if (d != 0.f) entry_push<G>(A, u, d, gl, sc);
  }
  warp_add_to(&A.cnt[1], sc);
}

template <uint32_t G>
__global__ void __launch_bounds__(256) k_sum_exits(SumArgs A, const uint32_t* list, uint32_t cnt) {
  if (rounds_done(A)) return;
  const uint32_t gl = threadIdx.x & (G - 1);
  const unsigned gm = group_mask<G>();
  unsigned long long ed = 0, sc = 0;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) / G; i < cnt;
       i += (gridDim.x * blockDim.x) / G) {
    const uint32_t u = list[i];
    float b = 0.f;
    if (gl == 0) {
      b = A.bound[u];
      b = fabsf(b) > A.thr_v ? atomicExch(&A.bound[u], 0.f) : 0.f;
      if (b != 0.f) A.x[u] += b;
    }
    b = __shfl_sync(gm, b, 0, G);
    if (b == 0.f) continue;
    // boundary edges with the original out-degree (g_function, pagerank_ingress.h:75-99)
    const float outv = b * A.damping / (float)A.out_deg_all[u];
    for (uint64_t e = A.ib_off[u] + gl; e < A.ib_off[u + 1]; e += G)
      atomicAdd(&A.delta[A.ib_nbr[e]], outv);
    if (gl == 0) ed += A.ib_off[u + 1] - A.ib_off[u];
    // a master forwards to its in-mirrors, which push at once
    const uint8_t t = A.ntype[u];
    if (t == kOutMaster || t == kBothOutInMaster) {
      for (uint64_t s = A.sync_off[u]; s < A.sync_off[u + 1]; ++s) {
        const uint32_t mm = A.sync_nbr[s];
        float dm = 0.f;
        if (gl == 0) {
          atomicAdd(&A.delta[mm], b);
          dm = atomicExch(&A.delta[mm], 0.f);
        }
        dm = __shfl_sync(gm, dm, 0, G);
        if (dm != 0.f) entry_push<G>(A, mm, dm, gl, sc);
      }
    }
  }
  warp_add_to(&A.cnt[0], ed);
  warp_add_to(&A.cnt[1], sc);
}

template <uint32_t G>
__global__ void __launch_bounds__(256) k_sum_singles(SumArgs A, const uint32_t* list, uint32_t cnt) {
  if (rounds_done(A)) return;
  const uint32_t gl = threadIdx.x & (G - 1);
  const unsigned gm = group_mask<G>();
  unsigned long long ed = 0;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) / G; i < cnt;
       i += (gridDim.x * blockDim.x) / G) {
    const uint32_t u = list[i];
    float d = 0.f;
    if (gl == 0) {
      d = A.delta[u];
      d = fabsf(d) > A.thr_v ? atomicExch(&A.delta[u], 0.f) : 0.f;
      if (d != 0.f) A.x[u] += d;
    }
    d = __shfl_sync(gm, d, 0, G);
    if (d == 0.f) continue;
    const uint64_t e0 = A.ib_off[u], e1 = A.ib_off[u + 1];
    if (e1 == e0) continue;
    const float outv = d * A.damping / (float)(e1 - e0);
    for (uint64_t e = e0 + gl; e < e1; e += G) atomicAdd(&A.delta[A.ib_nbr[e]], outv);
    if (gl == 0) ed += e1 - e0;
  }
  warp_add_to(&A.cnt[0], ed);
}

__global__ void k_sum_omirror(SumArgs A, const uint32_t* list, const uint32_t* master, uint32_t cnt) {
  if (rounds_done(A)) return;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const uint32_t m = list[i];
    if (fabsf(A.bound[m]) > A.thr_v) atomicAdd(&A.delta[master[i]], atomicExch(&A.bound[m], 0.f));
  }
}

// residual of a summarized round and, in its last block, the termination
// decision (termCheck, sum_sync_iter_worker.h:2873-2912)
__global__ void __launch_bounds__(256) k_sum_residual_decide(SumArgs A, uint32_t n) {
  __shared__ double s_red[8];
  __shared__ bool s_last;
  if (rounds_done(A)) return;
  float r = 0.f;  // the thread's vertices in FP32, the block and grid sums in FP64
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    r += fabsf(A.delta[v]);
  const double b = block_sum<256>((double)r, s_red);
  if (threadIdx.x == 0) {
    if (b != 0.0) atomicAdd(A.sres, b);
    __threadfence();
    s_last = atomicAdd(A.sctl + 1, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    const double R = atomicAdd(A.sres, 0.0);
    A.sres[0] = 0.0;
    A.sres[1] = R;
    A.sctl[1] = 0;
    A.sctl[2] += 1;
    if (R < A.tau) A.sctl[0] = 1;
  }
}

// correction through inner_delta / inner_value, a warp per supernode row
// (the other rows hold no correction lists)
__global__ void __launch_bounds__(256) k_sum_correct(SumArgs A) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < A.L.n_sp;
       i += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t u = A.L.sp_rows[i];
    const float d = A.spnode[u];
    if (!(fabsf(d) * (float)A.L.row_inner[u] > A.thr_v)) continue;
    const uint64_t b = A.L.slot[u];
    for (uint64_t e = b + lane; e < b + A.L.id_cnt[u]; e += 32)
      atomicAdd(&A.delta[A.L.id_nbr[e]], d * A.L.id_w[e]);
    for (uint64_t e = b + lane; e < b + A.L.iv_cnt[u]; e += 32)
      atomicAdd(&A.x[A.L.iv_nbr[e]], d * A.L.iv_w[e]);
    __syncwarp();
    if (lane == 0) A.spnode[u] = 0.f;
  }
}

// Cluster-local convergence of the current deltas (the precompute of
// iter_compressor.h:534-785: local iteration of each supernode until its delta
// mass, a float sum as the reference's Diff, falls under the per-vertex
// threshold times its size, at most 100 steps).
// One warp per cluster.  A cluster of up to kStageCap members and
// kStageEdges local edges is staged in shared memory and iterated in two
// phases per step with no atomics inside the cluster: each member takes its
// delta and publishes its push value (sending to the cluster's out-mirrors,
// which only this cluster writes, by global atomics), then each member sums
// the push values of its local in-edges.  Larger clusters push on global
// memory.  A member belongs to one cluster and the list holds each cluster
// once, so the staged copy is the only writer of its members' deltas.
__global__ void __launch_bounds__(256) k_sum_precompute(SumArgs A, const uint32_t* clusters,
                                                        uint32_t n_cl, const uint64_t* cm_off,
                                                        const uint32_t* cm_v,
                                                        const uint64_t* sub_off,
                                                        const uint32_t* sub_nbr, StageLists L,
                                                        double thr_v) {
  __shared__ float s_d[kStageWarps][kStageCap];
  __shared__ float s_x[kStageWarps][kStageCap];
  __shared__ float s_pv[kStageWarps][kStageCap];
  __shared__ float s_deg[kStageWarps][kStageCap];
  __shared__ uint16_t s_lo[kStageWarps][kStageCap + 2];
  __shared__ uint8_t s_ls[kStageWarps][kStageEdges];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n_cl; k += nwarps) {
    const uint32_t c = clusters[k];
    const uint64_t b = cm_off[c], e = cm_off[c + 1];
    const uint32_t m = (uint32_t)(e - b);
    const float thr = f32_at_most(thr_v * (double)m);  // the reference's float Diff
    const uint64_t l0 = L.lin_off[b], nl = L.lin_off[e] - l0;
    if (m <= (uint32_t)kStageCap && nl <= (uint64_t)kStageEdges) {
      for (uint32_t i = lane; i < m; i += 32) {
        const uint32_t v = cm_v[b + i];
        s_d[w][i] = A.delta[v];
        s_x[w][i] = 0.f;
        s_deg[w][i] = (float)A.out_deg_all[v];
        s_lo[w][i + 1] = (uint16_t)(L.lin_off[b + i + 1] - l0);
      }
      if (lane == 0) s_lo[w][0] = 0;
      for (uint32_t j = lane; j < (uint32_t)nl; j += 32) s_ls[w][j] = L.lin_src[l0 + j];
      __syncwarp();
      for (int step = 1;; ++step) {
        float diff = 0.f;
        for (uint32_t i = lane; i < m; i += 32) {
          const float ts = s_d[w][i];
          float pv = 0.f;
          if (ts != 0.f) {
            s_d[w][i] = 0.f;
            s_x[w][i] += ts;
            diff += fabsf(ts);
            pv = ts * A.damping / s_deg[w][i];
            for (uint64_t f = L.lout_off[b + i]; f < L.lout_off[b + i + 1]; ++f)
              atomicAdd(&A.delta[L.lout_dst[f]], pv);
          }
          s_pv[w][i] = pv;
        }
        __syncwarp();
        for (uint32_t j = lane; j < m; j += 32) {
          float acc = 0.f;
          for (uint32_t f = s_lo[w][j]; f < s_lo[w][j + 1]; ++f) acc += s_pv[w][s_ls[w][f]];
          if (acc != 0.f) s_d[w][j] += acc;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) diff += __shfl_xor_sync(0xffffffffu, diff, o);
        __syncwarp();  // this step's sums are visible to the next step's reads
        if (diff <= thr || step > 100) break;
      }
      for (uint32_t i = lane; i < m; i += 32) {
        const uint32_t v = cm_v[b + i];
        A.delta[v] = s_d[w][i];
        A.x[v] += s_x[w][i];
      }
      __syncwarp();
      continue;
    }
    for (int step = 1;; ++step) {
      float diff = 0.f;
      for (uint64_t i = b + lane; i < e; i += 32) {
        const uint32_t v = cm_v[i];
        const float ts = atomicExch(&A.delta[v], 0.f);
        if (ts == 0.f) continue;
        A.x[v] += ts;
        diff += fabsf(ts);
        const float outv = ts * A.damping / (float)A.out_deg_all[v];
        for (uint64_t f = sub_off[i]; f < sub_off[i + 1]; ++f) atomicAdd(&A.delta[sub_nbr[f]], outv);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) diff += __shfl_xor_sync(0xffffffffu, diff, o);
      __syncwarp();  // this step's pushes are visible to the next step's reads
      if (diff <= thr || step > 100) break;
    }
  }
}

// exits of the precomputed clusters push the mass that passed through them
__global__ void __launch_bounds__(256) k_sum_bound_push(SumArgs A, const uint32_t* clusters, uint32_t n_cl,
                                                        const uint64_t* bl_off, const uint32_t* bl) {
  const uint32_t lane = threadIdx.x & 31;
  unsigned long long sc = 0;
  for (uint32_t k = blockIdx.x; k < n_cl; k += gridDim.x) {
    const uint32_t c = clusters[k];
    for (uint64_t i = bl_off[c] + (threadIdx.x >> 5); i < bl_off[c + 1]; i += blockDim.x >> 5) {
      const uint32_t u = bl[i];
      const float val = A.x[u];
      if (val == 0.f) continue;
      const float outv = val * A.damping / (float)A.out_deg_all[u];
      for (uint64_t e = A.ib_off[u] + lane; e < A.ib_off[u + 1]; e += 32)
        atomicAdd(&A.delta[A.ib_nbr[e]], outv);
      for (uint64_t s = A.sync_off[u]; s < A.sync_off[u + 1]; ++s) {
        const uint32_t mm = A.sync_nbr[s];
        float dm = 0.f;
        if (lane == 0) {
          atomicAdd(&A.delta[mm], val);
          dm = atomicExch(&A.delta[mm], 0.f);
        }
        dm = __shfl_sync(0xffffffffu, dm, 0);
        if (dm != 0.f) entry_push<32>(A, mm, dm, lane, sc);
      }
    }
  }
}

__global__ void k_sum_mirror_to_master(float* delta, const uint32_t* om, const uint32_t* master,
                                       uint32_t cnt) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const float d = atomicExch(&delta[om[i]], 0.f);
    if (d != 0.f) atomicAdd(&delta[master[i]], d);
  }
}

__global__ void k_stash_x(uint32_t n, float* x, float* old_x, int restore) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    if (restore) {
      x[v] += old_x[v];
    } else {
      old_x[v] = x[v];
      x[v] = 0.f;
    }
  }
}

static SumArgs sum_args(sg_ctx* ctx, SummaryDev& D, unsigned long long* cnt) {
  SumArgs A;
  A.damping = (float)ctx->opt.damping;
  A.thr_v = (float)(ctx->opt.termcheck_threshold / (double)D.old_n);
  A.old_n = D.old_n;
  A.x = ctx->pr.x;
  A.delta = ctx->pr.delta;
  A.bound = D.bound;
  A.spnode = D.spnode;
  A.ib_off = D.ib_off; A.sync_off = D.sync_off;
  A.ib_nbr = D.ib_nbr; A.sync_nbr = D.sync_nbr;
  A.L = repair_lists(D);
  A.out_deg_all = D.out_deg_all;
  A.ntype = D.ntype;
  A.cnt = cnt;
  A.sctl = D.sctl;
  A.sres = D.d_res;
  A.tau = ctx->opt.termcheck_threshold;
  return A;
}

// first_step: precompute the given clusters (all for PEval), push exits,
// hand out-mirror deltas to their masters
static sg_status first_step_dev(sg_ctx* ctx, SummaryDev& D, const uint32_t* d_cls, uint32_t ncls,
                                unsigned long long* cnt);

static sg_status first_step(sg_ctx* ctx, SummaryDev& D, const std::vector<uint32_t>& cls,
                            unsigned long long* cnt) {
  uint32_t* d_cls = nullptr;
  if (!cls.empty()) SG_TRY(upload(ctx, &d_cls, cls));
  const sg_status st = first_step_dev(ctx, D, d_cls, (uint32_t)cls.size(), cnt);
  dfree(d_cls);
  return st;
}

// the same over a device list of clusters
static sg_status first_step_dev(sg_ctx* ctx, SummaryDev& D, const uint32_t* d_cls, uint32_t ncls,
                                unsigned long long* cnt) {
  cudaStream_t st = ctx->stream;
  SumArgs A = sum_args(ctx, D, cnt);
  SG_CUDA(ctx, cudaMemsetAsync(D.bound, 0, 4ull * D.all_n, st));
  SG_CUDA(ctx, cudaMemsetAsync(D.spnode, 0, 4ull * D.all_n, st));
  if (ncls == 0) return SG_OK;
  k_stash_x<<<grid_for(D.old_n, 256), 256, 0, st>>>(D.old_n, ctx->pr.x, D.old_x, 0);
  kprof_begin(ctx);
  k_sum_precompute<<<grid_for((uint64_t)ncls * 32, 32 * kStageWarps), 32 * kStageWarps, 0, st>>>(
      A, d_cls, ncls, D.cm_off, D.cm_v, D.sub_off, D.sub_nbr,
      StageLists{D.lin_off, D.lin_src, D.lout_off, D.lout_dst},
      ctx->opt.termcheck_threshold / (double)D.old_n);
  kprof_end(ctx, SG_K_SUM_LOCAL);
  k_sum_bound_push<<<std::min<uint32_t>(ncls, ctx->num_sms * 8), 256, 0, st>>>(
      A, d_cls, ncls, D.bl_off, D.bound_list);
  if (D.n_omirror)
    k_sum_mirror_to_master<<<grid_for(D.n_omirror, 256), 256, 0, st>>>(ctx->pr.delta, D.l_omirror,
                                                                      D.omirror_master, D.n_omirror);
  k_stash_x<<<grid_for(D.old_n, 256), 256, 0, st>>>(D.old_n, ctx->pr.x, D.old_x, 1);
  count_launch(ctx, 5);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  return SG_OK;
}

// summarized rounds until the residual test passes, then the correction
static sg_status summarized_rounds(sg_ctx* ctx, SummaryDev& D, unsigned long long* cnt,
                                   int* rounds_out) {
  cudaStream_t st = ctx->stream;
  SumArgs A = sum_args(ctx, D, cnt);
  const int cap = ctx->opt.max_rounds > 0 ? ctx->opt.max_rounds : 1000;
  // rounds in chunks of 4 with the residual test on the device; once it
  // passes, the chunk's remaining kernels return at once
  SG_CUDA(ctx, cudaMemsetAsync(D.sctl, 0, 4 * sizeof(uint32_t), st));
  SG_CUDA(ctx, cudaMemsetAsync(D.d_res, 0, 2 * sizeof(double), st));
  const unsigned rblocks = grid_for(D.old_n, 256, ctx->num_sms * 4);
  // lanes per row: shortcut lists hold at most a cluster's nodes (a few on
  // average); boundary rows get a short group while they average a few edges
  constexpr uint32_t kEntryLanes = 4, kShortLanes = 4;
  const bool short_ib = D.n_ib <= (uint64_t)kShortLanes * ((uint64_t)D.n_exit + D.n_single);
  uint32_t h_ctl[4] = {0, 0, 0, 0};
  int launched = 0;
  while (launched < cap) {
    for (int c = 0; c < 4 && launched < cap; ++c, ++launched) {
      kprof_begin(ctx);
      if (D.n_entry)
        k_sum_entries<kEntryLanes><<<grid_for((uint64_t)D.n_entry * kEntryLanes, 256), 256, 0, st>>>(
            A, D.l_entry, D.n_entry);
      if (D.n_exit) {
        if (short_ib)
          k_sum_exits<kShortLanes><<<grid_for((uint64_t)D.n_exit * kShortLanes, 256), 256, 0, st>>>(
              A, D.l_exit, D.n_exit);
        else
          k_sum_exits<32><<<grid_for((uint64_t)D.n_exit * 32, 256), 256, 0, st>>>(A, D.l_exit, D.n_exit);
      }
      if (D.n_single) {
        if (short_ib)
          k_sum_singles<kShortLanes><<<grid_for((uint64_t)D.n_single * kShortLanes, 256), 256, 0, st>>>(
              A, D.l_single, D.n_single);
        else
          k_sum_singles<32><<<grid_for((uint64_t)D.n_single * 32, 256), 256, 0, st>>>(A, D.l_single,
                                                                                    D.n_single);
      }
      if (D.n_omirror) k_sum_omirror<<<grid_for(D.n_omirror, 256), 256, 0, st>>>(A, D.l_omirror, D.omirror_master, D.n_omirror);
      k_sum_residual_decide<<<rblocks, 256, 0, st>>>(A, D.old_n);
      kprof_end(ctx, SG_K_SUMMARY);
      count_launch(ctx, 1 + (D.n_entry > 0) + (D.n_exit > 0) + (D.n_single > 0) + (D.n_omirror > 0));
    }
    SG_CUDA(ctx, cudaGetLastError());
    SG_CUDA(ctx, cudaMemcpyAsync(h_ctl, D.sctl, sizeof(h_ctl), cudaMemcpyDeviceToHost, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
    if (h_ctl[0]) break;
  }
  const int r = (int)h_ctl[2];
  if (A.L.n_sp) k_sum_correct<<<grid_for((uint64_t)A.L.n_sp * 32, 256), 256, 0, st>>>(A);
  count_launch(ctx);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  *rounds_out = r;
  return SG_OK;
}

// A summary whose benefit filter kept no cluster has no supernode, no
// mirror and every vertex of type 0 (single), and no batch can add one (the
// incremental repair works on the kept clusters): its summarized rounds are
// the plain Ingress rounds over the whole graph.  Such a summary runs the
// plain path (the dense pull), and its batches skip the repair.
bool summary_no_supernodes(sg_ctx* ctx) {
  SummaryDev* D = sdev(ctx);
  return D && D->valid && D->S.supernode_ids.empty();
}

sg_status pr_summarized(sg_ctx* ctx, bool inc) {
  SummaryDev* D = sdev(ctx);
  if (!D || !D->valid) return fail(ctx, SG_ERR_STATE, "compress=1 needs sg_summary_build first");
  if (summary_no_supernodes(ctx)) return pr_run(ctx, inc);
  PrState& s = ctx->pr;
  cudaStream_t st = ctx->stream;
  unsigned long long* cnt = nullptr;
  SG_TRY(dalloc(ctx, &cnt, 2));
  SG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 16, st));
  SG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  std::vector<uint32_t> cls;
  const uint32_t* d_pend = nullptr;
  uint32_t n_pend = 0;
  if (!inc) {
    const float init_c = (float)((1.0 - ctx->opt.damping) / (double)ctx->g.n);
    std::vector<float> z(D->all_n, 0.f), dl(D->all_n, 0.f);
    for (uint32_t v = 0; v < D->old_n; ++v) dl[v] = init_c;
    SG_CUDA(ctx, cudaMemcpyAsync(s.x, z.data(), 4ull * D->all_n, cudaMemcpyHostToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(s.delta, dl.data(), 4ull * D->all_n, cudaMemcpyHostToDevice, st));
    SG_CUDA(ctx, cudaStreamSynchronize(st));
    for (uint32_t c = 0; c < D->S.supernode_ids.size(); ++c) cls.push_back(c);
  } else {
    // clusters the batches since the last IncEval updated (device marks)
    SG_TRY(repair_pending_clusters(ctx, *D, &d_pend, &n_pend));
  }
  if (inc) SG_TRY(first_step_dev(ctx, *D, d_pend, n_pend, cnt));
  else SG_TRY(first_step(ctx, *D, cls, cnt));
  int srounds = 0;
  SG_TRY(summarized_rounds(ctx, *D, cnt, &srounds));
  SG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  unsigned long long hc[2];
  SG_CUDA(ctx, cudaMemcpyAsync(hc, cnt, 16, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms_sum = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms_sum, ctx->ev0, ctx->ev1));
  dfree(cnt);
  // the plain rounds finish the residual on the original graph
  s.valid = true;
  sg_status stt = pr_run(ctx, true);
  ctx->stats.rounds += srounds;
  ctx->stats.edges_relaxed += hc[0] + hc[1];
  ctx->stats.shortcut_edges = hc[1];
  ctx->stats.elapsed_ms += ms_sum;
  return stt;
}

// The host restatement of one batch's repair (the summary.cpp passes with
// the shortcut kernels on the device): entry changes, exits, subgraphs and
// shortcuts of the touched clusters, node types and the sketch CSRs of S.
// The device's PageRank tables are repaired by repair.cu; S serves the
// SSSP and pull-mode paths, the counters and the checks.
static sg_status host_repair_batch(sg_ctx* ctx, SummaryDev* D, const uint32_t* as,
                                   const uint32_t* ad, const uint32_t* ak, const uint32_t* af,
                                   const float* aw, uint64_t na, bool last) {
  PhaseTrace T("host repair");
  std::vector<std::pair<uint32_t, uint32_t>> deleted, added;
  std::vector<AdjOp> ops_out, ops_in;
  for (uint64_t i = 0; i < na; ++i) {
    const bool found = af[i] != kInvalidVid;
    if ((ak[i] & 1u) && found) deleted.push_back({as[i], ad[i]});
    if (ak[i] & 2u) added.push_back({as[i], ad[i]});
    // the applier's effect: a delete of a present edge removes it, an add
    // sets the weight of a present edge or inserts an absent one
    uint8_t kind = 255;
    if (ak[i] == 1u && found) kind = AdjOp::kRemove;
    else if ((ak[i] & 2u) && found) kind = AdjOp::kSetWeight;
    else if (ak[i] & 2u) kind = AdjOp::kInsert;
    if (kind == 255) continue;
    ops_out.push_back({as[i], ad[i], aw[i], kind});
    ops_in.push_back({ad[i], as[i], aw[i], kind});
  }
  // the new graph on the host: the batch merged into the host copy (rows
  // stay sorted), else a fresh download
  const uint32_t n = ctx->g.n;
  auto by_row_col = [](const AdjOp& a, const AdjOp& b) {
    return a.row != b.row ? a.row < b.row : a.col < b.col;
  };
  std::sort(ops_out.begin(), ops_out.end(), by_row_col);
  std::sort(ops_in.begin(), ops_in.end(), by_row_col);
  T.mark("actions");
  const bool patched = D->out.n == n && D->in.n == n && host_adj_patch(D->out, ops_out) &&
                       host_adj_patch(D->in, ops_in);
  // a batch before the last one of a replay has no device graph to fall
  // back on (the device holds the graph after the last)
  if (!patched && !last) return fail(ctx, SG_ERR_STATE, "host graph copy out of step with the batches");
  if (!patched || (last && D->out.rp[n] != ctx->g.m)) {
    const uint64_t m = ctx->g.m;
    std::vector<uint64_t> rp(n + 1);
    std::vector<uint32_t> col(m);
    std::vector<float> w(ctx->g.weighted ? m : 0);
    SG_TRY(download_csr(ctx, rp.data(), col.data(), ctx->g.weighted ? w.data() : nullptr));
    host_adj_from_csr(n, rp.data(), col.data(), ctx->g.weighted ? w.data() : nullptr, D->out);
    host_transpose(D->out, D->in);
  }
  Summary& S = D->S;
  T.mark("host graph patch");
  summary_inc_entries(S, D->out, D->in, deleted, added);
  T.mark("entries");
  summary_judge_out_bound(S, D->out, &S.update_cluster_ids);
  summary_build_subgraph(S, D->out, D->in, &S.update_cluster_ids);
  T.mark("exits and subgraphs");
  std::vector<uint32_t> sps;
  for (uint32_t v : S.update_source_id) {
    const uint32_t sp = S.Fc_map[v];
    if (sp != Summary::kIdDefault && sp < S.supernodes.size()) sps.push_back(sp);
  }
  SG_TRY(compute_shortcuts(ctx, *D, sps));
  T.mark("shortcut weights");
  summary_node_types(S);
  T.mark("node types");
  summary_sketch_csr(S, D->out);
  T.mark("sketch CSRs");
  return SG_OK;
}


// Brings S up to date: replays the batches the device repair logged.
static sg_status host_sync(sg_ctx* ctx, SummaryDev* D) {
  if (!D->rep || repair_logged_batches(*D) == 0) return SG_OK;
  std::vector<uint32_t> as, ad, ak, af;
  std::vector<float> aw;
  std::vector<uint64_t> ends;
  SG_TRY(repair_take_log(ctx, *D, &as, &ad, &ak, &af, &aw, &ends));
  uint64_t b = 0;
  for (uint64_t e : ends) {
    SG_TRY(host_repair_batch(ctx, D, as.data() + b, ad.data() + b, ak.data() + b, af.data() + b,
                             aw.data() + b, e - b, e == ends.back()));
    b = e;
  }
  return SG_OK;
}

// After sg_apply_updates on a summarized graph: the device repair of the
// PageRank tables (and of the SSSP distance blocks once SSSP over the
// summary has run); the host restatement follows on demand (and before its
// action log grows past 64 M actions).
sg_status summary_after_apply(sg_ctx* ctx) {
  SummaryDev* D = sdev(ctx);
  if (!D || !D->valid) return SG_OK;
  if (summary_no_supernodes(ctx) || !D->rep) return SG_OK;  // nothing to repair, ever
  D->pull_stale = true;
  SG_TRY(repair_after_apply(ctx, *D));
  if (repair_logged_actions(*D) > (1ull << 26)) SG_TRY(host_sync(ctx, D));
  return SG_OK;
}

// ------------------------------------------- in-indexes for message_type = pull

// SumSyncIterWorkerPull's classification and in-indexes
// (sum_sync_iter_worker_pull.h:286-509, rebuilt after each batch at
// :1166-1342): classes 0 (no cluster), 2 (entry), 4 (member, no out-edge
// leaving the cluster), then 1 / 3 for members with such an edge (3: also
// an entry).  The value index of an exit (1, 3) holds every (entry, w) of a
// bound_delta list ending at it, supernodes in index order (the shortcut
// construction puts exits in bound_delta and the other members in
// inner_value, so no inner_value entry ends at an exit).  Entries (2, 3)
// get their in-edges from vertices of other clusters, in row order.  The
// worker's remaining indexes (inner_value ending at classes 2 / 4,
// inner_delta at 1-4) only serve its correction, which scatters the
// supernodes' own lists instead.  The worker indexes per-vertex arrays by
// the shortcut targets, which with mirrors include out-mirror ids past the
// vertex range; a summary with mirrors is refused.
static sg_status pull_index_build(sg_ctx* ctx, SummaryDev& D) {
  const Summary& S = D.S;
  const uint32_t n = S.old_n;
  if (S.all_n != n)
    return fail(ctx, SG_ERR_INVALID,
                "message_type=pull needs a summary without mirrors (raise mirror_k)");
  std::vector<uint8_t> cls(n);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)n; ++i) {
    const int32_t fc = S.Fc[i];
    uint8_t t = 255;
    if (fc == Summary::kFcDefault) t = 0;
    else if (fc >= 0) t = 2;
    else if (!S.out_bound[i]) t = 4;
    if (S.out_bound[i]) t = fc >= 0 && fc != Summary::kFcDefault ? 3 : 1;
    cls[i] = t;
  }
  // bound_delta transposed: counts, offsets, then fills in supernode order
  const size_t nsp = S.supernodes.size();
  std::vector<uint64_t> bd_off(n + 1, 0);
  for (size_t sp = 0; sp < nsp; ++sp)
    for (const auto& e : S.supernodes[sp].bound_delta)
      if (e.first < n && (cls[e.first] == 1 || cls[e.first] == 3)) ++bd_off[e.first + 1];
  for (uint32_t v = 0; v < n; ++v) bd_off[v + 1] += bd_off[v];
  hvec<uint32_t> bd_src(bd_off[n]);
  hvec<float> bd_w(bd_off[n]);
  {
    std::vector<uint64_t> cur(bd_off.begin(), bd_off.end() - 1);
    for (size_t sp = 0; sp < nsp; ++sp) {
      const Supernode& P = S.supernodes[sp];
      for (const auto& e : P.bound_delta)
        if (e.first < n && (cls[e.first] == 1 || cls[e.first] == 3)) {
          bd_src[cur[e.first]] = P.id;
          bd_w[cur[e.first]++] = (float)e.second;
        }
    }
  }
  std::vector<uint64_t> ie_off(n + 1, 0);
  const HostAdj& in = D.in;
#pragma omp parallel for schedule(dynamic, 4096)
  for (long long v = 0; v < (long long)n; ++v) {
    if (cls[v] != 2 && cls[v] != 3) continue;
    const uint32_t c = S.id2spids[v];
    uint64_t k = 0;
    for (uint64_t e = in.rp[v]; e < in.rp[v + 1]; ++e) k += S.id2spids[in.col[e]] != c;
    ie_off[v + 1] = k;
  }
  for (uint32_t v = 0; v < n; ++v) ie_off[v + 1] += ie_off[v];
  hvec<uint32_t> ie_nbr(ie_off[n]);
#pragma omp parallel for schedule(dynamic, 4096)
  for (long long v = 0; v < (long long)n; ++v) {
    if (cls[v] != 2 && cls[v] != 3) continue;
    const uint32_t c = S.id2spids[v];
    uint64_t k = ie_off[v];
    for (uint64_t e = in.rp[v]; e < in.rp[v + 1]; ++e)
      if (S.id2spids[in.col[e]] != c) ie_nbr[k++] = in.col[e];
  }
  // the round's rows (classes 0-3; rows of more than 32 entries first, each
  // group in vertex order) and the entries: counts per chunk, offsets, fills
  auto row_len = [&](uint32_t v) -> uint64_t {
    switch (cls[v]) {
      case 0: return in.deg(v);
      case 1: return bd_off[v + 1] - bd_off[v];
      case 2: return ie_off[v + 1] - ie_off[v];
      case 3: return ie_off[v + 1] - ie_off[v] + bd_off[v + 1] - bd_off[v];
      default: return 0;
    }
  };
  const uint32_t nch = std::max<uint32_t>(1, std::min<uint32_t>(256, n / 16384));
  std::vector<uint64_t> cl_(nch + 1, 0), cs_(nch + 1, 0), ce(nch + 1, 0), ced(nch, 0), ccr(nch, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (long long ch = 0; ch < (long long)nch; ++ch) {
    const uint32_t v0 = (uint32_t)((uint64_t)n * ch / nch), v1 = (uint32_t)((uint64_t)n * (ch + 1) / nch);
    uint64_t lg = 0, sh = 0, e = 0, ed = 0, cr = 0;
    for (uint32_t v = v0; v < v1; ++v) {
      if (cls[v] == 4) continue;
      if (row_len(v) > 32) ++lg; else ++sh;
      if (cls[v] == 0) ed += in.deg(v);
      if (cls[v] == 2 || cls[v] == 3) {
        ++e;
        const uint32_t sp = S.Fc_map[v];
        if (sp < nsp) cr += S.supernodes[sp].inner_value.size() + S.supernodes[sp].inner_delta.size();
      }
    }
    cl_[ch + 1] = lg;
    cs_[ch + 1] = sh;
    ce[ch + 1] = e;
    ced[ch] = ed;
    ccr[ch] = cr;
  }
  uint64_t round_edges = ie_off[n] + bd_off[n], corr = 0;
  for (uint32_t ch = 0; ch < nch; ++ch) {
    cl_[ch + 1] += cl_[ch];
    cs_[ch + 1] += cs_[ch];
    ce[ch + 1] += ce[ch];
    round_edges += ced[ch];
    corr += ccr[ch];
  }
  const uint64_t n_long = cl_[nch];
  hvec<uint32_t> act(n_long + cs_[nch]), ent(ce[nch]);
#pragma omp parallel for schedule(dynamic, 1)
  for (long long ch = 0; ch < (long long)nch; ++ch) {
    const uint32_t v0 = (uint32_t)((uint64_t)n * ch / nch), v1 = (uint32_t)((uint64_t)n * (ch + 1) / nch);
    uint64_t lg = cl_[ch], sh = n_long + cs_[ch], e = ce[ch];
    for (uint32_t v = v0; v < v1; ++v) {
      if (cls[v] == 4) continue;
      if (row_len(v) > 32) act[lg++] = v; else act[sh++] = v;
      if (cls[v] == 2 || cls[v] == 3) ent[e++] = v;
    }
  }
  SG_TRY(reupload(ctx, D, &D.p_act, act));
  SG_TRY(reupload(ctx, D, &D.p_ent, ent));
  SG_TRY(reupload(ctx, D, &D.p_cls, cls));
  SG_TRY(reupload(ctx, D, &D.p_ie_off, ie_off));
  SG_TRY(reupload(ctx, D, &D.p_ie_nbr, ie_nbr));
  SG_TRY(reupload(ctx, D, &D.p_bd_off, bd_off));
  SG_TRY(reupload(ctx, D, &D.p_bd_src, bd_src));
  SG_TRY(reupload(ctx, D, &D.p_bd_w, bd_w));
  PullView& V = D.pv;
  V = PullView();
  V.n = n;
  V.cls = D.p_cls;
  V.act = D.p_act;
  V.n_act = (uint32_t)act.size();
  V.n_long = (uint32_t)n_long;
  V.ent = D.p_ent;
  V.n_ent = (uint32_t)ent.size();
  V.ie_off = D.p_ie_off; V.ie_nbr = D.p_ie_nbr;
  V.bd_off = D.p_bd_off; V.bd_src = D.p_bd_src; V.bd_w = D.p_bd_w;
  V.L = repair_lists(D);
  V.round_edges = round_edges;
  V.round_shortcuts = bd_off[n];
  V.corr_entries = corr;
  D.pull_stale = false;
  return SG_OK;
}

sg_status summary_pull_view(sg_ctx* ctx, PullView* out) {
  SummaryDev* D = sdev(ctx);
  if (!D || !D->valid) return fail(ctx, SG_ERR_STATE, "compress=1 needs sg_summary_build first");
  SG_TRY(host_sync(ctx, D));
  if (D->pull_stale) SG_TRY(pull_index_build(ctx, *D));
  *out = D->pv;
  return SG_OK;
}

uint32_t summary_rows(sg_ctx* ctx) {
  SummaryDev* D = sdev(ctx);
  return (D && D->valid) ? D->all_n : 0;
}

sg_status summary_info(sg_ctx* ctx, sg_summary_info* o) {
  SummaryDev* D = sdev(ctx);
  if (!D || !D->valid) return fail(ctx, SG_ERR_STATE, "no summary built");
  SG_TRY(host_sync(ctx, D));
  const Summary& S = D->S;
  std::memset(o, 0, sizeof(*o));
  o->clusters = S.supernode_ids.size();
  for (const auto& sp : S.supernodes)
    if (sp.id != Summary::kIdDefault) {
      o->supernodes++;
      o->bound_index = o->bound_index + sp.bound_delta.size();
      o->inner_index = o->inner_index + sp.inner_delta.size();
      o->inner_value_index = o->inner_value_index + sp.inner_value.size();
    }
  for (const auto& c : S.supernode_ids) o->cluster_members += c.size();
  for (const auto& c : S.supernode_source) o->sources += c.size();
  for (uint32_t v = 0; v < S.old_n; ++v) o->bound_nodes += S.out_bound[v] ? 1 : 0;
  o->all_rows = S.all_n;
  o->absorbed = S.mirror_node_cnt;
  for (const auto& c : S.cluster_in_mirror_ids) o->in_mirrors += c.size();
  for (const auto& c : S.cluster_out_mirror_ids) o->out_mirrors += c.size();
  o->sync_edges = S.sync_off.empty() ? 0 : S.sync_off.back();
  o->boundary_edges = S.ib_off.empty() ? 0 : S.ib_off.back();
  o->shortcut_edges = S.is_off.empty() ? 0 : S.is_off.back();
  for (uint32_t v = 0; v < S.old_n; ++v)
    if (S.node_type[v] >= 0 && S.node_type[v] < 7) o->node_type_count[(int)S.node_type[v]]++;
  return SG_OK;
}

// Device-repaired PageRank tables against the host restatement (S after
// replaying the logged batches).
template <typename T>
static sg_status fetch(sg_ctx* ctx, const T* d, uint64_t count, std::vector<T>* h) {
  h->resize(count);
  if (count)
    SG_CUDA(ctx, cudaMemcpyAsync(h->data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost, ctx->stream));
  return SG_OK;
}

sg_status summary_check(sg_ctx* ctx, sg_summary_check* o) {
  SummaryDev* Dp = sdev(ctx);
  if (!Dp || !Dp->valid) return fail(ctx, SG_ERR_STATE, "no summary built");
  std::memset(o, 0, sizeof(*o));
  if (summary_no_supernodes(ctx)) return SG_OK;
  SG_TRY(host_sync(ctx, Dp));
  SummaryDev& D = *Dp;
  const Summary& S = D.S;
  const uint32_t n = S.old_n, all = S.all_n;
  const SpLists L = repair_lists(D);
  std::vector<uint8_t> nt, rsp;
  std::vector<uint64_t> ibo, slot;
  std::vector<uint32_t> le, lx, ls, isc, ivc, idc;
  SG_TRY(fetch(ctx, D.ntype, n, &nt));
  SG_TRY(fetch(ctx, D.ib_off, (uint64_t)all + 1, &ibo));
  SG_TRY(fetch(ctx, L.slot, all, &slot));
  SG_TRY(fetch(ctx, L.row_sp, all, &rsp));
  SG_TRY(fetch(ctx, L.is_cnt, all, &isc));
  SG_TRY(fetch(ctx, L.iv_cnt, all, &ivc));
  SG_TRY(fetch(ctx, L.id_cnt, all, &idc));
  SG_TRY(fetch(ctx, D.l_entry, D.n_entry, &le));
  SG_TRY(fetch(ctx, D.l_exit, D.n_exit, &lx));
  SG_TRY(fetch(ctx, D.l_single, D.n_single, &ls));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<uint32_t> ibn, isn, ivn, idn;
  std::vector<float> isw, ivw, idw;
  SG_TRY(fetch(ctx, D.ib_nbr, ibo[all], &ibn));
  SG_TRY(fetch(ctx, L.is_nbr, L.pool, &isn));
  SG_TRY(fetch(ctx, L.is_w, L.pool, &isw));
  SG_TRY(fetch(ctx, L.iv_nbr, L.pool, &ivn));
  SG_TRY(fetch(ctx, L.iv_w, L.pool, &ivw));
  SG_TRY(fetch(ctx, L.id_nbr, L.pool, &idn));
  SG_TRY(fetch(ctx, L.id_w, L.pool, &idw));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  o->rows = all;
  std::vector<uint32_t> he, hx, hs;
  for (uint32_t v = 0; v < n; ++v) {
    const char t = S.node_type[v];
    if ((uint8_t)t != nt[v]) o->type_diff++;
    if (t == kOnlyIn || t == kBothOutIn || t == kBothOutInMaster) he.push_back(v);
    if (t == kOnlyOut || t == kBothOutIn || t == kOutMaster || t == kBothOutInMaster) hx.push_back(v);
    if (t == kSingle) hs.push_back(v);
  }
  o->list_diff = (he != le) + (hx != lx) + (hs != ls);
  double max_rel = 0.0;
  // (target, weight) lists compared as sets of targets, weights within 1e-4
  auto same = [&](std::vector<std::pair<uint32_t, double>> a,
                  std::vector<std::pair<uint32_t, double>> b) {
    if (a.size() != b.size()) return false;
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    for (size_t i = 0; i < a.size(); ++i) {
      if (a[i].first != b[i].first) return false;
      const double den = std::max(std::fabs(a[i].second), std::fabs(b[i].second));
      const double rel = den > 0 ? std::fabs(a[i].second - b[i].second) / den : 0.0;
      max_rel = std::max(max_rel, rel);
      if (rel > 1e-4) return false;
    }
    return true;
  };
  // a device row: cnt entries at the row's slot (none for other rows)
  auto dev_row = [&](const std::vector<uint32_t>& nbr, const std::vector<float>* w,
                     const std::vector<uint32_t>& cnt, uint32_t r) {
    std::vector<std::pair<uint32_t, double>> x;
    if (!rsp[r]) return x;
    for (uint64_t e = slot[r]; e < slot[r] + cnt[r]; ++e)
      x.push_back({nbr[e], w ? (double)(*w)[e] : 0.0});
    return x;
  };
  for (uint32_t r = 0; r < all; ++r) {
    {
      std::vector<std::pair<uint32_t, double>> h, d;
      for (uint64_t e = S.ib_off[r]; e < S.ib_off[r + 1]; ++e) h.push_back({S.ib_nbr[e], 0.0});
      for (uint64_t e = ibo[r]; e < ibo[r + 1]; ++e) d.push_back({ibn[e], 0.0});
      if (!same(d, h)) o->ib_diff++;
    }
    {
      std::vector<std::pair<uint32_t, double>> h;
      for (uint64_t e = S.is_off[r]; e < S.is_off[r + 1]; ++e) h.push_back({S.is_nbr[e], (double)S.is_w[e]});
      if (!same(dev_row(isn, &isw, isc, r), h)) o->is_diff++;
    }
    const uint32_t sp = S.Fc_map[r];
    const bool hsp = sp != Summary::kIdDefault && sp < S.supernodes.size() && S.supernodes[sp].id == r;
    if (hsp != (rsp[r] != 0)) {
      o->corr_diff++;
      continue;
    }
    if (!hsp) continue;
    const Supernode& h = S.supernodes[sp];
    std::vector<std::pair<uint32_t, double>> hv(h.inner_value.begin(), h.inner_value.end()),
        hd(h.inner_delta.begin(), h.inner_delta.end());
    for (auto& e : hv) e.second = (double)(float)e.second;
    for (auto& e : hd) e.second = (double)(float)e.second;
    if (!same(dev_row(ivn, &ivw, ivc, r), hv) || !same(dev_row(idn, &idw, idc, r), hd))
      o->corr_diff++;
  }
  o->max_rel = max_rel;
  return SG_OK;
}

// ================================================== SSSP over the summary
//
// The summarized traversal of SumSyncTraversalWorker (sum_sync_traversal_worker.h:
// 1097-1233, correction :1322-1403) with the shortcuts of TravCompressor
// (build_trav_index_mirror / run_to_convergence_mirror /
// fianl_build_trav_index_mirror, trav_compressor.h:244-430): for every
// supernode, the shortest distances inside its cluster from its entry (or
// in-mirror) to the exits and out-mirrors (bound shortcuts) and to the other
// members (inner shortcuts).  The summarized graph has one row per vertex and
// mirror: entries carry their bound shortcuts, exits and unclustered vertices
// their edges out of the cluster, masters a 0-weight edge to their in-mirrors,
// out-mirrors one to their master; inner members have no row.  Delta-stepping
// over it gives every non-inner vertex its exact distance (a shortest path
// enters a cluster through an entry and leaves through an exit); the
// correction then sets each inner member to the smallest entry distance plus
// inner shortcut.  A source inside a cluster is first expanded inside its
// cluster and seeds the run with its exits and members.

// One CTA per job: Bellman-Ford inside the cluster from the job's source,
// distances as ordered bits in shared memory.
__global__ void __launch_bounds__(128) k_sssp_shortcuts(const uint32_t* __restrict__ job_cl,
                                                        const uint32_t* __restrict__ job_src,
                                                        const uint64_t* __restrict__ cl_off,
                                                        const uint64_t* __restrict__ adj_off,
                                                        const uint32_t* __restrict__ adj_nbr,
                                                        const float* __restrict__ adj_w,
                                                        const uint64_t* __restrict__ out_off,
                                                        double* __restrict__ out, uint32_t njobs) {
  extern __shared__ unsigned long long sd[];
  __shared__ int s_changed;
  const uint32_t j = blockIdx.x;
  if (j >= njobs) return;
  const uint32_t c = job_cl[j];
  const uint64_t l0 = cl_off[c];
  const uint32_t L = (uint32_t)(cl_off[c + 1] - l0);
  const uint32_t src = job_src[j];
  for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) sd[i] = i == src ? 0ull : kInfBits;
  __syncthreads();
  for (uint32_t round = 0; round <= L; ++round) {
    if (threadIdx.x == 0) s_changed = 0;
    __syncthreads();
    int changed = 0;
    for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) {
      const unsigned long long di = sd[i];
      if (di >= kInfBits) continue;
      const double dv = bitsd(di);
      for (uint64_t e = adj_off[l0 + i]; e < adj_off[l0 + i + 1]; ++e) {
        const unsigned long long cb = dbits(dv + (double)adj_w[e]);
        const uint32_t t = adj_nbr[e];
        if (cb < sd[t] && cb < atomicMin(&sd[t], cb)) changed = 1;
      }
    }
    if (changed) s_changed = 1;
    __syncthreads();
    const int any = s_changed;
    __syncthreads();
    if (!any) break;
  }
  const uint64_t o = out_off[j];
  for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) out[o + i] = bitsd(sd[i]);
}

// inner member <- min over its cluster's entries of entry distance + shortcut
__global__ void k_sssp_correct(uint32_t nrows, const uint64_t* __restrict__ coff,
                               const uint32_t* __restrict__ crow, const uint32_t* __restrict__ cv,
                               const float* __restrict__ cd, unsigned long long* dist) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t wv = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wv < nrows;
       wv += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const unsigned long long de = dist[crow[wv]];
    if (de >= kInfBits) continue;
    const double d0 = bitsd(de);
    for (uint64_t e = coff[wv] + lane; e < coff[wv + 1]; e += 32)
      atomicMin(dist + cv[e], dbits(d0 + (double)cd[e]));
  }
}

__global__ void k_copy_u64(const unsigned long long* a, uint64_t n, unsigned long long* b) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

sg_status sssp_summarized(sg_ctx* ctx, uint32_t source) {
  SummaryDev* Dp = sdev(ctx);
  if (!Dp || !Dp->valid) return fail(ctx, SG_ERR_STATE, "compress=1 needs sg_summary_build first");
  SummaryDev& D = *Dp;
  Summary& S = D.S;  // (its membership part, fixed after the build)
  if (!ctx->g.weighted) return fail(ctx, SG_ERR_INVALID, "SSSP needs a weighted graph");
  if (source >= S.old_n) return fail(ctx, SG_ERR_INVALID, "source >= n");
  if (summary_no_supernodes(ctx) || !repair_active(D)) return sssp_run_peval(ctx, source);
  cudaStream_t st = ctx->stream;
  SG_CUDA(ctx, cudaEventRecord(ctx->kev0, st));
  SG_TRY(repair_sssp_refresh(ctx, D));
  // seeds: the source, expanded inside its cluster when it is a member (a
  // path from the source to its own cluster's members needs no entry)
  std::vector<uint32_t> seeds;
  std::vector<double> sdist;
  const bool member = S.id2spids[source] != Summary::kIdDefault;
  {
    const uint32_t* dv = nullptr;
    const double* dd = nullptr;
    uint32_t cnt = 0;
    SG_TRY(repair_source_seeds(ctx, D, source, &dv, &dd, &cnt));
    seeds.resize(cnt);
    sdist.resize(cnt);
    if (cnt) {
      SG_CUDA(ctx, cudaMemcpyAsync(seeds.data(), dv, 4ull * cnt, cudaMemcpyDeviceToHost, st));
      SG_CUDA(ctx, cudaMemcpyAsync(sdist.data(), dd, 8ull * cnt, cudaMemcpyDeviceToHost, st));
      SG_CUDA(ctx, cudaStreamSynchronize(st));
    }
  }
  if (!member) {
    seeds.push_back(source);
    sdist.push_back(0.0);
  }
  SG_TRY(sssp_prepare_external(ctx, source));
  unsigned long long* dist = nullptr;
  SG_TRY(stage_alloc(ctx, D, SP_DIST, S.all_n, &dist));
  SsspView G{S.all_n, D.sk_m, D.sk_off, D.sk_deg, D.sk_col, D.sk_w};
  unsigned long long h_cnt[4] = {0, 0, 0, 0};
  sg_status rs = sssp_run_view(ctx, G, seeds.data(), sdist.data(), (uint32_t)seeds.size(), dist,
                               h_cnt, D.view);
  if (rs != SG_OK) return rs;
  if (D.sk_ncorr)
    k_sssp_correct<<<grid_for((uint64_t)D.sk_ncorr * 32, 256), 256, 0, st>>>(
        D.sk_ncorr, D.sk_coff, D.sk_crow, D.sk_cv, D.sk_cd, dist);
  k_copy_u64<<<grid_for(S.old_n, 256), 256, 0, st>>>(dist, S.old_n, ctx->sp.dist);
  count_launch(ctx, 2);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaEventRecord(ctx->kev1, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->kev0, ctx->kev1));
  return sssp_finish_external(ctx, h_cnt, ms);
}


// ------------------------------------------- SSSP IncEval over the summary

// rows below n: the plain distances after the reset; mirror rows: unreached
__global__ void k_dist_all_init(const unsigned long long* __restrict__ dist, uint32_t n,
                                uint32_t all_n, unsigned long long* __restrict__ dall) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < all_n; v += gridDim.x * blockDim.x)
    dall[v] = v < n ? dist[v] : kInfBits;
}

// dist[v] <- min(dist[v], d) for a list of (vertex, distance)
__global__ void k_dist_min_list(const uint32_t* __restrict__ v, const double* __restrict__ d,
                                uint32_t cnt, unsigned long long* __restrict__ dall) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    atomicMin(dall + v[i], dbits(d[i]));
}

// an in-mirror starts from its master's distance (their edge weighs 0)
__global__ void k_dist_mirrors(const uint32_t* __restrict__ mir, const uint32_t* __restrict__ master,
                               uint32_t cnt, unsigned long long* __restrict__ dall) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    dall[mir[i]] = dall[master[i]];
}

bool sssp_summary_ready(sg_ctx* ctx) {
  SummaryDev* D = sdev(ctx);
  return D && D->valid && D->sssp_ready && ctx->g.weighted;
}

// The incremental stage of SumSyncTraversalWorker
// (sum_sync_traversal_worker.h:1424-1690): deltaCompute's reset, then rounds
// over the summary (boundary edges, entry -> exit shortcuts, master -> mirror
// edges) instead of the original graph, then the correction of the inner
// members through the entry -> member shortcuts.
//   1. The reset BFS over the shortest-path tree and the re-seed pulls of the
//      plain IncEval (shared code): every vertex whose distance can grow is
//      reset and restarts from the best in-neighbour that kept its distance;
//      the batch's new edges are relaxed.  Distances that are not reset are
//      final or too long, never too short.
//   2. Shortcut distances of the supernodes the batch touched are repaired and
//      the summarized CSR is rebuilt.
//   3. Delta-stepping over the summarized CSR from that warm state, seeded by
//      the reset vertices, the heads of new edges and every supernode's entry
//      (or in-mirror): a path into a cluster reaches its exits only through an
//      entry's shortcut, and repaired shortcuts may be shorter.
//      A source inside a cluster also seeds its cluster's members with their
//      distances from a local solve of the repaired cluster (paths from the
//      source to its own cluster's members need no entry).
//   4. Inner members: the minimum over their cluster's entries of entry
//      distance + shortcut (a reset member starts from its re-seed value, an
//      upper bound).
//   5. Parents over the in-rows of the original graph.
// The result equals the plain IncEval's (Dijkstra on the new graph).
sg_status sssp_summarized_inc(sg_ctx* ctx) {
  SummaryDev* Dp = sdev(ctx);
  if (!Dp || !Dp->valid) return fail(ctx, SG_ERR_STATE, "compress=1 needs sg_summary_build first");
  SummaryDev& D = *Dp;
  Summary& S = D.S;  // (its membership part, fixed after the build)
  if (!ctx->g.weighted) return fail(ctx, SG_ERR_INVALID, "SSSP needs a weighted graph");
  if (!repair_active(D)) return fail(ctx, SG_ERR_STATE, "no device summary");
  cudaStream_t st = ctx->stream;
  SG_CUDA(ctx, cudaEventRecord(ctx->kev0, st));
  SsspIncInfo info;
  SG_TRY(sssp_inc_prepare(ctx, &info));
  SG_TRY(repair_sssp_refresh(ctx, D));
  const uint32_t n = S.old_n, all = S.all_n;
  SsspState& sp = ctx->sp;
  unsigned long long* dall = nullptr;
  uint32_t* seeds = nullptr;
  const uint64_t nseeds = (uint64_t)info.total + info.nadd + D.sk_nspid;
  SG_TRY(stage_alloc(ctx, D, SI_DALL, all, &dall));
  SG_TRY(stage_alloc(ctx, D, SI_SEEDS, nseeds, &seeds));
  k_dist_all_init<<<grid_for(all, 256), 256, 0, st>>>(sp.dist, n, all, dall);
  if (D.sk_nimir)
    k_dist_mirrors<<<grid_for(D.sk_nimir, 256), 256, 0, st>>>(D.sk_imir, D.sk_imaster, D.sk_nimir,
                                                            dall);
  count_launch(ctx, 1 + (D.sk_nimir > 0));
  uint64_t o = 0;
  if (info.total)
    SG_CUDA(ctx, cudaMemcpyAsync(seeds, sp.seeds, 4ull * info.total, cudaMemcpyDeviceToDevice, st));
  o += info.total;
  if (info.nadd)
    SG_CUDA(ctx, cudaMemcpyAsync(seeds + o, sp.padd_dst, 4ull * info.nadd, cudaMemcpyDeviceToDevice,
                                 st));
  o += info.nadd;
  if (D.sk_nspid)
    SG_CUDA(ctx, cudaMemcpyAsync(seeds + o, D.sk_spid, 4ull * D.sk_nspid, cudaMemcpyDeviceToDevice,
                                 st));
  // the source's own cluster, solved locally on the repaired subgraph
  const uint32_t* d_cs = nullptr;
  const double* d_cd = nullptr;
  uint32_t ncs = 0;
  SG_TRY(repair_source_seeds(ctx, D, sp.source, &d_cs, &d_cd, &ncs));
  uint64_t nseeds_all = nseeds;
  if (ncs) {
    k_dist_min_list<<<grid_for(ncs, 256), 256, 0, st>>>(d_cs, d_cd, ncs, dall);
    count_launch(ctx);
    uint32_t* s2 = nullptr;
    SG_TRY(stage_alloc(ctx, D, SI_S2, nseeds + ncs, &s2));
    if (nseeds) SG_CUDA(ctx, cudaMemcpyAsync(s2, seeds, 4ull * nseeds, cudaMemcpyDeviceToDevice, st));
    SG_CUDA(ctx, cudaMemcpyAsync(s2 + nseeds, d_cs, 4ull * ncs, cudaMemcpyDeviceToDevice, st));
    seeds = s2;
    nseeds_all = nseeds + ncs;
  }
  SsspView G{all, D.sk_m, D.sk_off, D.sk_deg, D.sk_col, D.sk_w};
  unsigned long long h_cnt[4] = {0, 0, 0, 0};
  sg_status rs = sssp_run_view_warm(ctx, G, seeds, (uint32_t)nseeds_all, dall, h_cnt, D.view);
  if (rs != SG_OK) return rs;
  if (D.sk_ncorr)
    k_sssp_correct<<<grid_for((uint64_t)D.sk_ncorr * 32, 256), 256, 0, st>>>(
        D.sk_ncorr, D.sk_coff, D.sk_crow, D.sk_cv, D.sk_cd, dall);
  k_copy_u64<<<grid_for(n, 256), 256, 0, st>>>(dall, n, sp.dist);
  count_launch(ctx, 2);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaEventRecord(ctx->kev1, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.f;
  SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->kev0, ctx->kev1));
  ctx->stats.shortcut_edges = 0;
  return sssp_inc_finish_external(ctx, info, h_cnt, ms);
}

}  // namespace sg
