// Device state of a summarized graph, shared by the summary's translation
// units (summary.cu: construction, PageRank / SSSP over the summary and the
// host restatement of the repair; repair.cu: the device repair).
#pragma once

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <unordered_map>
#include <vector>

#include "ctx.h"
#include "summary.h"

namespace sg {

struct RepairDev;  // repair.cu

// Host phase times of the summary's maintenance, printed to stderr when the
// environment sets SUMINC_GB300_TRACE (a diagnostic; off by default).
struct PhaseTrace {
  bool on;
  const char* what;
  std::chrono::steady_clock::time_point t0, t;
  explicit PhaseTrace(const char* w) : what(w) {
    static const bool env = std::getenv("SUMINC_GB300_TRACE") != nullptr;
    on = env;
    t0 = t = std::chrono::steady_clock::now();
  }
  // with a stream, the phase's device work is waited for first
  void mark(const char* phase, cudaStream_t st = nullptr) {
    if (!on) return;
    if (st) cudaStreamSynchronize(st);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[suminc_gb300] %s %s %.2f ms\n", what, phase,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
  ~PhaseTrace() {
    if (on)
      std::fprintf(stderr, "[suminc_gb300] %s total %.2f ms\n", what,
                   std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                       .count());
  }
};


// cluster precompute staged in shared memory: clusters of up to kStageCap
// members (8-bit local indices) and kStageEdges local edges, one per warp
constexpr int kStageCap = 160;
constexpr int kStageEdges = 2048;
constexpr int kStageWarps = 8;

struct StageLists {
  const uint64_t* lin_off;   // per cm_v position: local in-edges
  const uint8_t* lin_src;    // their tails, as local indices
  const uint64_t* lout_off;  // per cm_v position: edges to out-mirrors
  const uint32_t* lout_dst;
};

// Exact FP32 -> FP64 widening of a normal float by its IEEE fields (sign,
// exponent rebased from 127 to 1023, mantissa shifted into the top of the
// 52-bit field); zero, subnormals and non-finite values take the
// conversion instruction.  Keeps the widening off the FP64 pipe, which
// GB300 runs at a small fraction of the FP32 rate.
__device__ __forceinline__ double widen_f32(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  if (e == 0u || e == 0xFFu) return (double)f;
  const unsigned long long bits = ((unsigned long long)(b >> 31) << 63) |
                                  ((unsigned long long)(e + (1023u - 127u)) << 52) |
                                  ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)bits);
}

// The largest float not above a non-negative double threshold t: for any
// float x, x <= f32_at_most(t) exactly when (double)x <= t.  Lets a loop
// test its FP32 step mass against an FP64 threshold with one FP32 compare
// (positive floats are ordered like their bit patterns, so the next float
// below is the pattern minus one).
__device__ __forceinline__ float f32_at_most(double t) {
  float f = __double2float_rn(t);
  if ((double)f > t) f = __uint_as_float(__float_as_uint(f) - 1u);
  return f;
}

// Cluster-local shortcut solves (summary.cu): one job per supernode, the
// cluster's nodes as local indices and its edges as a local CSR.
struct ShortcutArgs {
  uint32_t n_sp;
  const uint32_t* sp_cluster;   // cluster of each supernode job
  const uint32_t* sp_src;       // local index of the entry
  const uint64_t* cl_off;       // local node range of each cluster [cl_off[c], cl_off[c+1])
  const uint32_t* cl_inner;     // number of members (iterated nodes) of each cluster
  const uint64_t* adj_off;      // per local node (global local index) edge range
  const uint32_t* adj_nbr;      // local target index (relative to the cluster)
  const float* div;             // out-degree divisor per local node
  const uint64_t* out_off;      // per job output offset
  double* out_value;
  double* out_delta;
  float damping;
  double thr_per_node;          // threshold / N
  const uint32_t* jobs;         // the jobs this launch runs (null: all)
  const uint64_t* lin_off;      // warp kernel: per local node, its in-edges
  const uint8_t* lin_src;       // from members (local indices)
};

__global__ void __launch_bounds__(128) k_shortcuts(ShortcutArgs A, uint32_t njobs);
// dynamic shared memory of k_shortcuts for a cluster of L nodes
inline size_t shortcut_smem(size_t L) { return L * (sizeof(double) + 3 * sizeof(float)); }
// SSSP distances inside a cluster from each job's local source (summary.cu)
__global__ void __launch_bounds__(128) k_sssp_shortcuts(const uint32_t* __restrict__ job_cl,
                                                        const uint32_t* __restrict__ job_src,
                                                        const uint64_t* __restrict__ cl_off,
                                                        const uint64_t* __restrict__ adj_off,
                                                        const uint32_t* __restrict__ adj_nbr,
                                                        const float* __restrict__ adj_w,
                                                        const uint64_t* __restrict__ out_off,
                                                        double* __restrict__ out, uint32_t njobs);
// a warp per job for clusters of at most 32 x npl nodes (npl = 2 or 5), or
// half a warp per job for clusters of at most 48 nodes (npl = 3)
void launch_shortcuts_warp(int npl, ShortcutArgs A, uint32_t njobs, cudaStream_t st);
constexpr uint32_t kShortcutHalfL = 48;   // clusters the half-warp variant takes
constexpr uint32_t kShortcutSmallL = 64;  // clusters the npl = 2 variant takes

struct SummaryDev {
  bool valid = false;
  uint32_t old_n = 0, all_n = 0;
  Summary S;
  HostAdj out, in;  // host copy of the graph the summary was built on
  // The PageRank tables below are repaired on the device after each batch
  // (repair.cu).  The host restatement S (and the host graph copy) then
  // lags behind by the batches in the repair's action log; host_sync
  // replays them before anything reads S.
  RepairDev* rep = nullptr;
  // device sketch (the supernode lists live in the repair's slots)
  uint64_t *ib_off = nullptr, *sync_off = nullptr;
  uint32_t *ib_nbr = nullptr, *sync_nbr = nullptr;
  uint32_t* out_deg_all = nullptr;       // out-degree of each row (mirrors: master's)
  uint32_t *l_entry = nullptr, *l_exit = nullptr, *l_single = nullptr, *l_omirror = nullptr;
  uint32_t n_entry = 0, n_exit = 0, n_single = 0, n_omirror = 0;
  uint64_t n_ib = 0;                     // boundary edges of the exit and single rows
  uint32_t* omirror_master = nullptr;
  uint8_t* ntype = nullptr;
  // cluster precompute: members (cm layout: clusters in order) and, per
  // member position, the subgraph out-edges of clusters that are not staged
  uint64_t *cm_off = nullptr, *sub_off = nullptr;
  uint32_t *cm_v = nullptr, *sub_nbr = nullptr;
  uint64_t *lin_off = nullptr, *lout_off = nullptr;  // per cm_v position (staged clusters)
  uint8_t* lin_src = nullptr;
  uint32_t* lout_dst = nullptr;
  uint32_t *bound_list = nullptr;  // exit members per cluster (cm layout)
  uint64_t* bl_off = nullptr;
  // state
  float *bound = nullptr, *spnode = nullptr, *old_x = nullptr;
  double* d_res = nullptr;
  uint32_t* sctl = nullptr;  // summarized rounds: done flag, blocks finished, rounds run
  // SSSP over the summary (built by repair.cu on the first query): the
  // summarized CSR and the correction lists
  bool sssp_ready = false;
  uint64_t *sk_off = nullptr, *sk_coff = nullptr;
  uint32_t *sk_deg = nullptr, *sk_col = nullptr, *sk_crow = nullptr, *sk_cv = nullptr;
  float *sk_w = nullptr, *sk_cd = nullptr;
  uint64_t sk_m = 0;
  uint32_t sk_ncorr = 0;
  // IncEval over the summary: the rows whose shortcuts are relaxed again
  // (every supernode's entry or in-mirror) and the in-mirrors with their
  // masters (a mirror starts from its master's distance)
  uint32_t *sk_spid = nullptr, *sk_imir = nullptr, *sk_imaster = nullptr;
  uint32_t sk_nspid = 0, sk_nimir = 0;
  // the construction's state between its two halves, serialized
  std::vector<uint8_t> init_blob;
  std::unordered_map<const void*, uint64_t> dcap;  // reupload capacities
  // device staging of the shortcut and SSSP passes, kept between calls so a
  // batch costs copies instead of frees and allocations (slot -> buffer)
  struct Stage {
    void* p = nullptr;
    size_t cap = 0;
  };
  Stage stage[32];
  SsspViewScratch view;  // queues of the delta-stepping runs over the summary
  // message_type = pull: per-vertex in-indexes (summary_pull_view)
  bool pull_stale = true;
  PullView pv;
  uint8_t* p_cls = nullptr;
  uint64_t *p_ie_off = nullptr, *p_bd_off = nullptr;
  uint32_t *p_ie_nbr = nullptr, *p_bd_src = nullptr, *p_act = nullptr, *p_ent = nullptr;
  float* p_bd_w = nullptr;
};


// repair.cu: the incremental repair of the PageRank tables on the device
sg_status repair_init(sg_ctx* ctx, SummaryDev& D);
sg_status repair_after_apply(sg_ctx* ctx, SummaryDev& D);
sg_status repair_pending_clusters(sg_ctx* ctx, SummaryDev& D, const uint32_t** list, uint32_t* count);
SpLists repair_lists(const SummaryDev& D);
uint64_t repair_logged_actions(const SummaryDev& D);
uint64_t repair_logged_batches(const SummaryDev& D);
sg_status repair_take_log(sg_ctx* ctx, SummaryDev& D, std::vector<uint32_t>* src,
                          std::vector<uint32_t>* dst, std::vector<uint32_t>* kind,
                          std::vector<uint32_t>* found, std::vector<float>* w,
                          std::vector<uint64_t>* batch_end);
void repair_free(SummaryDev& D);
// SSSP over the summary from the device repair's state: distance blocks of
// every supernode (built on the first call, repaired with each batch), the
// summarized CSR and the correction lists in SummaryDev's sk_* tables.
bool repair_active(const SummaryDev& D);
sg_status repair_sssp_refresh(sg_ctx* ctx, SummaryDev& D);
// Seeds of a source inside a cluster: every member (an out-mirror as its
// master) with its distance from a local solve of the source's cluster, in
// device arrays valid until the next repair call.
sg_status repair_source_seeds(sg_ctx* ctx, SummaryDev& D, uint32_t source, const uint32_t** v,
                              const double** d, uint32_t* count);

}  // namespace sg
