// Header-only C++ drop-in for the reference's SumInc workers, over the C ABI
// of suminc_gb300.h.
//
//   suminc_gb300::GpuSumSyncIterWorker<APP_T>       for PageRankIngress apps
//   suminc_gb300::GpuSumSyncTraversalWorker<APP_T>  for SSSPIngress apps
//
// Same shape as grape::SumSyncIterWorker / grape::SumSyncTraversalWorker
// (grape/worker/sum_sync_iter_worker.h:61-65, :440, :2829-2870;
// grape/worker/sum_sync_traversal_worker.h:67-70, :2809): constructed from
// the app and its fragment, then Init / Query / Output / Finalize.  Query
// runs PEval on the GPU and, when an update file is set, applies it and runs
// IncEval.  The app's per-edge functions cannot run on the device, so the
// worker picks the device semantics by the app's type (app_traits below,
// specialised for grape::PageRankIngress and grape::SSSPIngress; other apps
// fail to compile), and reads the app's own init functions on the host to
// take the damping (PageRank: init_c = (1-d)/N) or the source (SSSP: the
// vertex whose initial delta is 0).
//
// Settings the reference takes from gflags are passed in GpuWorkerOptions;
// a driver fills them from its FLAGS_* of the same names.
#pragma once

#include <algorithm>
#include <cstdint>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "suminc_gb300.h"

namespace grape {
template <typename FRAG_T, typename VALUE_T>
class PageRankIngress;
template <typename FRAG_T, typename VALUE_T>
class SSSPIngress;
}  // namespace grape

namespace suminc_gb300 {

enum class AppKind { kPageRank, kSssp };

template <typename APP_T>
struct app_traits;  // no device semantics for this app

template <typename F, typename V>
struct app_traits<grape::PageRankIngress<F, V>> {
  static constexpr AppKind kind = AppKind::kPageRank;
};
template <typename F, typename V>
struct app_traits<grape::SSSPIngress<F, V>> {
  static constexpr AppKind kind = AppKind::kSssp;
};

struct GpuWorkerOptions {
  int device = 0;
  bool compress = true;              // FLAGS_compress
  double termcheck_threshold = 1e-6; // FLAGS_termcheck_threshold
  int max_node_num = 150;            // FLAGS_max_node_num
  int min_node_num = 8;              // FLAGS_min_node_num
  int mirror_k = 4;                  // FLAGS_mirror_k
  double compress_threshold = 1.0;   // FLAGS_compress_threshold
  bool pull = false;                 // FLAGS_message_type == "pull" (PageRank)
  std::string cluster_file;          // <efile>.c_<max_node_num>; empty: no summary
  std::string update_file;           // FLAGS_efile_update; empty: PEval only
};

class Error : public std::runtime_error {
 public:
  Error(sg_status st, const std::string& what) : std::runtime_error(what), status(st) {}
  sg_status status;
};

namespace detail {

inline void check(sg_status st, sg_ctx* ctx, const char* what) {
  if (st == SG_OK) return;
  std::string msg = std::string(what) + ": ";
  msg += ctx ? sg_last_error(ctx) : "context creation failed";
  throw Error(st, msg);
}

template <typename T, typename = void>
struct has_arith_edata : std::false_type {};
template <typename T>
struct has_arith_edata<T, typename std::enable_if<std::is_arithmetic<T>::value>::type>
    : std::true_type {};

// CSR of the fragment's inner vertices (one fragment: local vid = row)
template <typename FRAG_T>
void fragment_csr(const FRAG_T& frag, std::vector<uint64_t>& rp, std::vector<uint32_t>& col,
                  std::vector<float>& w, std::vector<uint64_t>& oid) {
  using edata_t = typename FRAG_T::edata_t;
  const auto iv = frag.InnerVertices();
  const uint32_t n = (uint32_t)frag.GetInnerVerticesNum();
  rp.assign((size_t)n + 1, 0);
  col.clear();
  w.clear();
  oid.resize(n);
  for (auto v : iv) {
    const uint32_t u = (uint32_t)v.GetValue();
    oid[u] = (uint64_t)frag.GetId(v);
    auto es = frag.GetOutgoingAdjList(v);
    std::vector<std::pair<uint32_t, float>> row;
    for (auto& e : es) {
      float x = 1.f;
      if constexpr (has_arith_edata<edata_t>::value) x = (float)e.data;
      row.emplace_back((uint32_t)e.neighbor.GetValue(), x);
    }
    std::sort(row.begin(), row.end());
    rp[u + 1] = row.size();
    for (auto& r : row) {
      col.push_back(r.first);
      if constexpr (has_arith_edata<edata_t>::value) w.push_back(r.second);
    }
  }
  for (uint32_t u = 0; u < n; ++u) rp[u + 1] += rp[u];
}

class Ctx {
 public:
  Ctx() = default;
  Ctx(const Ctx&) = delete;
  Ctx& operator=(const Ctx&) = delete;
  ~Ctx() { reset(); }
  void create(int device, const sg_options& opt) {
    reset();
    check(sg_ctx_create(device, &opt, &h_), nullptr, "sg_ctx_create");
  }
  void reset() {
    if (h_) sg_ctx_destroy(h_);
    h_ = nullptr;
  }
  sg_ctx* get() const { return h_; }

 private:
  sg_ctx* h_ = nullptr;
};

}  // namespace detail

template <typename APP_T, AppKind KIND>
class GpuWorkerBase {
 public:
  using fragment_t = typename APP_T::fragment_t;
  using vertex_t = typename APP_T::vertex_t;

  GpuWorkerBase(std::shared_ptr<APP_T> app, std::shared_ptr<fragment_t>& graph,
                GpuWorkerOptions opt = GpuWorkerOptions())
      : app_(app), graph_(graph), wopt_(std::move(opt)) {
    static_assert(app_traits<APP_T>::kind == KIND, "app kind does not match this worker");
  }

  // The reference's Init(comm_spec, pe_spec): one process, one GPU, so
  // both are accepted and unused.
  template <typename... SPEC>
  void Init(const SPEC&...) {
    sg_options o;
    sg_options_default(&o);
    o.compress = wopt_.compress ? 1 : 0;
    o.termcheck_threshold = wopt_.termcheck_threshold;
    o.max_node_num = wopt_.max_node_num;
    o.min_node_num = wopt_.min_node_num;
    o.mirror_k = wopt_.mirror_k;
    o.compress_threshold = wopt_.compress_threshold;
    o.message_type = wopt_.pull ? SG_MSG_PULL : SG_MSG_PUSH;
    configure(o);
    ctx_.create(wopt_.device, o);
    std::vector<float> w;
    detail::fragment_csr(*graph_, rp_, col_, w, oid_);
    detail::check(sg_graph_load_csr(ctx_.get(), (uint32_t)(rp_.size() - 1), rp_.data(),
                                    col_.data(), w.empty() ? nullptr : w.data()),
                  ctx_.get(), "sg_graph_load_csr");
    detail::check(sg_graph_set_vertex_oids(ctx_.get(), oid_.data()), ctx_.get(),
                  "sg_graph_set_vertex_oids");
    // the summary both workers run over (SumSyncIterWorker and
    // SumSyncTraversalWorker build their compressor in Init)
    if (wopt_.compress && !wopt_.cluster_file.empty())
      detail::check(sg_summary_build_file(ctx_.get(), wopt_.cluster_file.c_str()), ctx_.get(),
                    "sg_summary_build_file");
  }

  void Finalize() { ctx_.reset(); }

  sg_ctx* context() const { return ctx_.get(); }
  const sg_stats stats() const {
    sg_stats s{};
    sg_get_stats(ctx_.get(), &s);
    return s;
  }

 protected:
  virtual void configure(sg_options&) {}

  std::shared_ptr<APP_T> app_;
  std::shared_ptr<fragment_t> graph_;
  GpuWorkerOptions wopt_;
  detail::Ctx ctx_;
  std::vector<uint64_t> rp_, oid_;
  std::vector<uint32_t> col_;
};

// PageRank (SumSyncIterWorker with compress = 1, IngressSyncIterWorker with
// compress = 0).
template <typename APP_T>
class GpuSumSyncIterWorker : public GpuWorkerBase<APP_T, AppKind::kPageRank> {
  using Base = GpuWorkerBase<APP_T, AppKind::kPageRank>;

 public:
  using Base::Base;

  void Query() {
    sg_ctx* c = this->ctx_.get();
    detail::check(sg_pr_peval(c, nullptr), c, "sg_pr_peval");
    if (!this->wopt_.update_file.empty()) {
      detail::check(sg_apply_update_file(c, this->wopt_.update_file.c_str()), c,
                    "sg_apply_update_file");
      detail::check(sg_pr_inceval(c, nullptr), c, "sg_pr_inceval");
    }
    values_.resize(this->rp_.size() - 1);
    detail::check(sg_pr_values(c, values_.data()), c, "sg_pr_values");
  }

  // "oid value" per vertex, as SumSyncIterWorker::Output
  void Output(std::ostream& os) const {
    for (size_t v = 0; v < values_.size(); ++v) os << this->oid_[v] << " " << values_[v] << "\n";
  }

  const std::vector<float>& values() const { return values_; }

 protected:
  // damping from the app's own init_c: delta_0 = (1 - d) / N
  void configure(sg_options& o) override {
    const auto iv = this->graph_->InnerVertices();
    const double n = (double)this->graph_->GetInnerVerticesNum();
    for (auto v : iv) {
      typename APP_T::value_t delta{};
      this->app_->init_c(v, delta, *this->graph_);
      o.damping = 1.0 - (double)delta * n;
      break;
    }
  }

 private:
  std::vector<float> values_;
};

// SSSP (SumSyncTraversalWorker).
template <typename APP_T>
class GpuSumSyncTraversalWorker : public GpuWorkerBase<APP_T, AppKind::kSssp> {
  using Base = GpuWorkerBase<APP_T, AppKind::kSssp>;

 public:
  using Base::Base;

  void Query() {
    sg_ctx* c = this->ctx_.get();
    // the source: the vertex whose initial delta is 0 (GetInitDelta)
    uint32_t source = 0;
    for (auto v : this->graph_->InnerVertices()) {
      if (this->app_->GetInitDelta(v).value == 0) {
        source = (uint32_t)v.GetValue();
        break;
      }
    }
    detail::check(sg_sssp_peval(c, source, nullptr), c, "sg_sssp_peval");
    if (!this->wopt_.update_file.empty()) {
      detail::check(sg_apply_update_file(c, this->wopt_.update_file.c_str()), c,
                    "sg_apply_update_file");
      detail::check(sg_sssp_inceval(c, nullptr), c, "sg_sssp_inceval");
    }
    dist_.resize(this->rp_.size() - 1);
    detail::check(sg_sssp_distances(c, dist_.data()), c, "sg_sssp_distances");
  }

  void Output(std::ostream& os) const {
    for (size_t v = 0; v < dist_.size(); ++v) os << this->oid_[v] << " " << dist_[v] << "\n";
  }

  const std::vector<double>& distances() const { return dist_; }

 private:
  std::vector<double> dist_;
};

}  // namespace suminc_gb300
