// Reference harness driver (test infrastructure): loads a graph with the
// reference's loader, runs the reference's SumInc (or plain Ingress) worker
// for PageRank or SSSP exactly as CreateAndQueryTypeOne / TypeTwo do
// (examples/analytical_apps/ingress.h:71-177), and writes the per-vertex
// results as little-endian float64 to --out.
//
// usage: ref_driver <pagerank|pagerank_pull|pagerank_plain|sssp|sssp_plain> <out.bin> flag=value ...
// (pagerank_pull runs SumSyncIterWorkerPull, the message_type=pull worker)
//        (flags as in examples/analytical_apps/flags.cc)
#include <gflags/gflags.h>
#include <glog/logging.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "flags.h"
#include "grape/fragment/immutable_edgecut_fragment.h"
#include "grape/fragment/loader.h"
#include "grape/grape.h"
#include "grape/worker/ingress_sync_iter_worker.h"
#include "grape/worker/sum_sync_iter_worker.h"
#include "grape/worker/sum_sync_iter_worker_pull.h"
#include "grape/worker/ingress_sync_traversal_worker.h"
#include "grape/worker/sum_sync_traversal_worker.h"
#include "pagerank/pagerank_ingress.h"
#include "sssp/sssp_ingress.h"

namespace sg_harness {

// Thin subclasses that only expose the protected state arrays.
template <typename FRAG_T, typename VALUE_T>
struct PR : public grape::PageRankIngress<FRAG_T, VALUE_T> {
  std::vector<double> result(size_t n) {
    std::vector<double> r(n);
    for (size_t i = 0; i < n; ++i) r[i] = this->values_[typename FRAG_T::vertex_t(i)];
    return r;
  }
  double residual(size_t n) {
    double s = 0;
    for (size_t i = 0; i < n; ++i) s += std::fabs((double)this->deltas_[typename FRAG_T::vertex_t(i)]);
    return s;
  }
};

template <typename FRAG_T, typename VALUE_T>
struct SSSP : public grape::SSSPIngress<FRAG_T, VALUE_T> {
  // SSSP results are min(values_, deltas_.value): with -cilk=false the
  // shortcut correction updates only deltas_ (sssp_ingress.h:207-216).
  std::vector<double> result(size_t n) {
    std::vector<double> r(n);
    for (size_t i = 0; i < n; ++i) {
      typename FRAG_T::vertex_t v(i);
      VALUE_T a = this->values_[v], b = this->deltas_[v].value;
      VALUE_T m = a < b ? a : b;
      r[i] = (m == std::numeric_limits<VALUE_T>::max()) ? INFINITY : (double)m;
    }
    return r;
  }
};

void write(const std::string& path, const std::vector<double>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
}

template <typename FRAG_T>
std::shared_ptr<FRAG_T> load(const grape::CommSpec& cs) {
  grape::LoadGraphSpec spec = grape::DefaultLoadGraphSpec();
  spec.set_directed(FLAGS_directed);
  spec.set_rebalance(false, 0);
  return grape::LoadGraph<FRAG_T, grape::SegmentedPartitioner<typename FRAG_T::oid_t>>(
      FLAGS_efile, FLAGS_vfile, cs, spec);
}

}  // namespace sg_harness

int main(int argc, char** argv) {
  using namespace sg_harness;
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <app> <out.bin> flag=value...\n", argv[0]);
    return 2;
  }
  const std::string app = argv[1], out = argv[2];
  for (int i = 3; i < argc; ++i) {
    std::string a = argv[i];
    while (!a.empty() && a[0] == '-') a.erase(0, 1);
    const auto eq = a.find('=');
    if (eq == std::string::npos || !sg_gflags::Set(a.substr(0, eq), a.substr(eq + 1))) {
      std::fprintf(stderr, "unknown flag %s\n", argv[i]);
      return 2;
    }
  }
  grape::InitMPIComm();
  {
    grape::CommSpec cs;
    cs.Init(MPI_COMM_WORLD);
    auto pe = grape::DefaultParallelEngineSpec();
    if (FLAGS_app_concurrency != -1) {
      pe.thread_num = FLAGS_app_concurrency;
      setWorkers(FLAGS_app_concurrency);
    }
    if (app == "pagerank" || app == "pagerank_pull" || app == "pagerank_plain") {
      using G = grape::ImmutableEdgecutFragment<int32_t, uint32_t, grape::EmptyType,
                                                grape::EmptyType, grape::LoadStrategy::kBothOutIn>;
      using A = PR<G, float>;
      auto frag = load<G>(cs);
      const size_t n = frag->GetInnerVerticesNum();
      auto a = std::make_shared<A>();
      if (app == "pagerank") {
        grape::SumSyncIterWorker<A> w(a, frag);
        w.Init(cs, pe);
        w.Query();
        w.Finalize();
      } else if (app == "pagerank_pull") {
        grape::SumSyncIterWorkerPull<A> w(a, frag);
        w.Init(cs, pe);
        w.Query();
        w.Finalize();
      } else {
        grape::IngressSyncIterWorker<A> w(a, frag);
        w.Init(cs, pe);
        w.Query();
        w.Finalize();
      }
      std::fprintf(stderr, "#harness residual %.10e\n", a->residual(n));
      write(out, a->result(n));
    } else if (app == "sssp" || app == "sssp_plain") {
      using G = grape::ImmutableEdgecutFragment<int32_t, uint32_t, grape::EmptyType, uint16_t,
                                                grape::LoadStrategy::kBothOutIn>;
      using A = SSSP<G, int32_t>;
      auto frag = load<G>(cs);
      const size_t n = frag->GetInnerVerticesNum();
      auto a = std::make_shared<A>();
      if (app == "sssp") {
        grape::SumSyncTraversalWorker<A> w(a, frag);
        w.Init(cs, pe);
        w.Query();
        w.Finalize();
      } else {
        grape::IngressSyncTraversalWorker<A> w(a, frag);
        w.Init(cs, pe);
        w.Query();
        w.Finalize();
      }
      write(out, a->result(n));
    } else {
      std::fprintf(stderr, "unknown app %s\n", app.c_str());
      return 2;
    }
  }
  grape::FinalizeMPIComm();
  return 0;
}
