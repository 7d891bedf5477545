// Compile check (test infrastructure): the header-only C++ workers of
// include/suminc_gb300_worker.hpp instantiated with the reference's own
// fragment and app types, as a driver switching to them would write it.
// Built with -fsyntax-only against the reference checkout; never run.
#include "flags.h"
#include "grape/fragment/immutable_edgecut_fragment.h"
#include "grape/grape.h"
#include "pagerank/pagerank_ingress.h"
#include "sssp/sssp_ingress.h"
#include "suminc_gb300_worker.hpp"

void check_workers(const grape::CommSpec& cs, const grape::ParallelEngineSpec& pe) {
  using PRFrag = grape::ImmutableEdgecutFragment<int32_t, uint32_t, grape::EmptyType,
                                                 grape::EmptyType, grape::LoadStrategy::kBothOutIn>;
  using SSFrag = grape::ImmutableEdgecutFragment<int32_t, uint32_t, grape::EmptyType, uint16_t,
                                                 grape::LoadStrategy::kBothOutIn>;
  std::shared_ptr<PRFrag> pf;
  std::shared_ptr<SSFrag> sf;
  suminc_gb300::GpuWorkerOptions o;
  {
    using App = grape::PageRankIngress<PRFrag, float>;
    suminc_gb300::GpuSumSyncIterWorker<App> w(std::make_shared<App>(), pf, o);
    w.Init(cs, pe);
    w.Query();
    w.Output(std::cout);
    w.Finalize();
  }
  {
    using App = grape::SSSPIngress<SSFrag, int32_t>;
    suminc_gb300::GpuSumSyncTraversalWorker<App> w(std::make_shared<App>(), sf, o);
    w.Init(cs, pe);
    w.Query();
    w.Output(std::cout);
    w.Finalize();
  }
}
