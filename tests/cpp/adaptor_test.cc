// Drives the header-only C++ workers (include/suminc_gb300_worker.hpp) with
// a minimal stand-in for the reference's fragment and app types (the members
// the workers use: InnerVertices, GetInnerVerticesNum, GetId,
// GetOutgoingAdjList with neighbor / data, init_c, GetInitDelta).
//
// usage: adaptor_test <efile> <update_pr> <update_sssp> <out_pr> <out_sssp> <n> [clusters]
// (with a cluster file, also the pull worker over the summary into <out_pr>.pull)
//   efile lines "u v w" with oids 10 * vid + 7; n vertices
#include <cmath>
#include <cstdio>
#include <fstream>
#include <limits>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "suminc_gb300_worker.hpp"

namespace grape {

struct Vertex {
  uint32_t v;
  uint32_t GetValue() const { return v; }
};

template <typename E>
struct Nbr {
  Vertex neighbor;
  E data;
};

struct VertexList {
  uint32_t n;
  struct It {
    uint32_t i;
    Vertex operator*() const { return Vertex{i}; }
    It& operator++() { ++i; return *this; }
    bool operator!=(const It& o) const { return i != o.i; }
  };
  It begin() const { return It{0}; }
  It end() const { return It{n}; }
};

template <typename E>
class Fragment {
 public:
  using edata_t = E;
  using vertex_t = Vertex;
  std::vector<std::vector<Nbr<E>>> out;
  std::vector<int64_t> oid;
  VertexList InnerVertices() const { return VertexList{(uint32_t)out.size()}; }
  size_t GetInnerVerticesNum() const { return out.size(); }
  int64_t GetId(Vertex v) const { return oid[v.v]; }
  const std::vector<Nbr<E>>& GetOutgoingAdjList(Vertex v) const { return out[v.v]; }
};

template <typename FRAG_T, typename VALUE_T>
class PageRankIngress {
 public:
  using fragment_t = FRAG_T;
  using value_t = VALUE_T;
  using vertex_t = Vertex;
  void init_c(const vertex_t, value_t& delta, const FRAG_T& frag) {
    delta = (value_t)((1.0 - 0.85) / (double)frag.GetInnerVerticesNum());
  }
};

template <typename V>
struct DependencyData {
  uint32_t parent_gid;
  V value;
};

template <typename FRAG_T, typename VALUE_T>
class SSSPIngress {
 public:
  using fragment_t = FRAG_T;
  using value_t = VALUE_T;
  using vertex_t = Vertex;
  using delta_t = DependencyData<VALUE_T>;
  uint32_t source = 0;
  delta_t GetInitDelta(const vertex_t& v) const {
    return delta_t{v.v, v.v == source ? (VALUE_T)0 : std::numeric_limits<VALUE_T>::max()};
  }
};

}  // namespace grape

int main(int argc, char** argv) {
  if (argc != 7 && argc != 8) {
    std::fprintf(stderr, "usage: %s efile update_pr update_sssp out_pr out_sssp n [clusters]\n",
                 argv[0]);
    return 2;
  }
  using FragW = grape::Fragment<uint16_t>;
  auto frag = std::make_shared<FragW>();
  frag->out.resize((size_t)std::stoul(argv[6]));
  std::ifstream in(argv[1]);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    int64_t u, v;
    int w;
    if (!(ss >> u >> v >> w)) continue;
    const uint32_t a = (uint32_t)((u - 7) / 10), b = (uint32_t)((v - 7) / 10);
    const uint32_t need = std::max(a, b) + 1;
    if (frag->out.size() < need) frag->out.resize(need);
    frag->out[a].push_back(grape::Nbr<uint16_t>{grape::Vertex{b}, (uint16_t)w});
  }
  frag->oid.resize(frag->out.size());
  for (size_t i = 0; i < frag->oid.size(); ++i) frag->oid[i] = 10 * (int64_t)i + 7;
  try {
    {
      using App = grape::PageRankIngress<FragW, float>;
      suminc_gb300::GpuWorkerOptions o;
      o.compress = false;
      o.update_file = argv[2];
      suminc_gb300::GpuSumSyncIterWorker<App> w(std::make_shared<App>(), frag, o);
      w.Init(0, 0);
      w.Query();
      std::ofstream os(argv[4]);
      w.Output(os);
      w.Finalize();
    }
    if (argc > 7) {  // the pull worker over a summary (cluster file argv[7])
      using App = grape::PageRankIngress<FragW, float>;
      suminc_gb300::GpuWorkerOptions o;
      o.compress = true;
      o.pull = true;
      o.mirror_k = 1 << 30;
      o.cluster_file = argv[7];
      o.update_file = argv[2];
      suminc_gb300::GpuSumSyncIterWorker<App> w(std::make_shared<App>(), frag, o);
      w.Init(0, 0);
      w.Query();
      std::ofstream os(std::string(argv[4]) + ".pull");
      w.Output(os);
      w.Finalize();
    }
    {
      using App = grape::SSSPIngress<FragW, double>;
      auto app = std::make_shared<App>();
      app->source = 3;
      suminc_gb300::GpuWorkerOptions o;
      o.update_file = argv[3];
      suminc_gb300::GpuSumSyncTraversalWorker<App> w(app, frag, o);
      w.Init(0);
      w.Query();
      std::ofstream os(argv[5]);
      os.precision(17);
      w.Output(os);
      w.Finalize();
    }
    if (argc > 7) {  // SSSP over the summary (cluster file argv[7])
      using App = grape::SSSPIngress<FragW, double>;
      auto app = std::make_shared<App>();
      app->source = 3;
      suminc_gb300::GpuWorkerOptions o;
      o.compress = true;
      o.cluster_file = argv[7];
      o.update_file = argv[3];
      suminc_gb300::GpuSumSyncTraversalWorker<App> w(app, frag, o);
      w.Init(0);
      w.Query();
      std::ofstream os(std::string(argv[5]) + ".sum");
      os.precision(17);
      w.Output(os);
      w.Finalize();
    }
  } catch (const suminc_gb300::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
