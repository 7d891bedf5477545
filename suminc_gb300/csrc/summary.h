// Summarized graph ("sketch") built from a clustering: supernodes (one per
// entry vertex of each kept cluster), in/out mirrors, exit ("bound")
// vertices, per-cluster subgraphs, node types and the three sketch CSRs the
// summarized rounds traverse.  Host-side structures; the shortcut weights
// are computed on the device (summary.cu).
#pragma once

#include <stdint.h>

#include <unordered_set>
#include <utility>
#include <vector>

namespace sg {

struct HostAdj {
  uint32_t n = 0;
  std::vector<uint64_t> rp;
  std::vector<uint32_t> col;
  std::vector<float> w;  // empty for unweighted graphs
  // host_adj_patch writes the patched copy here and swaps: the buffers keep
  // their size between batches, so no pass zero-fills a fresh array
  std::vector<uint64_t> rp_spare;
  std::vector<uint32_t> col_spare;
  std::vector<float> w_spare;
  uint64_t deg(uint32_t v) const { return rp[v + 1] - rp[v]; }
};

// One change to a host adjacency (row, col), from the device applier's
// normalized actions: remove an edge that exists, set the weight of one
// that exists, or insert one that does not.
struct AdjOp {
  enum Kind : uint8_t { kRemove = 0, kSetWeight = 1, kInsert = 2 };
  uint32_t row, col;
  float w;
  uint8_t kind;
};

// Patches `a` (rows sorted by column) with `ops` sorted by (row, col); rows
// stay sorted.  Rows without changes are moved in bulk.  Returns false, with
// `a` unchanged, when an op does not fit `a` (an insert of an edge that
// exists, a removal of one that does not).
bool host_adj_patch(HostAdj& a, const std::vector<AdjOp>& ops);

// node types (grape/types.h:70-78)
enum NodeTypeCode : char {
  kSingle = 0, kOnlyOut = 1, kOnlyIn = 2, kBothOutIn = 3, kInner = 4, kOutMaster = 5,
  kBothOutInMaster = 6
};

struct Supernode {
  uint32_t id = 0;   // entry vertex or in-mirror id
  uint32_t ids = 0;  // cluster index
  bool status = false;
  std::vector<std::pair<uint32_t, double>> inner_value, inner_delta, bound_delta;
  void clear() {
    status = false;
    inner_value.clear();
    inner_delta.clear();
    bound_delta.clear();
  }
};

struct Summary {
  static constexpr int32_t kFcDefault = 0x7FFFFFFF;
  static constexpr uint32_t kIdDefault = 0xFFFFFFFFu;
  uint32_t old_n = 0, all_n = 0;
  std::vector<int32_t> Fc;          // < 0: member of cluster -(Fc+1); >= 0: entry of cluster Fc
  std::vector<uint32_t> id2spids;   // cluster of each vertex / mirror (all_n)
  std::vector<uint32_t> Fc_map;     // supernode of each entry / in-mirror (all_n)
  std::vector<std::vector<uint32_t>> supernode_ids;   // members (+ absorbed vertices)
  std::vector<std::vector<uint32_t>> cluster_ids;     // members + mirror ids
  std::vector<std::vector<uint32_t>> supernode_source;
  std::vector<std::vector<uint32_t>> cluster_in_mirror_ids, cluster_out_mirror_ids;
  std::vector<std::unordered_set<uint32_t>> supernode_in_mirror, supernode_out_mirror;
  std::vector<std::vector<uint32_t>> vid2in_mirror_mids;
  std::vector<uint32_t> mirrorid2vid;  // index: mirror id - old_n
  std::vector<Supernode> supernodes;
  std::vector<short> out_bound;
  std::vector<std::vector<uint32_t>> subgraph;      // inner edges (+ mirror edges)
  std::vector<std::vector<float>> subgraph_w;
  std::vector<char> node_type;                      // old_n entries
  std::vector<uint32_t> all_out_mirror;
  // sketch CSRs over all_n rows
  std::vector<uint64_t> is_off, ib_off, sync_off;
  std::vector<uint32_t> is_nbr, ib_nbr, sync_nbr;
  std::vector<float> is_w, ib_w;
  // incremental bookkeeping
  std::vector<uint32_t> update_cluster_ids, update_source_id;
  // statistics of the construction (compared with the reference's logs)
  uint64_t mirror_node_cnt = 0, inmirror2source_cnt = 0, outmirror2source_cnt = 0;

  uint32_t mirror_master(uint32_t m) const { return mirrorid2vid[m - old_n]; }
};

// In-repo greedy clustering (restates the flag-default builder).
std::vector<std::vector<uint32_t>> greedy_clusters(const HostAdj& out, const HostAdj& in,
                                                   int max_node_num, int min_node_num,
                                                   uint64_t seed);

// The two halves of the construction: supernode candidates and mirrors from
// the clustering (returns the mirror count), then the final build.
uint64_t summary_init_by_clusters(Summary& S, const HostAdj& out, const HostAdj& in,
                                  const std::vector<std::vector<uint32_t>>& clusters,
                                  int min_node_num, int mirror_k, double compress_threshold);
void summary_final_build(Summary& S, const HostAdj& in, uint64_t init_mirror_num);
// The state between the halves, in the reference's serialized layout.
std::vector<uint8_t> summary_serialize_init(const Summary& S, uint64_t init_mirror_num);
bool summary_deserialize_init(Summary& S, uint32_t n, const std::vector<uint8_t>& b,
                              uint64_t* init_mirror_num);
// Supernodes, mirrors and bookkeeping from a clustering.
void summary_from_clusters(Summary& S, const HostAdj& out, const HostAdj& in,
                           const std::vector<std::vector<uint32_t>>& clusters, int min_node_num,
                           int mirror_k, double compress_threshold);
void summary_judge_out_bound(Summary& S, const HostAdj& out, const std::vector<uint32_t>* only);
void summary_build_subgraph(Summary& S, const HostAdj& out, const HostAdj& in,
                            const std::vector<uint32_t>* only);
void summary_node_types(Summary& S);
void summary_sketch_csr(Summary& S, const HostAdj& out);
// Incremental entry changes for one batch (deleted / added pairs).
void summary_inc_entries(Summary& S, const HostAdj& new_out, const HostAdj& new_in,
                         const std::vector<std::pair<uint32_t, uint32_t>>& deleted,
                         const std::vector<std::pair<uint32_t, uint32_t>>& added);

}  // namespace sg
