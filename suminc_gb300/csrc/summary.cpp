// Host construction of the summarized graph.  Each function restates one
// step of the reference's CompressorBase (grape/fragment/compressor_base.h)
// and keeps its observable rules, including the container types whose
// iteration order feeds into the result (mirror sets are unordered sets of
// vertex ids with the identity hash, built from sorted ranges).
#include "summary.h"

#include <algorithm>
#include <cstring>
#include <cmath>
#include <set>
#include <unordered_map>

#include "common.h"

namespace sg {

// ---------------------------------------------------------------- greedy
//
// compressor_base.h:367-419 (dispatch, one compress thread) and :1448-1875
// (parallel_find_multi_source_supernode_2_sort_sample).  The reference draws
// its candidate samples from std::random_device; this restatement draws them
// from a seeded counter-based generator so the clustering is reproducible.

namespace {

struct CandidateQueue {  // grape/utils/Queue.h: vector queue with swap-erase
  std::vector<uint32_t> data;
  uint32_t head = 0, tail = 0;
  void push(uint32_t v) {
    if (tail >= data.size()) data.resize(std::max<size_t>(16, data.size() * 2));
    data[tail++] = v;
  }
  void erase(uint32_t id) {
    if (id != tail - 1) std::swap(data[id], data[tail - 1]);
    tail--;
  }
  uint32_t size() const { return tail - head; }
  bool empty() const { return size() == 0; }
};

struct Rng {
  uint64_t key, ctr = 0;
  explicit Rng(uint64_t seed) : key(mix64(seed ^ 0x94D049BB133111EBull)) {}
  uint64_t next() { return mix64(key + (ctr++)); }
};

// Membership of the find's sets P (cluster), S (vertices with in-edges from
// outside), B (vertices with out-edges to outside) and the visited marks are
// vertex-indexed stamps equal to the find's number, and every vertex touched
// by P keeps two counters: its in-edge entries from P and its out-edge
// entries into P, updated when a vertex joins P.  The score of a candidate d
// then needs no scan of the in-rows of its out-neighbours (or the out-rows of
// its in-neighbours): "every in-edge of o comes from P or from d" is
// in_deg(o) - (entries from P) - (entries from d) == 0.  The ordered sets
// are kept as std::set for their iteration order, which decides the cluster
// member order and the tie-breaking of the reference.  Scores, samples and
// clusters are the same as with a scan of the adjacency.
struct Greedy {
  const HostAdj& out;
  const HostAdj& in;
  int max_node_num;
  std::vector<int32_t> Fc;
  std::vector<std::vector<uint32_t>> clusters;
  Rng rng;
  uint32_t epoch = 0;
  std::vector<uint32_t> st_p, st_s, st_b, st_vis, st_cnt;
  std::vector<uint32_t> c_in_p, c_out_p;

  Greedy(const HostAdj& o, const HostAdj& i, int mx, uint64_t seed)
      : out(o), in(i), max_node_num(mx), Fc(o.n, Summary::kFcDefault), rng(seed),
        st_p(o.n, 0), st_s(o.n, 0), st_b(o.n, 0), st_vis(o.n, 0), st_cnt(o.n, 0),
        c_in_p(o.n, 0), c_out_p(o.n, 0) {}

  bool in_p(uint32_t v) const { return st_p[v] == epoch; }
  bool in_s(uint32_t v) const { return st_s[v] == epoch; }
  bool in_b(uint32_t v) const { return st_b[v] == epoch; }
  uint64_t cin(uint32_t v) const { return st_cnt[v] == epoch ? c_in_p[v] : 0; }
  uint64_t cout(uint32_t v) const { return st_cnt[v] == epoch ? c_out_p[v] : 0; }
  void touch(uint32_t v) {
    if (st_cnt[v] != epoch) {
      st_cnt[v] = epoch;
      c_in_p[v] = 0;
      c_out_p[v] = 0;
    }
  }
  // entries equal to x in the (sorted) row of v
  static uint64_t mult(const HostAdj& a, uint32_t v, uint32_t x) {
    const uint32_t* b = a.col.data() + a.rp[v];
    const uint32_t* e = a.col.data() + a.rp[v + 1];
    const auto r = std::equal_range(b, e, x);
    return (uint64_t)(r.second - r.first);
  }
  void join(uint32_t d, std::set<uint32_t>& P) {
    P.insert(d);
    st_p[d] = epoch;
    for (uint64_t e = out.rp[d]; e < out.rp[d + 1]; ++e) {
      touch(out.col[e]);
      c_in_p[out.col[e]]++;
    }
    for (uint64_t e = in.rp[d]; e < in.rp[d + 1]; ++e) {
      touch(in.col[e]);
      c_out_p[in.col[e]]++;
    }
  }
  void s_insert(std::set<uint32_t>& S, uint32_t v) { S.insert(v); st_s[v] = epoch; }
  void s_erase(std::set<uint32_t>& S, uint32_t v) { S.erase(v); st_s[v] = 0; }
  void b_insert(std::set<uint32_t>& B, uint32_t v) { B.insert(v); st_b[v] = epoch; }
  void b_erase(std::set<uint32_t>& B, uint32_t v) { B.erase(v); st_b[v] = 0; }

  // Members x of `set` (ascending) adjacent to d in `adj` row d whose rows in
  // `other` hold no entry outside P other than d: by the set when it is much
  // shorter than d's row, else by a pass over the row (sorted, so the result
  // is ascending either way).
  template <typename InSet, typename Count>
  void closed_members(uint32_t d, const HostAdj& adj, const HostAdj& other,
                      const std::set<uint32_t>& set, InSet member, Count from_p,
                      std::vector<uint32_t>& res) const {
    res.clear();
    if (set.empty()) return;
    const uint64_t b = adj.rp[d], e = adj.rp[d + 1];
    if ((uint64_t)set.size() * 8 < e - b) {
      for (uint32_t x : set) {
        const uint64_t m = mult(adj, d, x);
        if (m && other.deg(x) - from_p(x) - m == 0) res.push_back(x);
      }
      return;
    }
    for (uint64_t k = b; k < e;) {
      const uint32_t x = adj.col[k];
      uint64_t r = k + 1;
      while (r < e && adj.col[r] == x) ++r;
      if (member(x) && other.deg(x) - from_p(x) - (r - k) == 0) res.push_back(x);
      k = r;
    }
  }

  // compressor_base.h:1364-1440 (check_score): inner edges after adding d
  // minus |S'| x |B'|
  float check_score(uint32_t d, const std::set<uint32_t>& S, const std::set<uint32_t>& B,
                    uint32_t inner, bool& is_s, bool& is_b, uint32_t& temp_inner,
                    std::vector<uint32_t>& tS, std::vector<uint32_t>& tB) const {
    temp_inner = inner;
    // out-edges of d: into P or back to d are inner, any other makes d a B member
    const uint64_t inner_out = cout(d) + mult(out, d, d);
    temp_inner += (uint32_t)inner_out;
    is_b = out.deg(d) > inner_out;
    // in-edges of d: from P are inner, any other makes d an S member
    const uint64_t inner_in = cin(d);
    temp_inner += (uint32_t)inner_in;
    is_s = in.deg(d) > inner_in;
    // S members d points to whose in-edges then all come from P or d leave S;
    // B members pointing to d whose out-edges all go to P or d leave B
    closed_members(d, out, in, S, [&](uint32_t x) { return in_s(x); },
                   [&](uint32_t x) { return cin(x); }, tS);
    closed_members(d, in, out, B, [&](uint32_t x) { return in_b(x); },
                   [&](uint32_t x) { return cout(x); }, tB);
    uint32_t now_s = (uint32_t)S.size() - (uint32_t)tS.size();
    uint32_t now_b = (uint32_t)B.size() - (uint32_t)tB.size();
    if (is_s) now_s++;
    if (is_b) now_b++;
    return (float)(temp_inner * 1.0 - (double)(uint32_t)(now_s * now_b));
  }

  void sample(const CandidateQueue& D, uint32_t want, std::vector<uint32_t>& out_idx) {
    out_idx.clear();
    if (want >= D.size()) {
      for (uint32_t i = D.head; i < D.tail; ++i) out_idx.push_back(i);
      return;
    }
    std::set<uint32_t> taken;
    while (out_idx.size() < want) {
      const uint32_t pos = D.head + (uint32_t)(rng.next() % D.size());
      if (taken.insert(pos).second) out_idx.push_back(pos);
    }
  }

  void push_neighbours(uint32_t u, CandidateQueue& D, uint64_t try_max_node) {
    if (out.deg(u) >= try_max_node) return;
    for (uint64_t e = out.rp[u]; e < out.rp[u + 1]; ++e) {
      const uint32_t v = out.col[e];
      if (Fc[v] == Summary::kFcDefault && !in_p(v) && st_vis[v] != epoch) {
        D.push(v);
        st_vis[v] = epoch;
      }
    }
  }

  void find(uint32_t source, int now_min) {
    const uint64_t try_max_node = (uint64_t)max_node_num * 1000;
    const int try_max_step = max_node_num * 1000;
    const uint32_t sample_size = 32;
    const int try_sample_cnt = 3;
    ++epoch;
    std::set<uint32_t> S, P, B;
    CandidateQueue D;
    if (Fc[source] == Summary::kFcDefault) {
      join(source, P);
      st_vis[source] = epoch;
      push_neighbours(source, D, try_max_node);
    }
    uint32_t inner_edge_num = 0;
    for (uint32_t u : P) {
      bool f = true;
      for (uint64_t e = out.rp[u]; e < out.rp[u + 1]; ++e) {
        if (!in_p(out.col[e])) {
          if (f) {
            b_insert(B, u);
            f = false;
          }
        } else {
          inner_edge_num++;
        }
      }
      for (uint64_t e = in.rp[u]; e < in.rp[u + 1]; ++e)
        if (!in_p(in.col[e])) {
          s_insert(S, u);
          break;
        }
    }
    float pre_score = 0;
    int step = 0;
    std::vector<float> scores(sample_size);
    std::vector<char> is_s_vec(sample_size), is_b_vec(sample_size);
    std::vector<uint32_t> inner_vec(sample_size);
    std::vector<std::vector<uint32_t>> tS_vec(sample_size), tB_vec(sample_size);
    std::vector<uint32_t> smp;
    while (!D.empty() && P.size() <= (size_t)max_node_num) {
      step++;
      if (step > try_max_step) break;
      int max_id = -1;
      float max_score = 0;
      bool found = false;
      uint32_t d = 0;
      int cnt = 0;
      while (cnt < try_sample_cnt) {
        sample(D, sample_size, smp);
        const int real = (int)smp.size();
        for (int i = 0; i < real; ++i) {
          bool is_s, is_b;
          uint32_t ti;
          scores[i] = check_score(D.data[smp[i]], S, B, inner_edge_num, is_s, is_b, ti, tS_vec[i],
                                  tB_vec[i]);
          is_s_vec[i] = is_s;
          is_b_vec[i] = is_b;
          inner_vec[i] = ti;
        }
        max_score = -1e10f;
        for (int i = 0; i < real; ++i)
          if (max_score < scores[i]) {
            max_score = scores[i];
            max_id = i;
          }
        if ((max_score >= 0 && max_score >= pre_score) || (P.size() < (size_t)(now_min - 1))) {
          pre_score = max_score;
          d = D.data[smp[max_id]];
          D.erase(smp[max_id]);
          found = true;
          break;
        }
        if (sample_size >= D.size()) break;
        cnt++;
      }
      if (!found) break;
      if (is_b_vec[max_id]) b_insert(B, d);
      for (uint32_t v : tB_vec[max_id]) b_erase(B, v);
      if (is_s_vec[max_id]) s_insert(S, d);
      for (uint32_t v : tS_vec[max_id]) s_erase(S, v);
      inner_edge_num = inner_vec[max_id];
      join(d, P);
      push_neighbours(d, D, try_max_node);
    }
    if (P.size() >= (size_t)now_min) {
      if (S.empty()) S.insert(source);
      const int32_t ids = (int32_t)clusters.size();
      clusters.emplace_back(P.begin(), P.end());
      for (uint32_t u : P) Fc[u] = -(ids + 1);
      for (uint32_t s : S) Fc[s] = ids;
    }
  }
};
}  // namespace

std::vector<std::vector<uint32_t>> greedy_clusters(const HostAdj& out, const HostAdj& in,
                                                   int max_node_num, int min_node_num,
                                                   uint64_t seed) {
  Greedy G(out, in, max_node_num, seed);
  std::vector<std::pair<uint32_t, uint32_t>> order(out.n);
  for (uint32_t u = 0; u < out.n; ++u) order[u] = {u, (uint32_t)out.deg(u)};
  // big to small by out-degree, ties by id (cmp_pair_b2s, compressor_base.h:2789)
  std::sort(order.begin(), order.end(), [](const auto& a, const auto& b) {
    if (a.second != b.second) return a.second > b.second;
    return a.first < b.first;
  });
  for (int i = 1; i <= 3; ++i) {
    const int b = min_node_num * i;
    for (auto& pr : order) {
      if (G.Fc[pr.first] != Summary::kFcDefault) continue;
      G.find(pr.first, b);
    }
  }
  return G.clusters;
}

// ------------------------------------------------------- supernode build
//
// compress_by_cluster (compressor_base.h:3160-3250), the benefit filter and
// mirror selection of get_init_supernode_by_clusters (:3253-3611) and
// final_build_supernode (:3616-3783).

uint64_t summary_init_by_clusters(Summary& S, const HostAdj& out, const HostAdj& in,
                                  const std::vector<std::vector<uint32_t>>& clusters_in,
                                  int min_node_num, int mirror_k, double compress_threshold) {
  const uint32_t n = out.n;
  S = Summary();
  S.old_n = n;
  S.Fc.assign(n, Summary::kFcDefault);
  S.id2spids.assign(n, Summary::kIdDefault);
  S.out_bound.assign(n, 0);
  // cluster file records: a record smaller than min_node_num is dropped, but
  // its vertices keep the cluster number assigned while reading, which the
  // next kept cluster then takes (compressor_base.h:3211-3233).
  std::vector<uint32_t> id2clusterid(n, Summary::kIdDefault);
  std::vector<std::vector<uint32_t>> clusters;
  uint32_t cluster_num = 0;
  for (const auto& rec : clusters_in) {
    std::set<uint32_t> P;
    for (uint32_t v : rec) {
      if (v >= n) continue;
      P.insert(v);
      id2clusterid[v] = cluster_num;
    }
    if (P.size() >= (size_t)min_node_num) {
      clusters.emplace_back(P.begin(), P.end());
      cluster_num++;
    }
  }
  typedef long long count_t;
  const count_t k = mirror_k;
  const float obj = (float)compress_threshold;
  const bool use_mirror = mirror_k != 100000000;
  count_t mirror_node_num = 0;
  for (uint32_t j = 0; j < clusters.size(); ++j) {
    const auto& node_set = clusters[j];
    std::unordered_map<uint32_t, uint32_t> in_freq, out_freq;
    std::set<uint32_t> old_entry, old_exit;
    count_t inner_edges = 0;
    for (uint32_t u : node_set) {
      for (uint64_t e = in.rp[u]; e < in.rp[u + 1]; ++e) {
        const uint32_t x = in.col[e];
        if (id2clusterid[x] != j) {
          if (use_mirror) {
            const uint32_t newids = S.id2spids[x];
            if (newids != Summary::kIdDefault) {
              if (S.supernode_out_mirror[newids].count(u) == 0) in_freq[x] += 1;
            } else {
              in_freq[x] += 1;
            }
          }
          old_entry.insert(u);
        } else {
          inner_edges++;
        }
      }
      for (uint64_t e = out.rp[u]; e < out.rp[u + 1]; ++e) {
        const uint32_t x = out.col[e];
        if (id2clusterid[x] != j) {
          if (use_mirror) {
            const uint32_t newids = S.id2spids[x];
            if (newids != Summary::kIdDefault) {
              if (S.supernode_in_mirror[newids].count(u) == 0) out_freq[x] += 1;
            } else {
              out_freq[x] += 1;
            }
          }
          old_exit.insert(u);
        }
      }
    }
    count_t in_edge_num = 0, out_edge_num = 0, in_mirror_num = 0, out_mirror_num = 0;
    const count_t old_exit_num = (count_t)old_exit.size(), old_entry_num = (count_t)old_entry.size();
    std::set<uint32_t> in_P(node_set.begin(), node_set.end()), out_P(node_set.begin(), node_set.end());
    std::set<uint32_t> in_mirror, out_mirror;
    if (use_mirror) {
      for (const auto& f : in_freq)
        if ((count_t)f.second > k) {
          in_edge_num += f.second;
          in_mirror_num++;
          in_P.insert(f.first);
          in_mirror.insert(f.first);
        }
      for (const auto& f : out_freq)
        if ((count_t)f.second > k) {
          out_edge_num += f.second;
          out_mirror_num++;
          out_P.insert(f.first);
          out_mirror.insert(f.first);
        }
    }
    std::set<uint32_t> B, Sset;
    for (uint32_t v : node_set)
      for (uint64_t e = out.rp[v]; e < out.rp[v + 1]; ++e)
        if (out_P.count(out.col[e]) == 0) {
          B.insert(v);
          break;
        }
    for (uint32_t v : node_set)
      for (uint64_t e = in.rp[v]; e < in.rp[v + 1]; ++e)
        if (in_P.count(in.col[e]) == 0) {
          Sset.insert(v);
          break;
        }
    const count_t new_exit = (count_t)B.size() + out_mirror_num;
    const count_t new_entry = (count_t)Sset.size() + in_mirror_num;
    const count_t idx_old = old_exit_num * old_entry_num;
    const count_t idx_entry = old_exit_num * new_entry;
    const count_t idx_exit = new_exit * old_entry_num;
    const count_t idx_new = new_exit * new_entry;
    float benefit[4];
    benefit[0] = (float)(inner_edges * 1.0 - (double)idx_old);
    benefit[1] = (float)((inner_edges + in_edge_num) * 1.0 - (double)(idx_entry + in_mirror_num));
    benefit[2] = (float)((inner_edges + out_edge_num) * 1.0 - (double)(idx_exit + out_mirror_num));
    benefit[3] = (float)((inner_edges + in_edge_num + out_edge_num) * 1.0 -
                         (double)(idx_new + in_mirror_num + out_mirror_num));
    int max_i = 0;
    for (int i = 0; i < 4; ++i)
      if (benefit[max_i] < benefit[i]) max_i = i;
    if (!(benefit[max_i] > obj)) continue;
    std::set<uint32_t> src = Sset;
    if (max_i == 0) {
      src = old_entry;
      in_mirror.clear();
      out_mirror.clear();
    } else if (max_i == 1) {
      out_mirror.clear();
    } else if (max_i == 2) {
      src = old_entry;
      in_mirror.clear();
    }
    const uint32_t ids = (uint32_t)S.supernode_ids.size();
    S.supernode_ids.emplace_back(node_set.begin(), node_set.end());
    S.cluster_ids.emplace_back(node_set.begin(), node_set.end());
    S.supernode_source.emplace_back(src.begin(), src.end());
    S.supernode_in_mirror.emplace_back(in_mirror.begin(), in_mirror.end());
    S.supernode_out_mirror.emplace_back(out_mirror.begin(), out_mirror.end());
    mirror_node_num += (count_t)(in_mirror.size() + out_mirror.size());
    for (uint32_t u : node_set) {
      S.Fc[u] = -(int32_t)(ids + 1);
      S.id2spids[u] = ids;
    }
  }

  return (uint64_t)mirror_node_num;
}

// final_build_supernode (compressor_base.h:3616-3783) from the state above
// (or the same state read back from a serialized summary).
void summary_final_build(Summary& S, const HostAdj& in, uint64_t init_mirror_num) {
  const uint32_t n = S.old_n;
  S.all_n = n;
  const uint64_t cap_all = (uint64_t)n + init_mirror_num;
  S.Fc_map.assign(cap_all, Summary::kIdDefault);
  S.vid2in_mirror_mids.assign(n, {});
  const uint32_t n_clusters = (uint32_t)S.supernode_ids.size();
  std::vector<uint32_t> mirror_cluster;  // cluster of each mirror id (index m - n)
  for (uint32_t i = 0; i < n_clusters; ++i) {
    auto& old_P = S.supernode_ids[i];
    auto& src = S.supernode_source[i];
    auto& in_mirror = S.supernode_in_mirror[i];
    auto& out_mirror = S.supernode_out_mirror[i];
    std::vector<uint32_t> del_v;
    // an unclustered vertex chosen as a mirror joins the cluster instead
    for (uint32_t v : in_mirror) {
      if (S.Fc[v] != Summary::kFcDefault) continue;
      S.mirror_node_cnt++;
      old_P.push_back(v);
      S.cluster_ids[i].push_back(v);
      del_v.push_back(v);
      for (uint64_t e = in.rp[v]; e < in.rp[v + 1]; ++e) {
        const uint32_t x = in.col[e];
        if (S.id2spids[x] != i && in_mirror.count(x) == 0) {
          src.push_back(v);
          S.inmirror2source_cnt++;
          break;
        }
      }
      S.Fc[v] = -(int32_t)(i + 1);
      S.id2spids[v] = i;
    }
    for (uint32_t v : del_v) {
      in_mirror.erase(v);
      out_mirror.erase(v);
    }
    del_v.clear();
    for (uint32_t v : out_mirror) {
      if (S.Fc[v] != Summary::kFcDefault) continue;
      S.mirror_node_cnt++;
      old_P.push_back(v);
      S.cluster_ids[i].push_back(v);
      del_v.push_back(v);
      for (uint64_t e = in.rp[v]; e < in.rp[v + 1]; ++e) {
        const uint32_t x = in.col[e];
        if (S.id2spids[x] != i && in_mirror.count(x) == 0) {
          src.push_back(v);
          S.outmirror2source_cnt++;
          break;
        }
      }
      S.Fc[v] = -(int32_t)(i + 1);
      S.id2spids[v] = i;
    }
    for (uint32_t v : del_v) {
      out_mirror.erase(v);
      in_mirror.erase(v);
    }
    S.cluster_in_mirror_ids.emplace_back();
    S.cluster_out_mirror_ids.emplace_back();
    for (uint32_t v : in_mirror) {
      const uint32_t m = S.all_n++;
      S.mirrorid2vid.push_back(v);
      mirror_cluster.push_back(i);
      S.cluster_ids[i].push_back(m);
      S.cluster_in_mirror_ids[i].push_back(m);
    }
    for (uint32_t v : out_mirror) {
      const uint32_t m = S.all_n++;
      S.mirrorid2vid.push_back(v);
      mirror_cluster.push_back(i);
      S.cluster_ids[i].push_back(m);
      S.cluster_out_mirror_ids[i].push_back(m);
    }
    for (uint32_t s : src) {
      S.Fc[s] = (int32_t)i;
      const uint32_t spid = (uint32_t)S.supernodes.size();
      S.Fc_map[s] = spid;
      Supernode sp;
      sp.id = s;
      sp.ids = i;
      S.supernodes.push_back(sp);
    }
    for (uint32_t m : S.cluster_in_mirror_ids[i]) {
      const uint32_t spid = (uint32_t)S.supernodes.size();
      S.vid2in_mirror_mids[S.mirror_master(m)].push_back(m);
      S.Fc_map[m] = spid;
      Supernode sp;
      sp.id = m;
      sp.ids = i;
      S.supernodes.push_back(sp);
    }
  }
  S.Fc_map.resize(S.all_n);
  S.id2spids.resize(S.all_n, Summary::kIdDefault);
  for (uint32_t m = n; m < S.all_n; ++m) S.id2spids[m] = mirror_cluster[m - n];
  S.all_out_mirror.clear();
  for (uint32_t j = 0; j < n_clusters; ++j)
    for (uint32_t m : S.cluster_out_mirror_ids[j]) S.all_out_mirror.push_back(m);
}

// judge_out_bound_node (compressor_base.h:3924-3956, detail :3993-4007).
// Exit marks are only ever set; `only` restricts the pass to some clusters.
void summary_judge_out_bound(Summary& S, const HostAdj& out, const std::vector<uint32_t>* only) {
  const uint32_t nc = (uint32_t)S.supernode_ids.size();
  auto judge = [&](uint32_t j) {
    const auto& om = S.supernode_out_mirror[j];
    for (uint32_t v : S.supernode_ids[j])
      for (uint64_t e = out.rp[v]; e < out.rp[v + 1]; ++e) {
        const uint32_t x = out.col[e];
        if (S.id2spids[x] != j && om.count(x) == 0) {
          S.out_bound[v] = 1;
          break;
        }
      }
  };
  // a cluster's judgement writes only its own members (parallel); the
  // in-mirror masters live in other clusters (serial)
  if (only) {
    const std::vector<uint32_t>& L = *only;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long k = 0; k < (long long)L.size(); ++k) judge(L[k]);
    for (uint32_t j : L)
      for (uint32_t v : S.supernode_in_mirror[j]) S.out_bound[v] = 1;
  } else {
#pragma omp parallel for schedule(dynamic, 256)
    for (long long j = 0; j < (long long)nc; ++j) judge((uint32_t)j);
    for (uint32_t j = 0; j < nc; ++j)
      for (uint32_t v : S.supernode_in_mirror[j]) S.out_bound[v] = 1;
  }
}

// build_subgraph_mirror (compressor_base.h:3786-3856) and its incremental
// form (:3859-3922): inner edges of each cluster, the in-mirror's edges into
// its cluster and member edges redirected to out-mirrors.
void summary_build_subgraph(Summary& S, const HostAdj& out, const HostAdj& in,
                            const std::vector<uint32_t>* only) {
  const bool weighted = !out.w.empty();
  if (S.subgraph.size() != S.all_n) {
    S.subgraph.assign(S.all_n, {});
    if (weighted) S.subgraph_w.assign(S.all_n, {});
  }
  auto build = [&](uint32_t i) {
    for (uint32_t v : S.supernode_ids[i]) {
      S.subgraph[v].clear();
      if (weighted) S.subgraph_w[v].clear();
      for (uint64_t e = out.rp[v]; e < out.rp[v + 1]; ++e)
        if (S.id2spids[out.col[e]] == i) {
          S.subgraph[v].push_back(out.col[e]);
          if (weighted) S.subgraph_w[v].push_back(out.w[e]);
        }
    }
    for (uint32_t m : S.cluster_in_mirror_ids[i]) {
      S.subgraph[m].clear();
      if (weighted) S.subgraph_w[m].clear();
      const uint32_t v = S.mirror_master(m);
      for (uint64_t e = out.rp[v]; e < out.rp[v + 1]; ++e)
        if (S.id2spids[out.col[e]] == i) {
          S.subgraph[m].push_back(out.col[e]);
          if (weighted) S.subgraph_w[m].push_back(out.w[e]);
        }
    }
    for (uint32_t m : S.cluster_out_mirror_ids[i]) {
      const uint32_t v = S.mirror_master(m);
      const auto& v_in_mirror = S.supernode_in_mirror[S.id2spids[v]];
      for (uint64_t e = in.rp[v]; e < in.rp[v + 1]; ++e) {
        const uint32_t x = in.col[e];
        if (S.id2spids[x] == i && v_in_mirror.count(x) == 0) {
          S.subgraph[x].push_back(m);
          if (weighted) S.subgraph_w[x].push_back(in.w[e]);
        }
      }
    }
  };
  // a cluster writes the rows of its own members and mirrors only; the
  // lists hold each cluster once
  if (only) {
    const std::vector<uint32_t>& L = *only;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long k = 0; k < (long long)L.size(); ++k) build(L[k]);
  } else {
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)S.supernode_ids.size(); ++i) build((uint32_t)i);
  }
}

// get_nodetype_mirror (compressor_base.h:4144-4182).
void summary_node_types(Summary& S) {
  const uint32_t n = S.old_n;
  S.node_type.assign(n, 127);
  for (uint32_t i = 0; i < n; ++i) {
    const int32_t fc = S.Fc[i];
    if (fc == Summary::kFcDefault) S.node_type[i] = kSingle;
    else if (fc >= 0) S.node_type[i] = kOnlyIn;
    else if (!S.out_bound[i]) S.node_type[i] = kInner;
    if (S.out_bound[i]) {
      S.node_type[i] = kOnlyOut;
      if (fc >= 0) S.node_type[i] = kBothOutIn;
    }
  }
  for (size_t j = 0; j < S.supernode_in_mirror.size(); ++j)
    for (uint32_t v : S.supernode_in_mirror[j]) {
      if (S.node_type[v] == kOnlyOut) S.node_type[v] = kOutMaster;
      else if (S.node_type[v] == kBothOutIn) S.node_type[v] = kBothOutInMaster;
    }
}

// sketch2csr_mirror (compressor_base.h:4636-4880): is_e (entry / in-mirror ->
// exit shortcuts, from bound_delta), ib_e (exit -> outside edges, and every
// edge of unclustered vertices) and sync_e (master -> in-mirror,
// out-mirror -> master).
void summary_sketch_csr(Summary& S, const HostAdj& out) {
  const uint32_t all = S.all_n, n = S.old_n;
  const bool weighted = !out.w.empty();
  // sync edges: master -> its in-mirrors, out-mirror -> its master, in the
  // order of the clusters and their mirror lists (counting sort)
  S.sync_off.assign(all + 1, 0);
  for (size_t i = 0; i < S.cluster_in_mirror_ids.size(); ++i) {
    for (uint32_t m : S.cluster_in_mirror_ids[i]) S.sync_off[S.mirror_master(m) + 1]++;
    for (uint32_t m : S.cluster_out_mirror_ids[i]) S.sync_off[m + 1]++;
  }
  for (uint32_t i = 0; i < all; ++i) S.sync_off[i + 1] += S.sync_off[i];
  S.sync_nbr.assign(S.sync_off[all], 0);
  {
    std::vector<uint64_t> pos(S.sync_off.begin(), S.sync_off.end() - 1);
    for (size_t i = 0; i < S.cluster_in_mirror_ids.size(); ++i) {
      for (uint32_t m : S.cluster_in_mirror_ids[i]) S.sync_nbr[pos[S.mirror_master(m)]++] = m;
      for (uint32_t m : S.cluster_out_mirror_ids[i]) S.sync_nbr[pos[m]++] = S.mirror_master(m);
    }
  }
  // shortcut and boundary edges
  auto is_row = [&](uint32_t i) -> const Supernode* {
    if (i >= n) {
      const uint32_t sp = S.Fc_map[i];
      return sp != Summary::kIdDefault ? &S.supernodes[sp] : nullptr;
    }
    const char t = S.node_type[i];
    if (t == kOnlyIn || t == kBothOutIn || t == kBothOutInMaster) return &S.supernodes[S.Fc_map[i]];
    return nullptr;
  };
  auto ib_take = [&](uint32_t u, uint32_t x) {
    const uint32_t ids = S.id2spids[u];
    const uint32_t out_ids = S.id2spids[x];
    const auto& om = S.supernode_out_mirror[ids];
    if (out_ids != Summary::kIdDefault) {
      const auto& im = S.supernode_in_mirror[out_ids];
      return ids != out_ids && om.count(x) == 0 && im.count(u) == 0;
    }
    return ids != out_ids && om.count(x) == 0;
  };
  // 0: no boundary row, 1: filtered out-edges, 2: all out-edges
  auto ib_mode = [&](uint32_t i) -> int {
    if (i >= n) return 0;
    const char t = S.node_type[i];
    if (t == kOnlyOut || t == kBothOutIn || t == kBothOutInMaster || t == kOutMaster) return 1;
    return t == kSingle ? 2 : 0;
  };
  // two passes over the rows (counts, then fills at prefix offsets)
  S.is_off.assign(all + 1, 0);
  S.ib_off.assign(all + 1, 0);
#pragma omp parallel for schedule(dynamic, 4096)
  for (long long ii = 0; ii < (long long)all; ++ii) {
    const uint32_t i = (uint32_t)ii;
    if (const Supernode* sp = is_row(i)) S.is_off[i + 1] = sp->bound_delta.size();
    const int mode = ib_mode(i);
    uint64_t c = 0;
    if (mode == 2) {
      c = out.deg(i);
    } else if (mode == 1) {
      for (uint64_t e = out.rp[i]; e < out.rp[i + 1]; ++e) c += ib_take(i, out.col[e]);
    }
    S.ib_off[i + 1] = c;
  }
  for (uint32_t i = 0; i < all; ++i) {
    S.is_off[i + 1] += S.is_off[i];
    S.ib_off[i + 1] += S.ib_off[i];
  }
  S.is_nbr.assign(S.is_off[all], 0);
  S.is_w.assign(S.is_off[all], 0.f);
  S.ib_nbr.assign(S.ib_off[all], 0);
  S.ib_w.assign(weighted ? S.ib_off[all] : 0, 0.f);
#pragma omp parallel for schedule(dynamic, 4096)
  for (long long ii = 0; ii < (long long)all; ++ii) {
    const uint32_t i = (uint32_t)ii;
    if (const Supernode* sp = is_row(i)) {
      std::vector<std::pair<uint32_t, double>> row = sp->bound_delta;
      std::stable_sort(row.begin(), row.end(),
                       [](const auto& a, const auto& b) { return a.first < b.first; });
      uint64_t k = S.is_off[i];
      for (auto& e : row) {
        S.is_nbr[k] = e.first;
        S.is_w[k++] = (float)e.second;
      }
    }
    const int mode = ib_mode(i);
    uint64_t k = S.ib_off[i];
    for (uint64_t e = mode ? out.rp[i] : 0; mode && e < out.rp[i + 1]; ++e)
      if (mode == 2 || ib_take(i, out.col[e])) {
        S.ib_nbr[k] = out.col[e];
        if (weighted) S.ib_w[k] = out.w[e];
        ++k;
      }
  }
}

// inc_compress_mirror (compressor_base.h:5634-5803): cluster membership and
// mirrors stay; a deleted edge can retire an entry that has no other outside
// in-neighbour, an added edge from outside creates an entry; the clusters
// and supernodes touched by the batch are recorded for shortcut repair.
void summary_inc_entries(Summary& S, const HostAdj& new_out, const HostAdj& new_in,
                         const std::vector<std::pair<uint32_t, uint32_t>>& deleted,
                         const std::vector<std::pair<uint32_t, uint32_t>>& added) {
  (void)new_out;
  // touched clusters and supernode sources: marks plus the list of marked
  // ids (sorted at the end, so the order of marking does not matter)
  std::vector<uint8_t> mark_c(S.supernode_ids.size(), 0), mark_s(S.all_n, 0);
  std::vector<uint32_t> list_c, list_s;
  struct {
    std::vector<uint8_t>& mark;
    std::vector<uint32_t>& list;
    void insert(uint32_t x) {
      if (x < mark.size() && !mark[x]) {
        mark[x] = 1;
        list.push_back(x);
      }
    }
  } upd_c{mark_c, list_c}, upd_s{mark_s, list_s};
  std::vector<uint32_t> delete_spid;
  auto touch_source = [&](uint32_t u) {
    const uint32_t src_id = S.id2spids[u];
    upd_c.insert(src_id);
    for (uint32_t s : S.supernode_source[src_id]) upd_s.insert(s);
    for (uint32_t m : S.cluster_in_mirror_ids[src_id]) upd_s.insert(m);
    for (uint32_t m : S.vid2in_mirror_mids[u]) {
      upd_s.insert(m);
      upd_c.insert(S.id2spids[m]);
    }
  };
  for (const auto& pr : deleted) {
    const uint32_t u = pr.first, v = pr.second;
    if (S.Fc[u] != Summary::kFcDefault) touch_source(u);
    if (S.Fc[v] != Summary::kFcDefault && S.Fc[v] >= 0) {
      const uint32_t ids = S.id2spids[v];
      upd_c.insert(ids);
      if (ids != S.id2spids[u]) {
        const auto& im = S.supernode_in_mirror[ids];
        bool outside = false;
        for (uint64_t e = new_in.rp[v]; e < new_in.rp[v + 1]; ++e) {
          const uint32_t x = new_in.col[e];
          if (x != u && ids != S.id2spids[x] && im.count(x) == 0) {
            outside = true;
            break;
          }
        }
        if (!outside) {
          auto& srcs = S.supernode_source[ids];
          auto it = std::find(srcs.begin(), srcs.end(), v);
          if (it != srcs.end()) srcs.erase(it);
          const uint32_t sp = S.Fc_map[v];
          S.supernodes[sp].clear();
          delete_spid.push_back(sp);
          S.Fc[v] = -(int32_t)(ids + 1);
          S.Fc_map[v] = Summary::kIdDefault;
        }
      }
    }
  }
  int del_index = (int)delete_spid.size() - 1;
  for (const auto& pr : added) {
    const uint32_t u = pr.first, v = pr.second;
    if (S.Fc[u] != Summary::kFcDefault) touch_source(u);
    if (S.Fc[v] != Summary::kFcDefault) {
      const uint32_t ids = S.id2spids[v];
      upd_c.insert(ids);
      const auto& im = S.supernode_in_mirror[ids];
      if (S.Fc[v] < 0 && ids != S.id2spids[u] && im.count(u) == 0) {
        S.Fc[v] = (int32_t)ids;
        S.supernode_source[ids].push_back(v);
        uint32_t spid;
        if (del_index >= 0) {
          spid = delete_spid[del_index--];
        } else {
          spid = (uint32_t)S.supernodes.size();
          S.supernodes.emplace_back();
        }
        S.Fc_map[v] = spid;
        S.supernodes[spid].id = v;
        S.supernodes[spid].ids = ids;
        S.supernodes[spid].status = false;
        upd_s.insert(v);
      }
    }
  }
  // retired supernode ids that were not reused stay empty (id = kIdDefault)
  for (int i = 0; i <= del_index; ++i) {
    S.supernodes[delete_spid[i]].clear();
    S.supernodes[delete_spid[i]].id = Summary::kIdDefault;
  }
  S.update_cluster_ids = list_c;
  std::sort(S.update_cluster_ids.begin(), S.update_cluster_ids.end());
  S.update_source_id = list_s;
  std::sort(S.update_source_id.begin(), S.update_source_id.end());
}

void summary_from_clusters(Summary& S, const HostAdj& out, const HostAdj& in,
                           const std::vector<std::vector<uint32_t>>& clusters, int min_node_num,
                           int mirror_k, double compress_threshold) {
  const uint64_t m = summary_init_by_clusters(S, out, in, clusters, min_node_num, mirror_k,
                                              compress_threshold);
  summary_final_build(S, in, m);
}

// serialize_cluster / de_serialize_cluster (compressor_base.h:2987-3158):
// the state between get_init_supernode_by_clusters and final_build_supernode,
// native-endian: u32 init_mirror_num, u32 clusters; per cluster the member,
// cluster, source, in-mirror and out-mirror lists as (u32 count, u32 ids...);
// then Fc (i32) and id2spids (u32) of every vertex; then i32 -1.
static void put_u32(std::vector<uint8_t>& b, uint32_t x) {
  const uint8_t* p = reinterpret_cast<const uint8_t*>(&x);
  b.insert(b.end(), p, p + 4);
}

template <typename C>
static void put_list(std::vector<uint8_t>& b, const C& c) {
  put_u32(b, (uint32_t)c.size());
  for (uint32_t v : c) put_u32(b, v);
}

std::vector<uint8_t> summary_serialize_init(const Summary& S, uint64_t init_mirror_num) {
  std::vector<uint8_t> b;
  put_u32(b, (uint32_t)init_mirror_num);
  const uint32_t nc = (uint32_t)S.supernode_ids.size();
  put_u32(b, nc);
  for (uint32_t i = 0; i < nc; ++i) {
    put_list(b, S.supernode_ids[i]);
    put_list(b, S.cluster_ids[i]);
    put_list(b, S.supernode_source[i]);
    put_list(b, S.supernode_in_mirror[i]);
    put_list(b, S.supernode_out_mirror[i]);
  }
  for (uint32_t v = 0; v < S.old_n; ++v) put_u32(b, (uint32_t)S.Fc[v]);
  for (uint32_t v = 0; v < S.old_n; ++v) put_u32(b, S.id2spids[v]);
  put_u32(b, 0xFFFFFFFFu);
  return b;
}

bool summary_deserialize_init(Summary& S, uint32_t n, const std::vector<uint8_t>& b,
                              uint64_t* init_mirror_num) {
  size_t p = 0;
  auto get = [&](uint32_t* x) {
    if (p + 4 > b.size()) return false;
    std::memcpy(x, b.data() + p, 4);
    p += 4;
    return true;
  };
  auto get_list = [&](std::vector<uint32_t>& out) {
    uint32_t c = 0;
    if (!get(&c) || (uint64_t)c * 4 > b.size() - p) return false;
    out.resize(c);
    for (uint32_t i = 0; i < c; ++i) {
      get(&out[i]);
      if (out[i] >= n) return false;
    }
    return true;
  };
  S = Summary();
  S.old_n = n;
  uint32_t im = 0, nc = 0;
  if (!get(&im) || !get(&nc)) return false;
  S.supernode_ids.resize(nc);
  S.cluster_ids.resize(nc);
  S.supernode_source.resize(nc);
  S.supernode_in_mirror.resize(nc);
  S.supernode_out_mirror.resize(nc);
  std::vector<uint32_t> tmp;
  for (uint32_t i = 0; i < nc; ++i) {
    if (!get_list(S.supernode_ids[i]) || !get_list(S.cluster_ids[i]) ||
        !get_list(S.supernode_source[i]))
      return false;
    if (!get_list(tmp)) return false;
    S.supernode_in_mirror[i].insert(tmp.begin(), tmp.end());
    if (!get_list(tmp)) return false;
    S.supernode_out_mirror[i].insert(tmp.begin(), tmp.end());
  }
  S.Fc.resize(n);
  S.id2spids.resize(n);
  for (uint32_t v = 0; v < n; ++v) {
    uint32_t x;
    if (!get(&x)) return false;
    S.Fc[v] = (int32_t)x;
  }
  for (uint32_t v = 0; v < n; ++v)
    if (!get(&S.id2spids[v])) return false;
  uint32_t eof = 0;
  if (!get(&eof) || eof != 0xFFFFFFFFu || p != b.size()) return false;
  S.out_bound.assign(n, 0);
  *init_mirror_num = im;
  return true;
}

}  // namespace sg
