// Host utilities behind the C ABI that need no GPU: the host twin of the
// device R-MAT generator and a host adjacency mirror that draws update
// batches valid for the current graph.  Used to give the library, the oracle
// and the reference harness identical inputs.
#include <algorithm>
#include <cstring>
#include <new>
#include <unordered_set>
#include <utility>
#include <vector>

#include "../../include/suminc_gb300.h"
#include "common.h"

using namespace sg;

namespace {

struct PairHash {
  size_t operator()(uint64_t k) const noexcept { return (size_t)mix64(k); }
};

}  // namespace

struct sg_hostgraph {
  uint32_t n = 0;
  uint64_t m = 0;
  bool weighted = false;
  std::vector<std::vector<uint32_t>> adj;  // sorted per row
  std::vector<std::vector<float>> wt;      // parallel weights (weighted only)
  uint64_t draws = 0;                      // RNG counter across batches
};

extern "C" {

sg_status sg_util_rmat_host(int scale, uint64_t edges, double a, double b, double c,
                            uint64_t seed, int weight_kind, double wlo, double whi,
                            uint64_t* row_ptr, uint32_t* col, float* w) {
  if (scale < 1 || scale > 30 || !row_ptr || !col) return SG_ERR_INVALID;
  const uint64_t n = 1ull << scale;
  if (edges > n * (n - 1) || edges >= (1ull << 31)) return SG_ERR_INVALID;
  try {
    const RmatParams p = make_rmat_params(scale, a, b, c, seed);
    const uint64_t sentinel = (1ull << (2 * scale)) - 1;
    uint64_t M = edges + edges / 3 + 1024;
    std::vector<uint64_t> keys;
    for (int attempt = 0; attempt < 12; ++attempt) {
      std::vector<std::pair<uint64_t, uint32_t>> d(M);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)M; ++i) {
        const uint64_t e = rmat_draw(p, (uint64_t)i);
        const uint32_t s = (uint32_t)(e >> 32), t = (uint32_t)e;
        d[i] = {(s == t) ? sentinel : (((uint64_t)s << scale) | t), (uint32_t)i};
      }
      std::sort(d.begin(), d.end());
      std::vector<std::pair<uint32_t, uint64_t>> first;  // (first index, key)
      first.reserve(M);
      for (uint64_t i = 0; i < M; ++i) {
        if (d[i].first == sentinel) continue;
        if (i > 0 && d[i].first == d[i - 1].first) continue;
        first.push_back({d[i].second, d[i].first});
      }
      if (first.size() < edges) {
        const double ratio = (double)edges / (double)std::max<size_t>(first.size(), 1);
        M = (uint64_t)((double)M * ratio * 1.08) + 4096;
        continue;
      }
      std::sort(first.begin(), first.end());
      keys.resize(edges);
      for (uint64_t i = 0; i < edges; ++i) keys[i] = first[i].second;
      std::sort(keys.begin(), keys.end());
      break;
    }
    if (keys.size() != edges) return SG_ERR_INVALID;
    const WeightParams wp = make_weight_params(seed, weight_kind, wlo, whi);
    const uint64_t mask = (1ull << scale) - 1;
    std::fill(row_ptr, row_ptr + n + 1, 0);
    for (uint64_t i = 0; i < edges; ++i) {
      const uint64_t s = keys[i] >> scale, t = keys[i] & mask;
      row_ptr[s + 1]++;
      col[i] = (uint32_t)t;
      if (w && weight_kind != 0) w[i] = edge_weight(wp, (s << 32) | t);
    }
    for (uint64_t v = 0; v < n; ++v) row_ptr[v + 1] += row_ptr[v];
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return SG_ERR_OOM;
  }
}

sg_status sg_hostgraph_create(uint32_t n, const uint64_t* row_ptr, const uint32_t* col,
                              const float* w, sg_hostgraph** out) {
  if (!out || !row_ptr || n == 0) return SG_ERR_INVALID;
  *out = nullptr;
  try {
    sg_hostgraph* g = new sg_hostgraph();
    g->n = n;
    g->weighted = (w != nullptr);
    g->adj.resize(n);
    if (g->weighted) g->wt.resize(n);
    for (uint32_t v = 0; v < n; ++v) {
      const uint64_t b = row_ptr[v], e = row_ptr[v + 1];
      std::vector<std::pair<uint32_t, float>> row;
      row.reserve(e - b);
      for (uint64_t k = b; k < e; ++k) {
        if (col[k] >= n) {
          delete g;
          return SG_ERR_INVALID;
        }
        row.push_back({col[k], w ? w[k] : 0.f});
      }
      std::sort(row.begin(), row.end());
      g->adj[v].reserve(row.size());
      if (g->weighted) g->wt[v].reserve(row.size());
      for (auto& pr : row) {
        g->adj[v].push_back(pr.first);
        if (g->weighted) g->wt[v].push_back(pr.second);
      }
      g->m += row.size();
    }
    *out = g;
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return SG_ERR_OOM;
  }
}

sg_status sg_hostgraph_destroy(sg_hostgraph* g) {
  if (!g) return SG_ERR_INVALID;
  delete g;
  return SG_OK;
}

sg_status sg_hostgraph_num_edges(const sg_hostgraph* g, uint64_t* m) {
  if (!g || !m) return SG_ERR_INVALID;
  *m = g->m;
  return SG_OK;
}

sg_status sg_hostgraph_csr(const sg_hostgraph* g, uint64_t* row_ptr, uint32_t* col, float* w) {
  if (!g || !row_ptr || !col) return SG_ERR_INVALID;
  row_ptr[0] = 0;
  for (uint32_t v = 0; v < g->n; ++v) {
    const uint64_t b = row_ptr[v];
    const auto& r = g->adj[v];
    std::memcpy(col + b, r.data(), r.size() * sizeof(uint32_t));
    if (w) {
      if (g->weighted) std::memcpy(w + b, g->wt[v].data(), r.size() * sizeof(float));
      else std::fill(w + b, w + b + r.size(), 1.0f);
    }
    row_ptr[v + 1] = b + r.size();
  }
  return SG_OK;
}

sg_status sg_hostgraph_gen_updates(sg_hostgraph* g, uint64_t n_ins, uint64_t n_del,
                                   uint64_t n_rew, uint64_t seed, int integer_weights,
                                   double wlo, double whi, sg_update* out) {
  if (!g || (!out && (n_ins + n_del + n_rew) > 0)) return SG_ERR_INVALID;
  if (n_del + n_rew > g->m) return SG_ERR_INVALID;
  const uint64_t n = g->n;
  if (n_ins > n * (n - 1) - g->m) return SG_ERR_INVALID;
  try {
    const uint64_t key0 = mix64(seed ^ 0xA0761D6478BD642Full);
    uint64_t ctr = 0;
    auto rnd = [&]() { return mix64(key0 + (ctr++)); };
    auto new_weight = [&]() -> float {
      const uint64_t h = rnd();
      if (integer_weights) {
        const uint64_t span = (uint64_t)(whi - wlo + 1.0);
        return (float)(wlo + (double)(h % span));
      }
      volatile double prod = (whi - wlo) * ((double)(h >> 40) * (1.0 / 16777216.0));
      return (float)(wlo + prod);
    };
    auto has_edge = [&](uint32_t u, uint32_t v) {
      const auto& r = g->adj[u];
      return std::binary_search(r.begin(), r.end(), v);
    };
    // prefix of row sizes for uniform edge picks
    std::vector<uint64_t> pre(n + 1, 0);
    for (uint64_t v = 0; v < n; ++v) pre[v + 1] = pre[v] + g->adj[v].size();
    auto pick_edge = [&]() -> std::pair<uint32_t, uint32_t> {
      const uint64_t r = rnd() % g->m;
      const uint64_t v = (uint64_t)(std::upper_bound(pre.begin(), pre.end(), r) - pre.begin()) - 1;
      return {(uint32_t)v, g->adj[v][r - pre[v]]};
    };
    std::unordered_set<uint64_t, PairHash> chosen;
    chosen.reserve((n_ins + n_del + n_rew) * 2 + 16);
    std::vector<std::pair<uint32_t, uint32_t>> dels, rews, inss;
    std::vector<float> rew_w, ins_w;
    while (dels.size() < n_del) {
      auto e = pick_edge();
      const uint64_t k = ((uint64_t)e.first << 32) | e.second;
      if (chosen.insert(k).second) dels.push_back(e);
    }
    while (rews.size() < n_rew) {
      auto e = pick_edge();
      const uint64_t k = ((uint64_t)e.first << 32) | e.second;
      if (chosen.insert(k).second) {
        rews.push_back(e);
        rew_w.push_back(new_weight());
      }
    }
    while (inss.size() < n_ins) {
      const uint32_t u = (uint32_t)(rnd() % n), v = (uint32_t)(rnd() % n);
      if (u == v || has_edge(u, v)) continue;
      const uint64_t k = ((uint64_t)u << 32) | v;
      if (chosen.insert(k).second) {
        inss.push_back({u, v});
        ins_w.push_back(new_weight());
      }
    }
    // emit: deletes, re-weights (delete + add), inserts
    uint64_t o = 0;
    for (auto& e : dels) out[o++] = sg_update{e.first, e.second, 0.f, SG_UPD_DEL};
    for (size_t i = 0; i < rews.size(); ++i) {
      out[o++] = sg_update{rews[i].first, rews[i].second, 0.f, SG_UPD_DEL};
      out[o++] = sg_update{rews[i].first, rews[i].second, rew_w[i], SG_UPD_ADD};
    }
    for (size_t i = 0; i < inss.size(); ++i)
      out[o++] = sg_update{inss[i].first, inss[i].second, ins_w[i], SG_UPD_ADD};
    // apply to the mirror
    auto erase_edge = [&](uint32_t u, uint32_t v) {
      auto& r = g->adj[u];
      auto it = std::lower_bound(r.begin(), r.end(), v);
      const size_t pos = it - r.begin();
      r.erase(it);
      if (g->weighted) g->wt[u].erase(g->wt[u].begin() + pos);
      g->m--;
    };
    for (auto& e : dels) erase_edge(e.first, e.second);
    for (size_t i = 0; i < rews.size(); ++i) {
      if (!g->weighted) continue;
      auto& r = g->adj[rews[i].first];
      const size_t pos = std::lower_bound(r.begin(), r.end(), rews[i].second) - r.begin();
      g->wt[rews[i].first][pos] = rew_w[i];
    }
    for (size_t i = 0; i < inss.size(); ++i) {
      const uint32_t u = inss[i].first, v = inss[i].second;
      auto& r = g->adj[u];
      auto it = std::lower_bound(r.begin(), r.end(), v);
      const size_t pos = it - r.begin();
      r.insert(it, v);
      if (g->weighted) g->wt[u].insert(g->wt[u].begin() + pos, ins_w[i]);
      g->m++;
    }
    g->draws += ctr;
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return SG_ERR_OOM;
  }
}

}  // extern "C"

// ------------------------------------------------------ greedy clustering
#include "summary.h"

namespace sg {
// in-adjacency with rows sorted by source id
void host_transpose(const HostAdj& out, HostAdj& in) {
  in.n = out.n;
  in.rp.assign((size_t)out.n + 1, 0);
  for (uint64_t e = 0; e < out.rp[out.n]; ++e) in.rp[out.col[e] + 1]++;
  for (uint32_t v = 0; v < out.n; ++v) in.rp[v + 1] += in.rp[v];
  in.col.resize(out.rp[out.n]);
  if (!out.w.empty()) in.w.resize(out.rp[out.n]);
  std::vector<uint64_t> pos(in.rp.begin(), in.rp.end() - 1);
  for (uint32_t u = 0; u < out.n; ++u)
    for (uint64_t e = out.rp[u]; e < out.rp[u + 1]; ++e) {
      const uint64_t p = pos[out.col[e]]++;
      in.col[p] = u;
      if (!out.w.empty()) in.w[p] = out.w[e];
    }
}

bool host_adj_patch(HostAdj& a, const std::vector<AdjOp>& ops) {
  const uint32_t n = a.n;
  const bool weighted = !a.w.empty();
  for (const AdjOp& op : ops)
    if (op.row >= n || op.col >= n) return false;
  // new row pointers: old offsets shifted by the net insertions so far
  std::vector<uint64_t>& rp = a.rp_spare;
  rp.resize(n + 1);
  rp[0] = 0;
  {
    int64_t shift = 0;
    size_t k = 0;
    for (uint32_t v = 0; v < n; ++v) {
      for (; k < ops.size() && ops[k].row == v; ++k)
        shift += ops[k].kind == AdjOp::kInsert ? 1 : (ops[k].kind == AdjOp::kRemove ? -1 : 0);
      rp[v + 1] = (uint64_t)((int64_t)a.rp[v + 1] + shift);
    }
  }
  std::vector<uint32_t>& col = a.col_spare;
  std::vector<float>& w = a.w_spare;
  col.resize(rp[n]);
  w.resize(weighted ? rp[n] : 0);
  // rows r0..r1-1 unchanged: one bulk move
  auto move_rows = [&](uint32_t r0, uint32_t r1) {
    if (r1 <= r0) return;
    const uint64_t b = a.rp[r0], e = a.rp[r1];
    std::copy(a.col.begin() + b, a.col.begin() + e, col.begin() + rp[r0]);
    if (weighted) std::copy(a.w.begin() + b, a.w.begin() + e, w.begin() + rp[r0]);
  };
  // row r merged with ops[k, ke) (every write checked against the row's new
  // extent, so an op that does not fit cannot write past it)
  auto merge_row = [&](uint32_t r, size_t k, size_t ke) {
    uint64_t i = a.rp[r], o = rp[r];
    const uint64_t ie = a.rp[r + 1], oe = rp[r + 1];
    auto emit = [&](uint32_t c, float wv) {
      if (o >= oe) return false;
      col[o] = c;
      if (weighted) w[o] = wv;
      ++o;
      return true;
    };
    for (size_t j = k; j < ke; ++j) {
      const AdjOp& op = ops[j];
      for (; i < ie && a.col[i] < op.col; ++i)
        if (!emit(a.col[i], weighted ? a.w[i] : 0.f)) return false;
      const bool here = i < ie && a.col[i] == op.col;
      if (op.kind == AdjOp::kRemove) {
        if (!here) return false;
        ++i;
      } else if (op.kind == AdjOp::kSetWeight) {
        if (!here || !emit(op.col, op.w)) return false;
        ++i;
      } else {
        if (here || !emit(op.col, op.w)) return false;
      }
    }
    for (; i < ie; ++i)
      if (!emit(a.col[i], weighted ? a.w[i] : 0.f)) return false;
    return o == oe;
  };
  // row ranges in parallel, each with its slice of the ops
  const int64_t chunks = std::max<int64_t>(1, std::min<int64_t>(256, n / 4096));
  bool ok = true;
#pragma omp parallel for schedule(dynamic, 1) reduction(&& : ok)
  for (int64_t ch = 0; ch < chunks; ++ch) {
    const uint32_t r0 = (uint32_t)((uint64_t)n * ch / chunks);
    const uint32_t r1 = (uint32_t)((uint64_t)n * (ch + 1) / chunks);
    auto row_lt = [](const AdjOp& op, uint32_t r) { return op.row < r; };
    size_t k = std::lower_bound(ops.begin(), ops.end(), r0, row_lt) - ops.begin();
    const size_t kend = std::lower_bound(ops.begin(), ops.end(), r1, row_lt) - ops.begin();
    uint32_t next = r0;
    while (k < kend && ok) {
      const uint32_t r = ops[k].row;
      size_t ke = k;
      while (ke < kend && ops[ke].row == r) ++ke;
      move_rows(next, r);
      ok = merge_row(r, k, ke);
      next = r + 1;
      k = ke;
    }
    if (ok) move_rows(next, r1);
  }
  if (!ok) return false;
  a.rp.swap(rp);
  a.col.swap(col);
  a.w.swap(w);
  return true;
}

void host_adj_from_csr(uint32_t n, const uint64_t* rp, const uint32_t* col, const float* w,
                       HostAdj& out) {
  out.n = n;
  out.rp.assign(rp, rp + n + 1);
  out.col.assign(col, col + rp[n]);
  if (w) out.w.assign(w, w + rp[n]);
  // rows sorted by destination, as the reference fragment keeps them
  for (uint32_t v = 0; v < n; ++v) {
    const uint64_t b = out.rp[v], e = out.rp[v + 1];
    bool sorted = true;
    for (uint64_t k = b + 1; k < e; ++k)
      if (out.col[k - 1] > out.col[k]) { sorted = false; break; }
    if (sorted) continue;
    std::vector<std::pair<uint32_t, float>> row;
    for (uint64_t k = b; k < e; ++k) row.push_back({out.col[k], w ? out.w[k] : 0.f});
    std::sort(row.begin(), row.end());
    for (uint64_t k = b; k < e; ++k) {
      out.col[k] = row[k - b].first;
      if (w) out.w[k] = row[k - b].second;
    }
  }
}
}  // namespace sg

extern "C" sg_status sg_util_greedy_clusters(uint32_t n, const uint64_t* row_ptr,
                                             const uint32_t* col, int max_node_num,
                                             int min_node_num, uint64_t seed,
                                             uint32_t* cluster_ptr, uint32_t* members,
                                             uint32_t* n_clusters) {
  if (!row_ptr || !col || !cluster_ptr || !members || !n_clusters || n == 0 ||
      max_node_num < 1 || min_node_num < 1)
    return SG_ERR_INVALID;
  try {
    HostAdj out, in;
    host_adj_from_csr(n, row_ptr, col, nullptr, out);
    host_transpose(out, in);
    auto cl = greedy_clusters(out, in, max_node_num, min_node_num, seed);
    uint32_t k = 0;
    cluster_ptr[0] = 0;
    for (size_t i = 0; i < cl.size(); ++i) {
      for (uint32_t v : cl[i]) members[k++] = v;
      cluster_ptr[i + 1] = k;
    }
    *n_clusters = (uint32_t)cl.size();
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return SG_ERR_OOM;
  }
}

// The summary's cluster state (supernode candidates and mirrors chosen from a
// clustering) in the reference's serialized layout, computed on the host:
// lets the construction be compared byte for byte with the reference's
// serialize_cluster output without a GPU.
extern "C" sg_status sg_util_summary_serialize(uint32_t n, const uint64_t* row_ptr,
                                               const uint32_t* col, uint32_t n_clusters,
                                               const uint32_t* cluster_ptr,
                                               const uint32_t* members, int min_node_num,
                                               int mirror_k, double compress_threshold,
                                               uint8_t* out, uint64_t* size) {
  if (!row_ptr || !size || n == 0 || (n_clusters && (!cluster_ptr || !members)))
    return SG_ERR_INVALID;
  try {
    HostAdj adj, in;
    host_adj_from_csr(n, row_ptr, col, nullptr, adj);
    host_transpose(adj, in);
    std::vector<std::vector<uint32_t>> cl(n_clusters);
    for (uint32_t i = 0; i < n_clusters; ++i) {
      if (cluster_ptr[i + 1] < cluster_ptr[i]) return SG_ERR_INVALID;
      cl[i].assign(members + cluster_ptr[i], members + cluster_ptr[i + 1]);
    }
    Summary S;
    const uint64_t im = summary_init_by_clusters(S, adj, in, cl, min_node_num, mirror_k,
                                                 compress_threshold);
    const std::vector<uint8_t> b = summary_serialize_init(S, im);
    if (out) {
      if (*size < b.size()) return SG_ERR_INVALID;
      std::memcpy(out, b.data(), b.size());
    }
    *size = b.size();
    return SG_OK;
  } catch (const std::bad_alloc&) {
    return SG_ERR_OOM;
  }
}
