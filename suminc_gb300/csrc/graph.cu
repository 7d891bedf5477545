// Device graph: out-CSR and in-CSR with per-vertex slack, the seeded R-MAT
// generator, host load / download, edge-balanced work lists and the in-place
// delta-graph applier.
//
// Layout in HBM (one direction):
//   off[v]  u64  segment start (multiple of 4 entries, 16-byte aligned)
//   cap[v]  u32  segment capacity (multiple of 4)
//   deg[v]  u32  live entries, stored contiguously at the segment head
//   col[]   u32  neighbour ids;  w[] f32 weights (weighted graphs only)
// A segment that outgrows its capacity is re-allocated at the pool tail.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.h"
#include "dev.cuh"

namespace sg {

// ------------------------------------------------------------ small kernels

__global__ void k_fill_u32(uint32_t* p, uint64_t n, uint32_t v) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void k_iota_u32(uint32_t* p, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = (uint32_t)i;
}

// Run boundaries of a key array sorted by (hi32, lo32): first position and
// length of every hi32 value.
__global__ void k_runs(const uint64_t* __restrict__ keys, uint64_t m,
                       uint64_t* __restrict__ start, uint32_t* __restrict__ deg) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t s = (uint32_t)(keys[i] >> 32);
    if (i == 0 || (uint32_t)(keys[i - 1] >> 32) != s) start[s] = i;
    if (i == m - 1 || (uint32_t)(keys[i + 1] >> 32) != s) {
      // length = i + 1 - start[s]; start[s] is written by another thread of
      // the same run's first element, so derive it by search instead.
      uint64_t lo = 0, hi = i;
      while (lo < hi) {  // first index with hi32 == s
        const uint64_t mid = (lo + hi) >> 1;
        if ((uint32_t)(keys[mid] >> 32) < s) lo = mid + 1; else hi = mid;
      }
      deg[s] = (uint32_t)(i + 1 - lo);
    }
  }
}

__global__ void k_capacity(const uint32_t* __restrict__ deg, uint32_t n,
                           float slack, uint64_t* __restrict__ cap64,
                           uint32_t* __restrict__ cap) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += gridDim.x * blockDim.x) {
    const uint32_t d = deg[v];
    uint32_t c = 0;
    if (d > 0) {
      const uint32_t extra = (uint32_t)ceilf((float)d * slack);
      c = (d + extra + 3u) & ~3u;
    }
    cap[v] = c;
    cap64[v] = c;
  }
}

__global__ void k_scatter(const uint64_t* __restrict__ keys,
                          const float* __restrict__ wv, uint64_t m,
                          const uint64_t* __restrict__ start,
                          const uint64_t* __restrict__ off,
                          uint32_t* __restrict__ col, float* __restrict__ w) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    const uint32_t s = (uint32_t)(k >> 32);
    const uint64_t pos = off[s] + (i - start[s]);
    col[pos] = (uint32_t)k;
    if (w) w[pos] = wv[i];
  }
}

__global__ void k_reverse_keys(const uint64_t* __restrict__ keys, uint64_t m,
                               uint64_t* __restrict__ rk) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    rk[i] = (k << 32) | (k >> 32);
  }
}

// ------------------------------------------------------------ helpers

sg_status ensure_cub_tmp(sg_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->cub_tmp_bytes) return SG_OK;
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->cub_tmp) cudaFree(ctx->cub_tmp);
  ctx->cub_tmp = nullptr;
  ctx->cub_tmp_bytes = 0;
  size_t want = bytes + (bytes >> 3) + 4096;
  SG_TRY(dalloc(ctx, (char**)&ctx->cub_tmp, want));
  ctx->cub_tmp_bytes = want;
  return SG_OK;
}

template <typename K, typename V>
static sg_status sort_pairs(sg_ctx* ctx, const K* kin, K* kout, const V* vin,
                            V* vout, uint64_t n, int end_bit = sizeof(K) * 8) {
  size_t bytes = 0;
  SG_CUDA(ctx, cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout,
                                               (int64_t)n, 0, end_bit, ctx->stream));
  SG_TRY(ensure_cub_tmp(ctx, bytes));
  bytes = ctx->cub_tmp_bytes;
  SG_CUDA(ctx, cub::DeviceRadixSort::SortPairs(ctx->cub_tmp, bytes, kin, kout, vin, vout,
                                               (int64_t)n, 0, end_bit, ctx->stream));
  return SG_OK;
}

template <typename K>
static sg_status sort_keys(sg_ctx* ctx, const K* kin, K* kout, uint64_t n,
                           int end_bit = sizeof(K) * 8) {
  size_t bytes = 0;
  SG_CUDA(ctx, cub::DeviceRadixSort::SortKeys(nullptr, bytes, kin, kout, (int64_t)n,
                                              0, end_bit, ctx->stream));
  SG_TRY(ensure_cub_tmp(ctx, bytes));
  bytes = ctx->cub_tmp_bytes;
  SG_CUDA(ctx, cub::DeviceRadixSort::SortKeys(ctx->cub_tmp, bytes, kin, kout, (int64_t)n,
                                              0, end_bit, ctx->stream));
  return SG_OK;
}

template <typename T>
sg_status exclusive_sum(sg_ctx* ctx, const T* in, T* out, uint64_t n) {
  size_t bytes = 0;
  SG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int64_t)n,
                                             ctx->stream));
  SG_TRY(ensure_cub_tmp(ctx, bytes));
  bytes = ctx->cub_tmp_bytes;
  SG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(ctx->cub_tmp, bytes, in, out, (int64_t)n,
                                             ctx->stream));
  return SG_OK;
}
template sg_status exclusive_sum<uint64_t>(sg_ctx*, const uint64_t*, uint64_t*, uint64_t);
template sg_status exclusive_sum<uint32_t>(sg_ctx*, const uint32_t*, uint32_t*, uint64_t);

template <typename T>
static sg_status select_flagged(sg_ctx* ctx, const T* in, const uint8_t* flags,
                                T* out, uint64_t* d_count, uint64_t n) {
  size_t bytes = 0;
  SG_CUDA(ctx, cub::DeviceSelect::Flagged(nullptr, bytes, in, flags, out, d_count,
                                          (int64_t)n, ctx->stream));
  SG_TRY(ensure_cub_tmp(ctx, bytes));
  bytes = ctx->cub_tmp_bytes;
  SG_CUDA(ctx, cub::DeviceSelect::Flagged(ctx->cub_tmp, bytes, in, flags, out, d_count,
                                          (int64_t)n, ctx->stream));
  return SG_OK;
}

sg_status cub_exclusive_sum_u64(sg_ctx* ctx, const uint64_t* in, uint64_t* out, uint64_t n) {
  return exclusive_sum(ctx, in, out, n);
}
sg_status cub_select_flagged_u32(sg_ctx* ctx, const uint32_t* in, const uint8_t* flags,
                                 uint32_t* out, uint64_t* d_count, uint64_t n) {
  return select_flagged(ctx, in, flags, out, d_count, n);
}
sg_status cub_sort_pairs_u64_u32(sg_ctx* ctx, const uint64_t* kin, uint64_t* kout,
                                 const uint32_t* vin, uint32_t* vout, uint64_t n) {
  return sort_pairs(ctx, kin, kout, vin, vout, n);
}
sg_status cub_sort_pairs_u32_u32(sg_ctx* ctx, const uint32_t* kin, uint32_t* kout,
                                 const uint32_t* vin, uint32_t* vout, uint64_t n) {
  return sort_pairs(ctx, kin, kout, vin, vout, n);
}

static void csr_free(DevCSR& c) {
  dfree(c.off);
  dfree(c.deg);
  dfree(c.cap);
  dfree(c.col);
  dfree(c.w);
  dfree(c.pool_tail);
  c.pool_cap = 0;
}

sg_status graph_free(sg_ctx* ctx) {
  DevGraph& g = ctx->g;
  csr_free(g.out);
  csr_free(g.in);
  pull_lists_free(g.in_wl);
  pull_lists_free(g.out_wl);
  dfree(g.hub.rank);
  dfree(g.hub.col);
  dfree(g.hub_out.rank);
  dfree(g.hub_out.col);
  const uint64_t gen = g.gen;  // generations keep growing across graphs
  g = DevGraph();
  g.gen = gen + 1;
  return SG_OK;
}

// Builds one direction from keys sorted by (row, column).
static sg_status build_direction(sg_ctx* ctx, DevCSR& c, uint32_t n, uint64_t m,
                                 const uint64_t* keys, const float* wv,
                                 bool weighted) {
  const float slack = (float)(ctx->opt.slack >= 0 ? ctx->opt.slack : 0.125);
  uint64_t* start = nullptr;
  uint64_t* cap64 = nullptr;
  SG_TRY(dalloc(ctx, &c.off, (uint64_t)n + 1));
  SG_TRY(dalloc(ctx, &c.deg, n));
  SG_TRY(dalloc(ctx, &c.cap, n));
  SG_TRY(dalloc(ctx, &start, n));
  SG_TRY(dalloc(ctx, &cap64, (uint64_t)n + 1));
  SG_TRY(dalloc(ctx, &c.pool_tail, 1));
  SG_CUDA(ctx, cudaMemsetAsync(c.deg, 0, sizeof(uint32_t) * n, ctx->stream));
  if (m > 0) k_runs<<<grid_for(m, 256), 256, 0, ctx->stream>>>(keys, m, start, c.deg);
  k_capacity<<<grid_for(n, 256), 256, 0, ctx->stream>>>(c.deg, n, slack, cap64, c.cap);
  SG_CUDA(ctx, cudaMemsetAsync(cap64 + n, 0, sizeof(uint64_t), ctx->stream));
  SG_TRY(exclusive_sum(ctx, cap64, c.off, (uint64_t)n + 1));
  uint64_t total = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&total, c.off + n, sizeof(uint64_t),
                               cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  // room for relocated segments; a batch that may not fit repacks first
  uint64_t pool_extra = std::max<uint64_t>(total / 16, 1024);
  c.pool_cap = total + pool_extra;
  SG_TRY(dalloc(ctx, &c.col, c.pool_cap));
  if (weighted) SG_TRY(dalloc(ctx, &c.w, c.pool_cap));
  SG_CUDA(ctx, cudaMemcpyAsync(c.pool_tail, &total, sizeof(uint64_t),
                               cudaMemcpyHostToDevice, ctx->stream));
  if (m > 0)
    k_scatter<<<grid_for(m, 256), 256, 0, ctx->stream>>>(keys, weighted ? wv : nullptr, m,
                                                         start, c.off, c.col, c.w);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(start);
  dfree(cap64);
  return SG_OK;
}

sg_status graph_build_from_sorted_keys(sg_ctx* ctx, uint32_t n, uint64_t m,
                                       uint64_t* d_keys, float* d_w,
                                       bool weighted) {
  graph_free(ctx);
  DevGraph& g = ctx->g;
  g.n = n;
  g.m = m;
  g.weighted = weighted;
  SG_TRY(build_direction(ctx, g.out, n, m, d_keys, d_w, weighted));
  // reverse direction: keys (dst, src), weights permuted along
  uint64_t *rk = nullptr, *rk2 = nullptr;
  float* rw2 = nullptr;
  SG_TRY(dalloc(ctx, &rk, m));
  SG_TRY(dalloc(ctx, &rk2, m));
  if (m > 0) k_reverse_keys<<<grid_for(m, 256), 256, 0, ctx->stream>>>(d_keys, m, rk);
  if (weighted) {
    SG_TRY(dalloc(ctx, &rw2, m));
    SG_TRY(sort_pairs(ctx, rk, rk2, d_w, rw2, m));
  } else {
    SG_TRY(sort_keys(ctx, rk, rk2, m));
  }
  dfree(rk);
  SG_TRY(build_direction(ctx, g.in, n, m, rk2, rw2, weighted));
  dfree(rk2);
  dfree(rw2);
  g.valid = true;
  return graph_rebuild_worklists(ctx);
}

// ------------------------------------------------------------ work lists

__global__ void k_nz_flags(const uint32_t* __restrict__ deg, uint32_t n,
                           uint8_t* __restrict__ flags) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += gridDim.x * blockDim.x)
    flags[v] = deg[v] > 0;
}

__global__ void k_quads_of(const uint32_t* __restrict__ nz, uint64_t cnt,
                           const uint32_t* __restrict__ deg,
                           uint64_t* __restrict__ q) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= cnt;
       i += (uint64_t)gridDim.x * blockDim.x)
    q[i] = i < cnt ? (uint64_t)((deg[nz[i]] + 3u) >> 2) : 0;
}

static sg_status worklist_dir(sg_ctx* ctx, const DevCSR& c, uint32_t* nz,
                              uint64_t* qoff, uint32_t* nz_count,
                              uint64_t* quads) {
  const uint32_t n = ctx->g.n;
  uint8_t* flags = nullptr;
  uint32_t* iota = nullptr;
  uint64_t* cnt = nullptr;
  uint64_t* q = nullptr;
  SG_TRY(dalloc(ctx, &flags, n));
  SG_TRY(dalloc(ctx, &iota, n));
  SG_TRY(dalloc(ctx, &cnt, 1));
  SG_TRY(dalloc(ctx, &q, (uint64_t)n + 1));
  k_nz_flags<<<grid_for(n, 256), 256, 0, ctx->stream>>>(c.deg, n, flags);
  k_iota_u32<<<grid_for(n, 256), 256, 0, ctx->stream>>>(iota, n);
  SG_TRY(select_flagged(ctx, iota, flags, nz, cnt, n));
  uint64_t h_cnt = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&h_cnt, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  k_quads_of<<<grid_for(h_cnt + 1, 256), 256, 0, ctx->stream>>>(nz, h_cnt, c.deg, q);
  SG_TRY(exclusive_sum(ctx, q, qoff, h_cnt + 1));
  uint64_t h_q = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&h_q, qoff + h_cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *nz_count = (uint32_t)h_cnt;
  *quads = h_q;
  dfree(flags);
  dfree(iota);
  dfree(cnt);
  dfree(q);
  return SG_OK;
}

__global__ void k_tile_v0(const uint64_t* __restrict__ qoff, uint32_t nz_count, uint64_t ntiles,
                          uint32_t tq, uint32_t* __restrict__ tv0) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ntiles;
       t += (uint64_t)gridDim.x * blockDim.x)
    tv0[t] = upper_owner(qoff, 0u, nz_count, t * (uint64_t)tq);
}

__global__ void k_bnd_flags(const uint64_t* __restrict__ qoff, uint32_t nz_count, uint32_t tq,
                            uint8_t* __restrict__ f) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nz_count; i += gridDim.x * blockDim.x)
    f[i] = (qoff[i] / tq) != ((qoff[i + 1] - 1) / tq);
}

__global__ void k_nz_meta(const uint32_t* __restrict__ nz, uint32_t cnt, const uint64_t* __restrict__ off,
                          const uint32_t* __restrict__ deg, uint64_t* __restrict__ off_nz,
                          uint32_t* __restrict__ deg_nz) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const uint32_t v = nz[i];
    off_nz[i] = off[v];
    deg_nz[i] = deg[v];
  }
}

void pull_lists_free(PullLists& L) {
  dfree(L.nz);
  dfree(L.qoff);
  dfree(L.off_nz);
  dfree(L.deg_nz);
  dfree(L.wtile_v0);
  dfree(L.wbnd);
  L = PullLists();
}

// owners of the first quad of every tq-quad tile, and the vertices whose
// quads cross a tile edge
static sg_status tile_lists(sg_ctx* ctx, PullLists& L, uint32_t tq, uint32_t** tv0,
                            uint64_t* ntiles, uint64_t* cap, uint32_t* bnd, uint32_t* bnd_count) {
  *ntiles = (L.quads + tq - 1) / tq;
  if (*ntiles + 1 > *cap) {
    dfree(*tv0);
    *cap = *ntiles + *ntiles / 8 + 1024;
    SG_TRY(dalloc(ctx, tv0, *cap));
  }
  if (*ntiles)
    k_tile_v0<<<grid_for(*ntiles, 256), 256, 0, ctx->stream>>>(L.qoff, L.nz_count, *ntiles, tq, *tv0);
  uint8_t* flags = nullptr;
  uint64_t* cnt = nullptr;
  SG_TRY(dalloc(ctx, &flags, std::max<uint32_t>(L.nz_count, 1)));
  SG_TRY(dalloc(ctx, &cnt, 1));
  uint64_t h = 0;
  if (L.nz_count) {
    k_bnd_flags<<<grid_for(L.nz_count, 256), 256, 0, ctx->stream>>>(L.qoff, L.nz_count, tq, flags);
    SG_TRY(select_flagged(ctx, L.nz, flags, bnd, cnt, L.nz_count));
    SG_CUDA(ctx, cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *bnd_count = (uint32_t)h;
  dfree(flags);
  dfree(cnt);
  count_launch(ctx, 4);
  return SG_OK;
}

static sg_status build_lists(sg_ctx* ctx, const DevCSR& c, PullLists& L) {
  DevGraph& g = ctx->g;
  const uint32_t n = g.n;
  if (!L.nz || L.n_alloc != n) {
    pull_lists_free(L);
    SG_TRY(dalloc(ctx, &L.nz, n));
    SG_TRY(dalloc(ctx, &L.qoff, (uint64_t)n + 1));
    SG_TRY(dalloc(ctx, &L.wbnd, n));
    SG_TRY(dalloc(ctx, &L.off_nz, n));
    SG_TRY(dalloc(ctx, &L.deg_nz, n));
    L.n_alloc = n;
  }
  SG_TRY(worklist_dir(ctx, c, L.nz, L.qoff, &L.nz_count, &L.quads));
  if (L.nz_count)
    k_nz_meta<<<grid_for(L.nz_count, 256), 256, 0, ctx->stream>>>(L.nz, L.nz_count, c.off, c.deg,
                                                                   L.off_nz, L.deg_nz);
  SG_TRY(tile_lists(ctx, L, kWarpTileQuads, &L.wtile_v0, &L.nwtiles, &L.wtile_cap, L.wbnd,
                    &L.wbnd_count));
  L.gen = g.gen;
  return SG_OK;
}

// the adjacency changed: work lists are rebuilt by their next user
sg_status graph_rebuild_worklists(sg_ctx* ctx) {
  ctx->g.gen++;
  return SG_OK;
}

sg_status graph_in_worklists(sg_ctx* ctx) {
  DevGraph& g = ctx->g;
  if (g.in_wl.nz && g.in_wl.gen == g.gen && g.in_wl.n_alloc == g.n) return SG_OK;
  return build_lists(ctx, g.in, g.in_wl);
}

sg_status graph_out_worklists(sg_ctx* ctx) {
  DevGraph& g = ctx->g;
  if (g.out_wl.nz && g.out_wl.gen == g.gen && g.out_wl.n_alloc == g.n) return SG_OK;
  return build_lists(ctx, g.out, g.out_wl);
}

// ------------------------------------------------------------ R-MAT

__global__ void k_rmat_draws(RmatParams p, uint64_t first, uint64_t count,
                             uint64_t* __restrict__ keys, uint32_t* __restrict__ idx) {
  const uint64_t self_key = (p.scale == 32) ? ~0ull : ((1ull << (2 * p.scale)) - 1);
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t e = rmat_draw(p, first + i);
    const uint32_t s = (uint32_t)(e >> 32), d = (uint32_t)e;
    keys[i] = (s == d) ? self_key : (((uint64_t)s << p.scale) | d);
    idx[i] = (uint32_t)(first + i);
  }
}

__global__ void k_first_flags(const uint64_t* __restrict__ k, uint64_t n,
                              uint64_t sentinel, uint8_t* __restrict__ f) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    f[i] = (k[i] != sentinel) && (i == 0 || k[i] != k[i - 1]);
}

__global__ void k_unpack_keys(uint64_t* __restrict__ k, uint64_t n, int scale,
                              WeightParams wp, float* __restrict__ w) {
  const uint64_t mask = (1ull << scale) - 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t p = k[i];
    const uint64_t s = p >> scale, d = p & mask;
    const uint64_t key = (s << 32) | d;
    k[i] = key;
    if (w) w[i] = edge_weight(wp, key);
  }
}

sg_status generate_rmat(sg_ctx* ctx, int scale, uint64_t edges, double a, double b,
                        double c, uint64_t seed, int wkind, double wlo, double whi) {
  if (scale < 1 || scale > 31) return fail(ctx, SG_ERR_INVALID, "scale must be in [1,31]");
  const uint64_t n = 1ull << scale;
  if (edges > n * (n - 1)) return fail(ctx, SG_ERR_INVALID, "too many edges for scale");
  if (edges >= (1ull << 31)) return fail(ctx, SG_ERR_INVALID, "edges must be < 2^31");
  const RmatParams p = make_rmat_params(scale, a, b, c, seed);
  const uint64_t sentinel = (1ull << (2 * scale)) - 1;
  uint64_t M = edges + edges / 3 + 1024;
  for (int attempt = 0; attempt < 12; ++attempt) {
    if (M >= (1ull << 32)) return fail(ctx, SG_ERR_INVALID, "R-MAT needs too many draws");
    uint64_t *k0 = nullptr, *k1 = nullptr, *cnt = nullptr;
    uint32_t *i0 = nullptr, *i1 = nullptr;
    uint8_t* fl = nullptr;
    SG_TRY(dalloc(ctx, &k0, M));
    SG_TRY(dalloc(ctx, &k1, M));
    SG_TRY(dalloc(ctx, &i0, M));
    SG_TRY(dalloc(ctx, &i1, M));
    SG_TRY(dalloc(ctx, &fl, M));
    SG_TRY(dalloc(ctx, &cnt, 1));
    k_rmat_draws<<<grid_for(M, 256), 256, 0, ctx->stream>>>(p, 0, M, k0, i0);
    SG_TRY(sort_pairs(ctx, k0, k1, i0, i1, M, 2 * scale));
    k_first_flags<<<grid_for(M, 256), 256, 0, ctx->stream>>>(k1, M, sentinel, fl);
    SG_TRY(select_flagged(ctx, k1, fl, k0, cnt, M));  // distinct keys
    SG_TRY(select_flagged(ctx, i1, fl, i0, cnt, M));  // their first draw index
    uint64_t D = 0;
    SG_CUDA(ctx, cudaMemcpyAsync(&D, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (D < edges) {
      dfree(k0); dfree(k1); dfree(i0); dfree(i1); dfree(fl); dfree(cnt);
      const double ratio = (double)edges / (double)std::max<uint64_t>(D, 1);
      M = (uint64_t)((double)M * ratio * 1.08) + 4096;
      continue;
    }
    // order distinct keys by first occurrence, keep the first `edges`
    int idx_bits = 1;
    while ((1ull << idx_bits) < M) ++idx_bits;
    SG_TRY(sort_pairs(ctx, i0, i1, k0, k1, D, idx_bits));
    SG_TRY(sort_keys(ctx, k1, k0, edges, 2 * scale));
    float* w = nullptr;
    if (wkind != 0) SG_TRY(dalloc(ctx, &w, edges));
    const WeightParams wp = make_weight_params(seed, wkind, wlo, whi);
    k_unpack_keys<<<grid_for(edges, 256), 256, 0, ctx->stream>>>(k0, edges, scale, wp, w);
    SG_CUDA(ctx, cudaGetLastError());
    dfree(k1); dfree(i0); dfree(i1); dfree(fl); dfree(cnt);
    sg_status st = graph_build_from_sorted_keys(ctx, (uint32_t)n, edges, k0, w, wkind != 0);
    dfree(k0);
    dfree(w);
    return st;
  }
  return fail(ctx, SG_ERR_INVALID, "R-MAT generator could not reach the edge count");
}

// ------------------------------------------------------------ host load

__global__ void k_keys_from_csr(const uint64_t* __restrict__ rp,
                                const uint32_t* __restrict__ col, uint32_t n,
                                uint64_t* __restrict__ keys, uint32_t* __restrict__ bad) {
  // one warp per row
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t wv = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wv < n;
       wv += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (uint32_t)wv;
    for (uint64_t e = rp[v] + lane; e < rp[v + 1]; e += 32) {
      const uint32_t d = col[e];
      if (d >= n) atomicExch(bad, 1u);
      keys[e] = ((uint64_t)v << 32) | d;
    }
  }
}

sg_status load_csr(sg_ctx* ctx, uint32_t n, const uint64_t* row_ptr,
                   const uint32_t* col, const float* w) {
  if (n == 0 || !row_ptr || (!col && row_ptr[n] > 0))
    return fail(ctx, SG_ERR_INVALID, "empty graph or null arrays");
  const uint64_t m = row_ptr[n];
  for (uint32_t v = 0; v < n; ++v)
    if (row_ptr[v + 1] < row_ptr[v]) return fail(ctx, SG_ERR_INVALID, "row_ptr not monotone");
  uint64_t *d_rp = nullptr, *keys = nullptr, *keys2 = nullptr;
  uint32_t *d_col = nullptr, *bad = nullptr;
  float *d_w = nullptr, *d_w2 = nullptr;
  SG_TRY(dalloc(ctx, &d_rp, (uint64_t)n + 1));
  SG_TRY(dalloc(ctx, &d_col, m));
  SG_TRY(dalloc(ctx, &keys, m));
  SG_TRY(dalloc(ctx, &keys2, m));
  SG_TRY(dalloc(ctx, &bad, 1));
  SG_CUDA(ctx, cudaMemcpyAsync(d_rp, row_ptr, 8ull * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
  if (m) SG_CUDA(ctx, cudaMemcpyAsync(d_col, col, 4ull * m, cudaMemcpyHostToDevice, ctx->stream));
  SG_CUDA(ctx, cudaMemsetAsync(bad, 0, 4, ctx->stream));
  k_keys_from_csr<<<grid_for((uint64_t)n * 32, 256), 256, 0, ctx->stream>>>(d_rp, d_col, n, keys, bad);
  if (w) {
    SG_TRY(dalloc(ctx, &d_w, m));
    SG_TRY(dalloc(ctx, &d_w2, m));
    if (m) SG_CUDA(ctx, cudaMemcpyAsync(d_w, w, 4ull * m, cudaMemcpyHostToDevice, ctx->stream));
    SG_TRY(sort_pairs(ctx, keys, keys2, d_w, d_w2, m));
  } else {
    SG_TRY(sort_keys(ctx, keys, keys2, m));
  }
  uint32_t h_bad = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(d_rp); dfree(d_col); dfree(keys); dfree(bad); dfree(d_w);
  if (h_bad) {
    dfree(keys2); dfree(d_w2);
    return fail(ctx, SG_ERR_INVALID, "column index >= n");
  }
  // a repeated (u, v) pair keeps its first occurrence (the sort is stable)
  uint64_t m_u = m;
  if (m > 1) {
    uint8_t* fl = nullptr;
    uint64_t *kd = nullptr, *cnt = nullptr;
    float* wd = nullptr;
    SG_TRY(dalloc(ctx, &fl, m));
    SG_TRY(dalloc(ctx, &kd, m));
    SG_TRY(dalloc(ctx, &cnt, 1));
    k_first_flags<<<grid_for(m, 256), 256, 0, ctx->stream>>>(keys2, m, ~0ull, fl);
    SG_TRY(select_flagged(ctx, keys2, fl, kd, cnt, m));
    if (w) {
      SG_TRY(dalloc(ctx, &wd, m));
      SG_TRY(select_flagged(ctx, d_w2, fl, wd, cnt, m));
    }
    SG_CUDA(ctx, cudaMemcpyAsync(&m_u, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    count_launch(ctx, 3);
    dfree(fl);
    dfree(cnt);
    dfree(keys2);
    keys2 = kd;
    if (w) {
      dfree(d_w2);
      d_w2 = wd;
    }
  }
  sg_status st = graph_build_from_sorted_keys(ctx, n, m_u, keys2, d_w2, w != nullptr);
  dfree(keys2);
  dfree(d_w2);
  return st;
}

// ------------------------------------------------------------ download

__global__ void k_pack_rows(const DevCSR c, uint32_t n, const uint64_t* __restrict__ rp,
                            uint32_t* __restrict__ col, float* __restrict__ w) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t wv = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wv < n;
       wv += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (uint32_t)wv;
    const uint64_t src = c.off[v], dst = rp[v];
    const uint32_t d = c.deg[v];
    for (uint32_t k = lane; k < d; k += 32) {
      col[dst + k] = c.col[src + k];
      if (w) w[dst + k] = c.w[src + k];
    }
  }
}

__global__ void k_deg64(const uint32_t* __restrict__ deg, uint32_t n, uint64_t* __restrict__ o) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= n;
       i += (uint64_t)gridDim.x * blockDim.x)
    o[i] = i < n ? deg[i] : 0;
}

// ------------------------------------------------------------ weights

__global__ void k_row_wsum(const DevCSR c, uint32_t n, float* __restrict__ s) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t wv = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wv < n;
       wv += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (uint32_t)wv;
    const uint64_t o = c.off[v];
    const uint32_t d = c.deg[v];
    double acc = 0.0;
    for (uint32_t k = lane; k < d; k += 32) acc += (double)c.w[o + k];
#pragma unroll
    for (int x = 16; x > 0; x >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, x);
    if (lane == 0) s[v] = (float)acc;
  }
}

// out-CSR: w /= s[row]; in-CSR: w /= s[source] (col holds the source)
__global__ void k_row_wscale(const DevCSR c, uint32_t n, const float* __restrict__ s, bool by_col) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t wv = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wv < n;
       wv += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (uint32_t)wv;
    const uint64_t o = c.off[v];
    const uint32_t d = c.deg[v];
    for (uint32_t k = lane; k < d; k += 32) {
      const float t = by_col ? s[c.col[o + k]] : s[v];
      if (t > 0.f) c.w[o + k] /= t;
    }
  }
}

sg_status normalize_out_weights(sg_ctx* ctx) {
  DevGraph& g = ctx->g;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  if (!g.weighted) return fail(ctx, SG_ERR_INVALID, "graph has no weights");
  float* s = nullptr;
  SG_TRY(dalloc(ctx, &s, g.n));
  const unsigned b = grid_for((uint64_t)g.n * 32, 256);
  k_row_wsum<<<b, 256, 0, ctx->stream>>>(g.out, g.n, s);
  k_row_wscale<<<b, 256, 0, ctx->stream>>>(g.in, g.n, s, true);
  k_row_wscale<<<b, 256, 0, ctx->stream>>>(g.out, g.n, s, false);
  count_launch(ctx, 3);
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(s);
  g.gen++;  // values derived from the weights are stale
  return SG_OK;
}

sg_status packed_sorted_out(sg_ctx* ctx, uint64_t* d_rp, uint32_t* d_col) {
  DevGraph& g = ctx->g;
  const uint32_t n = g.n;
  const uint64_t m = g.m;
  uint64_t* d64 = nullptr;
  uint32_t* c1 = nullptr;
  SG_TRY(dalloc(ctx, &d64, (uint64_t)n + 1));
  SG_TRY(dalloc(ctx, &c1, m));
  k_deg64<<<grid_for((uint64_t)n + 1, 256), 256, 0, ctx->stream>>>(g.out.deg, n, d64);
  SG_TRY(exclusive_sum(ctx, d64, d_rp, (uint64_t)n + 1));
  k_pack_rows<<<grid_for((uint64_t)n * 32, 256), 256, 0, ctx->stream>>>(g.out, n, d_rp, c1, nullptr);
  size_t bytes = 0;
  SG_CUDA(ctx, cub::DeviceSegmentedSort::SortKeys(nullptr, bytes, c1, d_col, (int64_t)m,
                                                  (int64_t)n, d_rp, d_rp + 1, ctx->stream));
  SG_TRY(ensure_cub_tmp(ctx, bytes));
  bytes = ctx->cub_tmp_bytes;
  SG_CUDA(ctx, cub::DeviceSegmentedSort::SortKeys(ctx->cub_tmp, bytes, c1, d_col, (int64_t)m,
                                                  (int64_t)n, d_rp, d_rp + 1, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(d64);
  dfree(c1);
  count_launch(ctx, 4);
  return SG_OK;
}

sg_status download_csr(sg_ctx* ctx, uint64_t* row_ptr, uint32_t* col, float* w) {
  DevGraph& g = ctx->g;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  const uint32_t n = g.n;
  const uint64_t m = g.m;
  uint64_t *d64 = nullptr, *rp = nullptr;
  uint32_t *c1 = nullptr, *c2 = nullptr;
  float *w1 = nullptr, *w2 = nullptr;
  SG_TRY(dalloc(ctx, &d64, (uint64_t)n + 1));
  SG_TRY(dalloc(ctx, &rp, (uint64_t)n + 1));
  SG_TRY(dalloc(ctx, &c1, m));
  SG_TRY(dalloc(ctx, &c2, m));
  const bool want_w = (w != nullptr) && g.weighted;
  if (want_w) {
    SG_TRY(dalloc(ctx, &w1, m));
    SG_TRY(dalloc(ctx, &w2, m));
  }
  k_deg64<<<grid_for((uint64_t)n + 1, 256), 256, 0, ctx->stream>>>(g.out.deg, n, d64);
  SG_TRY(exclusive_sum(ctx, d64, rp, (uint64_t)n + 1));
  k_pack_rows<<<grid_for((uint64_t)n * 32, 256), 256, 0, ctx->stream>>>(g.out, n, rp, c1,
                                                                       want_w ? w1 : nullptr);
  size_t bytes = 0;
  if (want_w) {
    SG_CUDA(ctx, cub::DeviceSegmentedSort::SortPairs(nullptr, bytes, c1, c2, w1, w2, (int64_t)m,
                                                     (int64_t)n, rp, rp + 1, ctx->stream));
    SG_TRY(ensure_cub_tmp(ctx, bytes));
    bytes = ctx->cub_tmp_bytes;
    SG_CUDA(ctx, cub::DeviceSegmentedSort::SortPairs(ctx->cub_tmp, bytes, c1, c2, w1, w2,
                                                     (int64_t)m, (int64_t)n, rp, rp + 1,
                                                     ctx->stream));
  } else {
    SG_CUDA(ctx, cub::DeviceSegmentedSort::SortKeys(nullptr, bytes, c1, c2, (int64_t)m,
                                                    (int64_t)n, rp, rp + 1, ctx->stream));
    SG_TRY(ensure_cub_tmp(ctx, bytes));
    bytes = ctx->cub_tmp_bytes;
    SG_CUDA(ctx, cub::DeviceSegmentedSort::SortKeys(ctx->cub_tmp, bytes, c1, c2, (int64_t)m,
                                                    (int64_t)n, rp, rp + 1, ctx->stream));
  }
  if (row_ptr)
    SG_CUDA(ctx, cudaMemcpyAsync(row_ptr, rp, 8ull * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
  if (col && m)
    SG_CUDA(ctx, cudaMemcpyAsync(col, c2, 4ull * m, cudaMemcpyDeviceToHost, ctx->stream));
  if (w && m) {
    if (want_w) {
      SG_CUDA(ctx, cudaMemcpyAsync(w, w2, 4ull * m, cudaMemcpyDeviceToHost, ctx->stream));
    } else {
      SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      for (uint64_t i = 0; i < m; ++i) w[i] = 1.0f;
    }
  }
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(d64); dfree(rp); dfree(c1); dfree(c2); dfree(w1); dfree(w2);
  return SG_OK;
}

// ------------------------------------------------------------ applier
//
// 1. upload; key = (src, dst), value = (position << 1) | op
// 2. stable radix sort by key -> records of one pair are adjacent, in file
//    order;  one action per pair:  bit0 = "delete the old edge",
//    bit1 = "edge present afterwards with the first add's weight"
// 3. group actions by source (they are sorted by (src, dst)) and by
//    destination (second sort), one warp per group patches the segment.

__global__ void k_upd_keys(const sg_update* __restrict__ u, uint64_t cnt, uint32_t n,
                           uint64_t* __restrict__ key, uint32_t* __restrict__ val,
                           uint32_t* __restrict__ bad) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const sg_update r = u[i];
    if (r.src >= n || r.dst >= n || r.op > 1) atomicExch(bad, 1u);
    key[i] = ((uint64_t)(r.src % n) << 32) | (r.dst % n);
    val[i] = ((uint32_t)i << 1) | (r.op & 1u);
  }
}

__global__ void k_run_flags(const uint64_t* __restrict__ k, uint64_t n, uint8_t* __restrict__ f) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    f[i] = (i == 0 || k[i] != k[i - 1]);
}

// one thread per run of equal keys
__global__ void k_make_actions(const uint64_t* __restrict__ key, const uint32_t* __restrict__ val,
                               const uint32_t* __restrict__ run_start, uint64_t n_runs,
                               uint64_t n_rec, const sg_update* __restrict__ raw,
                               uint32_t* __restrict__ a_src, uint32_t* __restrict__ a_dst,
                               float* __restrict__ a_w, uint32_t* __restrict__ a_kind,
                               uint32_t* __restrict__ a_found) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_runs;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = run_start[r];
    const uint64_t e = (r + 1 < n_runs) ? run_start[r + 1] : n_rec;
    uint32_t kind = 0;
    float w = 0.f;
    for (uint64_t i = b; i < e; ++i) {
      const uint32_t v = val[i];
      if (v & 1u) {
        kind |= 1u;
      } else if (!(kind & 2u)) {
        kind |= 2u;
        w = raw[v >> 1].weight;
      }
    }
    const uint64_t k = key[b];
    a_src[r] = (uint32_t)(k >> 32);
    a_dst[r] = (uint32_t)k;
    a_w[r] = w;
    a_kind[r] = kind;
    a_found[r] = kInvalidVid;
  }
}

__global__ void k_group_flags(const uint32_t* __restrict__ v, const uint32_t* __restrict__ perm,
                              uint64_t n, uint8_t* __restrict__ f) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t cur = perm ? v[perm[i]] : v[i];
    f[i] = (i == 0) || cur != (perm ? v[perm[i - 1]] : v[i - 1]);
  }
}

__global__ void k_group_bounds(const uint32_t* __restrict__ starts, uint64_t n_grp,
                               uint64_t n_act, const uint32_t* __restrict__ v,
                               const uint32_t* __restrict__ perm, uint32_t* __restrict__ gv,
                               uint32_t* __restrict__ gb, uint32_t* __restrict__ ge) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_grp;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t b = starts[i];
    gb[i] = b;
    ge[i] = (i + 1 < n_grp) ? starts[i + 1] : (uint32_t)n_act;
    gv[i] = perm ? v[perm[b]] : v[b];
  }
}

__global__ void k_inv_keys(const uint32_t* __restrict__ s, const uint32_t* __restrict__ d,
                           uint64_t n, uint64_t* __restrict__ k, uint32_t* __restrict__ idx) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    k[i] = ((uint64_t)d[i] << 32) | s[i];
    idx[i] = (uint32_t)i;
  }
}


// ------------------------------------------------------------ repack
//
// Segments that outgrow their capacity move to the pool tail and leave their
// old slots unused.  Before a batch whose worst case no longer fits the free
// tail, a direction is repacked: fresh capacities with slack, live entries
// copied in vertex order, a new pool with room for the batch.

// slots a batch may need in one direction: a vertex moves to the pool tail
// only when its new length exceeds its capacity, and its new length is at
// most its live entries plus its actions, so a vertex whose bound fits its
// capacity needs nothing and any other at most the capacity the applier
// gives a moved row for that bound.  cap == nullptr counts every vertex with
// actions (the need after a repack, which resets every capacity).
__global__ void k_batch_need(const uint32_t* __restrict__ gv, const uint32_t* __restrict__ gb,
                             const uint32_t* __restrict__ ge, uint64_t n_grp,
                             const uint32_t* __restrict__ deg, const uint32_t* __restrict__ cap,
                             unsigned long long* need) {
  unsigned long long acc = 0;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < n_grp;
       g += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t v = gv[g];
    const uint64_t d1 = (uint64_t)deg[v] + (ge[g] - gb[g]);
    if (!cap || d1 > cap[v]) acc += ((d1 + d1 / 8 + 4 + 3) & ~3ull);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(need, acc);
}

__global__ void k_repack_rows(const uint64_t* __restrict__ off_old, const uint32_t* __restrict__ deg,
                              const uint32_t* __restrict__ col_old, const float* __restrict__ w_old,
                              uint32_t n, const uint64_t* __restrict__ off_new,
                              uint32_t* __restrict__ col_new, float* __restrict__ w_new) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t wv = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wv < n;
       wv += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (uint32_t)wv;
    const uint64_t a = off_old[v], b = off_new[v];
    const uint32_t d = deg[v];
    for (uint32_t k = lane; k < d; k += 32) {
      col_new[b + k] = col_old[a + k];
      if (w_new) w_new[b + k] = w_old[a + k];
    }
  }
}

static sg_status repack_direction(sg_ctx* ctx, DevCSR& c, uint64_t batch_need) {
  const uint32_t n = ctx->g.n;
  const float slack = (float)(ctx->opt.slack >= 0 ? ctx->opt.slack : 0.125);
  cudaStream_t st = ctx->stream;
  uint64_t *cap64 = nullptr, *off_new = nullptr;
  SG_TRY(dalloc(ctx, &cap64, (uint64_t)n + 1));
  SG_TRY(dalloc(ctx, &off_new, (uint64_t)n + 1));
  k_capacity<<<grid_for(n, 256), 256, 0, st>>>(c.deg, n, slack, cap64, c.cap);
  SG_CUDA(ctx, cudaMemsetAsync(cap64 + n, 0, sizeof(uint64_t), st));
  SG_TRY(exclusive_sum(ctx, cap64, off_new, (uint64_t)n + 1));
  uint64_t total = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&total, off_new + n, 8, cudaMemcpyDeviceToHost, st));
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  const uint64_t extra = std::max<uint64_t>({total / 16, 1024ull, 2 * batch_need});
  const uint64_t pool = total + extra;
  uint32_t* col_new = nullptr;
  float* w_new = nullptr;
  SG_TRY(dalloc(ctx, &col_new, pool));
  if (c.w) SG_TRY(dalloc(ctx, &w_new, pool));
  k_repack_rows<<<grid_for((uint64_t)n * 32, 256), 256, 0, st>>>(c.off, c.deg, c.col, c.w, n, off_new,
                                                                col_new, w_new);
  SG_CUDA(ctx, cudaMemcpyAsync(c.pool_tail, &total, 8, cudaMemcpyHostToDevice, st));
  SG_CUDA(ctx, cudaGetLastError());
  SG_CUDA(ctx, cudaStreamSynchronize(st));
  dfree(c.off);
  dfree(c.col);
  dfree(c.w);
  dfree(cap64);
  c.off = off_new;
  c.col = col_new;
  c.layout++;
  c.w = w_new;
  c.pool_cap = pool;
  count_launch(ctx, 4);
  ctx->repacks++;
  return SG_OK;
}

static sg_status batch_need(sg_ctx* ctx, const DevCSR& c, const uint32_t* gv, const uint32_t* gb,
                            const uint32_t* ge, uint64_t n_grp, const uint32_t* cap,
                            unsigned long long* d_need, unsigned long long* need) {
  SG_CUDA(ctx, cudaMemsetAsync(d_need, 0, 8, ctx->stream));
  if (n_grp) {
    k_batch_need<<<grid_for(n_grp, 256), 256, 0, ctx->stream>>>(gv, gb, ge, n_grp, c.deg, cap,
                                                                  d_need);
    count_launch(ctx);
  }
  SG_CUDA(ctx, cudaMemcpyAsync(need, d_need, 8, cudaMemcpyDeviceToHost, ctx->stream));
  return SG_OK;
}

// Repacks each direction whose free tail cannot hold the batch's need.  The
// need against the current capacities decides; a repack resets every
// capacity to the live degree plus slack, so it reserves the worst case
// (every vertex with actions moves).
static sg_status ensure_pool(sg_ctx* ctx, DevCSR& c, const uint32_t* gv, const uint32_t* gb,
                             const uint32_t* ge, uint64_t n_grp, unsigned long long* d_need) {
  unsigned long long need = 0, tail = 0;
  SG_TRY(batch_need(ctx, c, gv, gb, ge, n_grp, c.cap, d_need, &need));
  SG_CUDA(ctx, cudaMemcpyAsync(&tail, c.pool_tail, 8, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (tail + need <= c.pool_cap) return SG_OK;
  unsigned long long worst = 0;
  SG_TRY(batch_need(ctx, c, gv, gb, ge, n_grp, nullptr, d_need, &worst));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return repack_direction(ctx, c, worst);
}

constexpr uint32_t kApplyChunk = 1024;  // segment entries per find / amend work item

struct ApplyDirArgs {
  DevCSR c;
  const uint32_t* gv;     // group vertex
  const uint32_t* gb;     // group [begin, end) in action order
  const uint32_t* ge;
  uint64_t n_grp;
  const uint32_t* perm;   // null: identity; else action index of position j
  const uint32_t* a_nbr;  // neighbour id of each action in this direction
  const float* a_w;
  const uint32_t* a_kind;
  const uint32_t* a_found;  // out-direction slot of the pair before the batch
  uint32_t* a_pos;          // this direction's slot of the pair (written by find)
  uint32_t* a_tmp;          // per-action scratch (hole list)
  uint32_t* g_d0;           // degree before the batch
  uint32_t* g_ndel;         // deletions of the group
  uint32_t* g_nins;         // insertions of the group
  const uint32_t* chunk_off;  // [n_grp + 1] work-item prefix
  uint64_t n_chunks;
  bool out_dir;
  // PageRank amend (out direction; null when no PageRank state is live)
  float* pr_x;
  float* pr_delta;
  float damping;
  // SSSP reset seeds (out direction; null when no SSSP state is live)
  const uint32_t* sp_parent;
  uint32_t* sp_reset;
  uint32_t* sp_seeds;
  uint32_t* sp_seed_count;
  // the PageRank pull's encoded column copy (in direction; null when none
  // is current): every column write is mirrored there as the id's rank
  uint32_t* col2;
  const uint32_t* hub_rank;
  uint32_t n;
  // bookkeeping
  unsigned long long* d_dm;  // signed edge-count change (two's complement)
  uint32_t* d_err;
};

// a column write, mirrored into the encoded copy when there is one
__device__ __forceinline__ void put_col(const ApplyDirArgs& A, uint64_t p, uint32_t x) {
  A.c.col[p] = x;
  if (A.col2) A.col2[p] = x < A.n ? A.hub_rank[x] : x;
}

__device__ __forceinline__ uint32_t act_at(const ApplyDirArgs& A, uint32_t j) {
  return A.perm ? A.perm[j] : j;
}

// Position in [b, e) of the action whose neighbour is t, or -1.
__device__ __forceinline__ int find_action(const ApplyDirArgs& A, uint32_t b, uint32_t e,
                                           uint32_t t) {
  uint32_t lo = b, hi = e;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (A.a_nbr[act_at(A, mid)] < t) lo = mid + 1; else hi = mid;
  }
  if (lo < e && A.a_nbr[act_at(A, lo)] == t) return (int)lo;
  return -1;
}

// work items per group: ceil(d0 / chunk), at least one
__global__ void k_apply_chunks(ApplyDirArgs A, uint32_t* nch) {
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g <= A.n_grp;
       g += (uint64_t)gridDim.x * blockDim.x) {
    if (g == A.n_grp) {
      nch[g] = 0;
      continue;
    }
    const uint32_t d0 = A.c.deg[A.gv[g]];
    A.g_d0[g] = d0;
    nch[g] = d0 == 0 ? 1u : (d0 + kApplyChunk - 1) / kApplyChunk;
  }
}

__device__ __forceinline__ uint32_t group_of_chunk(const ApplyDirArgs& A, uint64_t c) {
  uint32_t lo = 0, hi = (uint32_t)A.n_grp;  // largest g with chunk_off[g] <= c
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (A.chunk_off[mid] <= c) lo = mid; else hi = mid;
  }
  return lo;
}

// 1. locate every action's pair in its segment (one warp per 1024-entry
//    chunk): record the slot, tombstone pure deletes, overwrite re-added
//    weights.
__global__ void __launch_bounds__(256) k_apply_find(ApplyDirArgs A) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; c < A.n_chunks;
       c += nwarps) {
    const uint32_t g = group_of_chunk(A, c);
    const uint32_t u = A.gv[g], b = A.gb[g], e = A.ge[g];
    const uint32_t d0 = A.g_d0[g];
    const uint64_t base = A.c.off[u];
    const uint32_t k0 = (uint32_t)(c - A.chunk_off[g]) * kApplyChunk;
    const uint32_t k1 = min(k0 + kApplyChunk, d0);
    for (uint32_t k = k0 + lane; k < k1; k += 32) {
      const uint32_t t = A.c.col[base + k];
      const int j = find_action(A, b, e, t);
      if (j < 0) continue;
      const uint32_t a = act_at(A, (uint32_t)j);
      const uint32_t kind = A.a_kind[a];
      A.a_pos[a] = k;
      if (kind == 1u) put_col(A, base + k, kInvalidVid);
      else if ((kind & 2u) && A.c.w) A.c.w[base + k] = A.a_w[a];
    }
  }
}

// 2. per vertex (warp per group, over its actions only): counts, the
//    PageRank amend of deleted / inserted targets, SSSP reset seeds.
__global__ void __launch_bounds__(256) k_apply_group(ApplyDirArgs A) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t g = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; g < A.n_grp;
       g += nwarps) {
    const uint32_t u = A.gv[g], b = A.gb[g], e = A.ge[g];
    const uint32_t d0 = A.g_d0[g];
    uint32_t ndel = 0, nins = 0;
    for (uint32_t j = b + lane; j < e; j += 32) {
      const uint32_t a = act_at(A, j);
      const uint32_t kind = A.a_kind[a];
      const bool found = A.a_found[a] != kInvalidVid;
      ndel += (kind == 1u && found);
      nins += ((kind & 2u) && !found);
    }
    ndel = __reduce_add_sync(0xffffffffu, ndel);
    nins = __reduce_add_sync(0xffffffffu, nins);
    if (lane == 0) {
      A.g_ndel[g] = ndel;
      A.g_nins[g] = nins;
    }
    if (!A.out_dir) continue;
    const uint32_t d1 = d0 - ndel + nins;
    // PageRank: AmendValue(-1) / AmendValue(+1) restricted to u (for every
    // other vertex the two cancel); surviving edges are amended by
    // k_apply_amend.
    if (A.pr_x && (ndel > 0 || nins > 0)) {
      const float xu = A.pr_x[u];
      if (xu != 0.f) {
        const float sub = d0 > 0 ? A.damping * xu / (float)d0 : 0.f;
        const float add = d1 > 0 ? A.damping * xu / (float)d1 : 0.f;
        for (uint32_t j = b + lane; j < e; j += 32) {
          const uint32_t a = act_at(A, j);
          const uint32_t kind = A.a_kind[a];
          const bool found = A.a_found[a] != kInvalidVid;
          if (kind == 1u && found && sub != 0.f) atomicAdd(&A.pr_delta[A.a_nbr[a]], -sub);
          if ((kind & 2u) && !found && add != 0.f) atomicAdd(&A.pr_delta[A.a_nbr[a]], add);
        }
      }
    }
    // SSSP: a deleted (or re-weighted) edge that is the tree edge of its
    // head resets the head (deltaCompute, sum_sync_traversal_worker.h:140-176)
    if (A.sp_parent) {
      for (uint32_t j = b + lane; j < e; j += 32) {
        const uint32_t a = act_at(A, j);
        if ((A.a_kind[a] & 1u) && A.a_found[a] != kInvalidVid) {
          const uint32_t v = A.a_nbr[a];
          if (A.sp_parent[v] == u && atomicExch(&A.sp_reset[v], 1u) == 0u)
            A.sp_seeds[atomicAdd(A.sp_seed_count, 1u)] = v;
        }
      }
    }
    if (lane == 0) atomicAdd(A.d_dm, (unsigned long long)((long long)nins - (long long)ndel));
  }
}

// 3. PageRank amend of the surviving edges of a vertex whose out-degree
//    changed (one warp per chunk).
__global__ void __launch_bounds__(256) k_apply_amend(ApplyDirArgs A) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; c < A.n_chunks;
       c += nwarps) {
    const uint32_t g = group_of_chunk(A, c);
    const uint32_t u = A.gv[g];
    const uint32_t d0 = A.g_d0[g];
    const uint32_t d1 = d0 - A.g_ndel[g] + A.g_nins[g];
    if (d0 == d1) continue;
    const float xu = A.pr_x[u];
    if (xu == 0.f) continue;
    const float sub = d0 > 0 ? A.damping * xu / (float)d0 : 0.f;
    const float add = d1 > 0 ? A.damping * xu / (float)d1 : 0.f;
    const float diff = add - sub;
    if (diff == 0.f) continue;
    const uint64_t base = A.c.off[u];
    const uint32_t k0 = (uint32_t)(c - A.chunk_off[g]) * kApplyChunk;
    const uint32_t k1 = min(k0 + kApplyChunk, d0);
    for (uint32_t k = k0 + lane; k < k1; k += 32) {
      const uint32_t t = A.c.col[base + k];
      if (t != kInvalidVid) atomicAdd(&A.pr_delta[t], diff);
    }
  }
}

// 4. per vertex: fill the tombstones below the new live length with the
//    live entries above it (O(deletions)), grow into the pool if needed,
//    append insertions.
__global__ void __launch_bounds__(256) k_apply_finish(ApplyDirArgs A) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t g = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; g < A.n_grp;
       g += nwarps) {
    const uint32_t u = A.gv[g], b = A.gb[g], e = A.ge[g];
    const uint32_t d0 = A.g_d0[g], ndel = A.g_ndel[g];
    uint64_t base = A.c.off[u];
    const uint32_t newlen = d0 - ndel;
    // tombstone slots below newlen, in action order
    uint32_t nh = 0;
    for (uint32_t jb = b; jb < e; jb += 32) {
      const uint32_t j = jb + lane;
      bool hole = false;
      uint32_t pos = 0;
      if (j < e) {
        const uint32_t a = act_at(A, j);
        if (A.a_kind[a] == 1u && A.a_found[a] != kInvalidVid) {
          pos = A.a_pos[a];
          hole = pos < newlen;
        }
      }
      const uint32_t mask = __ballot_sync(0xffffffffu, hole);
      if (hole) A.a_tmp[b + nh + __popc(mask & lanemask_lt())] = pos;
      nh += __popc(mask);
    }
    __syncwarp();
    // live entries at or above newlen move into those holes
    uint32_t r = 0;
    for (uint32_t kb = newlen; kb < d0; kb += 32) {
      const uint32_t k = kb + lane;
      uint32_t cval = kInvalidVid;
      float wv = 0.f;
      if (k < d0) {
        cval = A.c.col[base + k];
        if (A.c.w) wv = A.c.w[base + k];
      }
      const bool live = k < d0 && cval != kInvalidVid;
      const uint32_t mask = __ballot_sync(0xffffffffu, live);
      if (live) {
        const uint32_t h = A.a_tmp[b + r + __popc(mask & lanemask_lt())];
        put_col(A, base + h, cval);
        if (A.c.w) A.c.w[base + h] = wv;
      }
      r += __popc(mask);
    }
    if (r != nh && lane == 0) atomicExch(A.d_err, 3u);
    __syncwarp();
    const uint32_t d1 = newlen + A.g_nins[g];
    const uint32_t cap = A.c.cap[u];
    if (d1 > cap) {
      const uint32_t ncap = (d1 + d1 / 8u + 4u + 3u) & ~3u;
      unsigned long long nb = 0;
      if (lane == 0) nb = atomicAdd((unsigned long long*)A.c.pool_tail, (unsigned long long)ncap);
      nb = __shfl_sync(0xffffffffu, nb, 0);
      if (nb + ncap > A.c.pool_cap) {
        if (lane == 0) {
          atomicExch(A.d_err, 1u);
          A.c.deg[u] = newlen;
        }
        continue;  // insertions dropped; host reports SG_ERR_OOM
      }
      for (uint32_t k = lane; k < newlen; k += 32) {
        put_col(A, nb + k, A.c.col[base + k]);
        if (A.c.w) A.c.w[nb + k] = A.c.w[base + k];
      }
      __syncwarp();
      base = nb;
      if (lane == 0) {
        A.c.off[u] = nb;
        A.c.cap[u] = ncap;
      }
    }
    uint32_t wp = newlen;
    for (uint32_t jb = b; jb < e; jb += 32) {
      const uint32_t j = jb + lane;
      bool ins = false;
      uint32_t a = 0;
      if (j < e) {
        a = act_at(A, j);
        ins = (A.a_kind[a] & 2u) && A.a_found[a] == kInvalidVid;
      }
      const uint32_t mask = __ballot_sync(0xffffffffu, ins);
      const uint32_t pos = wp + __popc(mask & lanemask_lt());
      if (ins) {
        put_col(A, base + pos, A.a_nbr[a]);
        if (A.c.w) A.c.w[base + pos] = A.a_w[a];
      }
      wp += __popc(mask);
    }
    if (lane == 0) A.c.deg[u] = wp;
  }
}

static sg_status batch_reserve(sg_ctx* ctx, uint64_t count) {
  DevBatch& B = ctx->batch;
  if (count <= B.cap) return SG_OK;
  dfree(B.raw); dfree(B.key); dfree(B.key2); dfree(B.val); dfree(B.val2);
  dfree(B.a_src); dfree(B.a_dst); dfree(B.a_w); dfree(B.a_kind); dfree(B.a_found);
  dfree(B.grp_vertex); dfree(B.grp_begin); dfree(B.grp_end); dfree(B.perm);
  dfree(B.igrp_vertex); dfree(B.igrp_begin); dfree(B.igrp_end); dfree(B.d_count);
  dfree(B.a_pos_in); dfree(B.a_tmp); dfree(B.g_d0); dfree(B.g_ndel); dfree(B.g_nins);
  dfree(B.chunk_off); dfree(B.nch);
  uint64_t c = std::max<uint64_t>(count, 1024);
  SG_TRY(dalloc(ctx, &B.raw, c));
  SG_TRY(dalloc(ctx, &B.key, c));
  SG_TRY(dalloc(ctx, &B.key2, c));
  SG_TRY(dalloc(ctx, &B.val, c));
  SG_TRY(dalloc(ctx, &B.val2, c));
  SG_TRY(dalloc(ctx, &B.a_src, c));
  SG_TRY(dalloc(ctx, &B.a_dst, c));
  SG_TRY(dalloc(ctx, &B.a_w, c));
  SG_TRY(dalloc(ctx, &B.a_kind, c));
  SG_TRY(dalloc(ctx, &B.a_found, c));
  SG_TRY(dalloc(ctx, &B.grp_vertex, c));
  SG_TRY(dalloc(ctx, &B.grp_begin, c));
  SG_TRY(dalloc(ctx, &B.grp_end, c));
  SG_TRY(dalloc(ctx, &B.perm, c));
  SG_TRY(dalloc(ctx, &B.igrp_vertex, c));
  SG_TRY(dalloc(ctx, &B.igrp_begin, c));
  SG_TRY(dalloc(ctx, &B.igrp_end, c));
  SG_TRY(dalloc(ctx, &B.d_count, 4));
  SG_TRY(dalloc(ctx, &B.a_pos_in, c));
  SG_TRY(dalloc(ctx, &B.a_tmp, c));
  SG_TRY(dalloc(ctx, &B.g_d0, 2 * c));
  SG_TRY(dalloc(ctx, &B.g_ndel, 2 * c));
  SG_TRY(dalloc(ctx, &B.g_nins, 2 * c));
  SG_TRY(dalloc(ctx, &B.chunk_off, 2 * (c + 1)));
  SG_TRY(dalloc(ctx, &B.nch, c + 1));
  B.cap = c;
  return SG_OK;
}

// groups of equal vertex over an action order (perm == null: identity)
static sg_status make_groups(sg_ctx* ctx, const uint32_t* vtx, const uint32_t* perm,
                             uint64_t n_act, uint32_t* gv, uint32_t* gb, uint32_t* ge,
                             uint64_t* n_grp) {
  DevBatch& B = ctx->batch;
  uint8_t* flags = (uint8_t*)B.key2;  // scratch (n_act bytes)
  uint32_t* iota = B.val2;
  uint32_t* starts = B.val;
  k_group_flags<<<grid_for(n_act, 256), 256, 0, ctx->stream>>>(vtx, perm, n_act, flags);
  k_iota_u32<<<grid_for(n_act, 256), 256, 0, ctx->stream>>>(iota, n_act);
  SG_TRY(select_flagged(ctx, iota, flags, starts, B.d_count, n_act));
  uint64_t h = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&h, B.d_count, 8, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  k_group_bounds<<<grid_for(h, 256), 256, 0, ctx->stream>>>(starts, h, n_act, vtx, perm, gv, gb, ge);
  *n_grp = h;
  return SG_OK;
}

sg_status apply_updates_device(sg_ctx* ctx, uint64_t count, const sg_update* upd,
                               bool on_device) {
  DevGraph& g = ctx->g;
  DevBatch& B = ctx->batch;
  if (!g.valid) return fail(ctx, SG_ERR_STATE, "no graph loaded");
  if (count == 0) return SG_OK;
  if (!upd) return fail(ctx, SG_ERR_INVALID, "null update array");
  if (count >= (1ull << 31)) return fail(ctx, SG_ERR_INVALID, "batch too large");
  SG_TRY(batch_reserve(ctx, count));
  SG_CUDA(ctx, cudaMemcpyAsync(B.raw, upd, sizeof(sg_update) * count,
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               ctx->stream));
  uint32_t* d_err = (uint32_t*)B.d_count + 2;  // words 2..3 of the scalar block
  unsigned long long* d_dm = (unsigned long long*)B.d_count + 2;
  SG_CUDA(ctx, cudaMemsetAsync(B.d_count, 0, 32, ctx->stream));
  k_upd_keys<<<grid_for(count, 256), 256, 0, ctx->stream>>>(B.raw, count, g.n, B.key, B.val, d_err);
  count_launch(ctx, 3);
  SG_TRY(sort_pairs(ctx, B.key, B.key2, B.val, B.val2, count));
  // run starts
  uint8_t* flags = (uint8_t*)B.key;  // key no longer needed
  k_run_flags<<<grid_for(count, 256), 256, 0, ctx->stream>>>(B.key2, count, flags);
  k_iota_u32<<<grid_for(count, 256), 256, 0, ctx->stream>>>(B.perm, count);
  SG_TRY(select_flagged(ctx, B.perm, flags, B.grp_begin, B.d_count, count));
  uint64_t n_runs = 0;
  uint32_t h_err = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&n_runs, B.d_count, 8, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h_err) return fail(ctx, SG_ERR_INVALID, "update with vertex id >= n or bad op");
  count_launch(ctx, 4);
  k_make_actions<<<grid_for(n_runs, 256), 256, 0, ctx->stream>>>(
      B.key2, B.val2, B.grp_begin, n_runs, count, B.raw, B.a_src, B.a_dst, B.a_w, B.a_kind,
      B.a_found);
  B.n_act = n_runs;
  // applications amended by this batch (SSSP remembers its added edges)
  const SsspAmendArgs sa = sssp_amend_args(ctx);
  if (sa.active) SG_TRY(sssp_collect_adds(ctx));
  // out groups (actions sorted by (src, dst))
  SG_TRY(make_groups(ctx, B.a_src, nullptr, n_runs, B.grp_vertex, B.grp_begin, B.grp_end, &B.n_grp));
  // in groups (actions sorted by (dst, src))
  k_inv_keys<<<grid_for(n_runs, 256), 256, 0, ctx->stream>>>(B.a_src, B.a_dst, n_runs, B.key, B.val);
  SG_TRY(sort_pairs(ctx, B.key, B.key2, B.val, B.perm, n_runs));
  SG_TRY(make_groups(ctx, B.a_dst, B.perm, n_runs, B.igrp_vertex, B.igrp_begin, B.igrp_end,
                     &B.n_igrp));
  // room for the batch's worst case in each direction (repack when short)
  {
    unsigned long long* d_need = (unsigned long long*)B.d_count + 3;
    SG_TRY(ensure_pool(ctx, g.out, B.grp_vertex, B.grp_begin, B.grp_end, B.n_grp, d_need));
    SG_TRY(ensure_pool(ctx, g.in, B.igrp_vertex, B.igrp_begin, B.igrp_end, B.n_igrp, d_need));
  }
  // patch the out direction (with application amends), then the in direction
  ApplyDirArgs A{};
  A.c = g.out;
  A.gv = B.grp_vertex; A.gb = B.grp_begin; A.ge = B.grp_end; A.n_grp = B.n_grp;
  A.perm = nullptr;
  A.a_nbr = B.a_dst; A.a_w = B.a_w; A.a_kind = B.a_kind;
  A.a_found = B.a_found; A.a_pos = B.a_found; A.a_tmp = B.a_tmp;
  A.g_d0 = B.g_d0; A.g_ndel = B.g_ndel; A.g_nins = B.g_nins;
  A.chunk_off = B.chunk_off;
  A.out_dir = true;
  const PrAmendArgs pa = pr_amend_args(ctx);
  if (pa.active) { A.pr_x = pa.x; A.pr_delta = pa.delta; A.damping = pa.damping; }
  if (sa.active) {
    A.sp_parent = sa.parent; A.sp_reset = sa.reset; A.sp_seeds = sa.seeds;
    A.sp_seed_count = sa.seed_count;
  }
  A.d_dm = d_dm;
  A.d_err = d_err;
  ApplyDirArgs I = A;
  I.c = g.in;
  I.gv = B.igrp_vertex; I.gb = B.igrp_begin; I.ge = B.igrp_end; I.n_grp = B.n_igrp;
  I.perm = B.perm;
  I.a_nbr = B.a_src;
  I.a_pos = B.a_pos_in;
  I.g_d0 = B.g_d0 + B.cap; I.g_ndel = B.g_ndel + B.cap; I.g_nins = B.g_nins + B.cap;
  I.chunk_off = B.chunk_off + (B.cap + 1);
  I.out_dir = false;
  I.pr_x = nullptr; I.pr_delta = nullptr; I.sp_parent = nullptr;
  // the hub view's copy, when it reflects the adjacency before this batch in
  // the layout the batch edits (no repack above), is patched alongside
  const HubView& hv = g.hub;
  const bool patch_view = hv.col && hv.k > 0 && hv.gen == g.gen && hv.layout == g.in.layout &&
                          hv.cap == g.in.pool_cap;
  A.col2 = nullptr; A.hub_rank = nullptr; A.n = g.n;
  I.col2 = patch_view ? hv.col : nullptr;
  I.hub_rank = patch_view ? hv.rank : nullptr;
  I.n = g.n;
  // work items: ceil(degree / chunk) per group and direction
  k_apply_chunks<<<grid_for(A.n_grp + 1, 256), 256, 0, ctx->stream>>>(A, B.nch);
  SG_TRY(exclusive_sum(ctx, B.nch, B.chunk_off, A.n_grp + 1));
  k_apply_chunks<<<grid_for(I.n_grp + 1, 256), 256, 0, ctx->stream>>>(I, B.nch);
  SG_TRY(exclusive_sum(ctx, B.nch, B.chunk_off + (B.cap + 1), I.n_grp + 1));
  uint32_t nck[2] = {0, 0};
  SG_CUDA(ctx, cudaMemcpyAsync(&nck[0], B.chunk_off + A.n_grp, 4, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaMemcpyAsync(&nck[1], B.chunk_off + (B.cap + 1) + I.n_grp, 4,
                               cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  A.n_chunks = nck[0];
  I.n_chunks = nck[1];
  count_launch(ctx, 12);  // group, sort and scan kernels above
  kprof_begin(ctx);
  k_apply_find<<<grid_for(A.n_chunks * 32, 256), 256, 0, ctx->stream>>>(A);
  k_apply_find<<<grid_for(I.n_chunks * 32, 256), 256, 0, ctx->stream>>>(I);
  k_apply_group<<<grid_for(A.n_grp * 32, 256), 256, 0, ctx->stream>>>(A);
  k_apply_group<<<grid_for(I.n_grp * 32, 256), 256, 0, ctx->stream>>>(I);
  if (A.pr_x) k_apply_amend<<<grid_for(A.n_chunks * 32, 256), 256, 0, ctx->stream>>>(A);
  k_apply_finish<<<grid_for(A.n_grp * 32, 256), 256, 0, ctx->stream>>>(A);
  k_apply_finish<<<grid_for(I.n_grp * 32, 256), 256, 0, ctx->stream>>>(I);
  kprof_end(ctx, SG_K_APPLY);
  count_launch(ctx, 6);
  SG_CUDA(ctx, cudaGetLastError());
  long long dm = 0;
  SG_CUDA(ctx, cudaMemcpyAsync(&dm, d_dm, 8, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h_err) {
    g.valid = false;
    if (h_err == 3u) return fail(ctx, SG_ERR_INVALID, "applier found an inconsistent segment");
    return fail(ctx, SG_ERR_OOM, "adjacency pool exhausted while applying updates");
  }
  g.m = (uint64_t)((long long)g.m + dm);
  SG_TRY(graph_rebuild_worklists(ctx));
  SG_TRY(pr_hub_after_apply(ctx, B.igrp_vertex, B.n_igrp, patch_view));
  return SG_OK;
}

}  // namespace sg
