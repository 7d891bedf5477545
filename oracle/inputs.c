/*
 * Input generation and checks for the CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * The tests, the smoke check and the bench's CPU legs call into this file;
 * the product path never does.  It lets the CPU side of a comparison build
 * its inputs without loading the library under test:
 *
 *   or_rmat            the seeded R-MAT graph: draw i of a counter-based
 *                      splitmix64 stream descends `scale` quadrant levels
 *                      (Chakrabarti, Zhan, Faloutsos, SDM 2004; no noise, no
 *                      permutation); self loops are skipped and the graph is
 *                      the first `edges` distinct pairs in draw order, rows
 *                      sorted.  Same draw rule as the library's generators, so
 *                      a test can check that both give the same graph.
 *   or_gen_updates     an update batch valid for a graph: deletes of
 *                      uniformly chosen existing edges, re-weights (a delete
 *                      plus an add of the same pair, the form the reference's
 *                      update files need, inc_fragment_builder.h:38-70) and
 *                      inserts of absent uniform pairs, drawn from one
 *                      counter-based stream per batch.
 *   or_apply_updates   the reference's batch semantics
 *                      (IncFragmentBuilder::Init / Build,
 *                      inc_fragment_builder.h:29-133): the first add of a pair
 *                      wins, an add of an existing pair replaces it, a delete
 *                      of an absent pair is ignored.
 *   or_pr_residual_l1  || (1-d)/N + d P^T x - x ||_1 in FP64 for a given x;
 *                      with dangling rows dropped, ||x - x*||_1 is at most
 *                      that residual / (1 - d), an accuracy bound that needs
 *                      no fixed-point solve.
 *
 * All loops are OpenMP; results do not depend on the thread count.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* ------------------------------------------------------------- R-MAT */

typedef struct {
  uint64_t key;
  uint32_t ta, tab, tabc;
  int scale;
} rmat_params;

static rmat_params rmat_make(int scale, double a, double b, double c, uint64_t seed) {
  rmat_params p;
  p.key = mix64(seed ^ 0x5851F42D4C957F2Dull);
  p.ta = (uint32_t)(a * 16777216.0);
  p.tab = (uint32_t)((a + b) * 16777216.0);
  p.tabc = (uint32_t)((a + b + c) * 16777216.0);
  p.scale = scale;
  return p;
}

/* draw i: two 24-bit uniforms per 64-bit hash, most significant level first;
 * returns (src << 32) | dst */
static uint64_t rmat_edge(const rmat_params* p, uint64_t i) {
  uint32_t s = 0, d = 0;
  uint64_t h = 0;
  for (int l = 0; l < p->scale; ++l) {
    uint32_t r;
    if ((l & 1) == 0) {
      h = mix64(p->key + i * 32u + (uint64_t)(l >> 1));
      r = (uint32_t)(h >> 40);
    } else {
      r = (uint32_t)((h >> 16) & 0xFFFFFFu);
    }
    const uint32_t sb = r >= p->tab, db = (r >= p->ta && r < p->tab) || r >= p->tabc;
    s = (s << 1) | sb;
    d = (d << 1) | db;
  }
  return ((uint64_t)s << 32) | d;
}

/* weight of edge (s, t): a pure function of the weight seed and the pair */
static float rmat_weight(uint64_t wkey, int kind, double lo, double hi, uint64_t pair) {
  const uint64_t h = mix64(wkey ^ pair);
  if (kind == 1) return (float)(lo + (double)(h % (uint64_t)(hi - lo + 1.0)));
  const double u = (double)(h >> 40) * (1.0 / 16777216.0);
  volatile double prod = (hi - lo) * u;
  return (float)(lo + prod);
}

static void atomic_min_u32(uint32_t* a, uint32_t v) {
  uint32_t cur = __atomic_load_n(a, __ATOMIC_RELAXED);
  while (v < cur && !__atomic_compare_exchange_n(a, &cur, v, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
}

static int cmp_u32(const void* a, const void* b) {
  const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return (x > y) - (x < y);
}

/* The first `edges` distinct non-loop pairs of the draw stream.  The set of
 * distinct pairs among the first T draws does not depend on the order in
 * which draws are inserted, so the draws go into a concurrent hash table
 * that keeps each pair's smallest draw index; the graph is the pairs whose
 * smallest index is among the `edges` smallest.  Returns 0, or 1 when the
 * arguments are invalid, 2 when memory runs out. */
int or_rmat(int scale, uint64_t edges, double a, double b, double c, uint64_t seed,
            int weight_kind, double wlo, double whi, uint64_t* rp, uint32_t* col, float* w) {
  if (scale < 1 || scale > 30 || !rp || !col) return 1;
  const uint64_t n = 1ull << scale;
  if (edges > n * (n - 1) || edges >= (1ull << 31)) return 1;
  const rmat_params p = rmat_make(scale, a, b, c, seed);
  uint64_t M = edges + edges / 3 + 1024;
  for (int attempt = 0; attempt < 12; ++attempt) {
    uint64_t cap = 1024;
    while (cap < 2 * M) cap <<= 1;
    const uint64_t mask = cap - 1;
    uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * cap);
    uint32_t* first = (uint32_t*)malloc(sizeof(uint32_t) * cap);
    const uint64_t words = (M + 63) / 64;
    uint64_t* mark = (uint64_t*)calloc(words, sizeof(uint64_t));
    if (!key || !first || !mark || M >= 0xFFFFFFFFull) {
      free(key);
      free(first);
      free(mark);
      return 2;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)cap; ++i) {
      key[i] = ~0ull;
      first[i] = 0xFFFFFFFFu;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)M; ++i) {
      const uint64_t e = rmat_edge(&p, (uint64_t)i);
      const uint32_t s = (uint32_t)(e >> 32), t = (uint32_t)e;
      if (s == t) continue;
      const uint64_t k = ((uint64_t)s << scale) | t;
      uint64_t h = mix64(k) & mask;
      for (;;) {
        uint64_t cur = __atomic_load_n(&key[h], __ATOMIC_RELAXED);
        if (cur == ~0ull) {
          uint64_t expect = ~0ull;
          if (__atomic_compare_exchange_n(&key[h], &expect, k, 0, __ATOMIC_RELAXED,
                                          __ATOMIC_RELAXED))
            cur = k;
          else
            cur = expect;
        }
        if (cur == k) {
          atomic_min_u32(&first[h], (uint32_t)i);
          break;
        }
        h = (h + 1) & mask;
      }
    }
    /* the smallest draw index of every distinct pair, as a bitmap over draws */
#pragma omp parallel for schedule(static)
    for (int64_t h = 0; h < (int64_t)cap; ++h)
      if (key[h] != ~0ull) __atomic_fetch_or(&mark[first[h] >> 6], 1ull << (first[h] & 63),
                                             __ATOMIC_RELAXED);
    uint64_t total = 0;
#pragma omp parallel for reduction(+ : total)
    for (int64_t i = 0; i < (int64_t)words; ++i) total += (uint64_t)__builtin_popcountll(mark[i]);
    if (total < edges) {
      free(key);
      free(first);
      free(mark);
      const double ratio = (double)edges / (double)(total ? total : 1);
      M = (uint64_t)((double)M * ratio * 1.08) + 4096;
      continue;
    }
    /* T = draw index of the edges-th first occurrence */
    uint64_t limit = 0;
    if (edges > 0) {
      uint64_t seen = 0, wi = 0;
      while (seen + (uint64_t)__builtin_popcountll(mark[wi]) < edges) {
        seen += (uint64_t)__builtin_popcountll(mark[wi]);
        ++wi;
      }
      uint64_t bits = mark[wi];
      while (1) {
        const int bpos = __builtin_ctzll(bits);
        if (++seen == edges) {
          limit = wi * 64 + (uint64_t)bpos;
          break;
        }
        bits &= bits - 1;
      }
    }
    free(mark);
    /* rows: counts, offsets, fills, then a sort of each row */
    memset(rp, 0, sizeof(uint64_t) * (n + 1));
#pragma omp parallel for schedule(static)
    for (int64_t h = 0; h < (int64_t)cap; ++h)
      if (key[h] != ~0ull && edges > 0 && first[h] <= limit)
        __atomic_fetch_add(&rp[(key[h] >> scale) + 1], 1ull, __ATOMIC_RELAXED);
    for (uint64_t v = 0; v < n; ++v) rp[v + 1] += rp[v];
    uint64_t* pos = (uint64_t*)malloc(sizeof(uint64_t) * n);
    if (!pos) {
      free(key);
      free(first);
      return 2;
    }
    memcpy(pos, rp, sizeof(uint64_t) * n);
    const uint64_t dmask = n - 1;
#pragma omp parallel for schedule(static)
    for (int64_t h = 0; h < (int64_t)cap; ++h)
      if (key[h] != ~0ull && edges > 0 && first[h] <= limit) {
        const uint64_t s = key[h] >> scale;
        const uint64_t at = __atomic_fetch_add(&pos[s], 1ull, __ATOMIC_RELAXED);
        col[at] = (uint32_t)(key[h] & dmask);
      }
    free(pos);
    free(key);
    free(first);
    const uint64_t wkey = mix64(seed ^ 0xD1B54A32D192ED03ull);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      const uint64_t rb = rp[v], re = rp[v + 1];
      if (re - rb > 1) qsort(col + rb, re - rb, sizeof(uint32_t), cmp_u32);
      if (w && weight_kind != 0)
        for (uint64_t e = rb; e < re; ++e)
          w[e] = rmat_weight(wkey, weight_kind, wlo, whi, ((uint64_t)v << 32) | col[e]);
    }
    return 0;
  }
  return 1;
}

/* ----------------------------------------------------------- updates */

/* sg_update layout: u32 src, u32 dst, f32 weight, u32 op (0 add, 1 delete) */
typedef struct {
  uint32_t src, dst;
  float w;
  uint32_t op;
} or_update;

/* open-addressing set of (src << 32 | dst) keys */
typedef struct {
  uint64_t* slot;
  uint64_t mask;
} pair_set;

static int pset_init(pair_set* s, uint64_t want) {
  uint64_t cap = 64;
  while (cap < 2 * want + 16) cap <<= 1;
  s->slot = (uint64_t*)malloc(sizeof(uint64_t) * cap);
  if (!s->slot) return 0;
  memset(s->slot, 0xFF, sizeof(uint64_t) * cap);
  s->mask = cap - 1;
  return 1;
}

/* inserts k; returns 1 when it was absent */
static int pset_insert(pair_set* s, uint64_t k) {
  uint64_t h = mix64(k) & s->mask;
  while (s->slot[h] != ~0ull) {
    if (s->slot[h] == k) return 0;
    h = (h + 1) & s->mask;
  }
  s->slot[h] = k;
  return 1;
}

static int row_has(const uint64_t* rp, const uint32_t* col, uint32_t u, uint32_t v) {
  uint64_t lo = rp[u], hi = rp[u + 1];
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (col[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo < rp[u + 1] && col[lo] == v;
}

/* One batch for the graph (rp, col) with rows sorted: n_del deletes of
 * uniformly chosen distinct edges, n_rew re-weights (delete + add, new weight
 * drawn), n_ins inserts of distinct absent non-loop pairs, in that order, from
 * the stream mix64(key0 + counter) with key0 = mix64(seed ^ const).  Weights:
 * integer U[wlo, whi] or float U[wlo, whi].  Writes n_del + 2 n_rew + n_ins
 * records.  Returns 0, 1 on invalid sizes, 2 without memory. */
int or_gen_updates(uint32_t n, const uint64_t* rp, const uint32_t* col, uint64_t n_ins,
                   uint64_t n_del, uint64_t n_rew, uint64_t seed, int integer_weights,
                   double wlo, double whi, or_update* out) {
  const uint64_t m = rp[n];
  if (n_del + n_rew > m) return 1;
  if (n_ins > (uint64_t)n * (n - 1) - m) return 1;
  const uint64_t key0 = mix64(seed ^ 0xA0761D6478BD642Full);
  uint64_t ctr = 0;
  pair_set chosen;
  if (!pset_init(&chosen, n_ins + n_del + n_rew)) return 2;
#define OR_RND() mix64(key0 + (ctr++))
  uint64_t o = 0;
  /* deletes */
  for (uint64_t k = 0; k < n_del;) {
    const uint64_t r = OR_RND() % m;
    /* the row holding entry r: last v with rp[v] <= r */
    uint64_t lo = 0, hi = n;
    while (hi - lo > 1) {
      const uint64_t mid = (lo + hi) / 2;
      if (rp[mid] <= r) lo = mid;
      else hi = mid;
    }
    const uint32_t u = (uint32_t)lo, v = col[r];
    if (pset_insert(&chosen, ((uint64_t)u << 32) | v)) {
      out[o++] = (or_update){u, v, 0.f, 1u};
      ++k;
    }
  }
  /* re-weights: the delete now, the add after every delete of the batch */
  or_update* rew = n_rew ? (or_update*)malloc(sizeof(or_update) * n_rew) : NULL;
  if (n_rew && !rew) {
    free(chosen.slot);
    return 2;
  }
  for (uint64_t k = 0; k < n_rew;) {
    const uint64_t r = OR_RND() % m;
    uint64_t lo = 0, hi = n;
    while (hi - lo > 1) {
      const uint64_t mid = (lo + hi) / 2;
      if (rp[mid] <= r) lo = mid;
      else hi = mid;
    }
    const uint32_t u = (uint32_t)lo, v = col[r];
    if (pset_insert(&chosen, ((uint64_t)u << 32) | v)) {
      const uint64_t h = OR_RND();
      float wn;
      if (integer_weights) {
        wn = (float)(wlo + (double)(h % (uint64_t)(whi - wlo + 1.0)));
      } else {
        volatile double prod = (whi - wlo) * ((double)(h >> 40) * (1.0 / 16777216.0));
        wn = (float)(wlo + prod);
      }
      rew[k++] = (or_update){u, v, wn, 0u};
    }
  }
  for (uint64_t k = 0; k < n_rew; ++k) {
    out[o++] = (or_update){rew[k].src, rew[k].dst, 0.f, 1u};
    out[o++] = rew[k];
  }
  free(rew);
  /* inserts */
  for (uint64_t k = 0; k < n_ins;) {
    const uint32_t u = (uint32_t)(OR_RND() % n);
    const uint32_t v = (uint32_t)(OR_RND() % n);
    if (u == v || row_has(rp, col, u, v)) continue;
    if (pset_insert(&chosen, ((uint64_t)u << 32) | v)) {
      const uint64_t h = OR_RND();
      float wn;
      if (integer_weights) {
        wn = (float)(wlo + (double)(h % (uint64_t)(whi - wlo + 1.0)));
      } else {
        volatile double prod = (whi - wlo) * ((double)(h >> 40) * (1.0 / 16777216.0));
        wn = (float)(wlo + prod);
      }
      out[o++] = (or_update){u, v, wn, 0u};
      ++k;
    }
  }
#undef OR_RND
  free(chosen.slot);
  return 0;
}

/* ------------------------------------------------------- batch apply */

typedef struct {
  uint64_t pair; /* src << 32 | dst */
  uint64_t idx;  /* position in the batch */
  float w;
  uint32_t op;
} tagged_update;

static int cmp_tagged(const void* a, const void* b) {
  const tagged_update* x = (const tagged_update*)a;
  const tagged_update* y = (const tagged_update*)b;
  if (x->pair != y->pair) return x->pair < y->pair ? -1 : 1;
  return (x->idx > y->idx) - (x->idx < y->idx);
}

/* one entry per touched pair: present after the batch (first add's weight)
 * or removed */
typedef struct {
  uint64_t pair;
  float w;
  int present;
} pair_effect;

static pair_effect* batch_effects(const or_update* upd, uint64_t cnt, uint32_t n, uint64_t* n_eff) {
  tagged_update* t = (tagged_update*)malloc(sizeof(tagged_update) * (cnt ? cnt : 1));
  pair_effect* e = (pair_effect*)malloc(sizeof(pair_effect) * (cnt ? cnt : 1));
  if (!t || !e) {
    free(t);
    free(e);
    return NULL;
  }
  uint64_t k = 0;
  for (uint64_t i = 0; i < cnt; ++i) {
    if (upd[i].src >= n || upd[i].dst >= n || upd[i].op > 1u) continue;
    t[k++] = (tagged_update){((uint64_t)upd[i].src << 32) | upd[i].dst, i, upd[i].w, upd[i].op};
  }
  qsort(t, k, sizeof(tagged_update), cmp_tagged);
  uint64_t ne = 0;
  for (uint64_t i = 0; i < k;) {
    uint64_t j = i;
    int has_add = 0;
    float w = 0.f;
    for (; j < k && t[j].pair == t[i].pair; ++j)
      if (t[j].op == 0u && !has_add) {
        has_add = 1;
        w = t[j].w;
      }
    e[ne++] = (pair_effect){t[i].pair, w, has_add};
    i = j;
  }
  free(t);
  *n_eff = ne;
  return e;
}

/* The graph after the batch.  Rows of (rp, col[, w]) sorted by destination;
 * the result's rows too.  With col_new == NULL only rp_new[n + 1] is
 * written.  Records with an id >= n or an unknown op are skipped.  Returns 0,
 * or 2 without memory. */
int or_apply_updates(uint32_t n, const uint64_t* rp, const uint32_t* col, const float* w,
                     const or_update* upd, uint64_t cnt, uint64_t* rp_new, uint32_t* col_new,
                     float* w_new) {
  uint64_t ne = 0;
  pair_effect* e = batch_effects(upd, cnt, n, &ne);
  if (!e) return 2;
  /* effects of each row: [eb[u], eb[u + 1]) */
  uint64_t* eb = (uint64_t*)calloc((size_t)n + 1, sizeof(uint64_t));
  if (!eb) {
    free(e);
    return 2;
  }
  for (uint64_t i = 0; i < ne; ++i) eb[(e[i].pair >> 32) + 1]++;
  for (uint32_t v = 0; v < n; ++v) eb[v + 1] += eb[v];
  /* row sizes: old entries untouched by the batch plus present pairs */
  rp_new[0] = 0;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t vv = 0; vv < (int64_t)n; ++vv) {
    const uint32_t v = (uint32_t)vv;
    uint64_t size = rp[v + 1] - rp[v];
    for (uint64_t i = eb[v]; i < eb[v + 1]; ++i) {
      const uint32_t d = (uint32_t)e[i].pair;
      size -= (uint64_t)row_has(rp, col, v, d);
      size += (uint64_t)e[i].present;
    }
    rp_new[v + 1] = size;
  }
  for (uint32_t v = 0; v < n; ++v) rp_new[v + 1] += rp_new[v];
  if (col_new) {
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t vv = 0; vv < (int64_t)n; ++vv) {
      const uint32_t v = (uint32_t)vv;
      uint64_t a = rp[v], o = rp_new[v];
      const uint64_t ae = rp[v + 1];
      uint64_t i = eb[v];
      const uint64_t ie = eb[v + 1];
      if (i == ie) {
        memcpy(col_new + o, col + a, sizeof(uint32_t) * (ae - a));
        if (w_new) {
          if (w) memcpy(w_new + o, w + a, sizeof(float) * (ae - a));
          else for (uint64_t k = 0; k < ae - a; ++k) w_new[o + k] = 1.f;
        }
        continue;
      }
      /* merge: old entries not touched, touched pairs that stay present */
      while (a < ae || i < ie) {
        const uint32_t od = a < ae ? col[a] : 0xFFFFFFFFu;
        const uint32_t ed = i < ie ? (uint32_t)e[i].pair : 0xFFFFFFFFu;
        if (a < ae && (i >= ie || od < ed)) {
          col_new[o] = od;
          if (w_new) w_new[o] = w ? w[a] : 1.f;
          ++o;
          ++a;
        } else {
          if (a < ae && od == ed) ++a; /* the old edge is replaced or removed */
          if (e[i].present) {
            col_new[o] = ed;
            if (w_new) w_new[o] = e[i].w;
            ++o;
          }
          ++i;
        }
      }
    }
  }
  free(eb);
  free(e);
  return 0;
}

/* ------------------------------------------------ PageRank residual */

/* res = sum_v | (1-d)/N + d * sum_{u -> v} x_u / outdeg(u) - x_v |, FP64.
 * The in-edge sums are formed over a transpose built with atomic counters. */
int or_pr_residual_l1(uint32_t n, const uint64_t* rp, const uint32_t* col, double damping,
                      const float* x, double* res) {
  const uint64_t m = rp[n];
  uint64_t* trp = (uint64_t*)calloc((size_t)n + 1, sizeof(uint64_t));
  uint32_t* tcol = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
  double* pv = (double*)malloc(sizeof(double) * ((size_t)n ? n : 1));
  if (!trp || !tcol || !pv) {
    free(trp);
    free(tcol);
    free(pv);
    return 2;
  }
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < (int64_t)m; ++e)
    __atomic_fetch_add(&trp[col[e] + 1], 1ull, __ATOMIC_RELAXED);
  for (uint32_t v = 0; v < n; ++v) trp[v + 1] += trp[v];
  uint64_t* pos = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n ? n : 1));
  if (!pos) {
    free(trp);
    free(tcol);
    free(pv);
    return 2;
  }
  memcpy(pos, trp, sizeof(uint64_t) * n);
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    const uint64_t deg = rp[u + 1] - rp[u];
    pv[u] = deg ? damping * (double)x[u] / (double)deg : 0.0;
    for (uint64_t e = rp[u]; e < rp[u + 1]; ++e)
      tcol[__atomic_fetch_add(&pos[col[e]], 1ull, __ATOMIC_RELAXED)] = (uint32_t)u;
  }
  free(pos);
  const double c0 = (1.0 - damping) / (double)n;
  double r = 0.0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : r)
  for (int64_t v = 0; v < (int64_t)n; ++v) {
    double s = c0;
    for (uint64_t e = trp[v]; e < trp[v + 1]; ++e) s += pv[tcol[e]];
    r += fabs(s - (double)x[v]);
  }
  free(trp);
  free(tcol);
  free(pv);
  *res = r;
  return 0;
}
