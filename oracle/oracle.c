/*
 * CPU oracle for the GB300 SumInc workers -- TEST INFRASTRUCTURE ONLY.
 *
 * Only the test-suite, the smoke check and the bench's CPU-baseline leg call
 * into this file; the product path never does.  It restates, on the CPU, the
 * reference's algorithms for the hot path (paths relative to the SumInc
 * repository) and adds independent FP64 solvers to check against:
 *
 *   or_ingress_pr      delta-accumulative PageRank rounds as run by
 *                      SumSyncIterWorker::Query on the uncompressed graph
 *                      (grape/worker/sum_sync_iter_worker.h:857-882, isChange
 *                      :2914-2925, termCheck :2873-2912) with
 *                      PageRankIngress::g_function (pagerank_ingress.h:50-72),
 *                      init_c / init_v (:27-32).  OpenMP threads play the
 *                      reference's cilk_for; the float accumulate is an
 *                      atomic add like grape/utils/atomic_ops.h:172-179.
 *   or_pr_amend        AmendValue(-1) on the old graph followed by
 *                      AmendValue(+1) on the new one, every vertex, on all
 *                      threads (sum_sync_iter_worker.h:139-180, :289, :341).
 *   or_pr_fixed_point  FP64 Jacobi solve of x = (1-d)/N + d * P^T x with
 *                      dangling rows dropped (the fixed point the delta
 *                      iteration converges to), iterated to a tolerance.
 *   or_dijkstra        FP64 Dijkstra (binary heap); the SSSP ground truth.
 *   or_ppr_fixed_point personalised PageRank, FP64 (ppr/ppr.h:24-31 teleport).
 *   or_sssp_peval / or_sssp_inceval  the reference's plain SSSP traversal
 *                      and its incremental stage (deltaCompute), on all
 *                      threads (see the SSSP section below).
 *   or_pr_adjoint_solve FP64 solve of the transposed system for the
 *                      PageRank adjoint.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------- helpers */

static void atomic_add_f32(float* a, float b) {
#pragma omp atomic
  *a += b;
}

/* in-CSR (transpose) of an out-CSR with FP64 weights; caller frees */
static void transpose(uint32_t n, const uint64_t* rp, const uint32_t* col, const double* w,
                      uint64_t** trp, uint32_t** tcol, double** tw) {
  const uint64_t m = rp[n];
  uint64_t* r = (uint64_t*)calloc((size_t)n + 1, sizeof(uint64_t));
  uint32_t* c = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
  double* ww = w ? (double*)malloc(sizeof(double) * (m ? m : 1)) : NULL;
  for (uint64_t e = 0; e < m; ++e) r[col[e] + 1]++;
  for (uint32_t v = 0; v < n; ++v) r[v + 1] += r[v];
  uint64_t* pos = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n + 1));
  memcpy(pos, r, sizeof(uint64_t) * ((size_t)n + 1));
  for (uint32_t u = 0; u < n; ++u)
    for (uint64_t e = rp[u]; e < rp[u + 1]; ++e) {
      const uint64_t p = pos[col[e]]++;
      c[p] = u;
      if (ww) ww[p] = w[e];
    }
  free(pos);
  *trp = r;
  *tcol = c;
  if (tw) *tw = ww;
}

/* ------------------------------------------------------- PageRank (FP32) */

typedef struct {
  int32_t rounds;
  int32_t converged;
  double residual;
  uint64_t edges;
  uint64_t visits;
} or_stats;

/* Rounds of the delta iteration until sum|delta| < tau (or max_rounds).
 * init != 0 starts from init_v = 0, init_c = (1-d)/N.  threads <= 0 uses
 * every OpenMP thread. */
int or_ingress_pr(uint32_t n, const uint64_t* rp, const uint32_t* col, double damping,
                  double tau, int init, int max_rounds, int threads, float* x, float* delta,
                  or_stats* st) {
  const float d = (float)damping;
  const float thr_v = (float)(tau / (double)n);
  if (threads <= 0) threads = omp_get_max_threads();
  if (init) {
    const float c0 = (float)((1.0 - damping) / (double)n);
    for (uint32_t v = 0; v < n; ++v) {
      x[v] = 0.f;
      delta[v] = c0;
    }
  }
  int round = 0;
  double res = 0.0;
  uint64_t edges = 0, visits = 0;
  int converged = 0;
  while (round < max_rounds) {
    ++round;
    uint64_t e_round = 0, v_round = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1024) reduction(+ : e_round, v_round)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const uint32_t u = (uint32_t)i;
      float dl;
#pragma omp atomic read
      dl = delta[u];
      if (fabsf(dl) > thr_v) {
        /* atomic_exch(deltas[u], 0) */
#pragma omp atomic capture
        { dl = delta[u]; delta[u] = 0.f; }
        const uint64_t deg = rp[u + 1] - rp[u];
        if (deg > 0) {
          const float outv = dl * d / (float)deg;
          for (uint64_t e = rp[u]; e < rp[u + 1]; ++e) atomic_add_f32(&delta[col[e]], outv);
          e_round += deg;
        }
        x[u] += dl;
        v_round++;
      }
    }
    edges += e_round;
    visits += v_round;
    res = 0.0;
#pragma omp parallel for num_threads(threads) reduction(+ : res)
    for (int64_t i = 0; i < (int64_t)n; ++i) res += fabs((double)delta[i]);
    if (res < tau) {
      converged = 1;
      break;
    }
  }
  if (st) {
    st->rounds = round;
    st->converged = converged;
    st->residual = res;
    st->edges = edges;
    st->visits = visits;
  }
  return converged ? 0 : 5;
}

/* AmendValue(-1) over the old graph, AmendValue(+1) over the new graph. */
void or_pr_amend(uint32_t n, const uint64_t* rp_old, const uint32_t* col_old,
                 const uint64_t* rp_new, const uint32_t* col_new, double damping,
                 const float* x, float* delta) {
  const float d = (float)damping;
  for (int pass = 0; pass < 2; ++pass) {
    const uint64_t* rp = pass == 0 ? rp_old : rp_new;
    const uint32_t* col = pass == 0 ? col_old : col_new;
    const float sign = pass == 0 ? -1.f : 1.f;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const uint32_t u = (uint32_t)i;
      const float dl = sign * x[u];
      const uint64_t deg = rp[u + 1] - rp[u];
      if (dl == 0.f || deg == 0) continue;
      const float outv = dl * d / (float)deg;
      for (uint64_t e = rp[u]; e < rp[u + 1]; ++e) atomic_add_f32(&delta[col[e]], outv);
    }
  }
}

/* ------------------------------------------------- FP64 fixed points */

/* x = (1-d) * t + d * P^T x, P_uv = 1/outdeg(u) (or w_uv when w != NULL);
 * t = uniform 1/N when tele == NULL.  Returns iterations. */
int or_pr_fixed_point(uint32_t n, const uint64_t* rp, const uint32_t* col, const double* w,
                      double damping, const double* tele, double tol, int max_iter, double* x) {
  uint64_t* trp;
  uint32_t* tcol;
  double* tw = NULL;
  transpose(n, rp, col, w, &trp, &tcol, w ? &tw : NULL);
  double* y = (double*)malloc(sizeof(double) * n);
  double* pv = (double*)malloc(sizeof(double) * n);
  for (uint32_t v = 0; v < n; ++v) x[v] = 0.0;
  int it = 0;
  for (; it < max_iter; ++it) {
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < (int64_t)n; ++u) {
      const uint64_t deg = rp[u + 1] - rp[u];
      pv[u] = (w == NULL && deg > 0) ? damping * x[u] / (double)deg : damping * x[u];
    }
    double diff = 0.0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : diff)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      double s = tele ? (1.0 - damping) * tele[v] : (1.0 - damping) / (double)n;
      for (uint64_t e = trp[v]; e < trp[v + 1]; ++e) {
        const uint32_t u = tcol[e];
        if (w) s += pv[u] * tw[e];
        else if (rp[u + 1] > rp[u]) s += pv[u];
      }
      diff += fabs(s - x[v]);
      y[v] = s;
    }
    memcpy(x, y, sizeof(double) * n);
    if (diff < tol) {
      ++it;
      break;
    }
  }
  free(y);
  free(pv);
  free(trp);
  free(tcol);
  free(tw);
  return it;
}

/* Adjoint: lambda = g + d * P lambda, i.e. the transposed system of the
 * forward x = (1-d) t + d P^T x (weights w_uv on edge u->v).
 * lambda_u = g_u + d * sum_{v in out(u)} w_uv * lambda_v. */
int or_pr_adjoint_solve(uint32_t n, const uint64_t* rp, const uint32_t* col, const double* w,
                        double damping, const double* g, double tol, int max_iter,
                        double* lam) {
  double* y = (double*)malloc(sizeof(double) * n);
  for (uint32_t v = 0; v < n; ++v) lam[v] = 0.0;
  int it = 0;
  for (; it < max_iter; ++it) {
    double diff = 0.0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : diff)
    for (int64_t u = 0; u < (int64_t)n; ++u) {
      double s = g[u];
      for (uint64_t e = rp[u]; e < rp[u + 1]; ++e) s += damping * w[e] * lam[col[e]];
      diff += fabs(s - lam[u]);
      y[u] = s;
    }
    memcpy(lam, y, sizeof(double) * n);
    if (diff < tol) {
      ++it;
      break;
    }
  }
  free(y);
  return it;
}

/* ---------------------------------------------------------- Dijkstra */

typedef struct {
  double d;
  uint32_t v;
} heap_item;

static void heap_push(heap_item* h, uint64_t* sz, heap_item it) {
  uint64_t i = (*sz)++;
  h[i] = it;
  while (i > 0) {
    uint64_t p = (i - 1) / 2;
    if (h[p].d <= h[i].d) break;
    heap_item t = h[p];
    h[p] = h[i];
    h[i] = t;
    i = p;
  }
}

static heap_item heap_pop(heap_item* h, uint64_t* sz) {
  heap_item top = h[0];
  h[0] = h[--(*sz)];
  uint64_t i = 0;
  for (;;) {
    uint64_t l = 2 * i + 1, r = l + 1, s = i;
    if (l < *sz && h[l].d < h[s].d) s = l;
    if (r < *sz && h[r].d < h[s].d) s = r;
    if (s == i) break;
    heap_item t = h[s];
    h[s] = h[i];
    h[i] = t;
    i = s;
  }
  return top;
}

/* FP64 distances; +inf for unreachable.  Weights are summed in FP64. */
int or_dijkstra(uint32_t n, const uint64_t* rp, const uint32_t* col, const float* w,
                uint32_t source, double* dist) {
  for (uint32_t v = 0; v < n; ++v) dist[v] = INFINITY;
  if (source >= n) return 1;
  const uint64_t m = rp[n];
  heap_item* h = (heap_item*)malloc(sizeof(heap_item) * (m + 2));
  uint64_t sz = 0;
  dist[source] = 0.0;
  heap_item s0 = {0.0, source};
  heap_push(h, &sz, s0);
  while (sz) {
    heap_item it = heap_pop(h, &sz);
    if (it.d > dist[it.v]) continue;
    for (uint64_t e = rp[it.v]; e < rp[it.v + 1]; ++e) {
      const double nd = it.d + (double)w[e];
      if (nd < dist[col[e]]) {
        dist[col[e]] = nd;
        heap_item ni = {nd, col[e]};
        heap_push(h, &sz, ni);
      }
    }
  }
  free(h);
  return 0;
}

/* ------------------------------------------- SSSP traversal (the reference's)
 *
 * Label-correcting traversal as IngressSyncTraversalWorker::Query runs it for
 * SSSPIngress (grape/worker/ingress_sync_traversal_worker.h:235-330;
 * examples/analytical_apps/sssp/sssp_ingress.h:25-265): a vertex whose
 * delta improved its value relaxes its out-edges; the accumulate is an
 * atomic min of (distance, parent) packed into 8 bytes, like
 * DependencyData's SetIfLessThanAtomic (grape/utils/dependency_data.h:21-33).
 * Distances are integers (integer edge weights, as the reference's uint16
 * weights and int32 values); here 32 bits, packed above the parent, so the
 * minimum key also breaks distance ties by the smaller parent.
 *
 *   or_sssp_peval    the batch stage from a source
 *   or_sssp_inceval  deltaCompute (ingress_sync_traversal_worker.h:80-233):
 *                    reset the heads of deleted tree edges and, transitively
 *                    over the OLD graph's out-edges, every vertex whose parent
 *                    was reset; then one round in which every vertex with a
 *                    finite delta relaxes its out-edges in the NEW graph; then
 *                    the traversal until no vertex changes.
 */
#define OR_INF_KEY 0xFFFFFFFFFFFFFFFFull
#define OR_NO_PARENT 0xFFFFFFFFu

static int key_min(uint64_t* a, uint64_t k) {
  uint64_t cur = __atomic_load_n(a, __ATOMIC_RELAXED);
  while (k < cur)
    if (__atomic_compare_exchange_n(a, &cur, k, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return 1;
  return 0;
}

/* weights must be integers in [0, 2^16) */
static int int_weights(uint64_t m, const float* w, uint32_t** wi) {
  uint32_t* r = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
  for (uint64_t e = 0; e < m; ++e) {
    if (!(w[e] >= 0.f && w[e] < 65536.f) || floorf(w[e]) != w[e]) {
      free(r);
      return 1;
    }
    r[e] = (uint32_t)w[e];
  }
  *wi = r;
  return 0;
}

/* Frontier rounds from `front` until empty.  A vertex enters round r+1's
 * frontier whenever its key improves during round r (once per round, by
 * the stamp r+1), whether or not it is also in round r's frontier: a pop
 * that cleared a flag could otherwise race with an improvement and lose it
 * (the store-load pattern that weakly ordered hosts expose).  Rounds are
 * separated by the parallel loop's barrier. */
static void traverse(uint32_t n, const uint64_t* rp, const uint32_t* col, const uint32_t* w,
                     uint32_t* value, uint64_t* key, uint32_t* front, uint64_t nf, uint32_t* next,
                     uint32_t* stamp, uint32_t round, or_stats* st) {
  uint64_t edges = 0, visits = 0;
  int rounds = 0;
  (void)n;
  while (nf) {
    uint64_t nn = 0;
    const uint32_t tag = round + 1;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : edges, visits)
    for (uint64_t i = 0; i < nf; ++i) {
      const uint32_t u = front[i];
      const uint64_t k = __atomic_load_n(key + u, __ATOMIC_RELAXED);
      const uint32_t d = (uint32_t)(k >> 32);
      if (k == OR_INF_KEY || !(d < value[u])) continue;  /* CombineValueDelta */
      value[u] = d;
      ++visits;
      for (uint64_t e = rp[u]; e < rp[u + 1]; ++e) {
        const uint64_t c = (uint64_t)d + w[e];
        if (c >= 0xFFFFFFFFull) continue;
        ++edges;
        const uint32_t v = col[e];
        if (key_min(key + v, (c << 32) | u) &&
            __atomic_exchange_n(stamp + v, tag, __ATOMIC_RELAXED) != tag) {
          const uint64_t p = __atomic_fetch_add(&nn, 1, __ATOMIC_RELAXED);
          next[p] = v;
        }
      }
    }
    uint32_t* t = front;
    front = next;
    next = t;
    nf = nn;
    ++round;
    ++rounds;
  }
  st->rounds += rounds;
  st->edges += edges;
  st->visits += visits;
}

static void finish_sssp(uint32_t n, const uint32_t* value, const uint64_t* key, double* dist,
                        uint32_t* parent) {
  for (uint32_t v = 0; v < n; ++v) {
    const uint32_t kd = key[v] == OR_INF_KEY ? 0xFFFFFFFFu : (uint32_t)(key[v] >> 32);
    const uint32_t d = value[v] < kd ? value[v] : kd;
    dist[v] = d == 0xFFFFFFFFu ? INFINITY : (double)d;
    parent[v] = key[v] == OR_INF_KEY ? OR_NO_PARENT : (uint32_t)key[v];
  }
}

int or_sssp_peval(uint32_t n, const uint64_t* rp, const uint32_t* col, const float* w,
                  uint32_t source, int threads, double* dist, uint32_t* parent, or_stats* st) {
  if (source >= n) return 1;
  if (threads > 0) omp_set_num_threads(threads);
  uint32_t* wi = NULL;
  if (int_weights(rp[n], w, &wi)) return 2;
  uint32_t* value = (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * n);
  uint32_t* f0 = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  uint32_t* f1 = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  uint32_t* stamp = (uint32_t*)calloc(n, sizeof(uint32_t));
  for (uint32_t v = 0; v < n; ++v) {
    value[v] = 0xFFFFFFFFu;
    key[v] = OR_INF_KEY;
  }
  key[source] = ((uint64_t)0 << 32) | OR_NO_PARENT;
  f0[0] = source;
  stamp[source] = 1;
  memset(st, 0, sizeof(*st));
  traverse(n, rp, col, wi, value, key, f0, 1, f1, stamp, 1, st);
  st->converged = 1;
  finish_sssp(n, value, key, dist, parent);
  free(wi); free(value); free(key); free(f0); free(f1); free(stamp);
  return 0;
}

int or_sssp_inceval(uint32_t n, const uint64_t* rp_old, const uint32_t* col_old,
                    const uint64_t* rp, const uint32_t* col, const float* w, uint64_t n_del,
                    const uint32_t* del_src, const uint32_t* del_dst, int threads, double* dist,
                    uint32_t* parent, or_stats* st) {
  if (threads > 0) omp_set_num_threads(threads);
  uint32_t* wi = NULL;
  if (int_weights(rp[n], w, &wi)) return 2;
  uint32_t* value = (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * n);
  uint32_t* f0 = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  uint32_t* f1 = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  uint8_t* inq = (uint8_t*)calloc(n, 1);     /* reset marks */
  uint32_t* stamp = (uint32_t*)calloc(n, sizeof(uint32_t));
  for (uint32_t v = 0; v < n; ++v) {
    const int fin = isfinite(dist[v]);
    value[v] = fin ? (uint32_t)dist[v] : 0xFFFFFFFFu;
    key[v] = fin ? (((uint64_t)value[v] << 32) | parent[v]) : OR_INF_KEY;
  }
  memset(st, 0, sizeof(*st));
  /* deltaCompute: heads of deleted tree edges, then their tree descendants
   * over the old out-edges, reset to the identity */
  uint64_t nf = 0;
  for (uint64_t i = 0; i < n_del; ++i) {
    const uint32_t u = del_src[i], v = del_dst[i];
    if (u < n && v < n && key[v] != OR_INF_KEY && (uint32_t)key[v] == u && !inq[v]) {
      inq[v] = 1;
      f0[nf++] = v;
    }
  }
  uint64_t n_reset = 0;
  while (nf) {
    uint64_t nn = 0;
    for (uint64_t i = 0; i < nf; ++i) {
      const uint32_t u = f0[i];
      for (uint64_t e = rp_old[u]; e < rp_old[u + 1]; ++e) {
        const uint32_t v = col_old[e];
        if (key[v] != OR_INF_KEY && (uint32_t)key[v] == u && !inq[v]) {
          inq[v] = 1;
          f1[nn++] = v;
        }
      }
    }
    for (uint64_t i = 0; i < nf; ++i) {
      value[f0[i]] = 0xFFFFFFFFu;
      key[f0[i]] = OR_INF_KEY;
    }
    n_reset += nf;
    uint32_t* t = f0;
    f0 = f1;
    f1 = t;
    nf = nn;
  }
  /* one round from every vertex with a finite delta, over the new graph;
   * improved vertices form the traversal's first frontier (stamp 1) */
  uint64_t nn = 0, edges = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : edges)
  for (uint32_t u = 0; u < n; ++u) {
    const uint64_t k = key[u];
    if (k == OR_INF_KEY) continue;
    const uint32_t d = (uint32_t)(k >> 32);
    for (uint64_t e = rp[u]; e < rp[u + 1]; ++e) {
      const uint64_t c = (uint64_t)d + wi[e];
      if (c >= 0xFFFFFFFFull) continue;
      ++edges;
      const uint32_t v = col[e];
      if (key_min(key + v, (c << 32) | u) && __atomic_exchange_n(stamp + v, 1u, __ATOMIC_RELAXED) != 1u) {
        const uint64_t p = __atomic_fetch_add(&nn, 1, __ATOMIC_RELAXED);
        f1[p] = v;
      }
    }
  }
  st->edges += edges;
  traverse(n, rp, col, wi, value, key, f1, nn, f0, stamp, 1, st);
  st->converged = 1;
  st->residual = (double)n_reset;  /* reset vertices */
  finish_sssp(n, value, key, dist, parent);
  free(wi); free(value); free(key); free(f0); free(f1); free(inq); free(stamp);
  return 0;
}
