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
