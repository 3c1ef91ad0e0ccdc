/*
 * og_oracle.c — CPU restatement of OneGraph's BFS / SSSP / CC / PageRank
 * (test infrastructure only: the oracle libog.so's results are compared
 * with, never the product).
 * Each function cites the reference lines it restates; declarations and the
 * parity pins are described in og_oracle.h.
 *
 * Deliberate widening: the reference walks edges with 32-bit indices
 * (e.g. BFS/cpu_BFS/main.cpp:168,171 `uint edgeIndex`), which wraps for
 * E >= 2^32.  These restatements use 64-bit edge indices; for every graph with
 * E < 2^32 the results are identical.
 */
#include "og_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define INF32 0xFFFFFFFFu

/* BFS/cpu_BFS/main.cpp:114-209 */
int ora_bfs(uint32_t V, const uint64_t *off, const uint32_t *col, uint32_t src,
            uint32_t *out) {
  unsigned char *active = (unsigned char *)calloc(V ? V : 1, 1);
  unsigned char *next = (unsigned char *)calloc(V ? V : 1, 1);
  int rounds = 0;
  for (uint32_t i = 0; i < V; i++) out[i] = INF32;
  if (src >= V) goto done;
  active[src] = 1;
  out[src] = 1;
  for (uint32_t n_active = 1; n_active > 0;) {
    for (uint32_t u = 0; u < V; u++) {
      if (!active[u]) continue;
      const uint32_t cand = out[u] + 1;
      for (uint64_t e = off[u]; e < off[u + 1]; e++) {
        const uint32_t v = col[e];
        if (cand < out[v]) {
          out[v] = cand;
          next[v] = 1;
        }
      }
    }
    n_active = 0;
    for (uint32_t i = 0; i < V; i++) {
      active[i] = next[i];
      n_active += next[i];
      next[i] = 0;
    }
    rounds++;
  }
done:
  free(active);
  free(next);
  return rounds;
}

/* CC/serial/serial.cpp:154-213 */
int ora_cc(uint32_t V, const uint64_t *off, const uint32_t *col, uint32_t *out) {
  unsigned char *active = (unsigned char *)malloc(V ? V : 1);
  unsigned char *next = (unsigned char *)calloc(V ? V : 1, 1);
  int rounds = 0;
  for (uint32_t i = 0; i < V; i++) {
    out[i] = i;
    active[i] = 1;
  }
  for (uint32_t n_active = V; n_active > 0;) {
    for (uint32_t u = 0; u < V; u++) {
      if (!active[u]) continue;
      const uint32_t label = out[u];
      for (uint64_t e = off[u]; e < off[u + 1]; e++) {
        const uint32_t v = col[e];
        if (label < out[v]) {
          out[v] = label;
          next[v] = 1;
        }
      }
    }
    n_active = 0;
    for (uint32_t i = 0; i < V; i++) {
      active[i] = next[i];
      n_active += next[i];
      next[i] = 0;
    }
    rounds++;
  }
  free(active);
  free(next);
  return rounds;
}

/* The first round of ora_cc (every vertex active, labels = ids), stopped
 * after max_edges edges; edges are read with a stride of `stride` u32 words
 * (1: columns, 2: {column, weight} pairs).  Returns the edges scanned: a
 * bounded timing sample of the serial label propagation on a large graph. */
uint64_t ora_cc_round_bounded(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                              uint64_t max_edges, uint32_t *out) {
  uint64_t scanned = 0;
  for (uint32_t i = 0; i < V; i++) out[i] = i;
  for (uint32_t u = 0; u < V && scanned < max_edges; u++) {
    const uint32_t label = out[u];
    for (uint64_t e = off[u]; e < off[u + 1]; e++) {
      const uint32_t v = edges[e * stride];
      if (label < out[v]) out[v] = label;
    }
    scanned += off[u + 1] - off[u];
  }
  return scanned;
}

/* ---- binary min-heap of (distance, vertex) with lazy deletion ---- */
typedef struct {
  uint64_t key;
  uint32_t v;
} heap_item;

typedef struct {
  heap_item *a;
  size_t n, cap;
} heap;

static void heap_push(heap *h, uint64_t key, uint32_t v) {
  if (h->n == h->cap) {
    h->cap = h->cap ? 2 * h->cap : 1024;
    h->a = (heap_item *)realloc(h->a, h->cap * sizeof(heap_item));
  }
  size_t i = h->n++;
  while (i > 0) {
    size_t p = (i - 1) / 2;
    if (h->a[p].key <= key) break;
    h->a[i] = h->a[p];
    i = p;
  }
  h->a[i].key = key;
  h->a[i].v = v;
}

static heap_item heap_pop(heap *h) {
  heap_item top = h->a[0];
  heap_item last = h->a[--h->n];
  size_t i = 0;
  for (;;) {
    size_t c = 2 * i + 1;
    if (c >= h->n) break;
    if (c + 1 < h->n && h->a[c + 1].key < h->a[c].key) c++;
    if (last.key <= h->a[c].key) break;
    h->a[i] = h->a[c];
    i = c;
  }
  if (h->n) h->a[i] = last;
  return top;
}

/* Dijkstra with the conventions of SSSP/oneGraph/GraphMeta.h:376-381 */
uint64_t ora_sssp_dijkstra_bounded(uint32_t V, const uint64_t *off,
                                   const uint32_t *edges, uint32_t src,
                                   uint64_t max_edges, uint32_t *out) {
  uint64_t scanned = 0;
  for (uint32_t i = 0; i < V; i++) out[i] = INF32;
  if (src >= V) return 0;
  heap h = {0, 0, 0};
  out[src] = 1;
  heap_push(&h, 1, src);
  while (h.n && (max_edges == 0 || scanned < max_edges)) {
    heap_item it = heap_pop(&h);
    if (it.key != out[it.v]) continue; /* stale entry */
    for (uint64_t e = off[it.v]; e < off[it.v + 1]; e++) {
      const uint32_t v = edges[2 * e];
      const uint64_t cand = it.key + edges[2 * e + 1];
      if (cand < out[v]) {
        out[v] = (uint32_t)cand;
        heap_push(&h, cand, v);
      }
    }
    scanned += off[it.v + 1] - off[it.v];
  }
  free(h.a);
  return scanned;
}

void ora_sssp_dijkstra(uint32_t V, const uint64_t *off, const uint32_t *edges,
                       uint32_t src, uint32_t *out) {
  ora_sssp_dijkstra_bounded(V, off, edges, src, 0, out);
}

/* SSSP/usm/sssp_usm.cpp:192-236 */
int ora_sssp_frontier(uint32_t V, const uint64_t *off, const uint32_t *edges,
                      uint32_t src, uint32_t *out) {
  unsigned char *active = (unsigned char *)calloc(V ? V : 1, 1);
  unsigned char *next = (unsigned char *)calloc(V ? V : 1, 1);
  int rounds = 0;
  for (uint32_t i = 0; i < V; i++) out[i] = INF32;
  if (src >= V) goto done;
  active[src] = 1;
  out[src] = 1;
  for (uint32_t n_active = 1; n_active > 0;) {
    for (uint32_t u = 0; u < V; u++) {
      if (!active[u]) continue;
      const uint32_t du = out[u];
      for (uint64_t e = off[u]; e < off[u + 1]; e++) {
        const uint32_t v = edges[2 * e];
        const uint32_t cand = du + edges[2 * e + 1];
        if (cand < out[v]) {
          out[v] = cand;
          next[v] = 1;
        }
      }
    }
    n_active = 0;
    for (uint32_t i = 0; i < V; i++) {
      active[i] = next[i];
      n_active += next[i];
      next[i] = 0;
    }
    rounds++;
  }
done:
  free(active);
  free(next);
  return rounds;
}

/* Pull sum over the in-neighbours of v (PR/cpu/pr.cpp:134-143,
 * PR/OneGraph/gpu_kernels.h:143-155): dangling sources are skipped. */
static double pull_sum(const uint64_t *off, const uint32_t *col,
                       const uint32_t *outdeg, const double *val, uint32_t v) {
  double s = 0.0;
  for (uint64_t e = off[v]; e < off[v + 1]; e++) {
    const uint32_t u = col[e];
    if (outdeg[u]) s += val[u] / outdeg[u];
  }
  return s;
}

/* PR/cpu/pr.cpp:112-124 (pr_init) + 126-165 (pr_cal<double>) */
int ora_pr_cpu(uint32_t V, const uint64_t *off, const uint32_t *col,
               const uint32_t *outdeg, double *out) {
  unsigned char *active = (unsigned char *)malloc(V ? V : 1);
  double *next = (double *)calloc(V ? V : 1, sizeof(double));
  int rounds = 0;
  for (uint32_t i = 0; i < V; i++) {
    out[i] = 1.0 / V;
    active[i] = 1;
  }
  for (uint32_t n_active = V; n_active > 0;) {
    for (uint32_t v = 0; v < V; v++)
      if (active[v]) next[v] = 0.15 + 0.15 * pull_sum(off, col, outdeg, out, v);
    for (uint32_t v = 0; v < V; v++) {
      if (!active[v]) continue;
      const double diff = fabs(next[v] - out[v]);
      out[v] = next[v];
      next[v] = 0;
      if (diff < 0.001) {
        active[v] = 0;
        n_active--;
      }
    }
    rounds++;
  }
  free(active);
  free(next);
  return rounds;
}

/* PR/OneGraph/GraphMeta.h:354-357, gpu_kernels.h:135-158 and 295-319 */
int ora_pr_onegraph(uint32_t V, const uint64_t *off, const uint32_t *col,
                    const uint32_t *outdeg, double thresh, int max_rounds,
                    double *out) {
  unsigned char *active = (unsigned char *)malloc(V ? V : 1);
  double *sum = (double *)calloc(V ? V : 1, sizeof(double));
  int rounds = 0;
  for (uint32_t i = 0; i < V; i++) {
    out[i] = 1.0;
    active[i] = 1;
  }
  for (uint32_t n_active = V; n_active > 0 && rounds < max_rounds;) {
    for (uint32_t v = 0; v < V; v++)
      if (active[v]) sum[v] = pull_sum(off, col, outdeg, out, v);
    n_active = 0;
    for (uint32_t v = 0; v < V; v++) {
      if (!active[v]) continue;
      const double nv = 0.15 + 0.85 * sum[v];
      const double diff = nv > out[v] ? nv - out[v] : out[v] - nv;
      sum[v] = 0;
      if (diff > thresh) {
        out[v] = nv;
        n_active++;
      } else {
        active[v] = 0;
      }
    }
    rounds++;
  }
  free(active);
  free(sum);
  return rounds;
}

/* FP64 precision oracle, formula of PR/usm/pr.cpp:149-187 on the normalised scale */
int ora_pr_l1(uint32_t V, const uint64_t *off, const uint32_t *col,
              const uint32_t *outdeg, double damping, double tol, int max_iter,
              double *out, double *final_l1) {
  double *next = (double *)malloc((V ? V : 1) * sizeof(double));
  const double teleport = (1.0 - damping) / V;
  double l1 = 0.0;
  int it = 0;
  for (uint32_t i = 0; i < V; i++) out[i] = 1.0 / V;
  while (it < max_iter) {
    l1 = 0.0;
    for (uint32_t v = 0; v < V; v++) {
      next[v] = teleport + damping * pull_sum(off, col, outdeg, out, v);
      l1 += fabs(next[v] - out[v]);
    }
    memcpy(out, next, (size_t)V * sizeof(double));
    it++;
    if (l1 < tol) break;
  }
  if (final_l1) *final_l1 = l1;
  free(next);
  return it;
}

/* ---- multi-threaded FP64 precision oracle ---- */
typedef struct {
  uint32_t V, b, e;
  const uint64_t *off;
  const uint32_t *col, *outdeg;
  const double *cur;
  double *next, teleport, damping, l1;
} pr_job;

static void *pr_worker(void *arg) {
  pr_job *j = (pr_job *)arg;
  double l1 = 0.0;
  for (uint32_t v = j->b; v < j->e; v++) {
    j->next[v] = j->teleport + j->damping * pull_sum(j->off, j->col, j->outdeg, j->cur, v);
    l1 += fabs(j->next[v] - j->cur[v]);
  }
  j->l1 = l1;
  return NULL;
}

int ora_pr_l1_mt(uint32_t V, const uint64_t *off, const uint32_t *col,
                 const uint32_t *outdeg, double damping, double tol, int max_iter,
                 int threads, double *out, double *final_l1) {
  if (threads < 1) threads = 1;
  double *next = (double *)malloc((V ? V : 1) * sizeof(double));
  pr_job *jobs = (pr_job *)calloc((size_t)threads, sizeof(pr_job));
  pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
  double l1 = 0.0;
  int it = 0;
  for (uint32_t i = 0; i < V; i++) out[i] = 1.0 / V;
  double *cur = out;
  while (it < max_iter) {
    for (int t = 0; t < threads; t++) {
      pr_job *j = &jobs[t];
      j->V = V;
      j->b = (uint32_t)((uint64_t)V * t / threads);
      j->e = (uint32_t)((uint64_t)V * (t + 1) / threads);
      j->off = off;
      j->col = col;
      j->outdeg = outdeg;
      j->cur = cur;
      j->next = next;
      j->teleport = (1.0 - damping) / V;
      j->damping = damping;
      pthread_create(&tid[t], NULL, pr_worker, j);
    }
    l1 = 0.0;
    for (int t = 0; t < threads; t++) {
      pthread_join(tid[t], NULL);
      l1 += jobs[t].l1;
    }
    double *tmp = cur;
    cur = next;
    next = tmp;
    it++;
    if (l1 < tol) break;
  }
  if (cur != out) {
    memcpy(out, cur, (size_t)V * sizeof(double));
    next = cur;
  }
  if (final_l1) *final_l1 = l1;
  free(next);
  free(jobs);
  free(tid);
  return it;
}

/* ---------------------------------------------------- path certificates */

typedef struct {
  uint32_t V, stride, src, unreached, b, e;
  int unit;
  const uint64_t *off;
  const uint32_t *edges, *dist;
  uint64_t bad;
  uint32_t first_bad;
} cert_job;

/* weight of edge (u, v): v searched in u's sorted list; 0 if absent */
static uint64_t cert_weight(const cert_job *j, uint32_t u, uint32_t v, int *found) {
  uint64_t lo = j->off[u], hi = j->off[(uint64_t)u + 1];
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    const uint32_t x = j->edges[mid * j->stride];
    if (x < v) lo = mid + 1;
    else hi = mid;
  }
  *found = lo < j->off[(uint64_t)u + 1] && j->edges[lo * j->stride] == v;
  if (!*found) return 0;
  return j->unit ? 1u : j->edges[lo * j->stride + 1];
}

static void *cert_worker(void *arg) {
  cert_job *j = (cert_job *)arg;
  j->bad = 0;
  j->first_bad = j->V;
  for (uint32_t u = j->b; u < j->e; u++) {
    const uint32_t du = j->dist[u];
    int ok = 1;
    if (u == j->src && du != 1) ok = 0;
    if (du != j->unreached) {
      int tight = u == j->src;
      for (uint64_t i = j->off[u]; i < j->off[(uint64_t)u + 1]; i++) {
        const uint32_t v = j->edges[i * j->stride];
        const uint64_t w = j->unit ? 1u : j->edges[i * j->stride + 1];
        const uint32_t dv = j->dist[v];
        if (dv == j->unreached || (uint64_t)dv > (uint64_t)du + w) ok = 0;  /* u -> v could improve v */
        if (!tight && dv != j->unreached) {  /* v -> u is an in-edge of u (symmetric edge set) */
          int found = 0;
          const uint64_t wvu = cert_weight(j, v, u, &found);
          if (!found) ok = 0;
          else if ((uint64_t)dv + wvu == (uint64_t)du) tight = 1;
        }
      }
      if (!tight) ok = 0;
    }
    if (!ok) {
      if (j->bad == 0) j->first_bad = u;
      j->bad++;
    }
  }
  return NULL;
}

uint64_t ora_path_certify(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                          int unit, const uint32_t *dist, uint32_t src, uint32_t unreached,
                          int threads, uint32_t *first_bad) {
  if (threads < 1) threads = 1;
  cert_job *jobs = (cert_job *)calloc((size_t)threads, sizeof(cert_job));
  pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
  uint64_t bad = 0;
  uint32_t fb = V;
  if (src >= V) bad = 1;
  for (int t = 0; t < threads && src < V; t++) {
    cert_job *j = &jobs[t];
    j->V = V;
    j->stride = stride;
    j->src = src;
    j->unreached = unreached;
    j->unit = unit;
    j->off = off;
    j->edges = edges;
    j->dist = dist;
    j->b = (uint32_t)((uint64_t)V * t / threads);
    j->e = (uint32_t)((uint64_t)V * (t + 1) / threads);
    pthread_create(&tid[t], NULL, cert_worker, j);
  }
  for (int t = 0; t < threads && src < V; t++) {
    pthread_join(tid[t], NULL);
    bad += jobs[t].bad;
    if (jobs[t].bad && fb == V) fb = jobs[t].first_bad;
  }
  free(jobs);
  free(tid);
  if (first_bad) *first_bad = fb;
  return bad;
}

/* ---------------------------------------------------- union-find components */

typedef struct {
  uint32_t V, stride;
  const uint64_t *off;
  const uint32_t *edges;
  uint32_t *par;
  uint32_t v0, v1;
  int phase;
  uint64_t roots;
} UfJob;

static uint32_t uf_find(uint32_t *par, uint32_t x) {
  for (;;) {
    const uint32_t p = __atomic_load_n(&par[x], __ATOMIC_RELAXED);
    if (p == x) return x;
    const uint32_t gp = __atomic_load_n(&par[p], __ATOMIC_RELAXED);
    if (gp != p) __atomic_compare_exchange_n(&par[x], (uint32_t *)&p, gp, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
    x = gp;
  }
}

static void *uf_worker(void *arg) {
  UfJob *j = (UfJob *)arg;
  if (j->phase == 0) {
    for (uint32_t u = j->v0; u < j->v1; u++)
      for (uint64_t e = j->off[u]; e < j->off[u + 1]; e++) {
        const uint32_t v = j->edges[e * j->stride];
        if (v <= u) continue; /* each undirected edge once */
        for (;;) {
          uint32_t ru = uf_find(j->par, u), rv = uf_find(j->par, v);
          if (ru == rv) break;
          if (ru < rv) {
            const uint32_t t = ru;
            ru = rv;
            rv = t;
          }
          uint32_t expect = ru; /* link the larger root under the smaller */
          if (__atomic_compare_exchange_n(&j->par[ru], &expect, rv, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
            break;
        }
      }
  } else {
    for (uint32_t v = j->v0; v < j->v1; v++) {  /* no link is left: roots are final */
      const uint32_t r = uf_find(j->par, v);
      __atomic_store_n(&j->par[v], r, __ATOMIC_RELAXED);
      j->roots += (r == v);
    }
  }
  return NULL;
}

uint64_t ora_cc_uf_mt(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                      int threads, uint32_t *out) {
  if (threads < 1) threads = 1;
  for (uint32_t v = 0; v < V; v++) out[v] = v;
  UfJob *jobs = (UfJob *)calloc((size_t)threads, sizeof(UfJob));
  pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
  uint64_t comps = 0;
  if (!jobs || !tid) goto done;
  for (int phase = 0; phase < 2; phase++) {
    for (int t = 0; t < threads; t++) {
      UfJob *j = &jobs[t];
      j->V = V;
      j->stride = stride;
      j->off = off;
      j->edges = edges;
      j->par = out;
      j->v0 = (uint32_t)((uint64_t)V * t / threads);
      j->v1 = (uint32_t)((uint64_t)V * (t + 1) / threads);
      j->phase = phase;
      j->roots = 0;
      pthread_create(&tid[t], NULL, uf_worker, j);
    }
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
  }
  for (int t = 0; t < threads; t++) comps += jobs[t].roots;
done:
  free(jobs);
  free(tid);
  return comps;
}

/* ------------------------------------------------ bounded CPU-baseline samples */

/* runCPUBFS (BFS/cpu_BFS/main.cpp:114-209) on `stride`-spaced columns, stopped
 * once max_edges edges were scanned (0 = no bound).  Returns the edges scanned;
 * a timing sample of the reference's CPU BFS on graphs too large to finish. */
uint64_t ora_bfs_bounded(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                         uint32_t src, uint64_t max_edges, uint32_t *out) {
  unsigned char *active = (unsigned char *)calloc(V ? V : 1, 1);
  unsigned char *next = (unsigned char *)calloc(V ? V : 1, 1);
  uint64_t scanned = 0;
  for (uint32_t i = 0; i < V; i++) out[i] = INF32;
  if (src < V && active && next) {
    active[src] = 1;
    out[src] = 1;
    for (uint32_t n_active = 1; n_active > 0 && (max_edges == 0 || scanned < max_edges);) {
      for (uint32_t u = 0; u < V && (max_edges == 0 || scanned < max_edges); u++) {
        if (!active[u]) continue;
        const uint32_t cand = out[u] + 1;
        for (uint64_t e = off[u]; e < off[u + 1]; e++) {
          const uint32_t v = edges[e * stride];
          if (cand < out[v]) {
            out[v] = cand;
            next[v] = 1;
          }
        }
        scanned += off[u + 1] - off[u];
      }
      n_active = 0;
      for (uint32_t i = 0; i < V; i++) {
        active[i] = next[i];
        n_active += next[i];
        next[i] = 0;
      }
    }
  }
  free(active);
  free(next);
  return scanned;
}

/* One pull iteration of the reference's CPU PageRank (pr_cal, PR/cpu/pr.cpp:
 * 126-165: every vertex sums rank / out-degree over its in-neighbours) on a
 * symmetric graph (in-neighbours = the adjacency, out-degree = its length),
 * `stride`-spaced columns, ranks initialised to 1/V (pr.cpp:116), stopped once
 * max_edges edges were read.  Returns the edges read; out receives the sums. */
uint64_t ora_pr_pull_bounded(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                             uint64_t max_edges, double *out) {
  double *rank = (double *)malloc((V ? V : 1) * sizeof(double));
  uint64_t scanned = 0;
  if (!rank) return 0;
  for (uint32_t i = 0; i < V; i++) rank[i] = 1.0 / V;
  for (uint32_t v = 0; v < V && (max_edges == 0 || scanned < max_edges); v++) {
    double sum = 0;
    for (uint64_t e = off[v]; e < off[v + 1]; e++) {
      const uint32_t u = edges[e * stride];
      const uint64_t d = off[u + 1] - off[u];
      if (d) sum += rank[u] / (double)d;
    }
    out[v] = 0.15 + 0.15 * sum;
    scanned += off[v + 1] - off[v];
  }
  free(rank);
  return scanned;
}
