/*
 * og_oracle_rmat.c — the benchmark graphs rebuilt on the CPU, for the CPU
 * baselines and the reference arm of bench.py (test infrastructure only).
 *
 * The reference ships no graph generator (README.md:8 points at an external
 * converter), so the workloads are seeded R-MAT graphs (Chakrabarti, Zhan and
 * Faloutsos, 2004).  This file restates the draw used by the engine's own
 * generator from its definition, so that a process that must not load the
 * engine (the reference arm) builds the identical CSR:
 *  - tuple i: a 64-bit base hash of (seed, i), then `scale` quadrant choices,
 *    two per 64-bit hash, each a 32-bit value compared with the cumulative
 *    thresholds a, a+b, a+b+c scaled to 2^32 (row bit set in quadrants c/d,
 *    column bit set in quadrants b/d);
 *  - hashes are the splitmix64 finaliser (Steele, Lea and Flood, 2014);
 *  - vertex ids optionally pass a seeded bijection of [0, 2^scale): three
 *    rounds of odd multiply, xor-shift by ceil(scale/2), add, modulo 2^scale;
 *  - self-loops are dropped; a symmetric graph adds the reverse of every
 *    tuple; duplicates are removed; rows and the columns of a row are sorted;
 *  - the weight of {u, v} hashes (weight seed, min(u,v), max(u,v)) into
 *    [wmin, wmax], the same in both directions;
 *  - a PageRank graph is directed and stored by in-edges (row = target) with
 *    the out-degree of every vertex.
 * The pipeline is independent of the engine's: count tuples per row, scatter
 * columns into rows, sort and deduplicate every row, compact.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "og_oracle.h"

static uint64_t ora_mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

typedef struct {
  uint32_t scale, t1, t2, t3;
  uint64_t seed, mul[3], add[3];
  int permute;
} Draw;

static uint32_t thr32(double p) {
  if (p <= 0) return 0;
  if (p >= 1) return 0xFFFFFFFFu;
  return (uint32_t)(p * 4294967296.0);
}

static uint32_t draw_perm(const Draw *d, uint32_t x) {
  const uint64_t mask = (1ull << d->scale) - 1;
  const uint32_t sh = (d->scale + 1) / 2;
  uint64_t y = x;
  for (int r = 0; r < 3; r++) {
    y = (y * d->mul[r]) & mask;
    y ^= y >> sh;
    y = (y + d->add[r]) & mask;
  }
  return (uint32_t)y;
}

static void draw_tuple(const Draw *d, uint64_t i, uint32_t *u, uint32_t *v) {
  const uint64_t base = ora_mix64(d->seed + (i + 1) * 0x9e3779b97f4a7c15ull);
  uint32_t row = 0, col = 0;
  uint64_t h = 0;
  for (uint32_t l = 0; l < d->scale; l++) {
    const uint32_t r = (l & 1) ? (uint32_t)(h >> 32)
                               : (uint32_t)(h = ora_mix64(base + (uint64_t)(l + 1) * 0xd1b54a32d192ed03ull));
    row = (row << 1) | (r >= d->t2);
    col = (col << 1) | ((r >= d->t1 && r < d->t2) || r >= d->t3);
  }
  if (d->permute) {
    row = draw_perm(d, row);
    col = draw_perm(d, col);
  }
  *u = row;
  *v = col;
}

static uint32_t ora_weight(uint64_t wseed, uint32_t u, uint32_t v, uint32_t wmin, uint32_t wmax) {
  const uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
  const uint64_t h = ora_mix64(wseed ^ ora_mix64((lo << 32) | hi));
  return wmin + (uint32_t)(h % ((uint64_t)wmax - wmin + 1));
}

typedef struct {
  const Draw *d;
  uint64_t t0, t1;      /* tuple range */
  uint32_t v0, v1;      /* row range (sort / compact phases) */
  int sym, pr, phase;
  uint32_t *cnt;        /* per-row tuple counts (phase 0), then scatter cursors (phase 1) */
  uint64_t *start;      /* raw row starts (V+1) */
  uint32_t *raw;        /* raw columns */
  uint32_t *uniq;       /* unique columns per row (phase 2) */
} Job;

static void put(Job *j, uint32_t row, uint32_t col) {
  if (j->phase == 0) {
    __atomic_fetch_add(&j->cnt[row], 1u, __ATOMIC_RELAXED);
  } else {
    const uint32_t k = __atomic_fetch_add(&j->cnt[row], 1u, __ATOMIC_RELAXED);
    j->raw[j->start[row] + k] = col;
  }
}

static int cmp_u32(const void *a, const void *b) {
  const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return x < y ? -1 : x > y;
}

static void *worker(void *arg) {
  Job *j = (Job *)arg;
  if (j->phase <= 1) {
    for (uint64_t i = j->t0; i < j->t1; i++) {
      uint32_t u, v;
      draw_tuple(j->d, i, &u, &v);
      if (u == v) continue;
      if (j->pr) {
        put(j, v, u); /* in-edge CSR: row = target */
      } else {
        put(j, u, v);
        if (j->sym) put(j, v, u);
      }
    }
  } else {
    for (uint32_t r = j->v0; r < j->v1; r++) {
      uint32_t *c = j->raw + j->start[r];
      const uint64_t n = j->start[r + 1] - j->start[r];
      if (n < 2) {
        j->uniq[r] = (uint32_t)n;
        continue;
      }
      if (n <= 32) {
        for (uint64_t a = 1; a < n; a++) {
          const uint32_t x = c[a];
          uint64_t b = a;
          for (; b > 0 && c[b - 1] > x; b--) c[b] = c[b - 1];
          c[b] = x;
        }
      } else {
        qsort(c, n, 4, cmp_u32);
      }
      uint64_t m = 1;
      for (uint64_t a = 1; a < n; a++)
        if (c[a] != c[m - 1]) c[m++] = c[a];
      j->uniq[r] = (uint32_t)m;
    }
  }
  return NULL;
}

typedef struct {
  uint32_t v0, v1, weighted, pr, wmin, wmax;
  uint64_t wseed;
  const uint64_t *start, *off;
  const uint32_t *raw;
  uint32_t *edges, *outdeg;
} Fill;

static void *fill_worker(void *arg) {
  Fill *f = (Fill *)arg;
  for (uint32_t r = f->v0; r < f->v1; r++) {
    const uint32_t *c = f->raw + f->start[r];
    const uint64_t n = f->off[r + 1] - f->off[r];
    for (uint64_t a = 0; a < n; a++) {
      const uint64_t e = f->off[r] + a;
      if (f->weighted) {
        f->edges[2 * e] = c[a];
        f->edges[2 * e + 1] = ora_weight(f->wseed, r, c[a], f->wmin, f->wmax);
      } else {
        f->edges[e] = c[a];
      }
      if (f->pr) __atomic_fetch_add(&f->outdeg[c[a]], 1u, __ATOMIC_RELAXED);
    }
  }
  return NULL;
}

static int run_jobs(int nt, void *(*fn)(void *), void *jobs, size_t stride) {
  pthread_t *tid = (pthread_t *)calloc((size_t)nt, sizeof(pthread_t));
  if (!tid) return -1;
  for (int t = 0; t < nt; t++) pthread_create(&tid[t], NULL, fn, (char *)jobs + (size_t)t * stride);
  for (int t = 0; t < nt; t++) pthread_join(tid[t], NULL);
  free(tid);
  return 0;
}

int ora_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
             uint64_t weight_seed, uint32_t wmin, uint32_t wmax, uint32_t flags, int threads,
             ora_graph *out) {
  memset(out, 0, sizeof *out);
  if (scale < 1 || scale > 31 || edge_factor < 1 || (flags & ORA_RMAT_WEIGHTED && wmin > wmax)) return -1;
  if (threads < 1) threads = 1;
  const int sym = (flags & ORA_RMAT_SYMMETRIC) != 0, pr = (flags & ORA_RMAT_PR) != 0;
  const int weighted = (flags & ORA_RMAT_WEIGHTED) != 0;
  const uint64_t V = 1ull << scale, ntup = (uint64_t)edge_factor << scale;
  Draw d;
  d.scale = scale;
  d.t1 = thr32(a);
  d.t2 = thr32(a + b);
  d.t3 = thr32(a + b + c);
  d.seed = seed;
  d.permute = (flags & ORA_RMAT_PERMUTE) != 0;
  for (int r = 0; r < 3; r++) {
    d.mul[r] = ora_mix64(seed ^ (0x5851f42d4c957f2dull + (uint64_t)r)) | 1ull;
    d.add[r] = ora_mix64(seed ^ (0x14057b7ef767814full + 7ull * (uint64_t)r));
  }
  uint32_t *cnt = (uint32_t *)calloc(V, 4);
  uint64_t *start = (uint64_t *)malloc((V + 1) * 8);
  Job *jobs = (Job *)calloc((size_t)threads, sizeof(Job));
  if (!cnt || !start || !jobs) goto oom;
  for (int t = 0; t < threads; t++) {
    jobs[t].d = &d;
    jobs[t].t0 = ntup * (uint64_t)t / (uint64_t)threads;
    jobs[t].t1 = ntup * (uint64_t)(t + 1) / (uint64_t)threads;
    jobs[t].v0 = (uint32_t)(V * (uint64_t)t / (uint64_t)threads);
    jobs[t].v1 = (uint32_t)(V * (uint64_t)(t + 1) / (uint64_t)threads);
    jobs[t].sym = sym;
    jobs[t].pr = pr;
    jobs[t].cnt = cnt;
    jobs[t].start = start;
  }
  /* 1. tuples per row */
  run_jobs(threads, worker, jobs, sizeof(Job));
  start[0] = 0;
  for (uint64_t v = 0; v < V; v++) start[v + 1] = start[v] + cnt[v];
  /* 2. scatter the columns into their rows */
  uint32_t *raw = (uint32_t *)malloc((start[V] ? start[V] : 1) * 4);
  if (!raw) goto oom;
  memset(cnt, 0, V * 4);
  for (int t = 0; t < threads; t++) {
    jobs[t].phase = 1;
    jobs[t].raw = raw;
  }
  run_jobs(threads, worker, jobs, sizeof(Job));
  /* 3. sort and deduplicate every row (cnt now holds the unique counts) */
  for (int t = 0; t < threads; t++) {
    jobs[t].phase = 2;
    jobs[t].uniq = cnt;
  }
  run_jobs(threads, worker, jobs, sizeof(Job));
  /* 4. compact into the CSR */
  out->V = (uint32_t)V;
  out->off = (uint64_t *)malloc((V + 1) * 8);
  if (!out->off) {
    free(raw);
    goto oom;
  }
  out->off[0] = 0;
  for (uint64_t v = 0; v < V; v++) out->off[v + 1] = out->off[v] + cnt[v];
  out->E = out->off[V];
  out->weighted = weighted;
  out->edges = (uint32_t *)malloc((out->E ? out->E : 1) * (weighted ? 8 : 4));
  out->outdeg = pr ? (uint32_t *)calloc(V, 4) : NULL;
  Fill *fl = (Fill *)calloc((size_t)threads, sizeof(Fill));
  if (!out->edges || (pr && !out->outdeg) || !fl) {
    free(raw);
    free(fl);
    ora_graph_free(out);
    goto oom;
  }
  for (int t = 0; t < threads; t++) {
    fl[t].v0 = jobs[t].v0;
    fl[t].v1 = jobs[t].v1;
    fl[t].weighted = (uint32_t)weighted;
    fl[t].pr = (uint32_t)pr;
    fl[t].wmin = wmin;
    fl[t].wmax = wmax;
    fl[t].wseed = weight_seed;
    fl[t].start = start;
    fl[t].off = out->off;
    fl[t].raw = raw;
    fl[t].edges = out->edges;
    fl[t].outdeg = out->outdeg;
  }
  run_jobs(threads, fill_worker, fl, sizeof(Fill));
  free(fl);
  free(raw);
  free(cnt);
  free(start);
  free(jobs);
  return 0;
oom:
  free(cnt);
  free(start);
  free(jobs);
  return -2;
}

void ora_graph_free(ora_graph *g) {
  if (!g) return;
  free(g->off);
  free(g->edges);
  free(g->outdeg);
  memset(g, 0, sizeof *g);
}
