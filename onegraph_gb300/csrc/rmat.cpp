// rmat.cpp — seeded R-MAT graph generator on the host (and dispatch to the
// device generator).  The reference ships no generator; it expects CSR files
// from an external converter (README.md:8).  Output is the reference's CSR:
// rows sorted, columns sorted within a row, duplicates and self-loops removed.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

#include "og_internal.hpp"
#include "rmat_hash.hpp"

namespace og {
int rmat_generate_gpu(const og_rmat_params *p, og_graph **out);  // rmat_gpu.cu

int rmat_check_params(const og_rmat_params *p) {
  if (!p) return fail(OG_E_ARG, "null parameters");
  if (p->scale < 1 || p->scale > 31) return fail(OG_E_ARG, "scale %u out of [1,31]", p->scale);
  if (p->edge_factor < 1 || p->edge_factor > 1024) return fail(OG_E_ARG, "edge factor %u out of range", p->edge_factor);
  if (p->a < 0 || p->b < 0 || p->c < 0 || p->a + p->b + p->c > 1.0 + 1e-12)
    return fail(OG_E_ARG, "R-MAT probabilities must be >= 0 with a+b+c <= 1");
  if ((p->flags & OG_RMAT_WEIGHTED) && p->wmin > p->wmax) return fail(OG_E_ARG, "wmin > wmax");
  if ((p->flags & OG_RMAT_PR) && (p->flags & (OG_RMAT_SYMMETRIC | OG_RMAT_WEIGHTED)))
    return fail(OG_E_ARG, "a PageRank graph is directed and unweighted");
  return OG_OK;
}
}  // namespace og

using namespace og;

extern "C" int og_rmat_generate(const og_rmat_params *p, og_graph **out) {
  clear_error();
  if (!out) return fail(OG_E_ARG, "null output");
  *out = nullptr;
  int rc = rmat_check_params(p);
  if (rc != OG_OK) return rc;
  if (p->flags & OG_RMAT_ON_GPU) return rmat_generate_gpu(p, out);

  const uint32_t s = p->scale;
  const uint64_t V = 1ull << s;
  const uint64_t ntuples = (uint64_t)p->edge_factor << s;
  const bool sym = p->flags & OG_RMAT_SYMMETRIC;
  const bool pr = p->flags & OG_RMAT_PR;
  const bool weighted = p->flags & OG_RMAT_WEIGHTED;
  const RmatDraw draw = make_rmat_draw(s, p->a, p->b, p->c, p->seed, p->flags & OG_RMAT_PERMUTE);
  const unsigned nt = hw_threads(p->threads);
  const uint32_t bbits = std::min<uint32_t>(s, 10);
  const uint32_t nb = 1u << bbits;
  const uint32_t bshift = s - bbits;

  // 1. draw tuples into per-thread key lists, count keys per (thread, bucket)
  std::vector<std::vector<uint64_t>> local(nt);
  std::vector<uint64_t> counts((size_t)nt * nb, 0);
  parallel_for_threads(nt, [&](unsigned t, unsigned n) {
    const uint64_t b = ntuples * t / n, e = ntuples * (t + 1) / n;
    auto &L = local[t];
    L.reserve((size_t)(e - b) * (sym ? 2 : 1));
    uint64_t *cnt = &counts[(size_t)t * nb];
    for (uint64_t i = b; i < e; i++) {
      uint32_t u, v;
      draw.tuple(i, u, v);
      if (u == v) continue;
      const uint64_t k = pr ? (((uint64_t)v << 32) | u) : (((uint64_t)u << 32) | v);
      L.push_back(k);
      cnt[(uint32_t)(k >> 32) >> bshift]++;
      if (sym) {
        L.push_back(((uint64_t)v << 32) | u);
        cnt[v >> bshift]++;
      }
    }
  });
  // 2. scatter into buckets (bucket-major, thread-minor)
  std::vector<uint64_t> bstart((size_t)nb + 1, 0), pos((size_t)nt * nb);
  uint64_t total = 0;
  for (uint32_t bk = 0; bk < nb; bk++) {
    bstart[bk] = total;
    for (unsigned t = 0; t < nt; t++) {
      pos[(size_t)t * nb + bk] = total;
      total += counts[(size_t)t * nb + bk];
    }
  }
  bstart[nb] = total;
  std::vector<uint64_t> keys;
  try {
    keys.resize(total);
  } catch (...) {
    return fail(OG_E_NOMEM, "cannot allocate %llu keys", (unsigned long long)total);
  }
  parallel_for_threads(nt, [&](unsigned t, unsigned) {
    uint64_t *ps = &pos[(size_t)t * nb];
    for (uint64_t k : local[t]) keys[ps[(uint32_t)(k >> 32) >> bshift]++] = k;
    std::vector<uint64_t>().swap(local[t]);
  });
  // 3. sort + dedup each bucket; rows of a bucket are a contiguous id range
  std::vector<uint64_t> uniq(nb, 0);
  std::atomic<uint32_t> next_bucket{0};
  parallel_for_threads(nt, [&](unsigned, unsigned) {
    for (uint32_t bk; (bk = next_bucket.fetch_add(1)) < nb;) {
      uint64_t *b = keys.data() + bstart[bk], *e = keys.data() + bstart[bk + 1];
      std::sort(b, e);
      uniq[bk] = (uint64_t)(std::unique(b, e) - b);
    }
  });
  std::vector<uint64_t> ustart((size_t)nb + 1, 0);
  for (uint32_t bk = 0; bk < nb; bk++) ustart[bk + 1] = ustart[bk] + uniq[bk];
  const uint64_t E = ustart[nb];
  og_graph *g = graph_new((uint32_t)V, E, pr ? OG_GRAPH_PR : (weighted ? OG_GRAPH_WEIGHTED : OG_GRAPH_PLAIN));
  if (!g) return fail(OG_E_NOMEM, "cannot allocate host CSR (%llu edges)", (unsigned long long)E);
  g->symmetric = sym ? 1 : -1;
  // 4. CSR: per-row counts, offsets, columns (and weights / out-degrees)
  std::vector<uint32_t> rowcnt(V, 0);
  if (pr) memset(g->outdeg, 0, 4 * V);
  next_bucket = 0;
  parallel_for_threads(nt, [&](unsigned, unsigned) {
    for (uint32_t bk; (bk = next_bucket.fetch_add(1)) < nb;) {
      const uint64_t *b = keys.data() + bstart[bk];
      const uint64_t n = uniq[bk], e0 = ustart[bk];
      uint32_t *col = (uint32_t *)g->edges;
      for (uint64_t i = 0; i < n; i++) {
        const uint32_t r = (uint32_t)(b[i] >> 32), c = (uint32_t)b[i];
        rowcnt[r]++;
        if (weighted) {
          col[2 * (e0 + i)] = c;
          col[2 * (e0 + i) + 1] = edge_weight(p->weight_seed, r, c, p->wmin, p->wmax);
        } else {
          col[e0 + i] = c;
        }
        if (pr) __atomic_fetch_add(&g->outdeg[c], 1u, __ATOMIC_RELAXED);
      }
    }
  });
  uint64_t acc = 0;
  for (uint64_t v = 0; v < V; v++) {
    g->off[v] = acc;
    acc += rowcnt[v];
  }
  g->off[V] = acc;
  *out = g;
  return OG_OK;
}
