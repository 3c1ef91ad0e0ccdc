// graph_host.cpp — host side of libog.so: errors, CSR file I/O, validation,
// the region planner and the seeded R-MAT generator.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "og_internal.hpp"

namespace og {

static thread_local std::string t_err;

int fail(int status, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  return status;
}

void clear_error() { t_err.clear(); }

// Host CSR arrays start on a 64 KiB boundary and fill whole 64 KiB pages, so
// two graphs never share a page and each can be page-locked on its own
// (cudaHostRegister rejects ranges that overlap an earlier registration).
void *host_alloc(size_t bytes) {
  constexpr size_t kPage = 64 << 10;
  const size_t n = (bytes + kPage - 1) / kPage * kPage;
  void *p = nullptr;
  if (posix_memalign(&p, kPage, n ? n : kPage) != 0) return nullptr;
  return p;
}

void host_free(void *p) { free(p); }

unsigned hw_threads(unsigned requested) {
  unsigned n = std::thread::hardware_concurrency();
  if (n == 0) n = 1;
  if (requested && requested < n) n = requested;
  return n;
}

og_graph *graph_new(uint32_t V, uint64_t E, int kind) {
  og_graph *g = new (std::nothrow) og_graph;
  if (!g) return nullptr;
  g->V = V;
  g->E = E;
  g->kind = kind;
  g->off = (uint64_t *)host_alloc(sizeof(uint64_t) * ((size_t)V + 1));
  g->edges = host_alloc((size_t)E * g->edge_bytes());
  if (kind == OG_GRAPH_PR) g->outdeg = (uint32_t *)host_alloc(sizeof(uint32_t) * (size_t)(V ? V : 1));
  if (!g->off || !g->edges || (kind == OG_GRAPH_PR && !g->outdeg)) {
    graph_delete(g);
    return nullptr;
  }
  return g;
}

void graph_delete(og_graph *g) {
  if (!g) return;
  host_free(g->packed);
  host_free(g->off);
  host_free(g->edges);
  host_free(g->outdeg);
  delete g;
}

// Packs the edges into bpe-bit records (column in the low bc bits, weight
// minus the smallest weight above them), so that the host link and the static
// region carry bc + bw bits per edge: 33 bits for an R-MAT 27 graph with
// weights in [1, 64], 20 bits for an unweighted R-MAT 20 graph.  Threads pack
// ranges that start on multiples of 32 records, i.e. on whole words.  Runs
// once per graph; engines created concurrently on one graph serialise here.
int graph_prepare(og_graph *g) {
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  if (g->prepared) return OG_OK;
  const uint64_t E = g->E;
  const bool weighted = g->kind == OG_GRAPH_WEIGHTED;
  const uint32_t *ed = (const uint32_t *)g->edges;
  const unsigned nt = hw_threads(0);
  uint32_t wmin = 0, wmax = 0;
  if (weighted && E) {
    std::vector<uint32_t> tmin(nt, UINT32_MAX), tmax(nt, 0);
    parallel_for_threads(nt, [&](unsigned t, unsigned n) {
      uint32_t lo = UINT32_MAX, hi = 0;
      for (uint64_t e = E * t / n, ee = E * (t + 1) / n; e < ee; e++) {
        lo = std::min(lo, ed[2 * e + 1]);
        hi = std::max(hi, ed[2 * e + 1]);
      }
      tmin[t] = lo;
      tmax[t] = hi;
    });
    wmin = *std::min_element(tmin.begin(), tmin.end());
    wmax = *std::max_element(tmax.begin(), tmax.end());
  }
  const uint32_t bc = std::max<uint32_t>(1, bits_for(g->V - 1));
  const uint32_t bw = weighted ? bits_for(wmax - wmin) : 0;
  g->bc = bc;
  g->bw = bw;
  g->bpe = bc + bw;
  g->wmin = wmin;
  g->wmax = wmax;
  g->wbytes = weighted ? (wmax < 256 ? 1 : (wmax < 65536 ? 2 : 4)) : 0;
  const uint64_t words = g->packed_words_for(E);
  uint32_t *pk = (uint32_t *)host_alloc(4 * (size_t)words);
  if (!pk) return fail(OG_E_NOMEM, "cannot allocate the packed edge records (%llu words)", (unsigned long long)words);
  const uint64_t groups = (E + 31) / 32;
  const uint32_t bpe = g->bpe;
  parallel_for_threads(nt, [&](unsigned t, unsigned n) {
    const uint64_t e0 = std::min(E, groups * t / n * 32), e1 = std::min(E, groups * (t + 1) / n * 32);
    if (e0 >= e1) return;
    uint64_t q = e0 * bpe / 32;  // e0 is a multiple of 32: a word boundary
    unsigned __int128 acc = 0;
    uint32_t nb = 0;
    for (uint64_t e = e0; e < e1; e++) {
      const uint64_t rec = weighted ? ((uint64_t)ed[2 * e] | ((uint64_t)(ed[2 * e + 1] - wmin) << bc))
                                    : (uint64_t)ed[e];
      acc |= (unsigned __int128)rec << nb;
      nb += bpe;
      while (nb >= 32) {
        pk[q++] = (uint32_t)acc;
        acc >>= 32;
        nb -= 32;
      }
    }
    if (nb) pk[q++] = (uint32_t)acc;  // only the last range ends inside a word
  });
  const uint64_t full = (E * bpe + 31) / 32;
  for (uint64_t q = full; q < words; q++) pk[q] = 0;
  g->packed = pk;
  g->packed_words = words;
  g->prepared = true;
  return OG_OK;
}

int graph_validate(const og_graph *g) {
  const uint32_t V = g->V;
  if (V == 0) return fail(OG_E_FORMAT, "graph has no vertices");
  if (g->off[0] != 0) return fail(OG_E_FORMAT, "offsets[0] = %llu, expected 0", (unsigned long long)g->off[0]);
  if (g->off[V] != g->E) return fail(OG_E_FORMAT, "offset sentinel %llu != E %llu", (unsigned long long)g->off[V], (unsigned long long)g->E);
  const unsigned nt = hw_threads(0);
  std::atomic<uint64_t> bad_off{UINT64_MAX}, bad_col{UINT64_MAX};
  parallel_for_threads(nt, [&](unsigned t, unsigned n) {
    const uint64_t vb = (uint64_t)V * t / n, ve = (uint64_t)V * (t + 1) / n;
    for (uint64_t v = vb; v < ve; v++)
      if (g->off[v + 1] < g->off[v]) {
        uint64_t cur = bad_off.load();
        while (v < cur && !bad_off.compare_exchange_weak(cur, v)) {}
        break;
      }
    const uint64_t eb = g->E * t / n, ee = g->E * (t + 1) / n;
    const uint32_t *c = (const uint32_t *)g->edges;
    const uint64_t stride = g->kind == OG_GRAPH_WEIGHTED ? 2 : 1;
    for (uint64_t e = eb; e < ee; e++)
      if (c[e * stride] >= V) {
        uint64_t cur = bad_col.load();
        while (e < cur && !bad_col.compare_exchange_weak(cur, e)) {}
        break;
      }
  });
  if (bad_off.load() != UINT64_MAX)
    return fail(OG_E_FORMAT, "offsets decrease at vertex %llu", (unsigned long long)bad_off.load());
  if (bad_col.load() != UINT64_MAX)
    return fail(OG_E_FORMAT, "edge %llu has a column >= V", (unsigned long long)bad_col.load());
  return OG_OK;
}

// ------------------------------------------------------------------ planner

uint64_t engine_vertex_bytes(int kind, uint32_t flags) {
  // off_d u64 (8) + value u32 (4, also the f32 rank) + static/dynamic
  // compacted list u32 (4) + their u64 degree prefixes (8); the three frontier
  // bitmaps are counted in engine_fixed_bytes.  PageRank adds contrib f32,
  // sum f32 and outdeg u32.
  uint64_t b = 8 + 4 + 4 + 8;
  const bool pr = kind == OG_GRAPH_PR || (flags & OG_CFG_PR);
  // batched BFS: visited, frontier, next u64 masks; multi-source SSSP: a row
  // of distances, a pending-slot mask and a near-slot mask per list entry;
  // PageRank: contributions and sums (f32).  With either batch form they
  // share one allocation (a query context runs one computation at a time);
  // PageRank's out-degrees (u32) are resident.
  const bool arena = (flags & OG_CFG_BATCH) || sb_sources(flags);
  uint64_t shared = (flags & OG_CFG_BATCH) ? 24 : 0;
  if (sb_sources(flags)) shared = std::max<uint64_t>(shared, 4ull * sb_row_slots(sb_sources(flags)) + 8);
  if (pr) {
    b += 4;
    if (arena) shared = std::max<uint64_t>(shared, 8);
    else b += 8;
  }
  return b + shared;
}

uint64_t engine_fixed_bytes(uint32_t V, uint64_t E, uint32_t flags) {
  const uint64_t words = ((uint64_t)V + 31) / 32 + 2 * kCompactWords;
  const uint64_t bitmaps = 3 * 4 * words;
  const uint64_t ctiles = words / kCompactWords + 2;
  const uint64_t lookback = 2 * ctiles * 32;           // two scans in flight
  const uint64_t lbs_tiles = (E / kLbsTile + 8) * 16;  // tile maps + PR carries
  // batched BFS: per-level histogram (1024 x 64 u64), per-CTA scan slots and a
  // tile map for tiles as small as 1024 positions
  const uint64_t batch = (flags & OG_CFG_BATCH) ? (1024ull * 64 * 8 + 2048 * 16 + 4 * (E / 1024 + 8)) : 0;
  // 64 KiB covers the counters, the FP64 partials and the 256 B allocation floor
  return bitmaps + lookback + lbs_tiles + batch + (64u << 10);
}

int plan_compute(uint32_t V, uint64_t E, const uint64_t *off, int kind,
                 uint64_t budget, double advisek, uint32_t flags, og_plan *out,
                 uint32_t edge_bits, uint32_t stage_bytes) {
  if (!out || !off) return fail(OG_E_ARG, "plan_compute: null argument");
  if (kind < OG_GRAPH_PLAIN || kind > OG_GRAPH_PR) return fail(OG_E_ARG, "bad graph kind %d", kind);
  if (edge_bits == 0 || edge_bits > 64 || stage_bytes == 0) return fail(OG_E_ARG, "bad edge width");
  if (budget == 0) budget = kDefaultBudget;
  og_plan p;
  memset(&p, 0, sizeof p);
  p.budget_bytes = budget;
  p.edge_bits = edge_bits;
  p.edge_bytes = (edge_bits + 7) / 8;
  p.stage_edge_bytes = stage_bytes;
  p.vertex_bytes = engine_vertex_bytes(kind, flags) * ((uint64_t)V + 1);
  p.fixed_bytes = engine_fixed_bytes(V, E, flags);
  if (budget <= p.vertex_bytes + p.fixed_bytes)
    return fail(OG_E_BUDGET,
                "budget %llu B cannot hold the per-vertex state (%llu B) and scratch (%llu B)",
                (unsigned long long)budget, (unsigned long long)p.vertex_bytes,
                (unsigned long long)p.fixed_bytes);
  // T counts packed records (the static region's unit); staging buffers hold
  // unpacked edges of stage_bytes each and are charged in bytes below
  const uint64_t avail = budget - p.vertex_bytes - p.fixed_bytes;
  const uint64_t T = (uint64_t)((unsigned __int128)avail * 8 / edge_bits);
  p.edge_capacity = T;
  // GraphMeta.h:311-324: adviseK = (10 - E/T)/9, <0 -> 0.5, >1 -> 1, a positive
  // user value overrides it.  A user value above 1 is clamped to 1 here (the
  // reference would make partOverloadSize negative, GraphMeta.h:357).
  float ak = (10.0f - (float)E / (float)(T ? T : 1)) / 9.0f;
  if (ak < 0) ak = 0.5f;
  if (ak > 1) ak = 1.0f;
  p.advisek_auto = ak;
  double use = advisek > 0 ? std::min(advisek, 1.0) : (double)ak;
  p.advisek = use;
  uint64_t mps = (uint64_t)(use * (double)T);
  if (mps > E) mps = E;
  if (flags & OG_CFG_NO_STATIC) mps = 0;
  const bool direct = (flags & OG_CFG_DIRECT) != 0;
  auto prefix_for = [&](uint64_t limit) -> uint32_t {
    // largest Vs with off[Vs] <= limit (off is monotone, off[0] == 0)
    const uint64_t *it = std::upper_bound(off, off + (size_t)V + 1, limit);
    return (uint32_t)((it - off) - 1);
  };
  uint32_t Vs = prefix_for(mps);
  uint64_t st = off[Vs];
  uint64_t dyn = E - st;
  uint64_t chunk = 0;
  if (dyn > 0 && !direct) {
    // smallest acceptable staging buffer: 1M edges, or an eighth of the edge
    // budget when that is smaller (small budgets used to force many chunks),
    // never below one LBS tile and never above the dynamic region itself
    const uint64_t eighth = std::max<uint64_t>(kLbsTile, T / 8 / kLbsTile * kLbsTile);
    const uint64_t need = std::min<uint64_t>(
        std::min<uint64_t>(kMinChunkEdges, eighth), (dyn + kLbsTile - 1) / kLbsTile * kLbsTile);
    // bytes left after the static records, as staged edges per buffer
    auto room_for = [&](uint64_t st_edges) -> uint64_t {
      const uint64_t used = (st_edges * edge_bits + 7) / 8;
      return used >= avail ? 0 : (avail - used) / stage_bytes / 2 / kLbsTile * kLbsTile;
    };
    uint64_t room = room_for(st);
    if (room < need) {
      // leave room for two staging buffers by shrinking the static prefix
      const uint64_t stage = 2 * need * stage_bytes;
      if (avail < stage) return fail(OG_E_BUDGET, "budget leaves no room for the dynamic staging buffers");
      mps = std::min<uint64_t>(mps, (uint64_t)((unsigned __int128)(avail - stage) * 8 / edge_bits));
      Vs = prefix_for(mps);
      st = off[Vs];
      dyn = E - st;
      room = room_for(st);
    }
    chunk = std::min(room, (dyn + kLbsTile - 1) / kLbsTile * kLbsTile);
  }
  p.max_partition = mps;
  p.static_vertices = Vs;
  p.static_edges = st;
  p.dynamic_edges = dyn;
  p.chunk_edges = chunk;
  *out = p;
  return OG_OK;
}

}  // namespace og

// ====================================================================== C ABI

using namespace og;

#define RC_HOST(x)              \
  do {                          \
    int r_ = (x);               \
    if (r_ != OG_OK) return r_; \
  } while (0)

extern "C" const char *og_last_error(void) { return t_err.c_str(); }
extern "C" int og_abi_version(void) { return OG_ABI_VERSION; }

static bool read_exact(FILE *f, void *p, size_t n) {
  // large reads in pieces so that a short read is detected early
  char *c = (char *)p;
  while (n) {
    size_t k = std::min<size_t>(n, (size_t)1 << 30);
    if (fread(c, 1, k, f) != k) return false;
    c += k;
    n -= k;
  }
  return true;
}

extern "C" int og_graph_load(const char *path, int kind, og_graph **out) {
  clear_error();
  if (!path || !out) return fail(OG_E_ARG, "og_graph_load: null argument");
  if (kind < OG_GRAPH_PLAIN || kind > OG_GRAPH_PR) return fail(OG_E_ARG, "bad graph kind %d", kind);
  *out = nullptr;
  FILE *f = fopen(path, "rb");
  if (!f) return fail(OG_E_IO, "cannot open %s", path);
  uint64_t hdr[2];
  if (fread(hdr, 8, 2, f) != 2) {
    fclose(f);
    return fail(OG_E_FORMAT, "%s: short header", path);
  }
  // GraphMeta.h:130 reads the u64 V into a 32-bit field; V must fit in 32 bits.
  if (hdr[0] == 0 || hdr[0] > 0xFFFFFFFFull) {
    fclose(f);
    return fail(OG_E_FORMAT, "%s: vertex count %llu out of range", path, (unsigned long long)hdr[0]);
  }
  const uint32_t V = (uint32_t)hdr[0];
  const uint64_t E = hdr[1];
  const uint64_t eb = kind == OG_GRAPH_WEIGHTED ? 8 : 4;
  fseeko(f, 0, SEEK_END);
  const uint64_t size = (uint64_t)ftello(f);
  const uint64_t want = 16 + (kind == OG_GRAPH_PR ? 4ull * V : 0) + 8ull * V + E * eb;
  if (E > (1ull << 40) || size != want) {
    fclose(f);
    return fail(OG_E_FORMAT, "%s: file has %llu bytes, header implies %llu", path,
                (unsigned long long)size, (unsigned long long)want);
  }
  fseeko(f, 16, SEEK_SET);
  og_graph *g = graph_new(V, E, kind);
  if (!g) {
    fclose(f);
    return fail(OG_E_NOMEM, "cannot allocate host CSR (%llu edges)", (unsigned long long)E);
  }
  bool ok = true;
  if (kind == OG_GRAPH_PR) ok = read_exact(f, g->outdeg, 4ull * V);
  ok = ok && read_exact(f, g->off, 8ull * V) && read_exact(f, g->edges, E * eb);
  fclose(f);
  if (!ok) {
    graph_delete(g);
    return fail(OG_E_IO, "%s: read failed", path);
  }
  g->off[V] = E;
  int rc = graph_validate(g);
  if (rc != OG_OK) {
    graph_delete(g);
    return rc;
  }
  *out = g;
  return OG_OK;
}

extern "C" int og_graph_from_arrays(uint64_t V, uint64_t E, const uint64_t *offsets,
                                    int with_sentinel, const void *edges,
                                    const uint32_t *outdeg, int kind, og_graph **out) {
  clear_error();
  if (!out || !offsets || (E && !edges)) return fail(OG_E_ARG, "og_graph_from_arrays: null argument");
  if (V == 0 || V > 0xFFFFFFFFull) return fail(OG_E_ARG, "vertex count out of range");
  if (kind < OG_GRAPH_PLAIN || kind > OG_GRAPH_PR) return fail(OG_E_ARG, "bad graph kind %d", kind);
  if (kind == OG_GRAPH_PR && !outdeg) return fail(OG_E_ARG, "PR graph needs outdeg");
  *out = nullptr;
  og_graph *g = graph_new((uint32_t)V, E, kind);
  if (!g) return fail(OG_E_NOMEM, "cannot allocate host CSR");
  memcpy(g->off, offsets, 8 * V);
  g->off[V] = with_sentinel ? offsets[V] : E;
  if (E) memcpy(g->edges, edges, E * g->edge_bytes());
  if (kind == OG_GRAPH_PR) memcpy(g->outdeg, outdeg, 4 * V);
  int rc = graph_validate(g);
  if (rc != OG_OK) {
    graph_delete(g);
    return rc;
  }
  *out = g;
  return OG_OK;
}

extern "C" int og_graph_transpose(const og_graph *g, og_graph **out) {
  clear_error();
  if (!g || !out) return fail(OG_E_ARG, "og_graph_transpose: null argument");
  if (g->kind == OG_GRAPH_WEIGHTED) return fail(OG_E_UNSUPPORTED, "og_graph_transpose: weighted graph");
  *out = nullptr;
  const uint32_t V = g->V;
  const uint64_t E = g->E;
  og_graph *t = graph_new(V, E, OG_GRAPH_PLAIN);
  std::unique_ptr<std::atomic<uint64_t>[]> cur(new (std::nothrow) std::atomic<uint64_t>[(size_t)V]);
  if (!t || !cur) {
    if (t) graph_delete(t);
    return fail(OG_E_NOMEM, "og_graph_transpose: cannot allocate %llu edges", (unsigned long long)E);
  }
  const uint32_t *col = (const uint32_t *)g->edges;
  uint32_t *tcol = (uint32_t *)t->edges;
  const unsigned nt = hw_threads(0);
  auto parallel = [&](uint64_t n, auto body) {  // body(lo, hi) over nt contiguous ranges
    std::vector<std::thread> th;
    for (unsigned k = 0; k < nt; k++) {
      const uint64_t lo = n * k / nt, hi = n * (k + 1) / nt;
      th.emplace_back([=, &body] { body(lo, hi); });
    }
    for (auto &x : th) x.join();
  };
  // 1. list lengths of the reverse graph
  parallel(V, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t u = lo; u < hi; u++) cur[u].store(0, std::memory_order_relaxed);
  });
  parallel(E, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; i++) cur[col[i]].fetch_add(1, std::memory_order_relaxed);
  });
  t->off[0] = 0;
  for (uint64_t u = 0; u < V; u++) {
    const uint64_t n = cur[u].load(std::memory_order_relaxed);
    cur[u].store(t->off[u], std::memory_order_relaxed);
    t->off[u + 1] = t->off[u] + n;
  }
  // 2. scatter (v, u) into list u, then sort each list: the result does not
  //    depend on the threads' interleaving
  parallel(V, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t v = lo; v < hi; v++)
      for (uint64_t i = g->off[v]; i < g->off[v + 1]; i++)
        tcol[cur[col[i]].fetch_add(1, std::memory_order_relaxed)] = (uint32_t)v;
  });
  parallel(V, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t u = lo; u < hi; u++) std::sort(tcol + t->off[u], tcol + t->off[u + 1]);
  });
  t->symmetric = g->symmetric;
  const int rc = graph_validate(t);
  if (rc != OG_OK) {
    graph_delete(t);
    return rc;
  }
  *out = t;
  return OG_OK;
}

extern "C" int og_graph_save(const og_graph *g, const char *path) {
  clear_error();
  if (!g || !path) return fail(OG_E_ARG, "og_graph_save: null argument");
  FILE *f = fopen(path, "wb");
  if (!f) return fail(OG_E_IO, "cannot create %s", path);
  uint64_t hdr[2] = {g->V, g->E};
  bool ok = fwrite(hdr, 8, 2, f) == 2;
  if (ok && g->kind == OG_GRAPH_PR) ok = fwrite(g->outdeg, 4, g->V, f) == g->V;
  ok = ok && fwrite(g->off, 8, g->V, f) == g->V;
  const char *c = (const char *)g->edges;
  uint64_t left = g->E * g->edge_bytes();
  while (ok && left) {
    size_t k = (size_t)std::min<uint64_t>(left, 1ull << 30);
    ok = fwrite(c, 1, k, f) == k;
    c += k;
    left -= k;
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? OG_OK : fail(OG_E_IO, "write to %s failed", path);
}

extern "C" int og_graph_info(const og_graph *g, uint64_t *V, uint64_t *E, int *kind,
                             const uint64_t **offsets, const void **edges,
                             const uint32_t **outdeg) {
  if (!g) return fail(OG_E_ARG, "og_graph_info: null graph");
  if (V) *V = g->V;
  if (E) *E = g->E;
  if (kind) *kind = g->kind;
  if (offsets) *offsets = g->off;
  if (edges) *edges = g->edges;
  if (outdeg) *outdeg = g->outdeg;
  return OG_OK;
}

extern "C" int og_graph_save_bel(const og_graph *g, const char *prefix) {
  clear_error();
  if (!g || !prefix) return fail(OG_E_ARG, "og_graph_save_bel: null argument");
  const std::string base(prefix);
  const uint64_t zero = 0, V = g->V, E = g->E;
  const bool weighted = g->kind == OG_GRAPH_WEIGHTED;
  const uint32_t *c = (const uint32_t *)g->edges;
  const uint64_t stride = weighted ? 2 : 1;
  auto open_w = [&](const char *ext) { return fopen((base + ext).c_str(), "wb"); };
  FILE *f = open_w(".bel.col");
  if (!f) return fail(OG_E_IO, "cannot create %s.bel.col", prefix);
  bool ok = fwrite(&V, 8, 1, f) == 1 && fwrite(&zero, 8, 1, f) == 1 && fwrite(g->off, 8, V, f) == V;
  ok = (fclose(f) == 0) && ok;
  f = ok ? open_w(".bel.dst") : nullptr;
  ok = ok && f && fwrite(&E, 8, 1, f) == 1 && fwrite(&zero, 8, 1, f) == 1;
  std::vector<uint64_t> buf(1 << 20);
  for (uint64_t e0 = 0; ok && e0 < E; e0 += buf.size()) {
    const uint64_t n = std::min<uint64_t>(buf.size(), E - e0);
    for (uint64_t i = 0; i < n; i++) buf[i] = c[(e0 + i) * stride];
    ok = fwrite(buf.data(), 8, n, f) == n;
  }
  if (f) ok = (fclose(f) == 0) && ok;
  if (ok && weighted) {
    f = open_w(".bel.val");
    ok = f && fwrite(&E, 8, 1, f) == 1 && fwrite(&zero, 8, 1, f) == 1;
    std::vector<uint32_t> w(1 << 20);
    for (uint64_t e0 = 0; ok && e0 < E; e0 += w.size()) {
      const uint64_t n = std::min<uint64_t>(w.size(), E - e0);
      for (uint64_t i = 0; i < n; i++) w[i] = c[2 * (e0 + i) + 1];
      ok = fwrite(w.data(), 4, n, f) == n;
    }
    if (f) ok = (fclose(f) == 0) && ok;
  }
  return ok ? OG_OK : fail(OG_E_IO, "writing %s.bel.* failed", prefix);
}

extern "C" int og_graph_set_symmetric(og_graph *g, int symmetric) {
  clear_error();
  if (!g || (symmetric != 0 && symmetric != 1)) return fail(OG_E_ARG, "og_graph_set_symmetric: bad argument");
  g->symmetric = symmetric;
  return OG_OK;
}

extern "C" int og_graph_symmetric(og_graph *g, int *symmetric) {
  clear_error();
  if (!g || !symmetric) return fail(OG_E_ARG, "og_graph_symmetric: null argument");
  if (g->symmetric >= 0) {
    *symmetric = g->symmetric;
    return OG_OK;
  }
  const uint32_t V = g->V;
  const uint32_t stride = g->kind == OG_GRAPH_WEIGHTED ? 2 : 1;
  const uint32_t *ed = (const uint32_t *)g->edges;
  const uint64_t *off = g->off;
  std::atomic<int> bad{0};
  const unsigned nt = hw_threads(0);
  // sorted adjacency lists (strictly increasing columns)
  parallel_for_threads(nt, [&](unsigned t, unsigned n) {
    for (uint64_t u = (uint64_t)V * t / n, ue = (uint64_t)V * (t + 1) / n; u < ue && !bad.load(std::memory_order_relaxed); u++)
      for (uint64_t e = off[u] + 1; e < off[u + 1]; e++)
        if (ed[e * stride] <= ed[(e - 1) * stride]) {
          bad.store(1);
          break;
        }
  });
  if (!bad.load()) {
    parallel_for_threads(nt, [&](unsigned t, unsigned n) {
      for (uint64_t u = (uint64_t)V * t / n, ue = (uint64_t)V * (t + 1) / n; u < ue && !bad.load(std::memory_order_relaxed); u++)
        for (uint64_t e = off[u]; e < off[u + 1]; e++) {
          const uint32_t v = ed[e * stride];
          uint64_t lo = off[v], hi = off[v + 1];  // find u in adj(v)
          while (lo < hi) {
            const uint64_t mid = (lo + hi) / 2;
            if (ed[mid * stride] < u) lo = mid + 1;
            else hi = mid;
          }
          if (lo == off[v + 1] || ed[lo * stride] != u) {
            bad.store(1);
            break;
          }
        }
    });
  }
  g->symmetric = bad.load() ? 0 : 1;
  *symmetric = g->symmetric;
  return OG_OK;
}

extern "C" int og_graph_records(og_graph *g, const uint32_t **words, uint64_t *nwords, uint32_t *bpe,
                                uint32_t *bc, uint32_t *wmin) {
  clear_error();
  if (!g) return fail(OG_E_ARG, "og_graph_records: null graph");
  RC_HOST(graph_prepare(g));
  if (words) *words = g->packed;
  if (nwords) *nwords = g->packed_words;
  if (bpe) *bpe = g->bpe;
  if (bc) *bc = g->bc;
  if (wmin) *wmin = g->wmin;
  return OG_OK;
}

extern "C" int og_convert_uint_to_ulong(const char *in_path, const char *out_path) {
  clear_error();
  if (!in_path) return fail(OG_E_ARG, "og_convert_uint_to_ulong: null input path");
  std::string out = out_path ? std::string(out_path) : std::string(in_path);
  if (!out_path) {
    if (out.size() < 4) return fail(OG_E_ARG, "input path '%s' is shorter than its extension", in_path);
    out = out.substr(0, out.size() - 4) + "lcsr";
  }
  FILE *f = fopen(in_path, "rb");
  if (!f) return fail(OG_E_IO, "cannot open %s", in_path);
  uint32_t hdr[2];
  if (fread(hdr, 4, 2, f) != 2) {
    fclose(f);
    return fail(OG_E_FORMAT, "%s: truncated header", in_path);
  }
  const uint32_t V = hdr[0], E = hdr[1];
  std::vector<uint32_t> off(V), col(E);
  const bool ok_in = fread(off.data(), 4, V, f) == V && fread(col.data(), 4, E, f) == E;
  fclose(f);
  if (!ok_in) return fail(OG_E_FORMAT, "%s: file shorter than V=%u, E=%u", in_path, V, E);
  for (uint32_t v = 0; v < V; v++)
    if (off[v] > E || (v && off[v] < off[v - 1]))
      return fail(OG_E_FORMAT, "%s: offsets[%u] = %u out of order or above E", in_path, v, off[v]);
  FILE *o = fopen(out.c_str(), "wb");
  if (!o) return fail(OG_E_IO, "cannot create %s", out.c_str());
  bool ok = fwrite(hdr, 4, 2, o) == 2 && fwrite(off.data(), 4, V, o) == V;
  std::vector<uint64_t> buf(1 << 20);
  for (uint64_t e0 = 0; ok && e0 < E; e0 += buf.size()) {
    const uint64_t n = std::min<uint64_t>(buf.size(), E - e0);
    for (uint64_t i = 0; i < n; i++) buf[i] = col[e0 + i];
    ok = fwrite(buf.data(), 8, n, o) == n;
  }
  ok = (fclose(o) == 0) && ok;
  return ok ? OG_OK : fail(OG_E_IO, "writing %s failed", out.c_str());
}

extern "C" uint32_t og_graph_findbignode(const og_graph *g, uint32_t last) {
  // GraphMeta.h:150-165
  if (!g || g->V < 2) return last;
  for (uint64_t i = (uint64_t)last + 1; i < (uint64_t)g->V - 1; i++)
    if (g->off[i + 1] - g->off[i] > 3000) return (uint32_t)i;
  return last;
}

extern "C" int og_plan_compute(uint64_t V, uint64_t E, const uint64_t *offsets, int kind,
                               uint64_t budget_bytes, double advisek, uint32_t flags,
                               og_plan *out) {
  clear_error();
  if (V == 0 || V > 0xFFFFFFFFull) return fail(OG_E_ARG, "vertex count out of range");
  // the reference's accounting, sizeof(Edge) per edge (GraphMeta.h:307-309):
  // without the graph the packed record width is unknown
  const bool w = kind == OG_GRAPH_WEIGHTED;
  return plan_compute((uint32_t)V, E, offsets, kind, budget_bytes, advisek, flags, out, w ? 64 : 32,
                      w ? 8 : 4);
}

int og::plan_replace_split(const og_graph *g, uint32_t flags, og_plan *p, uint64_t *slot_bytes) {
  if (!(flags & OG_CFG_DIRECT) || (flags & (OG_CFG_NO_PIN | OG_CFG_NO_STATIC)))
    return fail(OG_E_ARG, "OG_CFG_REPLACE needs OG_CFG_DIRECT, a page-locked host copy and a static region");
  if (p->static_edges == 0 || p->dynamic_edges == 0)
    return fail(OG_E_BUDGET, "OG_CFG_REPLACE: the plan has no %s region to share",
                p->static_edges == 0 ? "static" : "dynamic");
  const uint64_t old_words = g->packed_words_for(p->static_edges);
  const uint64_t half = p->static_edges / 2;
  const uint32_t vs = (uint32_t)(std::upper_bound(g->off, g->off + (uint64_t)g->V + 1, half) - g->off - 1);
  p->static_vertices = vs;
  p->static_edges = g->off[vs];
  p->dynamic_edges = g->E - p->static_edges;
  *slot_bytes = 4 * (old_words - (p->static_edges ? g->packed_words_for(p->static_edges) : 0));
  return OG_OK;
}

extern "C" int og_graph_plan(og_graph *g, uint64_t budget_bytes, double advisek, uint32_t flags,
                             og_plan *out) {
  clear_error();
  if (!g) return fail(OG_E_ARG, "og_graph_plan: null graph");
  RC_HOST(graph_prepare(g));
  RC_HOST(plan_compute(g->V, g->E, g->off, g->kind, budget_bytes, advisek, flags, out, g->bpe,
                       4 + g->wbytes));
  if (flags & OG_CFG_REPLACE) {
    uint64_t slot_bytes = 0;
    RC_HOST(plan_replace_split(g, flags, out, &slot_bytes));
  }
  return OG_OK;
}
