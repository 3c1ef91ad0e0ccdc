// og_internal.hpp — host-side types shared by the libog.so translation units.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/onegraph.h"

// Host graph in the reference's CSR layout (GraphMeta.h:40-46) with the V+1
// offset sentinel added.  Arrays are 64-byte aligned host allocations; the
// engine page-locks them (cudaHostRegister) so kernels can gather from them.
struct og_graph {
  uint32_t V = 0;
  uint64_t E = 0;
  int kind = OG_GRAPH_PLAIN;
  uint64_t *off = nullptr;     // V+1
  void *edges = nullptr;       // E * edge_bytes()
  uint32_t *outdeg = nullptr;  // V (OG_GRAPH_PR only)
  int registered = 0;          // number of engines holding a registration
  bool host_pinned = false;    // allocated page-locked (cudaMallocHost)
  // every edge (u, v) has its reverse (v, u): 1 yes, 0 no, -1 not known.
  // Set by the symmetric R-MAT generator, asserted with og_graph_set_symmetric
  // or checked by og_graph_symmetric; CC takes the union-find path only at 1.
  int symmetric = -1;
  // Bit-packed edge records used by the engines (built once, on first use):
  // record e occupies bits [e*bpe, (e+1)*bpe) of the u32 word array `packed`
  // (little-endian bit order), low bc bits the column, the next bw bits the
  // weight minus wmin.  bc = bits of V-1, bw = bits of (wmax - wmin), 0 for
  // unweighted kinds.  Two zero words pad the end so that a record is always
  // read as two (three when bpe > 33) whole words.
  uint32_t *packed = nullptr;
  uint64_t packed_words = 0;
  uint32_t bpe = 0, bc = 0, bw = 0, wmin = 0, wmax = 0;
  // width of an unpacked weight in the device staging buffers (1, 2, 4; 0 unweighted)
  uint32_t wbytes = 0;
  bool prepared = false;
  // bytes of one edge in the reference layout (the `edges` array)
  uint32_t edge_bytes() const { return kind == OG_GRAPH_WEIGHTED ? 8u : 4u; }
  // words holding records [0, n) plus the padding
  uint64_t packed_words_for(uint64_t n) const { return (n * bpe + 31) / 32 + 2; }
};

namespace og {

// Thread-local error message behind og_last_error().
int fail(int status, const char *fmt, ...);
void clear_error();

// 64-byte aligned host allocation; returns nullptr on failure.
void *host_alloc(size_t bytes);
void host_free(void *p);

og_graph *graph_new(uint32_t V, uint64_t E, int kind);  // arrays allocated, not filled
void graph_delete(og_graph *g);

// Validates offsets (monotone, off[V] == E) and columns (< V).
int graph_validate(const og_graph *g);

unsigned hw_threads(unsigned requested);

// Runs fn(t, nthreads) on nthreads host threads.
template <class F>
void parallel_for_threads(unsigned nthreads, F fn);

// Builds the packed records (g->packed, bpe, bc, bw, wmin, wbytes) if not built yet.
int graph_prepare(og_graph *g);

// Region planner shared by og_plan_compute and the engine: edge_bits is the
// size of one packed record (static region), stage_bytes the bytes of one
// unpacked edge in a staging buffer (4 + weight bytes).
int plan_compute(uint32_t V, uint64_t E, const uint64_t *off, int kind,
                 uint64_t budget, double advisek, uint32_t flags, og_plan *out,
                 uint32_t edge_bits, uint32_t stage_bytes);

// OG_CFG_REPLACE on a plan made by plan_compute: the static prefix shrinks to
// the largest vertex prefix within half of its edges, and *slot_bytes gets
// the device bytes that frees for fragment slots.  OG_E_ARG for flags the
// mode cannot run with, OG_E_BUDGET for a plan without a static or a dynamic
// region.
int plan_replace_split(const og_graph *g, uint32_t flags, og_plan *p, uint64_t *slot_bytes);

// Bits needed to hold values 0..x (0 for x == 0).
inline uint32_t bits_for(uint64_t x) {
  uint32_t b = 0;
  while (x) {
    b++;
    x >>= 1;
  }
  return b;
}

// Slots of one multi-source SSSP row for k sources: 4, 8, 16 or 32 (a
// divisor of the warp size, so a warp covers whole rows in the reduction
// kernels).  4 slots (16 B) plus the two masks take the 24 B per vertex of the
// batched BFS masks, so such an engine needs no more memory for both.
inline uint32_t sb_row_slots(uint32_t k) { return k <= 4 ? 4u : (k <= 8 ? 8u : (k <= 16 ? 16u : 32u)); }
// Sources per multi-source SSSP pass requested by og_config flags (0: none).
inline uint32_t sb_sources(uint32_t flags) { return (flags >> 8) & 63u; }

// Per-vertex / fixed device bytes the engine allocates (planner inputs).
uint64_t engine_vertex_bytes(int kind, uint32_t flags);
uint64_t engine_fixed_bytes(uint32_t V, uint64_t E, uint32_t flags);

constexpr uint32_t kLbsTile = 2048;          // edge positions per LBS tile
constexpr uint32_t kCompactWords = 1024;     // bitmap words per compaction tile (kWordsPerCompactTile)
constexpr uint64_t kMinChunkEdges = 1u << 20;  // smallest staging buffer
constexpr uint64_t kDefaultBudget = 12ull << 30;  // GraphMeta.h:305

}  // namespace og

#include <thread>
template <class F>
void og::parallel_for_threads(unsigned nthreads, F fn) {
  if (nthreads <= 1) {
    fn(0u, 1u);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nthreads);
  for (unsigned t = 0; t < nthreads; t++) th.emplace_back(fn, t, nthreads);
  for (auto &x : th) x.join();
}
