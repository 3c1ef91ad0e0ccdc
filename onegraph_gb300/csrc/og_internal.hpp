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
  // Structure-of-arrays copy used by the engines (built once, on first use):
  // u32 columns (the edge array itself for unweighted kinds) and, for
  // weighted graphs, the weights in the narrowest of 1, 2 or 4 bytes.
  uint32_t *cols = nullptr;
  void *wts = nullptr;
  uint32_t wbytes = 0;
  bool soa = false;
  uint32_t edge_bytes() const { return kind == OG_GRAPH_WEIGHTED ? 8u : 4u; }
  uint32_t soa_edge_bytes() const { return 4u + wbytes; }
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

// Builds g->cols / g->wts / g->wbytes if not built yet.
int graph_prepare_soa(og_graph *g);

// Region planner shared by og_plan_compute and the engine; edge_bytes is the
// device bytes per edge (4 + weight bytes).
int plan_compute(uint32_t V, uint64_t E, const uint64_t *off, int kind,
                 uint64_t budget, double advisek, uint32_t flags, og_plan *out,
                 uint32_t edge_bytes);

// Per-vertex / fixed device bytes the engine allocates (planner inputs).
uint64_t engine_vertex_bytes(int kind, uint32_t flags);
uint64_t engine_fixed_bytes(uint32_t V, uint64_t E, uint32_t flags);

constexpr uint32_t kLbsTile = 2048;          // edge positions per LBS tile
constexpr uint32_t kCompactWords = 256;      // bitmap words per compaction tile
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
