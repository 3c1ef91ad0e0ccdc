// rmat_gpu.cu — the R-MAT generator of rmat.cpp run on the device: the same
// counter-based draws (rmat_hash.hpp), so the edge set is identical to the
// host generator's; keys are sorted and deduplicated on the GPU, which makes
// scale-27 graphs (4.3e9 directed tuples) a matter of seconds.  Setup only:
// nothing here is on the query path.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>

#include "og_internal.hpp"
#include "rmat_hash.hpp"

namespace og {

namespace {

#define GK(x)                                                                                \
  do {                                                                                       \
    cudaError_t e_ = (x);                                                                    \
    if (e_ != cudaSuccess) {                                                                 \
      rc = fail(OG_E_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
      goto done;                                                                             \
    }                                                                                        \
  } while (0)

// Key = row << scale | col.  Self-loops become the marker 1 << (2*scale),
// which sorts after every real key and is dropped after dedup.
__global__ void k_rmat_keys(RmatDraw d, uint64_t ntuples, int sym, int pr, uint64_t *keys) {
  const uint64_t marker = 1ull << (2 * d.scale);
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ntuples;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t u, v;
    d.tuple(i, u, v);
    const bool loop = (u == v);
    const uint64_t k0 = pr ? (((uint64_t)v << d.scale) | u) : (((uint64_t)u << d.scale) | v);
    if (sym) {
      keys[2 * i] = loop ? marker : k0;
      keys[2 * i + 1] = loop ? marker : (((uint64_t)v << d.scale) | u);
    } else {
      keys[i] = loop ? marker : k0;
    }
  }
}

// off[r] = first key index with row >= r (keys sorted, unique, markers removed)
__global__ void k_rmat_offsets(const uint64_t *keys, uint64_t n, uint32_t scale, uint64_t V,
                               uint64_t *off) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= V;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t target = r << scale;
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (keys[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    off[r] = lo;
  }
}

__global__ void k_rmat_edges(const uint64_t *keys, uint64_t n, uint32_t scale, int weighted, int pr,
                             uint64_t wseed, uint32_t wmin, uint32_t wmax, uint32_t *edges,
                             uint32_t *outdeg) {
  const uint64_t mask = (1ull << scale) - 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(keys[i] >> scale), c = (uint32_t)(keys[i] & mask);
    if (weighted) {
      edges[2 * i] = c;
      edges[2 * i + 1] = edge_weight(wseed, r, c, wmin, wmax);
    } else {
      edges[i] = c;
    }
    if (pr) atomicAdd(outdeg + c, 1u);
  }
}

}  // namespace

int rmat_check_params(const og_rmat_params *p);

int rmat_generate_gpu(const og_rmat_params *p, og_graph **out) {
  int rc = OG_OK;
  const uint32_t s = p->scale;
  const uint64_t V = 1ull << s;
  const uint64_t ntuples = (uint64_t)p->edge_factor << s;
  const int sym = (p->flags & OG_RMAT_SYMMETRIC) != 0;
  const int pr = (p->flags & OG_RMAT_PR) != 0;
  const int weighted = (p->flags & OG_RMAT_WEIGHTED) != 0;
  const uint64_t n = ntuples * (sym ? 2 : 1);
  const RmatDraw draw = make_rmat_draw(s, p->a, p->b, p->c, p->seed, p->flags & OG_RMAT_PERMUTE);
  const uint64_t marker = 1ull << (2 * s);
  uint64_t *k0 = nullptr, *k1 = nullptr, *off_d = nullptr;
  unsigned long long *nsel_d = nullptr;
  uint32_t *edges_d = nullptr, *outdeg_d = nullptr;
  void *tmp = nullptr;
  size_t tmp_bytes = 0, tb = 0;
  unsigned long long nsel = 0;
  uint64_t E = 0;
  og_graph *g = nullptr;
  cudaStream_t st = nullptr;
  const int grid = 152 * 16;
  if (2 * s + 1 > 64) return fail(OG_E_ARG, "scale %u too large for the device generator", s);
  GK(cudaSetDevice(0));
  GK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  GK(cudaMalloc(&k0, n * 8));
  GK(cudaMalloc(&k1, n * 8));
  GK(cudaMalloc(&nsel_d, 8));
  k_rmat_keys<<<grid, 256, 0, st>>>(draw, ntuples, sym, pr, k0);
  GK(cudaGetLastError());
  {
    cub::DoubleBuffer<uint64_t> db(k0, k1);
    GK(cub::DeviceRadixSort::SortKeys(nullptr, tb, db, n, 0, (int)(2 * s + 1), st));
    tmp_bytes = tb;
    GK(cub::DeviceSelect::Unique(nullptr, tb, k0, k1, nsel_d, (int64_t)n, st));
    tmp_bytes = std::max(tmp_bytes, tb);
    GK(cudaMalloc(&tmp, tmp_bytes));
    tb = tmp_bytes;
    GK(cub::DeviceRadixSort::SortKeys(tmp, tb, db, n, 0, (int)(2 * s + 1), st));
    uint64_t *sorted = db.Current(), *other = db.Alternate();
    tb = tmp_bytes;
    GK(cub::DeviceSelect::Unique(tmp, tb, sorted, other, nsel_d, (int64_t)n, st));
    GK(cudaMemcpyAsync(&nsel, nsel_d, 8, cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    uint64_t last = 0;
    E = nsel;
    if (E) {
      GK(cudaMemcpy(&last, other + E - 1, 8, cudaMemcpyDeviceToHost));
      if (last == marker) E--;
    }
    GK(cudaFree(tmp));
    tmp = nullptr;
    GK(cudaFree(sorted));  // one of k0/k1
    if (sorted == k0) k0 = nullptr;
    else k1 = nullptr;
    uint64_t *keys = other;
    GK(cudaMalloc(&off_d, (V + 1) * 8));
    k_rmat_offsets<<<grid, 256, 0, st>>>(keys, E, s, V, off_d);
    GK(cudaMalloc(&edges_d, std::max<uint64_t>(E, 1) * (weighted ? 8 : 4)));
    if (pr) {
      GK(cudaMalloc(&outdeg_d, V * 4));
      GK(cudaMemsetAsync(outdeg_d, 0, V * 4, st));
    }
    k_rmat_edges<<<grid, 256, 0, st>>>(keys, E, s, weighted, pr, p->weight_seed, p->wmin, p->wmax,
                                       edges_d, outdeg_d);
    GK(cudaGetLastError());
    g = graph_new((uint32_t)V, E, pr ? OG_GRAPH_PR : (weighted ? OG_GRAPH_WEIGHTED : OG_GRAPH_PLAIN));
    if (!g) {
      rc = fail(OG_E_NOMEM, "cannot allocate host CSR (%llu edges)", (unsigned long long)E);
      goto done;
    }
    g->symmetric = sym ? 1 : -1;
    GK(cudaMemcpyAsync(g->off, off_d, (V + 1) * 8, cudaMemcpyDeviceToHost, st));
    if (E) GK(cudaMemcpyAsync(g->edges, edges_d, E * (weighted ? 8 : 4), cudaMemcpyDeviceToHost, st));
    if (pr) GK(cudaMemcpyAsync(g->outdeg, outdeg_d, V * 4, cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    *out = g;
    g = nullptr;
  }
done:
  if (g) graph_delete(g);
  cudaFree(k0);
  cudaFree(k1);
  cudaFree(tmp);
  cudaFree(nsel_d);
  cudaFree(off_d);
  cudaFree(edges_d);
  cudaFree(outdeg_d);
  if (st) cudaStreamDestroy(st);
  return rc;
}

}  // namespace og
