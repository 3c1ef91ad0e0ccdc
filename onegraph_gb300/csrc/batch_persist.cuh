// batch_persist.cuh — batched BFS (up to 64 sources) as ONE persistent,
// cooperative kernel that runs every level: in-kernel frontier compaction
// (grid-wide prefix over per-CTA counts), edge-balanced expansion over the
// compacted list, and per-level bookkeeping, separated by bounded grid
// barriers.  Static-region edges are read from HBM, dynamic-region edges
// straight from the page-locked host CSR over NVLink-C2C (selected per edge
// by its CSR index), so an out-of-memory graph needs no host round trip per
// level.  Tunables (template): CTA size and edge positions per thread; the
// tile (CTA size x items) is also the split granularity of high-degree
// vertices.  No reference counterpart: the reference runs sources one by one
// (BFS/oneGraph_BFS/CalculateOpt.h:55-209).
// Data written by other CTAs during the launch (list, prefix, tile map,
// frontier words and masks) is read with __ldcg: L1 is not coherent within a
// kernel, so a plain load could return a line cached in an earlier level.
#pragma once
#include "kernels.cuh"

namespace og {

constexpr uint32_t kErrBarrier = 16u;   // a grid barrier wait gave up
constexpr uint32_t kErrLevels = 32u;    // more levels than the histogram holds
constexpr uint32_t kMaxBatchLevels = 1024;

struct PersistArgs {
  uint32_t V;
  uint64_t nwords;
  const uint64_t *off;
  SrcP<false> ssrc;        // packed static records [0, static_edges) in HBM
  SrcP<false> hsrc;        // packed page-locked host records (all edges); words null if E == static_edges
  uint64_t static_edges;
  uint64_t E;
  unsigned long long *visited, *cur, *next;
  uint32_t *cur_any, *next_any;
  uint32_t *list;
  uint64_t *pref;
  uint32_t *tile_first;
  uint64_t list_cap, tile_cap;
  uint32_t *cta_n;            // per-CTA counts of the compaction
  unsigned long long *cta_e;  // per-CTA degree sums
  unsigned int *bar;          // [0] arrivals, [1] generation
  unsigned long long *hist;   // [kMaxBatchLevels][64] first-reached counts
  uint32_t *depth;            // n x V depths or null
  uint32_t n_src;
  uint32_t *err;
  uint32_t *levels;           // number of expanded levels (out)
  unsigned long long *stat;   // [0] listed vertices, [1] edges expanded, [2] of them dynamic
  uint32_t Vs;                // first dynamic vertex
};

__device__ __forceinline__ bool grid_barrier(unsigned int *bar, uint32_t *err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned int gen = ld_acquire((const uint32_t *)&bar[1]);
    __threadfence();
    if (atomicAdd(&bar[0], 1u) == gridDim.x - 1) {
      bar[0] = 0;
      __threadfence();
      st_release((uint32_t *)&bar[1], gen + 1);
    } else {
      uint32_t spins = 0;
      while (ld_acquire((const uint32_t *)&bar[1]) == gen) {
        if (++spins > kSpinLimit) {
          atomicOr(err, kErrBarrier);
          ok = 0;
          break;
        }
        __nanosleep(128);
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <int BLOCK, int ITEMS>
struct PersistShared {
  static constexpr uint32_t TILE = BLOCK * ITEMS;
  uint32_t rs[TILE + 2];
  unsigned long long cb[TILE + 1];
  unsigned long long val[TILE + 1];
  unsigned short map[TILE];
  uint32_t wsum_n[BLOCK / 32];
  unsigned long long wsum_e[BLOCK / 32];
  uint32_t cnt[64];
  uint32_t red_n;
  unsigned long long red_e, red_tn, red_te;
};

// block-wide exclusive scan of (u32, u64) with totals; BLOCK threads
template <int BLOCK, class SH>
__device__ __forceinline__ void pscan(SH &sh, uint32_t c, uint64_t e, uint32_t &exc, uint64_t &exe,
                                      uint32_t &totc, uint64_t &tote) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t ic = c;
  uint64_t ie = e;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t a = __shfl_up_sync(0xffffffffu, ic, d);
    const uint64_t b = __shfl_up_sync(0xffffffffu, ie, d);
    if (lane >= d) {
      ic += a;
      ie += b;
    }
  }
  if (lane == 31) {
    sh.wsum_n[warp] = ic;
    sh.wsum_e[warp] = ie;
  }
  __syncthreads();
  if (warp == 0) {
    uint32_t wc = lane < BLOCK / 32 ? sh.wsum_n[lane] : 0;
    uint64_t we = lane < BLOCK / 32 ? sh.wsum_e[lane] : 0;
#pragma unroll
    for (int d = 1; d < BLOCK / 32; d <<= 1) {
      const uint32_t a = __shfl_up_sync(0xffffffffu, wc, d);
      const uint64_t b = __shfl_up_sync(0xffffffffu, we, d);
      if (lane >= d) {
        wc += a;
        we += b;
      }
    }
    if (lane < BLOCK / 32) {
      sh.wsum_n[lane] = wc;
      sh.wsum_e[lane] = we;
    }
  }
  __syncthreads();
  exc = (warp ? sh.wsum_n[warp - 1] : 0) + ic - c;
  exe = (warp ? sh.wsum_e[warp - 1] : 0) + ie - e;
  totc = sh.wsum_n[BLOCK / 32 - 1];
  tote = sh.wsum_e[BLOCK / 32 - 1];
  __syncthreads();
}

template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_batch_persistent(PersistArgs a) {
  using SH = PersistShared<BLOCK, ITEMS>;
  constexpr uint32_t TILE = SH::TILE;
  __shared__ SH sh;
  unsigned long long *cur = a.cur, *next = a.next;
  uint32_t *cur_any = a.cur_any, *next_any = a.next_any;
  // contiguous word range of this CTA, split into contiguous per-thread runs
  const uint64_t wper_cta = (a.nwords + gridDim.x - 1) / gridDim.x;
  const uint64_t wper_thr = (wper_cta + BLOCK - 1) / BLOCK;
  const uint64_t wb = min(a.nwords, blockIdx.x * wper_cta + threadIdx.x * wper_thr);
  const uint64_t we = min(min(a.nwords, (blockIdx.x + 1) * wper_cta), wb + wper_thr);
  uint32_t level = 1;
  for (;; level++) {
    // ---- 1. count the frontier (vertices with edges) in this thread's words
    uint32_t c = 0;
    uint64_t e = 0, dyn = 0;
    for (uint64_t w = wb; w < we; w++)
      for (uint32_t m = __ldcg(cur_any + w); m; m &= m - 1) {
        const uint64_t v = w * 32 + (__ffs(m) - 1);
        const uint64_t d = a.off[v + 1] - a.off[v];
        c += d ? 1u : 0u;
        e += d;
        if (v >= a.Vs) dyn += d;
      }
    if (dyn) atomicAdd(a.stat + 2, (unsigned long long)dyn);
    uint32_t exc, totc;
    uint64_t exe, tote;
    pscan<BLOCK>(sh, c, e, exc, exe, totc, tote);
    if (threadIdx.x == 0) {
      a.cta_n[blockIdx.x] = totc;
      a.cta_e[blockIdx.x] = tote;
    }
    if (!grid_barrier(a.bar, a.err)) return;
    // ---- 2. this CTA's offset and the grand totals, then write the list
    {
      uint32_t pn = 0, tn = 0;
      uint64_t pe = 0, te = 0;
      for (uint32_t b = threadIdx.x; b < gridDim.x; b += BLOCK) {
        const uint32_t bn = __ldcg(a.cta_n + b);
        const uint64_t be = __ldcg(a.cta_e + b);
        tn += bn;
        te += be;
        if (b < blockIdx.x) {
          pn += bn;
          pe += be;
        }
      }
      uint32_t x0, y0;
      uint64_t x1, y1;
      pscan<BLOCK>(sh, pn, pe, x0, x1, y0, y1);  // block sums of the predecessor parts
      uint32_t z0, z1;
      uint64_t z2, z3;
      pscan<BLOCK>(sh, tn, te, z0, z2, z1, z3);
      if (threadIdx.x == 0) {
        sh.red_n = y0;
        sh.red_e = y1;
        sh.red_tn = z1;
        sh.red_te = z3;
      }
      __syncthreads();
    }
    const uint64_t total_n = sh.red_tn, total_e = sh.red_te;
    if (total_n == 0) break;  // every CTA sees the same totals
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.stat[0] += total_n;
      a.stat[1] += total_e;
    }
    if (level >= kMaxBatchLevels) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.err, kErrLevels);
      break;
    }
    if (total_n > a.list_cap || total_e / TILE + 1 >= a.tile_cap) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.err, kErrTileMap);
      break;
    }
    {
      uint32_t pos = sh.red_n + exc;
      uint64_t ep = sh.red_e + exe;
      for (uint64_t w = wb; w < we; w++)
        for (uint32_t m = __ldcg(cur_any + w); m; m &= m - 1) {
          const uint64_t v = w * 32 + (__ffs(m) - 1);
          const uint64_t d = a.off[v + 1] - a.off[v];
          if (!d) continue;
          a.list[pos] = (uint32_t)v;
          a.pref[pos] = ep;
          for (uint64_t t = (ep + TILE - 1) / TILE; t * TILE < ep + d; t++) a.tile_first[t] = pos;
          pos++;
          ep += d;
        }
      if (blockIdx.x == gridDim.x - 1 && threadIdx.x == BLOCK - 1) a.pref[total_n] = total_e;
    }
    if (!grid_barrier(a.bar, a.err)) return;
    // ---- 3. edge-balanced expansion of all listed vertices
    const uint64_t ntiles = (total_e + TILE - 1) / TILE;
    for (uint64_t k = blockIdx.x; k < ntiles; k += gridDim.x) {
      const uint64_t pos0 = k * TILE;
      const uint32_t tlen = (uint32_t)min((uint64_t)TILE, total_e - pos0);
      const uint32_t i0 = __ldcg(a.tile_first + k);
      const uint32_t i1 = (k + 1 < ntiles) ? __ldcg(a.tile_first + k + 1) : (uint32_t)(total_n - 1);
      const uint32_t nl = i1 - i0 + 1;
      if (i1 < i0 || nl > TILE + 1) {  // uniform per tile
        if (threadIdx.x == 0) atomicOr(a.err, kErrTileMap);
        continue;
      }
      for (uint32_t j = threadIdx.x; j < nl; j += BLOCK) {
        const uint32_t v = __ldcg(a.list + i0 + j);
        const uint64_t p = __ldcg(a.pref + i0 + j);
        sh.rs[j] = p > pos0 ? (uint32_t)min(p - pos0, (uint64_t)TILE) : 0u;
        sh.cb[j] = a.off[v] - p + pos0;
        sh.val[j] = __ldcg(cur + v);
      }
      for (uint32_t x = threadIdx.x; x < TILE; x += BLOCK) sh.map[x] = 0;
      __syncthreads();
      for (uint32_t j = 1 + threadIdx.x; j < nl; j += BLOCK)
        if (sh.rs[j] < TILE) sh.map[sh.rs[j]] = 1;
      __syncthreads();
      {
        uint32_t f[ITEMS], s = 0;
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
          f[i] = sh.map[threadIdx.x * ITEMS + i];
          s += f[i];
        }
        uint32_t ex, tot;
        uint64_t ex64, tot64;
        pscan<BLOCK>(sh, s, 0, ex, ex64, tot, tot64);
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
          ex += f[i];
          sh.map[threadIdx.x * ITEMS + i] = (unsigned short)ex;
        }
      }
      __syncthreads();
      uint32_t ev[ITEMS];
      uint32_t lv[ITEMS];
      uint32_t okm = 0;
#pragma unroll
      for (int it = 0; it < ITEMS; it++) {
        const uint32_t x = it * BLOCK + threadIdx.x;
        lv[it] = 0;
        if (x < tlen) {
          const uint32_t l = sh.map[x];
          const uint64_t idx = sh.cb[l] + x;
          lv[it] = l;
          if (idx < a.static_edges) {
            ev[it] = a.ssrc.load(idx);
            okm |= 1u << it;
          } else if (idx < a.E && a.hsrc.words) {
            ev[it] = a.hsrc.load(idx);
            okm |= 1u << it;
          } else {
            atomicOr(a.err, kErrEdgeIndex);
          }
        }
      }
      // probe every target's visited mask before the first atomic (the reads
      // overlap; a stale probe only costs an extra atomic)
      unsigned long long pv[ITEMS];
#pragma unroll
      for (int it = 0; it < ITEMS; it++) {
        pv[it] = ~0ull;
        if ((okm >> it) & 1u) {
          const uint32_t v = edge_dst(ev[it]);
          if (v < a.V) pv[it] = __ldcg(a.visited + v);
        }
      }
#pragma unroll
      for (int it = 0; it < ITEMS; it++) {
        if (!(okm & (1u << it))) continue;
        const uint32_t v = edge_dst(ev[it]);
        if (v >= a.V) {
          atomicOr(a.err, kErrVertex);
          continue;
        }
        unsigned long long nb = sh.val[lv[it]] & ~pv[it];
        if (!nb) continue;
        nb &= ~atomicOr(a.visited + v, nb);
        if (!nb) continue;
        if (atomicOr(next + v, nb) == 0ull) atomicOr(next_any + (v >> 5), 1u << (v & 31));
      }
      __syncthreads();  // shared tables are rebuilt for the next tile
    }
    if (!grid_barrier(a.bar, a.err)) return;
    // ---- 4. per-source counts of the newly reached vertices, depths, and
    //         clearing of the consumed frontier
    if (threadIdx.x < 64) sh.cnt[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t w = wb; w < we; w++) {
      for (uint32_t m = __ldcg(next_any + w); m; m &= m - 1) {
        const uint64_t v = w * 32 + (__ffs(m) - 1);
        for (unsigned long long b = __ldcg(next + v); b; b &= b - 1) {
          const uint32_t s = __ffsll((long long)b) - 1;
          if (s < a.n_src) {
            atomicAdd(&sh.cnt[s], 1u);
            if (a.depth) a.depth[(uint64_t)s * a.V + v] = level + 1;
          }
        }
      }
      for (uint32_t m = __ldcg(cur_any + w); m; m &= m - 1) cur[w * 32 + (__ffs(m) - 1)] = 0ull;
      cur_any[w] = 0u;
    }
    __syncthreads();
    if (threadIdx.x < 64 && sh.cnt[threadIdx.x])
      atomicAdd(a.hist + (uint64_t)level * 64 + threadIdx.x, (unsigned long long)sh.cnt[threadIdx.x]);
    // the next level reads the counts and masks written above by other CTAs
    if (!grid_barrier(a.bar, a.err)) return;
    unsigned long long *tm = cur;
    cur = next;
    next = tm;
    uint32_t *ta = cur_any;
    cur_any = next_any;
    next_any = ta;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.levels = level - 1;
}

}  // namespace og
