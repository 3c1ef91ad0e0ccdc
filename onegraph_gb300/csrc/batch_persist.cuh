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
//
// On a symmetric graph each source chooses its direction per level (the
// direction-optimizing rule of Beamer et al., SC 2012, applied to every
// source's own frontier): bottom-up once the source's frontier edges exceed
// 1/14 of the edges of the vertices it has not reached, top-down again when
// its frontier is under V/24 vertices and shrinking.  A level then runs the
// bottom-up sources first (every vertex that one of them has not reached
// scans its own records and ORs in its neighbours' frontier masks,
// restricted to those sources, until all are found) and the top-down
// sources after (the frontier vertices of those sources push their masks,
// restricted to them).  A source whose frontier is small stays top-down, so
// it never forces full scans on the vertices it does not reach.  Every CTA
// computes the same per-source statistics and so the same choice; the masks
// produced are the same in every direction.
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
  uint8_t *depth8;            // n x V byte depths (0 unreached, 255 for 255 and more) or null
  uint32_t n_src;
  uint32_t *err;
  uint32_t *levels;           // number of expanded levels (out)
  unsigned long long *stat;   // [0] listed vertices, [1] edges expanded, [2] of them dynamic,
                              // [3] levels with bottom-up sources, [4..5] OR of the frontier masks
                              // by level parity
  unsigned long long *smf;    // [2][64] per-source frontier degree sums by level parity
  uint32_t *defer;            // bottom-up vertices handed to the pull pass (bitmap, zero between levels)
  uint32_t Vs;                // first dynamic vertex
  uint32_t dopt;              // bottom-up sources allowed (the graph is symmetric)
  __device__ __forceinline__ unsigned long long *act_slot(uint32_t level) const {
    return stat + 4 + (level & 1u);
  }
  __device__ __forceinline__ unsigned long long *smf_slot(uint32_t level) const {
    return smf + 64 * (level & 1u);
  }
};

constexpr uint64_t kBatchAlpha = 14, kBatchBeta = 24;

// Grid-wide barrier of a cooperative launch: the last of `expected` CTAs to
// arrive (default: the whole grid) releases the others by bumping the
// generation word.  A wait longer than spin_limit polls sets kErrBarrier and
// returns false instead of hanging.
__device__ __forceinline__ bool grid_barrier(unsigned int *bar, uint32_t *err, uint32_t expected = 0,
                                             uint32_t spin_limit = kSpinLimit) {
  __shared__ int s_ok;
  if (expected == 0) expected = gridDim.x;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned int gen = ld_acquire((const uint32_t *)&bar[1]);
    __threadfence();
    if (atomicAdd(&bar[0], 1u) == expected - 1) {
      bar[0] = 0;
      __threadfence();
      st_release((uint32_t *)&bar[1], gen + 1);
    } else {
      uint32_t spins = 0;
      while (ld_acquire((const uint32_t *)&bar[1]) == gen) {
        if (++spins > spin_limit) {
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
  unsigned long long act;
  unsigned long long msum[64];  // per-source degree sums of the newly reached vertices
  uint32_t bu_w[2];             // this level's bottom-up sources
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

// Records of vertex v beyond its first `skip`.
__device__ __forceinline__ uint64_t rest_deg(const PersistArgs &a, uint64_t v, uint64_t skip) {
  const uint64_t d = a.off[v + 1] - a.off[v];
  return d > skip ? d - skip : 0;
}

// Count the listed vertices of this thread's words of `bits` (those with
// records beyond `skip`) and their record sums; publish the CTA's totals.
// With `masks`, only vertices whose mask shares a bit with `sel` count.
template <int BLOCK, class SH>
__device__ __forceinline__ void count_list(const PersistArgs &a, SH &sh, const uint32_t *bits, uint64_t wb,
                                           uint64_t we, uint64_t skip, const unsigned long long *masks,
                                           unsigned long long sel, uint32_t &exc, uint64_t &exe,
                                           uint64_t &dyn) {
  uint32_t c = 0;
  uint64_t e = 0;
  dyn = 0;
  for (uint64_t w = wb; w < we; w++)
    for (uint32_t m = __ldcg(bits + w); m; m &= m - 1) {
      const uint64_t v = w * 32 + (__ffs(m) - 1);
      if (masks && !(__ldcg(masks + v) & sel)) continue;
      const uint64_t d = rest_deg(a, v, skip);
      c += d ? 1u : 0u;
      e += d;
      if (v >= a.Vs) dyn += d;
    }
  uint32_t totc;
  uint64_t tote;
  pscan<BLOCK>(sh, c, e, exc, exe, totc, tote);
  if (threadIdx.x == 0) {
    a.cta_n[blockIdx.x] = totc;
    a.cta_e[blockIdx.x] = tote;
  }
}

// After count_list and a grid barrier: this CTA's list offset (sh.red_n,
// sh.red_e) and the grid totals (sh.red_tn, sh.red_te).  Every CTA computes
// the same totals.
template <int BLOCK, class SH>
__device__ __forceinline__ void grid_totals(const PersistArgs &a, SH &sh) {
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

// Write the list (vertex, record prefix) of this thread's words of `bits` and
// the first list entry of every tile; positions come from count_list's scan.
template <uint32_t TILE>
__device__ __forceinline__ void write_list(const PersistArgs &a, const uint32_t *bits, uint64_t wb, uint64_t we,
                                           uint64_t skip, const unsigned long long *masks,
                                           unsigned long long sel, uint32_t pos, uint64_t ep,
                                           uint64_t total_n, uint64_t total_e) {
  for (uint64_t w = wb; w < we; w++)
    for (uint32_t m = __ldcg(bits + w); m; m &= m - 1) {
      const uint64_t v = w * 32 + (__ffs(m) - 1);
      if (masks && !(__ldcg(masks + v) & sel)) continue;
      const uint64_t d = rest_deg(a, v, skip);
      if (!d) continue;
      a.list[pos] = (uint32_t)v;
      a.pref[pos] = ep;
      for (uint64_t t = (ep + TILE - 1) / TILE; t * TILE < ep + d; t++) a.tile_first[t] = pos;
      pos++;
      ep += d;
    }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) a.pref[total_n] = total_e;
}

// Edge-balanced pass over the listed vertices' records (from record `skip` of
// each), TILE records per CTA tile, for the sources in `sel`.
//  push (top-down): a listed vertex's frontier mask goes to every neighbour
//    that a source of the mask has not reached (visited / next / next_any by
//    atomicOr).
//  pull (the deferred vertices of a bottom-up level): every neighbour's
//    frontier mask, restricted to the sources the listed vertex still lacks,
//    is ORed into a per-vertex accumulator in shared memory and then into the
//    vertex's next mask; visited and next_any are settled afterwards.
template <int BLOCK, int ITEMS, bool PULL>
__device__ __forceinline__ void expand_tiles(const PersistArgs &a, PersistShared<BLOCK, ITEMS> &sh,
                                             uint64_t total_n, uint64_t total_e, uint64_t skip,
                                             unsigned long long sel, const unsigned long long *cur,
                                             unsigned long long *next, uint32_t *next_any) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  const uint64_t ntiles = (total_e + TILE - 1) / TILE;
  unsigned long long pulled_s = 0, pulled_d = 0;  // pull: static / dynamic records read
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
      sh.cb[j] = a.off[v] + skip - p + pos0;
      if (PULL) sh.val[j] = ~__ldcg(a.visited + v) & sel & ~__ldcg(next + v);
      else sh.val[j] = __ldcg(cur + v) & sel;
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
        if (PULL && sh.val[l] == 0ull) {
          // every source this vertex lacked was found by an earlier tile
        } else if (idx < a.static_edges) {
          ev[it] = a.ssrc.load(idx);
          okm |= 1u << it;
          if (PULL) pulled_s++;
        } else if (idx < a.E && a.hsrc.words) {
          ev[it] = a.hsrc.load(idx);
          okm |= 1u << it;
          if (PULL) pulled_d++;
        } else {
          atomicOr(a.err, kErrEdgeIndex);
        }
      }
    }
    // probe every target before the first atomic (the reads overlap; a stale
    // visited probe only costs an extra atomic)
    unsigned long long pv[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; it++) {
      pv[it] = PULL ? 0ull : ~0ull;
      if ((okm >> it) & 1u) {
        const uint32_t v = edge_dst(ev[it]);
        if (v < a.V) pv[it] = __ldcg((PULL ? cur : a.visited) + v);
      }
    }
    if (PULL) {
      __syncthreads();  // the record bases are no longer needed: cb becomes the accumulator
      for (uint32_t j = threadIdx.x; j < nl; j += BLOCK) sh.cb[j] = 0ull;
      __syncthreads();
#pragma unroll
      for (int it = 0; it < ITEMS; it++) {
        if (!(okm & (1u << it))) continue;
        if (edge_dst(ev[it]) >= a.V) {
          atomicOr(a.err, kErrVertex);
          continue;
        }
        const unsigned long long x = pv[it] & sh.val[lv[it]];
        if (x) atomicOr(&sh.cb[lv[it]], x);
      }
      __syncthreads();
      for (uint32_t j = threadIdx.x; j < nl; j += BLOCK)
        if (sh.cb[j]) atomicOr(next + __ldcg(a.list + i0 + j), sh.cb[j]);
    } else {
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
    }
    __syncthreads();  // shared tables are rebuilt for the next tile
  }
  if (PULL) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      pulled_s += __shfl_xor_sync(0xffffffffu, pulled_s, o);
      pulled_d += __shfl_xor_sync(0xffffffffu, pulled_d, o);
    }
    if ((threadIdx.x & 31) == 0 && (pulled_s | pulled_d)) {
      atomicAdd(a.stat + 1, pulled_s + pulled_d);
      if (pulled_d) atomicAdd(a.stat + 2, pulled_d);
    }
  }
}

// Records a lane scans for one vertex in a bottom-up level before it hands
// the rest of the vertex's list to the edge-balanced pull pass.
constexpr uint64_t kBuLaneRecords = 64;
constexpr int kBuStep = 8;  // records loaded (and probed) together

// Bottom-up part of a level, for the sources in `sel`.  A warp owns 32-vertex
// words of the bitmaps; each lane scans its vertex's records (HBM for the
// static prefix, page-locked host memory beyond it) kBuStep at a time and ORs in
// its neighbours' frontier masks, restricted to the sources of `sel` that
// have not reached the vertex, until every one of them is found or kBuLaneRecords
// records are read.  A vertex with records left and sources still missing is
// deferred: its partial mask goes to next[v] and its bit to `defer`, and the
// pull pass scans the rest of its list in parallel, so no lane walks a long
// list alone.  A lane writes only its own vertex's masks and lane 0 its
// warp's words of next_any and defer, so nothing here needs an atomic.
template <int BLOCK>
__device__ __forceinline__ void bottom_up_scan(const PersistArgs &a, unsigned long long sel,
                                               const unsigned long long *cur, unsigned long long *next,
                                               uint32_t *next_any) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = (uint64_t)gridDim.x * (BLOCK / 32);
  unsigned long long ns = 0, nd = 0;  // static / dynamic records read
  // a vertex's visited mask and list bounds are fetched one word ahead, so
  // their latency overlaps the scan of the current word
  uint64_t w = ((uint64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5;
  unsigned long long vis_n = ~0ull;
  uint64_t e0_n = 0, e1_n = 0;
  auto fetch = [&](uint64_t wn) {
    const uint64_t vn = wn * 32 + lane;
    vis_n = ~0ull;
    if (wn < a.nwords && vn < a.V) {
      vis_n = __ldcg(a.visited + vn);
      e0_n = a.off[vn];
      e1_n = a.off[vn + 1];
    }
  };
  fetch(w);
  for (; w < a.nwords; w += nwarps) {
    const uint64_t v = w * 32 + lane;
    const unsigned long long vis = vis_n;
    const uint64_t e0 = e0_n, e1 = e1_n;
    fetch(w + nwarps);
    unsigned long long found = 0;
    bool defer = false;
    if (v < a.V) {
      const unsigned long long need = ~vis & sel;
      if (need) {
        const uint64_t lim = min(e1, e0 + kBuLaneRecords);
        for (uint64_t e = e0; e < lim && found != need; e += kBuStep) {
          uint32_t u[kBuStep];
#pragma unroll
          for (int j = 0; j < kBuStep; j++) {
            const uint64_t i = e + j;
            u[j] = 0xffffffffu;
            if (i >= lim) continue;
            if (i < a.static_edges) {
              u[j] = a.ssrc.load(i);
              ns++;
            } else if (i < a.E && a.hsrc.words) {
              u[j] = a.hsrc.load(i);
              nd++;
            } else {
              atomicOr(a.err, kErrEdgeIndex);
            }
          }
#pragma unroll
          for (int j = 0; j < kBuStep; j++) {
            if (u[j] < a.V) found |= __ldcg(cur + u[j]) & need;
            else if (u[j] != 0xffffffffu) atomicOr(a.err, kErrVertex);
          }
        }
        defer = found != need && lim < e1;
        if (defer) {
          next[v] = found;
        } else if (found) {
          next[v] = found;
          a.visited[v] = vis | found;
        }
      }
    }
    const uint32_t ball = __ballot_sync(0xffffffffu, found != 0ull && !defer);
    const uint32_t dball = __ballot_sync(0xffffffffu, defer);
    if (lane == 0) {
      if (ball) next_any[w] = ball;
      if (dball) a.defer[w] = dball;
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    ns += __shfl_xor_sync(0xffffffffu, ns, o);
    nd += __shfl_xor_sync(0xffffffffu, nd, o);
  }
  if (lane == 0 && (ns | nd)) {
    atomicAdd(a.stat + 1, ns + nd);
    if (nd) atomicAdd(a.stat + 2, nd);
  }
}

// Transpose of the 32 x 32 bit matrix whose row i is lane i's x: lane c
// gets column c (bit i = bit c of lane i's x).  Butterfly exchange of
// 16-, 8-, 4-, 2- and 1-bit blocks.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
  const uint32_t lane = threadIdx.x & 31;
  uint32_t m = 0x0000ffffu;
#pragma unroll
  for (int j = 16; j; j >>= 1, m ^= m << j) {
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & ~m) | ((y >> j) & m)) : ((x & m) | ((y << j) & ~m));
  }
  return x;
}

// Adds to lane c's count the vertices of this word (one per lane, masks `x`)
// that carry source c.  A transpose when many sources are present, a ballot
// per source otherwise.
__device__ __forceinline__ uint32_t word_counts(uint32_t x, uint32_t present) {
  const uint32_t lane = threadIdx.x & 31;
  if (__popc(present) > 12) return __popc(warp_transpose32(x));
  uint32_t c = 0;
  for (uint32_t m = present; m; m &= m - 1) {
    const uint32_t src = __ffs(m) - 1;
    const uint32_t n = __popc(__ballot_sync(0xffffffffu, (x >> src) & 1u));
    if (lane == src) c = n;
  }
  return c;
}

// Phase 4 of a level.  A warp takes kTallyWords consecutive 32-vertex words
// at a time (lane = vertex) and issues their loads together.  Deferred
// bottom-up vertices get their final mask into visited and next_any; the
// newly reached vertices are counted per source (hist), and for the sources
// in `msum_sel` their degrees are summed (the next level's direction
// choice); the consumed frontier is cleared.
constexpr int kTallyWords = 4;
template <int BLOCK, class SH>
__device__ __forceinline__ void level_tally(const PersistArgs &a, SH &sh, unsigned long long bu,
                                            unsigned long long msum_sel, unsigned long long all_src,
                                            uint32_t level, unsigned long long *cur,
                                            unsigned long long *next, uint32_t *cur_any, uint32_t *next_any) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = (uint64_t)gridDim.x * (BLOCK / 32);
  uint32_t cnt_lo = 0, cnt_hi = 0;  // sources lane and lane + 32
  unsigned long long ms_lo = 0, ms_hi = 0, nact = 0;
  for (uint64_t g = (((uint64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5) * kTallyWords; g < a.nwords;
       g += nwarps * kTallyWords) {
    uint32_t nw[kTallyWords], cw[kTallyWords];
#pragma unroll
    for (int j = 0; j < kTallyWords; j++) {
      const bool ok = g + j < a.nwords;
      nw[j] = ok ? __ldcg(next_any + g + j) : 0u;
      cw[j] = ok ? __ldcg(cur_any + g + j) : 0u;
      const uint32_t dm = (bu && ok) ? __ldcg(a.defer + g + j) : 0u;
      if (dm) {  // uniform: the word is the same for every lane
        const uint64_t v = (g + j) * 32 + lane;
        unsigned long long f = 0;
        if ((dm >> lane) & 1u) {
          f = __ldcg(next + v);
          if (f) a.visited[v] = __ldcg(a.visited + v) | f;
        }
        const uint32_t nb = __ballot_sync(0xffffffffu, f != 0ull);
        if (lane == 0) {
          if (nb & ~nw[j]) next_any[g + j] = nw[j] | nb;
          a.defer[g + j] = 0u;
        }
        nw[j] |= nb;
      }
    }
    unsigned long long nv[kTallyWords];
#pragma unroll
    for (int j = 0; j < kTallyWords; j++)
      nv[j] = ((nw[j] >> lane) & 1u) ? __ldcg(next + (g + j) * 32 + lane) : 0ull;
    uint64_t d[kTallyWords];
#pragma unroll
    for (int j = 0; j < kTallyWords; j++) {
      const uint64_t v = (g + j) * 32 + lane;
      d[j] = (nv[j] & msum_sel) ? a.off[v + 1] - a.off[v] : 0;
    }
#pragma unroll
    for (int j = 0; j < kTallyWords; j++) {
      if (!nw[j]) continue;  // uniform
      const unsigned long long x = nv[j] & all_src;
      nact |= x;
      const uint32_t plo = __reduce_or_sync(0xffffffffu, (uint32_t)x);
      const uint32_t phi = __reduce_or_sync(0xffffffffu, (uint32_t)(x >> 32));
      cnt_lo += word_counts((uint32_t)x, plo);
      cnt_hi += word_counts((uint32_t)(x >> 32), phi);
      const unsigned long long ms = (((unsigned long long)phi << 32) | plo) & msum_sel;
      if (ms) {
        const uint32_t dlo = (uint32_t)(d[j] & 0xffffu), dhi = (uint32_t)(d[j] >> 16);
        for (unsigned long long m = ms; m; m &= m - 1) {
          const uint32_t src = __ffsll((long long)m) - 1;
          const bool bit = (x >> src) & 1ull;
          const unsigned long long sum = __reduce_add_sync(0xffffffffu, bit ? dlo : 0u) +
                                         ((unsigned long long)__reduce_add_sync(0xffffffffu, bit ? dhi : 0u) << 16);
          if (lane == (src & 31u)) {
            if (src < 32) ms_lo += sum;
            else ms_hi += sum;
          }
        }
      }
      if (a.depth)
        for (unsigned long long b = x; b; b &= b - 1)
          a.depth[(uint64_t)(__ffsll((long long)b) - 1) * a.V + (g + j) * 32 + lane] = level + 1;
      if (a.depth8)
        for (unsigned long long b = x; b; b &= b - 1)
          a.depth8[(uint64_t)(__ffsll((long long)b) - 1) * a.V + (g + j) * 32 + lane] =
              (uint8_t)min(level + 1, 255u);
    }
#pragma unroll
    for (int j = 0; j < kTallyWords; j++) {
      if (!cw[j]) continue;  // uniform
      if ((cw[j] >> lane) & 1u) cur[(g + j) * 32 + lane] = 0ull;
      if (lane == 0) cur_any[g + j] = 0u;
    }
  }
  if (cnt_lo) atomicAdd(&sh.cnt[lane], cnt_lo);
  if (cnt_hi) atomicAdd(&sh.cnt[lane + 32], cnt_hi);
  if (ms_lo) atomicAdd(&sh.msum[lane], ms_lo);
  if (ms_hi) atomicAdd(&sh.msum[lane + 32], ms_hi);
#pragma unroll
  for (int o = 16; o; o >>= 1) nact |= __shfl_xor_sync(0xffffffffu, nact, o);
  if (lane == 0 && nact) atomicOr(&sh.act, nact);
}

// Resident threads per SM asked of the register allocator: 1024 (64
// registers a thread) for the short tiles; the long tiles keep more items in
// flight per thread and get 128 registers.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK, (ITEMS <= 4 ? 1024 : 512) / BLOCK) k_batch_persistent(PersistArgs a) {
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
  const unsigned long long all_src = a.n_src >= 64 ? ~0ull : (1ull << a.n_src) - 1ull;
  // direction state of source threadIdx.x (threads 0..63 of every CTA)
  bool src_bu = false;       // the source expands bottom-up
  uint64_t src_prev_n = 0;   // its previous frontier size
  // record count of the vertices it has reached in its top-down levels (the
  // bookkeeping sums degrees only for top-down sources, so after a bottom-up
  // stretch this undercounts and the unexplored estimate E - src_explored is
  // high: a source that has gone back to top-down is slow to switch again)
  uint64_t src_explored = 0;
  uint32_t level = 1;
  for (;; level++) {
    // sources whose frontier is not empty
    const unsigned long long act = level == 1 ? all_src : __ldcg(a.act_slot(level));
    // ---- 0. each source's direction for this level (symmetric graphs)
    unsigned long long bu = 0;
    if (a.dopt) {
      if (threadIdx.x < 64) {
        bool b = false;
        if (level > 1 && ((act >> threadIdx.x) & 1ull)) {
          const uint64_t mf = __ldcg(a.smf_slot(level) + threadIdx.x);
          const uint64_t nf = __ldcg(a.hist + (uint64_t)(level - 1) * 64 + threadIdx.x);
          const uint64_t mu = a.E > src_explored ? a.E - src_explored : 0;
          if (!src_bu) src_bu = mf > mu / kBatchAlpha;
          else src_bu = !(nf < a.V / kBatchBeta && nf < src_prev_n);
          src_prev_n = nf;
          src_explored += mf;
          b = src_bu;
        }
        const uint32_t ball = __ballot_sync(0xffffffffu, b);
        if ((threadIdx.x & 31) == 0) sh.bu_w[threadIdx.x >> 5] = ball;
      }
      __syncthreads();
      bu = (((unsigned long long)sh.bu_w[1] << 32) | sh.bu_w[0]) & act;
    }
    const unsigned long long td = act & ~bu;
    // ---- 1. count the frontier vertices of the top-down sources in this
    //         thread's words
    uint32_t exc;
    uint64_t exe, dyn_td;
    count_list<BLOCK>(a, sh, cur_any, wb, we, 0, a.dopt ? cur : nullptr, td, exc, exe, dyn_td);
    if (!grid_barrier(a.bar, a.err)) return;
    // ---- 2. grand totals, then the bottom-up and the top-down sources
    grid_totals<BLOCK>(a, sh);
    const uint64_t total_n = sh.red_tn, total_e = sh.red_te;
    const uint32_t td_pos = sh.red_n + exc;
    const uint64_t td_ep = sh.red_e + exe;
    if (total_n == 0 && bu == 0) break;  // every CTA sees the same totals
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) {
        a.stat[0] += total_n;
        if (bu) a.stat[3]++;
        *a.act_slot(level + 1) = 0ull;  // last read in phase 0 of the previous level
      }
      if (threadIdx.x < 64) a.smf_slot(level + 1)[threadIdx.x] = 0ull;
    }
    if (level >= kMaxBatchLevels) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.err, kErrLevels);
      break;
    }
    if (bu) {
      bottom_up_scan<BLOCK>(a, bu, cur, next, next_any);
      if (!grid_barrier(a.bar, a.err)) return;
      // the deferred vertices' remaining records, edge-balanced (the pull
      // pass counts the records it reads)
      uint64_t dyn;
      count_list<BLOCK>(a, sh, a.defer, wb, we, kBuLaneRecords, nullptr, 0, exc, exe, dyn);
      if (!grid_barrier(a.bar, a.err)) return;
      grid_totals<BLOCK>(a, sh);
      const uint64_t dn = sh.red_tn, de = sh.red_te;
      if (dn) {
        if (dn > a.list_cap || de / TILE + 1 >= a.tile_cap) {
          if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.err, kErrTileMap);
          break;
        }
        write_list<TILE>(a, a.defer, wb, we, kBuLaneRecords, nullptr, 0, sh.red_n + exc, sh.red_e + exe, dn,
                         de);
        if (!grid_barrier(a.bar, a.err)) return;
        expand_tiles<BLOCK, ITEMS, true>(a, sh, dn, de, kBuLaneRecords, bu, cur, next, next_any);
        // the list buffers are rebuilt for the top-down sources below
        if (!grid_barrier(a.bar, a.err)) return;
      }
    }
    if (total_n) {
      if (dyn_td) atomicAdd(a.stat + 2, (unsigned long long)dyn_td);
      if (blockIdx.x == 0 && threadIdx.x == 0) a.stat[1] += total_e;
      if (total_n > a.list_cap || total_e / TILE + 1 >= a.tile_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.err, kErrTileMap);
        break;
      }
      write_list<TILE>(a, cur_any, wb, we, 0, a.dopt ? cur : nullptr, td, td_pos, td_ep, total_n, total_e);
      if (!grid_barrier(a.bar, a.err)) return;
      expand_tiles<BLOCK, ITEMS, false>(a, sh, total_n, total_e, 0, td, cur, next, next_any);
    }
    if (!grid_barrier(a.bar, a.err)) return;
    // ---- 4. settle the deferred vertices; per-source counts of the newly
    //         reached vertices (and, for top-down sources, their degree
    //         sums), depths, and clearing of the consumed frontier
    if (threadIdx.x < 64) {
      sh.cnt[threadIdx.x] = 0;
      sh.msum[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) sh.act = 0ull;
    __syncthreads();
    level_tally<BLOCK>(a, sh, bu, a.dopt ? td & all_src : 0ull, all_src, level, cur, next, cur_any, next_any);
    __syncthreads();
    if (threadIdx.x < 64 && sh.cnt[threadIdx.x])
      atomicAdd(a.hist + (uint64_t)level * 64 + threadIdx.x, (unsigned long long)sh.cnt[threadIdx.x]);
    if (threadIdx.x < 64 && sh.msum[threadIdx.x])
      atomicAdd(a.smf_slot(level + 1) + threadIdx.x, sh.msum[threadIdx.x]);
    if (threadIdx.x == 0 && sh.act) atomicOr(a.act_slot(level + 1), sh.act);
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
