// sssp_batch.cuh — multi-source SSSP: up to 32 sources share every round, so
// that an edge record read once (from HBM or over the host link) relaxes the
// distances of every source for which its tail is active.
//
// No reference counterpart: the reference runs its SSSP sources one after
// another (SSSP/oneGraph/CalculateOpt.h:12-30, sssp_opt per source).  Each
// source's distances are those of a single-source run (exact, u32, source at
// distance 1, unreached 0xFFFFFFFF, SSSP/oneGraph/GraphMeta.h:376-381).
//
// State (device):
//   dist[v * ks + s]   distance of vertex v from source slot s (vertex-major,
//                      ks = 4, 8, 16 or 32 slots per row: the slots of one
//                      vertex share 32-byte sectors, so a probe of v serves up
//                      to 8 sources)
//   pend[v]            slots whose distance at v improved and has not been
//                      expanded yet
//   act                bitmap of vertices with pending slots to classify
//   wait               bitmap of vertices holding pending slots at or above the
//                      near threshold
// A round compacts the active bitmap (or, when it lists nothing, advances the
// threshold and compacts the waiting bitmap): a pending (vertex, slot) pair
// whose distance is below the threshold is "near" and expanded this round,
// the others wait.  This is the two-bucket near/far scheme of the single-source
// engine with one threshold shared by every slot.  Distances are exact for any
// threshold schedule: an improvement always leaves the pair pending, and a
// pending pair is eventually expanded.
#pragma once
#include "kernels.cuh"

namespace og {

constexpr uint32_t kSbMaxSources = 32;
// CTAs per SM of the relax (at most 64 registers at 256 threads) and
// positions in flight per thread, chosen with -Xptxas -v (no spills) and by
// measurement on R-MAT 23 and 27: 5 CTAs per SM at 48 registers ran 30-40 %
// slower, and a 58 % shared-memory carve-out (3 CTAs per SM, more L1) 5-8 %
// slower, than 4 CTAs per SM with the CUDA driver's carve-out.
constexpr int kSbMinBlocks = 4;
template <int KS>
constexpr int sb_positions_in_flight() { return 3; }

struct SbCompactArgs {
  uint32_t *bits;        // bitmap scanned this round: the active set, or the waiting set
  uint32_t *wait;        // the waiting set
  uint32_t v_begin, v_end;
  uint32_t w_begin, w_end, ntiles;
  const uint64_t *off;   // CSR offsets (V+1) on the device
  uint32_t *list;        // listed vertices
  uint64_t *pref;        // exclusive degree prefix, pref[n] = total
  uint32_t *tile_first;  // LBS tile map
  uint32_t *lmask;       // near slots of each listed vertex (parallel to list)
  Counts *counts;
  Lookback lb;
  uint32_t *err;
  uint64_t list_cap, tile_cap;
  uint32_t *pend;
  const uint32_t *dist;
  uint32_t ks;
  uint32_t thr;          // near threshold
  uint32_t scan_wait;    // 1: `bits` is the waiting set
  // atomicMax of (epoch << 32) | ~d over the waiting pairs (the far key of
  // the single-source compaction)
  unsigned long long *far_key;
  // masks[0] |= every pending mask classified; masks[1] |= the slots left
  // waiting
  uint32_t *masks;
  uint32_t epoch;
};

// Near slots of one row: the slots of m whose distance is below thr; the
// smallest distance among the others goes to fmin.
__device__ __forceinline__ uint32_t sb_split(const uint32_t *row, uint32_t m, uint32_t thr,
                                             uint32_t &fmin) {
  uint32_t near = 0;
  for (uint32_t t = m; t; t &= t - 1) {
    const uint32_t s = __ffs(t) - 1;
    const uint32_t d = __ldcg(row + s);
    if (d < thr) near |= 1u << s;
    else fmin = min(fmin, d);
  }
  return near;
}

// Compaction of one round for the vertex range [v_begin, v_end): the same
// tiles, ticket order and decoupled look-back as k_compact.  Every vertex of
// the scanned bitmap is classified: its near slots are consumed from pend
// (listed with their mask when the vertex has edges), its far slots stay
// pending and the vertex joins the waiting set; a scanned vertex leaves the
// active set, and leaves the waiting set once nothing of it waits.
__global__ void __launch_bounds__(kThreads) k_compact_sb(SbCompactArgs a) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_excl_n;
  __shared__ uint64_t s_excl_e;
  __shared__ int s_bad;
  __shared__ uint32_t s_wmin[kThreads / 32], s_seen[kThreads / 32], s_far[kThreads / 32];
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(a.lb.ticket, 1u);
    if (s_tile == a.ntiles - 1) *a.lb.ticket = 0u;
  }
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t w0 = a.w_begin + tile * kWordsPerCompactTile + threadIdx.x * kCompactWordsPerThread;
  uint32_t keep[kCompactWordsPerThread];
  uint32_t cnt = 0, tmin = 0xffffffffu, seen = 0, farm = 0;
  uint64_t sum = 0;
#pragma unroll
  for (uint32_t j = 0; j < kCompactWordsPerThread; j++) {
    const uint32_t w = w0 + j;
    const uint64_t vbase = (uint64_t)w * 32;
    uint32_t word = 0;
    if (w < a.w_end) {
      word = a.bits[w];
      if (vbase < a.v_begin) {
        const uint32_t sh = a.v_begin - (uint32_t)vbase;
        word = sh >= 32 ? 0 : word & (0xffffffffu << sh);
      }
      if (vbase + 32 > a.v_end) {
        const uint64_t k = a.v_end > vbase ? a.v_end - vbase : 0;
        word = k >= 32 ? word : word & ((1u << k) - 1u);
      }
    }
    uint32_t kp = 0, to_wait = 0, clr = 0;
    for (uint32_t m = word; m; m &= m - 1) {
      const uint32_t b = __ffs(m) - 1;
      const uint64_t v = vbase + b;
      const uint32_t pm = __ldcg(a.pend + v);
      uint32_t fmin = 0xffffffffu;
      const uint32_t near = sb_split(a.dist + v * a.ks, pm, a.thr, fmin);
      const uint32_t far = pm & ~near;
      seen |= pm;
      if (far) {
        farm |= far;
        tmin = min(tmin, fmin);
        if (!a.scan_wait) to_wait |= 1u << b;
      } else if (a.scan_wait) {
        clr |= 1u << b;  // nothing of it waits any more
      }
      if (!a.scan_wait) clr |= 1u << b;  // classified: leaves the active set
      if (near) {
        const uint64_t d = a.off[v + 1] - a.off[v];
        if (d) {
          kp |= 1u << b;
          cnt++;
          sum += d;
        } else {
          a.pend[v] = far;  // no edges: its near slots are final here
        }
      }
    }
    keep[j] = kp;
    if (to_wait) atomicOr(a.wait + w, to_wait);
    if (clr) atomicAnd(a.bits + w, ~clr);
  }
  {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t wm = __reduce_min_sync(0xffffffffu, tmin);
    const uint32_t ws = __reduce_or_sync(0xffffffffu, seen);
    const uint32_t wf = __reduce_or_sync(0xffffffffu, farm);
    if (lane == 0) {
      s_wmin[warp] = wm;
      s_seen[warp] = ws;
      s_far[warp] = wf;
    }
  }
  uint32_t ex_n, tot_n;
  uint64_t ex_e, tot_e;
  block_scan_pair(cnt, sum, ex_n, ex_e, tot_n, tot_e);  // its barriers publish the warp results
  if (threadIdx.x == 0) {
    uint32_t m = 0xffffffffu, o = 0, f = 0;
#pragma unroll
    for (int i = 0; i < kThreads / 32; i++) {
      m = min(m, s_wmin[i]);
      o |= s_seen[i];
      f |= s_far[i];
    }
    if (m != 0xffffffffu) atomicMax(a.far_key, ((unsigned long long)a.epoch << 32) | (~m & 0xffffffffu));
    if (o) atomicOr(a.masks, o);
    if (f) atomicOr(a.masks + 1, f);
  }
  if (threadIdx.x < 32) {
    uint32_t pn;
    uint64_t pe;
    int bad;
    lookback_prefix(a.lb, tile, a.epoch, tot_n, tot_e, a.err, pn, pe, bad);
    if (threadIdx.x == 0) {
      if (!bad && (uint64_t)pn + tot_n > a.list_cap) {
        atomicOr(a.err, kErrTileMap);
        bad = 1;
      }
      s_excl_n = pn;
      s_excl_e = pe;
      s_bad = bad;
      if (!bad && tile == a.ntiles - 1) {
        a.counts->n = pn + tot_n;
        a.counts->total = pe + tot_e;
        a.pref[pn + tot_n] = pe + tot_e;
      }
    }
  }
  __syncthreads();
  if (s_bad) return;  // positions unknown: write nothing (near slots stay pending)
  uint32_t pos = s_excl_n + ex_n;
  uint64_t ep = s_excl_e + ex_e;
#pragma unroll
  for (uint32_t j = 0; j < kCompactWordsPerThread; j++) {
    const uint64_t vbase = (uint64_t)(w0 + j) * 32;
    for (uint32_t m = keep[j]; m; m &= m - 1) {
      const uint32_t b = __ffs(m) - 1;
      const uint64_t v = vbase + b;
      const uint64_t d = a.off[v + 1] - a.off[v];
      // the same classification as above (nothing changed pend or dist since)
      const uint32_t pm = __ldcg(a.pend + v);
      uint32_t fmin = 0xffffffffu;
      const uint32_t near = sb_split(a.dist + v * a.ks, pm, a.thr, fmin);
      a.lmask[pos] = near;
      a.pend[v] = pm & ~near;
      a.list[pos] = (uint32_t)v;
      a.pref[pos] = ep;
      for (uint64_t t = (ep + kTile - 1) / kTile; t * kTile < ep + d; t++) {
        if (t >= a.tile_cap) {
          atomicOr(a.err, kErrTileMap);
          break;
        }
        a.tile_first[t] = pos;
      }
      pos++;
      ep += d;
    }
  }
}

// Relax of the listed vertices' near slots: for an edge (u, v, w) and every
// near slot s of u, dist[v][s] = min(dist[v][s], dist[u][s] + w); a slot that
// improved becomes pending at v and v joins the active set.  The probe reads
// v's distance for u's first near slot, the common case of one slot.  u's row
// is read through L1: a stale (higher) value only yields a larger candidate,
// and the improvement that lowered it left the slot pending at u, so u is
// expanded again with the new value.
struct SbOp {
  using Val = uint2;  // {near slots, vertex}
  static constexpr bool kNeedVal = true;
  static constexpr bool kProbeVal = true;
  // lmask is parallel to the list allocation that starts at list0 (both
  // regions' lists), so a list entry's mask sits at the same offset
  const uint32_t *list0;
  const uint32_t *lmask;
  uint32_t *dist, *pend, *act, *err;
  uint32_t V, ks;
  __device__ Val src_val(uint32_t v) const { return make_uint2(0u, v); }
  __device__ Val list_val(uint32_t v, const uint32_t *entry) const {
    return make_uint2(__ldcg(lmask + (entry - list0)), v);
  }
  using Probe = uint32_t;
  template <class Edge>
  __device__ __forceinline__ Probe probe(Edge) const {
    return 0u;
  }
  template <class Edge>
  __device__ __forceinline__ Probe probe_v(Edge e, Val val) const {
    const uint32_t v = edge_dst(e);
    if (v >= V || !val.x) return 0u;
    return __ldcg(dist + (uint64_t)v * ks + (__ffs(val.x) - 1));
  }
  template <class Edge>
  __device__ __forceinline__ void relax(Edge e, Val val, uint64_t, Probe p) const {
    const uint32_t v = edge_dst(e);
    if (v >= V) {
      atomicOr(err, kErrVertex);
      return;
    }
    uint32_t m = val.x;
    if (!m) return;
    const uint32_t w = edge_w(e);
    const uint32_t *ru = dist + (uint64_t)val.y * ks;
    uint32_t *rv = dist + (uint64_t)v * ks;
    uint32_t nb = 0;
    {
      const uint32_t s = __ffs(m) - 1;
      const uint32_t cand = ru[s] + w;
      if (cand < p) {
        atomicMin(rv + s, cand);
        nb |= 1u << s;
      }
      m &= m - 1;
    }
    for (; m; m &= m - 1) {
      const uint32_t s = __ffs(m) - 1;
      const uint32_t cand = ru[s] + w;
      if (cand < __ldcg(rv + s)) {
        atomicMin(rv + s, cand);
        nb |= 1u << s;
      }
    }
    if (nb) {
      atomicOr(pend + v, nb);
      atomicOr(act + (v >> 5), 1u << (v & 31));
    }
  }
};

// One LBS tile of the multi-source relax, a thread per edge position as in
// lbs_tile.  For each of its U positions a thread loads the edge record,
// then v's row 8 slots at a time as two 16-byte loads (one 32-byte sector;
// a 4-slot row is one 16-byte load),
// and relaxes u's near slots of that chunk from registers: the slot index is
// a compile-time loop, so the row never leaves registers.  u's distance is
// read through L1 (u's row repeats along its adjacency in the tile).  The
// slots a position improved reach v's pending mask and the active bitmap in
// one atomic each.
template <class Src, int KS>
__device__ __forceinline__ void sb_tile(const LbsArgs &a, const Src &src, const SbOp &op,
                                        LbsShared<uint2> &sh, uint64_t k) {
  static_assert(KS == 4 || KS == 8 || KS == 16 || KS == 32, "row width");
  constexpr int C = KS < 8 ? KS : 8;  // slots per chunk
  constexpr int U = sb_positions_in_flight<KS>();  // positions in flight per thread
  const uint64_t pos0 = k * kTile;
  if (pos0 >= a.pos_end) return;
  const uint32_t tlen = (uint32_t)(min(pos0 + kTile, a.pos_end) - pos0);
  uint32_t i0;
  const uint32_t nl = lbs_setup<true>(a, src, op, sh, k, pos0, i0);
  if (nl == 0) return;
  for (uint32_t base = 0; base < tlen; base += U * kThreads) {
    typename Src::Item ev[U];
    uint2 val[U];
    uint32_t okm = 0;
#pragma unroll
    for (int j = 0; j < U; j++) {
      const uint32_t x = base + j * kThreads + threadIdx.x;
      val[j] = make_uint2(0u, 0u);
      if (x < tlen) {
        const uint32_t l = sh.map[x];
        val[j] = sh.val[l];
        ev[j] = src.at(sh.cb[l], x);
        okm |= 1u << j;
      }
    }
    uint32_t nb[U];
#pragma unroll
    for (int j = 0; j < U; j++) {
      nb[j] = 0;
      if ((okm >> j) & 1u) {
        if (edge_dst(ev[j]) >= op.V) {
          atomicOr(op.err, kErrVertex);
          okm &= ~(1u << j);
        }
      }
    }
    constexpr uint32_t cmask = (1u << C) - 1u;
#pragma unroll
    for (int c = 0; c < KS / C; c++) {
      uint4 lo[U], hi[U];
#pragma unroll
      for (int j = 0; j < U; j++) {
        if (((okm >> j) & 1u) && ((val[j].x >> (C * c)) & cmask)) {
          const uint4 *r = (const uint4 *)(op.dist + (uint64_t)edge_dst(ev[j]) * KS + C * c);
          lo[j] = __ldcg(r);
          if constexpr (C == 8) hi[j] = __ldcg(r + 1);
        }
      }
#pragma unroll
      for (int j = 0; j < U; j++) {
        const uint32_t cm = ((okm >> j) & 1u) ? (val[j].x >> (C * c)) & cmask : 0u;
        if (!cm) continue;
        const uint32_t v = edge_dst(ev[j]);
        const uint32_t w = edge_w(ev[j]);
        const uint32_t *ru = op.dist + (uint64_t)val[j].y * KS + C * c;
        uint32_t *rv = op.dist + (uint64_t)v * KS + C * c;
        uint32_t d[8] = {lo[j].x, lo[j].y, lo[j].z, lo[j].w, 0u, 0u, 0u, 0u};
        if constexpr (C == 8) {
          d[4] = hi[j].x;
          d[5] = hi[j].y;
          d[6] = hi[j].z;
          d[7] = hi[j].w;
        }
#pragma unroll
        for (int t = 0; t < C; t++) {
          if ((cm >> t) & 1u) {
            const uint32_t cand = ru[t] + w;
            // distances only fall during a launch: cand < d[t] means the
            // pair improves in this launch (here, or lower by another
            // thread that marks it pending too), so no old value is waited for
            if (cand < d[t]) {
              atomicMin(rv + t, cand);
              nb[j] |= 1u << (C * c + t);
            }
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < U; j++) {
      if (nb[j]) {
        const uint32_t v = edge_dst(ev[j]);
        atomicOr(op.pend + v, nb[j]);
        atomicOr(op.act + (v >> 5), 1u << (v & 31));
      }
    }
  }
}

template <class Src, int KS>
__global__ void __launch_bounds__(kThreads, kSbMinBlocks) k_sb_relax(LbsArgs a, Src src, SbOp op) {
  __shared__ LbsShared<uint2> sh;
  sb_tile<Src, KS>(a, src, op, sh, a.pos_begin / kTile + blockIdx.x);
}

// Both regions in one launch, tiles interleaved as in k_lbs_pair.
template <class Src0, class Src1, int KS>
__global__ void __launch_bounds__(kThreads, kSbMinBlocks) k_sb_relax_pair(LbsArgs a0, Src0 s0, LbsArgs a1, Src1 s1, SbOp op,
                                                            uint64_t n0, uint64_t n) {
  __shared__ LbsShared<uint2> sh;
  const PairTile pt = pair_split_cta(n0, n);
  static_assert(std::is_same<Src0, Src1>::value, "one tile body for both regions");
  // one inlined tile body for both regions (two would double its registers)
  const bool st = pt.r == 0;
  sb_tile<Src0, KS>(st ? a0 : a1, st ? s0 : s1, op, sh, (st ? a0.pos_begin : a1.pos_begin) / kTile + pt.t);
}

// Slots in `cols` of every row set to unreached (one thread per row).
__global__ void k_sb_clear_cols(uint32_t *dist, uint64_t rows, uint32_t ks, uint32_t cols) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < rows;
       v += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t *r = dist + v * ks;
    for (uint32_t m = cols; m; m &= m - 1) r[__ffs(m) - 1] = 0xffffffffu;
  }
}

// Seeds slot slots[i] with source srcs[i]: distance 1, pending, active.
__global__ void k_sb_seed(const uint32_t *srcs, const uint32_t *slots, uint32_t n, uint32_t *dist,
                          uint32_t ks, uint32_t *pend, uint32_t *act, uint32_t V, uint32_t *err) {
  const uint32_t i = threadIdx.x;
  if (i >= n) return;
  const uint32_t v = srcs[i], s = slots[i];
  if (v >= V || s >= ks) {
    atomicOr(err, kErrVertex);
    return;
  }
  dist[(uint64_t)v * ks + s] = 1u;
  atomicOr(pend + v, 1u << s);
  atomicOr(act + (v >> 5), 1u << (v & 31));
}

// Per-slot {vertices reached, sum of their distances} for the slots in
// `cols`: out[2 s] and out[2 s + 1] (zeroed by the caller).  A warp covers
// 32 consecutive distances, so lane l always reads slot l % ks.
__global__ void __launch_bounds__(kThreads) k_sb_checks(const uint32_t *dist, uint64_t V, uint32_t ks,
                                                        uint32_t cols, unsigned long long *out) {
  __shared__ unsigned long long s_c[kSbMaxSources], s_s[kSbMaxSources];
  if (threadIdx.x < kSbMaxSources) {
    s_c[threadIdx.x] = 0;
    s_s[threadIdx.x] = 0;
  }
  __syncthreads();
  const uint64_t n = V * ks;
  const uint32_t lane = threadIdx.x & 31, s = lane % ks;
  unsigned long long c = 0, sum = 0;
  if ((cols >> s) & 1u) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < n;
         x += (uint64_t)gridDim.x * blockDim.x) {
      const uint32_t d = __ldcg(dist + x);
      if (d != 0xffffffffu) {
        c++;
        sum += d;
      }
    }
  }
  for (uint32_t o = ks; o < 32; o <<= 1) {
    c += __shfl_xor_sync(0xffffffffu, c, o);
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
  }
  if (lane < ks && ((cols >> s) & 1u)) {
    atomicAdd(&s_c[s], c);
    atomicAdd(&s_s[s], sum);
  }
  __syncthreads();
  if (threadIdx.x < kSbMaxSources && ((cols >> threadIdx.x) & 1u) && threadIdx.x < ks) {
    atomicAdd(out + 2 * threadIdx.x, s_c[threadIdx.x]);
    atomicAdd(out + 2 * threadIdx.x + 1, s_s[threadIdx.x]);
  }
}

// Column s of the distance rows as a V-array.
__global__ void k_sb_column(const uint32_t *dist, uint64_t V, uint32_t ks, uint32_t s, uint32_t *out) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V;
       v += (uint64_t)gridDim.x * blockDim.x)
    out[v] = __ldcg(dist + v * ks + s);
}

}  // namespace og
