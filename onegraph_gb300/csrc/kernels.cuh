// kernels.cuh — sm_103a kernels of the out-of-memory engine.
//
//  k_compact   frontier bitmap -> compacted vertex list + u64 degree prefix +
//              LBS tile map, one pass with a decoupled look-back scan.  Replaces
//              setStaticAndOverloadLabelBool / myReduction / myExclusive_scan /
//              setStaticActiveNodeArray / setOverloadNodePointerSwap and the
//              host degree scan (BFS/oneGraph_BFS/gpu_kernels.h:243-379,
//              CalculateOpt.h:78-124) and the Subway generator's
//              flag/scan/queue/pointer steps (PR/sbw/subgraph_generator.h:57-234).
//  k_lbs<Op>   edge-balanced ("load-balanced search") expansion: every CTA owns
//              2048 consecutive edge positions of the compacted list, whatever
//              the degrees; columns are read coalesced.  Op = BFS / SSSP / CC
//              relax (gpu_kernels.h:180-241, SSSP :106-203, CC :105-157) or
//              the dynamic-region gather from page-locked host memory
//              (GraphMeta.h:471-506 fillEdgeArrByMultiThread).
//  k_pr_*      PageRank pull sum with a deterministic segmented reduction
//              (PR/OneGraph/gpu_kernels.h:107-158) and the rank update with an
//              FP64 L1 reduction (gpu_kernels.h:295-319).
#pragma once
#include <cuda/atomic>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace og {

constexpr int kThreads = 256;
constexpr uint32_t kTile = 2048;             // LBS edge positions per CTA
constexpr uint32_t kItems = kTile / kThreads;  // 8
constexpr uint32_t kCompactWordsPerThread = 4;
constexpr uint32_t kWordsPerCompactTile = kThreads * kCompactWordsPerThread;  // 32768 vertices

// device error bits (OR-ed into the engine's error word)
constexpr uint32_t kErrLookback = 1u;    // look-back wait gave up
constexpr uint32_t kErrEdgeIndex = 2u;   // edge index outside the array
constexpr uint32_t kErrVertex = 4u;      // column >= V
constexpr uint32_t kErrTileMap = 8u;     // LBS tile map inconsistent

constexpr uint32_t kSpinLimit = 1u << 24;

// Nanosecond global timer (the same clock on every SM).
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Launch timer of the device-driven rounds: a one-thread kernel enqueued
// right before (end = 0) and right after (end = 1) a gated launch, in the
// same captured stream.  Stream order puts the first stamp before the launch
// starts and the second after it ends; kt[0] holds the start, kt[1] the
// accumulated ns.  Rounds whose gate is closed add nothing.
__global__ void k_stamp(const uint32_t *go, unsigned long long *kt, int end) {
  if (*go == 0u) return;
  const unsigned long long t = globaltimer_ns();
  if (end) kt[1] += t - kt[0];
  else kt[0] = t;
}


struct Counts {
  uint32_t n;        // compacted vertices
  uint32_t far_min;  // near/far split: smallest value left for later rounds
  uint64_t total;    // sum of their degrees (edge positions)
};

struct Lookback {
  uint32_t *status;  // (epoch << 2) | state; state 1 aggregate, 2 inclusive prefix
  uint32_t *agg_n;
  unsigned long long *agg_e;
  uint32_t *inc_n;
  unsigned long long *inc_e;
  uint32_t *ticket;
};

struct CompactArgs {
  const uint32_t *bits;  // frontier bitmap
  uint32_t v_begin, v_end;
  uint32_t w_begin, w_end, ntiles;
  const uint64_t *off;   // CSR offsets (V+1) on the device
  uint32_t *list;
  uint64_t *pref;        // exclusive degree prefix, pref[n] = total
  uint32_t *tile_first;  // LBS tile -> list index of the vertex holding its first position
  Counts *counts;
  Lookback lb;
  uint32_t *err;
  uint64_t list_cap;     // entries of list (pref has list_cap + 1)
  uint64_t tile_cap;     // entries of tile_first
  // near/far split (SSSP): when split != 0 only vertices with value < thr
  // are listed; the others stay waiting: they are OR-ed into far_bits (when
  // not null) and the smallest of their values goes to *far_min.  Vertices
  // that leave the waiting state (value < thr) have their bit cleared in
  // clear_bits (when not null).  The value is read before the offsets, so a
  // waiting vertex costs 4 bytes.
  const uint32_t *value;
  uint32_t thr;
  uint32_t split;
  uint32_t *far_bits;
  // atomicMax of (epoch << 32) | ~value over the waiting vertices: a key of
  // an older epoch (or zeroed memory) is always smaller, and within an epoch
  // the largest ~value is the smallest value
  unsigned long long *far_key;
  uint32_t *clear_bits;
  // Launch epoch in [1, 2^30): status words of other epochs read as empty, so
  // the status array needs no clearing between launches.  The CTA that takes
  // the last ticket resets the ticket counter for the next launch.
  uint32_t epoch;
  // Device-driven loops (launches replayed from a CUDA graph): when not null,
  // the epoch is read from *epoch_ptr and the launch does nothing while
  // *run_flag is 0.
  const uint32_t *epoch_ptr;
  const uint32_t *run_flag;
  const uint32_t *thr_ptr;  // when not null, thr is read from *thr_ptr
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  return cuda::atomic_ref<const uint32_t, cuda::thread_scope_device>(*p).load(
      cuda::memory_order_acquire);
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
  cuda::atomic_ref<uint32_t, cuda::thread_scope_device>(*p).store(v, cuda::memory_order_release);
}

// Block-wide exclusive scan of (u32, u64) pairs; returns the block totals.
__device__ __forceinline__ void block_scan_pair(uint32_t cnt, uint64_t sum, uint32_t &ex_cnt,
                                                uint64_t &ex_sum, uint32_t &tot_cnt,
                                                uint64_t &tot_sum) {
  __shared__ uint32_t s_wc[kThreads / 32];
  __shared__ uint64_t s_ws[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t ic = cnt;
  uint64_t is = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t c = __shfl_up_sync(0xffffffffu, ic, d);
    const uint64_t s = __shfl_up_sync(0xffffffffu, is, d);
    if (lane >= d) {
      ic += c;
      is += s;
    }
  }
  if (lane == 31) {
    s_wc[warp] = ic;
    s_ws[warp] = is;
  }
  __syncthreads();
  if (warp == 0) {
    uint32_t wc = lane < kThreads / 32 ? s_wc[lane] : 0;
    uint64_t ws = lane < kThreads / 32 ? s_ws[lane] : 0;
#pragma unroll
    for (int d = 1; d < kThreads / 32; d <<= 1) {
      const uint32_t c = __shfl_up_sync(0xffffffffu, wc, d);
      const uint64_t s = __shfl_up_sync(0xffffffffu, ws, d);
      if (lane >= d) {
        wc += c;
        ws += s;
      }
    }
    if (lane < kThreads / 32) {
      s_wc[lane] = wc;  // inclusive warp prefixes
      s_ws[lane] = ws;
    }
  }
  __syncthreads();
  const uint32_t wpc = warp ? s_wc[warp - 1] : 0;
  const uint64_t wps = warp ? s_ws[warp - 1] : 0;
  ex_cnt = wpc + ic - cnt;
  ex_sum = wps + is - sum;
  tot_cnt = s_wc[kThreads / 32 - 1];
  tot_sum = s_ws[kThreads / 32 - 1];
  __syncthreads();  // shared arrays are reused by the next call
}

// Warp-wide decoupled look-back of compaction tile `tile` (called by all 32
// lanes of warp 0): publishes the tile's totals (tot_n, tot_e) and returns in
// (pn, pe) the exclusive prefix of the tiles before it.  Each pass reads the
// status of the 32 nearest unaccounted predecessors at once, sums their
// aggregates up to the nearest one holding an inclusive prefix, and stops
// there; tiles before the first count as an inclusive prefix of 0.  Waits
// are bounded by `spin_limit` polls: a status that never appears sets
// kErrLookback in *err and bad = 1 (the caller then writes nothing), and the
// tile still publishes an inclusive prefix so that successors never wait
// forever.
__device__ __forceinline__ void lookback_prefix(const Lookback &lb, uint32_t tile, uint32_t epoch,
                                                uint32_t tot_n, uint64_t tot_e, uint32_t *err,
                                                uint32_t &pn, uint64_t &pe, int &bad,
                                                uint32_t spin_limit = kSpinLimit) {
  const int lane = threadIdx.x & 31;
  pn = 0;
  pe = 0;
  bad = 0;
  if (tile == 0) {
    if (lane == 0) {
      lb.inc_n[0] = tot_n;
      lb.inc_e[0] = tot_e;
      __threadfence();
      st_release(&lb.status[0], (epoch << 2) | 2u);
    }
    return;
  }
  if (lane == 0) {
    lb.agg_n[tile] = tot_n;
    lb.agg_e[tile] = tot_e;
    __threadfence();
    st_release(&lb.status[tile], (epoch << 2) | 1u);
  }
  for (int p = (int)tile - 1;; p -= 32) {
    const int q = p - lane;  // lane 0: nearest predecessor of the window
    uint32_t st = 2u;
    if (q >= 0) {
      uint32_t spins = 0;
      for (;;) {
        const uint32_t raw = ld_acquire(&lb.status[q]);
        st = (raw >> 2) == epoch ? (raw & 3u) : 0u;
        if (st != 0u || ++spins > spin_limit) break;
        __nanosleep(64);
      }
    }
    __syncwarp();
    if (__any_sync(0xffffffffu, st == 0u)) {  // bounded wait expired: report, never hang
      if (lane == 0) atomicOr(err, kErrLookback);
      bad = 1;
      break;
    }
    const unsigned incl = __ballot_sync(0xffffffffu, st == 2u);
    const int k = incl ? __ffs(incl) - 1 : 32;
    uint32_t vn = 0;
    uint64_t ve = 0;
    if (q >= 0 && lane < k) {
      vn = __ldcg(&lb.agg_n[q]);
      ve = __ldcg(&lb.agg_e[q]);
    } else if (q >= 0 && lane == k) {
      vn = __ldcg(&lb.inc_n[q]);
      ve = __ldcg(&lb.inc_e[q]);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      vn += __shfl_xor_sync(0xffffffffu, vn, o);
      ve += __shfl_xor_sync(0xffffffffu, ve, o);
    }
    pn += vn;
    pe += ve;
    if (k < 32) break;
  }
  if (lane == 0) {
    lb.inc_n[tile] = pn + tot_n;
    lb.inc_e[tile] = pe + tot_e;
    __threadfence();
    st_release(&lb.status[tile], (epoch << 2) | 2u);  // published even when bad
  }
}

// Frontier compaction for the vertex range [v_begin, v_end).  Four
// consecutive bitmap words (128 vertices) per thread, 1024 words per CTA
// tile, tiles ordered by a ticket so that every predecessor a tile waits for
// is already running.
__global__ void __launch_bounds__(kThreads) k_compact(CompactArgs a) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_excl_n;
  __shared__ uint64_t s_excl_e;
  __shared__ int s_bad;
  if (a.run_flag && *a.run_flag == 0u) return;  // every CTA of the launch reads the same flag
  if (a.epoch_ptr) a.epoch = *a.epoch_ptr;
  if (a.thr_ptr) a.thr = *a.thr_ptr;
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(a.lb.ticket, 1u);
    if (s_tile == a.ntiles - 1) *a.lb.ticket = 0u;  // every CTA of this launch has its ticket
  }
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t w0 = a.w_begin + tile * kWordsPerCompactTile + threadIdx.x * kCompactWordsPerThread;
  // drop vertices without edges: nothing to expand
  uint32_t keep[kCompactWordsPerThread];
  uint32_t cnt = 0, tmin = 0xffffffffu;  // smallest waiting value of this thread
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
    uint32_t kp = 0, far = 0, leave = 0;
    for (uint32_t m = word; m; m &= m - 1) {
      const uint32_t b = __ffs(m) - 1;
      const uint64_t v = vbase + b;
      if (a.split) {
        const uint32_t x = __ldcg(a.value + v);
        if (x >= a.thr) {
          far |= 1u << b;
          tmin = min(tmin, x);
          continue;
        }
        leave |= 1u << b;
      }
      const uint64_t d = a.off[v + 1] - a.off[v];
      if (!d) continue;
      kp |= 1u << b;
      cnt++;
      sum += d;
    }
    keep[j] = kp;
    if (far && a.far_bits) atomicOr(a.far_bits + w, far);
    if (leave && a.clear_bits) atomicAnd(a.clear_bits + w, ~leave);
  }
  uint32_t ex_n, tot_n;
  uint64_t ex_e, tot_e;
  // smallest waiting value of the CTA: one far-key atomic per CTA
  __shared__ uint32_t s_wmin[kThreads / 32];
  if (a.far_key) {
    const uint32_t wm = __reduce_min_sync(0xffffffffu, tmin);
    if ((threadIdx.x & 31) == 0) s_wmin[threadIdx.x >> 5] = wm;
  }
  block_scan_pair(cnt, sum, ex_n, ex_e, tot_n, tot_e);  // its barriers publish s_wmin
  if (a.far_key && threadIdx.x == 0) {
    uint32_t m = 0xffffffffu;
#pragma unroll
    for (int i = 0; i < kThreads / 32; i++) m = min(m, s_wmin[i]);
    if (m != 0xffffffffu) atomicMax(a.far_key, ((unsigned long long)a.epoch << 32) | (~m & 0xffffffffu));
  }
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    uint32_t pn = 0;
    uint64_t pe = 0;
    int bad = 0;
    lookback_prefix(a.lb, tile, a.epoch, tot_n, tot_e, a.err, pn, pe, bad);
    if (lane == 0) {
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
  if (s_bad) return;  // positions unknown: write nothing
  uint32_t pos = s_excl_n + ex_n;
  uint64_t ep = s_excl_e + ex_e;
#pragma unroll
  for (uint32_t j = 0; j < kCompactWordsPerThread; j++) {
    const uint64_t vbase = (uint64_t)(w0 + j) * 32;
    for (uint32_t m = keep[j]; m; m &= m - 1) {
      const uint32_t b = __ffs(m) - 1;
      const uint64_t v = vbase + b;
      const uint64_t d = a.off[v + 1] - a.off[v];
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

// ------------------------------------------------------------------ LBS

struct LbsArgs {
  const uint32_t *list;
  const uint64_t *pref;
  const uint32_t *tile_first;
  uint32_t n;            // list length
  uint64_t total;        // pref[n]
  uint64_t pos_begin;    // multiple of kTile
  uint64_t pos_end;
  const uint64_t *off;   // CSR mode: edge index = off[v] - pref[i] + q
  uint64_t stage_base;   // staging mode (off == nullptr): index = q - stage_base
  uint64_t edge_bound;   // entries addressable through the edge pointer
  uint32_t *err;
};

// Edge sources.  Staging buffers hold unpacked edges: u32 columns plus, for
// weighted graphs, weights in the narrowest width that holds them (W =
// uint8_t / uint16_t / uint32_t).  The static region and the page-locked host
// copy hold bit-packed records (SrcP).  A source yields one edge as a u32
// column or a {column, weight} pair; BFS, CC and PageRank read columns only.
//
// The LBS tiles address a vertex's edges through a cursor: cur(e) is the
// cursor of edge index e, at(c, x) the edge x positions after cursor c.
// Unpacked sources use the edge index itself; packed records use the bit
// offset, so a position costs a 32-bit multiply and a 64-bit add instead of a
// 64-bit multiply.  Cursor arithmetic is modulo 2^64 (a vertex that starts
// after the tile's first position has a "negative" base).
struct SrcU {
  using Item = uint32_t;
  const uint32_t *col;
  __device__ __forceinline__ Item load(uint64_t i) const { return col[i]; }
  __device__ __forceinline__ uint64_t cur(uint64_t e) const { return e; }
  __device__ __forceinline__ Item at(uint64_t c, uint32_t x) const { return col[c + x]; }
};
template <class W>
struct SrcW {
  using Item = uint2;
  const uint32_t *col;
  const W *w;
  __device__ __forceinline__ Item load(uint64_t i) const { return make_uint2(col[i], (uint32_t)w[i]); }
  __device__ __forceinline__ uint64_t cur(uint64_t e) const { return e; }
  __device__ __forceinline__ Item at(uint64_t c, uint32_t x) const { return load(c + x); }
};
// Bit-packed records (the page-locked host copy and the static region):
// record i holds bits [i*bpe, (i+1)*bpe) of `words`, column in the low bc
// bits, weight - wmin above it.  A record spans at most two words when
// bpe <= 33, else three; arrays carry two padding words at the end, so the
// reads below stay inside the array for every i below the record count.
// Consecutive lanes read consecutive records: the two loads of a warp touch
// the same bpe*4 contiguous bytes.
template <bool kW>
struct SrcP {
  using Item = typename std::conditional<kW, uint2, uint32_t>::type;
  const uint32_t *words;
  uint32_t bpe, bc, wmin;
  __device__ __forceinline__ uint64_t bits(uint64_t i) const {
    const uint64_t b = i * bpe;
    const uint64_t q = b >> 5;
    const uint32_t r = (uint32_t)b & 31u;
    uint64_t x = (((uint64_t)words[q + 1] << 32) | words[q]) >> r;
    if (r + bpe > 64) x |= (uint64_t)words[q + 2] << (64 - r);
    return x;
  }
  __device__ __forceinline__ Item load(uint64_t i) const {
    const uint64_t x = bits(i);
    const uint32_t col = bc >= 32 ? (uint32_t)x : (uint32_t)x & ((1u << bc) - 1u);
    if constexpr (kW) {
      const uint32_t bw = bpe - bc;
      const uint64_t w = bw == 0 ? 0 : (x >> bc) & ((bw >= 32) ? 0xffffffffull : ((1ull << bw) - 1));
      return make_uint2(col, (uint32_t)w + wmin);
    } else {
      return col;
    }
  }
  __device__ __forceinline__ uint64_t cur(uint64_t e) const { return e * bpe; }
  // x below 2^26 / bpe (a tile's positions).  The column is the low bc <= 32
  // bits of the record, so two words and one funnel shift hold it whatever
  // bpe is; a weight above it may need a third word.
  __device__ __forceinline__ Item at(uint64_t c, uint32_t x) const {
    const uint64_t b = c + x * bpe;
    return decode(words + (b >> 5), (uint32_t)b & 31u);
  }
  // The record starting at bit r of w[0] (w[1], w[2] hold its rest).
  __device__ __forceinline__ Item decode(const uint32_t *w, uint32_t r) const {
    const uint32_t lo = w[0], hi = w[1];
    const uint32_t f = __funnelshift_r(lo, hi, r);
    const uint32_t col = bc >= 32 ? f : f & ((1u << bc) - 1u);
    if constexpr (kW) {
      const uint32_t bw = bpe - bc;
      uint64_t y = (((uint64_t)hi << 32) | lo) >> r;
      if (r + bpe > 64) y |= (uint64_t)w[2] << (64 - r);
      const uint64_t wt = bw == 0 ? 0 : (y >> bc) & ((bw >= 32) ? 0xffffffffull : ((1ull << bw) - 1));
      return make_uint2(col, (uint32_t)wt + wmin);
    } else {
      return col;
    }
  }
};

// Dynamic-region records with fragment slots (the static-region replacement
// the reference declares as bfs_kernelStaticSwap / recordFragmentVisit,
// BFS/oneGraph_BFS/gpu_kernels.h:46-66,153-176): the page-locked record
// stream is cut into fragments of 2^fs words, and slot_of[f] >= 0 names a
// device slot holding a copy of fragment f followed by the stream's next
// words (a slot is 2^fs + kFragPad words), so a record whose first word lies
// in the fragment is read whole from the slot.  Other records are read from
// the host stream, which holds every record: slots only redirect reads, and
// results never depend on which fragments hold one.  The tile setup picks
// each vertex's source once (cur_range); note() counts, per fragment, the
// records a tile lists (by their first word); the host's replacement policy
// reads the counts between rounds.  The slot table only changes between
// launches.
constexpr uint32_t kFragPad = 4;  // words after a fragment's copy (keeps slots 16-byte aligned)
template <bool kW>
struct SrcF : SrcP<kW> {
  using Item = typename SrcP<kW>::Item;
  const uint32_t *slots;
  const int32_t *slot_of;
  uint32_t *visits;
  unsigned long long *miss;  // records of fragments with a slot that were read from the host copy
  uint32_t fs;
  // Cursors are absolute bit addresses (byte address x 8 + bit), so a
  // vertex's cursor points into its fragment's slot or into the host copy
  // and a record read needs no table lookup.  Device and host-mapped
  // addresses stay below 2^61, and a slot starts 16-byte aligned, so a
  // record's bit within its word is the same in both.
  __device__ __forceinline__ uint64_t cur(uint64_t e) const {
    return ((uint64_t)reinterpret_cast<uintptr_t>(this->words) << 3) + e * this->bpe;
  }
  // The cursor of edge index e for a vertex whose records in this tile are
  // [first, last]: into the slot when they all start in one fragment that
  // has one, else into the host copy.
  __device__ __forceinline__ uint64_t cur_range(uint64_t e, uint64_t first, uint64_t last) const {
    const uint64_t f = (first * this->bpe) >> (5 + fs);
    if (((last * this->bpe) >> (5 + fs)) == f) {
      const int32_t s = __ldg(slot_of + f);
      if (s >= 0) {
        const uint32_t *base = slots + (uint64_t)s * ((1ull << fs) + kFragPad);
        return ((uint64_t)reinterpret_cast<uintptr_t>(base) << 3) - (f << (5 + fs)) + e * this->bpe;
      }
    }
    return cur(e);
  }
  __device__ __forceinline__ Item at(uint64_t c, uint32_t x) const {
    const uint64_t b = c + x * this->bpe;
    return this->decode(reinterpret_cast<const uint32_t *>((uintptr_t)((b >> 5) << 2)), (uint32_t)b & 31u);
  }
  // cnt records from edge index e on: one visit count per fragment they start
  // in; a range over two fragments was read from the host copy, and its
  // records in fragments that have a slot are counted in *miss as well.
  __device__ __forceinline__ void note(uint64_t e, uint32_t cnt) const {
    uint64_t b = e * this->bpe;
    const bool split = (b >> (5 + fs)) != (((e + cnt - 1) * this->bpe) >> (5 + fs));
    while (cnt) {
      const uint64_t f = b >> (5 + fs);
      const uint32_t left = (uint32_t)(((f + 1) << (5 + fs)) - b);  // bits to the next fragment, < 2^26
      const uint32_t n = min(cnt, (left + this->bpe - 1) / this->bpe);
      atomicAdd(visits + f, n);
      if (split && __ldg(slot_of + f) >= 0) atomicAdd(miss, (unsigned long long)n);
      cnt -= n;
      b += (uint64_t)n * this->bpe;
    }
  }
};

// Copies fragment pairs[i].x of the record stream `words` (nwords words,
// padding included) into slot pairs[i].y: one CTA per pair.
__global__ void __launch_bounds__(kThreads) k_frag_fill(const uint32_t *words, uint64_t nwords, uint32_t *slots,
                                                        const uint2 *pairs, uint32_t n, uint32_t fs) {
  if (blockIdx.x >= n) return;
  const uint2 p = pairs[blockIdx.x];
  const uint64_t q0 = (uint64_t)p.x << fs;
  const uint64_t len = min((uint64_t)(1ull << fs) + kFragPad, nwords - min(nwords, q0));
  uint32_t *dst = slots + (uint64_t)p.y * ((1ull << fs) + kFragPad);
  // fragment starts are multiples of 2^fs >= 256 words and slots are
  // 16-byte aligned: whole uint4s first, then the tail
  const uint64_t n4 = len / 4;
  const uint4 *s4 = reinterpret_cast<const uint4 *>(words + q0);
  uint4 *d4 = reinterpret_cast<uint4 *>(dst);
  for (uint64_t i = threadIdx.x; i < n4; i += kThreads) d4[i] = s4[i];
  for (uint64_t i = n4 * 4 + threadIdx.x; i < len; i += kThreads) dst[i] = words[q0 + i];
}

// Slot table update after k_frag_fill: pairs[i] = (fragment, slot), and
// evict[i] the fragment that slot held before (UINT32_MAX: none).
__global__ void k_frag_table(int32_t *slot_of, const uint2 *pairs, const uint32_t *evict, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // a fragment is never both evicted and filled in one update
  if (evict[i] != 0xffffffffu) slot_of[evict[i]] = -1;
  slot_of[pairs[i].x] = (int32_t)pairs[i].y;
}

struct DstU {
  uint32_t *col;
  __device__ __forceinline__ void store(uint64_t i, uint32_t x) const { col[i] = x; }
};
template <class W>
struct DstW {
  uint32_t *col;
  W *w;
  __device__ __forceinline__ void store(uint64_t i, uint2 x) const {
    col[i] = x.x;
    w[i] = (W)x.y;
  }
};

// Per-tile tables.  kVal = false (BFS reads no source value) drops the value
// table, 8 KB of shared memory per CTA that L1 gets instead.
template <class Val, bool kVal = true>
struct LbsShared {
  uint32_t rs[kTile + 2];      // tile-relative start of each local vertex
  unsigned long long cb[kTile + 1];  // source cursor of tile position 0 for the vertex
  Val val[kVal ? kTile + 1 : 1];     // source value of each local vertex
  alignas(16) unsigned short map[kTile];  // tile position -> local vertex
};

// Shared tables of a PageRank pull tile, aliased by phase to fit 6 CTAs per
// SM: the tile-relative starts (rs) are dead once the position map is built
// and then hold the per-position contributions; the edge bases (cb) are dead
// once every record load is issued and then hold the per-vertex sums.
struct PrShared {
  union {
    uint32_t rs[kTile + 2];
    float c[kTile + 2];
  };
  union {
    unsigned long long cb[kTile + 1];
    float tot[kTile + 1];
  };
  uint32_t val[1];  // no source value in PageRank (lbs_setup<false> never writes it)
  alignas(16) unsigned short map[kTile];
};

// Optional op hooks, detected at compile time:
//  list_val(v, e)   the source value belongs to the list entry at address e
//                   (an array parallel to the compacted list) instead of
//                   src_val(v);
//  probe_v(e, val)  the probe also sees the source value;
// and source hooks (SrcF):
//  cur_range(e, first, last)  the cursor of a vertex whose records in the
//                             tile are [first, last];
//  note(e, n)                 the tile lists n records from edge index e on.
template <class T, class = void>
struct HasListVal : std::false_type {};
template <class T>
struct HasListVal<T, std::void_t<decltype(&T::list_val)>> : std::true_type {};
template <class T, class = void>
struct HasNote : std::false_type {};
template <class T>
struct HasNote<T, std::void_t<decltype(&T::note)>> : std::true_type {};
template <class T, class = void>
struct HasCurRange : std::false_type {};
template <class T>
struct HasCurRange<T, std::void_t<decltype(&T::cur_range)>> : std::true_type {};
template <class T, class = void>
struct HasProbeVal : std::false_type {};
template <class T>
struct HasProbeVal<T, std::void_t<decltype(T::kProbeVal)>> : std::true_type {};

// Block-wide exclusive scan of u32 counts; returns the block total.
__device__ __forceinline__ uint32_t block_scan_u32(uint32_t cnt, uint32_t &ex) {
  __shared__ uint32_t s_w[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t ic = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t c = __shfl_up_sync(0xffffffffu, ic, d);
    if (lane >= d) ic += c;
  }
  if (lane == 31) s_w[warp] = ic;
  __syncthreads();
  uint32_t wp = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < kThreads / 32; w++) {
    const uint32_t x = s_w[w];
    wp += w < warp ? x : 0u;
    tot += x;
  }
  ex = wp + ic - cnt;
  return tot;
}

// Builds the local-vertex tables of tile k; returns the local count (0 on
// error).  Sh is LbsShared<Val, *> or PrShared.  cb[j] is the source cursor
// (Src::cur) of tile position 0 for local vertex j, so position x of the tile
// reads src.at(cb[map[x]], x).  Every local vertex's edge indices in the tile
// are checked against edge_bound here, once per vertex; a tile with one out
// of bounds sets kErrEdgeIndex and relaxes nothing.
template <bool kNeedVal, class Src, class Op, class Sh>
__device__ __forceinline__ uint32_t lbs_setup(const LbsArgs &a, const Src &src, const Op &op, Sh &sh,
                                              uint64_t k, uint64_t pos0, uint32_t &i0_out) {
  __shared__ uint32_t s_bad;
  const uint64_t ntiles_total = (a.total + kTile - 1) / kTile;
  const uint32_t i0 = a.tile_first[k];
  const uint32_t i1 = (k + 1 < ntiles_total) ? a.tile_first[k + 1] : a.n - 1;
  i0_out = i0;
  if (i1 < i0 || i1 - i0 > kTile || i1 >= a.n) {
    if (threadIdx.x == 0) atomicOr(a.err, kErrTileMap);
    return 0;
  }
  const uint64_t pend = min(pos0 + kTile, a.pos_end);
  const uint32_t nl = i1 - i0 + 1;
  if (threadIdx.x == 0) s_bad = 0;
  // zero the position map: 2048 u16 = one 16-byte store per thread
  static_assert(kTile * sizeof(unsigned short) == kThreads * sizeof(uint4), "map zeroing");
  reinterpret_cast<uint4 *>(sh.map)[threadIdx.x] = make_uint4(0u, 0u, 0u, 0u);
  __syncthreads();
  bool bad = false;
#pragma unroll 1
  for (uint32_t j = threadIdx.x; j < nl; j += kThreads) {
    const uint32_t i = i0 + j;
    const uint32_t v = a.list[i];
    const uint64_t p = a.pref[i], pn = a.pref[i + 1];
    const uint32_t r = p > pos0 ? (uint32_t)min(p - pos0, (uint64_t)kTile) : 0u;
    sh.rs[j] = r;
    const uint64_t e0 = (a.off ? a.off[v] - p : (0ull - a.stage_base)) + pos0;  // edge index of position 0
    if constexpr (HasCurRange<Src>::value) {
      uint64_t cb = src.cur(e0);
      const uint64_t q1 = min(pn, pend);  // end of the vertex's positions in this tile
      if (q1 > pos0 + r) {
        const uint64_t first = e0 + r, last = e0 + (q1 - pos0) - 1;
        if (pn < p || last < first || last >= a.edge_bound) {
          bad = true;
        } else {
          cb = src.cur_range(e0, first, last);
          if constexpr (HasNote<Src>::value) src.note(first, (uint32_t)(last - first + 1));
        }
      }
      sh.cb[j] = cb;
    } else {
      sh.cb[j] = src.cur(e0);
      const uint64_t q1 = min(pn, pend);  // end of the vertex's positions in this tile
      if (q1 > pos0 + r) {
        const uint64_t first = e0 + r, last = e0 + (q1 - pos0) - 1;
        if (pn < p || last < first || last >= a.edge_bound) bad = true;
      }
    }
    if constexpr (HasListVal<Op>::value) sh.val[j] = op.list_val(v, a.list + i);
    else if constexpr (kNeedVal) sh.val[j] = op.src_val(v);
    // head flag.  Compacted lists hold no zero-degree vertex, so for j >= 1
    // the starts are distinct and strictly increasing (rs[0] = 0).
    if (j >= 1 && r < kTile) sh.map[r] = (unsigned short)1;
  }
  if (bad) {
    s_bad = 1;
    atomicOr(a.err, kErrEdgeIndex);
  }
  __syncthreads();
  // inclusive scan of the head flags (blocked: thread t owns positions 8t..8t+7)
  {
    uint4 m = reinterpret_cast<const uint4 *>(sh.map)[threadIdx.x];
    uint32_t f[kItems] = {m.x & 0xffffu, m.x >> 16, m.y & 0xffffu, m.y >> 16,
                          m.z & 0xffffu, m.z >> 16, m.w & 0xffffu, m.w >> 16};
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < (int)kItems; i++) s += f[i];
    uint32_t run;
    block_scan_u32(s, run);
#pragma unroll
    for (int i = 0; i < (int)kItems; i++) {
      run += f[i];
      f[i] = run;
    }
    m = make_uint4(f[0] | (f[1] << 16), f[2] | (f[3] << 16), f[4] | (f[5] << 16), f[6] | (f[7] << 16));
    reinterpret_cast<uint4 *>(sh.map)[threadIdx.x] = m;
  }
  __syncthreads();
  return s_bad ? 0u : nl;
}

// Shared tables of an LBS relax tile for Op.
template <class Op>
using LbsSh = LbsShared<typename Op::Val, Op::kNeedVal || HasListVal<Op>::value>;

// One LBS tile (kTile positions starting at tile k of the list) of a CTA.
template <class Src, class Op>
__device__ __forceinline__ void lbs_tile(const LbsArgs &a, const Src &src, const Op &op, LbsSh<Op> &sh,
                                         uint64_t k) {
  const uint64_t pos0 = k * kTile;
  if (pos0 >= a.pos_end) return;
  const uint32_t tlen = (uint32_t)(min(pos0 + kTile, a.pos_end) - pos0);
  uint32_t i0;
  const uint32_t nl = lbs_setup<Op::kNeedVal>(a, src, op, sh, k, pos0, i0);
  if (nl == 0) return;
  // All eight loads are issued before the first relax, so each thread keeps
  // eight edge reads in flight (the host-link gather is latency bound).
  typename Src::Item ev[kItems];
  uint32_t lv[kItems];
#pragma unroll
  for (int it = 0; it < (int)kItems; it++) {
    const uint32_t x = it * kThreads + threadIdx.x;
    lv[it] = 0;
    if (x < tlen) {
      const uint32_t l = sh.map[x];
      lv[it] = l;
      ev[it] = src.at(sh.cb[l], x);
    }
  }
  // Probe phase: every target's current state is read before the first
  // atomic, so the eight random reads of a thread overlap (in program order
  // the compiler may not lift a load above an earlier atomic).  A probe is
  // only a filter: relax() acts through atomics, so a stale probe costs an
  // extra atomic, never a wrong result.
  typename Op::Probe pr[kItems];
#pragma unroll
  for (int it = 0; it < (int)kItems; it++)
    if (it * kThreads + threadIdx.x < tlen) {
      if constexpr (HasProbeVal<Op>::value) pr[it] = op.probe_v(ev[it], sh.val[lv[it]]);
      else pr[it] = op.probe(ev[it]);
    }
#pragma unroll
  for (int it = 0; it < (int)kItems; it++) {
    if (it * kThreads + threadIdx.x < tlen)
      op.relax(ev[it], Op::kNeedVal ? sh.val[lv[it]] : typename Op::Val{},
               pos0 + it * kThreads + threadIdx.x, pr[it]);
  }
}

template <class Src, class Op>
__global__ void __launch_bounds__(kThreads) k_lbs(LbsArgs a, Src src, Op op) {
  __shared__ LbsSh<Op> sh;
  lbs_tile(a, src, op, sh, a.pos_begin / kTile + blockIdx.x);
}

// Both regions of a round in one launch: n0 tiles of list 0 (static region,
// read from HBM) and n1 tiles of list 1 (dynamic region, read over the host
// link), interleaved in CTA order in proportion to their counts, so that at
// any time about n0 / (n0 + n1) of the resident CTAs work from HBM while the
// rest keep the link busy.  CTA b is a static tile iff
// floor((b + 1) n0 / n) > floor(b n0 / n); its tile index is floor(b n0 / n),
// else b - floor((b + 1) n0 / n) among the dynamic tiles.
struct PairTile {
  unsigned long long t;  // tile index within its region
  uint32_t r;            // 0: static region, 1: dynamic region
};
__device__ __forceinline__ PairTile pair_split(uint64_t b, uint64_t n0, uint64_t n) {
  if (n0 == n) return PairTile{b, 0u};
  if (n0 == 0) return PairTile{b, 1u};
  const uint64_t lo = b * n0 / n, hi = (b + 1) * n0 / n;
  return hi > lo ? PairTile{lo, 0u} : PairTile{b - hi, 1u};
}
// The split of this CTA, computed once: a 64-bit division is a long
// instruction sequence, so thread 0 runs it and the CTA reads the result.
__device__ __forceinline__ PairTile pair_split_cta(uint64_t n0, uint64_t n) {
  __shared__ PairTile s_pt;
  if (threadIdx.x == 0) s_pt = pair_split(blockIdx.x, n0, n);
  __syncthreads();
  return s_pt;
}

template <class Src0, class Src1, class Op>
__global__ void __launch_bounds__(kThreads) k_lbs_pair(LbsArgs a0, Src0 s0, LbsArgs a1, Src1 s1, Op op,
                                                       uint64_t n0, uint64_t n) {
  __shared__ LbsSh<Op> sh;
  const PairTile pt = pair_split_cta(n0, n);
  if (pt.r == 0) lbs_tile(a0, s0, op, sh, a0.pos_begin / kTile + pt.t);
  else lbs_tile(a1, s1, op, sh, a1.pos_begin / kTile + pt.t);
}

template <int MULT>
constexpr size_t gather_smem_bytes() {
  return 8 * (MULT * kTile + 1) + 4 * (MULT * kTile + 2) + 2 * (MULT * kTile);
}

// Dynamic-region gather, specialised: MULT x 2048 positions per CTA (the
// per-tile setup is amortised over more edges) and no per-vertex value table.
// Positions of a vertex are contiguous both in the host CSR and in the staging
// buffer, so this is a segmented copy; reads are coalesced 8-byte (or 4-byte)
// loads over NVLink-C2C, all ITEMS of a thread issued before the first store.
template <class Src, class Dst, int MULT>
__global__ void __launch_bounds__(kThreads) k_gather(LbsArgs a, Src src, Dst stage) {
  constexpr uint32_t TILE = MULT * kTile;
  constexpr int ITEMS = TILE / kThreads;
  // dynamic shared memory (gather_smem_bytes<MULT>() bytes, above the static 48 KB)
  extern __shared__ __align__(16) unsigned char g_smem[];
  unsigned long long *cb = (unsigned long long *)g_smem;          // TILE + 1
  uint32_t *rs = (uint32_t *)(cb + TILE + 1);                      // TILE + 2
  unsigned short *map = (unsigned short *)(rs + TILE + 2);         // TILE
  const uint64_t pos0 = a.pos_begin + (uint64_t)blockIdx.x * TILE;
  if (pos0 >= a.pos_end) return;
  const uint64_t pend = min(pos0 + TILE, a.pos_end);
  const uint32_t i0 = a.tile_first[pos0 / kTile];
  const uint32_t i1 = pend < a.total ? a.tile_first[pend / kTile] : a.n - 1;
  if (i1 < i0 || i1 - i0 > TILE || i1 >= a.n) {
    if (threadIdx.x == 0) atomicOr(a.err, kErrTileMap);
    return;
  }
  const uint32_t nl = i1 - i0 + 1;
  for (uint32_t j = threadIdx.x; j < nl; j += kThreads) {
    const uint32_t v = a.list[i0 + j];
    const uint64_t p = a.pref[i0 + j];
    rs[j] = p > pos0 ? (uint32_t)min(p - pos0, (uint64_t)TILE) : 0u;
    cb[j] = a.off[v] - p + pos0;
  }
  for (uint32_t x = threadIdx.x; x < TILE; x += kThreads) map[x] = 0;
  __syncthreads();
  for (uint32_t j = 1 + threadIdx.x; j < nl; j += kThreads)
    if (rs[j] < TILE) map[rs[j]] = 1;
  __syncthreads();
  {
    uint32_t f[ITEMS], sacc = 0;
#pragma unroll
    for (int i = 0; i < ITEMS; i++) {
      f[i] = map[threadIdx.x * ITEMS + i];
      sacc += f[i];
    }
    uint32_t ex, tot;
    uint64_t ex64, tot64;
    block_scan_pair(sacc, 0, ex, ex64, tot, tot64);
#pragma unroll
    for (int i = 0; i < ITEMS; i++) {
      ex += f[i];
      map[threadIdx.x * ITEMS + i] = (unsigned short)ex;
    }
  }
  __syncthreads();
  const uint32_t tlen = (uint32_t)(pend - pos0);
  typename Src::Item ev[ITEMS];
  uint32_t okm = 0;
#pragma unroll
  for (int it = 0; it < ITEMS; it++) {
    const uint32_t x = it * kThreads + threadIdx.x;
    if (x < tlen) {
      const uint64_t idx = cb[map[x]] + x;
      if (idx < a.edge_bound) {
        ev[it] = src.load(idx);
        okm |= 1u << it;
      } else {
        atomicOr(a.err, kErrEdgeIndex);
      }
    }
  }
  const uint64_t base = pos0 - a.stage_base;
#pragma unroll
  for (int it = 0; it < ITEMS; it++)
    if (okm & (1u << it)) stage.store(base + it * kThreads + threadIdx.x, ev[it]);
}

// ------------------------------------------------------------------ ops

__device__ __forceinline__ uint32_t edge_dst(uint32_t e) { return e; }
__device__ __forceinline__ uint32_t edge_dst(uint2 e) { return e.x; }
__device__ __forceinline__ uint32_t edge_w(uint32_t) { return 1u; }
__device__ __forceinline__ uint32_t edge_w(uint2 e) { return e.y; }

// Level-synchronous BFS with a visited bitmap: every vertex is claimed once.
struct BfsOp {
  using Val = uint32_t;
  static constexpr bool kNeedVal = false;
  uint32_t *visited, *next, *depth, *err;
  uint32_t V, newdepth;
  __device__ uint32_t src_val(uint32_t) const { return 0; }
  // The target's visited word, read through L1: bits are only ever set
  // during a launch (and global data cached in L1 does not outlive the
  // launch), so a stale word lacks bits at most and costs an extra atomic,
  // never a wrong result.  Hub vertices' words are read over and over.
  using Probe = uint32_t;
  template <class Edge>
  __device__ __forceinline__ Probe probe(Edge e) const {
    const uint32_t v = edge_dst(e);
    return v < V ? visited[v >> 5] : 0u;
  }
  template <class Edge>
  __device__ __forceinline__ void relax(Edge e, uint32_t, uint64_t, Probe p) const {
    const uint32_t v = edge_dst(e);
    if (v >= V) {
      atomicOr(err, kErrVertex);
      return;
    }
    const uint32_t w = v >> 5, bit = 1u << (v & 31);
    if (p & bit) return;
    // The probe holds every bit set before this launch, so v is reached at
    // this level, by this thread or another one of the launch: every writer
    // stores the same depth and sets the same bits.  No atomic's old value
    // is needed, so none is waited for (the atomics compile to reductions).
    atomicOr(visited + w, bit);
    depth[v] = newdepth;
    atomicOr(next + w, bit);
  }
};

// atomicMin relax shared by SSSP (weighted) and CC (label push).
template <bool kWeighted>
struct MinOp {
  using Val = uint32_t;
  static constexpr bool kNeedVal = true;
  uint32_t *value, *next, *err;
  uint32_t V;
  __device__ uint32_t src_val(uint32_t v) const { return __ldcg(value + v); }
  // The target's current value, read through L1: values only decrease during
  // a launch, so a stale value is too large at most and costs an extra
  // atomicMin, never a wrong result.
  using Probe = uint32_t;
  template <class Edge>
  __device__ __forceinline__ Probe probe(Edge e) const {
    const uint32_t v = edge_dst(e);
    return v < V ? value[v] : 0u;
  }
  template <class Edge>
  __device__ __forceinline__ void relax(Edge e, uint32_t sv, uint64_t, Probe p) const {
    const uint32_t v = edge_dst(e);
    if (v >= V) {
      atomicOr(err, kErrVertex);
      return;
    }
    const uint32_t cand = kWeighted ? sv + edge_w(e) : sv;
    if (cand >= p) return;
    // cand < p: v's value drops in this launch, to cand here or lower by
    // another thread that marks v as well, so v is in the next frontier
    // either way.  The atomics' old values are not needed (reductions).
    atomicMin(value + v, cand);
    atomicOr(next + (v >> 5), 1u << (v & 31));
  }
};

// ------------------------------------------------------------------ batched BFS

// Up to 64 BFS sources share one pass: bit s of a vertex's masks belongs to
// source s.  visited = bits already reached, cur = bits first reached at the
// current level (frontier), next = bits first reached at the next level.
// Level-synchronous, so a bit's level is its BFS depth, exactly as a
// single-source run computes it.
struct BatchOp {
  using Val = unsigned long long;
  static constexpr bool kNeedVal = true;
  unsigned long long *visited, *cur, *next;
  uint32_t *next_any;  // bitmap of vertices with next != 0
  uint32_t *err;
  uint32_t V;
  __device__ Val src_val(uint32_t v) const { return __ldcg(cur + v); }
  using Probe = unsigned long long;  // the target's visited mask (through L1, as BfsOp)
  template <class Edge>
  __device__ __forceinline__ Probe probe(Edge e) const {
    const uint32_t v = edge_dst(e);
    return v < V ? visited[v] : ~0ull;
  }
  template <class Edge>
  __device__ __forceinline__ void relax(Edge e, Val m, uint64_t, Probe p) const {
    const uint32_t v = edge_dst(e);
    if (v >= V) {
      atomicOr(err, kErrVertex);
      return;
    }
    Val nb = m & ~p;
    if (!nb) return;
    nb &= ~atomicOr(visited + v, nb);
    if (!nb) return;
    if (atomicOr(next + v, nb) == 0ull) atomicOr(next_any + (v >> 5), 1u << (v & 31));
  }
};

// PageRank by push over an out-edge CSR: the listed vertex u adds its
// contribution (rank / out-degree, the LBS source value) to the sum of every
// out-neighbour with an FP32 atomicAdd.  Nothing to probe.
struct PushOp {
  using Val = float;
  static constexpr bool kNeedVal = true;
  const float *contrib;
  float *sum;
  uint32_t *err;
  uint32_t V;
  __device__ Val src_val(uint32_t u) const { return contrib[u]; }
  using Probe = uint32_t;
  template <class Edge>
  __device__ __forceinline__ Probe probe(Edge) const {
    return 0u;
  }
  template <class Edge>
  __device__ __forceinline__ void relax(Edge e, Val c, uint64_t, Probe) const {
    const uint32_t v = edge_dst(e);
    if (v >= V) {
      atomicOr(err, kErrVertex);
      return;
    }
    if (c != 0.f) atomicAdd(sum + v, c);
  }
};

// Seeds source i (bit slots[i], or bit i when slots is null) at depth 1.
__global__ void k_batch_init(const uint32_t *srcs, uint32_t n, unsigned long long *visited,
                             unsigned long long *cur, uint32_t *cur_any, uint32_t *depth,
                             uint64_t V, uint8_t *depth8 = nullptr, const uint32_t *slots = nullptr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t v = srcs[i], b = slots ? slots[i] : i;
  atomicOr(visited + v, 1ull << b);
  atomicOr(cur + v, 1ull << b);
  atomicOr(cur_any + (v >> 5), 1u << (v & 31));
  if (depth) depth[(uint64_t)b * V + v] = 1u;
  if (depth8) depth8[(uint64_t)b * V + v] = 1u;
}

// Clears the bits `mask` of every vertex's mask (slots released for reuse).
__global__ void k_batch_clear_bits(unsigned long long *m, uint64_t n, unsigned long long mask) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
    if (m[v] & mask) m[v] &= ~mask;
}

// Per-source count of the vertices first reached at this level (hist[s]),
// and, when depth != nullptr, their depth for the n x V output: level, less
// doff[s] when doff is not null (a source that joined a pass in flight).
__global__ void __launch_bounds__(kThreads) k_batch_level(const uint32_t *next_any,
                                                          const unsigned long long *next,
                                                          uint64_t nwords, uint32_t n,
                                                          unsigned long long *hist,
                                                          uint32_t *depth, uint64_t V,
                                                          uint32_t level, const uint32_t *doff = nullptr) {
  __shared__ uint32_t s_cnt[64];
  if (threadIdx.x < 64) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords;
       w += (uint64_t)gridDim.x * blockDim.x) {
    for (uint32_t bits = next_any[w]; bits; bits &= bits - 1) {
      const uint64_t v = w * 32 + (__ffs(bits) - 1);
      if (v >= V) break;
      for (unsigned long long m = next[v]; m; m &= m - 1) {
        const uint32_t s = __ffsll((long long)m) - 1;
        if (s < n) {
          atomicAdd(&s_cnt[s], 1u);
          if (depth) depth[(uint64_t)s * V + v] = doff ? level - doff[s] : level;
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < 64 && s_cnt[threadIdx.x]) atomicAdd(hist + threadIdx.x, (unsigned long long)s_cnt[threadIdx.x]);
}

// ------------------------------------------------------------------ PageRank

constexpr uint32_t kNoCarry = 0xffffffffu;

struct PrArgs {
  const float *contrib;   // rank[u] / outdeg[u] (0 for dangling u)
  float *sum;             // pull sums, written for every listed vertex
  float *cont;            // per LBS tile: partial of a vertex that began in an earlier tile
  float *carry;           // per LBS tile: partial of a vertex that began here and continues
  uint32_t *carry_idx;    // per LBS tile: list index of that vertex, kNoCarry if none
  uint32_t V;
};

// Pull sum sum[v] = sum over in-edges (u -> v) of contrib[u]
// (PR/OneGraph/gpu_kernels.h:107-158).  Contributions are staged in shared
// memory in edge order and each vertex's segment is added sequentially, so the
// result depends only on the tiling of the compacted list (deterministic).
template <class Src>
__device__ __forceinline__ void pr_tile(const LbsArgs &a, const Src &src, const PrArgs &p, PrShared &sh,
                                        uint64_t k) {
  float *s_c = sh.c;
  const uint64_t pos0 = k * kTile;
  if (pos0 >= a.pos_end) return;
  const uint64_t pend = min(pos0 + kTile, a.pos_end);
  const uint32_t tlen = (uint32_t)(pend - pos0);
  struct NoVal {
    __device__ uint32_t src_val(uint32_t) const { return 0; }
  } nv;
  uint32_t i0;
  const uint32_t nl = lbs_setup<false>(a, src, nv, sh, k, pos0, i0);
  if (nl == 0) return;
  // three phases, so that a thread keeps all eight record loads and then all
  // eight contribution gathers in flight
  uint32_t u[kItems];
#pragma unroll
  for (int it = 0; it < (int)kItems; it++) {
    const uint32_t x = it * kThreads + threadIdx.x;
    u[it] = 0xffffffffu;  // no edge at this position
    if (x < tlen) u[it] = edge_dst(src.at(sh.cb[sh.map[x]], x));
  }
  float c[kItems];
#pragma unroll
  for (int it = 0; it < (int)kItems; it++) {
    c[it] = 0.f;
    if (u[it] < p.V) c[it] = __ldg(p.contrib + u[it]);
    else if (u[it] != 0xffffffffu) atomicOr(a.err, kErrVertex);
  }
#pragma unroll
  for (int it = 0; it < (int)kItems; it++) s_c[it * kThreads + threadIdx.x] = c[it];
  __syncthreads();
  // Segmented reduction over the tile's positions: thread t sums positions
  // [8t, 8t + 8) (restarting at every segment head), a block-wide segmented
  // scan carries each thread's open segment into the next thread, and every
  // segment's total is stored at its last position into s_tot[local vertex]
  // (the per-vertex value table, unused by PageRank).  A high-degree vertex
  // filling the tile is summed by all 256 threads instead of one.  The order
  // of additions is fixed by the tiling, so sums are deterministic.
  float *s_tot = sh.tot;
  const uint32_t base = threadIdx.x * kItems;
  float run = 0.f;
  uint32_t head = 0;
#pragma unroll
  for (int it = 0; it < (int)kItems; it++) {
    const uint32_t x = base + it;
    if (x < tlen) {
      if (x == 0 || sh.map[x] != sh.map[x - 1]) {
        run = 0.f;
        head = 1;
      }
      run += s_c[x];
    }
  }
  // inclusive segmented scan of (head, run): (f1, v1) + (f2, v2) = (f1 | f2, f2 ? v2 : v1 + v2)
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float iv = run;
  uint32_t ifl = head;
#pragma unroll
  for (uint32_t d = 1; d < 32; d <<= 1) {
    const float v2 = __shfl_up_sync(0xffffffffu, iv, d);
    const uint32_t f2 = __shfl_up_sync(0xffffffffu, ifl, d);
    if (lane >= d) {
      if (!ifl) iv += v2;
      ifl |= f2;
    }
  }
  __shared__ float s_wv[kThreads / 32];
  __shared__ uint32_t s_wf[kThreads / 32];
  if (lane == 31) {
    s_wv[warp] = iv;
    s_wf[warp] = ifl;
  }
  __syncthreads();
  // exclusive prefix of this thread: warps before it, then lanes before it
  float cv = 0.f;
  for (uint32_t w = 0; w < warp; w++) {
    if (s_wf[w]) cv = s_wv[w];
    else cv += s_wv[w];
  }
  const float lv = __shfl_up_sync(0xffffffffu, iv, 1);
  const uint32_t lf = __shfl_up_sync(0xffffffffu, ifl, 1);
  if (lane > 0) cv = lf ? lv : cv + lv;
  run = cv;  // the open segment's sum before this thread's first position
#pragma unroll
  for (int it = 0; it < (int)kItems; it++) {
    const uint32_t x = base + it;
    if (x < tlen) {
      const uint32_t l = sh.map[x];
      if (x == 0 || l != sh.map[x - 1]) run = 0.f;
      run += s_c[x];
      if (x + 1 == tlen || sh.map[x + 1] != l) s_tot[l] = run;
    }
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < nl; j += kThreads) {
    const uint32_t i = i0 + j;
    if (j > 0 && a.pref[i] >= pend) continue;  // starts in the next tile: no position here
    const float s = s_tot[j];
    const bool before = (j == 0) && (a.pref[i] < pos0);
    const bool after = a.pref[i + 1] > pos0 + kTile;
    if (before) {
      p.cont[k] = s;
    } else if (after) {
      p.carry[k] = s;
      p.carry_idx[k] = i;
    } else {
      p.sum[a.list[i]] = s;
    }
  }
}

template <class Src>
__global__ void __launch_bounds__(kThreads, 6) k_pr_pull(LbsArgs a, Src src, PrArgs p) {
  __shared__ PrShared sh;
  pr_tile(a, src, p, sh, a.pos_begin / kTile + blockIdx.x);
}

// Both regions' pull sums in one launch, static and dynamic tiles interleaved
// in CTA order as in k_lbs_pair (each region keeps its own carry arrays, so
// the sums are the same as with two launches).
template <class Src0, class Src1>
__global__ void __launch_bounds__(kThreads, 6) k_pr_pull_pair(LbsArgs a0, Src0 s0, PrArgs p0, LbsArgs a1,
                                                              Src1 s1, PrArgs p1, uint64_t n0, uint64_t n) {
  __shared__ PrShared sh;
  const PairTile pt = pair_split_cta(n0, n);
  if (pt.r == 0) pr_tile(a0, s0, p0, sh, a0.pos_begin / kTile + pt.t);
  else pr_tile(a1, s1, p1, sh, a1.pos_begin / kTile + pt.t);
}

// Completes the sums of vertices split over several tiles, in tile order.
__global__ void k_pr_fixup(const uint32_t *list, const uint64_t *pref, uint64_t tile_begin,
                           uint64_t tile_end, PrArgs p) {
  const uint64_t k = tile_begin + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= tile_end) return;
  const uint32_t i = p.carry_idx[k];
  if (i == kNoCarry) return;
  float s = p.carry[k];
  const uint64_t end = pref[i + 1];
  for (uint64_t t = k + 1; t * kTile < end; t++) s += p.cont[t];
  p.sum[list[i]] = s;
}

// prKernel_Opt (PR/OneGraph/gpu_kernels.h:295-319): for every active vertex
// new = 0.15 + 0.85*sum; it stays active with the new rank iff |new-old| >
// thresh, otherwise it goes inactive keeping its rank.  One thread per bitmap
// word; writes the next active bitmap and counts the survivors.
__global__ void __launch_bounds__(kThreads) k_pr_update_delta(
    const uint32_t *cur, uint32_t *next, uint64_t nwords, float *rank, float *contrib,
    const float *sum, const uint32_t *outdeg, float thresh, uint32_t *active) {
  __shared__ uint32_t s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  uint32_t mine = 0;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords;
       w += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t word = cur[w];
    uint32_t keep = 0;
    for (uint32_t m = word; m; m &= m - 1) {
      const uint32_t b = __ffs(m) - 1;
      const uint64_t v = w * 32 + b;
      const float nvv = 0.15f + 0.85f * sum[v];
      const float old = rank[v];
      const float diff = nvv > old ? nvv - old : old - nvv;
      if (diff > thresh) {
        rank[v] = nvv;
        const uint32_t od = outdeg[v];
        contrib[v] = od ? nvv / (float)od : 0.f;
        keep |= 1u << b;
      }
    }
    next[w] = keep;
    mine += __popc(keep);
  }
  atomicAdd(&s_cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0 && s_cnt) atomicAdd(active, s_cnt);
}

// Normalised update p' = teleport + damping*sum for every vertex, with the L1
// delta accumulated in FP64: per-thread, then a fixed-shape block tree, one
// partial per block (the grid size is fixed, so the order never changes).
__global__ void __launch_bounds__(kThreads) k_pr_update_l1(uint64_t V, float *rank, float *contrib,
                                                           const float *sum, const uint32_t *outdeg,
                                                           float teleport, float damping,
                                                           double *part) {
  __shared__ double s_d[kThreads];
  double acc = 0.0;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const float nvv = teleport + damping * sum[v];
    acc += fabs((double)nvv - (double)rank[v]);
    rank[v] = nvv;
    const uint32_t od = outdeg[v];
    contrib[v] = od ? nvv / (float)od : 0.f;
  }
  s_d[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) s_d[threadIdx.x] += s_d[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s_d[0];
}

__global__ void k_reduce_f64(const double *part, uint32_t n, double *out) {
  __shared__ double s_d[kThreads];
  double acc = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += kThreads) acc += part[i];
  s_d[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) s_d[threadIdx.x] += s_d[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s_d[0];
}

__global__ void k_pr_init(uint64_t V, float *rank, float *contrib, float *sum, const uint32_t *outdeg,
                          float r0) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V;
       v += (uint64_t)gridDim.x * blockDim.x) {
    rank[v] = r0;
    const uint32_t od = outdeg[v];
    contrib[v] = od ? r0 / (float)od : 0.f;
    sum[v] = 0.f;
  }
}

__global__ void k_degree_from_offsets(uint64_t V, const uint64_t *off, uint32_t *deg) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V;
       v += (uint64_t)gridDim.x * blockDim.x)
    deg[v] = (uint32_t)(off[v + 1] - off[v]);
}

// ------------------------------------------------------------------ checksums

// Result checksum in a fixed reduction order (fixed grid, fixed trees):
// mode 0: {#v with value != unreached, sum of those values} (BFS, SSSP)
// mode 1: {#v with label == v (components), sum of labels}     (CC)
// mode 2: {#v, bits of the FP64 sum of the FP32 ranks}          (PR)
__global__ void __launch_bounds__(kThreads) k_checksum(const uint32_t *val, uint64_t V, int mode,
                                                       uint32_t unreached,
                                                       unsigned long long *part) {
  __shared__ unsigned long long s_c[kThreads], s_s[kThreads];
  __shared__ double s_d[kThreads];
  unsigned long long c = 0, sum = 0;
  double d = 0.0;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t x = val[v];
    if (mode == 0) {
      if (x != unreached) {
        c++;
        sum += x;
      }
    } else if (mode == 1) {
      c += (x == v) ? 1 : 0;
      sum += x;
    } else {
      c++;
      d += (double)__uint_as_float(x);
    }
  }
  s_c[threadIdx.x] = c;
  s_s[threadIdx.x] = sum;
  s_d[threadIdx.x] = d;
  __syncthreads();
  for (int k = kThreads / 2; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) {
      s_c[threadIdx.x] += s_c[threadIdx.x + k];
      s_s[threadIdx.x] += s_s[threadIdx.x + k];
      s_d[threadIdx.x] += s_d[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = s_c[0];
    part[3 * blockIdx.x + 1] = s_s[0];
    part[3 * blockIdx.x + 2] = __double_as_longlong(s_d[0]);
  }
}

__global__ void k_checksum_final(const unsigned long long *part, uint32_t n, int mode,
                                 unsigned long long *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long c = 0, sum = 0;
  double d = 0.0;
  for (uint32_t i = 0; i < n; i++) {
    c += part[3 * i];
    sum += part[3 * i + 1];
    d += __longlong_as_double(part[3 * i + 2]);
  }
  out[0] = c;
  out[1] = mode == 2 ? (unsigned long long)__double_as_longlong(d) : sum;
}

// ------------------------------------------------------------------ fills

__global__ void k_fill_u32(uint32_t *p, uint64_t n, uint32_t v) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// Byte depths of one source (0 unreached, 1 the source, at most 254 here)
// as u32 depths with `unreached` for 0, written to dst (device memory, or
// page-locked host memory through its device pointer).  Four vertices per
// thread, one 4-byte load each, when b is 4-byte aligned (rows of a matrix
// with V not a multiple of 4 are not); else one vertex per thread.
__global__ void k_depth_expand(const uint8_t *b, uint64_t n, uint32_t unreached, uint32_t *dst) {
  if (reinterpret_cast<uintptr_t>(b) & 3u) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x)
      dst[v] = b[v] ? b[v] : unreached;
    return;
  }
  const uint64_t n4 = n / 4;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n4;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uchar4 q = reinterpret_cast<const uchar4 *>(b)[i];
    dst[4 * i] = q.x ? q.x : unreached;
    dst[4 * i + 1] = q.y ? q.y : unreached;
    dst[4 * i + 2] = q.z ? q.z : unreached;
    dst[4 * i + 3] = q.w ? q.w : unreached;
  }
  if (blockIdx.x == 0 && threadIdx.x < n - 4 * n4) {
    const uint64_t v = 4 * n4 + threadIdx.x;
    dst[v] = b[v] ? b[v] : unreached;
  }
}

// ---------------------------------------------------------- bottom-up BFS
//
// One bottom-up level of a direction-optimizing BFS (Beamer et al., 2012)
// on a symmetric graph: every unvisited vertex scans its own neighbours, four
// records at a time, and stops at the first one in the current frontier; it
// then gets depth newdepth and joins the next frontier.  Valid because the
// graph is symmetric (a neighbour u of v has the edge u -> v).  The depths
// equal the top-down ones: a vertex is reached at level L + 1 exactly when
// one of its neighbours has depth L.  Warps cover 32 consecutive vertices
// (one bitmap word), so each word of next / visited has a single writer.
// cnt[0] += vertices reached, cnt[1] += their degrees, cnt[2] += records read
// from the host copy, cnt[3] += records read from the static region.
template <class PS>
__global__ void __launch_bounds__(kThreads) k_bfs_bottom_up(const uint64_t *off, uint32_t V, uint32_t Vs, PS stat,
                                                            PS host, const uint32_t *cur, uint32_t *visited,
                                                            uint32_t *next, uint32_t *depth, uint32_t newdepth,
                                                            unsigned long long *cnt, uint32_t *err,
                                                            const uint32_t *go = nullptr,
                                                            const uint32_t *level = nullptr) {
  // device-driven loops: run only when *go, at depth *level + 1
  if (go && *go == 0u) return;
  if (level) newdepth = *level + 1;
  const uint32_t lane = threadIdx.x & 31;
  unsigned long long nn = 0, nm = 0, nh = 0, ns = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < V; base += stride) {
    const uint64_t v = base + lane;
    const uint32_t w = (uint32_t)(base >> 5);
    const uint32_t vis = __ldcg(visited + w);
    bool found = false;
    uint64_t d = 0;
    if (v < V && !((vis >> lane) & 1u)) {
      const uint64_t o = off[v], e1 = off[v + 1];
      d = e1 - o;
      const bool st = v < Vs;
      const PS &src = st ? stat : host;
      for (uint64_t e = o; e < e1 && !found; e += 4) {
        uint32_t u[4];
#pragma unroll
        for (int j = 0; j < 4; j++) u[j] = e + j < e1 ? src.load(e + j) : 0xffffffffu;
        const uint64_t got = (e1 - e < 4) ? e1 - e : 4;
        if (st) ns += got;
        else nh += got;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (u[j] < V) {
            if ((__ldcg(cur + (u[j] >> 5)) >> (u[j] & 31)) & 1u) found = true;
          } else if (u[j] != 0xffffffffu) {
            atomicOr(err, kErrVertex);
          }
        }
      }
    }
    const uint32_t ball = __ballot_sync(0xffffffffu, found);
    if (lane == 0 && ball) {
      next[w] = ball;
      visited[w] = vis | ball;
    }
    if (found) {
      depth[v] = newdepth;
      nn++;
      nm += d;
    }
  }
  nn = __reduce_add_sync(0xffffffffu, (uint32_t)nn);
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    nm += __shfl_xor_sync(0xffffffffu, nm, o);
    nh += __shfl_xor_sync(0xffffffffu, nh, o);
    ns += __shfl_xor_sync(0xffffffffu, ns, o);
  }
  if (lane == 0) {
    if (nn) atomicAdd(cnt, nn);
    if (nm) atomicAdd(cnt + 1, nm);
    if (nh) atomicAdd(cnt + 2, nh);
    if (ns) atomicAdd(cnt + 3, ns);
  }
}

// ------------------------------------------------------------ union-find CC
//
// Connected components of a symmetric graph by sampling union-find (the
// Afforest scheme): hook every vertex with its first two neighbours, find the
// giant component, then expand only the edges of vertices outside it.  A
// root is hooked only under a smaller root (CAS on parent[hi] == hi), so
// parent[x] <= x holds at all times and the root of every tree is the
// smallest vertex id in it: after compression parent[] is exactly the
// reference's CC label (minimum id of the component) with no relabelling.
// Walks follow strictly decreasing ids, so they end within V steps; a broken
// invariant sets kErrVertex instead of looping.

__device__ __forceinline__ uint32_t uf_find(uint32_t *par, uint32_t x, uint32_t V, uint32_t *err) {
  for (uint32_t steps = 0; steps <= V; steps++) {
    const uint32_t p = __ldcg(par + x);
    if (p == x) return x;
    if (p > x) {
      atomicOr(err, kErrVertex);
      return x;
    }
    const uint32_t gp = __ldcg(par + p);
    if (gp < p) __stcg(par + x, gp);  // path halving: gp is an ancestor of x
    x = gp;
  }
  atomicOr(err, kErrVertex);
  return x;
}

__device__ __forceinline__ void uf_link(uint32_t *par, uint32_t a, uint32_t b, uint32_t V, uint32_t *err) {
  for (uint32_t tries = 0; tries <= V; tries++) {
    const uint32_t ra = uf_find(par, a, V, err), rb = uf_find(par, b, V, err);
    if (ra == rb) return;
    const uint32_t hi = max(ra, rb), lo = min(ra, rb);
    if (atomicCAS(par + hi, hi, lo) == hi) return;
    a = ra;  // hi gained a parent meanwhile: retry from the two roots
    b = rb;
  }
  atomicOr(err, kErrVertex);
}

// Sampling pass r: link every vertex of degree > r with its r-th neighbour
// (edge off[v] + r, from the static region or from the host copy).
template <class PS>
__global__ void __launch_bounds__(kThreads) k_uf_sample(const uint64_t *off, uint32_t V, uint64_t static_edges,
                                                        PS stat, PS host, uint32_t r, uint32_t *par,
                                                        unsigned long long *reads, uint32_t *err) {
  uint32_t nh = 0, ns = 0;  // records read from the host copy / the static region
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t o = off[v];
    if (off[v + 1] - o <= r) continue;
    const uint64_t idx = o + r;
    uint32_t u;
    if (idx < static_edges) {
      u = stat.load(idx);
      ns++;
    } else {
      u = host.load(idx);
      nh++;
    }
    if (u >= V) {
      atomicOr(err, kErrVertex);
      continue;
    }
    uf_link(par, (uint32_t)v, u, V, err);
  }
  nh = __reduce_add_sync(0xffffffffu, nh);
  ns = __reduce_add_sync(0xffffffffu, ns);
  if ((threadIdx.x & 31) == 0) {  // reads[0]: host records, reads[1]: static records
    if (nh) atomicAdd(reads, (unsigned long long)nh);
    if (ns) atomicAdd(reads + 1, (unsigned long long)ns);
  }
}

// parent[v] = root of v for every vertex.
__global__ void __launch_bounds__(kThreads) k_uf_compress(uint32_t *par, uint32_t V, uint32_t *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x)
    __stcg(par + v, uf_find(par, (uint32_t)v, V, err));
}

// Roots of k pseudo-random vertices (after compression), for the host to
// pick the most frequent one as the giant component.
__global__ void k_uf_roots(const uint32_t *par, uint32_t V, uint32_t k, uint32_t *roots) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  uint64_t z = 0x9e3779b97f4a7c15ull * (i + 1);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  roots[i] = __ldcg(par + (uint32_t)(z % V));
}

// Frontier of the final pass: vertices of degree > 2 (their first two edges
// are already linked) outside component c.  One thread per bitmap word.
__global__ void __launch_bounds__(kThreads) k_uf_mark(const uint64_t *off, const uint32_t *par, uint32_t V,
                                                      uint32_t c, uint32_t *bits, uint64_t nwords) {
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t word = 0;
    for (uint32_t b = 0; b < 32; b++) {
      const uint64_t v = w * 32 + b;
      if (v >= V) break;
      if (off[v + 1] - off[v] > 2 && __ldcg(par + v) != c) word |= 1u << b;
    }
    bits[w] = word;
  }
}

// LBS op of the final pass: link the source vertex with every neighbour.
struct UnionOp {
  using Val = uint32_t;
  static constexpr bool kNeedVal = true;
  uint32_t *par, *err;
  uint32_t V;
  __device__ uint32_t src_val(uint32_t v) const { return v; }
  using Probe = uint32_t;  // the neighbour's parent (read early; links re-read it)
  template <class Edge>
  __device__ __forceinline__ Probe probe(Edge e) const {
    const uint32_t v = edge_dst(e);
    return v < V ? __ldcg(par + v) : 0u;
  }
  template <class Edge>
  __device__ __forceinline__ void relax(Edge e, uint32_t sv, uint64_t, Probe) const {
    const uint32_t v = edge_dst(e);
    if (v >= V) {
      atomicOr(err, kErrVertex);
      return;
    }
    uf_link(par, sv, v, V, err);
  }
};

__global__ void k_iota_u32(uint32_t *p, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = (uint32_t)i;
}

// bits [0, V) set, the rest of the words cleared
__global__ void k_fill_bits(uint32_t *bits, uint64_t nwords, uint64_t V) {
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords;
       w += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = w * 32;
    bits[w] = b + 32 <= V ? 0xffffffffu : (b >= V ? 0u : ((1u << (V - b)) - 1u));
  }
}

__global__ void k_set_source(uint32_t *value, uint32_t src, uint32_t val, uint32_t *bits_a,
                             uint32_t *bits_b) {
  value[src] = val;
  bits_a[src >> 5] |= 1u << (src & 31);
  if (bits_b) bits_b[src >> 5] |= 1u << (src & 31);
}

}  // namespace og
