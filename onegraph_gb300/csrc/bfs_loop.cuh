// bfs_loop.cuh — device-driven level loop of single-source BFS.
//
// The host-driven loop (engine.cu run_frontier) waits for every level's
// counts before it launches the next kernels, so a BFS of a few levels on a
// resident graph spends more time in host round trips than in kernels.  Here
// every decision is taken on the GPU: a level is a fixed sequence of launches
// (both regions' compaction, a control kernel, the top-down relax over a
// fixed grid that reads its tile counts from device memory, the bottom-up
// expansion, a second control kernel, the clear of the expanded frontier),
// each gated by flags the control kernels write.  The sequence is captured
// once per frontier parity as a CUDA graph and the two graphs are replayed
// alternately; the host reads the done flag only every few levels.  Levels
// launched after the end do nothing but read their flags.
//
// The control logic is the host loop's, step for step (direction-optimizing
// BFS of Beamer et al. 2012 on symmetric graphs, top-down otherwise), so the
// depths are the same.
#pragma once
#include <type_traits>

#include "kernels.cuh"

namespace og {

struct BfsLoop {
  uint32_t done;          // the BFS has ended
  uint32_t level;         // depth of the current frontier (the source has 1)
  uint32_t bottom;        // the current level is expanded bottom-up
  uint32_t need_compact;  // the current frontier must be compacted
  uint32_t counted;       // its degrees are already out of `unexplored`
  uint32_t compact_go;    // gates of this level's launches
  uint32_t td_go;
  uint32_t bu_go;
  uint32_t epoch;         // compaction epoch of the current level
  uint32_t tile_next;     // tile counter of the top-down relax
  uint32_t pad[6];
  unsigned long long unexplored;  // degrees of the vertices never in a frontier
  unsigned long long fn;          // size of the current frontier
  unsigned long long bu[4];       // bottom-up: reached, their degrees, host / static records
  unsigned long long iterations, frontier_sum, edges_static, edges_dynamic;
  unsigned long long relax_timer[2];  // k_stamp slots of the top-down relax
};

constexpr uint64_t kBfsAlpha = 14, kBfsBeta = 24;

// After the compactions of a level: an empty frontier ends the BFS;
// otherwise choose the level's direction (bottom-up when the frontier's edges
// exceed unexplored / kBfsAlpha).
__global__ void k_bfs_ctl_mid(BfsLoop *st, const Counts *counts, int dopt) {
  if (threadIdx.x != 0) return;
  if (st->done) {
    st->td_go = 0;
    st->bu_go = 0;
    return;
  }
  if (st->need_compact) {
    const uint64_t n = (uint64_t)counts[0].n + counts[1].n;
    const uint64_t mf = counts[0].total + counts[1].total;
    if (n == 0) {
      st->done = 1;
      st->td_go = 0;
      st->bu_go = 0;
      return;
    }
    if (!st->counted) st->unexplored -= st->unexplored < mf ? st->unexplored : mf;
    st->fn = n;
    st->bottom = (dopt && mf > st->unexplored / kBfsAlpha) ? 1u : 0u;
    if (!st->bottom) {
      st->iterations++;
      st->frontier_sum += n;
      st->edges_static += counts[0].total;
      st->edges_dynamic += counts[1].total;
    }
  }
  st->td_go = st->bottom ? 0u : 1u;
  st->bu_go = st->bottom;
  st->tile_next = 0;
  if (st->bottom) st->bu[0] = st->bu[1] = st->bu[2] = st->bu[3] = 0;
}

// After the expansion: account a bottom-up level, decide whether the next
// frontier needs a compaction (top-down next), advance the level and epoch.
__global__ void k_bfs_ctl_end(BfsLoop *st, uint64_t V) {
  if (threadIdx.x != 0) return;
  if (st->done) {
    st->compact_go = 0;
    return;
  }
  if (st->bottom) {
    const uint64_t nn = st->bu[0];
    st->iterations++;
    st->frontier_sum += st->fn;
    st->edges_dynamic += st->bu[2];
    st->edges_static += st->bu[3];
    st->unexplored -= st->unexplored < st->bu[1] ? st->unexplored : st->bu[1];
    if (nn == 0) {
      st->done = 1;
      st->compact_go = 0;
      return;
    }
    const bool back = nn < V / kBfsBeta && nn < st->fn;  // small and shrinking: top-down again
    st->fn = nn;
    st->counted = 1;
    st->bottom = back ? 0u : 1u;
    st->need_compact = back ? 1u : 0u;
  } else {
    st->counted = 0;
    st->need_compact = 1;
  }
  st->level++;
  st->epoch++;
  st->compact_go = st->need_compact;
}

// Per-level op fields taken from device memory: the BFS depth of the level.
__device__ __forceinline__ void dev_prepare(BfsOp &op, const uint32_t *level) {
  if (level) op.newdepth = *level + 1;
}
template <bool W>
__device__ __forceinline__ void dev_prepare(MinOp<W> &, const uint32_t *) {}

// Relax of both regions over a fixed grid: tile counts come from the level's
// compaction (device memory); CTAs loop over the interleaved static / dynamic
// tiles as k_lbs_pair does.  Runs only when *go.
//
// Tiles are handed out by an atomic counter (*tile_next, zeroed by the
// control kernel that sets *go), not by a grid stride: a CTA that becomes
// resident late only finds fewer tiles, so the fixed grid may exceed what
// fits on the GPU at once without a second wave doing half the work.
template <class Src>
constexpr int dev_min_blocks() {  // CTAs per SM the register budget is sized for
  return std::is_same<Src, SrcP<true>>::value ? 4 : 5;
}
template <class Src0, class Src1, class Op>
__global__ void __launch_bounds__(kThreads, dev_min_blocks<Src0>()) k_lbs_pair_dev(LbsArgs a0, Src0 s0, LbsArgs a1, Src1 s1, Op op,
                                                           const Counts *counts, const uint32_t *go,
                                                           const uint32_t *level, uint32_t *tile_next) {
  static_assert(std::is_same<Src0, Src1>::value, "one tile body for both regions");
  if (*go == 0u) return;
  __shared__ LbsSh<Op> sh;
  __shared__ uint32_t s_b[2];
  __shared__ PairTile s_pt[2];
  // Both regions' arguments live in shared memory and one tile body serves
  // both: kept in registers across the tile loop they cost 98 registers per
  // thread (2 CTAs per SM) against 46 for the one-tile-per-CTA kernel.
  __shared__ LbsArgs s_a[2];
  __shared__ Src0 s_s[2];
  if (threadIdx.x == 0) {
    a0.n = counts[0].n;
    a0.total = counts[0].total;
    a0.pos_begin = 0;
    a0.pos_end = a0.total;
    a1.n = counts[1].n;
    a1.total = counts[1].total;
    a1.pos_begin = 0;
    a1.pos_end = a1.total;
    s_a[0] = a0;
    s_a[1] = a1;
    s_s[0] = s0;
    s_s[1] = s1;
  }
  dev_prepare(op, level);
  __syncthreads();
  const uint64_t n0 = (s_a[0].total + kTile - 1) / kTile, n1 = (s_a[1].total + kTile - 1) / kTile;
  const uint64_t n = n0 + n1;
  // The next tile's ticket (and its region split, by thread 0) is fetched
  // while the current tile runs (two slots).
  if (threadIdx.x == 0) {
    s_b[0] = atomicAdd(tile_next, 1u);
    s_pt[0] = pair_split(s_b[0], n0, n);
  }
  __syncthreads();
  for (int slot = 0;; slot ^= 1) {
    if (s_b[slot] >= n) break;
    const PairTile pt = s_pt[slot];
    if (threadIdx.x == 0) {
      const uint32_t nb = atomicAdd(tile_next, 1u);
      s_b[slot ^ 1] = nb;
      if (nb < n) s_pt[slot ^ 1] = pair_split(nb, n0, n);
    }
    lbs_tile(s_a[pt.r], s_s[pt.r], op, sh, pt.t);
    __syncthreads();  // the tile tables are rebuilt and the next slot is read after this
  }
}

// --------------------------------------------------- device-driven SSSP / CC
//
// Rounds of the min-relax algorithms (SSSP with or without the near/far
// split, CC by label propagation), driven the same way.  A round graph:
// compaction of the frontier (gated by round_go), k_min_ctl_a, compaction of
// the waiting set (gated by adv_go), k_min_ctl_b, the relax (gated by
// relax_go), k_min_ctl_end, the clear of the frontier.  A round that relaxes
// nothing hands an empty bitmap to the next parity, whose frontier
// compaction then finds nothing and moves on to the waiting set, as the host
// loop does.

struct MinLoop {
  uint32_t done;
  uint32_t epoch;      // epoch of the next compaction launch
  uint32_t thr;        // near threshold (SSSP split)
  uint32_t round_go;   // gates
  uint32_t adv_go;
  uint32_t relax_go;
  uint32_t far_min;    // smallest waiting distance (running, see the host loop)
  uint32_t delta;
  uint32_t split;
  uint32_t rounds;     // rounds that did work (the host's launch hint for the next query)
  uint32_t tile_next;  // tile counter of the relax
  uint32_t pad[5];
  unsigned long long iterations, frontier_sum, edges_static, edges_dynamic;
  unsigned long long relax_timer[2];  // k_stamp slots of the relax
};

// smallest waiting value a compaction of this epoch saw in its two regions
__device__ __forceinline__ uint32_t far_of_dev(const unsigned long long *keys, uint32_t epoch) {
  uint32_t m = 0xffffffffu;
  for (int r = 0; r < 2; r++)
    if ((uint32_t)(keys[r] >> 32) == epoch) m = min(m, ~(uint32_t)keys[r]);
  return m;
}

__device__ __forceinline__ void min_account(MinLoop *st, const Counts *counts) {
  st->iterations++;
  st->frontier_sum += (uint64_t)counts[0].n + counts[1].n;
  st->edges_static += counts[0].total;
  st->edges_dynamic += counts[1].total;
}

// After the frontier's compaction (epoch st->epoch).
__global__ void k_min_ctl_a(MinLoop *st, const Counts *counts, const unsigned long long *keys) {
  if (threadIdx.x != 0) return;
  st->adv_go = 0;
  st->relax_go = 0;
  st->tile_next = 0;
  if (st->done) return;
  st->rounds++;
  const uint64_t n = (uint64_t)counts[0].n + counts[1].n;
  if (st->split) st->far_min = min(st->far_min, far_of_dev(keys, st->epoch));
  st->epoch++;
  if (n) {
    st->relax_go = 1;
    min_account(st, counts);
  } else if (!st->split || st->far_min == 0xffffffffu) {
    st->done = 1;
  } else {
    const uint64_t t = (uint64_t)st->far_min + st->delta;
    st->thr = t > 0xffffffffull ? 0xffffffffu : (uint32_t)t;
    st->adv_go = 1;
  }
}

// After the waiting set's compaction (when it ran): its minimum is now exact.
__global__ void k_min_ctl_b(MinLoop *st, const Counts *counts, const unsigned long long *keys) {
  if (threadIdx.x != 0 || !st->adv_go) return;
  st->far_min = far_of_dev(keys, st->epoch);
  st->epoch++;
  if ((uint64_t)counts[0].n + counts[1].n) {
    st->relax_go = 1;
    min_account(st, counts);
  }
}

__global__ void k_min_ctl_end(MinLoop *st) {
  if (threadIdx.x != 0) return;
  st->round_go = st->done ? 0u : 1u;
}

}  // namespace og
