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
  uint32_t pad[7];
  unsigned long long unexplored;  // degrees of the vertices never in a frontier
  unsigned long long fn;          // size of the current frontier
  unsigned long long bu[4];       // bottom-up: reached, their degrees, host / static records
  unsigned long long iterations, frontier_sum, edges_static, edges_dynamic;
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

// Top-down relax of both regions over a fixed grid: tile counts come from
// the level's compaction (device memory); CTAs loop over the interleaved
// static / dynamic tiles as k_lbs_pair does.  Runs only when *go; the BFS
// depth written is *level + 1.
template <class Src0, class Src1>
__global__ void __launch_bounds__(kThreads) k_lbs_pair_dev(LbsArgs a0, Src0 s0, LbsArgs a1, Src1 s1, BfsOp op,
                                                           const Counts *counts, const uint32_t *go,
                                                           const uint32_t *level) {
  if (*go == 0u) return;
  __shared__ LbsShared<BfsOp::Val> sh;
  op.newdepth = *level + 1;
  a0.n = counts[0].n;
  a0.total = counts[0].total;
  a0.pos_begin = 0;
  a0.pos_end = a0.total;
  a1.n = counts[1].n;
  a1.total = counts[1].total;
  a1.pos_begin = 0;
  a1.pos_end = a1.total;
  const uint64_t n0 = (a0.total + kTile - 1) / kTile, n1 = (a1.total + kTile - 1) / kTile;
  const uint64_t n = n0 + n1;
  for (uint64_t b = blockIdx.x; b < n; b += gridDim.x) {
    const uint64_t lo = b * n0 / n, hi = (b + 1) * n0 / n;
    if (hi > lo) lbs_tile(a0, s0, op, sh, lo);
    else lbs_tile(a1, s1, op, sh, b - hi);
    __syncthreads();  // the tile tables are rebuilt for the next tile
  }
}

}  // namespace og
