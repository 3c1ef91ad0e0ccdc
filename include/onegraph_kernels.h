/*
 * onegraph_kernels.h — kernel-level launchers of libog.so on caller-owned
 * device buffers (all pointers are device pointers unless stated; `stream` is
 * a cudaStream_t, NULL = the legacy default stream).  They run one kernel of
 * the engine's round on a frontier the caller compacted (og_k_compact in
 * onegraph.h), for unit tests and for hosts that drive the reference's
 * kernel-at-a-time loop themselves.  Each call synchronises its stream and
 * returns an og_status (onegraph.h); out-of-range indices found by the
 * kernels' bounds checks give OG_E_DEVICE with nothing written out of bounds.
 */
#ifndef ONEGRAPH_KERNELS_H
#define ONEGRAPH_KERNELS_H

#include <stdint.h>

#include "onegraph.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Packed edge records in device memory (the layout og_graph_records
 * returns): record e holds bits [e*bpe, (e+1)*bpe) of `words`, column in the
 * low bc bits, weight - wmin above; words holds (nrecords*bpe + 31)/32 + 2
 * u32 (two padding words). */
typedef struct og_k_records {
  const uint32_t *words;
  uint64_t nrecords;
  uint32_t bpe, bc, wmin, reserved;
} og_k_records;

/* One edge-balanced relax of a compacted frontier: for every listed vertex u
 * and edge (u, v, w), with u's edges at records off[u] .. off[u+1]-1,
 *   OG_ALGO_BFS:  v not in `visited` -> set v in visited and next,
 *                 value[v] = level + 1;
 *   OG_ALGO_SSSP: value[v] = min(value[v], value[u] + w), v set in next when
 *                 lowered;
 *   OG_ALGO_CC:   value[v] = min(value[v], value[u]), v set in next when
 *                 lowered;
 * all by atomicOr / atomicMin.  Replaces bfs_kernelStatic
 * (BFS/oneGraph_BFS/gpu_kernels.h:211-241), sssp_kernel
 * (SSSP/oneGraph/gpu_kernels.h:177-203) and cc_kernelStaticSwap
 * (CC/onegraph/gpu_kernels.h:133-157), whose min-stores are not atomic.
 * list, pref, tile: og_k_compact's outputs; n, total: its og_counts.
 * value, next, visited (BFS only): V entries / V-bit bitmaps. */
int og_k_relax(int algo, const uint32_t *list, const uint64_t *pref, const uint32_t *tile,
               uint32_t n, uint64_t total, const uint64_t *off, const og_k_records *rec,
               uint32_t V, uint32_t *value, uint32_t *next, uint32_t *visited, uint32_t level,
               void *stream);

/* The dynamic-region gather (fillEdgeArrByMultiThread,
 * BFS/oneGraph_BFS/GraphMeta.h:471-506) on caller buffers: the edges at
 * positions [pos_begin, pos_end) of the compacted list's degree prefix
 * (pos_begin a multiple of 2048; pos_end a multiple of 2048 or equal to
 * total), unpacked in list order:
 * out_col[p - pos_begin] = column, out_w[p - pos_begin] = weight (out_w may
 * be NULL: columns only).  `rec` may point at page-locked host records
 * (a device view from cudaHostGetDevicePointer), as the engine gathers. */
int og_k_gather(const uint32_t *list, const uint64_t *pref, const uint32_t *tile, uint32_t n,
                uint64_t total, const uint64_t *off, const og_k_records *rec, uint64_t pos_begin,
                uint64_t pos_end, uint32_t *out_col, uint32_t *out_w, void *stream);

/* Check of the engine's bounded device-side waits: runs one of them, in a
 * one-CTA launch, on a signal that is never given.  which = 0: the
 * compaction look-back of a tile whose predecessor never publishes;
 * which = 1: the persistent kernel's grid barrier expecting one CTA more than
 * the launch has.  The wait gives up after spin_limit polls (the engine uses
 * 2^24), sets its error bit and lets the kernel end, so this returns
 * OG_E_TIMEOUT and the CUDA context stays usable.  No reference counterpart. */
int og_k_wait_check(int which, uint32_t spin_limit);

/* Host-link probe for rooflines: best GB/s over `reps` timed runs (after one
 * warm-up) of moving `bytes` (>= 1 MiB, a multiple of 16) of the caller's
 * page-locked host buffer to the GPU.  mode 0: SM loads of the buffer through
 * its device view, 16-byte coalesced, as the engine's direct-mode kernels
 * read host records; 1: one cudaMemcpyAsync; 2: two cudaMemcpyAsync of half
 * the bytes each on two streams at once.  No reference counterpart. */
int og_link_probe(const void *host, uint64_t bytes, int mode, int reps, double *gbs);

#ifdef __cplusplus
}
#endif
#endif /* ONEGRAPH_KERNELS_H */
