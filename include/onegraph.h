/*
 * onegraph.h — C ABI of the GB300 out-of-memory graph engine (libog.so).
 *
 * Drop-in for OneGraph's Ascetic path: the C++ entry points bfs_opt / sssp_opt /
 * cc_opt / pr_opt (BFS/oneGraph_BFS/CalculateOpt.h:9, SSSP/oneGraph/CalculateOpt.h:12,
 * CC/onegraph/CalculateOpt.h:6, PR/OneGraph/CalculateOpt.h:13) and the
 * GraphMeta loader/planner they drive (BFS/oneGraph_BFS/GraphMeta.h:31-557).
 *
 * Conventions
 *  - Every call returns an og_status; on failure og_last_error() gives a message
 *    (thread-local).  No C++ exception crosses this boundary.
 *  - The engine owns its device and pinned buffers; the caller owns every output
 *    array it passes in.  An output pointer may be NULL: the result then stays
 *    in device memory (used to time the device-resident path).
 *  - Vertex values follow the reference: BFS depth(src) = 1 and unreached = V+1
 *    (GraphMeta.h:376-381); SSSP dist(src) = 1 and unreached = 0xFFFFFFFF
 *    (SSSP/oneGraph/GraphMeta.h:376-381); CC label = minimum vertex id that
 *    reaches the vertex (CC/onegraph/GraphMeta.h:341-345 init value = id).
 *  - One host thread per engine at a time.  Engines are independent.
 */
#ifndef ONEGRAPH_H
#define ONEGRAPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OG_ABI_VERSION 6

typedef enum og_status {
  OG_OK = 0,
  OG_E_ARG = 1,         /* invalid argument */
  OG_E_IO = 2,          /* file could not be opened / read / written */
  OG_E_FORMAT = 3,      /* CSR file is malformed (short, non-monotone, dst >= V) */
  OG_E_BUDGET = 4,      /* device budget cannot hold the per-vertex state */
  OG_E_CUDA = 5,        /* a CUDA call failed */
  OG_E_TIMEOUT = 6,     /* a bounded device-side wait gave up */
  OG_E_NOMEM = 7,       /* host allocation failed */
  OG_E_STATE = 8,       /* call not valid in the current state */
  OG_E_UNSUPPORTED = 9, /* algorithm not available for this graph kind */
  OG_E_DEVICE = 10      /* a kernel reported an out-of-range index */
} og_status;

/* Edge layout of a CSR file (GraphMeta.h:126-145 readDataFromFile):
 *   u64 V, u64 E, [u32 outDegree[V] for PR], u64 offsets[V] (no sentinel),
 *   Edge[E] with Edge = u32 (BFS/CC/PR; PR lists IN-neighbours) or
 *   {u32 toNode, u32 weight} (SSSP, globals.h:18-21 EdgeWithWeight). */
typedef enum og_graph_kind {
  OG_GRAPH_PLAIN = 0,    /* u32 columns                          */
  OG_GRAPH_WEIGHTED = 1, /* {u32 dst, u32 weight} pairs           */
  OG_GRAPH_PR = 2        /* u32 outDegree[V] block + u32 in-edges */
} og_graph_kind;

typedef enum og_algo {
  OG_ALGO_BFS = 0,
  OG_ALGO_SSSP = 1,
  OG_ALGO_CC = 2,
  OG_ALGO_PR = 3
} og_algo;

typedef struct og_graph og_graph;
typedef struct og_engine og_engine;

/* ---------------------------------------------------------------- graphs */

/* GraphMeta::readDataFromFile (BFS/oneGraph_BFS/GraphMeta.h:126-145, PR variant
 * PR/OneGraph/GraphMeta.h:131-149).  Validates the header, monotone offsets,
 * offsets <= E and every column < V. */
int og_graph_load(const char *path, int kind, og_graph **out);

/* Builds a graph from caller arrays (copied).  offsets has V entries (the file
 * layout) or V+1 when with_sentinel != 0; outdeg only for OG_GRAPH_PR. */
int og_graph_from_arrays(uint64_t V, uint64_t E, const uint64_t *offsets,
                         int with_sentinel, const void *edges,
                         const uint32_t *outdeg, int kind, og_graph **out);

/* Writes the graph in the reference's file layout (inverse of readDataFromFile). */
int og_graph_save(const og_graph *g, const char *path);

/* V, E, kind, and borrowed pointers to the host arrays (offsets with the V+1
 * sentinel; outdeg NULL unless OG_GRAPH_PR).  Any out pointer may be NULL. */
int og_graph_info(const og_graph *g, uint64_t *V, uint64_t *E, int *kind,
                  const uint64_t **offsets, const void **edges,
                  const uint32_t **outdeg);

/* Destroy every engine created on a graph before freeing the graph: engines
 * page-lock and read its host arrays. */
void og_graph_free(og_graph *g);

/* Graph::convert2BEL (BFS/cpu_BFS/Graph.h:134-163): writes <prefix>.bel.col
 * (u64 V, u64 0, u64 offsets[V]), <prefix>.bel.dst (u64 E, u64 0, u64
 * dst[E]) and, for weighted graphs, <prefix>.bel.val (u64 E, u64 0, u32 w[E]). */
int og_graph_save_bel(const og_graph *g, const char *prefix);

/* GraphMeta::transFileUintToUlong (BFS/oneGraph_BFS/GraphMeta.h:169-193):
 * reads the 32-bit-header CSR (u32 V, u32 E, u32 offsets[V], u32 dst[E]) and
 * writes the same graph with 64-bit edge entries (u32 V, u32 E, u32
 * offsets[V], u64 dst[E]).  out_path NULL follows the reference's naming: the
 * input path without its last four characters, plus "lcsr". */
int og_convert_uint_to_ulong(const char *in_path, const char *out_path);

/* The reverse graph as a new OG_GRAPH_PLAIN CSR: list u holds, sorted, every
 * v whose list contains u.  For the reference's PageRank files, whose lists
 * are in-neighbours (PR/OneGraph/GraphMeta.h:131-149), this is the out-edge
 * CSR that og_pr_l1_push traverses.  Weighted graphs are not supported.  No
 * reference counterpart (the reference pulls only). */
int og_graph_transpose(const og_graph *g, og_graph **out);

/* Symmetry of the edge set (every (u, v) has its reverse (v, u)), which lets
 * og_cc use its union-find path.  og_graph_set_symmetric records the caller's
 * assertion (1 or 0) without checking it; a wrong 1 gives wrong components.
 * og_graph_symmetric stores 1 or 0 in *symmetric, checking exactly on first use when not
 * known: every adjacency list sorted and every reverse edge found by binary
 * search, on all host threads (one pass over the edges plus E binary
 * searches).  Graphs from og_rmat_generate with OG_RMAT_SYMMETRIC are known
 * symmetric; unsorted adjacency lists count as not symmetric. */
int og_graph_set_symmetric(og_graph *g, int symmetric);
int og_graph_symmetric(og_graph *g, int *symmetric);

/* GraphMeta::findbignode (GraphMeta.h:150-165): first vertex after `last`
 * whose degree exceeds 3000, or `last` when there is none. */
uint32_t og_graph_findbignode(const og_graph *g, uint32_t last);

/* Seeded R-MAT generator (no reference counterpart: the reference points at
 * an external converter, README.md:8).  Deterministic on every platform. */
typedef struct og_rmat_params {
  uint32_t scale;       /* V = 2^scale                                    */
  uint32_t edge_factor; /* edge_factor * V tuples are drawn               */
  double a, b, c;       /* quadrant probabilities; d = 1 - a - b - c      */
  uint64_t seed;        /* tuple seed                                      */
  uint64_t weight_seed; /* seed of the per-edge weights                    */
  uint32_t wmin, wmax;  /* weights uniform in [wmin, wmax] (weighted only) */
  uint32_t flags;       /* OG_RMAT_* below                                 */
  uint32_t threads;     /* host threads (0 = all)                          */
} og_rmat_params;

#define OG_RMAT_SYMMETRIC 1u /* add the reverse of every edge            */
#define OG_RMAT_PERMUTE 2u   /* seeded bijective relabelling of vertex ids */
#define OG_RMAT_WEIGHTED 4u  /* {dst, w} edges (OG_GRAPH_WEIGHTED)       */
#define OG_RMAT_PR 8u        /* directed in-edge CSR + outDegree (OG_GRAPH_PR) */
#define OG_RMAT_ON_GPU 16u   /* draw, sort and dedup on cuda device 0     */

/* Self-loops and duplicate edges are always removed. */
int og_rmat_generate(const og_rmat_params *p, og_graph **out);

/* ---------------------------------------------------------------- planner */

/* Result of the region planner (GraphMeta.h:300-360 getMaxPartitionSize). */
typedef struct og_plan {
  uint64_t budget_bytes;     /* device budget the plan was made for          */
  uint64_t vertex_bytes;     /* bytes of per-vertex device state             */
  uint64_t fixed_bytes;      /* scratch independent of V and E               */
  uint64_t edge_capacity;    /* T: edges the remaining budget holds          */
  double advisek;            /* static share of T actually used              */
  double advisek_auto;       /* the reference's (10 - E/T)/9 heuristic       */
  uint64_t max_partition;    /* floor(advisek * T) clamped to E              */
  uint32_t static_vertices;  /* Vs: vertices [0, Vs) are static              */
  uint64_t static_edges;     /* off[Vs]: edges preloaded once                */
  uint64_t dynamic_edges;    /* E - static_edges                             */
  uint64_t chunk_edges;      /* staging capacity per buffer (two buffers)    */
  uint32_t edge_bytes;       /* packed record size rounded up to bytes       */
  uint32_t edge_bits;        /* packed record size: column + weight bits     */
  uint32_t stage_edge_bytes; /* unpacked edge in a staging buffer            */
  uint32_t reserved;
} og_plan;

/* Pure host computation, no device needed.  `offsets` has V+1 entries.
 * budget_bytes == 0 selects the reference's 12 GiB (GraphMeta.h:305);
 * advisek <= 0 selects the heuristic (GraphMeta.h:311-324). */
int og_plan_compute(uint64_t V, uint64_t E, const uint64_t *offsets, int kind,
                    uint64_t budget_bytes, double advisek, uint32_t flags,
                    og_plan *out);

/* The planner for a given graph with the engine's real edge width: the
 * engine keeps edges as bit-packed records of bits(V-1) column bits plus
 * bits(wmax - wmin) weight bits (33 bits for R-MAT 27 with weights in
 * [1, 64]) in the page-locked host copy and the static region; staging
 * buffers hold unpacked edges (u32 column + 1, 2 or 4 weight bytes).
 * og_plan_compute, which has no graph, charges the reference's sizeof(Edge)
 * (4 or 8 bytes) per edge.  With OG_CFG_REPLACE in flags the plan is the one
 * such an engine runs: the static prefix halved as described there. */
int og_graph_plan(og_graph *g, uint64_t budget_bytes, double advisek, uint32_t flags,
                  og_plan *out);

/* The bit-packed edge records engines read (built on first use): record e
 * is bits [e*bpe, (e+1)*bpe) of `words` (bit i of the stream is bit i%32 of
 * word i/32), column in the low bc bits, weight - wmin in the bits above.
 * nwords includes two zero padding words.  The arrays belong to the graph. */
int og_graph_records(og_graph *g, const uint32_t **words, uint64_t *nwords, uint32_t *bpe,
                     uint32_t *bc, uint32_t *wmin);

/* ---------------------------------------------------------------- engine */

typedef struct og_config {
  uint64_t budget_bytes; /* 0 = 12 GiB (GraphMeta.h:305)                  */
  double advisek;        /* <= 0 = heuristic; the CLI's --advisek          */
  uint32_t flags;        /* OG_CFG_* below                                 */
  int32_t device;        /* CUDA device ordinal                            */
} og_config;

#define OG_CFG_DIRECT 1u  /* dynamic region relaxed straight from pinned host
                             memory instead of through device staging buffers */
#define OG_CFG_NO_PIN 2u  /* do not page-lock the host CSR (ATS access only)  */
#define OG_CFG_BATCH 8u   /* also hold the 3 x u64 per-vertex masks of og_bfs_batch */
#define OG_CFG_BATCH_LEVELS 16u /* og_bfs_batch drives levels from the host (one
                                   kernel sequence per level) instead of the
                                   persistent cooperative kernel */
#define OG_CFG_NO_STATIC 32u /* keep no static region: every active edge comes
                                 from host memory each round.  With staging this
                                 is the Subway scheme (BFS/sbw_BFS/main.cpp:323-506),
                                 with OG_CFG_DIRECT|OG_CFG_NO_PIN the unified-
                                 memory scheme (BFS/usm_BFS/main.cpp:120-222) */
/* Also hold the state of og_sssp_batch for up to k sources per pass
 * (1 <= k <= 32): a row of 4, 8, 16 or 32 u32 distances per vertex (k
 * rounded up), a pending-source mask per vertex and a near-source mask per
 * list entry, 4 B x row + 8 B per vertex, sharing one allocation with the
 * OG_CFG_BATCH masks (24 B per vertex: k <= 4 adds nothing to them).
 * Weighted graphs only. */
#define OG_CFG_SSSP_BATCH(k) ((uint32_t)(k) << 8)
#define OG_CFG_PR 4u      /* also hold PageRank state for a PLAIN/WEIGHTED
                             graph, read as symmetric (in-edges = out-edges,
                             outDegree = degree); implied for OG_GRAPH_PR    */
/* Static-region replacement (Ascetic's fragment swap, which the reference
 * declares and never defines: bfs_kernelStaticSwap, recordFragmentVisit,
 * setFragmentData in BFS/oneGraph_BFS/gpu_kernels.h:46-66,153-176 and
 * FragmentData in globals.h:22-33).  Half of the static region's device
 * bytes become slots for fragments of the dynamic region (the packed record
 * stream cut into fragments of OG_PARAM_FRAGMENT_WORDS words), first filled
 * with the fragments that follow the static prefix.  The relax counts the
 * records it lists per fragment; between rounds, once as many records as the
 * slots hold have been listed since the last step and at the end of every
 * query, the host replaces slots whose fragments were read least with
 * the most-read fragments that have none, copying at most a quarter of the
 * host-link bytes read since the last step, and a slot holds its fragment
 * across rounds and queries.  Reads of a fragment with a
 * slot come from device memory, the others from the host copy, so results
 * are identical to an engine without it.  Needs OG_CFG_DIRECT and a static
 * region; og_bfs, og_sssp and label-propagation og_cc run host-driven rounds
 * through the slots; other queries read the host copy; no clones. */
#define OG_CFG_REPLACE 64u

/* Per-query counters (what CalculateOpt.h:193-208 prints, plus rooflines). */
typedef struct og_stats {
  uint32_t iterations;       /* rounds of the hot loop                      */
  uint32_t chunks;           /* dynamic chunks moved                        */
  uint64_t frontier_sum;     /* "nodeSum": vertices expanded over all rounds */
  uint64_t static_vertices;  /* expanded in the static region               */
  uint64_t edges_static;     /* edges relaxed from the resident prefix      */
  uint64_t edges_dynamic;    /* edges gathered from host memory and relaxed */
  uint64_t link_bytes;       /* bytes read over the host link               */
  double ms_total;           /* host wall time of the query                 */
  double ms_static;          /* device time of static relax kernels         */
  double ms_dynamic;         /* device time of dynamic gather+relax         */
  double ms_compact;         /* device time of frontier compaction          */
  double residual;           /* PR: last L1 delta; otherwise 0              */
  uint64_t launches;         /* kernels launched for the query              */
  double ms_gather;          /* device time of the dynamic gather kernels   */
  double ms_relax;           /* device-driven rounds with
                                OG_PARAM_RELAX_TIMER: time of the (top-down)
                                relax launches, between stamp kernels
                                enqueued right before and after each;
                                otherwise 0                                 */
} og_stats;

/* initGraphHost + getMaxPartitionSize + initGraphDevice
 * (GraphMeta.h:204-291): plans the regions and preloads the static prefix. */
int og_engine_create(og_graph *g, const og_config *cfg, og_engine **out);
int og_engine_plan(const og_engine *e, og_plan *out);
void og_engine_destroy(og_engine *e);

/* bfs_opt loop body for one source (BFS/oneGraph_BFS/CalculateOpt.h:55-209).
 * out_depth: V entries or NULL. */
int og_bfs(og_engine *e, uint32_t src, uint32_t *out_depth, og_stats *st);

/* sssp_opt (SSSP/oneGraph/CalculateOpt.h:12-192); OG_GRAPH_WEIGHTED only. */
int og_sssp(og_engine *e, uint32_t src, uint32_t *out_dist, og_stats *st);

/* cc_opt (CC/onegraph/CalculateOpt.h:6-144). */
int og_cc(og_engine *e, uint32_t *out_label, og_stats *st);

/* pr_opt (PR/OneGraph/CalculateOpt.h:13-185): ranks start at 1.0, a vertex
 * keeps iterating while |new - old| > threshold (0.001 in the reference,
 * gpu_kernels.h:307).  Values are FP32.  max_rounds <= 0 means unbounded. */
int og_pr(og_engine *e, float *out_rank, double threshold, int max_rounds,
          og_stats *st);

/* Precision-study PageRank: normalised ranks (sum 1), FP32 values and FP32
 * accumulation, every vertex every iteration, stop when the FP64 L1 delta
 * (reduced on the GPU) drops below tol or after max_iter iterations.
 * No reference counterpart beyond the pr_cal_cpu formula (PR/usm/pr.cpp:149-187). */
int og_pr_l1(og_engine *e, float *out_rank, double damping, double tol,
             int max_iter, og_stats *st);
/* The same L1-stopped PageRank by push: the engine's graph holds OUT-edges
 * (og_graph_transpose of an in-edge PR graph; out-degrees are the list
 * lengths), every vertex adds rank / out-degree to each out-neighbour's sum
 * with an FP32 atomicAdd, then the update and the FP64 L1 reduction of
 * og_pr_l1 follow.  The summation order of atomics varies from run to run, so
 * results agree with og_pr_l1 to FP32 rounding, not bit for bit.  Needs
 * OG_CFG_PR. */
int og_pr_l1_push(og_engine *e, float *out_rank, double damping, double tol, int max_iter,
                  og_stats *st);

/* Multi-source BFS: up to 64 sources in one level-synchronous pass over
 * per-vertex 64-bit visited / frontier masks, so every edge read (including
 * those streamed from host memory) serves all sources.  No reference
 * counterpart: the reference runs its sources one after another
 * (CalculateOpt.h:55-209).  Needs OG_CFG_BATCH.  out: n x V depths,
 * source-major, same convention as og_bfs, or NULL (with out != NULL the
 * engine keeps an n x V u32 device depth matrix outside the budget);
 * checks: 2n values, {vertices reached, sum of their depths} per source, or
 * NULL.  Depths are identical to n separate og_bfs calls. */
int og_bfs_batch(og_engine *e, const uint32_t *srcs, int n, uint32_t *out,
                 uint64_t *checks, og_stats *st);

/* og_bfs_batch with source i's V depths written to outs[i] (n host arrays
 * of V u32 each) instead of one contiguous n x V array: callers whose
 * requests each own a result buffer (the server's BFS requests) share one
 * pass.  The persistent kernel writes byte depths (an n x V byte device
 * matrix kept between calls, outside the budget), and each row is widened
 * in a V-entry device buffer and copied to its output (page-locked outputs
 * copy at the link's rate).  If some depth reaches 255 the
 * outputs are filled by single-source runs instead.  Checks and depths equal
 * og_bfs_batch's; needs the persistent kernel (not OG_CFG_BATCH_LEVELS).
 * No reference counterpart (CalculateOpt.h:55-209 runs sources one by one). */
int og_bfs_batch_to(og_engine *e, const uint32_t *srcs, int n, uint32_t *const *outs,
                    uint64_t *checks, og_stats *st);
/* Multi-source SSSP: up to k sources (the engine's OG_CFG_SSSP_BATCH(k)) in
 * one pass.  Every round compacts the vertices whose distance from some
 * source improved, and one edge-balanced relax serves every source active at
 * a vertex, so an edge record read from HBM or over the host link is read once
 * for all of them; the sources share the near/far threshold of og_sssp
 * (OG_PARAM_SSSP_DELTA).  No reference counterpart: the reference runs
 * sssp_opt once per source (SSSP/oneGraph/CalculateOpt.h:12-30).
 * out: n x V distances, source-major, same convention as og_sssp, or NULL;
 * checks: 2n values, {vertices reached, sum of their distances} per source,
 * or NULL.  Distances are identical to n separate og_sssp calls. */
int og_sssp_batch(og_engine *e, const uint32_t *srcs, int n, uint32_t *out, uint64_t *checks,
                  og_stats *st);

/* og_sssp_batch round by round, so that sources can join a pass in flight
 * (the server's continuous batching).  Slots are 0..k-1.
 * og_sssp_batch_begin clears every slot.  og_sssp_batch_join seeds slots[i]
 * with source srcs[i], at any round boundary: a late source starts below the
 * shared threshold and is expanded every round until it has caught up, with
 * the same distances.  og_sssp_batch_step runs one round; *pending receives
 * the slots that still have work (a joined slot outside it holds its final
 * distances and may be read and joined again), *done = 1 once nothing is
 * left.  og_sssp_batch_checks writes {reached, sum of distances} of every
 * slot in the mask `slots` to out[2 s], out[2 s + 1] (64 values).
 * og_sssp_batch_fetch copies slot `slot`'s V distances to host memory.
 * Any other query on the engine (og_bfs, og_pr_l1, og_sssp_batch, ...) ends
 * the session: it reuses the session's state, and the session calls then
 * return OG_E_STATE until the next og_sssp_batch_begin.  No reference
 * counterpart. */
int og_sssp_batch_begin(og_engine *e);
int og_sssp_batch_join(og_engine *e, const uint32_t *srcs, const uint32_t *slots, int n);
int og_sssp_batch_step(og_engine *e, uint32_t *pending, int *done, og_stats *st);
int og_sssp_batch_checks(og_engine *e, uint32_t slots, uint64_t *out);
int og_sssp_batch_fetch(og_engine *e, uint32_t slot, uint32_t *out);

/* og_bfs_batch level by level, so that sources can join a batch in flight
 * (the server's continuous batching of BFS requests).  Needs OG_CFG_BATCH;
 * slots are 0..63, one bit of the per-vertex masks each.
 * og_bfs_batch_begin clears every slot; with record_depths != 0 it keeps a
 * 64 x V u32 device depth matrix (outside the budget) for
 * og_bfs_batch_fetch.  og_bfs_batch_join seeds slots[i] with source srcs[i]
 * at the current level boundary: a source that joins at level L has depth 1
 * there and its vertices get depth (level - L + 1), so its depths and checks
 * are those of og_bfs from that source.  A slot still in flight cannot be
 * joined (OG_E_STATE).  og_bfs_batch_step expands one level for every slot in
 * flight; *pending receives the slots still in flight (a slot that reached no
 * new vertex has finished: its checks are final and it may be joined again),
 * *done = 1 once none is.  og_bfs_batch_checks writes {vertices reached, sum
 * of depths} of every slot in the mask `slots` to out[2 s], out[2 s + 1] (128
 * values, 0 for slots outside the mask).  og_bfs_batch_fetch copies a
 * finished slot's V depths (og_bfs's convention) to host memory.  Every level
 * is expanded top-down.  Any other query on the engine ends the session, as
 * for og_sssp_batch_begin.  No reference counterpart: the reference runs its
 * BFS sources one after another (BFS/oneGraph_BFS/CalculateOpt.h:55-209). */
int og_bfs_batch_begin(og_engine *e, int record_depths);
int og_bfs_batch_join(og_engine *e, const uint32_t *srcs, const uint32_t *slots, int n);
int og_bfs_batch_step(og_engine *e, uint64_t *pending, int *done, og_stats *st);
int og_bfs_batch_checks(og_engine *e, uint64_t slots, uint64_t *out);
int og_bfs_batch_fetch(og_engine *e, uint32_t slot, uint32_t *out);

/* og_bfs_batch with byte depths, for hosts that fetch many depth arrays:
 * out[s*V + v] = the depth when it is at most 254 (the source has 1), 0 when
 * v is unreached, 255 when the depth is 255 or more (*clamped, when not
 * NULL, receives the number of such entries; their exact depths come from
 * og_bfs_batch).  A quarter of og_bfs_batch's bytes to copy to the host.
 * Both keep their n x V device depth matrix (outside the budget) until the
 * engine is destroyed, so repeated calls allocate nothing.  No reference
 * counterpart. */
int og_bfs_batch_u8(og_engine *e, const uint32_t *srcs, int n, uint8_t *out, uint64_t *clamped,
                    uint64_t *checks, og_stats *st);

/* Page-locked host memory for result buffers: device-to-host copies of
 * results into it run at the host link's rate, where pageable memory is
 * staged by the CUDA driver.  Free with og_host_free. */
int og_host_alloc(uint64_t bytes, void **out);
void og_host_free(void *p);

/* og_bfs_batch runs all levels in one persistent cooperative kernel (static
 * edges from HBM, dynamic edges read straight from page-locked host memory);
 * with out == NULL the whole batch is captured once as a CUDA graph and
 * replayed (og_stats.chunks == 1 reports a replay).  The persistent kernel
 * has candidate (CTA size, edges per thread) configurations; the tile they
 * span is also where high-degree vertices are split. */
typedef struct og_tune_result {
  int configs;      /* candidates timed                          */
  int best;         /* index of the fastest                      */
  int block[8];     /* CTA size of each candidate                */
  int items[8];     /* edge positions per thread of each         */
  float ms[8];      /* best kernel time of each (ms)             */
} og_tune_result;

/* Autotuner: times every candidate on this engine and these sources (reps
 * timed runs each after one warm-up run) and keeps the fastest for later
 * og_bfs_batch calls. */
int og_bfs_batch_tune(og_engine *e, const uint32_t *srcs, int n, int reps,
                      og_tune_result *res);

/* Selects a candidate directly (-1 = default), e.g. from a saved tuning. */
int og_bfs_batch_set_config(og_engine *e, int config);

/* A query context on a parent engine's resident graph: the offsets, static
 * edges and page-locked host CSR are shared, the per-query state (values,
 * frontiers, lists, staging, PageRank/batch arrays, streams) is its own, so
 * several host threads can run queries on one graph concurrently, one context
 * each.  Destroy every clone before its parent.  No reference counterpart
 * (the reference runs one query at a time). */
int og_engine_clone(og_engine *parent, og_engine **out);

/* Engine parameters.
 * OG_PARAM_SSSP_DELTA: width of og_sssp's near/far split.  0 relaxes every
 *   frontier vertex each round, as the reference does
 *   (SSSP/oneGraph/CalculateOpt.h:73-185); d > 0 expands only frontier
 *   vertices whose distance is below a threshold that moves in steps of d,
 *   which re-expands fewer vertices (fewer edges over the host link) at the
 *   cost of more rounds.  Default: (smallest + largest weight) / 16, at least
 *   1 (4 for weights in [1, 64]).  Distances are exact for every value.
 *   Clones inherit it. */
#define OG_PARAM_SSSP_DELTA 1
/* OG_PARAM_CC_METHOD: how og_cc computes the labels (minimum vertex id that
 *   reaches each vertex; the component minimum on a symmetric graph).
 *   OG_CC_AUTO (default): union-find when the graph is known symmetric
 *   (og_graph_symmetric / og_graph_set_symmetric / symmetric R-MAT), label
 *   propagation otherwise.  OG_CC_LABEL_PROPAGATION: the reference's frontier
 *   propagation (CC/onegraph/gpu_kernels.h:105-157).  OG_CC_UNION_FIND:
 *   sampling union-find (hook each vertex with its first two neighbours,
 *   expand only the edges of vertices outside the giant component), an error
 *   on a graph not known symmetric.  Labels are identical either way. */
#define OG_PARAM_CC_METHOD 2
#define OG_CC_AUTO 0
#define OG_CC_LABEL_PROPAGATION 1
#define OG_CC_UNION_FIND 2
/* OG_PARAM_BFS_DIRECTION: OG_BFS_AUTO (default) expands large BFS levels
 *   bottom-up on graphs known to be symmetric: every unvisited vertex scans
 *   its own neighbours and stops at the first one in the frontier (Beamer's
 *   direction optimization: a level goes bottom-up when the frontier's edges
 *   exceed the unexplored edges / 14, and back to top-down when the frontier
 *   is below V / 24 and shrinking).  og_bfs_batch applies the same rule to
 *   each source of the batch separately: in one level the bottom-up sources
 *   are found by scans of the vertices missing them and the top-down sources
 *   by pushes from their frontiers.  OG_BFS_TOP_DOWN expands every level from
 *   the frontier, as the reference does.  Depths are identical either way. */
#define OG_PARAM_BFS_DIRECTION 3
#define OG_BFS_AUTO 0
#define OG_BFS_TOP_DOWN 1
/* OG_PARAM_LEVEL_LOOP: OG_LOOP_AUTO (default) runs the levels / rounds of
 *   og_bfs, og_sssp and label-propagation og_cc from two CUDA graphs replayed
 *   back to back, with every per-round decision taken by kernels (direct mode
 *   or a fully resident graph; staged engines keep the host loop); the host
 *   checks for the end every few rounds.  OG_LOOP_HOST waits for each round's
 *   counts on the host.  Results are identical. */
#define OG_PARAM_LEVEL_LOOP 4
#define OG_LOOP_AUTO 0
#define OG_LOOP_HOST 1
/* OG_PARAM_RELAX_TIMER: 1 brackets every relax launch of the device-driven
 *   rounds with two one-thread stamp kernels that read the GPU's global timer
 *   (og_stats.ms_relax); 0 (default) leaves them out of the captured rounds. */
#define OG_PARAM_RELAX_TIMER 5
/* OG_PARAM_SSSP_BATCH_DELTA: near/far width of og_sssp_batch, shared by its
 *   sources.  0 (default) expands every improved (vertex, source) pair every
 *   round, as the reference's SSSP rounds do: the sources then advance in
 *   lockstep by hops and one edge read serves many of them at once; d > 0
 *   applies og_sssp's split with one threshold for all sources (fewer
 *   re-expansions per source, less sharing).  Distances are exact for every
 *   value.  Clones inherit it. */
#define OG_PARAM_SSSP_BATCH_DELTA 6
/* OG_PARAM_FRAGMENT_WORDS: words per fragment of an OG_CFG_REPLACE engine,
 *   a power of two in [2^8, 2^20].  Default: the power of two nearest
 *   packed words / 4096, clamped to [2^8, 2^14].  Setting it lays the slots
 *   out again (same device bytes) and refills them as at creation. */
#define OG_PARAM_FRAGMENT_WORDS 7
int og_engine_set_param(og_engine *e, int param, double value);
int og_engine_get_param(const og_engine *e, int param, double *value);

/* Device bytes of the shared resident graph (0 for a clone) and of one
 * query context. */
int og_engine_bytes(const og_engine *e, uint64_t *resident, uint64_t *context);

/* Counters of an OG_CFG_REPLACE engine since its creation (or the last
 * OG_PARAM_FRAGMENT_WORDS change).  The reference declares the fragment
 * records (recordFragmentVisit, BFS/oneGraph_BFS/gpu_kernels.h:168-170) but
 * reports nothing. */
typedef struct og_fragment_stats {
  uint64_t fragments;       /* fragments of the record stream               */
  uint32_t slots;           /* device slots                                 */
  uint32_t fragment_words;  /* words per fragment                           */
  uint64_t swaps;           /* fragments copied into a slot after creation  */
  uint64_t swap_bytes;      /* bytes those copies read over the host link   */
  uint64_t records_slots;   /* dynamic-region records read from slots       */
  uint64_t records_host;    /* dynamic-region records read from host memory */
} og_fragment_stats;
int og_engine_fragment_stats(const og_engine *e, og_fragment_stats *out);

/* Checksum of the last result on the device, reduced in a fixed order:
 * BFS/SSSP {vertices reached, sum of their values}; CC {components, sum of
 * labels}; PR {V, bits of the FP64 sum of the ranks}. */
int og_result_checksum(og_engine *e, int algo, uint64_t *out);

/* Copies the last result of the given algorithm from device memory into out
 * (V entries: u32 for BFS/SSSP/CC, float for PR). */
int og_result_fetch(og_engine *e, int algo, void *out);

/* ------------------------------------------------------- kernel launchers */

/* Frontier counts written by og_k_compact (device memory, 16 bytes). */
typedef struct og_counts {
  uint32_t n;      /* vertices listed (active and with at least one edge) */
  uint32_t pad;
  uint64_t total;  /* sum of their degrees                                */
} og_counts;

/* The frontier compaction kernel on caller-owned device buffers: the active
 * vertices of [v_begin, v_end) in the bitmap `bits` that have edges, in
 * increasing id order, their exclusive u64 degree prefix (out_pref[n] =
 * total) and the 2048-edge tile map of the edge-balanced expansion.  Replaces
 * setStaticAndOverloadLabelBool + myReduction + myExclusive_scan +
 * setStaticActiveNodeArray / setOverloadNodePointerSwap
 * (BFS/oneGraph_BFS/gpu_kernels.h:243-379) and the flag / scan / queue /
 * pointer steps of SubgraphGenerator::generate (PR/sbw/subgraph_generator.h:189-234).
 * bits: ceil(v_end/32) u32 words; off: V+1 u64 offsets with V >= v_end;
 * out_list: list_cap entries; out_pref: list_cap+1; out_tile: tile_cap
 * (>= total/2048 + 1); out_counts: one og_counts.  The look-back scratch is
 * allocated and released inside the call; the call synchronises `stream`
 * (a cudaStream_t, NULL = legacy default stream) and returns OG_E_DEVICE if a
 * capacity was too small. */
int og_k_compact(const uint32_t *bits, uint32_t v_begin, uint32_t v_end,
                 const uint64_t *off, uint32_t *out_list, uint64_t *out_pref,
                 uint64_t list_cap, uint32_t *out_tile, uint64_t tile_cap,
                 og_counts *out_counts, void *stream);

/* og_k_compact without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc at the point
 * where they compact a frontier, e.g. a host application that has handed all
 * device memory to its own pool allocator, a plugin loaded into another
 * runtime that only allows that runtime's allocator, or a latency-critical
 * loop that cannot pay for the device synchronisation cudaMalloc/cudaFree
 * imply.  Same arguments, results and status as og_k_compact; the caller
 * still passes every input and output buffer.
 * Scratch: a fixed array of 229,700 bytes (28 B per compaction tile for 8192
 * tiles, plus 324 B) inside libog.so, present on every device that loads the
 * library until the process exits.  Limit: 8192 tiles of 1024 bitmap words
 * (32768 vertices) per call, i.e. 2^28 vertices when v_begin is a multiple
 * of 32 and 2^28 - 32 otherwise; larger ranges return OG_E_ARG.
 * The first call on a device looks up that array's device address, so make it
 * before any stream capture.  Every call shares the array: calls that overlap
 * on the GPU (other streams, other host threads) race and must not be issued;
 * each call clears the part it uses and synchronises `stream` before
 * returning. */
int og_k_compact_noalloc(const uint32_t *bits, uint32_t v_begin, uint32_t v_end,
                         const uint64_t *off, uint32_t *out_list,
                         uint64_t *out_pref, uint64_t list_cap,
                         uint32_t *out_tile, uint64_t tile_cap,
                         og_counts *out_counts, void *stream);

/* ---------------------------------------------------------------- serving */

/* A request loop over several resident graphs (no reference counterpart).
 * Requests are queued as they arrive and admitted by worker threads when a
 * query context of their graph is free or a new one fits budget_bytes; the
 * work of concurrent requests overlaps on the GPU.  On a graph added with
 * OG_CFG_SSSP_BATCH(k), k > 1, SSSP requests run in multi-source passes
 * (og_sssp_batch_*) of up to min(k, max_batch) sources: requests that arrive
 * while a pass runs join its free slots between rounds, and each is answered
 * as soon as its own distances are final.  BFS requests for the same graph
 * that queue up while others run are fused into one og_bfs_batch pass (up to
 * max_batch), and queued PageRank requests for the same graph and iteration
 * count share one computation.  Results are identical to running each
 * request alone. */
typedef struct og_server og_server;

typedef struct og_server_config {
  uint64_t budget_bytes; /* device bytes for all resident graphs and query
                            contexts (0 = limited only by device memory)   */
  int32_t workers;       /* host threads driving queries (1..64)           */
  int32_t max_batch;     /* BFS requests per fused pass (1 = no batching)  */
  int32_t device;
  uint32_t flags;        /* OG_SERVER_* below                              */
} og_server_config;

/* BFS requests of a graph run as a level-by-level pass (og_bfs_batch_begin /
 * _join / _step) that requests queued meanwhile join at every level
 * boundary, each answered as soon as its source has finished.  Without it a
 * BFS pass takes the requests queued at its start (og_bfs_batch, persistent
 * kernel with a per-source direction choice). */
#define OG_SERVER_BFS_JOIN 1u

typedef struct og_request {
  int32_t graph;      /* id from og_server_add_graph                       */
  int32_t algo;       /* og_algo                                           */
  uint32_t source;    /* BFS / SSSP                                        */
  int32_t iterations; /* PageRank iterations (og_pr_l1, tol 0), 0 = 5       */
  void *out;          /* optional caller buffer of V results, valid until the
                         response arrives; NULL = checksum only             */
  uint64_t user;      /* echoed in the response                            */
} og_request;

typedef struct og_response {
  uint64_t ticket;
  uint64_t user;
  int32_t status;     /* og_status of the request                          */
  int32_t graph;
  int32_t algo;
  uint32_t source;
  uint32_t batch;     /* requests served by the same GPU pass (a
                         multi-source SSSP pass: those it had answered when
                         this one finished, this one included)            */
  uint32_t reserved;
  double t_submit_ms; /* server clock (ms since og_server_create)          */
  double t_start_ms;
  double t_done_ms;
  uint64_t checksum[2]; /* og_result_checksum, or {reached, depth sum} of a
                           fused BFS                                       */
} og_response;

typedef struct og_server_stats {
  uint64_t submitted, completed, gpu_passes, batched_requests;
  uint64_t contexts_created, used_bytes;
  uint64_t launches;  /* kernels the server's passes launched */
} og_server_stats;

int og_server_create(const og_server_config *cfg, og_server **out);
/* Creates the graph's resident engine with gcfg (its budget and advisek);
 * must precede the first submit.  The graph must outlive the server. */
int og_server_add_graph(og_server *s, og_graph *g, const og_config *gcfg, int *graph_id);
int og_server_submit(og_server *s, const og_request *r, uint64_t *ticket);
/* Up to max responses; waits up to wait_ms (-1 = until one is ready or
 * nothing is in flight, 0 = no wait). */
int og_server_poll(og_server *s, og_response *out, int max, int *n, int wait_ms);
/* Waits until every submitted request has a response (timeout_ms < 0: no limit). */
int og_server_drain(og_server *s, int timeout_ms);
int og_server_get_stats(og_server *s, og_server_stats *out);
void og_server_destroy(og_server *s);

const char *og_last_error(void);
int og_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ONEGRAPH_H */
