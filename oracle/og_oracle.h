/*
 * og_oracle.h — CPU restatement of OneGraph's BFS / SSSP / CC / PageRank paths.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the CUDA engine
 * (libog.so) is compared against; it is never linked into the product.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Graph layout used by every function: the reference's CSR (GraphMeta.h:126-145)
 * with the V+1 sentinel added, i.e. off[0..V] (off[V] == E), u32 columns (or
 * {u32 dst, u32 w} pairs for SSSP) and, for PageRank, u32 outDegree[V] with the
 * column array holding IN-neighbours.
 *
 * Parity pins: ora_bfs, ora_cc and ora_pr_cpu are checked bit-for-bit against
 * the reference's own CPU programs compiled from its sources
 * (oracle/build_ref.sh -> oracle/_ref/, fixtures in tests/golden/).
 * ora_sssp_dijkstra has no reference CPU counterpart (the reference ships no CPU
 * SSSP); it is cross-checked against ora_sssp_frontier, a restatement of the
 * reference's label-correcting loop.
 */
#ifndef OG_ORACLE_H
#define OG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* BFS/cpu_BFS/main.cpp:114-209 (runCPUBFS): dense level sweep, in-place
 * updates, separate next-frontier flags.  depth(src) = 1, unreached = 0xFFFFFFFF.
 * Returns the number of rounds executed. */
int ora_bfs(uint32_t V, const uint64_t *off, const uint32_t *col, uint32_t src,
            uint32_t *out);

/* CC/serial/serial.cpp:154-213: min-label propagation, labels start at the
 * vertex id, every vertex active in round 0.  Returns the number of rounds. */
int ora_cc(uint32_t V, const uint64_t *off, const uint32_t *col, uint32_t *out);
uint64_t ora_cc_round_bounded(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                              uint64_t max_edges, uint32_t *out);

/* Serial binary-heap Dijkstra with the reference's SSSP conventions
 * (SSSP/oneGraph/GraphMeta.h:376-381): dist(src) = 1, unreached = 0xFFFFFFFF.
 * edges = V-indexed pairs {dst, w} (globals.h:18-21 EdgeWithWeight). */
void ora_sssp_dijkstra(uint32_t V, const uint64_t *off, const uint32_t *edges,
                       uint32_t src, uint32_t *out);

/* ora_sssp_dijkstra stopped after `max_edges` edge relaxations (0 = no limit);
 * returns the number of edges scanned (used to time a bounded sample of a
 * query that is too large to finish on one core in seconds). */
uint64_t ora_sssp_dijkstra_bounded(uint32_t V, const uint64_t *off,
                                   const uint32_t *edges, uint32_t src,
                                   uint64_t max_edges, uint32_t *out);

/* SSSP/usm/sssp_usm.cpp:192-236: frontier label-correcting relaxation,
 * same conventions.  Returns the number of rounds. */
int ora_sssp_frontier(uint32_t V, const uint64_t *off, const uint32_t *edges,
                      uint32_t src, uint32_t *out);

/* PR/cpu/pr.cpp:112-165 (pr_init + pr_cal<double>): init 1/V, Jacobi pull,
 * value = 0.15 + 0.15*sum (the reference's own constant), a vertex stops after
 * the round whose |delta| < 0.001.  Returns the number of rounds. */
int ora_pr_cpu(uint32_t V, const uint64_t *off, const uint32_t *col,
               const uint32_t *outdeg, double *out);

/* PR/OneGraph semantics (GraphMeta.h:354-357 init 1.0; gpu_kernels.h:135-158
 * pull sum; gpu_kernels.h:295-319 prKernel_Opt): value = 0.15 + 0.85*sum; a
 * vertex stays active and takes the new value iff |new-old| > thresh, otherwise
 * it goes inactive keeping the old value.  Returns the number of rounds. */
int ora_pr_onegraph(uint32_t V, const uint64_t *off, const uint32_t *col,
                    const uint32_t *outdeg, double thresh, int max_rounds,
                    double *out);

/* FP64 precision oracle: the pull formula of PR/usm/pr.cpp:149-187
 * (pr_cal_cpu, dangling vertices contribute nothing) on the normalised scale
 * p = r/V: p' = (1-d)/V + d*sum(p[u]/outdeg[u]), all vertices every iteration,
 * stop when sum|p'-p| < tol or after max_iter iterations.  Returns the number
 * of iterations; *final_l1 receives the last L1 delta. */
int ora_pr_l1(uint32_t V, const uint64_t *off, const uint32_t *col,
              const uint32_t *outdeg, double damping, double tol, int max_iter,
              double *out, double *final_l1);

/* ora_pr_l1 on `threads` host threads (vertex ranges; the L1 partials are
 * added in thread order, so the result does not depend on scheduling). */
int ora_pr_l1_mt(uint32_t V, const uint64_t *off, const uint32_t *col,
                 const uint32_t *outdeg, double damping, double tol, int max_iter,
                 int threads, double *out, double *final_l1);

/* Shortest-path certificate of a BFS depth or SSSP distance array on a graph
 * whose edge set is symmetric with sorted lists (the symmetric R-MAT graphs):
 * dist[src] == 1; no edge (u, v, w) out of a reached u can lower dist[v]
 * (dist[v] <= dist[u] + w); every reached v != src has an in-edge (u, v, w)
 * with dist[u] + w == dist[v], the in-edge's weight found by binary search of
 * v in u's list.  With weights >= 1 these prove that dist holds the exact
 * shortest distances (a tight in-edge chain strictly decreases to the
 * source).  edges: V-indexed u32 entries, `stride` per edge (1 columns, 2
 * {dst, w} pairs); unit != 0 takes every weight as 1 (BFS depths).  Vertices
 * with dist == unreached are unreached.  Runs on `threads` host threads;
 * returns the number of violations (0: certified) and the first violating
 * vertex in *first_bad (V if none).  Not a restatement of reference code: a
 * size-independent check for inputs too large to run the oracle on. */
uint64_t ora_path_certify(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                          int unit, const uint32_t *dist, uint32_t src, uint32_t unreached,
                          int threads, uint32_t *first_bad);

/* Components of a symmetric graph by union-find on `threads` host threads:
 * every edge (u, v) links the roots of u and v, the larger root under the
 * smaller (compare-and-swap, retried on contention), so every root is the
 * smallest id of its component; out[v] = root of v.  On a symmetric graph
 * this is the reference's CC label (the minimum vertex id that reaches v,
 * CC/serial/serial.cpp:154-213), found without its rounds.  stride as in
 * ora_path_certify.  Returns the number of components. */
uint64_t ora_cc_uf_mt(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                      int threads, uint32_t *out);

/* Bounded timing samples for the CPU baselines (0 = no bound): runCPUBFS
 * (BFS/cpu_BFS/main.cpp:114-209) and one pull iteration of pr_cal
 * (PR/cpu/pr.cpp:126-165) on a symmetric graph, over `stride`-spaced
 * columns; both return the edges scanned. */
uint64_t ora_bfs_bounded(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                         uint32_t src, uint64_t max_edges, uint32_t *out);
uint64_t ora_pr_pull_bounded(uint32_t V, const uint64_t *off, const uint32_t *edges, uint32_t stride,
                             uint64_t max_edges, double *out);

/* A seeded R-MAT graph in CSR (og_oracle_rmat.c): off has V+1 entries,
 * edges E u32 columns or E {dst, w} pairs (weighted), outdeg V entries for a
 * PageRank graph (else NULL).  Free with ora_graph_free. */
typedef struct ora_graph {
  uint32_t V;
  int weighted;
  uint64_t E;
  uint64_t *off;
  uint32_t *edges;
  uint32_t *outdeg;
} ora_graph;

#define ORA_RMAT_SYMMETRIC 1u
#define ORA_RMAT_PERMUTE 2u
#define ORA_RMAT_WEIGHTED 4u
#define ORA_RMAT_PR 8u

/* Returns 0, -1 for bad parameters, -2 when memory ran out. */
int ora_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
             uint64_t weight_seed, uint32_t wmin, uint32_t wmax, uint32_t flags, int threads,
             ora_graph *out);
void ora_graph_free(ora_graph *g);

#ifdef __cplusplus
}
#endif
#endif
