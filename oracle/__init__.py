"""ctypes binding of the CPU oracle (og_oracle.c) — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, and only as the oracle that results are compared with or as
the timed CPU baseline; libog.so never calls it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None
_P = C.c_void_p


class OraGraph(C.Structure):
    _fields_ = [("V", C.c_uint32), ("weighted", C.c_int), ("E", C.c_uint64),
                ("off", C.POINTER(C.c_uint64)), ("edges", C.POINTER(C.c_uint32)),
                ("outdeg", C.POINTER(C.c_uint32))]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build_oracle()
        L = C.CDLL(path)
        u32, u64 = C.c_uint32, C.c_uint64
        L.ora_bfs.argtypes = [u32, _P, _P, u32, _P]
        L.ora_cc.argtypes = [u32, _P, _P, _P]
        L.ora_sssp_dijkstra.argtypes = [u32, _P, _P, u32, _P]
        L.ora_sssp_dijkstra.restype = None
        L.ora_sssp_frontier.argtypes = [u32, _P, _P, u32, _P]
        L.ora_sssp_dijkstra_bounded.argtypes = [u32, _P, _P, u32, u64, _P]
        L.ora_sssp_dijkstra_bounded.restype = u64
        L.ora_cc_round_bounded.argtypes = [u32, _P, _P, u32, u64, _P]
        L.ora_cc_round_bounded.restype = u64
        L.ora_pr_cpu.argtypes = [u32, _P, _P, _P, _P]
        L.ora_pr_onegraph.argtypes = [u32, _P, _P, _P, C.c_double, C.c_int, _P]
        L.ora_pr_l1.argtypes = [u32, _P, _P, _P, C.c_double, C.c_double, C.c_int, _P,
                                C.POINTER(C.c_double)]
        L.ora_pr_l1_mt.argtypes = [u32, _P, _P, _P, C.c_double, C.c_double, C.c_int, C.c_int, _P,
                                   C.POINTER(C.c_double)]
        L.ora_path_certify.argtypes = [u32, _P, _P, u32, C.c_int, _P, u32, u32, C.c_int, _P]
        L.ora_path_certify.restype = u64
        L.ora_bfs_bounded.argtypes = [u32, _P, _P, u32, u32, u64, _P]
        L.ora_bfs_bounded.restype = u64
        L.ora_pr_pull_bounded.argtypes = [u32, _P, _P, u32, u64, _P]
        L.ora_pr_pull_bounded.restype = u64
        L.ora_cc_uf_mt.argtypes = [u32, _P, _P, u32, C.c_int, _P]
        L.ora_cc_uf_mt.restype = u64
        L.ora_rmat.argtypes = [u32, u32, C.c_double, C.c_double, C.c_double, u64, u64, u32, u32, u32,
                               C.c_int, C.POINTER(OraGraph)]
        L.ora_rmat.restype = C.c_int
        L.ora_graph_free.argtypes = [C.POINTER(OraGraph)]
        L.ora_graph_free.restype = None
        for f in ("ora_bfs", "ora_cc", "ora_sssp_frontier", "ora_pr_cpu", "ora_pr_onegraph",
                  "ora_pr_l1", "ora_pr_l1_mt"):
            getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_P)


def _csr(off, edges):
    off = np.ascontiguousarray(off, dtype=np.uint64)
    edges = np.ascontiguousarray(edges, dtype=np.uint32)
    return off, edges, off.size - 1


def bfs(off, col, src):
    """runCPUBFS restatement: depth(src) = 1, unreached = 0xFFFFFFFF."""
    off, col, V = _csr(off, col)
    out = np.empty(V, np.uint32)
    rounds = lib().ora_bfs(V, _p(off), _p(col), src, _p(out))
    return out, rounds


def cc(off, col):
    off, col, V = _csr(off, col)
    out = np.empty(V, np.uint32)
    rounds = lib().ora_cc(V, _p(off), _p(col), _p(out))
    return out, rounds


def cc_round_bounded_raw(V, off_ptr, edges_ptr, stride, max_edges, out):
    """Pointer form of the first label-propagation round of cc(), stopped after
    max_edges edges (stride 2 reads {column, weight} pairs); returns edges scanned."""
    return lib().ora_cc_round_bounded(V, off_ptr, edges_ptr, stride, max_edges, _p(out))


def sssp_dijkstra(off, pairs, src):
    off, pairs, V = _csr(off, pairs)
    out = np.empty(V, np.uint32)
    lib().ora_sssp_dijkstra(V, _p(off), _p(pairs), src, _p(out))
    return out


def sssp_dijkstra_bounded_raw(V, off_ptr, pairs_ptr, src, max_edges, out):
    """Pointer form (no copies) for timing on large graphs; returns edges scanned."""
    return int(lib().ora_sssp_dijkstra_bounded(V, off_ptr, pairs_ptr, src, max_edges,
                                               out.ctypes.data_as(_P)))


def sssp_frontier(off, pairs, src):
    off, pairs, V = _csr(off, pairs)
    out = np.empty(V, np.uint32)
    rounds = lib().ora_sssp_frontier(V, _p(off), _p(pairs), src, _p(out))
    return out, rounds


def pr_cpu(off, col, outdeg):
    off, col, V = _csr(off, col)
    od = np.ascontiguousarray(outdeg, dtype=np.uint32)
    out = np.empty(V, np.float64)
    rounds = lib().ora_pr_cpu(V, _p(off), _p(col), _p(od), _p(out))
    return out, rounds


def pr_onegraph(off, col, outdeg, thresh=0.001, max_rounds=1 << 30):
    off, col, V = _csr(off, col)
    od = np.ascontiguousarray(outdeg, dtype=np.uint32)
    out = np.empty(V, np.float64)
    rounds = lib().ora_pr_onegraph(V, _p(off), _p(col), _p(od), thresh, max_rounds, _p(out))
    return out, rounds


def pr_l1(off, col, outdeg, damping=0.85, tol=1e-6, max_iter=1000):
    off, col, V = _csr(off, col)
    od = np.ascontiguousarray(outdeg, dtype=np.uint32)
    out = np.empty(V, np.float64)
    l1 = C.c_double()
    it = lib().ora_pr_l1(V, _p(off), _p(col), _p(od), damping, tol, max_iter, _p(out), C.byref(l1))
    return out, it, l1.value


def pr_l1_mt_raw(V, off_ptr, col_ptr, outdeg_ptr, damping, tol, max_iter, threads, out):
    """Pointer form of the multi-threaded FP64 oracle (no copies of large graphs)."""
    l1 = C.c_double()
    it = lib().ora_pr_l1_mt(V, off_ptr, col_ptr, outdeg_ptr, damping, tol, max_iter, threads,
                            out.ctypes.data_as(_P), C.byref(l1))
    return it, l1.value


def normalise_bfs(depth, V):
    """Maps OneGraph's unreached value V+1 (GraphMeta.h:378) to cpu_BFS's
    0xFFFFFFFF (BFS/cpu_BFS/main.cpp:141)."""
    d = np.array(depth, dtype=np.uint32, copy=True)
    d[d == np.uint32(V + 1)] = np.uint32(0xFFFFFFFF)
    return d


def path_certify_raw(V, off_ptr, edges_ptr, stride, unit, dist, src, unreached, threads):
    """Shortest-path certificate (ora_path_certify) on a graph given by
    pointers (no copies of large graphs).  Returns (violations, first bad
    vertex or V)."""
    fb = C.c_uint32()
    d = np.ascontiguousarray(dist, dtype=np.uint32)
    bad = lib().ora_path_certify(V, off_ptr, edges_ptr, stride, 1 if unit else 0, _p(d), src, unreached,
                                 threads, C.byref(fb))
    return int(bad), int(fb.value)


def bfs_bounded_raw(V, off_ptr, edges_ptr, stride, src, max_edges, out):
    """runCPUBFS restatement on pointers, stopped after max_edges edges
    (0: complete); returns the edges scanned."""
    return int(lib().ora_bfs_bounded(V, off_ptr, edges_ptr, stride, src, max_edges, out.ctypes.data_as(_P)))


def pr_pull_bounded_raw(V, off_ptr, edges_ptr, stride, max_edges, out):
    """One pr_cal pull iteration on a symmetric graph given by pointers,
    stopped after max_edges edges; returns the edges read."""
    return int(lib().ora_pr_pull_bounded(V, off_ptr, edges_ptr, stride, max_edges, out.ctypes.data_as(_P)))


def cc_uf_mt_raw(V, off_ptr, edges_ptr, stride, threads, out):
    """Union-find components of a symmetric graph given by pointers (no
    copies): out[v] = smallest id of v's component.  Returns the count."""
    return int(lib().ora_cc_uf_mt(V, off_ptr, edges_ptr, stride, threads, out.ctypes.data_as(_P)))


RMAT_SYMMETRIC, RMAT_PERMUTE, RMAT_WEIGHTED, RMAT_PR = 1, 2, 4, 8


class RmatGraph:
    """A seeded R-MAT graph built on the CPU by the oracle (og_oracle_rmat.c):
    .V, .E, .offsets (V+1 u64), .edges (E u32 columns or (E, 2) {dst, w}
    pairs), .outdeg (PageRank graphs) as views of C-owned arrays, and the raw
    pointers off_p / edges_p for the pointer-form oracle calls."""

    def __init__(self, scale, edge_factor=16, seed=1, weight_seed=2, weighted=False, symmetric=True,
                 permute=True, pagerank=False, wmin=1, wmax=64, abc=(0.57, 0.19, 0.19), threads=0):
        self._g = OraGraph()
        flags = ((RMAT_SYMMETRIC if symmetric else 0) | (RMAT_PERMUTE if permute else 0) |
                 (RMAT_WEIGHTED if weighted else 0) | (RMAT_PR if pagerank else 0))
        nt = threads or (os.cpu_count() or 1)
        rc = lib().ora_rmat(scale, edge_factor, abc[0], abc[1], abc[2], seed, weight_seed, wmin, wmax,
                            flags, nt, C.byref(self._g))
        if rc != 0:
            raise MemoryError("ora_rmat failed (%d)" % rc)
        g = self._g
        self.V, self.E, self.weighted = g.V, g.E, bool(g.weighted)
        self.off_p = C.cast(g.off, _P)
        self.edges_p = C.cast(g.edges, _P)
        self.offsets = np.ctypeslib.as_array(g.off, (self.V + 1,))
        n = self.E * (2 if self.weighted else 1)
        self.edges = np.ctypeslib.as_array(g.edges, (max(n, 1),))[:n]
        if self.weighted:
            self.edges = self.edges.reshape(-1, 2)
        self.outdeg = np.ctypeslib.as_array(g.outdeg, (self.V,)) if g.outdeg else None

    def degrees(self):
        return np.diff(self.offsets).astype(np.uint32)

    def close(self):
        if self._g is not None and self._g.off:
            lib().ora_graph_free(C.byref(self._g))
        self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
