"""Python mirror of the GB300 OneGraph engine's C ABI (include/onegraph.h).

The compute path is libog.so (hand-written sm_103a CUDA + C++ host code); this
module only binds it with ctypes and mirrors the reference's driver entry
points (``bfs_opt`` / ``sssp_opt`` / ``cc_opt`` / ``pr_opt``,
BFS/oneGraph_BFS/CalculateOpt.h:9, SSSP/oneGraph/CalculateOpt.h:12,
CC/onegraph/CalculateOpt.h:6, PR/OneGraph/CalculateOpt.h:13).  There is no
fallback: if libog.so is missing, importing the library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libog.so")
BIN_DIR = os.path.join(_PKG, "bin")

OG_OK = 0
STATUS = {0: "OG_OK", 1: "OG_E_ARG", 2: "OG_E_IO", 3: "OG_E_FORMAT", 4: "OG_E_BUDGET",
          5: "OG_E_CUDA", 6: "OG_E_TIMEOUT", 7: "OG_E_NOMEM", 8: "OG_E_STATE",
          9: "OG_E_UNSUPPORTED", 10: "OG_E_DEVICE"}
PLAIN, WEIGHTED, PR = 0, 1, 2
ALGO_BFS, ALGO_SSSP, ALGO_CC, ALGO_PR = 0, 1, 2, 3
RMAT_SYMMETRIC, RMAT_PERMUTE, RMAT_WEIGHTED, RMAT_PR, RMAT_ON_GPU = 1, 2, 4, 8, 16
CFG_DIRECT, CFG_NO_PIN, CFG_PR, CFG_BATCH, CFG_BATCH_LEVELS, CFG_NO_STATIC = 1, 2, 4, 8, 16, 32
CFG_REPLACE = 64  # fragment slots: Ascetic's static-region replacement


def CFG_SSSP_BATCH(k: int) -> int:
    """OG_CFG_SSSP_BATCH(k): hold og_sssp_batch state for up to k (1..32) sources."""
    return (int(k) & 63) << 8


PARAM_SSSP_DELTA = 1
PARAM_CC_METHOD = 2
CC_AUTO, CC_LABEL_PROPAGATION, CC_UNION_FIND = 0, 1, 2
PARAM_BFS_DIRECTION = 3
BFS_AUTO, BFS_TOP_DOWN = 0, 1
PARAM_LEVEL_LOOP = 4
LOOP_AUTO, LOOP_HOST = 0, 1
PARAM_RELAX_TIMER = 5
PARAM_SSSP_BATCH_DELTA = 6
PARAM_FRAGMENT_WORDS = 7
SERVER_BFS_JOIN = 1  # og_server_config.flags: BFS requests join level-by-level passes in flight
# R-MAT quadrant probabilities of the benchmark graphs
RMAT_ABC = (0.57, 0.19, 0.19)


class OGError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__("%s: %s (%s)" % (where, msg, STATUS.get(status, status)))
        self.status = status


class RmatParams(C.Structure):
    _fields_ = [("scale", C.c_uint32), ("edge_factor", C.c_uint32), ("a", C.c_double),
                ("b", C.c_double), ("c", C.c_double), ("seed", C.c_uint64),
                ("weight_seed", C.c_uint64), ("wmin", C.c_uint32), ("wmax", C.c_uint32),
                ("flags", C.c_uint32), ("threads", C.c_uint32)]


class Plan(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("vertex_bytes", C.c_uint64),
                ("fixed_bytes", C.c_uint64), ("edge_capacity", C.c_uint64),
                ("advisek", C.c_double), ("advisek_auto", C.c_double),
                ("max_partition", C.c_uint64), ("static_vertices", C.c_uint32),
                ("static_edges", C.c_uint64), ("dynamic_edges", C.c_uint64),
                ("chunk_edges", C.c_uint64), ("edge_bytes", C.c_uint32), ("edge_bits", C.c_uint32),
                ("stage_edge_bytes", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class TuneResult(C.Structure):
    _fields_ = [("configs", C.c_int), ("best", C.c_int), ("block", C.c_int * 8),
                ("items", C.c_int * 8), ("ms", C.c_float * 8)]

    def as_dict(self):
        n = self.configs
        return {"best": self.best, "candidates": [
            {"block": self.block[i], "items": self.items[i], "ms": self.ms[i]} for i in range(n)]}


class Config(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("advisek", C.c_double), ("flags", C.c_uint32),
                ("device", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("chunks", C.c_uint32), ("frontier_sum", C.c_uint64),
                ("static_vertices", C.c_uint64), ("edges_static", C.c_uint64),
                ("edges_dynamic", C.c_uint64), ("link_bytes", C.c_uint64),
                ("ms_total", C.c_double), ("ms_static", C.c_double), ("ms_dynamic", C.c_double),
                ("ms_compact", C.c_double), ("residual", C.c_double), ("launches", C.c_uint64),
                ("ms_gather", C.c_double), ("ms_relax", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("workers", C.c_int32), ("max_batch", C.c_int32),
                ("device", C.c_int32), ("flags", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("graph", C.c_int32), ("algo", C.c_int32), ("source", C.c_uint32),
                ("iterations", C.c_int32), ("out", C.c_void_p), ("user", C.c_uint64)]


class Response(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("user", C.c_uint64), ("status", C.c_int32),
                ("graph", C.c_int32), ("algo", C.c_int32), ("source", C.c_uint32),
                ("batch", C.c_uint32), ("reserved", C.c_uint32), ("t_submit_ms", C.c_double),
                ("t_start_ms", C.c_double), ("t_done_ms", C.c_double),
                ("checksum", C.c_uint64 * 2)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f not in ("checksum", "reserved")}
        d["checksum"] = (self.checksum[0], self.checksum[1])
        return d


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("gpu_passes", C.c_uint64),
                ("batched_requests", C.c_uint64), ("contexts_created", C.c_uint64),
                ("used_bytes", C.c_uint64), ("launches", C.c_uint64)]


class FragmentStats(C.Structure):
    _fields_ = [("fragments", C.c_uint64), ("slots", C.c_uint32), ("fragment_words", C.c_uint32),
                ("swaps", C.c_uint64), ("swap_bytes", C.c_uint64), ("records_slots", C.c_uint64),
                ("records_host", C.c_uint64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class KRecords(C.Structure):
    """og_k_records (include/onegraph_kernels.h): packed records in device memory."""
    _fields_ = [("words", C.c_void_p), ("nrecords", C.c_uint64), ("bpe", C.c_uint32), ("bc", C.c_uint32),
                ("wmin", C.c_uint32), ("reserved", C.c_uint32)]


_lib = None

# (name, restype, argtypes) for every symbol declared in include/*.h
_P = C.c_void_p
SIGNATURES = [
    ("og_graph_load", C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P)]),
    ("og_graph_from_arrays", C.c_int, [C.c_uint64, C.c_uint64, _P, C.c_int, _P, _P, C.c_int,
                                       C.POINTER(_P)]),
    ("og_graph_save", C.c_int, [_P, C.c_char_p]),
    ("og_graph_info", C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                C.POINTER(C.c_int), C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    ("og_graph_free", None, [_P]),
    ("og_graph_findbignode", C.c_uint32, [_P, C.c_uint32]),
    ("og_graph_save_bel", C.c_int, [_P, C.c_char_p]),
    ("og_convert_uint_to_ulong", C.c_int, [C.c_char_p, C.c_char_p]),
    ("og_graph_transpose", C.c_int, [_P, C.POINTER(_P)]),
    ("og_graph_set_symmetric", C.c_int, [_P, C.c_int]),
    ("og_graph_symmetric", C.c_int, [_P, C.POINTER(C.c_int)]),
    ("og_graph_records", C.c_int, [_P, C.POINTER(_P), C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("og_rmat_generate", C.c_int, [C.POINTER(RmatParams), C.POINTER(_P)]),
    ("og_plan_compute", C.c_int, [C.c_uint64, C.c_uint64, _P, C.c_int, C.c_uint64, C.c_double,
                                  C.c_uint32, C.POINTER(Plan)]),
    ("og_graph_plan", C.c_int, [_P, C.c_uint64, C.c_double, C.c_uint32, C.POINTER(Plan)]),
    ("og_engine_create", C.c_int, [_P, C.POINTER(Config), C.POINTER(_P)]),
    ("og_engine_plan", C.c_int, [_P, C.POINTER(Plan)]),
    ("og_engine_destroy", None, [_P]),
    ("og_bfs", C.c_int, [_P, C.c_uint32, _P, C.POINTER(Stats)]),
    ("og_sssp", C.c_int, [_P, C.c_uint32, _P, C.POINTER(Stats)]),
    ("og_cc", C.c_int, [_P, _P, C.POINTER(Stats)]),
    ("og_pr", C.c_int, [_P, _P, C.c_double, C.c_int, C.POINTER(Stats)]),
    ("og_pr_l1", C.c_int, [_P, _P, C.c_double, C.c_double, C.c_int, C.POINTER(Stats)]),
    ("og_pr_l1_push", C.c_int, [_P, _P, C.c_double, C.c_double, C.c_int, C.POINTER(Stats)]),
    ("og_bfs_batch", C.c_int, [_P, _P, C.c_int, _P, _P, C.POINTER(Stats)]),
    ("og_sssp_batch", C.c_int, [_P, _P, C.c_int, _P, _P, C.POINTER(Stats)]),
    ("og_sssp_batch_begin", C.c_int, [_P]),
    ("og_sssp_batch_join", C.c_int, [_P, _P, _P, C.c_int]),
    ("og_sssp_batch_step", C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_int), C.POINTER(Stats)]),
    ("og_sssp_batch_checks", C.c_int, [_P, C.c_uint32, _P]),
    ("og_sssp_batch_fetch", C.c_int, [_P, C.c_uint32, _P]),
    ("og_bfs_batch_begin", C.c_int, [_P, C.c_int]),
    ("og_bfs_batch_join", C.c_int, [_P, _P, _P, C.c_int]),
    ("og_bfs_batch_step", C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_int), C.POINTER(Stats)]),
    ("og_bfs_batch_checks", C.c_int, [_P, C.c_uint64, _P]),
    ("og_bfs_batch_fetch", C.c_int, [_P, C.c_uint32, _P]),
    ("og_bfs_batch_to", C.c_int, [_P, _P, C.c_int, _P, _P, C.POINTER(Stats)]),
    ("og_bfs_batch_u8", C.c_int, [_P, _P, C.c_int, _P, C.POINTER(C.c_uint64), _P, C.POINTER(Stats)]),
    ("og_host_alloc", C.c_int, [C.c_uint64, C.POINTER(_P)]),
    ("og_host_free", None, [_P]),
    ("og_bfs_batch_tune", C.c_int, [_P, _P, C.c_int, C.c_int, C.POINTER(TuneResult)]),
    ("og_bfs_batch_set_config", C.c_int, [_P, C.c_int]),
    ("og_result_fetch", C.c_int, [_P, C.c_int, _P]),
    ("og_result_checksum", C.c_int, [_P, C.c_int, _P]),
    ("og_engine_clone", C.c_int, [_P, C.POINTER(_P)]),
    ("og_engine_bytes", C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("og_engine_set_param", C.c_int, [_P, C.c_int, C.c_double]),
    ("og_engine_get_param", C.c_int, [_P, C.c_int, C.POINTER(C.c_double)]),
    ("og_engine_fragment_stats", C.c_int, [_P, C.POINTER(FragmentStats)]),
    ("og_k_compact", C.c_int, [_P, C.c_uint32, C.c_uint32, _P, _P, _P, C.c_uint64, _P,
                               C.c_uint64, _P, _P]),
    ("og_k_compact_noalloc", C.c_int, [_P, C.c_uint32, C.c_uint32, _P, _P, _P, C.c_uint64, _P,
                                       C.c_uint64, _P, _P]),
    ("og_k_relax", C.c_int, [C.c_int, _P, _P, _P, C.c_uint32, C.c_uint64, _P, C.POINTER(KRecords), C.c_uint32,
                             _P, _P, _P, C.c_uint32, _P]),
    ("og_k_gather", C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint64, _P, C.POINTER(KRecords), C.c_uint64,
                              C.c_uint64, _P, _P, _P]),
    ("og_k_wait_check", C.c_int, [C.c_int, C.c_uint32]),
    ("og_link_probe", C.c_int, [_P, C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    ("og_server_create", C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    ("og_server_add_graph", C.c_int, [_P, _P, C.POINTER(Config), C.POINTER(C.c_int)]),
    ("og_server_submit", C.c_int, [_P, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    ("og_server_poll", C.c_int, [_P, C.POINTER(Response), C.c_int, C.POINTER(C.c_int), C.c_int]),
    ("og_server_drain", C.c_int, [_P, C.c_int]),
    ("og_server_get_stats", C.c_int, [_P, C.POINTER(ServerStats)]),
    ("og_server_destroy", None, [_P]),
    ("og_last_error", C.c_char_p, []),
    ("og_abi_version", C.c_int, []),
]


ABI_VERSION = 6  # OG_ABI_VERSION of include/onegraph.h these bindings follow


def lib():
    """Loads libog.so (built by onegraph_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libog.so not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if L.og_abi_version() != ABI_VERSION:
            raise OSError("libog.so ABI %d, bindings expect %d: rebuild" % (L.og_abi_version(), ABI_VERSION))
        _lib = L
    return _lib


def _check(rc: int, where: str):
    if rc != OG_OK:
        raise OGError(rc, where, lib().og_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Graph:
    """Host CSR in the reference layout (GraphMeta.h:126-145) owned by libog."""

    def __init__(self, handle):
        self._h = handle
        self._engines = 0          # live engines on this graph
        self._free_pending = False  # close() asked for while engines were alive
        V, E, kind = C.c_uint64(), C.c_uint64(), C.c_int()
        off, edges, outdeg = _P(), _P(), _P()
        _check(lib().og_graph_info(handle, C.byref(V), C.byref(E), C.byref(kind), C.byref(off),
                                   C.byref(edges), C.byref(outdeg)), "og_graph_info")
        self.V, self.E, self.kind = V.value, E.value, kind.value
        self._off_p, self._edges_p, self._outdeg_p = off.value, edges.value, outdeg.value

    @classmethod
    def load(cls, path: str, kind: int = PLAIN) -> "Graph":
        h = _P()
        _check(lib().og_graph_load(path.encode(), kind, C.byref(h)), "og_graph_load")
        return cls(h)

    @classmethod
    def from_arrays(cls, offsets, edges, outdeg=None, kind: int = PLAIN,
                    with_sentinel: bool = True) -> "Graph":
        """offsets: V+1 entries (with_sentinel) or the file's V entries."""
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        ed = np.ascontiguousarray(edges, dtype=np.uint32)
        od = None if outdeg is None else np.ascontiguousarray(outdeg, dtype=np.uint32)
        E = ed.size // (2 if kind == WEIGHTED else 1)
        V = off.size - (1 if with_sentinel else 0)
        h = _P()
        _check(lib().og_graph_from_arrays(V, E, _ptr(off), 1 if with_sentinel else 0,
                                          _ptr(ed) if E else None, _ptr(od), kind, C.byref(h)),
               "og_graph_from_arrays")
        return cls(h)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, seed: int = 1, weight_seed: int = 2,
             symmetric: bool = True, permute: bool = True, weighted: bool = False,
             pagerank: bool = False, on_gpu: bool = False, wmin: int = 1, wmax: int = 64,
             abc=RMAT_ABC, threads: int = 0) -> "Graph":
        flags = ((RMAT_SYMMETRIC if symmetric else 0) | (RMAT_PERMUTE if permute else 0) |
                 (RMAT_WEIGHTED if weighted else 0) | (RMAT_PR if pagerank else 0) |
                 (RMAT_ON_GPU if on_gpu else 0))
        p = RmatParams(scale, edge_factor, abc[0], abc[1], abc[2], seed, weight_seed, wmin, wmax,
                       flags, threads)
        h = _P()
        _check(lib().og_rmat_generate(C.byref(p), C.byref(h)), "og_rmat_generate")
        return cls(h)

    def save(self, path: str):
        _check(lib().og_graph_save(self._h, path.encode()), "og_graph_save")

    def save_bel(self, prefix: str):
        _check(lib().og_graph_save_bel(self._h, prefix.encode()), "og_graph_save_bel")

    def transpose(self) -> "Graph":
        """The reverse graph (PLAIN): the out-edge CSR of an in-edge PageRank graph."""
        h = _P()
        _check(lib().og_graph_transpose(self._h, C.byref(h)), "og_graph_transpose")
        return Graph(h)

    @property
    def offsets(self) -> np.ndarray:
        """V+1 offsets (borrowed view, valid while the graph lives)."""
        return np.ctypeslib.as_array(C.cast(self._off_p, C.POINTER(C.c_uint64)), (self.V + 1,))

    @property
    def edges(self) -> np.ndarray:
        """u32 columns, or an (E, 2) array of {dst, weight} for weighted graphs."""
        n = self.E * (2 if self.kind == WEIGHTED else 1)
        if n == 0:
            return np.zeros((0, 2) if self.kind == WEIGHTED else 0, np.uint32)
        a = np.ctypeslib.as_array(C.cast(self._edges_p, C.POINTER(C.c_uint32)), (n,))
        return a.reshape(-1, 2) if self.kind == WEIGHTED else a

    @property
    def columns(self) -> np.ndarray:
        e = self.edges
        return e[:, 0] if self.kind == WEIGHTED else e

    @property
    def outdeg(self) -> np.ndarray | None:
        if not self._outdeg_p:
            return None
        return np.ctypeslib.as_array(C.cast(self._outdeg_p, C.POINTER(C.c_uint32)), (self.V,))

    def degrees(self) -> np.ndarray:
        return np.diff(self.offsets).astype(np.uint32)

    def plan(self, budget: int = 0, advisek: float = 0.0, flags: int = 0) -> dict:
        """The engine's plan for this graph (with its real per-edge bytes)."""
        p = Plan()
        _check(lib().og_graph_plan(self._h, budget, advisek, flags, C.byref(p)), "og_graph_plan")
        return p.as_dict()

    def set_symmetric(self, symmetric: bool):
        """Asserts (without checking) whether every edge has its reverse."""
        _check(lib().og_graph_set_symmetric(self._h, 1 if symmetric else 0), "og_graph_set_symmetric")

    def symmetric(self) -> bool:
        """Whether every edge has its reverse (exact check on first use)."""
        v = C.c_int()
        _check(lib().og_graph_symmetric(self._h, C.byref(v)), "og_graph_symmetric")
        return bool(v.value)

    def records(self) -> dict:
        """The packed edge records the engines read: words (borrowed view),
        bits per record, column bits and the weight offset."""
        w, n, bpe, bc, wmin = _P(), C.c_uint64(), C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(lib().og_graph_records(self._h, C.byref(w), C.byref(n), C.byref(bpe), C.byref(bc),
                                      C.byref(wmin)), "og_graph_records")
        words = np.ctypeslib.as_array(C.cast(w, C.POINTER(C.c_uint32)), (n.value,))
        return {"words": words, "bpe": bpe.value, "bc": bc.value, "wmin": wmin.value}

    def findbignode(self, last: int) -> int:
        return int(lib().og_graph_findbignode(self._h, last))

    def close(self):
        """Frees the host CSR; deferred until the last engine on it is closed
        (an engine page-locks and reads the graph's arrays).  Finalisers of a
        garbage cycle run in no fixed order, so this ordering is enforced here."""
        if not self._h:
            return
        if self._engines > 0:
            self._free_pending = True
            return
        lib().og_graph_free(self._h)
        self._h = None

    def _engine_closed(self):
        self._engines -= 1
        if self._engines == 0 and self._free_pending:
            self._free_pending = False
            self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def convert_uint_to_ulong(in_path: str, out_path: str | None = None):
    """GraphMeta::transFileUintToUlong: 32-bit-header CSR -> 64-bit edge entries."""
    _check(lib().og_convert_uint_to_ulong(in_path.encode(), out_path.encode() if out_path else None),
           "og_convert_uint_to_ulong")


def plan(V: int, E: int, offsets: np.ndarray, kind: int = PLAIN, budget: int = 0,
         advisek: float = 0.0, flags: int = 0) -> dict:
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    assert off.size == V + 1
    p = Plan()
    _check(lib().og_plan_compute(V, E, _ptr(off), kind, budget, advisek, flags, C.byref(p)),
           "og_plan_compute")
    return p.as_dict()


class Engine:
    """og_engine: a graph planned against a device budget, static prefix resident."""

    def __init__(self, graph: Graph, budget: int = 0, advisek: float = 0.0, direct: bool = False,
                 pagerank: bool = False, no_pin: bool = False, batch: bool = False,
                 batch_levels: bool = False, no_static: bool = False, sssp_batch: int = 0,
                 replace: bool = False, device: int = 0):
        self.graph = graph
        cfg = Config(budget, advisek, (CFG_DIRECT if direct else 0) | (CFG_PR if pagerank else 0) |
                     (CFG_NO_PIN if no_pin else 0) | (CFG_BATCH if batch or batch_levels else 0) |
                     (CFG_BATCH_LEVELS if batch_levels else 0) |
                     (CFG_NO_STATIC if no_static else 0) | CFG_SSSP_BATCH(sssp_batch) |
                     (CFG_REPLACE if replace else 0), device)
        h = _P()
        _check(lib().og_engine_create(graph._h, C.byref(cfg), C.byref(h)), "og_engine_create")
        self._h = h
        graph._engines += 1
        p = Plan()
        _check(lib().og_engine_plan(h, C.byref(p)), "og_engine_plan")
        self.plan = p.as_dict()
        self.stats: dict = {}

    def fragment_stats(self) -> dict:
        """og_engine_fragment_stats of an engine created with replace=True."""
        fs = FragmentStats()
        _check(lib().og_engine_fragment_stats(self._h, C.byref(fs)), "og_engine_fragment_stats")
        return fs.as_dict()

    def _out(self, out, dtype):
        if out is False:
            return None
        if out is None:
            return np.empty(self.graph.V, dtype)
        assert out.dtype == dtype and out.size >= self.graph.V and out.flags.c_contiguous
        return out

    def bfs(self, src: int, out=None) -> np.ndarray | None:
        """Depths, depth(src) = 1, unreached = V+1.  out=False keeps them on the device."""
        o = self._out(out, np.uint32)
        st = Stats()
        _check(lib().og_bfs(self._h, src, _ptr(o), C.byref(st)), "og_bfs")
        self.stats = st.as_dict()
        return o

    def sssp(self, src: int, out=None) -> np.ndarray | None:
        o = self._out(out, np.uint32)
        st = Stats()
        _check(lib().og_sssp(self._h, src, _ptr(o), C.byref(st)), "og_sssp")
        self.stats = st.as_dict()
        return o

    def cc(self, out=None) -> np.ndarray | None:
        o = self._out(out, np.uint32)
        st = Stats()
        _check(lib().og_cc(self._h, _ptr(o), C.byref(st)), "og_cc")
        self.stats = st.as_dict()
        return o

    def pr(self, threshold: float = 0.001, max_rounds: int = 0, out=None) -> np.ndarray | None:
        o = self._out(out, np.float32)
        st = Stats()
        _check(lib().og_pr(self._h, _ptr(o), threshold, max_rounds, C.byref(st)), "og_pr")
        self.stats = st.as_dict()
        return o

    def pr_l1(self, damping: float = 0.85, tol: float = 1e-6, max_iter: int = 200,
              out=None) -> np.ndarray | None:
        o = self._out(out, np.float32)
        st = Stats()
        _check(lib().og_pr_l1(self._h, _ptr(o), damping, tol, max_iter, C.byref(st)), "og_pr_l1")
        self.stats = st.as_dict()
        return o

    def pr_l1_push(self, damping: float = 0.85, tol: float = 1e-6, max_iter: int = 200,
                   out=None) -> np.ndarray | None:
        """pr_l1 by push; the engine's graph must hold out-edges (Graph.transpose)."""
        o = self._out(out, np.float32)
        st = Stats()
        _check(lib().og_pr_l1_push(self._h, _ptr(o), damping, tol, max_iter, C.byref(st)),
               "og_pr_l1_push")
        self.stats = st.as_dict()
        return o

    def bfs_batch(self, srcs, out=None, checks: bool = True):
        """Up to 64 BFS sources in one pass.  Returns (depths n x V or None,
        checks n x 2 {reached, depth sum} or None); out=False skips the depths."""
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        n = s.size
        o = None if out is False else (np.empty((n, self.graph.V), np.uint32) if out is None else out)
        ck = np.empty((n, 2), np.uint64) if checks else None
        st = Stats()
        _check(lib().og_bfs_batch(self._h, _ptr(s), n, _ptr(o), _ptr(ck), C.byref(st)),
               "og_bfs_batch")
        self.stats = st.as_dict()
        return o, ck

    def bfs_batch_to(self, srcs, outs):
        """og_bfs_batch_to: source i's depths into outs[i] (one V-array each).
        Returns the n x 2 checks."""
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        n = s.size
        assert len(outs) == n
        for o in outs:
            assert o.dtype == np.uint32 and o.size >= self.graph.V and o.flags.c_contiguous
        ptrs = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
        ck = np.empty((n, 2), np.uint64)
        st = Stats()
        _check(lib().og_bfs_batch_to(self._h, _ptr(s), n, C.cast(ptrs, C.c_void_p), _ptr(ck), C.byref(st)),
               "og_bfs_batch_to")
        self.stats = st.as_dict()
        return ck

    def sssp_batch(self, srcs, out=None, checks: bool = True):
        """Up to k SSSP sources (Engine(sssp_batch=k)) in one pass.  Returns
        (distances n x V or None, checks n x 2 {reached, distance sum} or None);
        out=False skips the distances."""
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        n = s.size
        o = None if out is False else (np.empty((n, self.graph.V), np.uint32) if out is None else out)
        ck = np.empty((n, 2), np.uint64) if checks else None
        st = Stats()
        _check(lib().og_sssp_batch(self._h, _ptr(s), n, _ptr(o), _ptr(ck), C.byref(st)),
               "og_sssp_batch")
        self.stats = st.as_dict()
        return o, ck

    # og_sssp_batch round by round (sources may join a pass in flight)
    def sssp_batch_begin(self):
        _check(lib().og_sssp_batch_begin(self._h), "og_sssp_batch_begin")

    def sssp_batch_join(self, srcs, slots):
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        k = np.ascontiguousarray(slots, dtype=np.uint32)
        assert s.size == k.size
        _check(lib().og_sssp_batch_join(self._h, _ptr(s), _ptr(k), s.size), "og_sssp_batch_join")

    def sssp_batch_step(self) -> tuple:
        """One round: (slots still pending as a bit mask, done)."""
        p, d, st = C.c_uint32(), C.c_int(), Stats()
        _check(lib().og_sssp_batch_step(self._h, C.byref(p), C.byref(d), C.byref(st)), "og_sssp_batch_step")
        self.stats = st.as_dict()
        return p.value, bool(d.value)

    def sssp_batch_checks(self, slots: int) -> np.ndarray:
        out = np.zeros((32, 2), np.uint64)
        _check(lib().og_sssp_batch_checks(self._h, slots, _ptr(out)), "og_sssp_batch_checks")
        return out

    def sssp_batch_fetch(self, slot: int) -> np.ndarray:
        o = np.empty(self.graph.V, np.uint32)
        _check(lib().og_sssp_batch_fetch(self._h, slot, _ptr(o)), "og_sssp_batch_fetch")
        return o

    # og_bfs_batch level by level (sources may join a batch in flight)
    def bfs_batch_begin(self, record_depths: bool = False):
        _check(lib().og_bfs_batch_begin(self._h, 1 if record_depths else 0), "og_bfs_batch_begin")

    def bfs_batch_join(self, srcs, slots):
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        k = np.ascontiguousarray(slots, dtype=np.uint32)
        assert s.size == k.size
        _check(lib().og_bfs_batch_join(self._h, _ptr(s), _ptr(k), s.size), "og_bfs_batch_join")

    def bfs_batch_step(self) -> tuple:
        """One level: (slots still in flight as a 64-bit mask, done)."""
        p, d, st = C.c_uint64(), C.c_int(), Stats()
        _check(lib().og_bfs_batch_step(self._h, C.byref(p), C.byref(d), C.byref(st)), "og_bfs_batch_step")
        self.stats = st.as_dict()
        return p.value, bool(d.value)

    def bfs_batch_checks(self, slots: int) -> np.ndarray:
        out = np.zeros((64, 2), np.uint64)
        _check(lib().og_bfs_batch_checks(self._h, C.c_uint64(slots), _ptr(out)), "og_bfs_batch_checks")
        return out

    def bfs_batch_fetch(self, slot: int) -> np.ndarray:
        o = np.empty(self.graph.V, np.uint32)
        _check(lib().og_bfs_batch_fetch(self._h, slot, _ptr(o)), "og_bfs_batch_fetch")
        return o

    def bfs_batch_u8(self, srcs, out=None, checks: bool = True):
        """og_bfs_batch_u8: byte depths (0 unreached, 255 for depth >= 255).
        Returns (depths n x V u8, clamped entries, checks or None)."""
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        n = s.size
        o = np.empty((n, self.graph.V), np.uint8) if out is None else out
        assert o.dtype == np.uint8 and o.size >= n * self.graph.V and o.flags.c_contiguous
        ck = np.empty((n, 2), np.uint64) if checks else None
        cl = C.c_uint64()
        st = Stats()
        _check(lib().og_bfs_batch_u8(self._h, _ptr(s), n, _ptr(o), C.byref(cl), _ptr(ck), C.byref(st)),
               "og_bfs_batch_u8")
        self.stats = st.as_dict()
        return o, cl.value, ck

    def bfs_batch_tune(self, srcs, reps: int = 2) -> dict:
        s = np.ascontiguousarray(srcs, dtype=np.uint32)
        r = TuneResult()
        _check(lib().og_bfs_batch_tune(self._h, _ptr(s), s.size, reps, C.byref(r)),
               "og_bfs_batch_tune")
        return r.as_dict()

    def bfs_batch_set_config(self, config: int):
        _check(lib().og_bfs_batch_set_config(self._h, config), "og_bfs_batch_set_config")

    def clone(self) -> "Engine":
        """A query context sharing this engine's resident graph (og_engine_clone)."""
        c = Engine.__new__(Engine)
        h = _P()
        _check(lib().og_engine_clone(self._h, C.byref(h)), "og_engine_clone")
        c._h, c.graph, c.plan, c.stats, c._parent = h, self.graph, self.plan, {}, self
        c._clones, c._close_pending = 0, False
        self.graph._engines += 1
        self._clones = getattr(self, "_clones", 0) + 1
        return c

    def set_param(self, param: int, value: float):
        _check(lib().og_engine_set_param(self._h, param, value), "og_engine_set_param")

    def get_param(self, param: int) -> float:
        v = C.c_double()
        _check(lib().og_engine_get_param(self._h, param, C.byref(v)), "og_engine_get_param")
        return v.value

    def bytes(self) -> tuple:
        """(device bytes of the resident graph, of one query context)."""
        r, c = C.c_uint64(), C.c_uint64()
        _check(lib().og_engine_bytes(self._h, C.byref(r), C.byref(c)), "og_engine_bytes")
        return r.value, c.value

    def checksum(self, algo: int) -> tuple:
        out = np.zeros(2, np.uint64)
        _check(lib().og_result_checksum(self._h, algo, _ptr(out)), "og_result_checksum")
        return int(out[0]), int(out[1])

    def fetch(self, algo: int, dtype=np.uint32) -> np.ndarray:
        o = np.empty(self.graph.V, dtype)
        _check(lib().og_result_fetch(self._h, algo, _ptr(o)), "og_result_fetch")
        return o

    def close(self):
        """Destroys the engine; a parent waits for its clones (they share its
        resident graph), whatever order finalisers run in."""
        if not getattr(self, "_h", None):
            return
        if getattr(self, "_clones", 0) > 0:
            self._close_pending = True
            return
        lib().og_engine_destroy(self._h)
        self._h = None
        self.graph._engine_closed()
        parent = getattr(self, "_parent", None)
        if parent is not None:
            parent._clones -= 1
            if parent._clones == 0 and getattr(parent, "_close_pending", False):
                parent._close_pending = False
                parent.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """og_server: resident graphs, pooled query contexts, continuous batching."""

    def __init__(self, budget: int = 0, workers: int = 4, max_batch: int = 64, device: int = 0,
                 bfs_join: bool = False):
        cfg = ServerConfig(budget, workers, max_batch, device, SERVER_BFS_JOIN if bfs_join else 0)
        h = _P()
        _check(lib().og_server_create(C.byref(cfg), C.byref(h)), "og_server_create")
        self._h = h
        self.graphs: list[Graph] = []
        self._bufs: dict[int, np.ndarray] = {}

    def add_graph(self, graph: Graph, budget: int = 0, advisek: float = 0.0, direct: bool = True,
                  pagerank: bool = False, sssp_batch: int = 0) -> int:
        """sssp_batch = k > 1 serves the graph's SSSP requests in multi-source
        passes of up to k sources that requests join and leave while they run."""
        cfg = Config(budget, advisek, (CFG_DIRECT if direct else 0) | (CFG_PR if pagerank else 0) |
                     CFG_SSSP_BATCH(sssp_batch), 0)
        gid = C.c_int()
        _check(lib().og_server_add_graph(self._h, graph._h, C.byref(cfg), C.byref(gid)),
               "og_server_add_graph")
        graph._engines += 1  # the server's engines read the graph until destroy
        self.graphs.append(graph)
        return gid.value

    def submit(self, graph: int, algo: int, source: int = 0, iterations: int = 0, out=None,
               user: int = 0) -> int:
        if out is not None:
            assert out.flags.c_contiguous and out.size >= self.graphs[graph].V
        r = Request(graph, algo, source, iterations, _ptr(out), user)
        t = C.c_uint64()
        _check(lib().og_server_submit(self._h, C.byref(r), C.byref(t)), "og_server_submit")
        if out is not None:
            self._bufs[t.value] = out  # keep the buffer alive until its response
        return t.value

    def poll(self, max_n: int = 256, wait_ms: int = -1) -> list[dict]:
        arr = (Response * max_n)()
        n = C.c_int()
        _check(lib().og_server_poll(self._h, arr, max_n, C.byref(n), wait_ms), "og_server_poll")
        out = [arr[i].as_dict() for i in range(n.value)]
        for r in out:
            self._bufs.pop(r["ticket"], None)
        return out

    def drain(self, timeout_ms: int = -1):
        _check(lib().og_server_drain(self._h, timeout_ms), "og_server_drain")

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().og_server_get_stats(self._h, C.byref(st)), "og_server_get_stats")
        return {f: getattr(st, f) for f, _ in st._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().og_server_destroy(self._h)
            self._h = None
            for g in self.graphs:
                g._engine_closed()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------- reference-named drivers

def bfs_opt(path: str, sourceNode: int | None = None, adviseRate: float = 0.0, budget: int = 0,
            testTimes: int = 5):
    """bfs_opt (BFS/oneGraph_BFS/CalculateOpt.h:9): without a source, the
    reference's five findbignode sources.  Returns [(source, depths, stats)]."""
    g = Graph.load(path, PLAIN)
    eng = Engine(g, budget=budget, advisek=adviseRate)
    if sourceNode is None:
        srcs, last = [], 0
        for _ in range(testTimes):
            last = g.findbignode(last)
            srcs.append(last)
    else:
        srcs = [sourceNode]
    res = [(s, eng.bfs(s), dict(eng.stats)) for s in srcs]
    eng.close()
    return res


def sssp_opt(path: str, sourceNode: int = 0, adviseRate: float = 0.0, budget: int = 0):
    g = Graph.load(path, WEIGHTED)
    eng = Engine(g, budget=budget, advisek=adviseRate)
    d = eng.sssp(sourceNode)
    st = dict(eng.stats)
    eng.close()
    return d, st


def cc_opt(path: str, adviseRate: float = 0.0, budget: int = 0):
    g = Graph.load(path, PLAIN)
    eng = Engine(g, budget=budget, advisek=adviseRate)
    lab = eng.cc()
    st = dict(eng.stats)
    eng.close()
    return lab, st


def pr_opt(path: str, adviseRate: float = 0.0, budget: int = 0, threshold: float = 0.001):
    g = Graph.load(path, PR)
    eng = Engine(g, budget=budget, advisek=adviseRate)
    r = eng.pr(threshold)
    st = dict(eng.stats)
    eng.close()
    return r, st


def link_probe(host_buffer, mode: int, reps: int = 3) -> float:
    """og_link_probe on a page-locked host buffer (a pinned torch tensor or an
    object with data_ptr(), numel(), element_size()): 0 SM reads, 1 one DMA
    copy, 2 two DMA copies at once; GB/s."""
    v = C.c_double()
    nbytes = host_buffer.numel() * host_buffer.element_size() // 16 * 16
    _check(lib().og_link_probe(C.c_void_p(host_buffer.data_ptr()), nbytes, mode, reps, C.byref(v)),
           "og_link_probe")
    return v.value


class PinnedArray(np.ndarray):
    """A numpy array in page-locked host memory from og_host_alloc, released
    with the last array that views it."""


class _PinnedBlock:
    def __init__(self, nbytes):
        p = _P()
        _check(lib().og_host_alloc(max(int(nbytes), 1), C.byref(p)), "og_host_alloc")
        self.ptr = p.value
        self.nbytes = nbytes

    def __del__(self):
        try:
            lib().og_host_free(C.c_void_p(self.ptr))
        except Exception:
            pass


def pinned_empty(shape, dtype=np.uint32) -> np.ndarray:
    """An uninitialised array in page-locked host memory (og_host_alloc), for
    result buffers: results are copied into it at the host link's rate."""
    dt = np.dtype(dtype)
    count = int(np.prod(shape))
    blk = _PinnedBlock(count * dt.itemsize)
    raw = np.ctypeslib.as_array(C.cast(blk.ptr, C.POINTER(C.c_uint8)), (max(count * dt.itemsize, 1),))
    a = raw[:count * dt.itemsize].view(dt).reshape(shape).view(PinnedArray)
    a._block = blk  # the memory lives as long as any view of it
    return a
