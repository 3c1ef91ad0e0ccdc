"""Generates tests/golden/golden.npz from the reference's own CPU programs.

Run where the reference tree is present:  python tests/golden/make_golden.py
It compiles BFS/cpu_BFS/main.cpp, CC/serial/serial.cpp and PR/cpu/pr.cpp from
their sources (oracle/build_oracle.py -> oracle/_ref/), writes every fixture
graph as a CSR file in the reference layout, runs the programs on it and stores
graph + outputs.  The tests compare the CPU oracle (and through it the GPU
engine) against these vectors; nothing here runs at test time.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402


def csr_from_edges(V, edges, symmetric=True):
    """Sorted, deduplicated CSR without self-loops from (u, v) pairs."""
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    if symmetric:
        e = np.concatenate([e, e[:, ::-1]])
    e = e[e[:, 0] != e[:, 1]]
    key = np.unique(e[:, 0] * (1 << 32) + e[:, 1])
    rows, cols = key >> 32, key & 0xFFFFFFFF
    off = np.zeros(V + 1, np.uint64)
    np.add.at(off, rows + 1, 1)
    return np.cumsum(off).astype(np.uint64), cols.astype(np.uint32)


def write_csr(path, off, col, outdeg=None):
    V = off.size - 1
    with open(path, "wb") as f:
        np.array([V, col.size], np.uint64).tofile(f)
        if outdeg is not None:
            np.asarray(outdeg, np.uint32).tofile(f)
        off[:V].astype(np.uint64).tofile(f)
        col.astype(np.uint32).tofile(f)


def rmat(scale, ef, permute=True, pagerank=False):
    import onegraph_gb300 as og
    g = og.Graph.rmat(scale, ef, seed=1, permute=permute, symmetric=not pagerank,
                      pagerank=pagerank)
    return (np.array(g.offsets), np.array(g.columns),
            None if g.outdeg is None else np.array(g.outdeg))


def graphs():
    out = {}
    out["path5"] = csr_from_edges(5, [(i, i + 1) for i in range(4)])
    out["star21"] = csr_from_edges(21, [(0, i) for i in range(1, 21)])
    out["two_comp_isolated"] = csr_from_edges(
        12, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0), (7, 8), (8, 9), (9, 10)])
    rng = np.random.default_rng(7)
    e = rng.integers(1, 64, size=(200, 2))
    out["vertex0_isolated"] = csr_from_edges(64, e)
    hub = [(0, i) for i in range(1, 5001)] + [(i, i + 1) for i in range(1, 5000, 7)]
    out["hub5000"] = csr_from_edges(5001, hub)
    out["rmat8"] = rmat(8, 16)[:2]
    out["rmat10"] = rmat(10, 16)[:2]
    out["rmat11_noperm"] = rmat(11, 8, permute=False)[:2]
    return out


def pr_graphs():
    out = {}
    # in-edge CSR of a directed graph with a dangling vertex (3) and a vertex
    # without in-edges (4): edges u->v
    d = [(0, 1), (1, 2), (2, 0), (0, 2), (4, 0), (4, 3), (2, 3), (1, 3)]
    V = 5
    rows = np.array([v for _, v in d]); cols = np.array([u for u, _ in d])
    key = np.unique(rows * (1 << 32) + cols)
    off = np.zeros(V + 1, np.uint64)
    np.add.at(off, (key >> 32) + 1, 1)
    outdeg = np.zeros(V, np.uint32)
    np.add.at(outdeg, key & 0xFFFFFFFF, 1)
    out["pr_tiny"] = (np.cumsum(off).astype(np.uint64), (key & 0xFFFFFFFF).astype(np.uint32), outdeg)
    out["pr_rmat10"] = rmat(10, 16, pagerank=True)
    out["pr_rmat12"] = rmat(12, 8, pagerank=True)
    return out


def run(prog, *args):
    r = subprocess.run([prog, *map(str, args)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s failed: %s" % (prog, r.stderr[-2000:]))


def main():
    progs = build_oracle.build_ref(force=True)
    if len(progs) != 3:
        sys.exit("reference programs unavailable (reference tree missing?)")
    data = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (off, col) in graphs().items():
            V = off.size - 1
            path = os.path.join(tmp, name + ".csr")
            write_csr(path, off, col)
            deg = np.diff(off.astype(np.int64))
            srcs = sorted({0, int(np.argmax(deg)), V // 2, V - 1})
            out = os.path.join(tmp, name + ".bfs")
            run(progs["ref_bfs"], path, out, *srcs)
            bfs = np.fromfile(out, np.uint32).reshape(len(srcs), V)
            out = os.path.join(tmp, name + ".cc")
            run(progs["ref_cc"], path, out)
            cc = np.fromfile(out, np.uint32)
            data[name + "/off"] = off
            data[name + "/col"] = col
            data[name + "/bfs_src"] = np.array(srcs, np.uint32)
            data[name + "/bfs"] = bfs
            data[name + "/cc"] = cc
        for name, (off, col, outdeg) in pr_graphs().items():
            V = off.size - 1
            path = os.path.join(tmp, name + ".csr")
            write_csr(path, off, col, outdeg)
            out = os.path.join(tmp, name + ".pr")
            run(progs["ref_pr"], path, out)
            raw = np.fromfile(out, np.uint8)
            data[name + "/off"] = off
            data[name + "/col"] = col
            data[name + "/outdeg"] = outdeg
            data[name + "/pr_cpu"] = raw[:8 * V].view(np.float64)
            data[name + "/pr_cpu_rounds"] = raw[8 * V:8 * V + 4].view(np.uint32)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **data)
    print("wrote", os.path.join(HERE, "golden.npz"), len(data), "arrays")


if __name__ == "__main__":
    main()
