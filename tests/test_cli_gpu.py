"""The four reference-compatible programs end to end on the GPU: CSR file in,
--dump of per-vertex results out, compared with the oracle."""
import os
import subprocess

import numpy as np
import pytest

import onegraph_gb300 as og
import oracle

pytestmark = pytest.mark.gpu


def run(name, *args):
    r = subprocess.run([os.path.join(og.BIN_DIR, name), *map(str, args)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_bfs_cli_reference_flags_and_findbignode(tmp_path):
    g = og.Graph.rmat(14, 16, permute=False)  # hubs above degree 3000 exist
    p, out = str(tmp_path / "g.csr"), str(tmp_path / "bfs.bin")
    g.save(p)
    o = run("BFS_OneGraph", "--type", "bfs", "-f", p, "--adviseK", "0.3", "--budget", "2M",
            "--dump", out, "--json", "1")
    assert "nodeSum" in o and "move overload size" in o
    V = g.V
    dumps = np.fromfile(out, np.uint32).reshape(-1, V)
    last, srcs = 0, []
    for _ in range(5):
        last = g.findbignode(last)
        srcs.append(last)
    assert dumps.shape[0] == 5
    off, col = np.array(g.offsets), np.array(g.columns)
    for d, s in zip(dumps, srcs):
        np.testing.assert_array_equal(oracle.normalise_bfs(d, V), oracle.bfs(off, col, s)[0])


def test_sssp_cc_pr_cli(tmp_path):
    gw = og.Graph.rmat(12, 16, weighted=True)
    p = str(tmp_path / "w.csr")
    gw.save(p)
    out = str(tmp_path / "sssp.bin")
    run("SSSP_OneGraph", "-type", "sssp", "-f", p, "-r", 17, "-adviseK", "0.4", "--budget", "300K",
        "--dump", out)
    off, pairs = np.array(gw.offsets), np.array(gw.edges)
    np.testing.assert_array_equal(np.fromfile(out, np.uint32), oracle.sssp_dijkstra(off, pairs, 17))
    g = og.Graph.rmat(12, 16)
    p = str(tmp_path / "p.csr")
    g.save(p)
    out = str(tmp_path / "cc.bin")
    run("CC_OneGraph", "-f", p, "--advisek", "0.5", "--budget", "300K", "--dump", out, "--direct", "1")
    want_cc = oracle.cc(np.array(g.offsets), np.array(g.columns))[0]
    np.testing.assert_array_equal(np.fromfile(out, np.uint32), want_cc)
    # the same through union-find, with the symmetry checked or asserted
    for flag in ("check", "1"):
        o = run("CC_OneGraph", "-f", p, "--advisek", "0.5", "--budget", "300K", "--dump", out,
                "--direct", "1", "--symmetric", flag)
        assert flag == "1" or "symmetric 1" in o
        np.testing.assert_array_equal(np.fromfile(out, np.uint32), want_cc)
    gp = og.Graph.rmat(11, 16, pagerank=True, symmetric=False)
    p = str(tmp_path / "pr.csr")
    gp.save(p)
    out = str(tmp_path / "pr.bin")
    run("PR_OneGraph", "-f", p, "-adviseK", "0.5", "--budget", "220K", "--dump", out)
    want, _ = oracle.pr_onegraph(np.array(gp.offsets), np.array(gp.columns), np.array(gp.outdeg))
    got = np.fromfile(out, np.float32).astype(np.float64)
    assert (np.abs(got - want) / want).max() < 5e-3
