"""The CPU oracle pinned against the reference's own CPU programs.

tests/golden/golden.npz holds outputs of BFS/cpu_BFS (runCPUBFS),
CC/serial and PR/cpu compiled from the reference sources
(tests/golden/make_golden.py).  The restatement must match them bit for bit.
"""
import numpy as np
import pytest

import onegraph_gb300 as og
import oracle

from conftest import golden_names


def test_bfs_matches_reference_cpu_bfs(golden):
    names = golden_names(golden, "bfs")
    assert len(names) >= 8
    for n in names:
        off, col = golden[n + "/off"], golden[n + "/col"]
        for i, s in enumerate(golden[n + "/bfs_src"]):
            got, _ = oracle.bfs(off, col, int(s))
            np.testing.assert_array_equal(got, golden[n + "/bfs"][i], err_msg="%s src %d" % (n, s))


def test_cc_matches_reference_serial_cc(golden):
    for n in golden_names(golden, "cc"):
        got, _ = oracle.cc(golden[n + "/off"], golden[n + "/col"])
        np.testing.assert_array_equal(got, golden[n + "/cc"], err_msg=n)


def test_pr_cpu_matches_reference_bit_for_bit(golden):
    names = golden_names(golden, "pr_cpu")
    assert names
    for n in names:
        got, rounds = oracle.pr_cpu(golden[n + "/off"], golden[n + "/col"], golden[n + "/outdeg"])
        assert rounds == int(golden[n + "/pr_cpu_rounds"][0])
        np.testing.assert_array_equal(got.view(np.uint64), golden[n + "/pr_cpu"].view(np.uint64))


def test_golden_edge_cases_present(golden):
    # isolated vertices, vertex 0 without edges, a hub above one LBS tile
    cc = golden["two_comp_isolated/cc"]
    assert len(np.unique(cc)) == 5
    off = golden["vertex0_isolated/off"]
    assert off[1] == off[0]
    assert np.diff(golden["hub5000/off"].astype(np.int64)).max() > 4096


def _weighted(scale=9, seed=5):
    import onegraph_gb300 as og
    g = og.Graph.rmat(scale, 16, seed=seed, weighted=True)
    return np.array(g.offsets), np.array(g.edges)


def test_dijkstra_equals_label_correcting_restatement():
    off, pairs = _weighted()
    deg = np.diff(off.astype(np.int64))
    for s in [0, int(np.argmax(deg)), 100]:
        d = oracle.sssp_dijkstra(off, pairs, s)
        f, _ = oracle.sssp_frontier(off, pairs, s)
        np.testing.assert_array_equal(d, f)
        assert d[s] == 1


def test_dijkstra_certificate():
    """Every edge satisfies d[v] <= d[u] + w and every reached vertex other than
    the source has a tight in-edge (exact shortest paths)."""
    off, pairs = _weighted(10, 9)
    s = 3
    d = oracle.sssp_dijkstra(off, pairs, s).astype(np.int64)
    rows = np.repeat(np.arange(off.size - 1), np.diff(off.astype(np.int64)))
    u, v, w = rows, pairs[:, 0].astype(np.int64), pairs[:, 1].astype(np.int64)
    INF = 0xFFFFFFFF
    reach = d[u] != INF
    assert (d[v][reach] <= d[u][reach] + w[reach]).all()
    tight = np.zeros(off.size - 1, bool)
    tight[v[reach & (d[v] == d[u] + w)]] = True
    reached = np.nonzero(d != INF)[0]
    assert all(tight[x] or x == s for x in reached)


def test_pr_onegraph_semantics_small():
    """0.15 + 0.85*sum, start 1.0, a vertex freezes its old rank once |delta| <= thresh."""
    off = np.array([0, 1, 2, 3], np.uint64)  # 3-cycle of in-edges: 1->0, 2->1, 0->2
    col = np.array([1, 2, 0], np.uint32)
    od = np.array([1, 1, 1], np.uint32)
    r, rounds = oracle.pr_onegraph(off, col, od)
    np.testing.assert_allclose(r, 1.0)  # fixed point of the un-normalised form
    assert rounds == 1


def test_pr_l1_converges_to_stationary_distribution():
    import onegraph_gb300 as og
    g = og.Graph.rmat(9, 8, pagerank=True, symmetric=False)
    off, col, od = np.array(g.offsets), np.array(g.columns), np.array(g.outdeg)
    p, it, l1 = oracle.pr_l1(off, col, od, 0.85, 1e-12, 1000)
    assert l1 < 1e-12 and it < 1000
    # fixed point check with dense matrices
    V = g.V
    M = np.zeros((V, V))
    rows = np.repeat(np.arange(V), np.diff(off.astype(np.int64)))
    np.add.at(M, (rows, col), 1.0 / np.maximum(od[col], 1))
    np.testing.assert_allclose(p, 0.15 / V + 0.85 * M @ p, rtol=0, atol=1e-12)


@pytest.mark.parametrize("n", ["bfs", "cc"])
def test_normalise_bfs_unreached(n):
    d = np.array([1, 2, 6, 6], np.uint32)
    out = oracle.normalise_bfs(d, 5)
    assert out.tolist() == [1, 2, 0xFFFFFFFF, 0xFFFFFFFF]


def test_pr_l1_multithreaded_equals_serial():
    import onegraph_gb300 as og
    g = og.Graph.rmat(11, 16, pagerank=True, symmetric=False)
    off, col, od = np.array(g.offsets), np.array(g.columns), np.array(g.outdeg)
    a, ia, la = oracle.pr_l1(off, col, od, 0.85, 1e-9, 500)
    b = np.empty(g.V)
    ib, lb = oracle.pr_l1_mt_raw(g.V, g._off_p, g._edges_p, g._outdeg_p, 0.85, 1e-9, 500, 5, b)
    assert ia == ib and la == lb
    np.testing.assert_array_equal(a, b)


def test_cc_round_bounded_is_the_first_round():
    """The bounded timing sample performs exactly cc()'s first round over the
    edges it scans (pairs read with stride 2)."""
    import onegraph_gb300 as og
    g = og.Graph.rmat(10, 16, weighted=True)
    off, pairs = np.array(g.offsets), np.array(g.edges)
    out = np.empty(g.V, np.uint32)
    n = oracle.cc_round_bounded_raw(g.V, g._off_p, g._edges_p, 2, 1 << 62, out)
    assert n == g.E
    want = np.arange(g.V, dtype=np.uint32)
    for u in range(g.V):  # serial order, labels updated in place as in ora_cc
        lab = want[u]
        for v in pairs[off[u]:off[u + 1], 0]:
            if lab < want[v]:
                want[v] = lab
    np.testing.assert_array_equal(out, want)
    assert oracle.cc_round_bounded_raw(g.V, g._off_p, g._edges_p, 2, 100, out) < g.E


def test_path_certificate_accepts_exact_and_rejects_planted_errors():
    """ora_path_certify: exact SSSP distances and BFS depths pass; a distance
    raised or lowered by one (planted here, in the oracle's output) fails."""
    g = og.Graph.rmat(11, 16, weighted=True, seed=4)
    off, pairs = np.array(g.offsets), np.array(g.edges)
    s = int(np.argmax(np.diff(off.astype(np.int64))))
    d = oracle.sssp_dijkstra(off, pairs, s)
    assert oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, False, d, s, 0xFFFFFFFF, 4) == (0, g.V)
    b, _ = oracle.bfs(off, pairs[:, 0].copy(), s)
    assert oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, True, b, s, 0xFFFFFFFF, 4)[0] == 0
    reached = np.nonzero((d != 0xFFFFFFFF) & (np.arange(g.V) != s))[0]
    for delta in (1, -1):
        bad = d.copy()
        v = int(reached[len(reached) // 2])
        bad[v] = np.uint32(int(bad[v]) + delta)
        n, first = oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, False, bad, s, 0xFFFFFFFF, 4)
        assert n > 0
    wrong_src = d.copy()
    wrong_src[s] = 2
    assert oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, False, wrong_src, s, 0xFFFFFFFF, 4)[0] > 0


def test_union_find_components_match_reference_serial_cc(golden):
    """ora_cc_uf_mt (the full-size CC oracle) gives CC/serial's labels on
    every symmetric golden graph, on 1 and 8 threads."""
    for n in golden_names(golden, "cc"):
        off = np.ascontiguousarray(golden[n + "/off"], np.uint64)
        col = np.ascontiguousarray(golden[n + "/col"], np.uint32)
        for threads in (1, 8):
            lab = np.empty(off.size - 1, np.uint32)
            comps = oracle.cc_uf_mt_raw(off.size - 1, off.ctypes.data_as(oracle._P),
                                        col.ctypes.data_as(oracle._P), 1, threads, lab)
            np.testing.assert_array_equal(lab, golden[n + "/cc"], err_msg="%s/%d" % (n, threads))
            assert comps == len(np.unique(golden[n + "/cc"]))


@pytest.mark.parametrize("scale,kw", [
    (10, dict(weighted=True)), (12, {}), (11, dict(pagerank=True, symmetric=False)),
    (13, dict(weighted=True, permute=False)), (9, dict(weighted=True, wmin=5, wmax=70000)),
    (14, dict(edge_factor=8, seed=7, weight_seed=9, weighted=True)),
])
def test_oracle_rmat_equals_the_engine_generator(scale, kw):
    """The oracle's CPU R-MAT (used where the engine must not be loaded)
    builds the engine generator's CSR bit for bit."""
    r = oracle.RmatGraph(scale, **kw)
    g = og.Graph.rmat(scale, **kw)
    assert (r.V, r.E) == (g.V, g.E)
    np.testing.assert_array_equal(r.offsets, g.offsets)
    np.testing.assert_array_equal(np.asarray(r.edges), np.asarray(g.edges))
    if kw.get("pagerank"):
        np.testing.assert_array_equal(r.outdeg, g.outdeg)
    r.close()
    g.close()


def test_bounded_baseline_samples_agree_with_the_complete_runs(golden):
    """The bounded BFS sample is runCPUBFS when unbounded (and stops early when
    bounded); the bounded pull is pr_cal's first iteration sum on a symmetric graph."""
    for n in golden_names(golden, "bfs")[:4]:
        off = np.ascontiguousarray(golden[n + "/off"], np.uint64)
        col = np.ascontiguousarray(golden[n + "/col"], np.uint32)
        V = off.size - 1
        s = int(golden[n + "/bfs_src"][0])
        out = np.empty(V, np.uint32)
        scanned = oracle.bfs_bounded_raw(V, off.ctypes.data_as(oracle._P), col.ctypes.data_as(oracle._P), 1,
                                         s, 0, out)
        np.testing.assert_array_equal(out, golden[n + "/bfs"][0], err_msg=n)
        assert scanned >= 1 or off[-1] == 0
        if off[-1] > 8:
            assert oracle.bfs_bounded_raw(V, off.ctypes.data_as(oracle._P), col.ctypes.data_as(oracle._P), 1,
                                          s, 1, out) <= scanned
    g = og.Graph.rmat(10, 16, weighted=True)
    off, pairs = np.array(g.offsets), np.ascontiguousarray(np.array(g.edges))
    sums = np.empty(g.V)
    read = oracle.pr_pull_bounded_raw(g.V, off.ctypes.data_as(oracle._P), pairs.ctypes.data_as(oracle._P), 2, 0, sums)
    assert read == g.E
    deg = np.diff(off.astype(np.int64)).astype(np.float64)
    contrib = np.where(deg > 0, 1.0 / g.V / np.maximum(deg, 1), 0.0)
    want = np.array([0.15 + 0.15 * contrib[pairs[off[v]:off[v + 1], 0]].sum() for v in range(g.V)])
    np.testing.assert_allclose(sums, want, rtol=1e-12)
