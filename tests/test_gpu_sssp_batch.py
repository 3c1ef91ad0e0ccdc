"""Multi-source SSSP (og_sssp_batch and its round-by-round session): every
source's distances must equal a single-source og_sssp run, and the oracle's
Dijkstra, bit for bit, in every region layout, for every near/far width, and
for sources that join a pass in flight or reuse a finished slot."""
import numpy as np
import pytest

import onegraph_gb300 as og
import oracle

from test_gpu_engine import budget_for

pytestmark = pytest.mark.gpu


def sb_configs(g, k):
    flags = og.CFG_SSSP_BATCH(k)
    T = max(int(0.3 * g.E), 3 * 2048)
    return [
        ("resident", dict(budget=1 << 30, advisek=1.0)),
        ("oom", dict(budget=budget_for(g, T, flags), advisek=0.5)),
        ("tiny_static", dict(budget=budget_for(g, max(int(0.1 * g.E), 3 * 2048), flags), advisek=0.02)),
        ("direct", dict(budget=budget_for(g, T, flags | og.CFG_DIRECT), advisek=0.5, direct=True)),
    ]


def sources(g, n, seed):
    deg = g.degrees()
    rng = np.random.default_rng(seed)
    s = rng.integers(0, g.V, n).astype(np.uint32)
    s[0] = np.argmax(deg)                    # the hub
    if n > 2:
        s[1] = s[2]                          # a duplicate source
    if n > 3 and (deg == 0).any():
        s[3] = np.nonzero(deg == 0)[0][0]    # an isolated source
    return s


def check_rows(dist, checks, want):
    np.testing.assert_array_equal(dist, want)
    reached = want != 0xFFFFFFFF
    np.testing.assert_array_equal(checks[:, 0], reached.sum(1))
    np.testing.assert_array_equal(checks[:, 1], np.where(reached, want, 0).sum(1, dtype=np.uint64))


def test_sssp_batch_equals_single_source_and_dijkstra():
    g = og.Graph.rmat(12, 16, weighted=True, seed=7)
    off, pairs = np.array(g.offsets), np.array(g.edges)
    srcs = sources(g, 32, 5)
    want = None
    for cname, kw in sb_configs(g, 32):
        e = og.Engine(g, sssp_batch=32, **kw)
        if want is None:
            want = np.stack([e.sssp(int(s)) for s in srcs])
            for i in (0, 4, 31):
                np.testing.assert_array_equal(want[i], oracle.sssp_dijkstra(off, pairs, int(srcs[i])))
        dist, checks = e.sssp_batch(srcs)
        check_rows(dist, checks, want)
        assert e.stats["iterations"] > 0
        _, ck2 = e.sssp_batch(srcs, out=False)  # checks alone, second pass on the same engine
        np.testing.assert_array_equal(ck2, checks, err_msg=cname)
        e.close()


@pytest.mark.parametrize("k,n", [(4, 4), (8, 5), (16, 16), (20, 7)])
@pytest.mark.parametrize("delta", [0, 1, 64])
def test_sssp_batch_widths_and_deltas(k, n, delta):
    """Rows of 8, 16 and 32 slots, partly used; near/far width 0 (every
    improved vertex expanded every round, as the reference does), 1 and 64."""
    g = og.Graph.rmat(11, 16, weighted=True, seed=11, wmin=1, wmax=64)
    srcs = sources(g, n, 13 + k)
    T = max(int(0.3 * g.E), 3 * 2048)
    e = og.Engine(g, sssp_batch=k, budget=budget_for(g, T, og.CFG_SSSP_BATCH(k) | og.CFG_DIRECT),
                  advisek=0.5, direct=True)
    want = np.stack([e.sssp(int(s)) for s in srcs])
    assert e.get_param(og.PARAM_SSSP_BATCH_DELTA) == 0
    e.set_param(og.PARAM_SSSP_BATCH_DELTA, delta)
    dist, checks = e.sssp_batch(srcs)
    check_rows(dist, checks, want)
    e.close()


def test_sssp_batch_weights_beyond_a_byte():
    """Weights up to 70000 (32-bit staging weights, 17-bit record weights)."""
    g = og.Graph.rmat(10, 8, weighted=True, seed=3, wmin=5, wmax=70000)
    srcs = sources(g, 12, 2)
    for cname, kw in sb_configs(g, 12):
        e = og.Engine(g, sssp_batch=12, **kw)
        want = np.stack([e.sssp(int(s)) for s in srcs])
        dist, checks = e.sssp_batch(srcs)
        check_rows(dist, checks, want)
        e.close()


def test_sssp_batch_sources_join_in_flight():
    """Round-by-round session: three sources start, four more join after
    three rounds, each slot that leaves the pending mask already holds its
    final distances, and a new source reuses a finished slot."""
    g = og.Graph.rmat(12, 16, weighted=True, seed=21)
    srcs = sources(g, 9, 17)
    T = max(int(0.3 * g.E), 3 * 2048)
    e = og.Engine(g, sssp_batch=8, budget=budget_for(g, T, og.CFG_SSSP_BATCH(8) | og.CFG_DIRECT),
                  advisek=0.5, direct=True)
    want = {int(s): e.sssp(int(s)) for s in srcs}
    e.sssp_batch_begin()
    e.sssp_batch_join(srcs[:3], [0, 1, 2])
    slot_src = {0: int(srcs[0]), 1: int(srcs[1]), 2: int(srcs[2])}
    finished = []
    joined_late = False
    reused = False
    rounds = 0
    while True:
        pending, done = e.sssp_batch_step()
        rounds += 1
        for slot in list(slot_src):
            if not (pending >> slot) & 1:
                np.testing.assert_array_equal(e.sssp_batch_fetch(slot), want[slot_src[slot]],
                                              err_msg="slot %d" % slot)
                ck = e.sssp_batch_checks(1 << slot)[slot]
                w = want[slot_src[slot]]
                assert ck[0] == (w != 0xFFFFFFFF).sum()
                finished.append(slot_src.pop(slot))
                if joined_late and not reused:
                    # a finished slot takes a new source
                    e.sssp_batch_join([srcs[8]], [slot])
                    slot_src[slot] = int(srcs[8])
                    reused = True
        if rounds == 3:
            e.sssp_batch_join(srcs[3:7], [3, 4, 5, 6])
            slot_src.update({3 + i: int(s) for i, s in enumerate(srcs[3:7])})
            joined_late = True
        if done and not slot_src:
            break
        assert rounds < 100000
    assert reused
    assert sorted(finished) == sorted(int(s) for s in list(srcs[:7]) + [srcs[8]])
    e.close()


def test_sssp_batch_rejects_bad_use():
    g = og.Graph.rmat(9, 8, weighted=True)
    e = og.Engine(g, sssp_batch=4, budget=1 << 30)
    with pytest.raises(og.OGError):
        e.sssp_batch(np.arange(5, dtype=np.uint32))  # more sources than slots
    with pytest.raises(og.OGError):
        e.sssp_batch([g.V])  # source out of range
    with pytest.raises(og.OGError):
        e.sssp_batch_join([1, 2], [0, 0])  # one slot twice
    e.close()
    plain = og.Engine(g, budget=1 << 30)
    with pytest.raises(og.OGError):
        plain.sssp_batch([1])  # no batch state
    plain.close()
    gu = og.Graph.rmat(9, 8)
    with pytest.raises(og.OGError):
        og.Engine(gu, sssp_batch=4, budget=1 << 30)  # unweighted graph


def test_other_queries_end_a_session_and_share_its_memory():
    """PageRank, batched BFS and multi-source SSSP share one per-vertex
    allocation on an engine that has them all: each gives its own correct
    result when they alternate, and a query between the rounds of an open
    session ends the session (OG_E_STATE) instead of corrupting it."""
    g = og.Graph.rmat(11, 16, weighted=True, seed=13)
    off, pairs = np.array(g.offsets), np.array(g.edges)
    col = np.ascontiguousarray(pairs[:, 0])
    deg = np.diff(off.astype(np.int64)).astype(np.uint32)
    T = max(int(0.3 * g.E), 3 * 2048)
    flags = og.CFG_SSSP_BATCH(8) | og.CFG_BATCH | og.CFG_PR | og.CFG_DIRECT
    e = og.Engine(g, sssp_batch=8, batch=True, pagerank=True, direct=True, advisek=0.5,
                  budget=budget_for(g, T, flags))
    ref, _, _ = oracle.pr_l1(off, col, deg, 0.85, 1e-6, 200)
    srcs = sources(g, 8, 3)
    want = np.stack([e.sssp(int(s)) for s in srcs])
    for _ in range(2):
        r = e.pr_l1(0.85, 1e-6, 200)
        assert np.abs(r.astype(np.float64) - ref).max() < 1e-6
        dist, _ = e.sssp_batch(srcs)
        np.testing.assert_array_equal(dist, want)
        depths, _ = e.bfs_batch(srcs)
        np.testing.assert_array_equal(depths[0], e.bfs(int(srcs[0])))
    e.sssp_batch_begin()
    e.sssp_batch_join(srcs[:2], [0, 1])
    e.sssp_batch_step()
    e.bfs(int(srcs[0]))
    with pytest.raises(og.OGError):
        e.sssp_batch_step()
    e.close()
