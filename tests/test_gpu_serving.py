"""Serving loop: every request's result must be the same alone and in the mix
(bit for bit: BFS depths, SSSP distances, and the FP32 PageRank ranks, whose
pull sums are deterministic for a given plan) and equal the oracle's (BFS
and Dijkstra bit for bit; PageRank within 1e-6 max-abs of the FP64 oracle's
five iterations), while requests overlap on the GPU, queued BFS requests are
fused into batched passes and SSSP requests join multi-source passes in
flight."""
import numpy as np
import pytest

import onegraph_gb300 as og
import oracle

from test_gpu_engine import budget_for

pytestmark = pytest.mark.gpu

SSSP_SLOTS = 8
FLAGS = og.CFG_BATCH | og.CFG_PR | og.CFG_DIRECT | og.CFG_SSSP_BATCH(SSSP_SLOTS)


def _graphs():
    return [og.Graph.rmat(s, 16, weighted=True, seed=s) for s in (10, 11, 12)]


def _budget(g):
    return budget_for(g, max(int(0.3 * g.E), 3 * 2048), FLAGS)


def _requests(graphs, n, seed=4):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        gid = int(rng.integers(0, len(graphs)))
        deg = graphs[gid].degrees()
        u = rng.random()
        algo = og.ALGO_BFS if u < 0.6 else (og.ALGO_SSSP if u < 0.9 else og.ALGO_PR)
        src = int(rng.choice(np.nonzero(deg)[0]))
        reqs.append((gid, algo, src))
    return reqs


def _collect(srv, n):
    srv.drain()
    resp = {}
    while True:
        got = srv.poll(512, wait_ms=0)
        if not got:
            break
        for r in got:
            resp[r["user"]] = r
    assert len(resp) == n
    return resp


def test_results_identical_alone_in_the_mix_and_to_the_oracle():
    graphs = _graphs()
    reqs = _requests(graphs, 240)
    srv = og.Server(budget=sum(_budget(g) for g in graphs) + (64 << 20), workers=4, max_batch=64)
    gids = [srv.add_graph(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True,
                          sssp_batch=SSSP_SLOTS) for g in graphs]
    assert gids == [0, 1, 2]
    outs = {}
    for i, (gid, algo, src) in enumerate(reqs):
        out = None
        if i % 3 == 0:  # every third request also returns its per-vertex result
            out = np.empty(graphs[gid].V, np.float32 if algo == og.ALGO_PR else np.uint32)
            outs[i] = out
        srv.submit(gid, algo, src, iterations=5, out=out, user=i)
    resp = _collect(srv, len(reqs))
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert any(r["batch"] > 1 and r["algo"] == og.ALGO_BFS for r in resp.values()), \
        "queued BFS requests should be fused"
    assert any(r["batch"] > 1 and r["algo"] == og.ALGO_SSSP for r in resp.values()), \
        "queued SSSP requests should share multi-source passes"
    # alone: each request on its own engine planned exactly like the server's
    alone = [og.Engine(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True, batch=True,
                       sssp_batch=SSSP_SLOTS) for g in graphs]
    pr_ref = {}
    for i, (gid, algo, src) in enumerate(reqs):
        r = resp[i]
        assert r["status"] == 0, r
        e, g = alone[gid], graphs[gid]
        off = np.array(g.offsets)
        if algo == og.ALGO_BFS:
            full = e.bfs(src)
        elif algo == og.ALGO_SSSP:
            full = e.sssp(src)
        else:
            full = e.pr_l1(0.85, 0.0, 5)
        assert r["checksum"] == e.checksum(algo), (i, algo, r)
        if i not in outs:
            continue
        got = outs[i]
        np.testing.assert_array_equal(got.view(np.uint32), full.view(np.uint32), err_msg="request %d" % i)
        if algo == og.ALGO_BFS:
            want, _ = oracle.bfs(off, np.array(g.columns), src)
            np.testing.assert_array_equal(oracle.normalise_bfs(got, g.V), want, err_msg="bfs %d" % i)
        elif algo == og.ALGO_SSSP:
            np.testing.assert_array_equal(got, oracle.sssp_dijkstra(off, np.array(g.edges), src),
                                          err_msg="sssp %d" % i)
        else:
            if gid not in pr_ref:
                deg = np.diff(off.astype(np.int64)).astype(np.uint32)
                pr_ref[gid] = oracle.pr_l1(off, np.array(g.columns), deg, 0.85, 0.0, 5)[0]
            assert np.abs(got.astype(np.float64) - pr_ref[gid]).max() < 1e-6, i
    for e in alone:
        e.close()
    srv.close()


def test_sssp_requests_join_a_pass_in_flight():
    """One worker, 3 x SSSP_SLOTS requests on one graph: a pass holds at most
    SSSP_SLOTS sources at a time, so answering more than that from one pass
    means requests took the slots of finished ones while it ran."""
    g = og.Graph.rmat(12, 16, weighted=True, seed=5)
    srv = og.Server(budget=0, workers=1, max_batch=64)
    srv.add_graph(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True, sssp_batch=SSSP_SLOTS)
    deg = g.degrees()
    rng = np.random.default_rng(11)
    srcs = [int(x) for x in rng.choice(np.nonzero(deg)[0], 3 * SSSP_SLOTS)]
    outs = [np.empty(g.V, np.uint32) for _ in srcs]
    for i, s in enumerate(srcs):
        srv.submit(0, og.ALGO_SSSP, s, out=outs[i], user=i)
    resp = _collect(srv, len(srcs))
    assert max(r["batch"] for r in resp.values()) > SSSP_SLOTS
    e = og.Engine(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True)
    for i, s in enumerate(srcs):
        assert resp[i]["status"] == 0
        np.testing.assert_array_equal(outs[i], e.sssp(s), err_msg="request %d" % i)
        assert resp[i]["checksum"] == e.checksum(og.ALGO_SSSP)
    e.close()
    srv.close()


def test_admission_waits_for_memory():
    """With a budget that holds only the resident graphs, no extra context is
    created: requests queue for the one context per graph and still complete."""
    graphs = _graphs()[:2]
    used = 0
    for g in graphs:  # device bytes the server's engines will hold (same configuration)
        probe = og.Engine(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True)
        resident, ctx = probe.bytes()
        used += resident + ctx
        probe.close()
    srv = og.Server(budget=used, workers=4, max_batch=1)
    for g in graphs:
        srv.add_graph(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True)
    reqs = _requests(graphs, 40, seed=7)
    for i, (gid, algo, src) in enumerate(reqs):
        srv.submit(gid, algo, src, user=i)
    srv.drain()
    st = srv.stats()
    assert st["completed"] == 40 and st["contexts_created"] == 0 and st["gpu_passes"] == 40
    srv.close()


def test_clone_shares_the_resident_graph():
    g = og.Graph.rmat(11, 16, weighted=True)
    e = og.Engine(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True, batch=True)
    c = e.clone()
    a = e.sssp(3)
    b = c.sssp(3)
    np.testing.assert_array_equal(a, b)
    resident, ctx = c.bytes()
    assert resident == 0 and ctx > 0  # a clone holds only per-query state
    c.close()
    e.close()


def test_bfs_requests_join_a_pass_in_flight():
    """With OG_SERVER_BFS_JOIN, one worker and max_batch 8: 24 BFS requests on
    one graph are answered by passes of at most 8 slots, so a response
    numbered above 8 took the slot of a finished source while the pass ran;
    every checksum equals og_bfs's for its source alone."""
    g = og.Graph.rmat(12, 16, weighted=True, seed=9)
    srv = og.Server(budget=0, workers=1, max_batch=8, bfs_join=True)
    srv.add_graph(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True, sssp_batch=SSSP_SLOTS)
    deg = g.degrees()
    rng = np.random.default_rng(12)
    srcs = [int(x) for x in rng.choice(np.nonzero(deg)[0], 24)]
    for i, s in enumerate(srcs):
        srv.submit(0, og.ALGO_BFS, s, user=i)
    resp = _collect(srv, len(srcs))
    assert max(r["batch"] for r in resp.values()) > 8
    e = og.Engine(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True)
    for i, s in enumerate(srcs):
        assert resp[i]["status"] == 0
        e.bfs(s)
        assert resp[i]["checksum"] == e.checksum(og.ALGO_BFS), "request %d" % i
    e.close()
    srv.close()
