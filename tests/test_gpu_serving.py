"""Serving loop: every request's result must be the same alone and in the mix
(bit for bit: BFS depths, SSSP distances, and the FP32 PageRank ranks, whose
pull sums are deterministic for a given plan), while requests overlap on the
GPU and queued BFS requests are fused into batched passes."""
import numpy as np
import pytest

import onegraph_gb300 as og

from test_gpu_engine import budget_for

pytestmark = pytest.mark.gpu

FLAGS = og.CFG_BATCH | og.CFG_PR | og.CFG_DIRECT


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


def test_results_identical_alone_and_in_the_mix():
    graphs = _graphs()
    reqs = _requests(graphs, 240)
    srv = og.Server(budget=sum(_budget(g) for g in graphs) + (64 << 20), workers=4, max_batch=64)
    gids = [srv.add_graph(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True)
            for g in graphs]
    assert gids == [0, 1, 2]
    outs = {}
    for i, (gid, algo, src) in enumerate(reqs):
        out = None
        if i % 7 == 0:  # a subset also returns the full per-vertex result
            out = np.empty(graphs[gid].V, np.float32 if algo == og.ALGO_PR else np.uint32)
            outs[i] = out
        srv.submit(gid, algo, src, iterations=5, out=out, user=i)
    srv.drain()
    resp = {}
    while True:
        got = srv.poll(512, wait_ms=0)
        if not got:
            break
        for r in got:
            resp[r["user"]] = r
    assert len(resp) == len(reqs)
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert any(r["batch"] > 1 and r["algo"] == og.ALGO_BFS for r in resp.values()), \
        "queued BFS requests should be fused"
    # alone: each request on its own engine planned exactly like the server's
    alone = [og.Engine(g, budget=_budget(g), advisek=0.5, direct=True, pagerank=True, batch=True)
             for g in graphs]
    for i, (gid, algo, src) in enumerate(reqs):
        r = resp[i]
        assert r["status"] == 0, r
        e = alone[gid]
        if algo == og.ALGO_BFS:
            full = e.bfs(src)
        elif algo == og.ALGO_SSSP:
            full = e.sssp(src)
        else:
            full = e.pr_l1(0.85, 0.0, 5)
        assert r["checksum"] == e.checksum(algo), (i, algo, r)
        if i in outs:
            np.testing.assert_array_equal(outs[i].view(np.uint32), full.view(np.uint32))
    for e in alone:
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
