"""Parity at the benchmarks' full sizes: R-MAT 27 (V = 2^27, 4.2 G symmetric
weighted edges) under an 8 GiB device budget with advisek 0.8, and the
serving mix's four graphs (R-MAT 22/24/26/27) under 24 GiB.  The oracle's
serial algorithms cannot finish at this size in test time, so:
- SSSP distances and BFS depths pass the shortest-path certificate
  (ora_path_certify: no edge can improve a value, every reached vertex has a
  tight in-edge, the source is 1);
- CC labels (union-find and label propagation) equal the oracle's
  multi-threaded union-find bit for bit (component minima, the reference's
  CC/serial labels on a symmetric graph);
- all 64 depth arrays of one batched BFS equal 64 single-source runs;
- every served request of a 300-request mix returns the same per-vertex
  result as the request run alone, and served BFS/SSSP results pass the
  certificate.
"""
import os

import numpy as np
import pytest

import onegraph_gb300 as og
import oracle

pytestmark = pytest.mark.gpu

GIB = 1 << 30


@pytest.fixture(scope="module")
def rmat27():
    try:
        g = og.Graph.rmat(27, 16, seed=1, weight_seed=2, weighted=True, on_gpu=True)
    except og.OGError:
        g = og.Graph.rmat(27, 16, seed=1, weight_seed=2, weighted=True)
    yield g
    g.close()


def _sources(g, n):
    deg = g.degrees()
    rng = np.random.default_rng(3)
    out = [int(np.argmax(deg))]
    while len(out) < n:
        s = int(rng.integers(0, g.V))
        if deg[s] > 0:
            out.append(s)
    return out


def test_rmat27_sssp_bfs_cc_certified(rmat27):
    g = rmat27
    threads = os.cpu_count() or 4
    e = og.Engine(g, budget=8 * GIB, advisek=0.8, direct=True)
    assert e.plan["dynamic_edges"] > 0  # the out-of-memory path
    for s in _sources(g, 2):
        d = e.sssp(s)
        assert e.stats["link_bytes"] > 0
        bad, first = oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, False, d, s, 0xFFFFFFFF, threads)
        assert bad == 0, ("sssp", s, bad, first)
    s = _sources(g, 1)[0]
    b = oracle.normalise_bfs(e.bfs(s), g.V)
    bad, first = oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, True, b, s, 0xFFFFFFFF, threads)
    assert bad == 0, ("bfs", bad, first)
    want = np.empty(g.V, np.uint32)
    comps = oracle.cc_uf_mt_raw(g.V, g._off_p, g._edges_p, 2, threads, want)
    uf = e.cc()
    np.testing.assert_array_equal(uf, want)
    e.set_param(og.PARAM_CC_METHOD, og.CC_LABEL_PROPAGATION)
    lp = e.cc()
    np.testing.assert_array_equal(lp, want)
    assert e.checksum(og.ALGO_CC)[0] == comps
    e.close()


def test_rmat27_batched_bfs_matches_single_source(rmat27):
    """All 64 depth arrays of one og_bfs_batch equal single-source og_bfs."""
    g = rmat27
    e = og.Engine(g, budget=8 * GIB, advisek=0.8, batch=True, direct=True)
    srcs = np.array(_sources(g, 64), np.uint32)
    depths, checks = e.bfs_batch(srcs)
    _, ck2 = e.bfs_batch(srcs, out=False)  # the replayed CUDA graph gives the same checks
    np.testing.assert_array_equal(ck2, checks)
    one = np.empty(g.V, np.uint32)
    for i in range(64):
        e.bfs(int(srcs[i]), out=one)
        np.testing.assert_array_equal(depths[i], one, err_msg="source %d" % i)
        reached = one != g.V + 1
        assert checks[i, 0] == reached.sum(), i
    del depths
    e.close()


def test_rmat27_multi_source_sssp_certified(rmat27):
    """A multi-source SSSP pass at full size: every source's distances equal
    single-source og_sssp's, and two pass the certificate."""
    g = rmat27
    threads = os.cpu_count() or 4
    e = og.Engine(g, budget=11 * GIB, advisek=1.0, direct=True, sssp_batch=4, batch=True)
    srcs = np.array(_sources(g, 4), np.uint32)
    dist, checks = e.sssp_batch(srcs)
    assert e.stats["link_bytes"] > 0
    one = np.empty(g.V, np.uint32)
    for i in range(4):
        e.sssp(int(srcs[i]), out=one)
        np.testing.assert_array_equal(dist[i], one, err_msg="source %d" % i)
    for i in (0, 3):
        bad, first = oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, False, dist[i], int(srcs[i]),
                                             0xFFFFFFFF, threads)
        assert bad == 0, (i, bad, first)
    e.close()


SERVING = {22: (1.0, 16), 24: (3.75, 16), 26: (6.75, 8), 27: (11.0, 4)}


def test_serving_mix_full_size_alone_equals_served(rmat27):
    """The serving configuration at full size (R-MAT 22/24/26/27 under 24 GiB,
    Poisson arrivals, 60/30/10 BFS/SSSP/PR5): every request returns its whole
    per-vertex result, which must equal the request run alone on an engine
    planned like the server's (bit for bit, PageRank included), and a sample
    of served BFS and SSSP results pass the shortest-path certificate."""
    import bench
    threads = os.cpu_count() or 4
    graphs = []
    for sc in (22, 24, 26):
        graphs.append(og.Graph.rmat(sc, 16, seed=1, weight_seed=2, weighted=True, on_gpu=True))
    graphs.append(rmat27)
    n = 300
    arrivals, gsel, algos, srcs = bench.serving_requests([g.degrees() for g in graphs], n, 2000.0)
    cfgs = [SERVING[sc] for sc in (22, 24, 26, 27)]
    srv = og.Server(budget=24 * GIB, workers=4, max_batch=64)
    for g, (b, k) in zip(graphs, cfgs):
        srv.add_graph(g, budget=int(b * GIB), advisek=1.0, direct=True, pagerank=True, sssp_batch=k)
    outs = [np.empty(graphs[gi].V, np.float32 if algos[i] == bench.ALGO_PR else np.uint32)
            for i, gi in enumerate(gsel)]
    resp, _ = bench.serve_pass(srv, arrivals, gsel, algos, srcs, outs=outs)
    srv.close()
    assert all(resp[i]["status"] == 0 for i in range(n))
    assert any(resp[i]["batch"] > 1 and algos[i] == bench.ALGO_SSSP for i in range(n))
    one = [np.empty(g.V, np.uint32) for g in graphs]
    certified = {bench.ALGO_BFS: 0, bench.ALGO_SSSP: 0}
    for gi, (g, (b, k)) in enumerate(zip(graphs, cfgs)):
        e = og.Engine(g, budget=int(b * GIB), advisek=1.0, direct=True, pagerank=True, batch=True, sssp_batch=k)
        for i in np.nonzero(gsel == gi)[0]:
            a, s = int(algos[i]), srcs[i]
            if a == bench.ALGO_BFS:
                e.bfs(s, out=one[gi])
            elif a == bench.ALGO_SSSP:
                e.sssp(s, out=one[gi])
            else:
                e.pr_l1(0.85, 0.0, 5, out=one[gi].view(np.float32))
            np.testing.assert_array_equal(outs[i].view(np.uint32), one[gi], err_msg="request %d" % i)
            assert resp[i]["checksum"] == e.checksum(a), i
            if a != bench.ALGO_PR and certified[a] < 2 and gi >= 2:
                d = oracle.normalise_bfs(outs[i], g.V) if a == bench.ALGO_BFS else outs[i]
                bad, first = oracle.path_certify_raw(g.V, g._off_p, g._edges_p, 2, a == bench.ALGO_BFS, d, s,
                                                     0xFFFFFFFF, threads)
                assert bad == 0, (i, a, bad, first)
                certified[a] += 1
        e.close()
    assert certified == {bench.ALGO_BFS: 2, bench.ALGO_SSSP: 2}
    for g in graphs[:3]:
        g.close()
