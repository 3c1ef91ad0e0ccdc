"""Parity at the benchmark's full size: R-MAT 27 (V = 2^27, 4.2 G symmetric
weighted edges) under an 8 GiB device budget with advisek 0.8, too large for
the oracle's algorithms to finish in test time.  Size-independent
properties stand in for them:
- SSSP distances and BFS depths pass the shortest-path certificate
  (ora_path_certify: no edge can improve a value, every reached vertex has a
  tight in-edge, the source is 1);
- union-find CC and label propagation, two unrelated algorithms, return the
  same labels;
- the batched BFS's per-source {reached, depth sum} equal single-source runs.
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
    uf = e.cc()
    e.set_param(og.PARAM_CC_METHOD, og.CC_LABEL_PROPAGATION)
    lp = e.cc()
    np.testing.assert_array_equal(uf, lp)
    assert (uf <= np.arange(g.V, dtype=np.uint32)).all()
    e.close()


def test_rmat27_batched_bfs_matches_single_source(rmat27):
    g = rmat27
    e = og.Engine(g, budget=8 * GIB, advisek=0.8, batch=True, direct=True)
    srcs = np.array(_sources(g, 64), np.uint32)
    _, checks = e.bfs_batch(srcs, out=False)
    for i in (0, 1, 63):
        d = e.bfs(int(srcs[i]))
        reached = d != g.V + 1
        assert checks[i, 0] == reached.sum(), i
        assert checks[i, 1] == d[reached].sum(dtype=np.uint64), i
    e.close()
