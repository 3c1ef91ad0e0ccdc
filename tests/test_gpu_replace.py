"""Static-region replacement (OG_CFG_REPLACE, Ascetic's fragment swap that
the reference declares in BFS/oneGraph_BFS/gpu_kernels.h:46-66,153-176 and
never defines): results through the fragment slots against the oracle, the
policy moving a repeatedly read part of the dynamic region into the slots,
and the argument checks.  Results are compared bit for bit."""
import numpy as np
import pytest

import onegraph_gb300 as og
import oracle

pytestmark = pytest.mark.gpu


def budget_for(g, edge_slots, flags):
    # per-vertex and fixed bytes do not depend on the replacement mode (whose
    # split needs a dynamic region, which a 1 TiB plan does not have)
    p = g.plan(budget=1 << 40, flags=flags & ~og.CFG_REPLACE)
    return p["vertex_bytes"] + p["fixed_bytes"] + int(edge_slots) * p["stage_edge_bytes"]


FLAGS = og.CFG_DIRECT | og.CFG_REPLACE


@pytest.mark.parametrize("words", [256, 1024])
def test_replace_results_equal_oracle(words):
    """BFS (both directions), SSSP (plain rounds and near/far) and label
    propagation CC through the slots, queries back to back so that the slots
    change between and within them."""
    g = og.Graph.rmat(12, 16, weighted=True)
    off, pairs, col = np.array(g.offsets), np.array(g.edges), np.array(g.columns)
    b = budget_for(g, int(0.4 * g.E), FLAGS)
    e = og.Engine(g, budget=b, advisek=0.6, direct=True, replace=True)
    assert 0 < e.plan["static_edges"] < g.E
    assert e.plan == g.plan(budget=b, advisek=0.6, flags=FLAGS)  # the planner reports the same split
    e.set_param(og.PARAM_FRAGMENT_WORDS, words)
    assert e.get_param(og.PARAM_FRAGMENT_WORDS) == words
    fs = e.fragment_stats()
    assert fs["slots"] > 0 and fs["fragment_words"] == words and fs["swaps"] == 0
    rng = np.random.default_rng(5)
    srcs = [int(np.argmax(g.degrees()))] + rng.integers(0, g.V, 4).tolist()
    for rep in range(2):
        for s in srcs:
            for direction in (og.BFS_TOP_DOWN, og.BFS_AUTO):
                e.set_param(og.PARAM_BFS_DIRECTION, direction)
                np.testing.assert_array_equal(oracle.normalise_bfs(e.bfs(s), g.V), oracle.bfs(off, col, s)[0],
                                              err_msg="bfs src %d direction %d" % (s, direction))
            want = oracle.sssp_dijkstra(off, pairs, s)
            for delta in (0, 4):
                e.set_param(og.PARAM_SSSP_DELTA, delta)
                np.testing.assert_array_equal(e.sssp(s), want, err_msg="sssp src %d delta %d" % (s, delta))
        e.set_param(og.PARAM_CC_METHOD, og.CC_LABEL_PROPAGATION)
        np.testing.assert_array_equal(e.cc(), oracle.cc(off, col)[0])
    fs = e.fragment_stats()
    assert fs["records_slots"] > 0 and fs["records_host"] > 0
    assert fs["swaps"] > 0 and fs["swap_bytes"] == fs["swaps"] * 4 * (words + 4)
    e.close()


def two_components():
    """R-MAT 12 on vertices [0, 4096) and R-MAT 10 on [4096, 5120): the
    planner's static prefix holds part of the first, none of the second."""
    a = og.Graph.rmat(12, 16, seed=1)
    b = og.Graph.rmat(10, 16, seed=9)
    oa, ca = np.array(a.offsets), np.array(a.columns)
    ob, cb = np.array(b.offsets), np.array(b.columns)
    off = np.concatenate([oa, ob[1:] + oa[-1]]).astype(np.uint64)
    col = np.concatenate([ca, cb + a.V]).astype(np.uint32)
    return og.Graph.from_arrays(off, col), a.V, a.E


def test_replace_moves_a_repeatedly_read_component_into_slots():
    """Queries that keep reading one part of the dynamic region: the policy
    moves its fragments into slots, so later queries read fewer records over
    the host link than the first, and results stay exact."""
    g, va, ea = two_components()
    off, col = np.array(g.offsets), np.array(g.columns)
    # direct mode: the whole edge share is static, 32 / 13 packed records per
    # 4-byte staging slot, so the planned prefix holds about 0.8 of the first
    # component's edges (0.4 after the slots take half of its bytes) and the
    # slots about as many records as the second component has
    e = og.Engine(g, budget=budget_for(g, int(0.33 * ea), FLAGS), advisek=1.0, direct=True, replace=True)
    e.set_param(og.PARAM_FRAGMENT_WORDS, 256)
    assert 0 < e.plan["static_vertices"] < va  # the second component is all dynamic
    assert e.fragment_stats()["slots"] * 256 * 32 > 1.2 * (g.E - ea) * e.plan["edge_bits"]
    e.set_param(og.PARAM_BFS_DIRECTION, og.BFS_TOP_DOWN)
    s = va + int(np.argmax(g.degrees()[va:]))
    want = oracle.bfs(off, col, s)[0]
    link, host = [], []
    for _ in range(6):
        before = e.fragment_stats()["records_host"]
        np.testing.assert_array_equal(oracle.normalise_bfs(e.bfs(s), g.V), want)
        link.append(e.stats["link_bytes"])
        host.append(e.fragment_stats()["records_host"] - before)
    assert host[-1] < 0.5 * host[0], host
    assert link[-1] < link[0], link
    fs = e.fragment_stats()
    assert fs["swaps"] > 0
    e.close()


def test_replace_argument_checks():
    g = og.Graph.rmat(11, 16, weighted=True)
    b = budget_for(g, int(0.4 * g.E), FLAGS)
    with pytest.raises(og.OGError) as ex:  # staged mode has no fragment slots
        og.Engine(g, budget=b, advisek=0.6, replace=True)
    assert ex.value.status == 1
    with pytest.raises(og.OGError) as ex:  # a resident graph has no dynamic region to share
        og.Engine(g, budget=1 << 30, advisek=1.0, direct=True, replace=True)
    assert ex.value.status == 4
    e = og.Engine(g, budget=b, advisek=0.6, direct=True, replace=True)
    for bad in (100, 128, 1 << 21):
        with pytest.raises(og.OGError) as ex:
            e.set_param(og.PARAM_FRAGMENT_WORDS, bad)
        assert ex.value.status == 1
    # a size whose one slot does not fit the slot bytes is refused before the
    # current layout is released: the engine keeps answering through it
    words = e.get_param(og.PARAM_FRAGMENT_WORDS)
    with pytest.raises(og.OGError) as ex:
        e.set_param(og.PARAM_FRAGMENT_WORDS, 1 << 20)
    assert ex.value.status == 4
    assert e.get_param(og.PARAM_FRAGMENT_WORDS) == words
    s = int(np.argmax(g.degrees()))
    np.testing.assert_array_equal(e.sssp(s), oracle.sssp_dijkstra(np.array(g.offsets), np.array(g.edges), s))
    with pytest.raises(og.OGError) as ex:
        e.clone()
    assert ex.value.status == 9
    e.close()
    plain = og.Engine(g, budget=b, advisek=0.6, direct=True)
    with pytest.raises(og.OGError) as ex:
        plain.fragment_stats()
    assert ex.value.status == 8
    with pytest.raises(og.OGError) as ex:
        plain.set_param(og.PARAM_FRAGMENT_WORDS, 256)
    assert ex.value.status == 8
    plain.close()
