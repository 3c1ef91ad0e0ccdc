"""Batched multi-source BFS: every source's depths must equal a single-source
og_bfs run bit for bit, in every region layout."""
import numpy as np
import pytest

import onegraph_gb300 as og
import oracle

from test_gpu_engine import budget_for

pytestmark = pytest.mark.gpu


def batch_configs(g):
    flags = og.CFG_BATCH
    T = max(int(0.3 * g.E), 3 * 2048)
    return [
        ("resident", dict(budget=1 << 30, advisek=1.0)),
        ("oom", dict(budget=budget_for(g, T, flags), advisek=0.5)),
        ("direct", dict(budget=budget_for(g, T, flags | og.CFG_DIRECT), advisek=0.5, direct=True)),
    ]


@pytest.mark.parametrize("weighted", [False, True])
def test_batch_equals_single_source(weighted):
    g = og.Graph.rmat(12, 16, weighted=weighted, seed=7)
    deg = g.degrees()
    rng = np.random.default_rng(5)
    srcs = rng.integers(0, g.V, 64).astype(np.uint32)
    srcs[0] = np.argmax(deg)
    srcs[1] = srcs[2]  # duplicate source
    srcs[3] = np.nonzero(deg == 0)[0][0] if (deg == 0).any() else srcs[3]  # isolated source
    single = None
    for cname, kw in batch_configs(g):
        e = og.Engine(g, batch=True, **kw)
        if single is None:
            single = np.stack([e.bfs(int(s)) for s in srcs])
        depths, checks = e.bfs_batch(srcs)
        np.testing.assert_array_equal(depths, single, err_msg=cname)
        reached = single != g.V + 1
        np.testing.assert_array_equal(checks[:, 0], reached.sum(1))
        np.testing.assert_array_equal(checks[:, 1], np.where(reached, single, 0).sum(1, dtype=np.uint64))
        # checks alone (no depth matrix) give the same numbers
        _, ck2 = e.bfs_batch(srcs, out=False)
        np.testing.assert_array_equal(ck2, checks)
        e.close()


def test_batch_to_separate_buffers_equals_single_source():
    """og_bfs_batch_to: each source's depths land in its own host array
    (page-locked and pageable), equal to og_bfs and to og_bfs_batch's rows;
    a host-driven-levels engine refuses it."""
    g = og.Graph.rmat(12, 16, seed=11)
    rng = np.random.default_rng(2)
    srcs = rng.integers(0, g.V, 9).astype(np.uint32)
    for cname, kw in batch_configs(g):
        e = og.Engine(g, batch=True, **kw)
        want = np.stack([e.bfs(int(s)) for s in srcs])
        outs = [og.pinned_empty(g.V, np.uint32) if i % 2 else np.full(g.V, 7, np.uint32)
                for i in range(srcs.size)]
        ck = e.bfs_batch_to(srcs, outs)
        for i in range(srcs.size):
            np.testing.assert_array_equal(outs[i], want[i], err_msg="%s source %d" % (cname, i))
        _, ck2 = e.bfs_batch(srcs, out=False)
        np.testing.assert_array_equal(ck, ck2)
        e.close()
    lv = og.Engine(g, batch_levels=True, budget=1 << 30, advisek=1.0)
    with pytest.raises(og.OGError) as ex:
        lv.bfs_batch_to(srcs[:2], [np.empty(g.V, np.uint32) for _ in range(2)])
    assert ex.value.status == 9
    lv.close()


def test_batch_to_depths_beyond_a_byte():
    """A path of 601 vertices (depths up to 601, beyond the byte matrix),
    a separate R-MAT part and two isolated vertices, V = 1627 (rows of the
    byte matrix not 4-byte aligned): a batch with a deep source falls back
    to single-source runs, a shallow batch takes the byte path, and both
    equal og_bfs."""
    L = 601
    r = og.Graph.rmat(10, 8, seed=4)
    ro, rc = np.array(r.offsets), np.array(r.columns)
    V = L + r.V + 2
    adj = [[] for _ in range(V)]
    for i in range(L - 1):
        adj[i].append(i + 1)
        adj[i + 1].append(i)
    for u in range(r.V):
        adj[L + u].extend(int(c) + L for c in rc[ro[u]:ro[u + 1]])
    adj = [sorted(set(a)) for a in adj]
    off = np.concatenate([[0], np.cumsum([len(a) for a in adj])]).astype(np.uint64)
    col = np.array([c for a in adj for c in a], np.uint32)
    g = og.Graph.from_arrays(off, col)
    assert g.V % 4 != 0
    srcs = np.array([0, L // 2, L + 5, V - 1], np.uint32)
    for kw in (dict(budget=1 << 30, advisek=1.0), dict(budget=budget_for(g, g.E // 3, og.CFG_BATCH | og.CFG_DIRECT),
                                                       advisek=0.5, direct=True)):
        e = og.Engine(g, batch=True, **kw)
        want = [e.bfs(int(s)) for s in srcs]
        assert want[0].max() > 255
        outs = [og.pinned_empty(g.V, np.uint32) for _ in srcs]
        e.bfs_batch_to(srcs, outs)
        for i in range(srcs.size):
            np.testing.assert_array_equal(outs[i], want[i])
        # a batch whose depths all fit a byte takes the byte path
        outs2 = [np.zeros(g.V, np.uint32) for _ in range(2)]
        e.bfs_batch_to(srcs[2:], outs2)
        np.testing.assert_array_equal(outs2[0], want[2])
        np.testing.assert_array_equal(outs2[1], want[3])
        e.close()


def test_persistent_graph_levels_and_all_configs_agree():
    """The persistent kernel (direct launch or CUDA-graph replay), the
    host-driven level loop and every autotuner candidate give the same depths."""
    g = og.Graph.rmat(13, 16, seed=3)
    rng = np.random.default_rng(9)
    srcs = rng.integers(0, g.V, 40).astype(np.uint32)
    for cname, kw in batch_configs(g):
        e = og.Engine(g, batch=True, **kw)
        lv = og.Engine(g, batch_levels=True, **kw)
        want, wck = lv.bfs_batch(srcs)
        got, ck = e.bfs_batch(srcs)  # persistent, depth matrix (direct launch)
        np.testing.assert_array_equal(got, want, err_msg=cname)
        np.testing.assert_array_equal(ck, wck)
        for rep in range(2):  # captured once, then replayed
            _, ck2 = e.bfs_batch(srcs, out=False)
            np.testing.assert_array_equal(ck2, wck)
        assert e.stats["chunks"] == 1, "second call should replay the CUDA graph"
        res = e.bfs_batch_tune(srcs, reps=1)
        assert len(res["candidates"]) == 5 and 0 <= res["best"] < 5
        for ci in range(5):
            e.bfs_batch_set_config(ci)
            d, ck3 = e.bfs_batch(srcs)
            np.testing.assert_array_equal(d, want, err_msg="%s config %d" % (cname, ci))
        e.close()
        lv.close()


def test_batch_small_counts_and_oracle():
    g = og.Graph.rmat(11, 16)
    off, col = np.array(g.offsets), np.array(g.columns)
    e = og.Engine(g, batch=True, **dict(batch_configs(g))["oom"])
    for n in (1, 5, 33):
        srcs = np.arange(n, dtype=np.uint32) * 7
        depths, _ = e.bfs_batch(srcs)
        for i, s in enumerate(srcs):
            np.testing.assert_array_equal(oracle.normalise_bfs(depths[i], g.V), oracle.bfs(off, col, int(s))[0])


def test_batch_errors():
    g = og.Graph.rmat(8, 8)
    e = og.Engine(g, budget=1 << 28)
    with pytest.raises(og.OGError) as ex:
        e.bfs_batch([1, 2])
    assert ex.value.status == 9
    b = og.Engine(g, budget=1 << 28, batch=True)
    with pytest.raises(og.OGError) as ex:
        b.bfs_batch(np.zeros(65, np.uint32))
    assert ex.value.status == 1
    with pytest.raises(og.OGError) as ex:
        b.bfs_batch([g.V])
    assert ex.value.status == 1


@pytest.mark.parametrize("scale", [10, 13])
def test_batch_bottom_up_levels(scale):
    """On a symmetric graph the persistent kernel expands the wide levels
    bottom-up; its depths equal the top-down-only kernel's and single-source
    runs, in every region layout, and it examines fewer edges.  A directed
    graph (no reverse edges) stays top-down."""
    g = og.Graph.rmat(scale, 16, seed=11)
    assert g.symmetric()
    deg = g.degrees()
    rng = np.random.default_rng(scale)
    srcs = rng.integers(0, g.V, 64).astype(np.uint32)
    srcs[0] = np.argmax(deg)
    for cname, kw in batch_configs(g):
        e = og.Engine(g, batch=True, **kw)
        got, ck = e.bfs_batch(srcs)
        _, ck_r = e.bfs_batch(srcs, out=False)  # captured graph
        auto_edges = e.stats["edges_static"] + e.stats["edges_dynamic"]
        e.set_param(og.PARAM_BFS_DIRECTION, og.BFS_TOP_DOWN)
        want, wck = e.bfs_batch(srcs)
        _, ck_t = e.bfs_batch(srcs, out=False)  # recaptured for the new direction
        td_edges = e.stats["edges_static"] + e.stats["edges_dynamic"]
        np.testing.assert_array_equal(got, want, err_msg=cname)
        np.testing.assert_array_equal(ck, wck)
        np.testing.assert_array_equal(ck_r, wck)
        np.testing.assert_array_equal(ck_t, wck)
        assert auto_edges < td_edges, (cname, auto_edges, td_edges)
        for i in (0, 1, 63):
            np.testing.assert_array_equal(got[i], e.bfs(int(srcs[i])), err_msg="%s source %d" % (cname, i))
        e.close()
    gd = og.Graph.rmat(scale, 16, seed=11, symmetric=False)
    e = og.Engine(gd, batch=True, budget=1 << 30, advisek=1.0)
    got, _ = e.bfs_batch(srcs)
    for i in (0, 1, 63):
        np.testing.assert_array_equal(got[i], e.bfs(int(srcs[i])))
    e.close()


def _irregular_symmetric_graph():
    """V = 1000 (not a multiple of 32): a 300-leaf star whose hub (vertex 950)
    lies in the dynamic region and has a longer list than a bottom-up lane
    scans, so it goes to the pull pass; a 200-vertex path hanging off a leaf
    (many levels); random edges among 501..940; isolated vertices."""
    rng = np.random.default_rng(17)
    V = 1000
    edges = set()
    for leaf in range(1, 301):
        edges.add((950, leaf))
    prev = 5
    for v in range(301, 501):
        edges.add((prev, v))
        prev = v
    for _ in range(1500):
        a, b = rng.integers(501, 941, 2)
        if a != b:
            edges.add((int(a), int(b)))
    edges.add((700, 37))  # joins the random part to the star
    edges = {(min(a, b), max(a, b)) for a, b in edges}
    adj = [[] for _ in range(V)]
    for a, b in edges:
        adj[a].append(b)
        adj[b].append(a)
    off = np.zeros(V + 1, np.uint64)
    for v in range(V):
        off[v + 1] = off[v] + len(adj[v])
    col = np.array([u for v in range(V) for u in sorted(adj[v])], np.uint32)
    return off, col


def test_batch_irregular_graph_directions():
    off, col = _irregular_symmetric_graph()
    g = og.Graph.from_arrays(off, col)
    g.set_symmetric(True)
    V = off.size - 1
    rng = np.random.default_rng(3)
    srcs = rng.integers(0, V, 64).astype(np.uint32)
    srcs[:6] = [950, 500, 999, 150, 301, 37]  # hub, path end, isolated, leaf, path start, star-side
    for cname, kw in [("resident", dict(budget=1 << 30, advisek=1.0)),
                      ("direct", dict(budget=budget_for(g, 400, og.CFG_BATCH | og.CFG_DIRECT),
                                      advisek=0.5, direct=True))]:
        e = og.Engine(g, batch=True, **kw)
        single = np.stack([e.bfs(int(s)) for s in srcs])
        for direction in (og.BFS_AUTO, og.BFS_TOP_DOWN):
            e.set_param(og.PARAM_BFS_DIRECTION, direction)
            for n in (64, 7):
                got, ck = e.bfs_batch(srcs[:n])
                np.testing.assert_array_equal(got, single[:n], err_msg="%s direction %d n %d" % (cname, direction, n))
                _, ck2 = e.bfs_batch(srcs[:n], out=False)
                np.testing.assert_array_equal(ck2, ck)
        for i in (0, 1, 2):
            np.testing.assert_array_equal(oracle.normalise_bfs(single[i], V), oracle.bfs(off, col, int(srcs[i]))[0])
        e.close()


def test_batch_byte_depths_and_pinned_outputs():
    """og_bfs_batch_u8 equals og_bfs_batch's depths as bytes (0 unreached),
    on repeated calls that reuse and then grow the kept depth matrix, into
    pageable and page-locked (og_host_alloc) buffers."""
    g = og.Graph.rmat(12, 16, seed=4)
    rng = np.random.default_rng(2)
    T = max(int(0.3 * g.E), 3 * 2048)
    e = og.Engine(g, batch=True, direct=True, advisek=0.5, budget=budget_for(g, T, og.CFG_BATCH | og.CFG_DIRECT))
    for n in (7, 3, 64, 64):
        srcs = rng.integers(0, g.V, n).astype(np.uint32)
        want, ck = e.bfs_batch(srcs)
        pinned = og.pinned_empty((n, g.V), np.uint32)
        got, ck2 = e.bfs_batch(srcs, out=pinned)
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(ck2, ck)
        b8, clamped, ck8 = e.bfs_batch_u8(srcs, out=og.pinned_empty((n, g.V), np.uint8))
        assert clamped == 0
        np.testing.assert_array_equal(ck8, ck)
        np.testing.assert_array_equal(b8, np.where(want == g.V + 1, 0, want).astype(np.uint8))
        b8p, _, _ = e.bfs_batch_u8(srcs)
        np.testing.assert_array_equal(b8p, b8)
    e.close()


def test_batch_byte_depths_clamp_long_paths():
    """A path of 300 vertices: depths of 255 and more become 255 and are counted."""
    V = 300
    col = np.arange(1, V, dtype=np.uint32)  # 0 -> 1 -> ... -> 299, vertex 299 has no edge
    off = np.concatenate([np.arange(V, dtype=np.uint64), [V - 1]]).astype(np.uint64)
    g = og.Graph.from_arrays(off, col)
    e = og.Engine(g, batch=True, budget=1 << 28)
    want, _ = e.bfs_batch([0])
    b8, clamped, _ = e.bfs_batch_u8([0])
    assert want[0, 299] == 300 and clamped == (want[0] >= 255).sum() == 46
    np.testing.assert_array_equal(b8[0], np.minimum(want[0], 255).astype(np.uint8))
    e.close()


@pytest.mark.parametrize("layout", ["resident", "oom", "direct"])
def test_batch_session_sources_join_in_flight(layout):
    """Level-by-level session: four sources start, four more join after two
    levels (their depths count from the level they joined at), every slot
    that leaves the in-flight mask holds final depths and checks equal to a
    single-source og_bfs, and a new source reuses a finished slot (its
    visited bits are cleared first)."""
    g = og.Graph.rmat(12, 16, seed=23)
    deg = g.degrees()
    rng = np.random.default_rng(31)
    srcs = [int(x) for x in rng.integers(0, g.V, 10)]
    srcs[0] = int(np.argmax(deg))
    srcs[5] = srcs[4]  # a duplicate source
    if (deg == 0).any():
        srcs[6] = int(np.nonzero(deg == 0)[0][0])  # an isolated source
    kw = dict(batch_configs(g))[layout]
    e = og.Engine(g, batch=True, **kw)
    want = {s: e.bfs(s) for s in set(srcs)}
    e.bfs_batch_begin(record_depths=True)
    e.bfs_batch_join(srcs[:4], [0, 5, 17, 63])
    slot_src = {0: srcs[0], 5: srcs[1], 17: srcs[2], 63: srcs[3]}
    finished, levels, reused, joined_late = [], 0, False, False
    while True:
        pending, done = e.bfs_batch_step()
        levels += 1
        assert e.stats["launches"] > 0 or done
        for slot in list(slot_src):
            if (pending >> slot) & 1:
                continue
            w = want[slot_src[slot]]
            np.testing.assert_array_equal(e.bfs_batch_fetch(slot), w, err_msg="%s slot %d" % (layout, slot))
            ck = e.bfs_batch_checks(1 << slot)[slot]
            reached = w != g.V + 1
            assert ck[0] == reached.sum() and ck[1] == np.where(reached, w, 0).sum(dtype=np.uint64)
            finished.append(slot_src.pop(slot))
            if joined_late and not reused:
                e.bfs_batch_join([srcs[8]], [slot])  # a finished slot takes a new source
                slot_src[slot] = srcs[8]
                reused = True
        if levels == 2:
            e.bfs_batch_join(srcs[4:8], [1, 2, 40, 41])
            slot_src.update({1: srcs[4], 2: srcs[5], 40: srcs[6], 41: srcs[7]})
            joined_late = True
        if done and not slot_src:
            break
        assert levels < 10000
    assert reused
    assert sorted(finished) == sorted(srcs[:8] + [srcs[8]])
    e.close()


def test_batch_session_rejects_bad_use():
    g = og.Graph.rmat(10, 8)
    plain = og.Engine(g, budget=1 << 30)
    with pytest.raises(og.OGError):
        plain.bfs_batch_begin()  # no batch state
    plain.close()
    e = og.Engine(g, batch=True, budget=1 << 30)
    with pytest.raises(og.OGError):
        e.bfs_batch_step()  # no session yet
    e.bfs_batch_begin()
    with pytest.raises(og.OGError):
        e.bfs_batch_join([1], [64])  # slot out of range
    with pytest.raises(og.OGError):
        e.bfs_batch_join([g.V], [0])  # source out of range
    with pytest.raises(og.OGError):
        e.bfs_batch_join([1, 2], [3, 3])  # one slot twice
    e.bfs_batch_join([int(np.argmax(g.degrees()))], [3])
    with pytest.raises(og.OGError):
        e.bfs_batch_join([2], [3])  # slot in flight
    e.bfs_batch_step()
    with pytest.raises(og.OGError):
        e.bfs_batch_fetch(0)  # opened without depth recording
    e.bfs(1)  # another query ends the session
    with pytest.raises(og.OGError):
        e.bfs_batch_step()
    e.close()
