"""Host-side logic of libog.so that needs no GPU: CSR file format, validation,
the seeded R-MAT generator, the region planner, findbignode, the exported
ABI and the CLI's argument handling."""
import os
import re
import subprocess

import numpy as np
import pytest

import onegraph_gb300 as og

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _write(path, header, *arrays):
    with open(path, "wb") as f:
        np.asarray(header, np.uint64).tofile(f)
        for a in arrays:
            a.tofile(f)


def test_abi_exports_every_header_symbol():
    declared = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        hdr = open(os.path.join(ROOT, "include", h)).read()
        declared |= set(re.findall(r"^\s*(?:[a-z_ ]+\*?\s*)\b(og_[a-z0-9_]+)\s*\(", hdr, re.M))
    assert "og_bfs" in declared and "og_engine_create" in declared
    assert {"og_sssp_batch", "og_k_relax", "og_k_gather", "og_k_wait_check", "og_link_probe"} <= declared
    lib = og.lib()
    for name in sorted(declared):
        assert hasattr(lib, name), name
    bound = {n for n, _, _ in og.SIGNATURES}
    assert declared <= bound, declared - bound
    assert lib.og_abi_version() == og.ABI_VERSION == 6


def test_csr_roundtrip_all_kinds(tmp_path):
    for kind, kw in [(og.PLAIN, {}), (og.WEIGHTED, {"weighted": True}),
                     (og.PR, {"pagerank": True, "symmetric": False})]:
        g = og.Graph.rmat(8, 8, **kw)
        p = str(tmp_path / ("g%d.csr" % kind))
        g.save(p)
        h = og.Graph.load(p, kind)
        assert (h.V, h.E, h.kind) == (g.V, g.E, kind)
        np.testing.assert_array_equal(h.offsets, g.offsets)
        np.testing.assert_array_equal(h.edges, g.edges)
        if kind == og.PR:
            np.testing.assert_array_equal(h.outdeg, g.outdeg)
        # file layout: V, E, [outdeg], offsets[V] (no sentinel), edges
        raw = np.fromfile(p, np.uint8)
        eb = 8 if kind == og.WEIGHTED else 4
        assert raw.size == 16 + (4 * g.V if kind == og.PR else 0) + 8 * g.V + eb * g.E


def test_load_rejects_malformed_files(tmp_path):
    p = str(tmp_path / "bad.csr")
    with pytest.raises(og.OGError) as e:
        og.Graph.load(str(tmp_path / "missing.csr"))
    assert e.value.status == 2
    open(p, "wb").write(b"\x01\x02")
    with pytest.raises(og.OGError) as e:
        og.Graph.load(p)
    assert e.value.status == 3  # short header
    _write(p, [3, 4], np.array([0, 2, 1], np.uint64), np.array([1, 2, 0, 1], np.uint32))
    with pytest.raises(og.OGError) as e:
        og.Graph.load(p)
    assert e.value.status == 3 and "decrease" in str(e.value)
    _write(p, [3, 4], np.array([0, 2, 3], np.uint64), np.array([1, 2, 0, 7], np.uint32))
    with pytest.raises(og.OGError) as e:
        og.Graph.load(p)
    assert "column" in str(e.value)
    _write(p, [3, 5], np.array([0, 2, 3], np.uint64), np.array([1, 2, 0, 1], np.uint32))
    with pytest.raises(og.OGError) as e:  # header says 5 edges, file has 4
        og.Graph.load(p)
    assert e.value.status == 3
    _write(p, [0, 0])
    with pytest.raises(og.OGError):
        og.Graph.load(p)
    _write(p, [1 << 33, 0])
    with pytest.raises(og.OGError):  # V must fit the reference's 32-bit vertex ids
        og.Graph.load(p)


def test_rmat_properties_and_determinism():
    g = og.Graph.rmat(10, 16, seed=1)
    h = og.Graph.rmat(10, 16, seed=1, threads=1)
    np.testing.assert_array_equal(g.offsets, h.offsets)
    np.testing.assert_array_equal(g.columns, h.columns)
    off = g.offsets.astype(np.int64)
    rows = np.repeat(np.arange(g.V), np.diff(off))
    col = g.columns.astype(np.int64)
    assert (rows != col).all()
    key = (rows << 32) | col
    assert (np.diff(key) > 0).all()  # sorted rows and columns, no duplicates
    rev = np.sort((col << 32) | rows)
    np.testing.assert_array_equal(rev, key)  # symmetric
    assert og.Graph.rmat(10, 16, seed=2).E != g.E
    w = og.Graph.rmat(10, 16, seed=1, weighted=True)
    np.testing.assert_array_equal(w.edges[:, 0], g.columns)
    ww = w.edges[:, 1]
    assert ww.min() >= 1 and ww.max() <= 64
    # weight of {u, v} is the same in both directions
    wmap = dict(zip(((rows << 32) | col).tolist(), ww.tolist()))
    assert all(wmap[(c << 32) | r] == x for r, c, x in zip(rows[:500], col[:500], ww[:500]))


def test_rmat_pagerank_graph_is_in_edge_csr():
    g = og.Graph.rmat(9, 8, pagerank=True, symmetric=False)
    assert g.kind == og.PR
    off = g.offsets.astype(np.int64)
    dst = np.repeat(np.arange(g.V), np.diff(off))
    outdeg = np.bincount(g.columns, minlength=g.V)
    np.testing.assert_array_equal(outdeg, g.outdeg)
    assert (dst != g.columns).all()


def test_rmat_rejects_bad_parameters():
    with pytest.raises(og.OGError):
        og.Graph.rmat(0)
    with pytest.raises(og.OGError):
        og.Graph.rmat(8, abc=(0.7, 0.3, 0.3))
    with pytest.raises(og.OGError):
        og.Graph.rmat(8, weighted=True, pagerank=True)


def test_findbignode_matches_reference_rule():
    g = og.Graph.rmat(12, 16, permute=False)
    deg = np.diff(g.offsets.astype(np.int64))
    last = 0
    for _ in range(5):
        nxt = g.findbignode(last)
        cand = [i for i in range(last + 1, g.V - 1) if deg[i] > 3000]
        assert nxt == (cand[0] if cand else last)
        last = nxt


def test_planner_reference_semantics():
    g = og.Graph.rmat(10, 16)
    off = np.array(g.offsets)
    base = og.plan(g.V, g.E, off, og.PLAIN, budget=1 << 30)
    # huge budget: heuristic (10 - E/T)/9 > 1 -> 1.0, everything static
    assert base["advisek"] == 1.0 and base["dynamic_edges"] == 0 and base["chunk_edges"] == 0
    vb, fb = base["vertex_bytes"], base["fixed_bytes"]
    T = g.E // 2
    p = og.plan(g.V, g.E, off, og.PLAIN, budget=vb + fb + 4 * T, advisek=0.5)
    assert p["edge_capacity"] == T
    assert p["max_partition"] == int(0.5 * T)
    Vs = p["static_vertices"]
    # the static region is the largest vertex prefix whose edges fit the partition
    assert off[Vs] <= p["max_partition"] < off[Vs + 1]
    assert p["static_edges"] == off[Vs] and p["dynamic_edges"] == g.E - off[Vs]
    assert p["chunk_edges"] % 2048 == 0 and p["chunk_edges"] > 0
    assert p["static_edges"] + 2 * p["chunk_edges"] <= T
    # heuristic: E/T = 2 -> (10 - 2)/9
    q = og.plan(g.V, g.E, off, og.PLAIN, budget=vb + fb + 4 * T)
    assert abs(q["advisek_auto"] - 8 / 9) < 1e-6 and abs(q["advisek"] - 8 / 9) < 1e-6
    # E/T > 10 -> negative -> 0.5
    big = og.Graph.rmat(13, 16)
    boff = np.array(big.offsets)
    bb = og.plan(big.V, big.E, boff, og.PLAIN, budget=1 << 30)
    r = og.plan(big.V, big.E, boff, og.PLAIN,
                budget=bb["vertex_bytes"] + bb["fixed_bytes"] + 4 * (big.E // 12))
    assert r["advisek_auto"] == 0.5 and r["static_edges"] <= r["max_partition"]
    # too small for even two staging tiles
    with pytest.raises(og.OGError) as e:
        og.plan(g.V, g.E, off, og.PLAIN, budget=vb + fb + 4 * 3000)
    assert e.value.status == 4
    # user value above 1 is clamped
    s = og.plan(g.V, g.E, off, og.PLAIN, budget=vb + fb + 4 * T, advisek=3.0)
    assert s["advisek"] == 1.0
    # direct mode needs no staging
    d = og.plan(g.V, g.E, off, og.PLAIN, budget=vb + fb + 4 * T, advisek=0.5, flags=og.CFG_DIRECT)
    assert d["chunk_edges"] == 0 and d["dynamic_edges"] > 0


def test_planner_budget_errors_and_weighted_edges():
    g = og.Graph.rmat(10, 16, weighted=True)
    off = np.array(g.offsets)
    with pytest.raises(og.OGError) as e:
        og.plan(g.V, g.E, off, og.WEIGHTED, budget=1000)
    assert e.value.status == 4
    p = og.plan(g.V, g.E, off, og.WEIGHTED, budget=1 << 30)
    assert p["edge_bytes"] == 8
    pr = og.plan(g.V, g.E, off, og.WEIGHTED, budget=1 << 30, flags=og.CFG_PR)
    assert pr["vertex_bytes"] > p["vertex_bytes"]
    bt = og.plan(g.V, g.E, off, og.WEIGHTED, budget=1 << 30, flags=og.CFG_BATCH)
    assert bt["vertex_bytes"] == p["vertex_bytes"] + 24 * (g.V + 1)  # three u64 masks
    # an advisek of 1.0 that leaves no staging room shrinks the static prefix
    T = g.E // 3
    q = og.plan(g.V, g.E, off, og.WEIGHTED, budget=p["vertex_bytes"] + p["fixed_bytes"] + 8 * T,
                advisek=1.0)
    assert q["chunk_edges"] >= 2048 and q["static_edges"] + 2 * q["chunk_edges"] <= T


def test_default_budget_is_reference_12GiB():
    g = og.Graph.rmat(8, 4)
    p = og.plan(g.V, g.E, g.offsets, og.PLAIN)
    assert p["budget_bytes"] == 12 << 30


def _cli(name):
    return os.path.join(og.BIN_DIR, name)


def test_cli_argument_errors(tmp_path):
    for name in ["BFS_OneGraph", "SSSP_OneGraph", "CC_OneGraph", "PR_OneGraph"]:
        assert os.access(_cli(name), os.X_OK)
    r = subprocess.run([_cli("BFS_OneGraph")], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    g = og.Graph.rmat(6, 4)
    p = str(tmp_path / "g.csr")
    g.save(p)
    r = subprocess.run([_cli("BFS_OneGraph"), "--type", "sssp", "-f", p], capture_output=True, text=True)
    assert r.returncode == 2 and "not this program" in r.stderr
    r = subprocess.run([_cli("SSSP_OneGraph"), "-type", "cc", "-f", p], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([_cli("CC_OneGraph"), "-f", str(tmp_path / "nope.csr")], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "og_graph_load" in r.stderr


def test_cli_reference_binary_names(tmp_path):
    """The reference's makefiles name the SSSP and PageRank programs
    sssp_OneGraph and PR_OneGrpah; both exist and behave as SSSP_OneGraph and
    PR_OneGraph (a --type of another algorithm is refused the same way)."""
    g = og.Graph.rmat(6, 4)
    p = str(tmp_path / "g.csr")
    g.save(p)
    for alias, name, other in [("sssp_OneGraph", "SSSP_OneGraph", "bfs"), ("PR_OneGrpah", "PR_OneGraph", "cc")]:
        assert os.access(_cli(alias), os.X_OK)
        a = subprocess.run([_cli(alias), "--type", other, "-f", p], capture_output=True, text=True)
        b = subprocess.run([_cli(name), "--type", other, "-f", p], capture_output=True, text=True)
        assert a.returncode == b.returncode == 2 and "not this program" in a.stderr


def test_bel_export_layout(tmp_path):
    g = og.Graph.rmat(8, 8, weighted=True)
    prefix = str(tmp_path / "g")
    g.save_bel(prefix)
    col = np.fromfile(prefix + ".bel.col", np.uint64)
    dst = np.fromfile(prefix + ".bel.dst", np.uint64)
    val = np.fromfile(prefix + ".bel.val", np.uint8)
    assert col[0] == g.V and col[1] == 0
    np.testing.assert_array_equal(col[2:], g.offsets[:-1])
    assert dst[0] == g.E and dst[1] == 0
    np.testing.assert_array_equal(dst[2:], g.edges[:, 0])
    assert val[:16].view(np.uint64).tolist() == [g.E, 0]
    np.testing.assert_array_equal(val[16:].view(np.uint32), g.edges[:, 1])


def test_no_static_plan_keeps_every_edge_dynamic():
    g = og.Graph.rmat(10, 16)
    p = og.plan(g.V, g.E, g.offsets, og.PLAIN, budget=1 << 30, flags=og.CFG_NO_STATIC)
    assert p["static_edges"] == 0 and p["static_vertices"] == 0 and p["dynamic_edges"] == g.E
    assert p["chunk_edges"] > 0


def decode_records(rec, E):
    """Independent decoder of the packed edge records: record e is bits
    [e*bpe, (e+1)*bpe) of the little-endian bit stream of the u32 words."""
    words, bpe, bc = rec["words"], rec["bpe"], rec["bc"]
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")
    idx = np.arange(E, dtype=np.int64)[:, None] * bpe + np.arange(bpe, dtype=np.int64)[None, :]
    vals = (bits[idx].astype(np.uint64) << np.arange(bpe, dtype=np.uint64)[None, :]).sum(axis=1)
    cols = (vals & np.uint64((1 << bc) - 1)).astype(np.uint32)
    w = (vals >> np.uint64(bc)).astype(np.uint64) + np.uint64(rec["wmin"])
    return cols, w


def test_packed_records_rmat():
    """R-MAT weights in [1, 64]: bits(V-1) column bits + 6 weight bits; the
    records decode to exactly the graph's (column, weight) pairs."""
    g = og.Graph.rmat(10, 16, weighted=True, seed=3)
    rec = g.records()
    assert rec["bc"] == 10 and rec["wmin"] == 1 and rec["bpe"] == 16
    assert rec["words"].size == (g.E * rec["bpe"] + 31) // 32 + 2
    assert (rec["words"][-2:] == 0).all()
    pairs = np.array(g.edges)
    cols, w = decode_records(rec, g.E)
    np.testing.assert_array_equal(cols, pairs[:, 0])
    np.testing.assert_array_equal(w, pairs[:, 1].astype(np.uint64))
    u = og.Graph.rmat(9, 8, seed=4)
    ru = u.records()
    assert ru["bpe"] == ru["bc"] == 9
    np.testing.assert_array_equal(decode_records(ru, u.E)[0], np.array(u.columns))


@pytest.mark.parametrize("V,wlo,whi", [(1, 7, 7), (2, 0, 1), (3, 5, 300), (200, 5, 5 + (1 << 26)),
                                       (70, 0, 0xFFFFFFFF)])
def test_packed_records_widths(V, wlo, whi):
    """Edge widths from 1 bit up to 64 bits per record (bc + bw > 33 takes
    three words), constant weights (no weight bits) and E not a multiple of 32."""
    rng = np.random.default_rng(V)
    E = 1000 + V
    off = np.sort(rng.integers(0, E + 1, V + 1)).astype(np.uint64)
    off[0], off[-1] = 0, E
    pairs = np.empty((E, 2), np.uint32)
    pairs[:, 0] = rng.integers(0, V, E)
    pairs[:, 1] = rng.integers(wlo, whi, E, endpoint=True, dtype=np.uint64)
    pairs[0, 1], pairs[1, 1] = wlo, whi
    g = og.Graph.from_arrays(off, pairs, kind=og.WEIGHTED)
    rec = g.records()
    bc = max(1, int(V - 1).bit_length())
    assert rec["bc"] == bc and rec["wmin"] == wlo
    assert rec["bpe"] == bc + int(whi - wlo).bit_length()
    cols, w = decode_records(rec, E)
    np.testing.assert_array_equal(cols, pairs[:, 0])
    np.testing.assert_array_equal(w, pairs[:, 1].astype(np.uint64))


def test_graph_plan_uses_packed_width():
    """The planner budgets bpe bits per static edge: a fixed budget holds more
    static edges than the graph-free planner's 32-bit-weight assumption."""
    g = og.Graph.rmat(10, 16, weighted=True, seed=3)
    pg = g.plan(budget=1 << 40)
    pc = og.plan(g.V, g.E, g.offsets, og.WEIGHTED, budget=1 << 40)
    assert pg["edge_bits"] == 16 and pg["stage_edge_bytes"] == 5
    assert pc["edge_bits"] == 64 and pc["stage_edge_bytes"] == 8  # the reference's sizeof(Edge)
    b = pg["vertex_bytes"] + pg["fixed_bytes"] + g.E * 4
    assert g.plan(budget=b, advisek=1.0, flags=og.CFG_DIRECT)["static_edges"] == g.E
    assert og.plan(g.V, g.E, g.offsets, og.WEIGHTED, budget=b, advisek=1.0,
                   flags=og.CFG_DIRECT)["static_edges"] <= g.E // 2
    u = og.Graph.rmat(10, 16, seed=3)
    assert u.plan(budget=1 << 40)["edge_bits"] == 10


def test_graph_plan_replace_split():
    """OG_CFG_REPLACE: the static prefix becomes the largest vertex prefix
    within half of the plain plan's static edges (the slots take the rest);
    the mode needs direct mode and both regions."""
    g = og.Graph.rmat(12, 16, weighted=True, seed=2)
    off = np.array(g.offsets)
    pg = g.plan(budget=1 << 40)
    b = pg["vertex_bytes"] + pg["fixed_bytes"] + int(0.4 * g.E * pg["edge_bits"] / 8)
    plain = g.plan(budget=b, advisek=0.6, flags=og.CFG_DIRECT)
    rep = g.plan(budget=b, advisek=0.6, flags=og.CFG_DIRECT | og.CFG_REPLACE)
    assert 0 < plain["static_edges"] < g.E
    vs = int(np.searchsorted(off, plain["static_edges"] // 2, side="right")) - 1
    assert rep["static_vertices"] == vs
    assert rep["static_edges"] == int(off[vs]) <= plain["static_edges"] // 2
    assert rep["dynamic_edges"] == g.E - rep["static_edges"]
    for k in ("budget_bytes", "vertex_bytes", "fixed_bytes", "edge_capacity", "edge_bits"):
        assert rep[k] == plain[k], k
    with pytest.raises(og.OGError) as ex:  # staged mode
        g.plan(budget=b, advisek=0.6, flags=og.CFG_REPLACE)
    assert ex.value.status == 1
    with pytest.raises(og.OGError) as ex:  # fully resident: no dynamic region
        g.plan(budget=1 << 40, advisek=1.0, flags=og.CFG_DIRECT | og.CFG_REPLACE)
    assert ex.value.status == 4


def test_graph_plan_staged_budget():
    """Staged mode: static records + two staging buffers of unpacked edges fit
    the budget's edge share."""
    g = og.Graph.rmat(11, 16, weighted=True, seed=5)
    pg = g.plan(budget=1 << 40)
    avail = int(0.5 * g.E * pg["edge_bits"] / 8)
    p = g.plan(budget=pg["vertex_bytes"] + pg["fixed_bytes"] + avail, advisek=0.8)
    assert p["dynamic_edges"] > 0 and p["chunk_edges"] > 0
    used = (p["static_edges"] * p["edge_bits"] + 7) // 8 + 2 * p["chunk_edges"] * p["stage_edge_bytes"]
    assert used <= avail


def test_convert_uint_to_ulong(tmp_path):
    """transFileUintToUlong: header and offsets kept as u32, edges widened to u64,
    output named <input minus 4 chars>lcsr."""
    rng = np.random.default_rng(0)
    V, E = 50, 300
    off = np.sort(rng.integers(0, E + 1, V)).astype(np.uint32)
    off[0] = 0
    col = rng.integers(0, V, E).astype(np.uint32)
    src = tmp_path / "g.bcsr"
    with open(src, "wb") as f:
        f.write(np.array([V, E], np.uint32).tobytes() + off.tobytes() + col.tobytes())
    og.convert_uint_to_ulong(str(src))
    raw = (tmp_path / "g.lcsr").read_bytes()
    assert len(raw) == 8 + 4 * V + 8 * E
    assert np.frombuffer(raw[:8], np.uint32).tolist() == [V, E]
    np.testing.assert_array_equal(np.frombuffer(raw[8:8 + 4 * V], np.uint32), off)
    np.testing.assert_array_equal(np.frombuffer(raw[8 + 4 * V:], np.uint64), col.astype(np.uint64))
    bad = tmp_path / "bad.bcsr"
    bad.write_bytes(np.array([V, E], np.uint32).tobytes() + off.tobytes())  # no edges
    with pytest.raises(og.OGError):
        og.convert_uint_to_ulong(str(bad), str(tmp_path / "x.lcsr"))


def test_symmetry_flag_and_exact_check():
    g = og.Graph.rmat(10, 16)  # symmetric generator: known without a check
    assert g.symmetric()
    d = og.Graph.rmat(10, 16, pagerank=True, symmetric=False)
    assert not d.symmetric()
    # loaded / built graphs are checked exactly: drop one reverse edge
    off = np.array(g.offsets)
    col = np.array(g.columns)
    assert og.Graph.from_arrays(off, col).symmetric()
    u = int(np.argmax(np.diff(off.astype(np.int64))))
    keep = np.ones(col.size, bool)
    keep[off[u]] = False  # remove u -> col[off[u]] but keep its reverse
    off2 = off.copy()
    off2[u + 1:] -= 1
    assert not og.Graph.from_arrays(off2, col[keep]).symmetric()
    # unsorted adjacency counts as not symmetric; an assertion overrides
    col3 = col.copy()
    col3[off[u]], col3[off[u] + 1] = col3[off[u] + 1], col3[off[u]]
    g3 = og.Graph.from_arrays(off, col3)
    assert not g3.symmetric()
    g4 = og.Graph.from_arrays(off, col3)
    g4.set_symmetric(True)
    assert g4.symmetric()
    w = og.Graph.rmat(9, 16, weighted=True)
    assert og.Graph.from_arrays(np.array(w.offsets), np.array(w.edges), kind=og.WEIGHTED).symmetric()


def test_transpose_is_the_reverse_graph():
    """og_graph_transpose: list u of the result holds, sorted, every v whose
    list holds u; a PageRank in-edge graph becomes its out-edge CSR, a
    symmetric graph maps to itself, a weighted graph is refused."""
    g = og.Graph.rmat(10, 16, pagerank=True, symmetric=False)
    off, col, od = np.array(g.offsets), np.array(g.columns), np.array(g.outdeg)
    t = g.transpose()
    toff, tcol = np.array(t.offsets), np.array(t.columns)
    assert t.kind == og.PLAIN and t.V == g.V and t.E == g.E
    v_of = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(off).astype(np.int64))
    order = np.lexsort((v_of, col))  # by source u, then destination v
    np.testing.assert_array_equal(tcol, v_of[order])
    np.testing.assert_array_equal(np.diff(toff), np.bincount(col, minlength=g.V))
    np.testing.assert_array_equal(np.diff(toff), od)  # the file's out-degrees
    tt = t.transpose()
    np.testing.assert_array_equal(np.array(tt.offsets), off)
    np.testing.assert_array_equal(np.array(tt.columns), col)
    s = og.Graph.rmat(9, 8)
    st = s.transpose()
    np.testing.assert_array_equal(np.array(st.offsets), np.array(s.offsets))
    np.testing.assert_array_equal(np.array(st.columns), np.array(s.columns))
    with pytest.raises(og.OGError) as ex:
        og.Graph.rmat(8, 8, weighted=True).transpose()
    assert ex.value.status == 9
