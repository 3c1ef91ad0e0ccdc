"""Kernel-level launchers of libog.so on caller-owned device buffers."""
import ctypes as C

import numpy as np
import pytest

import onegraph_gb300 as og

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def compact_model(bits_words, vb, ve, off):
    """Active vertices of [vb, ve) with edges, degree prefix and 2048-tile map."""
    V = off.size - 1
    bits = np.unpackbits(bits_words.view(np.uint8), bitorder="little")[:V].astype(bool)
    deg = np.diff(off.astype(np.int64))
    v = np.arange(V)
    sel = v[(v >= vb) & (v < ve) & bits & (deg > 0)]
    pref = np.concatenate([[0], np.cumsum(deg[sel])]).astype(np.uint64)
    total = int(pref[-1])
    ntiles = (total + 2047) // 2048
    tiles = np.searchsorted(pref[1:], np.arange(ntiles, dtype=np.uint64) * 2048, side="right")
    return sel.astype(np.uint32), pref, tiles.astype(np.uint32)


def dptr(t):
    return C.c_void_p(t.data_ptr())


def run_compact(bits_d, vb, ve, off_d, list_cap, tile_cap):
    lst = torch.zeros(max(list_cap, 1), dtype=torch.int32, device="cuda")
    pref = torch.zeros(max(list_cap, 1) + 1, dtype=torch.int64, device="cuda")
    tile = torch.zeros(max(tile_cap, 1), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    rc = og.lib().og_k_compact(dptr(bits_d), vb, ve, dptr(off_d), dptr(lst), dptr(pref), list_cap,
                               dptr(tile), tile_cap, dptr(cnt),
                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    c = cnt.cpu().numpy().view(np.uint64)
    n, total = int(c[0] & 0xFFFFFFFF), int(c[1])
    return rc, n, total, (lst.cpu().numpy().view(np.uint32), pref.cpu().numpy().view(np.uint64),
                          tile.cpu().numpy().view(np.uint32))


def test_compact_matches_model():
    g = og.Graph.rmat(16, 8)
    off = np.array(g.offsets)
    V = g.V
    rng = np.random.default_rng(0)
    words = rng.integers(0, 1 << 32, (V + 31) // 32, dtype=np.uint64).astype(np.uint32)
    words &= rng.integers(0, 1 << 32, words.size, dtype=np.uint64).astype(np.uint32)  # ~25% dense
    bits_d = torch.from_numpy(words.view(np.int32)).cuda()
    off_d = torch.from_numpy(off.view(np.int64)).cuda()
    for vb, ve in [(0, V), (37, V - 5), (1000, 1001), (V // 3, 2 * V // 3 + 17), (5, 5)]:
        lst, pref, tiles = compact_model(words, vb, ve, off)
        rc, n, total, (glist, gpref, gtile) = run_compact(bits_d, vb, ve, off_d, V, g.E // 2048 + 2)
        assert rc == 0, og.lib().og_last_error()
        assert n == lst.size and total == int(pref[-1])
        np.testing.assert_array_equal(glist[:n], lst)
        np.testing.assert_array_equal(gpref[:n + 1], pref)
        np.testing.assert_array_equal(gtile[:tiles.size], tiles)


@pytest.mark.parametrize("density", [0.0005, 0.1, 1.0])
def test_compact_many_tiles(density):
    """About 367 look-back tiles (3M vertices, 8192 per tile): the warp-wide
    look-back crosses many 32-tile windows, with sparse tiles of zero
    aggregate and dense ones."""
    rng = np.random.default_rng(7)
    V = 3_000_017
    deg = rng.integers(0, 40, V).astype(np.uint64)
    deg[rng.random(V) < 0.2] = 0
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    bits = rng.random(((V + 31) // 32) * 32) < density
    words = np.packbits(bits, bitorder="little").view(np.uint32).copy()
    bits_d = torch.from_numpy(words.view(np.int32)).cuda()
    off_d = torch.from_numpy(off.view(np.int64)).cuda()
    E = int(off[-1])
    for vb, ve in [(0, V), (12345, V - 77)]:
        lst, pref, tiles = compact_model(words, vb, ve, off)
        rc, n, total, (glist, gpref, gtile) = run_compact(bits_d, vb, ve, off_d, V, E // 2048 + 2)
        assert rc == 0, og.lib().og_last_error()
        assert n == lst.size and total == int(pref[-1])
        np.testing.assert_array_equal(glist[:n], lst)
        np.testing.assert_array_equal(gpref[:n + 1], pref)
        np.testing.assert_array_equal(gtile[:tiles.size], tiles)


def test_compact_reports_small_capacity():
    g = og.Graph.rmat(12, 8)
    off_d = torch.from_numpy(np.array(g.offsets).view(np.int64)).cuda()
    words = np.full((g.V + 31) // 32, 0xFFFFFFFF, np.uint32)
    bits_d = torch.from_numpy(words.view(np.int32)).cuda()
    rc, *_ = run_compact(bits_d, 0, g.V, off_d, 10, g.E // 2048 + 2)
    assert rc == 10  # OG_E_DEVICE: the kernel's own capacity checks, nothing written past the end
    rc, *_ = run_compact(bits_d, 0, g.V, off_d, g.V, 1)
    assert rc == 10


def _records(g):
    r = g.records()
    words_d = torch.from_numpy(np.ascontiguousarray(r["words"]).view(np.int32)).cuda()
    rec = og.KRecords(words_d.data_ptr(), g.E, r["bpe"], r["bc"], r["wmin"], 0)
    return rec, words_d


def _frontier(g, density, seed):
    """A compacted frontier built by the numpy model (independent of
    og_k_compact): listed vertices, degree prefix, tile map, on the device."""
    off = np.array(g.offsets)
    rng = np.random.default_rng(seed)
    words = np.packbits(rng.random(((g.V + 31) // 32) * 32) < density, bitorder="little").view(np.uint32)
    lst, pref, tiles = compact_model(words, 0, g.V, off)
    dev = [torch.from_numpy(a.view(np.int32 if a.dtype == np.uint32 else np.int64).copy()).cuda()
           for a in (lst, pref, np.concatenate([tiles, [0]]).astype(np.uint32))]
    return off, lst, pref, dev


def _bits(vs, V):
    b = np.zeros(((V + 31) // 32) * 32, bool)
    b[vs] = True
    return np.packbits(b, bitorder="little").view(np.uint32)


@pytest.mark.parametrize("algo", [og.ALGO_BFS, og.ALGO_SSSP, og.ALGO_CC])
def test_relax_launcher_matches_model(algo):
    """og_k_relax on a caller-built frontier against a numpy model of one
    round.  Listed vertices carry values no edge can lower, so the result of
    the concurrent relax is the same as the sequential model's."""
    g = og.Graph.rmat(13, 16, weighted=True, seed=5)
    V = g.V
    off, lst, pref, (lst_d, pref_d, tile_d) = _frontier(g, 0.05, 3)
    pairs = np.array(g.edges)
    rng = np.random.default_rng(11)
    rec, words_d = _records(g)
    if algo == og.ALGO_BFS:
        value = rng.integers(1, 9, V).astype(np.uint32)
        visited = rng.random(V) < 0.3
        visited[lst] = True
    elif algo == og.ALGO_SSSP:
        value = np.where(rng.random(V) < 0.5, 0xFFFFFFFF, rng.integers(50, 200, V)).astype(np.uint32)
        value[lst] = 40  # + weight >= 41 > 40: listed values cannot drop
        visited = None
    else:
        value = rng.integers(100, 1000, V).astype(np.uint32)
        value[lst] = 60
        visited = None
    want, nxt = value.copy(), np.zeros(V, bool)
    vis = None if visited is None else visited.copy()
    for u in lst:
        for e in range(int(off[u]), int(off[u + 1])):
            v, w = int(pairs[e, 0]), int(pairs[e, 1])
            if algo == og.ALGO_BFS:
                if not vis[v]:
                    vis[v] = True
                    nxt[v] = True
                    want[v] = 7 + 1
            else:
                cand = int(value[u]) + (w if algo == og.ALGO_SSSP else 0)
                if cand < want[v]:
                    want[v] = cand
                    nxt[v] = True
    value_d = torch.from_numpy(value.view(np.int32).copy()).cuda()
    next_d = torch.zeros((V + 31) // 32, dtype=torch.int32, device="cuda")
    vis_d = None if visited is None else torch.from_numpy(_bits(np.nonzero(visited)[0], V).view(np.int32)).cuda()
    off_d = torch.from_numpy(off.view(np.int64)).cuda()
    rc = og.lib().og_k_relax(algo, dptr(lst_d), dptr(pref_d), dptr(tile_d), lst.size, int(pref[-1]), dptr(off_d),
                             C.byref(rec), V, dptr(value_d), dptr(next_d), dptr(vis_d) if vis_d is not None else None,
                             7, None)
    assert rc == 0, og.lib().og_last_error()
    np.testing.assert_array_equal(value_d.cpu().numpy().view(np.uint32), want)
    np.testing.assert_array_equal(next_d.cpu().numpy().view(np.uint32), _bits(np.nonzero(nxt)[0], V))
    if vis is not None:
        np.testing.assert_array_equal(vis_d.cpu().numpy().view(np.uint32), _bits(np.nonzero(vis)[0], V))


@pytest.mark.parametrize("weights", [True, False])
def test_gather_launcher_matches_model(weights):
    """og_k_gather: the edges at positions [b, e) of a compacted list, in list
    order, unpacked from the records (the dynamic-region gather)."""
    g = og.Graph.rmat(13, 16, weighted=True, seed=9)
    off, lst, pref, (lst_d, pref_d, tile_d) = _frontier(g, 0.2, 4)
    pairs = np.array(g.edges)
    order = np.concatenate([np.arange(off[u], off[u + 1]) for u in lst]).astype(np.int64)
    rec, words_d = _records(g)
    off_d = torch.from_numpy(off.view(np.int64)).cuda()
    total = int(pref[-1])
    assert total > 4096 * 3
    for b, e in [(0, total), (2048, 2048 * 5), (4096 * 3, total)]:
        col = torch.zeros(max(e - b, 1), dtype=torch.int32, device="cuda")
        w = torch.zeros(max(e - b, 1), dtype=torch.int32, device="cuda") if weights else None
        rc = og.lib().og_k_gather(dptr(lst_d), dptr(pref_d), dptr(tile_d), lst.size, total, dptr(off_d), C.byref(rec),
                                  b, e, dptr(col), dptr(w) if weights else None, None)
        assert rc == 0, og.lib().og_last_error()
        np.testing.assert_array_equal(col.cpu().numpy()[:e - b].view(np.uint32), pairs[order[b:e], 0])
        if weights:
            np.testing.assert_array_equal(w.cpu().numpy()[:e - b].view(np.uint32), pairs[order[b:e], 1])
    col = torch.zeros(8, dtype=torch.int32, device="cuda")
    assert og.lib().og_k_gather(dptr(lst_d), dptr(pref_d), dptr(tile_d), lst.size, total, dptr(off_d), C.byref(rec),
                                100, total, dptr(col), None, None) == 1  # start not on a 2048 boundary
    assert og.lib().og_k_gather(dptr(lst_d), dptr(pref_d), dptr(tile_d), lst.size, total, dptr(off_d), C.byref(rec),
                                0, 2048 + 17, dptr(col), None, None) == 1  # end inside a tile


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_waits_give_up_and_report_timeout(which):
    """The compaction look-back (0) and the persistent kernel's grid barrier
    (1) on a signal nothing gives: the wait ends after its poll limit, the
    call returns OG_E_TIMEOUT, and the GPU stays usable."""
    rc = og.lib().og_k_wait_check(which, 2000)
    assert rc == 6, og.lib().og_last_error()  # OG_E_TIMEOUT
    assert b"gave up" in og.lib().og_last_error()
    x = torch.arange(1000, device="cuda").sum().item()  # the context still works
    assert x == 499500


def test_link_probe_modes():
    """og_link_probe: SM reads, one and two DMA copies of a page-locked buffer
    all report a positive rate; an unpinned buffer is refused."""
    buf = torch.empty(64 << 20, dtype=torch.uint8, pin_memory=True)
    rates = [og.link_probe(buf, m, 2) for m in (0, 1, 2)]
    assert all(r > 1.0 for r in rates), rates
    plain = torch.empty(64 << 20, dtype=torch.uint8)
    with pytest.raises(og.OGError):
        og.link_probe(plain, 0, 1)
