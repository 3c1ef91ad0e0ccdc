"""og_k_compact_noalloc: the frontier compaction for callers that cannot
allocate device memory (their scratch comes from a fixed array inside
libog.so).  Checked through the C ABI against og_k_compact, which allocates
its own scratch, on two calls in a row with different inputs so that state
left in the shared array by the first call would show in the second.  This
file is collected last so that a failure here leaves every other test run."""
import ctypes as C

import numpy as np
import pytest

import onegraph_gb300 as og

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _call(fn, bits_d, vb, ve, off_d, list_cap, tile_cap):
    lst = torch.full((list_cap,), -1, dtype=torch.int32, device="cuda")
    pref = torch.full((list_cap + 1,), -1, dtype=torch.int64, device="cuda")
    tile = torch.full((tile_cap,), -1, dtype=torch.int32, device="cuda")
    cnt = torch.full((2,), -1, dtype=torch.int64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    rc = fn(p(bits_d), vb, ve, p(off_d), p(lst), p(pref), list_cap, p(tile), tile_cap, p(cnt),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, og.lib().og_last_error()
    c = cnt.cpu().numpy().view(np.uint64)
    n = int(c[0] & 0xFFFFFFFF)
    return n, int(c[1]), lst.cpu().numpy()[:n], pref.cpu().numpy()[:n + 1], tile.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    L = og.lib()
    g = og.Graph.rmat(16, 8)
    off_d = torch.from_numpy(np.array(g.offsets).view(np.int64)).cuda()
    rng = np.random.default_rng(11)
    cases = [(0.5, 0, g.V), (0.1, 77, g.V - 33)]  # dense then sparse frontier
    results = []
    for density, vb, ve in cases:
        words = (rng.random(((g.V + 31) // 32) * 32) < density)
        bits = np.packbits(words, bitorder="little").view(np.uint32)
        bits_d = torch.from_numpy(bits.view(np.int32)).cuda()
        tile_cap = g.E // 2048 + 2
        want = _call(L.og_k_compact, bits_d, vb, ve, off_d, g.V, tile_cap)
        got = _call(L.og_k_compact_noalloc, bits_d, vb, ve, off_d, g.V, tile_cap)
        assert got[0] == want[0] and got[1] == want[1]
        for a, b in zip(got[2:], want[2:]):
            np.testing.assert_array_equal(a, b)
        results.append(got[0])
    assert results[0] != results[1]


def _model(words, vb, ve, off):
    """Listed vertices and degree prefix of [vb, ve) (as test_gpu_kernels' model)."""
    V = off.size - 1
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[:V].astype(bool)
    deg = np.diff(off.astype(np.int64))
    v = np.arange(V)
    sel = v[(v >= vb) & (v < ve) & bits & (deg > 0)]
    return sel.astype(np.uint32), np.concatenate([[0], np.cumsum(deg[sel])]).astype(np.uint64)


def test_noalloc_many_tiles_then_few_matches_model():
    """A 367-tile call, then a 2-tile call: the second must not see the first
    call's look-back state in the part of the array it does not clear."""
    L = og.lib()
    rng = np.random.default_rng(7)
    V = 3_000_017
    deg = rng.integers(0, 40, V).astype(np.uint64)
    deg[rng.random(V) < 0.2] = 0
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    words = np.packbits(rng.random(((V + 31) // 32) * 32) < 0.3, bitorder="little").view(np.uint32).copy()
    bits_d = torch.from_numpy(words.view(np.int32)).cuda()
    off_d = torch.from_numpy(off.view(np.int64)).cuda()
    E = int(off[-1])
    for vb, ve in [(0, V), (4096 * 7 + 5, 4096 * 7 + 40000)]:
        lst, pref = _model(words, vb, ve, off)
        got = _call(L.og_k_compact_noalloc, bits_d, vb, ve, off_d, V, E // 2048 + 2)
        want = _call(L.og_k_compact, bits_d, vb, ve, off_d, V, E // 2048 + 2)
        assert got[0] == lst.size and got[1] == int(pref[-1])
        np.testing.assert_array_equal(got[2].view(np.uint32), lst)
        np.testing.assert_array_equal(got[3].view(np.uint64), pref)
        for a, b in zip(got[2:], want[2:]):
            np.testing.assert_array_equal(a, b)


def test_noalloc_accepts_exactly_its_tile_limit():
    """2^28 vertices from vertex 0 is 8192 tiles, the limit: accepted (a few
    vertices with one edge each, the rest without edges)."""
    L = og.lib()
    V = 1 << 28
    rng = np.random.default_rng(3)
    hot = np.unique(rng.integers(0, V, 2000))
    deg = torch.zeros(V, dtype=torch.int64, device="cuda")
    deg[torch.from_numpy(hot).cuda()] = 1
    off_d = torch.cat([torch.zeros(1, dtype=torch.int64, device="cuda"), torch.cumsum(deg, 0)])
    del deg
    bits_d = torch.full(((V + 31) // 32,), -1, dtype=torch.int32, device="cuda")  # every vertex active
    got = _call(L.og_k_compact_noalloc, bits_d, 0, V, off_d, hot.size + 1, hot.size // 2048 + 4)
    assert got[0] == hot.size and got[1] == hot.size
    np.testing.assert_array_equal(got[2].view(np.uint32), hot.astype(np.uint32))
    del bits_d, off_d
    torch.cuda.empty_cache()


def test_noalloc_rejects_ranges_beyond_its_scratch():
    L = og.lib()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.og_k_compact_noalloc(dummy, 0, (1 << 28) + 8193, dummy, dummy, dummy, 1, dummy, 1,
                                dummy, None)
    assert rc == 1  # OG_E_ARG
    assert "2^28" in L.og_last_error().decode()
    # 2^28 vertices not starting on a 32-vertex word boundary need 8193 tiles
    rc = L.og_k_compact_noalloc(dummy, 5, (1 << 28) + 5, dummy, dummy, dummy, 1, dummy, 1, dummy, None)
    assert rc == 1
