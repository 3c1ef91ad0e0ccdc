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
