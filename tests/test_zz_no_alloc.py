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


def test_noalloc_rejects_ranges_beyond_its_scratch():
    L = og.lib()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.og_k_compact_noalloc(dummy, 0, (1 << 28) + 8193, dummy, dummy, dummy, 1, dummy, 1,
                                dummy, None)
    assert rc == 1  # OG_E_ARG
    assert "2^28" in L.og_last_error().decode()
