"""The device exclusive scan behind every radix sort (hierarchy build,
edge-sample queue, deterministic reduction), against numpy.

The scan runs in one block for up to one tile of 16,384 counters and over
several blocks (one per tile, then a pass adding the totals of earlier
tiles) beyond that.  The library's own sorts scan whole tiles (256 digits x
a fixed grid), so the sizes here also cover the partial last tile and the
16-counter groups that straddle its end."""
import ctypes as C

import numpy as np
import pytest

from diffrender_tutorials_gb300 import native as N

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 15, 16, 17, 1000, 16383, 16384, 16385, 40000, 131072, 131072 + 7, 1 << 20])
def test_exclusive_scan_matches_numpy(n):
    lib = N.load()
    rng = np.random.default_rng(n)
    counts = rng.integers(0, 1000, size=n, dtype=np.uint32)
    out = np.zeros(n, np.uint32)
    N.check(lib.drgb_debug_exclusive_scan(C.c_void_p(counts.ctypes.data), n, C.c_void_p(out.ctypes.data)))
    ref = np.concatenate([[0], np.cumsum(counts.astype(np.uint64))[:-1]]).astype(np.uint32)
    assert np.array_equal(out, ref), int(np.flatnonzero(out != ref)[0])
