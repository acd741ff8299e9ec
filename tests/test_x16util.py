"""The X16 layout helpers of the tests round-trip (CPU)."""
import numpy as np

from x16util import phys_index, swizzle_x16, unswizzle_x16


def test_swizzle_round_trip():
    rng = np.random.default_rng(0)
    for ne, nch, nsp in [(3, 2, 33), (17, 4, 64), (40, 1, 100)]:
        X = rng.integers(-127, 128, size=(nch, nsp, ne, 2)).astype(np.float32)
        nep = (ne + 15) // 16 * 16
        buf = swizzle_x16(X, nep)
        nkc = (nsp + 31) // 32
        assert buf.size == nkc * nch * nep * 128
        assert np.array_equal(unswizzle_x16(buf, nch, nsp, ne, nep), X)
        # chunk-major: the first 32 spectra of every channel come first
        rows = buf.view(np.float16).reshape(nkc, nch, nep, 64)
        assert rows[0, 0, 0, phys_index(np.arange(1), 0)[0]] == X[0, 0, 0, 0]
