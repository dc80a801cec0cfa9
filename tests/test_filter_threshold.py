"""The fused passes test pair inclusion as s <= T, with s = fma(y, y, x*x) in fp32 and T the
largest fp32 value whose correctly rounded sqrt divided by h rounds to <= 1. This checks,
exhaustively over a window of fp32 values around h^2, that the comparison equals the
reference's test fl(fl(sqrt(s)) / h) <= 1 (src/diffSPH/v2/modules/neighborhood.py:451-456)."""
import numpy as np
import pytest


def threshold(h):
    h = np.float32(h)

    def ok(s):
        return np.float32(np.sqrt(np.float32(s))) / h <= np.float32(1.0)

    s = np.float32(h * h)
    while not ok(s):
        s = np.nextafter(s, np.float32(0))
    while ok(np.nextafter(s, np.float32(np.inf))):
        s = np.nextafter(s, np.float32(np.inf))
    return s


@pytest.mark.parametrize("h", [0.5, 0.125, 4.0 / 1024, 4.0 / 256, 0.37, 1e-3 * 3.3, 17.25])
def test_threshold_equals_reference_test(h):
    T = threshold(h)
    hh = np.float32(h) * np.float32(h)
    base = hh.view(np.int32)
    bits = np.arange(base - 200000, base + 200000, dtype=np.int32)
    s = bits.view(np.float32)
    ref = (np.sqrt(s).astype(np.float32) / np.float32(h)).astype(np.float32) <= np.float32(1.0)
    assert np.array_equal(s <= T, ref)
