"""CPU checks of the learned-layer oracle (no GPU): the transposed aggregation is the exact
adjoint of the aggregation (both forms), the basis has the stated properties, and the
bfloat16 rounding is round-to-nearest-even."""
import numpy as np
import pytest

from oracle import cconv_oracle as CO


def _case(n=48, H=0.55, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 2))
    dom = {"min": [-1.0, -1.0], "max": [1.0, 1.0], "periodic": [True, True]}
    rows = []
    for i in range(n):
        d = CO.min_image(x[i] - x, dom["min"], dom["max"], dom["periodic"])
        rows.append(np.where(np.linalg.norm(d, axis=1) <= H)[0])
    off = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int64)
    return x, off, np.concatenate(rows), dom, H


@pytest.mark.parametrize("relative", [False, True])
@pytest.mark.parametrize("C", [16, 64])
def test_transpose_is_the_adjoint(relative, C):
    x, off, nbr, dom, H = _case()
    rng = np.random.default_rng(1)
    h = rng.standard_normal((x.shape[0], C))
    G = rng.standard_normal((x.shape[0], 64 * C))
    E = CO.aggregate(x, off, nbr, dom, H, 0.07, h, relative)
    dh = CO.aggregate_t(x, off, nbr, dom, H, 0.07, G, C, relative)
    a, b = float(np.sum(E * G)), float(np.sum(h * dh))
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)


def test_basis_properties():
    H = 0.5
    phi0 = CO.basis(np.zeros((1, 2)), H)[0]
    # self pair: only the angular-order-0 terms survive, T_a(-1) = (-1)^a
    for a in range(8):
        assert phi0[8 * a] == pytest.approx((-1.0) ** a)
        assert np.all(phi0[8 * a + 1:8 * a + 8] == 0.0)
    # the window vanishes at the support radius
    assert np.abs(CO.basis(np.array([[H, 0.0], [0.0, -H]]), H)).max() < 1e-12
    # parity under x -> -x: odd angular terms F_1, F_2, F_5, F_6 flip sign
    rng = np.random.default_rng(2)
    v = rng.uniform(-0.3, 0.3, (20, 2))
    p, m = CO.basis(v, H), CO.basis(-v, H)
    for b in range(64):
        sg = -1.0 if (b % 8) in (1, 2, 5, 6) else 1.0
        assert np.allclose(m[:, b], sg * p[:, b])


def test_bf16_rounding():
    vals = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.14159265], np.float32)
    got = CO.bf16(vals)
    assert got[0] == 1.0
    assert got[1] == 1.0                       # tie to even
    assert got[2] == np.float32(1.0 + 2.0 ** -6)  # tie to even (upwards)
    assert got[3] == -2.5
    assert got[4] == np.float32(3.140625)
