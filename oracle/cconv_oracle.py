"""CPU oracle of the learned continuous-convolution layer (test infrastructure only).

Parity unpinned: the network has no reference implementation (the reference project has
no learned model; the continuous-convolution code it builds on is a separate package that
is not part of it). This restates, in numpy float64, the layer the sm_103a kernels
implement, so that the kernels (aggregation, its transpose, the tcgen05 contraction) and the
layer gradients can be checked against an independent computation:

    E_i[b C + c] = inv_norm * sum_{j in N(i)} phi_b(x_i - x_j) h_j[c]
                   (relative form: h_j[c] - h_i[c] in place of h_j[c])
    y_i          = E_i W                                   (W: [64 C, C_out])
    phi_{8a+m}(x) = (1 - q^2)^2 T_a(2q - 1) F_m(x / (|x| + 1e-6 H)),  q = min(|x| / H, 1)
    F = (1, Re z, Im z, Re z^2, Im z^2, Re z^3, Im z^3, Re z^4)

Backward: dW = E^T dy, dE = dy W^T, dh_j = inv_norm * sum_{i in N(j)} phi(x_i - x_j)^T dE_i.
``bf16`` rounds like the GPU path (round to nearest even), so the oracle can reproduce the
points where the kernels round their operands.
"""
from __future__ import annotations

import numpy as np

BASIS = 64


def bf16(a):
    """Round to bfloat16 (nearest even) and return float32 values."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    b = a32.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).reshape(a32.shape)


def min_image(d, lo, hi, periodic):
    """Minimum-image pair vectors for a box [lo, hi] with periodic axes."""
    d = np.array(d, dtype=np.float64)
    for a in range(2):
        if periodic[a]:
            ext = hi[a] - lo[a]
            d[:, a] -= ext * np.round(d[:, a] / ext)
    return d


def basis(xv, H):
    """phi_b(x) for pair vectors xv [E, 2] -> [E, 64] (float64)."""
    xv = np.asarray(xv, np.float64)
    r = np.sqrt(np.sum(xv * xv, axis=1))
    q = np.minimum(r / H, 1.0)
    w = (1.0 - q * q) ** 2
    s = 2.0 * q - 1.0
    T = [np.ones_like(s), s]
    for _ in range(2, 8):
        T.append(2.0 * s * T[-1] - T[-2])
    inv = 1.0 / (r + 1e-6 * H)
    z = (xv[:, 0] + 1j * xv[:, 1]) * inv
    F = [np.ones_like(s), z.real, z.imag, (z ** 2).real, (z ** 2).imag, (z ** 3).real, (z ** 3).imag, (z ** 4).real]
    out = np.empty((xv.shape[0], BASIS))
    for a in range(8):
        for m in range(8):
            out[:, 8 * a + m] = w * T[a] * F[m]
    return out


def edges(x, offsets, nbr, domain, sign=1.0):
    """Row index, column index and pair vectors sign * (x_row - x_col) of a CSR list."""
    offsets = np.asarray(offsets, np.int64)
    n = offsets.shape[0] - 1
    rows = np.repeat(np.arange(n), np.diff(offsets))
    cols = np.asarray(nbr, np.int64)
    x = np.asarray(x, np.float64)
    d = min_image(x[rows] - x[cols], domain["min"], domain["max"], domain["periodic"])
    return rows, cols, sign * d


def aggregate(x, offsets, nbr, domain, H, inv_norm, h, relative=False, round_operands=False):
    """E [n, 64 C] from features h [n, C] (float64). round_operands rounds the basis values
    and the (difference) features to bf16 first, as the tensor-core kernel does."""
    rows, cols, d = edges(x, offsets, nbr, domain)
    phi = basis(d, H)
    n, C = h.shape
    h = np.asarray(h, np.float64)
    hv = h[cols] - h[rows] if relative else h[cols]
    if round_operands:
        phi = bf16(phi).astype(np.float64)
        hv = bf16(hv).astype(np.float64)
    E = np.zeros((n, BASIS, C))
    np.add.at(E, rows, phi[:, :, None] * hv[:, None, :])
    return (E * inv_norm).reshape(n, BASIS * C)


def aggregate_t(x, offsets, nbr, domain, H, inv_norm, dE, C, relative=False):
    """dh [n, C] = transpose of ``aggregate`` applied to dE [n, 64 C] (symmetric lists)."""
    rows, cols, d = edges(x, offsets, nbr, domain, sign=-1.0)  # row j lists i; phi(x_i - x_j)
    phi = basis(d, H)
    n = offsets.shape[0] - 1 if hasattr(offsets, "shape") else len(offsets) - 1
    dEr = np.asarray(dE, np.float64).reshape(-1, BASIS, C)
    contrib = np.einsum("eb,ebc->ec", phi, dEr[cols])
    dh = np.zeros((n, C))
    np.add.at(dh, rows, contrib)
    if relative:  # own term: -sum_b dE_j[b] sum_{i in N(j)} phi_b(x_j - x_i)
        S = np.zeros((n, BASIS))
        np.add.at(S, rows, basis(-d, H))
        dh -= np.einsum("nb,nbc->nc", S, dEr[:n])
    return dh * inv_norm


def layer_forward(x, offsets, nbr, domain, H, inv_norm, h, W, round_like_gpu=True, relative=False):
    """y = aggregate(h) W, rounding h, the aggregation operands (tensor-core kernel), E and
    W to bf16 where the GPU path does."""
    hq = bf16(h) if round_like_gpu else h
    E = aggregate(x, offsets, nbr, domain, H, inv_norm, np.asarray(hq, np.float64), relative,
                  round_operands=round_like_gpu)
    Eq = bf16(E).astype(np.float64) if round_like_gpu else E
    Wq = bf16(W).astype(np.float64) if round_like_gpu else np.asarray(W, np.float64)
    return Eq @ Wq, Eq


def layer_backward(x, offsets, nbr, domain, H, inv_norm, Eq, W, dy, C, round_like_gpu=True, relative=False):
    """(dh, dW) of the layer for the upstream gradient dy [n, C_out]."""
    dyq = bf16(dy).astype(np.float64) if round_like_gpu else np.asarray(dy, np.float64)
    Wq = bf16(W).astype(np.float64) if round_like_gpu else np.asarray(W, np.float64)
    dW = Eq.T @ dyq
    dE = dyq @ Wq.T
    dh = aggregate_t(x, offsets, nbr, domain, H, inv_norm, dE, C, relative)
    return dh, dW
