"""Generate golden vectors of the reference's closed-form 2x2 pseudo-inverse on CPU.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_pinv_golden.py

Writes ``tests/golden/pinv2x2_cases.npz``: fp32 matrices M and the reference's
``pinv2x2(M)`` (src/diffSPH/v2/math.py:11-57), its result L and its singular values
(eigVals), on the edge cases its regularisation decides:
- well-conditioned matrices (L = M^-1);
- rank-1 matrices u v^T and the zero matrix: the smaller singular value is replaced by
  sqrt(1e-7 / 2), which exceeds the 1e-5 cut, so L is not the Moore-Penrose inverse there;
- near-singular matrices (condition 1e3-1e5), negative determinants, diagonal and
  symmetric matrices, rotations, and normalisation matrices of the size the solver sees.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from ref_harness import load_reference  # noqa: E402


def cases(rng):
    out = []
    out.append(rng.uniform(-2, 2, (64, 2, 2)))                      # general
    u, v = rng.normal(size=(32, 2)), rng.normal(size=(32, 2))
    out.append(u[:, :, None] * v[:, None, :])                        # rank 1
    out.append(np.zeros((4, 2, 2)))                                  # zero
    s = np.logspace(-5, -3, 16)                                      # near-singular
    r1, r2 = rng.uniform(0, np.pi, 16), rng.uniform(0, np.pi, 16)
    R = lambda t: np.stack([np.stack([np.cos(t), -np.sin(t)], -1), np.stack([np.sin(t), np.cos(t)], -1)], -2)
    D = np.zeros((16, 2, 2)); D[:, 0, 0] = 1.0; D[:, 1, 1] = s
    out.append(R(r1) @ D @ R(r2))
    out.append(np.array([[[0.0, 1.0], [1.0, 0.0]], [[1.0, 0.0], [0.0, -1.0]], [[-2.0, 0.5], [0.3, 1.0]]]))  # det < 0
    dg = np.zeros((8, 2, 2)); dg[:, 0, 0] = rng.uniform(0.1, 3, 8); dg[:, 1, 1] = rng.uniform(0.1, 3, 8)
    out.append(dg)                                                   # diagonal
    a = rng.uniform(-1, 1, (16, 2, 2)); out.append(a + np.swapaxes(a, 1, 2))  # symmetric
    out.append(R(rng.uniform(0, 2 * np.pi, 8)))                      # rotations
    out.append(np.eye(2)[None] + rng.uniform(-0.02, 0.02, (32, 2, 2)))  # normalisation matrices
    return np.concatenate(out).astype(np.float32)


def main():
    R = load_reference()
    from diffSPH.v2.math import pinv2x2
    M = cases(np.random.default_rng(23))
    L, ev = pinv2x2(torch.from_numpy(M))
    path = os.path.join(HERE, "pinv2x2_cases.npz")
    np.savez_compressed(path, M=M, L=L.numpy(), eigVals=ev.numpy())
    print(f"pinv2x2_cases: {M.shape[0]} matrices -> {path}")


if __name__ == "__main__":
    main()
