"""Golden vectors of the reference's pair operators (sphOperationStates, src/diffSPH/v2/sphOps.py:
278-303) on the jittered periodic case ``tgv24_jitter_wrap`` (its stored reference neighborhood).

Run in the development container with the reference's source tree:

    DIFFSPH_REF_SRC=<reference checkout>/src python tests/golden/make_ops_golden.py

Writes ``tests/golden/ops_tgv24.npz``: for every operation and mode the GPU operator
(diffsph_gb300.ops, sph_operation) implements, the reference's output on the same inputs
(scalar, 2-vector, 2x2-matrix and per-pair quantities).
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

from golden_io import load_case  # noqa: E402
from ref_harness import load_reference  # noqa: E402


def quantities(st):
    """The fields the operators act on (fixed, seeded)."""
    fl = st["fluid"]
    n = fl["positions"].shape[0]
    rng = np.random.default_rng(5)
    mat = rng.normal(size=(n, 2, 2)).astype(np.float32)
    pres = (rng.normal(size=n) * 10).astype(np.float32)
    return {"rho": fl["densities"], "u": fl["velocities"], "p": pres, "mat": mat}


def cases():
    """(name, operation, gradientMode, divergenceMode, quantity key or 'pair')."""
    out = [("density", "density", "naive", "div", None)]
    for q in ("rho", "u", "pair"):
        out.append((f"interpolate_{q}", "interpolate", "naive", "div", q))
    for mode in ("naive", "difference", "summation", "symmetric"):
        for q in ("p", "u"):
            out.append((f"gradient_{mode}_{q}", "gradient", mode, "div", q))
        out.append((f"divergence_{mode}_u", "divergence", mode, "div", "u"))
        out.append((f"curl_{mode}_u", "curl", mode, "div", "u"))
        for dm in ("div", "dot"):
            out.append((f"divergence_{mode}_mat_{dm}", "divergence", mode, dm, "mat"))
    out.append(("gradient_pair", "gradient", "difference", "div", "pair"))
    out.append(("divergence_pair", "divergence", "difference", "div", "pair"))
    out.append(("laplacian_p", "laplacian", "difference", "div", "p"))
    for t in ("difference", "conserving", "divergenceFree", "dot"):
        out.append((f"laplacian_{t}_u", "laplacian", t, "div", "u"))
    return out


def main():
    R = load_reference()
    z, cfg, st = load_case("tgv24_jitter_wrap")
    fl = {k: torch.from_numpy(np.ascontiguousarray(v)) for k, v in st["fluid"].items()}
    fl["numParticles"] = fl["positions"].shape[0]
    nb = {"indices": (torch.from_numpy(z["nb/i"]), torch.from_numpy(z["nb/j"]))}
    for k in ("distances", "vectors", "supports", "kernels", "gradients", "numNeighbors", "neighborOffsets"):
        nb[k] = torch.from_numpy(z[f"nb/{k}"])
    qs = {k: torch.from_numpy(v) for k, v in quantities(st).items()}
    pair_q = -(nb["distances"] * nb["supports"]).view(-1, 1) * nb["vectors"]
    out = {}
    for name, op, mode, dm, q in cases():
        quant = None if q is None else (pair_q if q == "pair" else (qs[q], qs[q]))
        r = R.sphOps.sphOperationStates(fl, fl, quant, nb, operation=op, gradientMode=mode, divergenceMode=dm)
        out[f"out/{name}"] = r.numpy()
    np.savez_compressed(os.path.join(HERE, "ops_tgv24.npz"), **out)
    print(f"{len(out)} operator outputs -> ops_tgv24.npz")


if __name__ == "__main__":
    main()
