"""Generate golden vectors of the reference's implicit particle shifting (IPS) on CPU.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_ips_golden.py

Writes ``tests/golden/ips_<case>.npz``: the input particle arrays, the configuration
(JSON) and the reference's output of ``solveShifting`` (src/diffSPH/v2/modules/shifting.py:
882-1019) with ``shifting.scheme = 'IPS'`` (``computeShifting`` :780-880, BiCGStab
``bicgstab_shifting`` :322-493 on the matrices of ``getShiftingMatrices`` :611-705), and
the solve's iteration count and status. All other shifting parameters are the reference's
defaults (rtol 1e-4, 64 iterations, solver threshold dx / 2, zero initial guess, no
free-surface handling).
"""
import copy
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from make_golden import reference_config, to_torch_state, npy  # noqa: E402
from ref_harness import load_reference  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402

torch.set_num_threads(min(8, os.cpu_count() or 1))


def run_case(R, name, cfg, st):
    cfg = copy.deepcopy(cfg)
    cfg["shifting"]["scheme"] = "IPS"
    rc = reference_config(R, cfg)
    rc["shifting"]["scheme"] = "IPS"
    out = {"config_json": np.frombuffer(json.dumps(cfg).encode(), dtype=np.uint8)}
    for part, arrs in st.items():
        for k, v in arrs.items():
            out[f"in/{part}/{k}"] = v
    state = {p: to_torch_state(v) for p, v in st.items()}
    # the solve's statistics, recorded from inside the reference's own call
    stats = {}
    orig = R.shifting.computeShifting

    def recording(*a, **k):
        res = orig(*a, **k)
        stats["iterations"] = int(res[6])
        stats["residual"] = float(res[7])
        stats["B"] = npy(res[4])
        return res

    R.shifting.computeShifting = recording
    try:
        dx, _ = R.shifting.solveShifting(copy.deepcopy(state), rc)
    finally:
        R.shifting.computeShifting = orig
    out["ips/shift"] = npy(dx)
    out["ips/B"] = stats["B"]
    out["ips/iterations"] = np.array(stats["iterations"])
    out["ips/residual"] = np.array(stats["residual"])
    path = os.path.join(HERE, f"ips_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"ips_{name}: fluid {st['fluid']['positions'].shape[0]}, iterations {stats['iterations']}, "
          f"residual {stats['residual']:.3e}, max |dx| {np.abs(out['ips/shift']).max():.3e} -> {path}")


def main():
    R = load_reference()
    # jittered periodic flow (a lattice has J = 0 and returns at once)
    cfg, st = scenes.taylor_green(24, jitter=0.1, seed=7)
    run_case(R, "tgv24_jitter", cfg, st)
    cfg, st = scenes.fourier_periodic(20, seed=3)
    run_case(R, "fourier20", cfg, st)
    # walls: wall rows are excluded from the system
    cfg, st = scenes.dam_break(dx=1.0 / 16)
    run_case(R, "dambreak16", cfg, st)


if __name__ == "__main__":
    main()
