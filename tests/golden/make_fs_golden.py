"""Generate golden vectors of the reference's free-surface shifting on CPU.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_fs_golden.py

Writes ``tests/golden/fs_<case>.npz``: the input particle arrays, the configuration (JSON)
and the reference's ``solveShifting`` (src/diffSPH/v2/modules/shifting.py:882-1019) with
``shifting.freeSurface = True`` and the reference's defaults for everything else (surface
detection 'Barcasco', normals 'lambda', projection 'mat', mask expansion 2 iterations,
surface scaling 0.1), for the delta+ and the IPS scheme. Besides the shift it records, on
the merged fluid + wall particle set, the intermediates of that call:
``detectFreeSurfaceBarecasco`` (src/diffSPH/v2/modules/surfaceDetection.py:95-107),
``expandFreeSurfaceMask`` (:54-63), ``computeNormalsMaronne`` (:41-52) with its
normalization-matrix eigenvalues, and the normalised ``computeLambdaGrad``
(shifting.py:151-171).
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


def run_case(R, name, cfg, st, scheme):
    cfg = copy.deepcopy(cfg)
    cfg["shifting"]["scheme"] = scheme
    cfg["shifting"]["freeSurface"] = True
    rc = reference_config(R, cfg)
    rc["shifting"]["scheme"] = scheme
    rc["shifting"]["freeSurface"] = True
    out = {"config_json": np.frombuffer(json.dumps(cfg).encode(), dtype=np.uint8)}
    for part, arrs in st.items():
        for k, v in arrs.items():
            out[f"in/{part}/{k}"] = v
    state = {p: to_torch_state(v) for p, v in st.items()}
    rec = {}
    sh = R.shifting
    originals = {k: getattr(sh, k) for k in ("detectFreeSurfaceBarecasco", "expandFreeSurfaceMask",
                                            "computeNormalsMaronne", "computeLambdaGrad")}

    def wrap(key, fn):
        def f(*a, **k):
            res = fn(*a, **k)
            rec.setdefault(key, res)
            if key == "computeNormalsMaronne":
                rec.setdefault("L.EVs", a[0]["L.EVs"])
            return res
        return f

    for k, fn in originals.items():
        setattr(sh, k, wrap(k, fn))
    try:
        dx, _ = sh.solveShifting(copy.deepcopy(state), rc)
    finally:
        for k, fn in originals.items():
            setattr(sh, k, fn)
    out["fs/shift"] = npy(dx)
    out["fs/freeSurface"] = npy(rec["detectFreeSurfaceBarecasco"])
    out["fs/freeSurfaceMask"] = npy(rec["expandFreeSurfaceMask"])
    out["fs/normalsMaronne"] = npy(rec["computeNormalsMaronne"][0])
    out["fs/Lambdas"] = npy(rec["computeNormalsMaronne"][1])
    out["fs/eigenvalues"] = npy(rec["L.EVs"])
    out["fs/lambdaGrad"] = npy(rec["computeLambdaGrad"])
    path = os.path.join(HERE, f"fs_{name}.npz")
    np.savez_compressed(path, **out)
    n = out["fs/freeSurface"]
    print(f"fs_{name}: particles {n.shape[0]}, surface {int(n.sum())}, mask {int(out['fs/freeSurfaceMask'].sum())}, "
          f"max |dx| {np.abs(out['fs/shift']).max():.3e} -> {path}")


def _moving(cfg, st, seed, jitter):
    """A dam-break state in motion (delta+ shifts scale with the Mach number, zero at rest),
    optionally with the fluid lattice jittered so that the surface is not lattice-aligned."""
    rng = np.random.default_rng(seed)
    st = copy.deepcopy(st)
    dx = float(cfg["particle"]["dx"])
    fl = st["fluid"]
    fl["velocities"] = rng.uniform(-1.0, 1.0, fl["velocities"].shape).astype(np.float32)
    if jitter:
        fl["positions"] += (rng.uniform(-jitter, jitter, fl["positions"].shape) * dx).astype(np.float32)
    return st


def main():
    R = load_reference()
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    st = _moving(cfg, st, 3, 0.0)
    run_case(R, "dambreak32_dplus", cfg, st, "deltaSPH")
    run_case(R, "dambreak32_ips", cfg, st, "IPS")
    cfg, st = scenes.dam_break(dx=1.0 / 24)
    run_case(R, "dambreak24_jitter_dplus", cfg, _moving(cfg, st, 5, 0.1), "deltaSPH")


if __name__ == "__main__":
    main()
