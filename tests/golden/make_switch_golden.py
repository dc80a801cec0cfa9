"""Generate golden vectors of the reference's Antuono pressure switch on CPU.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_switch_golden.py

Writes ``tests/golden/switch_dambreak32.npz``. The state is a moving dx = 1/32 dam break with
densities scattered around rho0 (pressures of both signs) after one ``simulationStep`` (src/diffSPH/v2/simulationSchemes/deltaPlus.py:176-422), which
leaves the pressures and the wall densities in it. The surface mask is the reference's
``detectFreeSurfaceBarecasco`` (src/diffSPH/v2/modules/surfaceDetection.py:95-107) on the
fluid. The file holds ``computePressureAccelSwitch`` (src/diffSPH/v2/modules/pressureForce.py:
15-33) for the fluid-fluid and the fluid-wall neighborhoods, with those neighborhoods.
"""
import copy
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


def main():
    R = load_reference()
    import diffSPH.v2.modules.pressureForce as pf
    import diffSPH.v2.modules.surfaceDetection as sd
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    st = copy.deepcopy(st)
    rng = np.random.default_rng(13)
    st["fluid"]["velocities"] = rng.uniform(-1.0, 1.0, st["fluid"]["velocities"].shape).astype(np.float32)
    # densities on both sides of rho0, so that the pressures take both signs
    rho = st["fluid"]["densities"]
    st["fluid"]["densities"] = (rho * (1 + rng.uniform(-5e-3, 5e-3, rho.shape))).astype(np.float32)
    rc = reference_config(R, cfg)
    state = {p: to_torch_state(v) for p, v in st.items()}
    R.deltaPlus.simulationStep(state, rc)
    fl, bd = state["fluid"], state["boundary"]
    fs = sd.detectFreeSurfaceBarecasco(fl, fl, fl["neighborhood"], rc)
    fl["surfaceMask"] = fs.to(torch.float32)
    out = {}
    for k in ("positions", "densities", "masses", "pressures", "surfaceMask"):
        out[f"fluid/{k}"] = npy(fl[k])
    bd_p = bd["pressures"] if "pressures" in bd else torch.zeros_like(bd["densities"])
    for k, v in (("densities", bd["densities"]), ("masses", bd["masses"]), ("pressures", bd_p)):
        out[f"boundary/{k}"] = npy(v)
    for name, (sB, nb) in {"ff": (fl, fl["neighborhood"]),
                           "fb": ({**bd, "pressures": bd_p}, state["boundaryToFluidNeighborhood"])}.items():
        acc = pf.computePressureAccelSwitch(fl, sB, nb, rc)
        out[f"{name}/accel"] = npy(acc)
        out[f"{name}/i"], out[f"{name}/j"] = npy(nb["indices"][0]), npy(nb["indices"][1])
        out[f"{name}/gradients"] = npy(nb["gradients"])
        out[f"{name}/numNeighbors"] = npy(nb["numNeighbors"])
        out[f"{name}/neighborOffsets"] = npy(nb["neighborOffsets"])
    path = os.path.join(HERE, "switch_dambreak32.npz")
    np.savez_compressed(path, **out)
    p = out["fluid/pressures"]
    print(f"switch_dambreak32: fluid {p.shape[0]}, negative pressures {int((p < 0).sum())}, surface "
          f"{int(out['fluid/surfaceMask'].sum())}, pairs ff {out['ff/i'].shape[0]}, fb {out['fb/i'].shape[0]} -> {path}")


if __name__ == "__main__":
    main()
