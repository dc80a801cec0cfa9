"""Generate golden input/output vectors by running the reference diffSPH v2 code on CPU.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_golden.py

Writes ``tests/golden/<case>.npz``. Each file holds the inputs (particle arrays and
the configuration as JSON) and the reference's outputs for:

* ``neighborSearch`` fluid-fluid (src/diffSPH/v2/modules/neighborhood.py:491-593);
* one ``simulationStep`` (src/diffSPH/v2/simulationSchemes/deltaPlus.py:176-422) with
  its intermediate fields (covariance, L, gradRho^L, diffusion terms, pressures ...);
* one ``integrate`` step with scheme ``symplecticEuler``
  (src/diffSPH/v2/modules/integration.py:357-392) followed by ``solveShifting``
  (src/diffSPH/v2/modules/shifting.py:882-1019), as the runner does
  (src/diffSPH/v2/runner.py:37-42).

The reference is imported through ``ref_harness`` (stubs for plotting/IO packages and a
brute-force stand-in for the external candidate search).
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

from ref_harness import load_reference  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402

torch.set_num_threads(min(8, os.cpu_count() or 1))


def reference_config(R, cfg):
    """Build the reference's parsed config for one of our scene configs."""
    d = cfg["domain"]
    raw = {
        "domain": {"minExtent": d["minExtent"], "maxExtent": d["maxExtent"], "dim": 2,
                   "periodic": d["periodic"]},
        "particle": {"dx": cfg["particle"]["dx"], "nx": int(round((d["maxExtent"][0] - d["minExtent"][0]) / cfg["particle"]["dx"]))},
        "compute": {"device": "cpu", "checkNaN": False},
        "fluid": {"cs": cfg["fluid"]["cs"], "rho0": cfg["fluid"]["rho0"]},
        "kernel": {"targetNeighbors": 16 * np.pi},
        "EOS": {"type": "stiffTait", "polytropicExponent": 7},
        "diffusion": {k: v for k, v in cfg["diffusion"].items()},
        "integration": {"scheme": "symplecticEuler"},
        "timestep": {"dt": cfg["timestep"]["dt"], "active": False},
        "shifting": {"scheme": "deltaSPH", "threshold": cfg["shifting"]["threshold"], "maxIterations": 1,
                     "freeSurface": False},
        "gravity": {"active": cfg["gravity"]["active"]},
        "boundary": {"active": cfg["boundary"]["active"]},
        "export": {"active": False},
        "simulation": {"densityScheme": cfg.get("simulation", {}).get("densityScheme", "continuity")},
    }
    if raw["particle"]["dx"] > 0:
        raw["particle"]["dx"] = float(cfg["particle"]["dx"])
    c = R.parameters.parseDefaultParameters(raw)
    c = R.parameters.parseModuleParameters(c)
    c["timestep"]["dt"] = cfg["timestep"]["dt"]
    return c


def to_torch_state(st):
    out = {}
    for k, v in st.items():
        out[k] = torch.from_numpy(np.ascontiguousarray(v)) if isinstance(v, np.ndarray) else v
    out["numParticles"] = out["positions"].shape[0]
    return out


def npy(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


def run_case(R, name, cfg, st, store_pairs=True):
    rc = reference_config(R, cfg)
    derived = {
        "support": float(rc["particle"]["support"]), "dx": float(rc["particle"]["dx"]),
        "kernelScale": float(rc["kernel"]["kernelScale"]), "cs": float(rc["fluid"]["cs"]),
    }
    for k, mine in (("support", cfg["particle"]["support"]), ("dx", cfg["particle"]["dx"]),
                    ("kernelScale", cfg["kernel"]["kernelScale"]), ("cs", cfg["fluid"]["cs"])):
        assert abs(derived[k] - mine) <= 1e-6 * abs(mine), (k, derived[k], mine)
    out = {"config_json": np.frombuffer(json.dumps(cfg).encode(), dtype=np.uint8),
           "ref_derived_json": np.frombuffer(json.dumps(derived).encode(), dtype=np.uint8)}
    for part, arrs in st.items():
        for k, v in arrs.items():
            out[f"in/{part}/{k}"] = v

    state = {p: to_torch_state(v) for p, v in st.items()}
    # 1) fluid-fluid neighbor search
    _, nb = R.neighborhood.neighborSearch(state["fluid"], state["fluid"], rc, True, None, None, False)
    out["nb/numNeighbors"] = npy(nb["numNeighbors"])
    if store_pairs:
        for k in ("distances", "vectors", "supports", "kernels", "gradients", "neighborOffsets"):
            out[f"nb/{k}"] = npy(nb[k])
        out["nb/i"], out["nb/j"] = npy(nb["indices"][0]), npy(nb["indices"][1])

    # 2) one right-hand-side evaluation with its intermediates
    s1 = copy.deepcopy(state)
    (u, dudt, drhodt), bnd = R.deltaPlus.simulationStep(s1, rc)
    out["rhs/dudt"], out["rhs/drhodt"] = npy(dudt), npy(drhodt)
    for k in ("covarianceMatrix", "L", "gradRho^L", "densityDiffusion", "velocityDiffusion",
              "momentumEquation", "pressures", "pressureAccel", "gravityAccel"):
        out[f"rhs/{k}"] = npy(s1["fluid"][k])
    out["rhs/densities"] = npy(s1["fluid"]["densities"])
    if "boundary" in s1:
        out["rhs/boundary_densities"] = npy(s1["boundary"]["densities"])
        out["rhs/ghost_shepard"] = npy(s1["boundaryGhost"]["densities"])
        out["rhs/ghost_numNeighbors"] = npy(s1["boundaryGhost"]["numNeighbors"])
        out["rhs/ghost_positions"] = npy(s1["boundaryGhost"]["positions"])
        btf = s1["boundaryToFluidNeighborhood"]
        out["rhs/btf_numNeighbors"] = npy(btf["numNeighbors"])
        if store_pairs:
            out["rhs/btf_i"], out["rhs/btf_j"] = npy(btf["indices"][0]), npy(btf["indices"][1])

    # 3) one full time step: integrate (symplectic Euler) + delta+ shifting
    s2 = copy.deepcopy(state)
    perennial = dict(s2)
    perennial.update(time=0.0, timestep=0, dt=rc["timestep"]["dt"])
    perennial, prior, *_ = R.integration.integrate(R.deltaPlus.simulationStep, perennial, rc, None)
    out["step/positions_integrated"] = npy(perennial["fluid"]["positions"]).copy()
    out["step/velocities"] = npy(perennial["fluid"]["velocities"])
    out["step/densities"] = npy(perennial["fluid"]["densities"])
    out["step/dudt"] = npy(perennial["fluid"]["dudt"])
    if "boundary" in perennial:
        out["step/boundary_densities"] = npy(perennial["boundary"]["densities"])
    dxs, _ = R.shifting.solveShifting(perennial, rc)
    out["step/shift"] = npy(dxs)
    perennial["fluid"]["positions"] += dxs
    out["step/positions"] = npy(perennial["fluid"]["positions"])
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: fluid {st['fluid']['positions'].shape[0]}, pairs {int(out['nb/numNeighbors'].sum())} -> {path}")


def summation(cfg_st):
    """The same scene with simulation.densityScheme 'summation' (deltaPlus.py:193-198)."""
    cfg, st = cfg_st
    cfg = copy.deepcopy(cfg)
    cfg.setdefault("simulation", {})["densityScheme"] = "summation"
    return cfg, st


def main(only=None):
    R = load_reference()
    if only == "extra":
        extra(R)
        return
    # lattice TGV (many pairs exactly at r = H)
    cfg, st = scenes.taylor_green(16)
    run_case(R, "tgv16_lattice", cfg, st)
    # jittered TGV with particles pushed outside the periodic box (wrap path)
    cfg, st = scenes.taylor_green(24, jitter=0.1, seed=7)
    x = st["fluid"]["positions"]
    rng = np.random.default_rng(11)
    sel = rng.choice(x.shape[0], size=40, replace=False)
    x[sel[:20], 0] += np.float32(2.0)
    x[sel[20:], 1] -= np.float32(2.0)
    run_case(R, "tgv24_jitter_wrap", cfg, st)
    # random Fourier-mode periodic flow
    cfg, st = scenes.fourier_periodic(20, seed=3)
    run_case(R, "fourier20", cfg, st)
    # dam break with mDBC walls (coarse: dx = 1/16)
    cfg, st = scenes.dam_break(dx=1.0 / 16)
    run_case(R, "dambreak16", cfg, st)
    extra(R)


def extra(R):
    # summation density: a jittered periodic flow and the coarse dam break
    cfg, st = summation(scenes.taylor_green(24, jitter=0.1, seed=7))
    run_case(R, "tgv24_summation", cfg, st, store_pairs=False)
    cfg, st = summation(scenes.dam_break(dx=1.0 / 16))
    run_case(R, "dambreak16_summation", cfg, st, store_pairs=False)
    # the dam break at dx = 1/32 (outputs only: its pair list would be several MB)
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    run_case(R, "dambreak32", cfg, st, store_pairs=False)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
