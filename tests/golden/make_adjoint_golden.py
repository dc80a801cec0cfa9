"""Reference gradients of a 100-step rollout loss by torch autograd through the reference.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_adjoint_golden.py

The reference has no adjoint; its operators are torch code, so autograd through them is
the reference's own gradient. Each step composes, as the runner does
(src/diffSPH/v2/runner.py:37-42):

* the symplecticEuler stages of integrate (src/diffSPH/v2/modules/integration.py:357-392)
  around two calls of simulationStep (src/diffSPH/v2/simulationSchemes/deltaPlus.py:176-422),
  with the density update the reference's integrate leaves in the state (the half-step
  density, integration.py:439-513). integrate itself is not used because it writes its
  results through in-place state updates that cut the autograd graph;
* solveShifting (src/diffSPH/v2/modules/shifting.py:882-1019) added to the positions.

Case: random Fourier-mode periodic flow, 24x24 particles with 0.1 dx jitter. Loss: mean
squared difference between the velocity after 100 steps and a target field from the same
generator with another seed. The gradients with respect to the initial velocity,
positions, densities and diffusion.nu are written for an fp32 and an fp64 run to
``tests/golden/adjoint_fourier24_100.npz``.
"""
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ref_harness import load_reference  # noqa: E402
from make_golden import reference_config, to_torch_state  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402

torch.set_num_threads(min(8, os.cpu_count() or 1))

NX, SEED, TARGET_SEED, STEPS = 24, 3, 99, 100


def case():
    cfg, st = scenes.fourier_periodic(NX, seed=SEED, jitter=0.1)
    target = scenes.fourier_velocity(np.asarray(st["fluid"]["positions"], np.float64),
                                     np.random.default_rng(TARGET_SEED))
    return cfg, st, target


def reference_gradients(R, cfg, st, target, dtype):
    rc = reference_config(R, cfg)
    fl0 = {k: (v.astype(dtype) if isinstance(v, np.ndarray) and v.dtype.kind == "f" else v)
           for k, v in st["fluid"].items()}
    base = to_torch_state(fl0)
    x0 = base["positions"].clone().requires_grad_(True)
    u0 = base["velocities"].clone().requires_grad_(True)
    r0 = base["densities"].clone().requires_grad_(True)
    nu = torch.tensor(float(cfg["diffusion"]["nu"]), dtype=x0.dtype, requires_grad=True)
    rc["diffusion"]["nu"] = nu
    dt = rc["timestep"]["dt"]

    def rhs(fl):
        (_, dudt, drhodt), _ = R.deltaPlus.simulationStep({"fluid": dict(fl)}, rc)
        return dudt, drhodt

    fl = dict(base)
    fl.update(positions=x0, velocities=u0, densities=r0)
    for _ in range(STEPS):
        a1, d1 = rhs(fl)
        fh = dict(fl)
        fh.update(positions=fl["positions"] + fl["velocities"] * (dt / 2),
                  velocities=fl["velocities"] + a1 * (dt / 2), densities=fl["densities"] + d1 * (dt / 2))
        a2, _ = rhs(fh)
        un = fl["velocities"] + a2 * dt
        xn = fl["positions"] + 0.5 * (fl["velocities"] + un) * dt
        fl = dict(fl)
        fl.update(positions=xn, velocities=un, densities=fh["densities"])
        dxs, _ = R.shifting.solveShifting({"fluid": dict(fl)}, rc)
        fl["positions"] = fl["positions"] + dxs
    tgt = torch.as_tensor(target, dtype=x0.dtype)
    loss = torch.mean((fl["velocities"] - tgt) ** 2)
    loss.backward()
    return {"loss": float(loss), "u0": u0.grad.numpy().copy(), "x0": x0.grad.numpy().copy(),
            "rho0": r0.grad.numpy().copy(), "nu": float(nu.grad),
            "u_final": fl["velocities"].detach().numpy().copy()}


def main():
    R = load_reference()
    cfg, st, target = case()
    out = {"config_json": np.frombuffer(json.dumps(cfg).encode(), dtype=np.uint8),
           "steps": np.int64(STEPS), "target": target}
    for k, v in st["fluid"].items():
        out[f"in/fluid/{k}"] = v
    for tag, dtype in (("f32", np.float32), ("f64", np.float64)):
        g = reference_gradients(R, cfg, st, target, dtype)
        for k, v in g.items():
            out[f"{tag}/{k}"] = np.asarray(v)
        print(tag, "loss", g["loss"], "|du0|", float(np.linalg.norm(g["u0"])), "dnu", g["nu"])
    path = os.path.join(HERE, "adjoint_fourier24_100.npz")
    np.savez_compressed(path, **out)
    print("->", path)


if __name__ == "__main__":
    main()
