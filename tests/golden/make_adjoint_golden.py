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

Cases: random Fourier-mode periodic flows with 0.1 dx jitter, 24x24 particles (seeds 3 and
99, 100 steps) and 128x128 particles (the 128^2 adjoint rollout, seeds 0 and 1: its first 100
steps, and all 1000). Loss: mean squared difference between the final velocity and a
target field from the same generator with another seed. The gradients with respect to the initial velocity,
positions, densities and diffusion.nu are written for an fp32 and an fp64 run to
``tests/golden/adjoint_<case>.npz``. The 128^2 run
keeps only every step's inputs from a forward pass without a graph and rebuilds one step's
graph at a time in the backward pass (per-step checkpointing), so that memory stays at one
step's graph; the gradients are those of the whole graph.

    python tests/golden/make_adjoint_golden.py [fourier24_100 | fourier128_100 | fourier128_1000]
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

# name: (particles per side, seed, target seed, steps, checkpoint every step)
CASES = {"fourier24_100": (24, 3, 99, 100, False), "fourier128_100": (128, 0, 1, 100, True),
         "fourier128_1000": (128, 0, 1, 1000, True)}


def case(name="fourier24_100"):
    nx, seed, target_seed, steps, _ = CASES[name]
    cfg, st = scenes.fourier_periodic(nx, seed=seed, jitter=0.1)
    target = scenes.fourier_velocity(np.asarray(st["fluid"]["positions"], np.float64),
                                     np.random.default_rng(target_seed))
    return cfg, st, target, steps


def reference_gradients(R, cfg, st, target, dtype, steps, checkpoint=False):
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

    def step(x, u, r, nu_t):
        rc["diffusion"]["nu"] = nu_t
        fl = dict(base)
        fl.update(positions=x, velocities=u, densities=r)
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
        return fl["positions"] + dxs, un, fh["densities"]

    tgt = torch.as_tensor(target, dtype=x0.dtype)
    if not checkpoint:
        x, u, r = x0, u0, r0
        for _ in range(steps):
            x, u, r = step(x, u, r, nu)
        loss = torch.mean((u - tgt) ** 2)
        loss.backward()
        return {"loss": float(loss), "u0": u0.grad.numpy().copy(), "x0": x0.grad.numpy().copy(),
                "rho0": r0.grad.numpy().copy(), "nu": float(nu.grad), "u_final": u.detach().numpy().copy()}
    # checkpointed: a forward pass without a graph keeps every step's inputs; the backward
    # pass rebuilds one step's graph at a time from them and pulls the adjoint through it
    states = [(x0.detach(), u0.detach(), r0.detach())]
    with torch.no_grad():
        for k in range(steps):
            states.append(step(*states[-1], nu.detach()))
            if (k + 1) % 10 == 0:
                print(f"  forward {k + 1}/{steps}", flush=True)
    uf = states[-1][1].clone().requires_grad_(True)
    loss = torch.mean((uf - tgt) ** 2)
    (gu,) = torch.autograd.grad(loss, uf)
    gx, gr = torch.zeros_like(x0), torch.zeros_like(r0)
    gnu = torch.zeros_like(nu)
    for k in reversed(range(steps)):
        xi, ui, ri = (t.clone().requires_grad_(True) for t in states[k])
        nk = nu.detach().clone().requires_grad_(True)
        xo, uo, ro = step(xi, ui, ri, nk)
        gx, gu, gr, gn = torch.autograd.grad((xo, uo, ro), (xi, ui, ri, nk), grad_outputs=(gx, gu, gr),
                                             allow_unused=True)
        gx = torch.zeros_like(x0) if gx is None else gx
        gr = torch.zeros_like(r0) if gr is None else gr
        gnu = gnu + (gn if gn is not None else 0.0)
        if k % 10 == 0:
            print(f"  backward {k}/{steps}", flush=True)
    return {"loss": float(loss), "u0": gu.numpy().copy(), "x0": gx.numpy().copy(), "rho0": gr.numpy().copy(),
            "nu": float(gnu), "u_final": states[-1][1].numpy().copy()}


def main(names):
    R = load_reference()
    for name in names:
        cfg, st, target, steps = case(name)
        ckpt = CASES[name][4]
        out = {"config_json": np.frombuffer(json.dumps(cfg).encode(), dtype=np.uint8),
               "steps": np.int64(steps), "target": target}
        for k, v in st["fluid"].items():
            out[f"in/fluid/{k}"] = v
        for tag, dtype in (("f32", np.float32), ("f64", np.float64)):
            g = reference_gradients(R, cfg, st, target, dtype, steps, checkpoint=ckpt)
            for k, v in g.items():
                # the large case keeps its arrays in fp32 (the tests compare at 1e-3)
                out[f"{tag}/{k}"] = np.asarray(v, np.float32) if ckpt and np.ndim(v) else np.asarray(v)
            print(name, tag, "loss", g["loss"], "|du0|", float(np.linalg.norm(g["u0"])), "dnu", g["nu"], flush=True)
        path = os.path.join(HERE, f"adjoint_{name}.npz")
        np.savez_compressed(path, **out)
        print("->", path)


if __name__ == "__main__":
    main(sys.argv[1:] or ["fourier24_100"])
