"""Generate golden vectors of the reference's mirror-outlet update on CPU.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_outlet_step_golden.py

Writes ``tests/golden/outlet_step_block32.npz``. The scene is the bench's mirror-outlet block
at dx = 1/32 (the lower unit square of the dam break's fluid, random velocities, no walls),
with a mirror region x > 0.9 given by its signed distance function. The update is the
reference's own outlet processing of simulationStep
(src/diffSPH/v2/simulationSchemes/deltaPlus.py:188-189 and 209-229), run with its
functions: buildOutletGhostParticles (inletOutlet.py:67-147), then LiuLiuConsistent
(sphOps.py:313-341) for the density and each velocity component, written back where a
ghost has at least 10 neighbors. The three calls to LiuLiuConsistent and their order are
those of deltaPlus.py; the density is updated before the velocities are interpolated.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from make_golden import reference_config, to_torch_state, npy  # noqa: E402
from ref_harness import load_reference  # noqa: E402

MIRROR_X = 0.9


def main():
    R = load_reference()
    import bench
    import diffSPH.v2.modules.inletOutlet as io_mod
    from diffSPH.v2.sphOps import LiuLiuConsistent
    fl, cfg = bench._regions_block(32, MIRROR_X)
    rc = reference_config(R, cfg)
    rc["particle"]["volume"] = cfg["particle"]["volume"]
    rc["compute"]["dtype"] = torch.float32
    out = {f"in/fluid/{k}": v.copy() for k, v in fl.items()}
    state = {"fluid": to_torch_state(fl)}
    regions = [{"type": "mirror", "sdf": lambda p: MIRROR_X - p[:, 0]}]
    ghost = io_mod.buildOutletGhostParticles(regions, state, rc)
    f = state["fluid"]
    cond = ghost["numNeighbors"] >= 10
    shift = ghost["sdf_dist"][:, None] * ghost["sdf_grad"] * 2

    def update(quantity, solution):
        return torch.where(cond, solution[:, 0] + torch.einsum("nd, nd -> n", shift, solution[:, 1:]), quantity)

    idx = ghost["fluidIndex"]
    sol, _, _ = LiuLiuConsistent(ghost, f, f["densities"])
    f["densities"][idx] = update(f["densities"][idx], sol)
    sol, _, _ = LiuLiuConsistent(ghost, f, f["velocities"][:, 0])
    f["velocities"][idx, 0] = update(f["velocities"][idx][:, 0], sol)
    sol, _, _ = LiuLiuConsistent(ghost, f, f["velocities"][:, 1])
    f["velocities"][idx, 1] = update(f["velocities"][idx][:, 1], sol)
    out["out/densities"], out["out/velocities"] = npy(f["densities"]), npy(f["velocities"])
    out["out/ghosts"] = np.array(ghost["positions"].shape[0])
    out["out/updated"] = npy(idx[cond])
    path = os.path.join(HERE, "outlet_step_block32.npz")
    np.savez_compressed(path, **out)
    print(f"outlet_step_block32: fluid {fl['positions'].shape[0]}, ghosts {int(out['out/ghosts'])}, "
          f"updated {out['out/updated'].shape[0]} -> {path}")


if __name__ == "__main__":
    main()
