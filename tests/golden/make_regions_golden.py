"""Generate golden vectors of the reference's open-boundary (inlet / outlet) functions on CPU.

Run in the development container (the reference source tree must be importable):

    python tests/golden/make_regions_golden.py

Writes ``tests/golden/regions_block32.npz``. The scene is a moving 1 x 1 block of fluid on a
dx = 1/32 lattice with densities scattered around rho0, and four half-plane regions given by
signed distance functions (negative inside):
- mirror:  x > 0.8
- outlet:  x > 0.95
- forcing: y < 0.1, velocity (0.5, 0);
- inlet:   an emitter of particles on the lattice columns x = -dx/2 and x = -3 dx / 2.

Recorded, each from the reference's own functions (src/diffSPH/v2/modules/inletOutlet.py):
- ``buildOutletGhostParticles`` (:67-147): the ghost positions, their fluid indices, SDF
  distances and gradients, and the ghost-to-fluid neighborhood;
- ``LiuLiuConsistent`` (src/diffSPH/v2/sphOps.py:313-341) on it for the densities and both
  velocity components: solution, M and b;
- ``processOutlet`` (:14-33), ``processForcing`` (:35-48) and ``processInlet`` (:150-189) on
  copies of the state.
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

MIRROR_X, OUTLET_X, FORCING_Y = 0.8, 0.95, 0.1


def sdf_mirror(p):
    return MIRROR_X - p[:, 0]


def sdf_outlet(p):
    return OUTLET_X - p[:, 0]


def sdf_forcing(p):
    return p[:, 1] - FORCING_Y


def block_scene(dx, seed):
    """A 1 x 1 fluid block on the lattice (no walls), moving, densities around rho0."""
    cfg, st = scenes.dam_break(dx=dx)
    fl = st["fluid"]
    keep = fl["positions"][:, 1] < 1.0
    fl = {k: v[keep].copy() for k, v in fl.items()}
    rng = np.random.default_rng(seed)
    fl["velocities"] = rng.uniform(-1.0, 1.0, fl["velocities"].shape).astype(np.float32)
    fl["densities"] = (fl["densities"] * (1 + rng.uniform(-5e-3, 5e-3, fl["densities"].shape))).astype(np.float32)
    cfg = copy.deepcopy(cfg)
    cfg["boundary"]["active"] = False
    return cfg, {"fluid": fl}


def emitter_positions(dx):
    ys = (np.arange(32) + 0.5) * dx
    cols = [np.stack([np.full_like(ys, x), ys], axis=1) for x in (-0.5 * dx, -1.5 * dx)]
    return np.concatenate(cols).astype(np.float32)


def main():
    R = load_reference()
    import diffSPH.v2.modules.inletOutlet as io_mod
    from diffSPH.v2.sphOps import LiuLiuConsistent
    dx = 1.0 / 32
    cfg, st = block_scene(dx, 17)
    rc = reference_config(R, cfg)
    rc["particle"]["volume"] = dx * dx
    rc["compute"]["dtype"] = torch.float32
    state = {"fluid": to_torch_state(st["fluid"]), "uidCounter": st["fluid"]["positions"].shape[0]}
    out = {}
    for k, v in st["fluid"].items():
        out[f"in/fluid/{k}"] = v
    # mirror ghosts and the consistent interpolation
    regions = [{"type": "mirror", "sdf": sdf_mirror}]
    ghost = io_mod.buildOutletGhostParticles(regions, state, rc)
    for k in ("positions", "fluidIndex", "sdf_dist", "sdf_grad", "numNeighbors"):
        out[f"ghost/{k}"] = npy(ghost[k])
    nb = ghost["neighborhood"]
    out["ghost/i"], out["ghost/j"] = npy(nb["indices"][0]), npy(nb["indices"][1])
    for k in ("distances", "vectors", "supports", "kernels", "gradients", "neighborOffsets"):
        out[f"ghost/nb_{k}"] = npy(nb[k])
    fl = state["fluid"]
    for name, q in (("rho", fl["densities"]), ("u", fl["velocities"][:, 0]), ("v", fl["velocities"][:, 1])):
        sol, M, b = LiuLiuConsistent(ghost, fl, q)
        out[f"liuliu/{name}/solution"], out[f"liuliu/{name}/M"], out[f"liuliu/{name}/b"] = npy(sol), npy(M), npy(b)
    # outlet, forcing and inlet on copies
    s = copy.deepcopy(state)
    io_mod.processOutlet({"type": "outlet", "sdf": sdf_outlet}, rc, s)
    out["outlet/positions"] = npy(s["fluid"]["positions"])
    s = copy.deepcopy(state)
    io_mod.processForcing({"type": "forcing", "sdf": sdf_forcing, "velocity": [0.5, 0.0]}, rc, s)
    out["forcing/velocities"], out["forcing/densities"] = npy(s["fluid"]["velocities"]), npy(s["fluid"]["densities"])
    s = copy.deepcopy(state)
    em = emitter_positions(dx)
    emitter = {"particles": {"positions": torch.from_numpy(em), "supports": torch.full((em.shape[0],), float(
        cfg["particle"]["support"])), "numParticles": em.shape[0], "masses": torch.full((em.shape[0],), dx * dx * 1000.0),
        "densities": torch.full((em.shape[0],), 1000.0)}, "velocity": [1.0, 0.0]}
    out["inlet/emitter"] = em
    # the block's left column sits dx/2 from the emitter's first column: that column is
    # blocked, the second (3 dx / 2 away) is not
    io_mod.processInlet(s, rc, emitter)
    out["inlet/positions"] = npy(s["fluid"]["positions"])
    out["inlet/velocities"] = npy(s["fluid"]["velocities"])
    out["inlet/uidCounter"] = np.array(s["uidCounter"])
    path = os.path.join(HERE, "regions_block32.npz")
    np.savez_compressed(path, **out)
    print(f"regions_block32: fluid {st['fluid']['positions'].shape[0]}, ghosts {out['ghost/positions'].shape[0]}, "
          f"after outlet {out['outlet/positions'].shape[0]}, after inlet {out['inlet/positions'].shape[0]} -> {path}")


if __name__ == "__main__":
    main()
