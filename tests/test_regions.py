"""Open-boundary regions (drop-ins for src/diffSPH/v2/modules/inletOutlet.py) against the
reference's own results (tests/golden/make_regions_golden.py). The CPU tests cover the
functions that need no neighbor search; the GPU tests the ghost construction with its
neighborhood, the emitter and the consistent interpolation kernel."""
import copy
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from golden_io import GOLDEN, rel_max  # noqa: E402
from oracle import sph_oracle as O  # noqa: E402

MIRROR_X, OUTLET_X, FORCING_Y = 0.8, 0.95, 0.1


def sdf_mirror(p):
    return MIRROR_X - p[:, 0]


def sdf_outlet(p):
    return OUTLET_X - p[:, 0]


def sdf_forcing(p):
    return p[:, 1] - FORCING_Y


def _golden():
    z = np.load(os.path.join(GOLDEN, "regions_block32.npz"))
    fluid = {k[len("in/fluid/"):]: z[k] for k in z.files if k.startswith("in/fluid/")}
    return z, fluid


def _config():
    from diffsph_gb300 import scenes
    cfg, _ = scenes.dam_break(dx=1.0 / 32)
    cfg = copy.deepcopy(cfg)
    cfg["boundary"]["active"] = False
    cfg["particle"]["volume"] = (1.0 / 32) ** 2
    return cfg


def _state(fluid, device):
    fl = {k: torch.from_numpy(v.copy()).to(device) for k, v in fluid.items()}
    fl["numParticles"] = fl["positions"].shape[0]
    return {"fluid": fl, "uidCounter": fl["positions"].shape[0]}


def test_outlet_and_forcing_match_reference():
    from diffsph_gb300 import regions
    z, fluid = _golden()
    cfg = _config()
    s = _state(fluid, "cpu")
    regions.processOutlet({"type": "outlet", "sdf": sdf_outlet}, cfg, s)
    assert torch.equal(s["fluid"]["positions"], torch.from_numpy(z["outlet/positions"]))
    assert s["fluid"]["numParticles"] == z["outlet/positions"].shape[0]
    s = _state(fluid, "cpu")
    regions.processForcing({"type": "forcing", "sdf": sdf_forcing, "velocity": [0.5, 0.0]}, cfg, s)
    assert torch.equal(s["fluid"]["velocities"], torch.from_numpy(z["forcing/velocities"]))
    assert torch.equal(s["fluid"]["densities"], torch.from_numpy(z["forcing/densities"]))


def test_sdf_gradient_matches_reference():
    from diffsph_gb300 import regions
    z, fluid = _golden()
    cfg = _config()
    idx = torch.from_numpy(z["ghost/fluidIndex"])
    p = torch.from_numpy(fluid["positions"])[idx]
    g = regions._sdf_gradient(sdf_mirror, p, float(cfg["particle"]["support"]) * 0.01)
    g = g / (torch.linalg.norm(g, dim=1, keepdim=True) + 1e-7)
    assert torch.equal(g, torch.from_numpy(z["ghost/sdf_grad"]))


@pytest.mark.gpu
def test_outlet_ghosts_match_reference():
    from diffsph_gb300 import regions
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    z, fluid = _golden()
    cfg = _config()
    s = _state(fluid, "cuda")
    g = regions.buildOutletGhostParticles([{"type": "mirror", "sdf": sdf_mirror}], s, cfg)
    assert torch.equal(g["fluidIndex"].cpu(), torch.from_numpy(z["ghost/fluidIndex"]))
    assert torch.equal(g["positions"].cpu(), torch.from_numpy(z["ghost/positions"]))
    nb = g["neighborhood"]
    i, j = nb["indices"][0].cpu().numpy(), nb["indices"][1].cpu().numpy()
    o, oz = np.lexsort((j, i)), np.lexsort((z["ghost/j"], z["ghost/i"]))
    assert np.array_equal(i[o], z["ghost/i"][oz]) and np.array_equal(j[o], z["ghost/j"][oz])
    assert np.array_equal(nb["distances"].cpu().numpy()[o], z["ghost/nb_distances"][oz])
    assert np.array_equal(g["numNeighbors"].cpu().numpy(), z["ghost/numNeighbors"])


@pytest.mark.gpu
def test_liuliu_consistent_matches_reference():
    """The kernel's moment sums follow the reference's fp32 order (M and b agree to rounding);
    the solution divides determinants, computed in fp64 here and from fp32 LU factors in the
    reference, so it is held to |gpu - o64| <= 4 |ref - o64| + 1e-4 max|o64|."""
    from diffsph_gb300 import regions
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    z, fluid = _golden()
    nb = {"indices": (torch.from_numpy(z["ghost/i"]), torch.from_numpy(z["ghost/j"])),
          "numNeighbors": torch.from_numpy(z["ghost/numNeighbors"]),
          "neighborOffsets": torch.from_numpy(z["ghost/nb_neighborOffsets"])}
    for k in ("distances", "vectors", "supports", "kernels", "gradients"):
        nb[k] = torch.from_numpy(z[f"ghost/nb_{k}"])
    ghost = {"positions": torch.from_numpy(z["ghost/positions"]), "neighborhood": nb}
    fl = {k: torch.from_numpy(v) for k, v in fluid.items()}
    f64 = {k: v.astype(np.float64) if v.dtype == np.float32 else v for k, v in fluid.items()}
    nb64 = {"indices": (z["ghost/i"], z["ghost/j"])}
    for k in ("distances", "vectors", "supports", "kernels", "gradients"):
        nb64[k] = z[f"ghost/nb_{k}"].astype(np.float64)
    for name, q in (("rho", fl["densities"]), ("u", fl["velocities"][:, 0]), ("v", fl["velocities"][:, 1])):
        sol, M, b = regions.LiuLiuConsistent(ghost, fl, q)
        assert rel_max(M.numpy(), z[f"liuliu/{name}/M"]) < 1e-6, name
        assert rel_max(b.numpy(), z[f"liuliu/{name}/b"]) < 1e-6, name
        s64, _, _ = O.liuliu_consistent({"positions": z["ghost/positions"]}, f64, nb64, q.numpy().astype(np.float64))
        e_gpu = np.abs(sol.numpy() - s64).max()
        e_ref = np.abs(z[f"liuliu/{name}/solution"] - s64).max()
        assert e_gpu <= 4 * e_ref + 1e-4 * np.abs(s64).max(), name


@pytest.mark.gpu
def test_inlet_matches_reference():
    from diffsph_gb300 import regions
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    z, fluid = _golden()
    cfg = _config()
    s = _state(fluid, "cuda")
    em = z["inlet/emitter"]
    n = em.shape[0]
    emitter = {"particles": {"positions": torch.from_numpy(em).cuda(),
                             "supports": torch.full((n,), float(cfg["particle"]["support"]), device="cuda"),
                             "numParticles": n}, "velocity": [1.0, 0.0]}
    regions.processInlet(s, cfg, emitter)
    assert torch.equal(s["fluid"]["positions"].cpu(), torch.from_numpy(z["inlet/positions"]))
    assert torch.equal(s["fluid"]["velocities"].cpu(), torch.from_numpy(z["inlet/velocities"]))
    assert s["uidCounter"] == int(z["inlet/uidCounter"])
