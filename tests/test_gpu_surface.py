"""GPU parity of the free-surface handling of the shift (shifting.freeSurface = True).

The golden vectors (tests/golden/make_fs_golden.py) hold the reference's own surface flags,
expanded mask, Lambdas and lambda-gradient normals of the merged fluid + wall set, and its
shift. Flags and masks are compared exactly, Lambdas at 1e-3 of their magnitude. A normal
normalises a sum of pair terms that cancels on a lattice, where it is rounding noise in any
fp32 evaluation, the reference's included: normals are compared at 1e-3 on the fluid rows
of the expanded mask (where the projection uses them; they are zero elsewhere) whose fp64
gradient is at least 1e-2 of the largest. The shift follows the normals through
the projection, so it is held to the fp32-parity bound against the fp64 oracle, with the
reference's own fp32 result as the fp32 run: |gpu - o64| <= 4 |ref - o64| + 1e-3 max|o64|.
"""
import copy

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from golden_io import load_case, rel_max  # noqa: E402
from oracle import sph_oracle as O  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402

FS_CASES = ["dambreak32_dplus", "dambreak32_ips", "dambreak24_jitter_dplus"]
TOL = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from diffsph_gb300 import _lib
    _lib.load()


def _np(t):
    return t.detach().cpu().numpy()


def _as64(st):
    return {p: {k: (v.astype(np.float64) if v.dtype == np.float32 else v.copy()) for k, v in a.items()}
            for p, a in st.items()}


def _solver(cfg, st):
    from diffsph_gb300.solver import Solver
    return Solver(cfg, st["fluid"], st.get("boundary"))


def assert_fp32_parity(gpu, o32, o64, tol, what=""):
    """|gpu - o64| <= 4 |o32 - o64| + tol * max|o64| (element-wise maxima)."""
    gpu, o32, o64 = (np.asarray(a, np.float64) for a in (gpu, o32, o64))
    e_gpu = float(np.max(np.abs(gpu - o64)))
    e_32 = float(np.max(np.abs(o32 - o64)))
    scale = float(np.max(np.abs(o64)))
    assert e_gpu <= 4 * e_32 + tol * scale, f"{what}: gpu err {e_gpu:.3e}, fp32 err {e_32:.3e}, scale {scale:.3e}"


def _moving_dam_break(dx, seed):
    cfg, st = scenes.dam_break(dx=dx)
    st = copy.deepcopy(st)
    rng = np.random.default_rng(seed)
    st["fluid"]["velocities"] = rng.uniform(-1.0, 1.0, st["fluid"]["velocities"].shape).astype(np.float32)
    cfg = copy.deepcopy(cfg)
    cfg["shifting"]["freeSurface"] = True
    return cfg, st


@pytest.mark.parametrize("case", FS_CASES)
def test_free_surface_shift_matches_reference_vectors(case):
    z, cfg, st = load_case(f"fs_{case}")
    assert cfg["shifting"]["freeSurface"]
    sol = _solver(cfg, st)
    dx = _np(sol.shift())
    sol.check()
    f = sol.free_surface_fields()
    nF = st["fluid"]["positions"].shape[0]
    assert np.array_equal(_np(f["freeSurface"]), z["fs/freeSurface"])
    assert np.array_equal(_np(f["freeSurfaceMask"]), z["fs/freeSurfaceMask"])
    assert rel_max(_np(f["Lambdas"]), z["fs/Lambdas"]) < TOL
    st64 = _as64(st)
    keys = ("positions", "velocities", "masses", "densities", "supports", "areas")
    ps = {k: np.concatenate([st64["fluid"][k], st64["boundary"][k]]) for k in keys}
    g64 = O.normals_lambda(ps, O.neighbor_search(ps, ps, cfg), gradient=True)
    gm = np.sqrt(np.sum(g64 * g64, axis=1))[:nF]
    # normals are computed on the rows of the expanded mask (the only ones the projection uses)
    firm = (gm >= 1e-2 * gm.max()) & z["fs/freeSurfaceMask"][:nF]
    assert firm.sum() > 0.1 * nF
    assert rel_max(_np(f["normals"])[:nF][firm], z["fs/lambdaGrad"][:nF][firm]) < TOL
    off = ~z["fs/freeSurfaceMask"]
    assert float(np.abs(_np(f["normals"])[off]).max(initial=0.0)) == 0.0
    d64, _ = O.solve_shifting(st64, cfg)
    assert_fp32_parity(dx, z["fs/shift"], d64, TOL, "shift")
    if cfg["shifting"]["scheme"] == "IPS":
        info = {}
        O.solve_shifting(copy.deepcopy(st), cfg, info)
        assert sol.ips_result() == (info["iterations"], info["code"])


@pytest.mark.parametrize("scheme", ["deltaSPH", "IPS"])
def test_free_surface_step_matches_oracle(scheme):
    """One fused step (integrate, then the shift with free-surface handling)."""
    cfg, st = _moving_dam_break(1.0 / 32, 7)
    cfg["shifting"]["scheme"] = scheme
    r32, _ = O.full_step(copy.deepcopy(st), cfg)
    r64, _ = O.full_step(_as64(st), cfg)
    sol = _solver(cfg, st)
    sol.step(1)
    sol.check()
    got = sol.download()
    a, b = r32["fluid"], r64["fluid"]
    assert_fp32_parity(_np(got["velocities"]), a["velocities"], b["velocities"], 1e-4, "velocities")
    x0 = st["fluid"]["positions"]
    assert_fp32_parity(_np(got["positions"]) - x0, a["positions"] - x0, b["positions"] - x0, TOL, "x' - x")


def test_free_surface_graph_replay_equals_eager_steps():
    cfg, st = _moving_dam_break(1.0 / 32, 9)
    a = _solver(cfg, st)
    a.step(4)
    b = _solver(cfg, st)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.graph_step(2)
        b.graph_step(2)
    s.synchronize()
    ga, gb = a.download(), b.download()
    for k in ("positions", "velocities", "densities", "boundary_densities"):
        assert torch.equal(ga[k], gb[k]), k


def test_free_surface_off_restores_the_plain_shift():
    cfg, st = _moving_dam_break(1.0 / 32, 11)
    a = _solver(cfg, st)
    a.set_free_surface(None)
    cfg_plain = copy.deepcopy(cfg)
    cfg_plain["shifting"]["freeSurface"] = False
    b = _solver(cfg_plain, st)
    assert torch.equal(a.shift(), b.shift())
    # the handling changes the shift of surface particles
    c = _solver(cfg, st)
    assert not torch.equal(c.shift(), b.shift())


def test_pressure_switch_matches_reference():
    """computePressureAccelSwitch on the reference's state, neighborhoods and surface mask;
    each fp32 step follows the reference's order, so the sums agree to rounding."""
    import os
    from golden_io import GOLDEN
    from diffsph_gb300.scheme import computePressureAccelSwitch
    z = np.load(os.path.join(GOLDEN, "switch_dambreak32.npz"))
    fl = {k: torch.from_numpy(z[f"fluid/{k}"]) for k in ("densities", "masses", "pressures", "surfaceMask")}
    bd = {k: torch.from_numpy(z[f"boundary/{k}"]) for k in ("densities", "masses", "pressures")}
    for name, sB in (("ff", fl), ("fb", bd)):
        nb = {"indices": (torch.from_numpy(z[f"{name}/i"]), torch.from_numpy(z[f"{name}/j"])),
              "gradients": torch.from_numpy(z[f"{name}/gradients"]),
              "numNeighbors": torch.from_numpy(z[f"{name}/numNeighbors"]),
              "neighborOffsets": torch.from_numpy(z[f"{name}/neighborOffsets"])}
        got = _np(computePressureAccelSwitch(fl, sB, nb, None))
        assert rel_max(got, z[f"{name}/accel"]) < 1e-6, name
        # without a surface mask every negative-pressure particle takes the difference form
        fl0 = {k: v for k, v in fl.items() if k != "surfaceMask"}
        ref0 = O.pressure_accel_switch({k: v.numpy() for k, v in fl.items()} | {"surfaceMask": np.zeros(
            fl["pressures"].shape[0], np.float32)}, {k: v.numpy() for k, v in sB.items()},
            {"indices": (z[f"{name}/i"], z[f"{name}/j"]), "gradients": z[f"{name}/gradients"]}, None)
        assert rel_max(_np(computePressureAccelSwitch(fl0, sB, nb, None)), ref0) < 1e-6, name
