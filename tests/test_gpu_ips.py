"""GPU parity of the implicit particle shifting (shifting.scheme 'IPS').

The reference solves a 2N x 2N sparse system with an fp32 BiCGStab that stops at a relative
residual of 1e-4 (src/diffSPH/v2/modules/shifting.py:322-493, 780-880). Iterates of a Krylov
solve carry the rounding of every product and dot product, so the GPU solve is compared
with the reference's vectors and the oracle at 1e-3 of the shift's magnitude (the
reference's own fp32 solve differs from the fp64 one by about 6e-5 of it), after checking
that it ends the same way: same iteration count and the same return code of
bicgstab_shifting. Components at the clamp (threshold dx) agree exactly.
"""
import copy

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from golden_io import load_case, rel_max  # noqa: E402
from oracle import sph_oracle as O  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402

IPS_CASES = ["tgv24_jitter", "fourier20", "dambreak16"]
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


def _ips(cfg):
    c = copy.deepcopy(cfg)
    c["shifting"]["scheme"] = "IPS"
    return c


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


@pytest.mark.parametrize("case", IPS_CASES)
def test_ips_shift_matches_reference_vectors(case):
    """solveShifting with scheme 'IPS' on the reference's own inputs (golden vectors)."""
    z, cfg, st = load_case(f"ips_{case}")
    assert cfg["shifting"]["scheme"] == "IPS"
    sol = _solver(cfg, st)
    dx = _np(sol.shift())
    sol.check()
    it, code = sol.ips_result()
    info = {}
    O.solve_shifting(copy.deepcopy(st), cfg, info)
    assert code == int(z["ips/iterations"]) == info["code"]
    assert it == info["iterations"]
    assert rel_max(dx, z["ips/shift"]) < TOL
    thr = 0.05 * float(cfg["particle"]["dx"])
    at_clamp = np.abs(z["ips/shift"]) >= thr * (1 - 1e-6)
    assert np.all(np.abs(dx[at_clamp] - z["ips/shift"][at_clamp]) <= 2e-7 + 1e-6 * thr)


@pytest.mark.parametrize("scene", ["fourier_periodic", "dam_break"])
def test_ips_step_matches_oracle(scene):
    """One fused step (integrate + implicit shift) against the oracle's full step."""
    if scene == "fourier_periodic":
        cfg, st = scenes.fourier_periodic(64, seed=2, jitter=0.1)
    else:
        cfg, st = scenes.dam_break(dx=1.0 / 32)
    cfg = _ips(cfg)
    r32, _ = O.full_step(copy.deepcopy(st), cfg)
    r64, _ = O.full_step(_as64(st), cfg)
    sol = _solver(cfg, st)
    sol.step(1)
    sol.check()
    got = sol.download()
    a, b = r32["fluid"], r64["fluid"]
    assert_fp32_parity(_np(got["velocities"]), a["velocities"], b["velocities"], 1e-4, "velocities")
    assert_fp32_parity(_np(got["densities"]), a["densities"], b["densities"], 1e-5, "densities")
    x0 = st["fluid"]["positions"]
    assert_fp32_parity(_np(got["positions"]) - x0, a["positions"] - x0, b["positions"] - x0, TOL, "x' - x")
    # the integrate half alone (no shift) is the solver's usual step: the shifts differ
    cfg_d = copy.deepcopy(cfg)
    cfg_d["shifting"]["scheme"] = "deltaSPH"
    d = _solver(cfg_d, st)
    d.step(1)
    gd = d.download()
    assert torch.equal(gd["velocities"], got["velocities"])
    assert not torch.equal(gd["positions"], got["positions"])


def test_ips_larger_periodic_shift_matches_oracle():
    """A 128 x 128 jittered periodic flow (16,384 particles): one implicit shift against the
    fp32 and fp64 oracle solves, which end at the same iteration."""
    cfg, st = scenes.fourier_periodic(128, seed=4, jitter=0.1)
    cfg = _ips(cfg)
    i32, i64 = {}, {}
    d32, _ = O.solve_shifting(copy.deepcopy(st), cfg, i32)
    d64, _ = O.solve_shifting(_as64(st), cfg, i64)
    sol = _solver(cfg, st)
    dx = _np(sol.shift())
    it, code = sol.ips_result()
    assert (it, code) == (i32["iterations"], i32["code"])
    assert_fp32_parity(dx, d32, d64, TOL, "shift")


def test_ips_five_steps_track_oracle():
    cfg, st = scenes.fourier_periodic(48, seed=6, jitter=0.1)
    cfg = _ips(cfg)
    s = copy.deepcopy(st)
    for _ in range(5):
        s, _ = O.full_step(s, cfg)
    sol = _solver(cfg, st)
    sol.step(5)
    sol.check()
    got = sol.download()
    assert rel_max(_np(got["velocities"]), s["fluid"]["velocities"]) < 1e-3
    x0 = st["fluid"]["positions"]
    assert rel_max(_np(got["positions"]) - x0, s["fluid"]["positions"] - x0) < 1e-3


def test_ips_graph_replay_equals_eager_steps():
    """A captured step holds every iteration (those after the solve returned do nothing);
    the eager step stops launching instead. Both give the same state bit for bit."""
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    cfg = _ips(cfg)
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


def test_ips_zero_iterations_and_switching_back():
    """maxSolveIter = 0 returns x = 0 (no shift); set_ips(None) restores delta+."""
    cfg, st = scenes.fourier_periodic(32, seed=1, jitter=0.1)
    a = _solver(cfg, st)
    a.set_ips(max_iter=0)
    dx = a.shift()
    assert float(dx.abs().max()) == 0.0
    assert a.ips_result() == (0, 0)
    b = _solver(cfg, st)
    b.set_ips()
    b.set_ips(None)
    c = _solver(cfg, st)
    assert torch.equal(b.shift(), c.shift())
