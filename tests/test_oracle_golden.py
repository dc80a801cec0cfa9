"""Pins the CPU oracle against vectors produced by running the reference itself.

The golden files come from tests/golden/make_golden.py (reference v2 torch code on CPU).
Tolerances are relative to the magnitude of each field (max |a-b| / max |b|).
"""
import copy

import numpy as np
import pytest

from golden_io import CASES, load_case, rel_max
from oracle import sph_oracle as O

TGV_CASES = [c for c in CASES if not c.startswith("dambreak")]


def _sorted_pairs(i, j):
    o = np.lexsort((j, i))
    return i[o], j[o]


@pytest.mark.parametrize("case", CASES)
def test_neighbor_set_bit_exact(case):
    z, cfg, st = load_case(case)
    nb = O.neighbor_search(st["fluid"], st["fluid"], cfg)
    i, j = nb["indices"]
    ri, rj = _sorted_pairs(z["nb/i"], z["nb/j"])
    assert np.array_equal(i, ri) and np.array_equal(j, rj)
    # the filtered geometry follows the reference's fp32 operation order exactly
    assert np.array_equal(nb["distances"], z["nb/distances"])
    assert np.array_equal(nb["vectors"], z["nb/vectors"])
    assert np.array_equal(nb["numNeighbors"], z["nb/numNeighbors"])
    assert np.array_equal(nb["neighborOffsets"], z["nb/neighborOffsets"])
    assert rel_max(nb["kernels"], z["nb/kernels"]) < 1e-6
    assert rel_max(nb["gradients"], z["nb/gradients"]) < 1e-6


def test_lattice_has_pairs_at_exactly_h():
    z, cfg, st = load_case("tgv16_lattice")
    q = z["nb/distances"]
    assert np.sum(q == 1.0) == 4 * st["fluid"]["positions"].shape[0]


@pytest.mark.parametrize("case", TGV_CASES)
def test_rhs_fields(case):
    z, cfg, st = load_case(case)
    s = copy.deepcopy(st)
    (u, dudt, drhodt), _ = O.simulation_step(s, cfg)
    fl = s["fluid"]
    for k in ("covarianceMatrix", "L", "gradRho^L", "densityDiffusion", "velocityDiffusion",
              "momentumEquation", "pressures", "pressureAccel"):
        assert rel_max(fl[k], z[f"rhs/{k}"]) < 1e-5, k
    assert rel_max(dudt, z["rhs/dudt"]) < 1e-5
    assert rel_max(drhodt, z["rhs/drhodt"]) < 1e-5


@pytest.mark.parametrize("case", TGV_CASES)
def test_full_step(case):
    z, cfg, st = load_case(case)
    out, _ = O.full_step(copy.deepcopy(st), cfg)
    f = out["fluid"]
    assert rel_max(f["velocities"], z["step/velocities"]) < 1e-6
    # the reference ends the symplectic Euler step on the half-step density
    assert rel_max(f["densities"], z["step/densities"]) < 1e-6
    # positions: within a few fp32 ulps of |x| ~ 1
    assert np.max(np.abs(f["positions"] - z["step/positions"])) < 5e-7
    assert np.max(np.abs(f["shiftAmount"] - z["step/shift"])) < 5e-7


def test_mdbc_boundary_density_against_reference_pinv():
    z, cfg, st = load_case("dambreak16")
    cfg["oracle"] = {"pinv": "torch"}
    s = copy.deepcopy(st)
    O.simulation_step(s, cfg)
    assert rel_max(s["boundary"]["densities"], z["rhs/boundary_densities"]) < 1e-5
    assert np.array_equal(s["boundaryGhost"]["neighborhood"]["numNeighbors"], z["rhs/ghost_numNeighbors"])
    assert rel_max(s["boundaryGhost"]["densities"], z["rhs/ghost_shepard"]) < 1e-5


def test_dambreak_fluid_fields_given_reference_boundary_density(monkeypatch):
    """With the reference's mDBC densities substituted, every fluid field of the
    boundary-coupled right-hand side matches to 1e-5 of its magnitude."""
    z, cfg, st = load_case("dambreak16")
    orig = O.mdbc_density

    def fixed(bd, fl, config, ghost_nb=None):
        _, shep, nb = orig(bd, fl, config, ghost_nb)
        return z["rhs/boundary_densities"].copy(), shep, nb

    monkeypatch.setattr(O, "mdbc_density", fixed)
    s = copy.deepcopy(st)
    (u, dudt, drhodt), _ = O.simulation_step(s, cfg)
    fl = s["fluid"]
    for k in ("covarianceMatrix", "L", "gradRho^L", "densityDiffusion", "velocityDiffusion",
              "momentumEquation", "pressures", "pressureAccel"):
        assert rel_max(fl[k], z[f"rhs/{k}"]) < 1e-5, k
    assert rel_max(dudt, z["rhs/dudt"]) < 1e-5


def test_dambreak_step_end_to_end():
    """Unpatched dam-break step. The mDBC moment matrices reach condition numbers ~1e4,
    so the reference's fp32 solve carries ~1e-6 relative noise in the boundary density,
    which the delta-diffusion term (a near-cancelling sum) amplifies."""
    z, cfg, st = load_case("dambreak16")
    cfg["oracle"] = {"pinv": "torch"}
    out, _ = O.integrate_symplectic_euler(copy.deepcopy(st), cfg)
    assert rel_max(out["fluid"]["velocities"], z["step/velocities"]) < 2e-4
    assert rel_max(out["fluid"]["densities"], z["step/densities"]) < 1e-6
    assert rel_max(out["boundary"]["densities"], z["step/boundary_densities"]) < 1e-5


def test_pinv2x2_matches_numpy_pinv_when_well_conditioned():
    """The reference's closed form (math.py:11-57) regularises the smaller singular
    value by 1e-7 (an error ~5e-8 / sigma_min^3), so it equals the pseudo-inverse for
    well-conditioned matrices."""
    rng = np.random.default_rng(0)
    M = np.eye(2)[None] * rng.uniform(0.5, 2.0, size=(1000, 1, 1)) + 0.05 * rng.normal(size=(1000, 2, 2))
    assert np.min(np.linalg.svd(M)[1]) > 0.3
    assert np.allclose(O.pinv2x2(M), np.linalg.pinv(M), rtol=1e-6, atol=1e-6)


def test_wendland_normalisation():
    """integral of W over the disc of radius h equals 1 (2D, C_d = 7/pi)."""
    h = 0.37
    r = np.linspace(0, h, 200001)
    q = r / h
    W = O.wendland_kernel(q, np.float64(h))
    integral = np.trapezoid(W * 2 * np.pi * r, r)
    assert abs(integral - 1.0) < 1e-8


IPS_CASES = ["tgv24_jitter", "fourier20", "dambreak16"]


@pytest.mark.parametrize("case", IPS_CASES)
def test_ips_shift_against_reference(case):
    """Implicit particle shifting (shifting.scheme 'IPS'): the oracle's BiCGStab solve ends
    the way the reference's does (same return code) with the same shift."""
    z, cfg, st = load_case(f"ips_{case}")
    info = {}
    dx, _ = O.solve_shifting(copy.deepcopy(st), cfg, info)
    assert info["code"] == int(z["ips/iterations"])
    # the reference's right-hand side B = sum grad W omega_j (interleaved, wall rows zero)
    ps_n = st["fluid"]["positions"].shape[0]
    assert rel_max(dx, z["ips/shift"]) < 1e-4
    assert dx.shape == z["ips/shift"].shape and ps_n == dx.shape[0]


FS_CASES = ["dambreak32_dplus", "dambreak32_ips", "dambreak24_jitter_dplus"]


@pytest.mark.parametrize("case", FS_CASES)
def test_free_surface_shift_against_reference(case):
    """solveShifting with shifting.freeSurface: the oracle's surface flags and expanded mask
    equal the reference's, its Lambdas and fluid normals agree to rounding, and so does the
    shift (the IPS case ends with the reference's return code)."""
    z, cfg, st = load_case(f"fs_{case}")
    info = {}
    dx, _ = O.solve_shifting(copy.deepcopy(st), cfg, info)
    nF = st["fluid"]["positions"].shape[0]
    assert np.array_equal(info["freeSurface"], z["fs/freeSurface"])
    assert np.array_equal(info["freeSurfaceMask"], z["fs/freeSurfaceMask"])
    assert rel_max(info["Lambdas"], z["fs/Lambdas"]) < 1e-5
    # normals of vanishing lambda gradients (wall rows deep in the wall) are rounding noise
    assert rel_max(info["normals"][:nF], z["fs/lambdaGrad"][:nF]) < 1e-3
    assert rel_max(dx, z["fs/shift"]) < 1e-3
    if "code" in info:
        assert info["code"] == -12 or info["code"] >= 0


def test_pressure_switch_against_reference():
    """computePressureAccelSwitch on the reference's own state, neighborhoods and surface mask."""
    import os
    from golden_io import GOLDEN
    z = np.load(os.path.join(GOLDEN, "switch_dambreak32.npz"))
    fl = {k: z[f"fluid/{k}"] for k in ("densities", "masses", "pressures", "surfaceMask")}
    bd = {k: z[f"boundary/{k}"] for k in ("densities", "masses", "pressures")}
    for name, sB in (("ff", fl), ("fb", bd)):
        nb = {"indices": (z[f"{name}/i"], z[f"{name}/j"]), "gradients": z[f"{name}/gradients"]}
        got = O.pressure_accel_switch(fl, sB, nb, None)
        assert rel_max(got, z[f"{name}/accel"]) < 1e-6, name
    assert np.any(fl["pressures"] < 0) and np.any(fl["surfaceMask"] > 0.5)


def test_liuliu_consistent_against_reference():
    """LiuLiuConsistent on the reference's mirror-outlet ghosts (buildOutletGhostParticles)."""
    import os
    from golden_io import GOLDEN
    z = np.load(os.path.join(GOLDEN, "regions_block32.npz"))
    fluid = {k: z[f"in/fluid/{k}"] for k in ("positions", "velocities", "densities", "masses")}
    ghost = {"positions": z["ghost/positions"]}
    nb = {"indices": (z["ghost/i"], z["ghost/j"]), "distances": z["ghost/nb_distances"],
          "vectors": z["ghost/nb_vectors"], "supports": z["ghost/nb_supports"], "kernels": z["ghost/nb_kernels"],
          "gradients": z["ghost/nb_gradients"]}
    for name, q in (("rho", fluid["densities"]), ("u", fluid["velocities"][:, 0]), ("v", fluid["velocities"][:, 1])):
        sol, M, b = O.liuliu_consistent(ghost, fluid, nb, q)
        assert rel_max(M, z[f"liuliu/{name}/M"]) < 1e-5, name
        assert rel_max(b, z[f"liuliu/{name}/b"]) < 1e-5, name
        assert rel_max(sol, z[f"liuliu/{name}/solution"]) < 1e-3, name


def test_pinv2x2_edge_cases_against_reference():
    """The reference's closed-form pinv2x2 (math.py:11-57) on 183 fp32 matrices
    (tests/golden/make_pinv_golden.py): general, zero, near-singular (condition up to 1e5,
    where the 1e-7 floor replaces the smaller singular value), negative-determinant, diagonal,
    symmetric, rotation and normalisation-like matrices agree within 1e-6 of each result's
    magnitude, and the singular values of all of them within 1e-6. The 32 rank-1 matrices are
    compared by their singular values only: there S1 - S2 cancels to rounding noise and the
    sign s22 of a cancelling sum picks the direction of the floored value, so L is noise in
    any fp32 evaluation, the reference's included."""
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pinv2x2_cases.npz"))
    M, L, ev = z["M"], z["L"], z["eigVals"]
    Lo, evo = O.pinv2x2(M.copy(), eigenvalues=True)
    n = M.shape[0]
    rank1 = np.zeros(n, bool)
    rank1[64:96] = True
    assert np.linalg.matrix_rank(M[rank1].astype(np.float64), tol=1e-5).max() == 1
    err = np.abs(Lo - L).reshape(n, -1).max(1) / np.maximum(np.abs(L).reshape(n, -1).max(1), 1e-30)
    assert err[~rank1].max() < 1e-6
    assert np.array_equal(L[96:100], np.zeros_like(L[96:100]))  # the zero matrix maps to zero
    assert np.array_equal(Lo[96:100], L[96:100])
    ev_err = np.abs(evo - ev).max(1) / np.abs(ev).max(1)
    assert ev_err.max() < 1e-6


@pytest.mark.parametrize("name", ["tgv24_summation", "dambreak16_summation"])
def test_summation_density_against_reference(name):
    """simulation.densityScheme 'summation' (deltaPlus.py:193-198): the summed densities, the
    rates they feed and the step (whose densities are the sums at the half-step positions)
    against the reference's run of the same case."""
    z, cfg, st = load_case(name)
    cfg["oracle"] = {"pinv": "torch"}
    s = copy.deepcopy(st)
    (_, dudt, drhodt), _ = O.simulation_step(s, cfg)
    assert rel_max(s["fluid"]["densities"], z["rhs/densities"]) < 1e-6
    out, _ = O.full_step(copy.deepcopy(st), cfg)
    assert rel_max(out["fluid"]["densities"], z["step/densities"]) < 1e-6
    if "boundary" not in st:
        assert rel_max(dudt, z["rhs/dudt"]) < 1e-5
        assert rel_max(drhodt, z["rhs/drhodt"]) < 1e-5
        assert rel_max(out["fluid"]["velocities"], z["step/velocities"]) < 1e-6


@pytest.mark.parametrize("name", ["dambreak32", "dambreak16_summation"])
def test_walled_fluid_fields_given_reference_walls(name, monkeypatch):
    """With the reference's wall densities substituted, the walled right-hand side matches
    the reference's to 1e-5 of each field's magnitude (the GPU twin of this check calls
    sph_solver_rhs_walls)."""
    z, cfg, st = load_case(name)
    orig = O.mdbc_density

    def fixed(bd, fl, config, ghost_nb=None):
        _, shep, nb = orig(bd, fl, config, ghost_nb)
        return z["rhs/boundary_densities"].copy(), shep, nb

    monkeypatch.setattr(O, "mdbc_density", fixed)
    s = copy.deepcopy(st)
    (_, dudt, drhodt), _ = O.simulation_step(s, cfg)
    assert rel_max(s["fluid"]["gradRho^L"], z["rhs/gradRho^L"]) < 1e-5
    assert rel_max(drhodt, z["rhs/drhodt"]) < 1e-5
    assert rel_max(dudt, z["rhs/dudt"]) < 1e-5
