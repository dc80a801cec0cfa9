"""Known answers of the SPH operators, written from the reference's formulas and checked on
the oracle in fp64.

- Kernel gradients are antisymmetric: grad W_ij = -grad W_ji, bit for bit. Both x_i - x_j
  and the periodic minimum image (src/diffSPH/v2/math.py:5-6) are odd in the difference.
- With uniform supports the pair sums of the density diffusion (densityDiffusion.py:49-73)
  and of the symmetric pressure gradient (pressureForce.py:10-12) are antisymmetric, and so
  is the viscid viscosity (viscosity.py:200-218): sum_i V_i D_i = 0, sum_i m_i a_i = 0.
- On a uniform lattice the normalisation matrix (normalizationMatrices.py:18-23) is
  isotropic, so L = c I, with c within 1e-3 of 1 at h = 4 dx.
- The Tait equation of state (pressureEOS.py:5-11) inverts in closed form:
  rho = rho0 (1 + gamma p / (rho0 c0^2))^(1 / gamma).
- Density summation on a uniform lattice is the kernel's lattice sum.
"""
import copy

import numpy as np
import pytest

from golden_io import load_case
from oracle import sph_oracle as O


def _as64(st):
    return {p: {k: (v.astype(np.float64) if v.dtype == np.float32 else v.copy()) for k, v in a.items()}
            for p, a in st.items()}


def _rhs(case, uniform_density=False):
    _, cfg, st = load_case(case)
    s = _as64(st)
    if uniform_density:
        s["fluid"]["densities"][:] = float(cfg["fluid"]["rho0"])
    O.simulation_step(s, cfg)
    return cfg, s["fluid"]


@pytest.mark.parametrize("case", ["tgv16_lattice", "tgv24_jitter_wrap", "fourier20"])
def test_kernel_gradient_is_antisymmetric(case):
    _, cfg, st = load_case(case)
    nb = O.neighbor_search(st["fluid"], st["fluid"], cfg)
    i, j = nb["indices"]
    n = st["fluid"]["positions"].shape[0]
    key = i.astype(np.int64) * n + j
    rev = np.searchsorted(key, j.astype(np.int64) * n + i)
    assert np.array_equal(key[rev], j.astype(np.int64) * n + i)
    assert np.array_equal(nb["gradients"][rev], -nb["gradients"])
    assert np.array_equal(nb["kernels"][rev], nb["kernels"])


@pytest.mark.parametrize("case", ["tgv16_lattice", "tgv24_jitter_wrap", "fourier20"])
def test_pair_sums_conserve_mass_and_momentum(case):
    _, fl = _rhs(case)
    V = fl["masses"] / fl["densities"]
    vd = V * fl["densityDiffusion"]
    assert abs(vd.sum()) <= 1e-12 * np.abs(vd).sum()
    m = fl["masses"][:, None]
    for k in ("pressureAccel", "velocityDiffusion"):
        f = m * fl[k]
        assert np.all(np.abs(f.sum(0)) <= 1e-12 * np.abs(f).sum(0) + 1e-300), k


def test_normalisation_matrix_is_isotropic_on_a_uniform_lattice():
    _, fl = _rhs("tgv16_lattice", uniform_density=True)
    L = fl["L"]
    c = L[:, 0, 0]
    assert np.max(np.abs(L[:, 0, 1])) < 1e-6 and np.max(np.abs(L[:, 1, 0])) < 1e-6
    assert np.max(np.abs(L[:, 1, 1] - c)) < 1e-6
    assert np.max(np.abs(c - 1.0)) < 1e-3
    # a uniform density has no gradient and drives no diffusion
    assert np.max(np.abs(fl["gradRho^L"])) < 1e-12
    assert np.max(np.abs(fl["densityDiffusion"])) < 1e-12


def test_tait_equation_of_state_round_trip():
    _, cfg, _ = load_case("tgv16_lattice")
    rho0, cs = float(cfg["fluid"]["rho0"]), float(cfg["fluid"]["cs"])
    gamma = float(cfg["EOS"]["polytropicExponent"])
    p = np.linspace(-0.2, 0.2, 101) * rho0 * cs ** 2 / gamma
    rho = rho0 * (1 + gamma * p / (rho0 * cs ** 2)) ** (1 / gamma)
    back = O.stiff_tait_eos({"densities": rho}, cfg)
    assert np.max(np.abs(back - p)) < 1e-12 * rho0 * cs ** 2
    assert O.stiff_tait_eos({"densities": np.array([rho0])}, cfg)[0] == 0.0


@pytest.mark.parametrize("nx", [16, 64])
def test_lattice_density_is_the_kernel_lattice_sum(nx):
    """Density summation (density.py:6-15) on a uniform periodic lattice with h = 4 dx is
    the same at every particle: rho0 sum_{|k| <= 4} W(|k| / 4) dx^2 over the integer offsets
    k, 1.0012058 rho0 for the Wendland C2 kernel, whatever the resolution."""
    from diffsph_gb300 import scenes
    cfg, st = scenes.taylor_green(nx)
    fl = _as64(st)["fluid"]
    nb = O.neighbor_search(fl, fl, cfg)
    rho = O.compute_density(fl, fl, nb, cfg)
    k = np.arange(-4, 5)
    I, J = np.meshgrid(k, k)
    q = np.sqrt(I ** 2 + J ** 2) / 4.0
    lattice = np.sum(np.where(q <= 1, (1 - q) ** 4 * (1 + 4 * q), 0.0)) * 7 / np.pi / 16
    rho0 = float(cfg["fluid"]["rho0"])
    assert abs(lattice - 1.0012058) < 1e-7
    assert np.max(np.abs(rho - lattice * rho0)) < 1e-12 * rho0


def test_workload_time_steps_are_the_acoustic_limit():
    """The workloads step at the acoustic limit of computeTimestep (timestep.py:18),
    dt = CFL h / (c0 kappa) with CFL 0.3, h = 4 dx, kappa = 2: 0.6 dx / c0. For the
    Taylor-Green vortex c0 = 10 (10 max|u|), dt = 1.875e-3 at 64^2; for the dam break
    c0 = 10 sqrt(2 g H) with a 2 m column, dt = 3.74e-5 at dx = 1/256 and 9.35e-6 at 1/1024."""
    import math
    from diffsph_gb300 import scenes
    cfg, _ = scenes.taylor_green(64)
    assert cfg["timestep"]["dt"] == pytest.approx(1.875e-3, rel=1e-12)
    assert cfg["timestep"]["dt"] == pytest.approx(O.acoustic_timestep(cfg, 0.3), rel=1e-12)
    c0 = 10 * math.sqrt(2 * 9.81 * 2.0)
    for dx, dt in ((1 / 256, 3.7415e-5), (1 / 1024, 9.3538e-6)):
        cfg, _ = scenes.dam_break(dx=dx)
        assert cfg["fluid"]["cs"] == pytest.approx(c0, rel=1e-12)
        assert cfg["timestep"]["dt"] == pytest.approx(0.6 * dx / c0, rel=1e-12)
        assert cfg["timestep"]["dt"] == pytest.approx(dt, rel=1e-4)
        assert cfg["timestep"]["dt"] == pytest.approx(O.acoustic_timestep(cfg, 0.3), rel=1e-12)
