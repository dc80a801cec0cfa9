"""Operator-level drop-ins (diffsph_gb300.ops) against the reference's own outputs.

* The generic sphOperationStates on the GPU against the reference's sphOperationStates for
  every operation and mode (tests/golden/make_ops_golden.py, jittered periodic case).
* Each module function against the per-stage intermediates the reference's simulationStep
  left in the golden files (tests/golden/make_golden.py), called the way simulationStep
  calls them (callModule directions: fluid, boundary -> fluid), walls included.

Each query row sums its pairs in the reference's order with the reference's fp32 operation
order, so the results agree to a few ulps; the tolerance is 2e-6 of the field's magnitude
(``rel_max``). The mDBC wall density solves its 3x3 system in fp64 where the reference uses
an fp32 pseudo-inverse: its Shepard densities are held to 2e-6, the extrapolated densities
to |gpu - o64| <= 4 |ref32 - o64| + 1e-5 max|o64|.
"""
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from golden_io import GOLDEN, CASES, load_case, rel_max  # noqa: E402
from oracle import sph_oracle as O  # noqa: E402

TOL = 2e-6


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from diffsph_gb300 import _lib
    _lib.load()


def _np(t):
    return t.detach().cpu().numpy()


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _state(arrs, **extra):
    s = {k: _t(v) for k, v in arrs.items()}
    s.update({k: _t(v) for k, v in extra.items()})
    s["numParticles"] = int(arrs["positions"].shape[0])
    return s


def _golden_nb(z):
    nb = {"indices": (_t(z["nb/i"]), _t(z["nb/j"]))}
    for k in ("distances", "vectors", "supports", "kernels", "gradients", "numNeighbors", "neighborOffsets"):
        nb[k] = _t(z[f"nb/{k}"])
    return nb


def test_generic_operations_match_the_reference():
    from diffsph_gb300 import ops
    sys.path.insert(0, GOLDEN)
    import make_ops_golden as G  # the generator's case list and quantities
    g = np.load(os.path.join(GOLDEN, "ops_tgv24.npz"))
    z, cfg, st = load_case("tgv24_jitter_wrap")
    fl = _state(st["fluid"])
    nb = _golden_nb(z)
    qs = {k: _t(v) for k, v in G.quantities(st).items()}
    dist, sup, vec = z["nb/distances"], z["nb/supports"], z["nb/vectors"]
    pair_q = _t(-(dist * sup)[:, None] * vec)
    worst = {}
    for name, op, mode, dm, q in G.cases():
        quant = None if q is None else (pair_q if q == "pair" else (qs[q], qs[q]))
        got = ops.sphOperationStates(fl, fl, quant, nb, operation=op, gradientMode=mode, divergenceMode=dm)
        ref = g[f"out/{name}"]
        assert tuple(got.shape) == ref.shape, name
        err = rel_max(_np(got), ref)
        worst[name] = err
        assert err < TOL, f"{name}: {err:.2e}"
    print("largest relative error:", max(worst.values()), max(worst, key=worst.get))


@pytest.mark.parametrize("name", CASES)
def test_module_functions_match_the_reference_intermediates(name):
    from diffsph_gb300 import ops
    from diffsph_gb300.neighborhood import neighborSearch
    z, cfg, st = load_case(name)
    rhs = {k[4:]: z[k] for k in z.files if k.startswith("rhs/")}
    fl = _state(st["fluid"], L=rhs["L"], **{"gradRho^L": rhs["gradRho^L"], "pressures": rhs["pressures"]})
    nb = _golden_nb(z)
    walls = "boundary" in st
    if walls:
        bd_np = dict(st["boundary"])
        bd_np["densities"] = rhs["boundary_densities"]
        bd_np["pressures"] = O.stiff_tait_eos(bd_np, cfg)
        bd = _state(bd_np)
        _, btf = neighborSearch({k: v for k, v in fl.items()}, bd, cfg)

    def both(fn, *a, boundary_fn=None):
        out = fn(fl, fl, nb, cfg, *a)
        if walls:
            out = out + (boundary_fn or fn)(fl, bd, btf, cfg, *a)
        return out

    # normalisation matrices, 'fluidwBoundary' (deltaPlus.py:240-252)
    M = both(ops.computeCovarianceMatrices)
    M[_t(z["nb/numNeighbors"]) < 4] = torch.eye(2, device="cuda")
    assert rel_max(_np(M), rhs["covarianceMatrix"]) < TOL
    # renormalised density gradient (+ the boundary part, deltaPlus.py:256-262)
    g = ops.renormalizedDensityGradient(fl, fl, nb, cfg)
    if walls:
        g = g + ops.densityGradient(fl, bd, btf, cfg)
    assert rel_max(_np(g), rhs["gradRho^L"]) < TOL
    # density diffusion (fluid), viscosity, continuity, pressure, gravity (deltaPlus.py:266-341)
    assert rel_max(_np(ops.computeDensityDeltaTerm(fl, fl, nb, cfg)), rhs["densityDiffusion"]) < TOL
    visc = both(ops.computeViscosity, boundary_fn=ops.computeViscosity_Boundary)
    assert rel_max(_np(visc), rhs["velocityDiffusion"]) < TOL
    assert rel_max(_np(both(ops.computeMomentumEquation)), rhs["momentumEquation"]) < TOL
    assert rel_max(_np(both(ops.computePressureAccel)), rhs["pressureAccel"]) < TOL
    assert rel_max(_np(ops.computeGravity(fl, cfg)), rhs["gravityAccel"]) == 0.0


def test_density_summation_matches_the_reference():
    """computeDensity on both directions ('all': ftf + btf) against the summation densities the
    reference's simulationStep wrote (dambreak16_summation)."""
    from diffsph_gb300 import ops
    from diffsph_gb300.neighborhood import neighborSearch
    z, cfg, st = load_case("dambreak16_summation")
    fl = _state(st["fluid"])
    bd = _state(st["boundary"])
    _, ftf = neighborSearch(fl, fl, cfg)
    _, btf = neighborSearch(fl, bd, cfg)
    rho = ops.computeDensity(fl, fl, ftf, cfg) + ops.computeDensity(fl, bd, btf, cfg)
    assert rel_max(_np(rho), z["rhs/densities"]) < TOL


def test_mdbc_density_matches_the_reference():
    from diffsph_gb300 import ops
    from diffsph_gb300.neighborhood import neighborSearch
    z, cfg, st = load_case("dambreak16")
    fl, bd_np = st["fluid"], st["boundary"]
    ghost_x = O.boundary_ghosts(bd_np, cfg)
    assert np.array_equal(ghost_x, z["rhs/ghost_positions"])
    ghost = _state({k: bd_np[k] for k in ("masses", "supports", "densities", "velocities", "areas")} |
                   {"positions": ghost_x})
    fls = _state(fl)
    _, gnb = neighborSearch(ghost, fls, cfg)
    assert np.array_equal(_np(gnb["numNeighbors"]), z["rhs/ghost_numNeighbors"])
    ghost["neighborhood"] = gnb
    state = {"fluid": fls, "boundary": _state(bd_np), "boundaryGhost": ghost}
    rho, shep = ops.mDBCDensity(state, cfg)
    assert rel_max(_np(shep), z["rhs/ghost_shepard"]) < TOL
    s64 = {p: {k: (v.astype(np.float64) if v.dtype == np.float32 else v.copy()) for k, v in a.items()}
           for p, a in st.items()}
    o64, _, _ = O.mdbc_density(s64["boundary"], s64["fluid"], cfg)
    e_gpu = float(np.max(np.abs(_np(rho) - o64)))
    e_ref = float(np.max(np.abs(z["rhs/boundary_densities"] - o64)))
    assert e_gpu <= 4 * e_ref + 1e-5 * float(np.max(np.abs(o64)))


def test_operator_argument_errors():
    from diffsph_gb300 import ops
    z, cfg, st = load_case("tgv16_lattice")
    fl = _state(st["fluid"])
    nb = _golden_nb(z)
    with pytest.raises(ValueError):
        ops.sphOperationStates(fl, fl, (fl["densities"], fl["densities"]), nb, operation="divergence")
    with pytest.raises(ValueError):
        ops.sphOperationStates(fl, fl, (fl["densities"], fl["densities"]), nb, operation="laplacian",
                               gradientMode="naive")
    bad = dict(cfg)
    bad["diffusion"] = dict(cfg["diffusion"], velocityScheme="Monaghan1992")
    with pytest.raises(ValueError):
        ops.computeViscosity(fl, fl, nb, bad)
