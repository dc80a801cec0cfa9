"""Operator-level drop-ins: the reference's pair operators and module functions on the GPU.

Same signatures and return values as:

* ``sphOperation(...)``, ``sphOperationStates(...)``     src/diffSPH/v2/sphOps.py:243-303
* ``computeDensity``                                     src/diffSPH/v2/modules/density.py:6-15
* ``computeCovarianceMatrices``                          src/diffSPH/v2/modules/normalizationMatrices.py:18-23
* ``renormalizedDensityGradient``, ``densityGradient``,
  ``computeDensityDeltaTerm``                            src/diffSPH/v2/modules/densityDiffusion.py:7-73
* ``computeMomentumEquation``                            src/diffSPH/v2/modules/momentumEquation.py:6-39
* ``computePressureAccel``                               src/diffSPH/v2/modules/pressureForce.py:10-12
* ``computeViscosity``                                   src/diffSPH/v2/modules/viscosity.py:222-241
* ``computeViscosity_Boundary``                          src/diffSPH/v2/modules/boundaryViscosity.py (its dispatcher)
* ``computeGravity``                                     src/diffSPH/v2/modules/gravity.py:8-29
* ``mDBCDensity``                                        src/diffSPH/v2/modules/mDBC.py:50-163

Each takes the reference's state dicts and a neighborhood in its format (what
``neighborSearch`` returns: pairs sorted by query index with ``neighborOffsets`` and
``numNeighbors``) and runs one sm_103a kernel of libsph103.so (``sph_operation``,
``sph_covariance``, ...; include/sph103.h). Every query row sums its pairs in the stored
order with the reference's fp32 operation order, so the results follow the reference's own
arithmetic. Inputs on another device are copied to the GPU; results come back on the
device of the query state's tensors. Schemes the kernels do not implement raise
``ValueError``; there is no fallback to any other implementation.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib

OPERATIONS = {"density": 0, "interpolate": 1, "gradient": 2, "divergence": 3, "curl": 4, "laplacian": 5}
MODES = {"naive": 0, "difference": 1, "summation": 2, "symmetric": 3, "conserving": 4, "divergenceFree": 5,
         "dot": 6}


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _dev(t, dtype=torch.float32):
    if t is None:
        return None
    return torch.as_tensor(t).to(device="cuda", dtype=dtype).contiguous()


def _f(x) -> float:
    if isinstance(x, torch.Tensor):
        return float(x.detach().cpu().reshape(-1)[0])
    return float(x)


class _Pairs:
    """sph_pairs_t over a reference-format neighborhood (keeps the device copies alive)."""

    def __init__(self, neighborhood, n_query, need=("distances", "vectors", "supports", "kernels", "gradients")):
        i, j = neighborhood["indices"]
        self.keep = {
            "offsets": _dev(neighborhood["neighborOffsets"], torch.int32),
            "counts": _dev(neighborhood["numNeighbors"], torch.int32),
            "pair_j": _dev(j, torch.int64),
        }
        for k in need:
            self.keep[k] = _dev(neighborhood[k]) if k in neighborhood else None
        if self.keep["counts"].numel() != n_query:
            raise ValueError("the neighborhood's numNeighbors must have one entry per query particle")
        s = _lib.Pairs()
        s.n_query = int(n_query)
        for k in ("offsets", "counts", "pair_j", "distances", "vectors", "supports", "kernels", "gradients"):
            setattr(s, k, _ptr(self.keep.get(k)))
        self.s = s

    def ref(self):
        return ctypes.byref(self.s)


def _components(t):
    """Per-entry value count of a quantity tensor ([n], [n, 2] or [n, 2, 2])."""
    if t.dim() == 1:
        return 1
    c = 1
    for d in t.shape[1:]:
        c *= int(d)
    if c not in (1, 2, 4) or (c == 4 and tuple(t.shape[1:]) != (2, 2)):
        raise ValueError(f"quantities of shape {tuple(t.shape)} are not supported (scalars, 2-vectors, 2x2 matrices)")
    return c


def _out_shape(n, op, C, qshape):
    if op == "density" or op == "curl":
        return (n,)
    if op in ("interpolate", "laplacian"):
        return (n,) + tuple(qshape[1:])
    if op == "gradient":
        return (n,) + tuple(qshape[1:]) + (2,)
    if op == "divergence":
        return (n,) if C == 2 else (n, 2)
    raise ValueError(op)


def sphOperation(masses, densities, quantities, neighborhood, kernels, kernelGradients, radialDistances, directions,
                 supports, numParticles, operation="interpolate", gradientMode="symmetric", divergenceMode="div",
                 kernelLaplacians=None):
    """sphOperation (sphOps.py:243-275) on the GPU. ``neighborhood`` is the (i, j) index pair as
    in the reference; the CSR offsets are derived from it (pairs sorted by i)."""
    i = torch.as_tensor(neighborhood[0])
    counts = torch.bincount(i.to(torch.int64), minlength=int(numParticles)).to(torch.int32)
    offsets = torch.cumsum(counts, 0, dtype=torch.int32) - counts
    nb = {"indices": neighborhood, "numNeighbors": counts, "neighborOffsets": offsets, "kernels": kernels,
          "gradients": kernelGradients, "distances": radialDistances, "vectors": directions, "supports": supports}
    return _operation(masses, densities, quantities, nb, int(numParticles), operation, gradientMode, divergenceMode)


def sphOperationStates(stateA, stateB, quantities, neighborhood, operation="interpolate", gradientMode="symmetric",
                       divergenceMode="div"):
    """sphOperationStates (sphOps.py:278-303) on the GPU."""
    if operation == "density":
        masses = (stateA["masses"], stateB["masses"])
        return _operation(masses, masses, None, neighborhood, int(stateA["numParticles"]), "density", gradientMode,
                          divergenceMode)
    return _operation((stateA["masses"], stateB["masses"]), (stateA["densities"], stateB["densities"]), quantities,
                      neighborhood, int(stateA["numParticles"]), operation, gradientMode, divergenceMode)


def _operation(masses, densities, quantities, nb, n, operation, gradientMode, divergenceMode):
    if operation not in OPERATIONS:
        raise ValueError(f"operation {operation} is not implemented on the GPU ({', '.join(OPERATIONS)} are)")
    mode = MODES.get(gradientMode)
    if operation == "laplacian":
        if gradientMode == "naive":
            raise ValueError("the naive laplacian needs kernel laplacians, which the GPU neighborhood does not hold")
        if mode is None:
            mode = MODES["difference"]  # sphLaplacian's default formula
    elif operation in ("gradient", "divergence", "curl") and mode is None:
        raise ValueError(f"gradientMode {gradientMode} is not implemented")
    mode = 0 if mode is None else mode
    dmode = {"div": 0, "dot": 1}.get(divergenceMode)
    if dmode is None:
        raise ValueError(f"divergenceMode {divergenceMode} is not supported")
    dev = torch.as_tensor(masses[0]).device
    pairs = _Pairs(nb, n)
    m_b = _dev(masses[1])
    rho_a, rho_b = _dev(densities[0]), _dev(densities[1])
    q_a = q_b = q_pair = None
    if operation == "density":
        C, qshape = 1, (n,)
    elif isinstance(quantities, tuple):
        qa, qb = torch.as_tensor(quantities[0]), torch.as_tensor(quantities[1])
        C, qshape = _components(qb), tuple(qb.shape)
        q_a, q_b = _dev(qa).reshape(-1), _dev(qb).reshape(-1)
    else:
        qp = torch.as_tensor(quantities)
        C, qshape = _components(qp), tuple(qp.shape)
        q_pair = _dev(qp).reshape(-1)
    if operation in ("divergence",) and C == 1:
        raise ValueError("Cannot compute divergence on non vector fields!")
    if operation == "curl" and C != 2:
        raise ValueError("the GPU curl takes 2D vector fields")
    if operation == "laplacian" and C == 4:
        raise ValueError("the GPU laplacian takes scalar and vector fields")
    out = torch.empty(_out_shape(n, operation, C, qshape), device="cuda")
    lib = _lib.load()
    _lib.check("sph_operation", lib.sph_operation(
        pairs.ref(), OPERATIONS[operation], mode, dmode, C, _ptr(m_b), _ptr(rho_a), _ptr(rho_b), _ptr(q_a), _ptr(q_b),
        _ptr(q_pair), _ptr(out), _stream()))
    return out.to(dev)


# ------------------------------------------------------------------------------------------
# Module functions
# ------------------------------------------------------------------------------------------
def _n(state):
    return int(state["numParticles"]) if "numParticles" in state else int(torch.as_tensor(state["positions"]).shape[0])


def _device(state):
    return torch.as_tensor(state["masses"]).device


def computeDensity(stateA, stateB, neighborhood, simConfig):
    """computeDensity (density.py:6-15): sum_j m_j W_ij."""
    return sphOperationStates(stateA, stateB, None, neighborhood, operation="density")


def computeCovarianceMatrices(stateA, stateB, neighborhood, simConfig):
    """computeCovarianceMatrices (normalizationMatrices.py:18-23)."""
    n = _n(stateA)
    pairs = _Pairs(neighborhood, n)
    out = torch.empty(n, 2, 2, device="cuda")
    m_b, rho_b = _dev(stateB["masses"]), _dev(stateB["densities"])
    _lib.check("sph_covariance", _lib.load().sph_covariance(pairs.ref(), _ptr(m_b), _ptr(rho_b), _ptr(out), _stream()))
    return out.to(_device(stateA))


def _density_gradient(stateA, stateB, neighborhood, L):
    n = _n(stateA)
    pairs = _Pairs(neighborhood, n)
    out = torch.empty(n, 2, device="cuda")
    args = [_dev(stateB["masses"]), _dev(stateA["densities"]), _dev(stateB["densities"]),
            _dev(L).reshape(n, 4) if L is not None else None]
    _lib.check("sph_density_gradient", _lib.load().sph_density_gradient(
        pairs.ref(), *[_ptr(a) for a in args], _ptr(out), _stream()))
    return out.to(_device(stateA))


def renormalizedDensityGradient(stateA, stateB, neighborhood, simConfig):
    """renormalizedDensityGradient (densityDiffusion.py:7-26): sum (rho_i - rho_j) V_j L_i gradW."""
    return _density_gradient(stateA, stateB, neighborhood, stateA["L"])


def densityGradient(stateA, stateB, neighborhood, simConfig):
    """densityGradient (densityDiffusion.py:28-46): sum (rho_i - rho_j) V_j gradW."""
    return _density_gradient(stateA, stateB, neighborhood, None)


def computeDensityDeltaTerm(stateA, stateB, neighborhood, simConfig, schemeOverride=None):
    """computeDensityDeltaTerm (densityDiffusion.py:49-73), scheme 'deltaSPH'."""
    scheme = simConfig["diffusion"]["densityScheme"] if schemeOverride is None else schemeOverride
    if scheme != "deltaSPH":
        raise ValueError(f"density diffusion scheme {scheme} is not implemented on the GPU (deltaSPH is)")
    n = _n(stateA)
    pairs = _Pairs(neighborhood, n)
    out = torch.empty(n, device="cuda")
    args = [_dev(stateB["masses"]), _dev(stateA["densities"]), _dev(stateB["densities"]), _dev(stateA["gradRho^L"]),
            _dev(stateB["gradRho^L"]), _dev(stateA["supports"])]
    _lib.check("sph_delta_term", _lib.load().sph_delta_term(
        pairs.ref(), *[_ptr(a) for a in args], _f(simConfig["diffusion"]["delta"]),
        _f(simConfig["kernel"]["kernelScale"]), _f(simConfig["fluid"]["cs"]), _ptr(out), _stream()))
    return out.to(_device(stateA))


def computeMomentumEquation(stateA, stateB, neighborhood, config):
    """computeMomentumEquation (momentumEquation.py:6-39): -sum (u_j - u_i) m_j . gradW rho_i / rho_j."""
    n = _n(stateA)
    pairs = _Pairs(neighborhood, n)
    out = torch.empty(n, device="cuda")
    args = [_dev(stateB["masses"]), _dev(stateA["densities"]), _dev(stateB["densities"]), _dev(stateA["velocities"]),
            _dev(stateB["velocities"])]
    _lib.check("sph_momentum", _lib.load().sph_momentum(pairs.ref(), *[_ptr(a) for a in args], _ptr(out), _stream()))
    return out.to(_device(stateA))


def computePressureAccel(stateA, stateB, neighborhood, config):
    """computePressureAccel (pressureForce.py:10-12): -(sum (p_i + p_j) V_j gradW) / rho_i."""
    n = _n(stateA)
    pairs = _Pairs(neighborhood, n)
    out = torch.empty(n, 2, device="cuda")
    args = [_dev(stateB["masses"]), _dev(stateA["densities"]), _dev(stateB["densities"]), _dev(stateA["pressures"]),
            _dev(stateB["pressures"])]
    _lib.check("sph_pressure_accel", _lib.load().sph_pressure_accel(
        pairs.ref(), *[_ptr(a) for a in args], _ptr(out), _stream()))
    return out.to(_device(stateA))


_VISC = {"deltaSPH_viscid": 0, "deltaSPH_inviscid": 1}


def _viscosity(stateA, stateB, neighborhood, config, section, wall):
    p = config[section]
    scheme = p["velocityScheme"]
    if scheme not in _VISC:
        raise ValueError(f"viscosity scheme {scheme} is not implemented on the GPU (deltaSPH_viscid, "
                         "deltaSPH_inviscid are)")
    prm = _lib.ViscosityParams()
    prm.scheme = _VISC[scheme]
    prm.wall_volume = int(wall)
    prm.pi_switch = int(bool(p.get("pi-switch", False)))
    prm.nu, prm.alpha, prm.eps = _f(p.get("nu", 0.0)), _f(p.get("alpha", 0.0)), _f(p["eps"])
    prm.cs, prm.rho0 = _f(config["fluid"]["cs"]), _f(config["fluid"]["rho0"])
    n = _n(stateA)
    pairs = _Pairs(neighborhood, n)
    out = torch.empty(n, 2, device="cuda")
    args = [_dev(stateB["masses"]), _dev(stateA["densities"]), _dev(stateB["densities"]), _dev(stateA["velocities"]),
            _dev(stateB["velocities"]), _dev(stateA["supports"])]
    _lib.check("sph_viscosity", _lib.load().sph_viscosity(
        pairs.ref(), *[_ptr(a) for a in args], ctypes.byref(prm), _ptr(out), _stream()))
    return out.to(_device(stateA))


def computeViscosity(stateA, stateB, neighborhood, config):
    """computeViscosity (viscosity.py:222-241) for the deltaSPH schemes."""
    return _viscosity(stateA, stateB, neighborhood, config, "diffusion", False)


def computeViscosity_Boundary(stateA, stateB, neighborhood, config):
    """computeViscosity_Boundary (boundaryViscosity.py) for the deltaSPH schemes: the
    boundaryDiffusion section, and m_j / (rho_i + rho_j) in the inviscid scheme."""
    return _viscosity(stateA, stateB, neighborhood, config, "boundaryDiffusion", True)


def computeGravity(fluidState, config):
    """computeGravity (gravity.py:8-29), constant mode: direction * magnitude for every particle."""
    v = torch.as_tensor(fluidState["velocities"])
    g = config["gravity"]
    if not g["active"]:
        return torch.zeros_like(v)
    if g.get("gravityMode", "constant") == "potentialField":
        raise ValueError("the potential-field gravity mode is not implemented on the GPU (constant is)")
    x = torch.as_tensor(fluidState["positions"])
    # the parameter defaults of gravity.py:31-38
    direction = torch.as_tensor(g.get("direction", [0, -1, 0]), dtype=x.dtype, device=x.device)
    return (direction[:v.shape[1]] * g.get("magnitude", 9.81)).repeat(v.shape[0], 1)


def mDBCDensity(perennialState, config):
    """mDBCDensity (mDBC.py:50-163): (boundary densities, Shepard densities) from the ghost
    state (``perennialState['boundaryGhost']``, its neighborhood over the fluid) on the GPU;
    the moment system is solved in fp64 (sph_mdbc_density)."""
    ghost = perennialState["boundaryGhost"]
    fluid = perennialState["fluid"]
    n = int(ghost["numParticles"])
    pairs = _Pairs(ghost["neighborhood"], n, need=("distances", "vectors", "kernels", "gradients"))
    rho = torch.empty(n, device="cuda")
    shep = torch.empty(n, device="cuda")
    args = [_dev(fluid["masses"]), _dev(fluid["densities"]), _dev(perennialState["boundary"]["positions"]),
            _dev(ghost["positions"])]
    _lib.check("sph_mdbc_density", _lib.load().sph_mdbc_density(
        pairs.ref(), *[_ptr(a) for a in args], _f(config["particle"]["support"]), _f(config["fluid"]["rho0"]),
        _ptr(rho), _ptr(shep), _stream()))
    dev = torch.as_tensor(perennialState["boundary"]["positions"]).device
    return rho.to(dev), shep.to(dev)
