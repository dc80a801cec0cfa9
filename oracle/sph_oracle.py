"""CPU oracle for the diffSPH per-timestep particle path (test infrastructure).

This module is the checker: only the tests, the smoke check and the benchmark's
CPU-baseline leg import it. The product never routes through it.

It restates, in numpy, the reference's v2 torch implementation of the delta-SPH
step (plus a small C helper, ``geometry.c``, for the bit-exact fp32 neighbor
filter). Every function names the reference file:line it follows. Arithmetic
runs in the dtype of the inputs: float32 mirrors the reference's default
precision, float64 gives the FP64 run of the same scheme.

Parity: pinned against golden vectors produced by running the reference itself
on CPU (``tests/golden/make_golden.py`` -> ``tests/golden/*.npz``), checked by
``tests/test_oracle_golden.py``.

Conventions: a "state" is a dict with numpy arrays ``positions [N,2]``,
``velocities [N,2]``, ``densities [N]``, ``masses [N]``, ``supports [N]``
(and for boundaries ``normals [N,2]``, ``distances [N]``). A "neighborhood" is
a dict with the reference's keys (``indices``, ``distances`` (= r/h_j),
``vectors`` (unit x_ij), ``supports`` (h_j), ``kernels``, ``gradients``,
``numNeighbors``, ``neighborOffsets``). ``config`` uses the reference's nested
config keys; tensors in it may be given as floats or lists.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB = None

C_D_2D = 7.0 / np.pi  # Wendland C2 normalisation in 2D, kernelFunctions/Wendland2.py:24-27


def build_oracle(force: bool = False) -> str:
    """Compile geometry.c into oracle/_build/libsphoracle.so (gcc, no fp contraction)."""
    os.makedirs(_BUILD, exist_ok=True)
    so = os.path.join(_BUILD, "libsphoracle.so")
    src = os.path.join(_HERE, "geometry.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        tmp = so + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                               "-fno-fast-math", src, "-o", tmp, "-lm"])
        os.replace(tmp, so)
    return so


class _Domain(ctypes.Structure):
    _fields_ = [("min", ctypes.c_double * 2), ("max", ctypes.c_double * 2),
                ("periodic", ctypes.c_int * 2)]


def _lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build_oracle())
        for name, ft in (("oracle_neighbors_f32", ctypes.c_float), ("oracle_neighbors_f64", ctypes.c_double)):
            fn = getattr(_LIB, name)
            P = ctypes.c_void_p
            fn.argtypes = [P, P, ctypes.c_int64, P, P, ctypes.c_int64, ctypes.POINTER(_Domain),
                           ctypes.c_int64, P, P, P, P, P]
            fn.restype = ctypes.c_int64
        for name in ("oracle_wrap_positions_f32", "oracle_wrap_positions_f64"):
            fn = getattr(_LIB, name)
            fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(_Domain)]
            fn.restype = None
    return _LIB


def _flt(x):
    if hasattr(x, "item") and getattr(x, "ndim", 0) == 0:
        return float(x.item())
    return float(x)


def _vec2(x):
    if hasattr(x, "tolist"):
        x = x.tolist()
    if isinstance(x, (list, tuple)):
        return [float(v) for v in x][:2]
    return [float(x)] * 2


def domain_of(config) -> _Domain:
    d = config["domain"]
    mn = _vec2(d["minExtent"])
    mx = _vec2(d["maxExtent"])
    per = d.get("periodicity", d.get("periodic", False))
    if hasattr(per, "tolist"):
        per = per.tolist()
    if isinstance(per, bool):
        per = [per, per]
    dom = _Domain()
    dom.min[0], dom.min[1] = mn
    dom.max[0], dom.max[1] = mx
    dom.periodic[0], dom.periodic[1] = int(bool(per[0])), int(bool(per[1]))
    return dom


def periodic_positions(x, config):
    """getPeriodicPosition, src/diffSPH/v2/modules/neighborhood.py:406-431."""
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    dom = domain_of(config)
    fn = _lib().oracle_wrap_positions_f32 if x.dtype == np.float32 else _lib().oracle_wrap_positions_f64
    fn(x.ctypes.data, out.ctypes.data, x.shape[0], ctypes.byref(dom))
    return out


# ----------------------------------------------------------------------------------------
# Wendland C2 kernel, src/diffSPH/kernelFunctions/Wendland2.py:6-38, cpow kernels.py:69-70
# ----------------------------------------------------------------------------------------
def _cpow(q, p):
    return np.clip(q, 0, 1) ** p


def wendland_kernel(q, h):
    """W = (1-q)_+^4 (1+4q) C_d / h^2 (Wendland2.py:6-10, 28-30)."""
    dt = q.dtype.type
    return _cpow(1 - q, 4) * (1 + 4 * q) * dt(C_D_2D) / h ** 2


def wendland_gradient(q, xhat, h):
    """grad W = xhat * (-20 q (1-q)_+^3) C_d / h^3 (Wendland2.py:12-16, 32-34)."""
    dt = q.dtype.type
    return xhat * (-20 * q * _cpow(1 - q, 3) * dt(C_D_2D) / h ** 3)[:, None]


# ----------------------------------------------------------------------------------------
# Neighbor search, src/diffSPH/v2/modules/neighborhood.py:433-460 and :491-593
# ----------------------------------------------------------------------------------------
def neighbor_search(query, reference, config, compute_kernels=True):
    """Exact neighbor list (scatter mode, h_ij = h_j), rows sorted by i, columns by j.

    Returns a dict with the reference neighborhood keys. The candidate stage of the
    reference (torchCompactRadius, an external package) only has to deliver a superset,
    since every candidate is re-filtered by computeNeighborhood; this oracle generates
    candidates from a cell grid and applies the same fp32 filter.
    """
    xq = np.ascontiguousarray(query["positions"])
    xr = np.ascontiguousarray(reference["positions"])
    dt = xq.dtype
    hq = np.ascontiguousarray(query["supports"], dtype=dt)
    hr = np.ascontiguousarray(reference["supports"], dtype=dt)
    dom = domain_of(config)
    fn = _lib().oracle_neighbors_f32 if dt == np.float32 else _lib().oracle_neighbors_f64
    cap = max(1024, 64 * xq.shape[0])
    while True:
        oi = np.empty(cap, np.int64)
        oj = np.empty(cap, np.int64)
        oq = np.empty(cap, dt)
        ox = np.empty((cap, 2), dt)
        oh = np.empty(cap, dt)
        n = fn(xq.ctypes.data, hq.ctypes.data, xq.shape[0], xr.ctypes.data, hr.ctypes.data,
               xr.shape[0], ctypes.byref(dom), cap, oi.ctypes.data, oj.ctypes.data,
               oq.ctypes.data, ox.ctypes.data, oh.ctypes.data)
        if n <= cap:
            break
        cap = int(n)
    i, j, q, xh, h = oi[:n], oj[:n], oq[:n], ox[:n], oh[:n]
    num = np.bincount(i, minlength=xq.shape[0]).astype(np.int32)
    off = np.concatenate([[0], np.cumsum(num)[:-1]]).astype(np.int32)
    nb = {"indices": (i, j), "distances": q, "vectors": xh, "supports": h,
          "numNeighbors": num, "neighborOffsets": off}
    if compute_kernels:
        nb["kernels"] = wendland_kernel(q, h)
        nb["gradients"] = wendland_gradient(q, xh, h)
    return nb


# ----------------------------------------------------------------------------------------
# Algebra helpers: scatter_sum (math.py:77-93), pinv2x2 (math.py:11-57)
# ----------------------------------------------------------------------------------------
def scatter_sum(src, index, n):
    out = np.zeros((n,) + src.shape[1:], dtype=src.dtype)
    np.add.at(out, index, src)
    return out


def pinv2x2(M, eigenvalues=False):
    """Closed-form 2x2 pseudo-inverse via an SVD built from atan2/cos/sin, math.py:11-57
    (with its singular values, ordered by magnitude, when ``eigenvalues``)."""
    a, b, c, d = M[:, 0, 0], M[:, 0, 1], M[:, 1, 0], M[:, 1, 1]
    theta = 0.5 * np.arctan2(2 * a * c + 2 * b * d, a ** 2 + b ** 2 - c ** 2 - d ** 2)
    ct, st = np.cos(theta), np.sin(theta)
    U = np.zeros_like(M)
    U[:, 0, 0], U[:, 0, 1], U[:, 1, 0], U[:, 1, 1] = ct, -st, st, ct
    S1 = a ** 2 + b ** 2 + c ** 2 + d ** 2
    S2 = np.sqrt((a ** 2 + b ** 2 - c ** 2 - d ** 2) ** 2 + 4 * (a * c + b * d) ** 2)
    o1 = np.sqrt((S1 + S2) / 2)
    o2 = np.sqrt(np.maximum(S1 - S2 + M.dtype.type(1e-7), M.dtype.type(1e-7)) / 2)
    phi = 0.5 * np.arctan2(2 * a * b + 2 * c * d, a ** 2 - b ** 2 + c ** 2 - d ** 2)
    cp, sp = np.cos(phi), np.sin(phi)
    s11 = np.sign((a * ct + c * st) * cp + (b * ct + d * st) * sp)
    s22 = np.sign((a * st - c * ct) * sp + (-b * st + d * ct) * cp)
    V = np.zeros_like(M)
    V[:, 0, 0], V[:, 0, 1], V[:, 1, 0], V[:, 1, 1] = cp * s11, -sp * s22, sp * s11, cp * s22
    o1i = np.where(np.abs(o1) > 1e-5, 1 / np.where(o1 == 0, 1, o1), 0).astype(M.dtype)
    o2i = np.where(np.abs(o2) > 1e-5, 1 / np.where(o2 == 0, 1, o2), 0).astype(M.dtype)
    S = np.zeros_like(M)
    S[:, 0, 0], S[:, 1, 1] = o1i, o2i
    L = np.matmul(np.matmul(V, S), np.swapaxes(U, 1, 2))
    if not eigenvalues:
        return L
    # eigVals: (o1, o2), swapped where |o2| > |o1| (math.py:53-54)
    ev = np.stack([o1, o2], axis=1)
    sw = np.abs(ev[:, 1]) > np.abs(ev[:, 0])
    ev[sw] = ev[sw][:, ::-1]
    return L, ev


# ----------------------------------------------------------------------------------------
# Physics modules (each cites the reference function it restates)
# ----------------------------------------------------------------------------------------
def _vol(sB, j):
    return sB["masses"][j] / sB["densities"][j]


def compute_density(sA, sB, nb, config):
    """computeDensity density.py:6-15 -> sphDensityInterpolation sphOps.py:20-29."""
    i, j = nb["indices"]
    return scatter_sum(sB["masses"][j] * nb["kernels"], i, sA["positions"].shape[0])


def compute_covariance(sA, sB, nb, config):
    """computeCovarianceMatrices normalizationMatrices.py:18-23 (gradient, 'difference' on a pair tensor)."""
    i, j = nb["indices"]
    d = -(nb["distances"] * nb["supports"])[:, None] * nb["vectors"]
    k = _vol(sB, j)[:, None] * nb["gradients"]
    return scatter_sum(np.einsum("na,nb->nab", d, k), i, sA["positions"].shape[0])


def renormalized_density_gradient(sA, sB, nb, config):
    """renormalizedDensityGradient densityDiffusion.py:7-26 (gradient 'difference' with L_i grad W)."""
    i, j = nb["indices"]
    g = np.einsum("nab,nb->na", sA["L"][i], nb["gradients"])
    k = _vol(sB, j)[:, None] * g
    q = sA["densities"][i] - sB["densities"][j]
    return scatter_sum(q[:, None] * k, i, sA["positions"].shape[0])


def density_gradient(sA, sB, nb, config):
    """densityGradient densityDiffusion.py:28-46 (un-normalised, 'difference')."""
    i, j = nb["indices"]
    k = _vol(sB, j)[:, None] * nb["gradients"]
    q = sA["densities"][i] - sB["densities"][j]
    return scatter_sum(q[:, None] * k, i, sA["positions"].shape[0])


def density_delta_term(sA, sB, nb, config):
    """computeDensityDeltaTerm densityDiffusion.py:49-73, scheme 'deltaSPH'."""
    i, j = nb["indices"]
    dt = sA["densities"].dtype.type
    rij = nb["distances"] * nb["supports"]
    grad_ij = sA["gradRho^L"][i] + sB["gradRho^L"][j]
    rho_ij = 2 * (sB["densities"][j] - sA["densities"][i]) / (rij + dt(1e-6) * nb["supports"])
    psi = -rho_ij[:, None] * nb["vectors"] + grad_ij
    k = _vol(sB, j)[:, None] * nb["gradients"]
    div = scatter_sum(np.einsum("nd,nd->n", psi, k), i, sA["positions"].shape[0])
    delta = dt(_flt(config["diffusion"]["delta"]))
    kappa = dt(_flt(config["kernel"]["kernelScale"]))
    cs = dt(_flt(config["fluid"]["cs"]))
    return delta * sA["supports"] / kappa * cs * div


def momentum_equation(sA, sB, nb, config):
    """computeMomentumEquation momentumEquation.py:6-39 (continuity: -sum m_j (u_j-u_i).gradW rho_i/rho_j)."""
    i, j = nb["indices"]
    q = (sB["velocities"][j] - sA["velocities"][i]) * sB["masses"][j][:, None]
    k = nb["gradients"]
    kq = q[:, 0] * k[:, 0] + q[:, 1] * k[:, 1]
    kq = kq * sA["densities"][i] / sB["densities"][j]
    return -scatter_sum(kq, i, sA["positions"].shape[0])


def stiff_tait_eos(state, config):
    """stiffTaitEOS pressureEOS.py:5-11."""
    dt = state["densities"].dtype.type
    rho0 = _flt(config["fluid"]["rho0"])
    cs = _flt(config["fluid"]["cs"])
    gamma = _flt(config["EOS"]["polytropicExponent"])
    return dt(rho0 * cs ** 2 / gamma) * ((state["densities"] / dt(rho0)) ** dt(gamma) - 1)


def pressure_accel(sA, sB, nb, config):
    """computePressureAccel pressureForce.py:10-12 (gradient 'summation', divided by rho_i)."""
    i, j = nb["indices"]
    k = _vol(sB, j)[:, None] * nb["gradients"]
    q = sA["pressures"][i] + sB["pressures"][j]
    return -scatter_sum(q[:, None] * k, i, sA["positions"].shape[0]) / sA["densities"][:, None]


def pressure_accel_switch(sA, sB, nb, config):
    """computePressureAccelSwitch pressureForce.py:15-33 (Antuono's switch): p_ij = p_j + p_i
    where p_i >= 0 or the particle is on the surface (surfaceMask > 0.5), else p_j - p_i;
    a_i = -sum_j m_j / (rho_i rho_j) p_ij gradW_ij."""
    i, j = nb["indices"]
    p_i, p_j = sA["pressures"][i], sB["pressures"][j]
    pij = np.where((p_i >= 0) | (sA["surfaceMask"][i] > 0.5), p_j + p_i, p_j - p_i)
    k = (sB["masses"][j] / (sA["densities"][i] * sB["densities"][j]))[:, None] * nb["gradients"]
    return -scatter_sum(pij[:, None] * k, i, sA["densities"].shape[0])


def liuliu_consistent(ghost, fluid, nb, q):
    """LiuLiuConsistent sphOps.py:313-341: first-order consistent interpolation of the fluid
    quantity q at the query (ghost) particles. With V_j = m_j / rho_j, x_ij = -xhat q h,
        b = [sum V q_j W, sum V q_j gradW]
        M = [[sum V W, sum V W x_ij^T], [sum V gradW_a, sum V x_ij,a gradW^T]  (a = 0, 1)]
    and the solution by Cramer's rule, det(M with column k <- b) / (det M + 1e-7).
    Returns (solution [n, 3], M [n, 3, 3], b [n, 3])."""
    i, j = nb["indices"]
    n = ghost["positions"].shape[0]
    V = fluid["masses"][j] / fluid["densities"][j]
    W, G = nb["kernels"], nb["gradients"]
    dt = W.dtype.type
    x = -nb["vectors"] * nb["distances"][:, None] * nb["supports"][:, None]
    b = np.concatenate([scatter_sum(q[j] * (V * W), i, n)[:, None],
                        scatter_sum(q[j][:, None] * (V[:, None] * G), i, n)], axis=1)
    M0 = scatter_sum(V * W, i, n)
    Mg = scatter_sum(V[:, None] * G, i, n)
    Mx = scatter_sum(x * (V * W)[:, None], i, n)
    Mxg = scatter_sum(np.einsum("na,nd->nad", x, V[:, None] * G), i, n)
    M = np.zeros((n, 3, 3), dtype=dt)
    M[:, 0, 0], M[:, 0, 1:] = M0, Mx
    for a in range(2):
        M[:, 1 + a, 0], M[:, 1 + a, 1:] = Mg[:, a], Mxg[:, a, :]
    d0 = np.linalg.det(M)
    sol = np.empty((n, 3), dtype=dt)
    for k in range(3):
        Mk = M.copy()
        Mk[:, :, k] = b
        sol[:, k] = np.linalg.det(Mk) / (d0 + dt(1e-7))
    return sol, M, b


def _pi_term(sA, sB, nb, eps):
    i, j = nb["indices"]
    h = nb["supports"]
    v = sA["velocities"][i] - sB["velocities"][j]
    r = nb["distances"] * h
    vr = np.einsum("nd,nd->n", v, nb["vectors"])
    return vr / (r + eps * h ** 2)


def viscosity(sA, sB, nb, config, section="diffusion", boundary=False):
    """computeViscosity viscosity.py:222-241: deltaSPH_viscid :200-218, deltaSPH_inviscid :123-170;
    boundary variant boundaryViscosity.py:123-173 (V_j = m_j/(rho_i+rho_j)) and :199-219."""
    i, j = nb["indices"]
    dt = sA["densities"].dtype.type
    p = config[section]
    eps = dt(_flt(p["eps"]))
    scheme = p["velocityScheme"]
    pi = _pi_term(sA, sB, nb, eps)
    if p.get("pi-switch", False):
        pi = np.where(np.einsum("nd,nd->n", sA["velocities"][i] - sB["velocities"][j], nb["vectors"]) < 0, pi, 0)
    rho0 = _flt(config["fluid"]["rho0"])
    n = sA["positions"].shape[0]
    if scheme == "deltaSPH_viscid":
        Vj = _vol(sB, j)
        s = scatter_sum((Vj * pi)[:, None] * nb["gradients"], i, n)
        dim = 2
        return (dt(2 * (dim + 2)) * dt(_flt(p["nu"])) * dt(rho0) / sA["densities"])[:, None] * s
    if scheme == "deltaSPH_inviscid":
        if boundary:
            Vj = sB["masses"][j] / (sA["densities"][i] + sB["densities"][j])
        else:
            Vj = _vol(sB, j)
        s = scatter_sum((Vj * pi)[:, None] * nb["gradients"], i, n)
        alpha = dt(_flt(p["alpha"]))
        cs = dt(_flt(config["fluid"]["cs"]))
        return (alpha * sA["supports"] * cs * dt(rho0) / sA["densities"])[:, None] * s
    raise ValueError(f"viscosity scheme {scheme} not in the oracle")


def gravity(state, config):
    """computeGravity gravity.py:8-29, constant mode."""
    g = config.get("gravity", {})
    v = state["velocities"]
    if not g.get("active", False):
        return np.zeros_like(v)
    direction = np.asarray(g.get("direction", [0, -1, 0]), dtype=v.dtype)[:2]
    return np.tile(direction * v.dtype.type(_flt(g.get("magnitude", 9.81))), (v.shape[0], 1))


# ----------------------------------------------------------------------------------------
# mDBC, src/diffSPH/v2/modules/mDBC.py:9-36 and :50-163
# ----------------------------------------------------------------------------------------
def boundary_ghosts(boundary, config):
    """buildBoundaryGhostParticles mDBC.py:9-36: mirror each boundary particle along its normal."""
    d = boundary["distances"]
    h = d.dtype.type(_flt(config["particle"]["support"]))
    mapping = d + np.maximum(d, -np.ones_like(d) * h)
    return boundary["positions"] + mapping[:, None] * boundary["normals"]


def _pinv3(A, config):
    """Batched 3x3 pseudo-inverse as torch.linalg.pinv computes it (SVD, singular values
    below rtol = eps(dtype) * 3 of the largest are dropped).

    ``config['oracle']['pinv']``: 'fp64' (default) evaluates it in float64 (the exact
    pseudo-inverse the reference approximates); 'torch' calls torch.linalg.pinv in the
    input dtype, which reproduces the reference's own fp32 LAPACK result and is used to
    pin this oracle against the reference's vectors. The moment matrices reach condition
    numbers of ~1e4 near free edges, where the fp32 solve differs from the fp64 one by
    ~1e-4 relative."""
    mode = config.get("oracle", {}).get("pinv", "fp64")
    if mode == "torch":
        import torch
        return torch.linalg.pinv(torch.from_numpy(np.ascontiguousarray(A))).numpy()
    rc = np.finfo(A.dtype).eps * 3
    return np.linalg.pinv(A.astype(np.float64), rcond=rc).astype(A.dtype)


def mdbc_density(boundary, fluid, config, ghost_nb=None):
    """mDBCDensity mDBC.py:50-163 (Python path): Shepard sums, 3x3 moment system,
    pinv where the ghost has > 4 neighbors, first-order extrapolation where > 5,
    Shepard where > 0, rest density otherwise. Returns (boundary densities, shepard)."""
    dt = fluid["densities"].dtype.type
    ghost = {"positions": boundary_ghosts(boundary, config), "supports": boundary["supports"],
             "masses": boundary["masses"], "densities": boundary["densities"]}
    nb = ghost_nb if ghost_nb is not None else neighbor_search(ghost, fluid, config)
    i, j = nb["indices"]
    nG = ghost["positions"].shape[0]
    W, G = nb["kernels"], nb["gradients"]
    Vj = fluid["masses"][j] / fluid["densities"][j]
    num = scatter_sum(fluid["masses"][j] * W, i, nG)
    den = scatter_sum(Vj * W, i, nG)
    shepard = num / (den + dt(1e-7))
    gsum = scatter_sum((fluid["densities"][j] * Vj)[:, None] * G, i, nG)
    b = np.concatenate([num[:, None], gsum], axis=1)
    vgrad = scatter_sum(Vj[:, None] * G, i, nG)
    xij = -nb["vectors"] * nb["distances"][:, None] * dt(_flt(config["particle"]["support"]))
    psum = scatter_sum((Vj * W)[:, None] * xij, i, nG)
    pmat = scatter_sum(np.einsum("na,nb->nab", xij, Vj[:, None] * G), i, nG)
    A = np.zeros((nG, 3, 3), dtype=dt)
    A[:, 0, 0] = den
    A[:, 1, 0], A[:, 2, 0] = vgrad[:, 0], vgrad[:, 1]
    A[:, 0, 1], A[:, 0, 2] = psum[:, 0], psum[:, 1]
    A[:, 1, 1], A[:, 1, 2] = pmat[:, 0, 0], pmat[:, 0, 1]
    A[:, 2, 1], A[:, 2, 2] = pmat[:, 1, 0], pmat[:, 1, 1]
    cnt = nb["numNeighbors"]
    Ainv = np.zeros_like(A)
    sel = cnt > 4
    if sel.any():
        Ainv[sel] = _pinv3(A[sel], config)
    res = np.einsum("nab,nb->na", Ainv, b)
    rho0 = dt(_flt(config["fluid"]["rho0"]))
    out = np.ones(nG, dtype=dt) * rho0
    out[cnt > 0] = shepard[cnt > 0]
    rel = boundary["positions"] - ghost["positions"]
    s5 = cnt > 5
    out[s5] = res[s5, 0] + np.einsum("nu,nu->n", rel[s5], res[s5, 1:])
    return out, shepard, nb


# ----------------------------------------------------------------------------------------
# Scheme: simulationStep deltaPlus.py:176-422 (+ callModule :30-96)
# ----------------------------------------------------------------------------------------
def _boundary_active(config, state):
    return bool(config.get("boundary", {}).get("active", False)) and "boundary" in state


def simulation_step(state, config):
    """One right-hand-side evaluation. Returns ((u, dudt, drhodt), (u_b, None, drhodt_b))
    and leaves intermediate fields in the state dicts like the reference does."""
    fl = state["fluid"]
    fl["neighborhood"] = neighbor_search(fl, fl, config)
    fl["numNeighbors"] = fl["neighborhood"]["numNeighbors"]
    bnd = _boundary_active(config, state)
    if bnd:
        bd = state["boundary"]
        state["boundaryToFluidNeighborhood"] = neighbor_search(fl, bd, config)
    # summation density (deltaPlus.py:193-198, direction 'all': ftf + btf for the fluid rows),
    # before the mDBC extrapolation, which reads the fluid densities
    if config.get("simulation", {}).get("densityScheme", "continuity") == "summation":
        ftf = compute_density(fl, fl, fl["neighborhood"], config)
        fl["densities"] = ftf + compute_density(fl, bd, state["boundaryToFluidNeighborhood"], config) if bnd else ftf
    if bnd:
        # mDBC boundary density (deltaPlus.py:200-202)
        bd["densities"], shep, gnb = mdbc_density(bd, fl, config)
        state["boundaryGhost"] = {"densities": shep, "neighborhood": gnb}
    nbf = fl["neighborhood"]
    # normalisation matrices (deltaPlus.py:240-252), direction 'fluidwBoundary'
    M = compute_covariance(fl, fl, nbf, config)
    if bnd:
        M = M + compute_covariance(fl, bd, state["boundaryToFluidNeighborhood"], config)
    M[fl["numNeighbors"] < 4] = np.eye(2, dtype=M.dtype)[None]
    fl["covarianceMatrix"] = M
    fl["L"] = pinv2x2(M)
    # renormalised density gradient (deltaPlus.py:256-262)
    fl["gradRho^L"] = renormalized_density_gradient(fl, fl, nbf, config)
    if bnd:
        fl["gradRho^L"] = fl["gradRho^L"] + density_gradient(fl, bd, state["boundaryToFluidNeighborhood"], config)
    # diffusion and momentum (deltaPlus.py:268-309)
    fl["densityDiffusion"] = density_delta_term(fl, fl, nbf, config)
    fl["velocityDiffusion"] = viscosity(fl, fl, nbf, config)
    if bnd:
        fl["velocityDiffusion"] = fl["velocityDiffusion"] + viscosity(
            fl, bd, state["boundaryToFluidNeighborhood"], config, section="boundaryDiffusion", boundary=True)
        fl["momentumEquation"] = momentum_equation(fl, fl, nbf, config) + momentum_equation(
            fl, bd, state["boundaryToFluidNeighborhood"], config)
    else:
        fl["momentumEquation"] = momentum_equation(fl, fl, nbf, config)
    fl["pressures"] = stiff_tait_eos(fl, config)
    if bnd:
        bd["pressures"] = stiff_tait_eos(bd, config)
        fl["pressureAccel"] = pressure_accel(fl, fl, nbf, config) + pressure_accel(
            fl, bd, state["boundaryToFluidNeighborhood"], config)
    else:
        fl["pressureAccel"] = pressure_accel(fl, fl, nbf, config)
    fl["gravityAccel"] = gravity(fl, config)
    dudt = fl["pressureAccel"] + fl["gravityAccel"] + fl["velocityDiffusion"]
    drhodt = fl["momentumEquation"] + fl["densityDiffusion"]
    if not bnd:
        return (fl["velocities"].copy(), dudt, drhodt), (None, None, None)
    return (fl["velocities"].copy(), dudt, drhodt), (bd["velocities"].copy(), None, np.zeros_like(bd["densities"]))


def _copy_state(s):
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items() if k not in ("neighborhood",)}


def integrate_symplectic_euler(state, config):
    """symplecticEuler integration.py:357-392: k1 at t^n, half step, k2, then
    v' = v + dt k2_u; x' = x + (v + v')/2 dt; rho' = rho (2-eps)/(2+eps), eps = -dt k2_rho / rho_half."""
    dt_ = state["fluid"]["densities"].dtype.type
    dt = dt_(_flt(config["timestep"]["dt"]))
    base = state["fluid"]
    t1 = {"fluid": _copy_state(base)}
    if "boundary" in state:
        t1["boundary"] = _copy_state(state["boundary"])
    k1, _ = simulation_step(t1, config)
    t2 = {"fluid": _copy_state(base)}
    if "boundary" in state:
        t2["boundary"] = _copy_state(t1["boundary"])
    f2 = t2["fluid"]
    f2["positions"] = f2["positions"] + k1[0] * (dt / 2)
    f2["velocities"] = f2["velocities"] + k1[1] * (dt / 2)
    f2["densities"] = f2["densities"] + k1[2] * (dt / 2)
    k2, _ = simulation_step(t2, config)
    dudt = k2[1]
    newV = base["velocities"] + dudt * dt
    dxdt = dt_(0.5) * (base["velocities"] + newV) * dt
    newX = base["positions"] + dxdt
    eps = -dt * k2[2] / f2["densities"]
    newRho = base["densities"] * (2 - eps) / (2 + eps)
    if config.get("integration", {}).get("densityUpdate", "reference") == "reference":
        # integration.py:381-392 never assigns the local ``drhodt``, so the state sync at
        # integration.py:439-513 replaces the densities by the temporary state's, i.e. the
        # half-step density rho^n + dt/2 k1_rho. The reference's observable update is that.
        newRho = f2["densities"].copy()
    out = {"fluid": dict(base)}
    out["fluid"].update(positions=newX, velocities=newV, densities=newRho,
                        dudt=dudt, drhodt=eps, dxdt=dxdt)
    if "boundary" in state:
        out["boundary"] = dict(state["boundary"])
        out["boundary"]["densities"] = t2["boundary"]["densities"]
    return out, {"k1": k1, "k2": k2, "temp": t2}


def delta_plus_shifting(ps, nb, config):
    """deltaPlusShifting shifting.py:119-147."""
    dt = ps["densities"].dtype.type
    h = _flt(config["particle"]["support"])
    dx = _flt(config["particle"]["dx"])
    # W_0 is built from torch.tensor(python float) arguments (shifting.py:121-122), i.e. in
    # fp32 whatever the state's precision: q0 = fp32(dx / h), h = fp32(h)
    W0 = wendland_kernel(np.asarray([np.float32(dx / h)], dtype=np.float32), np.float32(h))[0]
    i, j = nb["indices"]
    k = nb["kernels"] / W0
    R = dt(_flt(config["shifting"]["R"]))
    n = dt(_flt(config["shifting"]["n"]))
    term = 1 + R * k ** n
    dens = ps["masses"][j] / (ps["densities"][i] + ps["densities"][j])
    s = scatter_sum((term * dens)[:, None] * nb["gradients"], i, ps["positions"].shape[0])
    CFL = dt(_flt(config["shifting"]["CFL"]))
    if config["shifting"].get("computeMach", True):
        Ma = np.max(np.linalg.norm(ps["velocities"], axis=-1)) / dt(_flt(config["fluid"]["cs"]))
    else:
        Ma = dt(0.1)
    kappa = dt(_flt(config["kernel"]["kernelScale"]))
    scale = -CFL * Ma * (ps["supports"] / kappa * 2) ** 2
    return scale[:, None] * s


def _d2kdq2(q):
    """Wendland C2 second q-derivative (2D), Wendland2.py:18-22: 20 (4q - 1) (1-q)_+^2."""
    return 20 * (4 * q - 1) * _cpow(1 - q, 2)


def wendland_hessian(q, xhat, h):
    """Per-pair kernel Hessian, the reference's closed form with its regularisers
    (KernelWrapper.Hessian2D, src/diffSPH/kernels.py:263-303). Returns [E, 2, 2]."""
    dt = q.dtype.type
    cd = dt(C_D_2D)
    factor = cd / h ** 2
    r = q * h
    x = xhat * r[:, None]
    k2 = _d2kdq2(q)
    k1 = -20 * q * _cpow(1 - q, 3)
    dA = h ** 2 * r ** 2 + dt(1e-5) * h
    dB = h * r ** 3 + dt(1e-10) * h
    self_term = np.where(q < dt(1e-5), _d2kdq2(np.zeros(1, dt))[0], dt(0))  # d2kdq2(0) at the particle itself
    dxx = factor * (x[:, 0] ** 2 / dA * k2 + x[:, 1] ** 2 / dB * k1 + 1 / h ** 2 * self_term)
    dyy = factor * (x[:, 1] ** 2 / dA * k2 + x[:, 0] ** 2 / dB * k1 + 1 / h ** 2 * self_term)
    dxy = cd * h ** dt(-2) * np.where(q > dt(-1e-7), (x[:, 0] * x[:, 1]) / (h * r ** 2 + dt(1e-5) * h)
                                      * (1 / h * k2 - 1 / (r + dt(1e-3) * h) * k1), dt(0))
    H = np.zeros((q.shape[0], 2, 2), dtype=dt)
    inside = q <= 1
    H[:, 0, 0] = np.where(inside, dxx, 0)
    H[:, 1, 1] = np.where(inside, dyy, 0)
    H[:, 0, 1] = np.where(inside, dxy, 0)
    H[:, 1, 0] = H[:, 0, 1]
    return H


def ips_matrices(ps, nb, marker):
    """getShiftingMatrices shifting.py:611-705 without free-surface handling and with
    shifting.summationDensity off (omega = areas), initialization 'zero': the 2x2 blocks
    H_ij omega_j of the active rows (fluid i), the right-hand side J_i = sum grad W omega_j
    (zero on wall rows) and x0 = 0."""
    i, j = nb["indices"]
    n = ps["positions"].shape[0]
    omega = ps["areas"]
    J = scatter_sum(nb["gradients"] * omega[j, None], i, n)
    H = wendland_hessian(nb["distances"], nb["vectors"], nb["supports"]) * omega[j, None, None]
    B = J.reshape(-1).copy()
    B.reshape(-1, 2)[marker != 0] = 0
    active = marker[i] == 0
    return H[active], i[active], j[active], B


def _spmv(H, i, j, x, n):
    """multiplySparseShifting shifting.py:707-716: block rows summed per component."""
    xv = x.reshape(-1, 2)
    out = np.zeros_like(x)
    out[0::2] = out[0::2] + scatter_sum(H[:, 0, 0] * xv[j, 0], i, n)
    out[0::2] = out[0::2] + scatter_sum(H[:, 0, 1] * xv[j, 1], i, n)
    out[1::2] = out[1::2] + scatter_sum(H[:, 1, 0] * xv[j, 0], i, n)
    out[1::2] = out[1::2] + scatter_sum(H[:, 1, 1] * xv[j, 1], i, n)
    return out


def bicgstab_shifting(H, i, j, n, b, rtol, maxiter, threshold):
    """bicgstab_shifting shifting.py:322-493 from x0 = 0: unpreconditioned BiCGStab (the
    Jacobi matrix it is given is never applied) with the reference's stopping rules:
    |r| < rtol |b| before an iteration, |s| < rtol |b| mid-iteration, rho / rv / omega
    breakdowns, and any per-particle |x_i| > threshold. Returns (x, iterations, code) where
    code is the reference's second return value: the iteration count when |r| converged
    at the top of an iteration, 0 when |s| converged mid-iteration, -10 / -11 for the rho /
    rv and omega breakdowns, -12 for the threshold, maxiter when the loop ran out."""
    dt = b.dtype.type
    norm = lambda v: dt(np.sqrt(np.dot(v, v)))
    bnrm2 = norm(b)
    atol = dt(max(0.0, float(rtol) * float(bnrm2)))
    xk = np.zeros_like(b)
    if bnrm2 == 0:
        return b.copy(), 0, 0
    rhotol = dt(float(np.finfo(dt).eps) ** 2)
    rk = b.copy()
    r0 = rk.copy()
    pk = rk.copy()
    for it in range(maxiter):
        if norm(rk) < atol:
            return xk, it, it
        rho = dt(np.dot(rk, r0))
        if abs(rho) < rhotol:
            return xk, it, -10
        apk = _spmv(H, i, j, pk, n)
        rv = dt(np.dot(apk, r0))
        if rv == 0:
            return xk, it, -11
        alpha = dt(rho / rv)
        sk = rk - alpha * apk
        if norm(sk) < atol:
            return xk + alpha * pk, it + 1, 0
        ask = _spmv(H, i, j, sk, n)
        omega = dt(dt(np.dot(ask, sk)) / dt(np.dot(ask, ask)))
        xk = xk + alpha * pk + omega * sk
        rk = sk - omega * ask
        beta = dt(dt(np.dot(rk, r0)) / rho) * dt(alpha / omega)
        pk = rk + beta * (pk - omega * apk)
        if it > 0 and abs(omega) < rhotol:
            return xk, it + 1, -11
        if np.any(np.sqrt(np.sum(xk.reshape(-1, 2) ** 2, axis=1)) > threshold):
            return xk, it + 1, -12
    return xk, maxiter, maxiter


def ips_shift(ps, nb, marker, config):
    """computeShifting shifting.py:780-880 (scheme 'IPS', solver 'BiCGStab_wJacobi'):
    returns the update -x of the solve (before the clamp) and (iterations, code) as
    ``bicgstab_shifting`` returns them."""
    sh = config["shifting"]
    dx = _flt(config["particle"]["dx"])
    thr = sh.get("solverThreshold", -0.5)
    thr = dx / 2 if thr < 0 else thr  # parameters.py:238
    H, i, j, B = ips_matrices(ps, nb, marker)
    n = ps["positions"].shape[0]
    xk, iters, status = bicgstab_shifting(H, i, j, n, B, sh.get("rtol", 1e-4), int(sh.get("maxSolveIter", 64)),
                                          thr)
    return -xk.reshape(-1, 2), (iters, status)


# ----------------------------------------------------------------------------------------
# Free-surface handling of the shift (solveShifting with shifting.freeSurface)
# ----------------------------------------------------------------------------------------
def _normalize(v):
    """torch.nn.functional.normalize: v / max(|v|, 1e-12) per row."""
    nrm = np.sqrt(np.sum(v * v, axis=1))
    return v / np.maximum(nrm, v.dtype.type(1e-12))[:, None]


def _scatter_or(flags, index, n):
    out = np.zeros(n, dtype=bool)
    np.logical_or.at(out, index, flags)
    return out


def detect_free_surface_barecasco(ps, nb, config):
    """detectFreeSurfaceBarecasco surfaceDetection.py:95-107: a particle is on the surface
    when no neighbor lies within the cone of half-angle threshold / 2 around its normalised
    cover vector sum_j -xhat_ij (a vanishing cover vector marks it interior)."""
    i, j = nb["indices"]
    n = ps["positions"].shape[0]
    xij = nb["vectors"]
    nrm = _normalize(scatter_sum(-xij, i, n))
    with np.errstate(invalid="ignore"):
        angle = np.arccos(np.einsum("ij,ij->i", xij, nrm[i]))
    dt = xij.dtype.type
    half = dt(_flt(config.get("surfaceDetection", {}).get("BarecascoThreshold", np.pi / 3)) / 2)
    cond = ((angle <= half) & (i != j)) | (np.sqrt(np.sum(nrm * nrm, axis=1))[i] <= dt(1e-5))
    return ~_scatter_or(cond, i, n)


def expand_free_surface_mask(fs, nb, config):
    """expandFreeSurfaceMask surfaceDetection.py:54-63: expansionIterations rounds of OR over
    the neighbors."""
    i, j = nb["indices"]
    fsm = fs.copy()
    for _ in range(int(config.get("surfaceDetection", {}).get("expansionIterations", 2))):
        fsm = _scatter_or(fsm[j], i, fs.shape[0])
    return fsm


def normals_lambda(ps, nb, gradient=False):
    """computeNormalizationMatrices normalizationMatrices.py:7-16 (L and its singular values),
    computeNormalsMaronne surfaceDetection.py:41-52 (Lambdas = the smaller one) and the
    normalised computeLambdaGrad shifting.py:151-171: sum_j V_j (Lambda_i - Lambda_j) L_i gradW.
    Returns (normals, Lambdas, L), or the gradient before normalisation when ``gradient``."""
    i, j = nb["indices"]
    n = ps["positions"].shape[0]
    M = compute_covariance(ps, ps, nb, None)
    L, ev = pinv2x2(M, eigenvalues=True)
    lam = np.min(np.abs(ev), axis=1)
    ng = np.einsum("ijk,ik->ij", L[i], nb["gradients"])
    k = _vol(ps, j)[:, None] * ng
    grad = scatter_sum((lam[i] - lam[j])[:, None] * k, i, n)
    if gradient:
        return grad
    return _normalize(grad), lam, L


def free_surface_projection(update, fs, fsm, normals, lam, config):
    """solveShifting shifting.py:972-982 (projectionScheme 'mat'): (I - n n^T) update on the
    expanded mask, zero where Lambdas < 0.4, times surfaceScaling on the surface."""
    dt = update.dtype.type
    nmat = np.einsum("ij,ik->ikj", normals, normals)
    Mp = np.eye(2, dtype=dt)[None] - nmat
    res = np.einsum("nab,nb->na", Mp, update)
    update = update.copy()
    update[fsm] = res[fsm]
    update[lam < dt(0.4)] = 0
    update[fs] = update[fs] * dt(_flt(config["shifting"].get("surfaceScaling", 0.1)))
    return update


def solve_shifting(state, config, info=None):
    """solveShifting shifting.py:882-1019 with maxIterations = 1, delta+ (deltaPlusShifting)
    or implicit (IPS) scheme, with the free-surface handling of shifting.freeSurface
    (Barecasco detection, 'lambda' normals, 'mat' projection): returns the position
    increment of the fluid particles. ``info`` (a dict) receives the IPS solve's iteration
    count and return code, and the free-surface fields of the merged particle set."""
    fl = state["fluid"]
    nF = fl["positions"].shape[0]
    keys = ("positions", "velocities", "masses", "densities", "supports", "areas")
    if "boundary" in state:
        bd = state["boundary"]
        ps = {k: np.concatenate([fl[k], bd[k]]) for k in keys}
        marker = np.concatenate([np.zeros(nF, np.int32), np.ones(bd["positions"].shape[0], np.int32)])
    else:
        ps = {k: fl[k] for k in keys}
        marker = np.zeros(nF, np.int32)
    nb = neighbor_search(ps, ps, config)
    free = bool(config["shifting"].get("freeSurface", False))
    if free:
        fs = detect_free_surface_barecasco(ps, nb, config)
        fsm = expand_free_surface_mask(fs, nb, config)
    if config["shifting"].get("scheme", "deltaSPH") == "IPS":
        # surface particles leave the system like wall rows (getShiftingMatrices :657-678)
        update, stats = ips_shift(ps, nb, np.where(fs, 1, marker) if free else marker, config)
        if info is not None:
            info["iterations"], info["code"] = stats
    else:
        update = -delta_plus_shifting(ps, nb, config)
    if free:
        normals, lam, _ = normals_lambda(ps, nb)
        update = free_surface_projection(update, fs, fsm, normals, lam, config)
        if info is not None:
            info.update(freeSurface=fs, freeSurfaceMask=fsm, normals=normals, Lambdas=lam)
    dt = fl["densities"].dtype.type
    thr = dt(_flt(config["shifting"]["threshold"]) * _flt(config["particle"]["dx"]))
    update = np.clip(update, -thr, thr)
    update[marker != 0] = 0
    newpos = ps["positions"] - update
    dx = (newpos - ps["positions"])[:nF]
    return dx, nb


def full_step(state, config):
    """One complete time step as the reference runner does it (runner.py:37-42):
    integrate (symplectic Euler), then delta+ shifting added to the positions."""
    out, aux = integrate_symplectic_euler(state, config)
    dx, _ = solve_shifting(out, config)
    out["fluid"]["positions"] = out["fluid"]["positions"] + dx
    out["fluid"]["shiftAmount"] = dx
    return out, aux


def acoustic_timestep(config, CFL):
    """computeTimestep timestep.py:8-39, acoustic limit dt_c = CFL h / c_s / kappa."""
    return CFL * _flt(config["particle"]["support"]) / _flt(config["fluid"]["cs"]) / _flt(config["kernel"]["kernelScale"])
