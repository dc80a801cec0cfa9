"""Drop-in versions of the reference's step functions, backed by the sm_103a solver.

Same signatures and return values as:

* ``simulationStep(state, config)``            src/diffSPH/v2/simulationSchemes/deltaPlus.py:176-422
* ``integrate(simulationStep, perennialState, config, previousStep=None)``
                                              src/diffSPH/v2/modules/integration.py:92-513
                                              (scheme 'symplecticEuler')
* ``solveShifting(simulationState, config)``   src/diffSPH/v2/modules/shifting.py:882-1019
* ``computePressureAccelSwitch(stateA, stateB, neighborhood, config)``
                                                src/diffSPH/v2/modules/pressureForce.py:15-33

State dicts hold torch tensors (any device). One solver (its workspace, captured graphs
and tuned launch shape) is cached per state dict under the key ``'sph103'`` and reused
while the particle counts and the config object stay the same. Each call uploads the
state's current positions, velocities and densities, since the runner may have changed
them (``positions += dx`` after ``solveShifting``), and an upload always sorts.
``simulationStep`` writes the intermediates the reference leaves in the state (``L``,
``gradRho^L``, ``pressures``, wall densities, ``numNeighbors``).
"""
from __future__ import annotations

import torch

from .solver import Solver

_KEY = "sph103"


def _boundary(state, config):
    if bool(config.get("boundary", {}).get("active", False)) and "boundary" in state:
        return state["boundary"]
    return None


def _solver_for(state, config, upload=True):
    fl = state["fluid"]
    bd = _boundary(state, config)
    sol = state.get(_KEY)
    nF = int(fl["positions"].shape[0])
    nB = int(bd["positions"].shape[0]) if bd is not None else 0
    if sol is None or sol.nF != nF or sol.nB != nB or sol.config is not config:
        sol = Solver(config, fl, bd)
        state[_KEY] = sol
    elif upload:
        sol.upload(fl, bd)
    return sol


def simulationStep(state, config):
    """One right-hand side; returns ((u, dudt, drhodt), (u_b, None, drhodt_b))."""
    sol = _solver_for(state, config)
    out = sol.rhs()
    fl = state["fluid"]
    dev = fl["positions"].device
    fl["L"] = out["L"].to(dev)
    fl["gradRho^L"] = out["gradRho^L"].to(dev)
    fl["pressures"] = out["pressures"].to(dev)
    fl["numNeighbors"] = out["numNeighbors"][:, 0].to(dev)
    dudt, drhodt = out["dudt"].to(dev), out["drhodt"].to(dev)
    u = torch.as_tensor(fl["velocities"]).clone()
    bd = _boundary(state, config)
    if bd is None:
        return (u, dudt, drhodt), (None, None, None)
    bd["densities"] = out["boundary_densities"].to(bd["positions"].device)
    return (u, dudt, drhodt), (torch.as_tensor(bd["velocities"]).clone(), None, torch.zeros_like(bd["densities"]))


def integrate(simulationStep, perennialState, config, previousStep=None):
    """symplecticEuler step of the reference (both right-hand sides fused on the GPU).

    ``simulationStep`` is accepted for signature compatibility; the fused kernels
    evaluate the δ-SPH right-hand side themselves. Returns
    (perennialState, tempState, dxdt, dudt, drhodt) like the reference; the rates of
    the fused step are not materialised, so the last three are None."""
    scheme = config.get("integration", {}).get("scheme", "symplecticEuler")
    if scheme != "symplecticEuler":
        raise ValueError(f"integration scheme {scheme} is not implemented (symplecticEuler is)")
    sol = _solver_for(perennialState, config)
    sol.integrate()
    got = sol.download()
    fl = perennialState["fluid"]
    dev = fl["positions"].device
    fl["positions"] = got["positions"].to(dev)
    fl["velocities"] = got["velocities"].to(dev)
    fl["densities"] = got["densities"].to(dev)
    bd = _boundary(perennialState, config)
    if bd is not None:
        bd["densities"] = got["boundary_densities"].to(bd["positions"].device)
    return perennialState, {"fluid": fl}, None, None, None


def solveShifting(simulationState, config):
    """Shifting (δ+, or the implicit IPS scheme when config['shifting']['scheme'] is 'IPS');
    returns (dx, overallStates) like the reference. overallStates collects the IPS solve's
    diagnostics: one (convergence, code, residual) entry per shifting iteration, of which
    only bicgstab_shifting's return code is kept here; it is empty for δ+."""
    sol = _solver_for(simulationState, config)
    dx = sol.shift()
    states = []
    if config.get("shifting", {}).get("scheme", "deltaSPH") == "IPS":
        states.append(([], sol.ips_result()[1], None))
    return dx.to(simulationState["fluid"]["positions"].device), states


def computePressureAccelSwitch(stateA, stateB, neighborhood, config):
    """Pressure acceleration with Antuono's switch (pressureForce.py:15-33) on a neighborhood
    in the reference's format (the drop-in ``neighborSearch`` returns one), on the GPU.
    ``stateA['surfaceMask']`` (optional) marks the surface particles."""
    import ctypes

    from . import _lib

    def dev(t, dtype=torch.float32):
        return torch.as_tensor(t).to(device="cuda", dtype=dtype).contiguous()

    def ptr(t):
        return ctypes.c_void_p(t.data_ptr()) if t is not None else None

    n = int(torch.as_tensor(stateA["pressures"]).shape[0])
    i, j = neighborhood["indices"]
    off = dev(neighborhood["neighborOffsets"], torch.int32)
    cnt = dev(neighborhood["numNeighbors"], torch.int32)
    pj = dev(j, torch.int64)
    grad = dev(neighborhood["gradients"])
    mask = dev(stateA["surfaceMask"]) if "surfaceMask" in stateA else None
    args = [dev(stateA["pressures"]), dev(stateA["densities"]), mask, dev(stateB["pressures"]),
            dev(stateB["densities"]), dev(stateB["masses"])]
    out = torch.empty(n, 2, device="cuda")
    lib = _lib.load()
    _lib.check("sph_pressure_switch", lib.sph_pressure_switch(
        n, ptr(off), ptr(cnt), ptr(pj), ptr(grad), *[ptr(a) for a in args], ptr(out),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out.to(torch.as_tensor(stateA["pressures"]).device)
