"""Reverse-mode gradients of plain delta-SPH rollouts on the sm_103a VJP kernels.

Scope: one periodic or walled (mDBC) domain with either deltaSPH viscosity (and the
boundary viscosity), gravity, the symplectic Euler step of the reference runner
(integration.py:357-392, both density updates) followed by delta+ shifting
(shifting.py:119-147, 882-1019) without the free-surface handling. The reference has no
adjoint of its own: it differentiates its torch operators with autograd step by step.

One step z = (x, u, rho) -> z'' is, with rates (a, drho) = RHS(z, rho_b(z)) (simulationStep;
rho_b(z) the mDBC wall densities extrapolated from the fluid state z):

    stage 1   x_h = x + dt/2 u,  u_h = u + dt/2 a(z),  rho_h = rho + dt/2 drho(z)
    stage 2   u'  = u + dt a(z_h),  x' = x + dt (u + u')/2,
              rho' = rho_h                                    (density update 'reference')
              rho' = rho (2 - e)/(2 + e), e = -dt drho(z_h)/rho_h   ('rational')
    shift     x'' = x' + clamp(dx(x', rho', rho_b(z_h), Ma(u'))),  u'' = u',  rho'' = rho'

The backward pass runs those three lines in reverse; the operator VJPs (shift, RHS pass B,
the renormalised density gradient of pass A and the mDBC extrapolation) are the CUDA
kernels of libsph103.so, the elementwise integrator algebra is done here in torch. The wall
densities' adjoint of the shift and of stage 2 meets at z_h, where one mDBC VJP returns it
to the fluid. ``rollout`` checkpoints the state every ``checkpoint_every`` steps of the
fused forward and recomputes a segment's stage states when its turn comes in the backward
pass, so memory stays at O(n / checkpoint_every + checkpoint_every) states.
"""
from __future__ import annotations

import copy

import numpy as np
import torch

from .solver import Solver

__all__ = ["rollout", "rollout_loss_and_grad", "step_stages", "step_vjp", "Rollout"]


def _f32(v) -> float:
    return float(np.float32(v))


class _Consts:
    def __init__(self, config):
        dt = float(config["timestep"]["dt"])
        self.dt = _f32(dt)
        self.dth = _f32(dt / 2.0)
        self.cs = float(config["fluid"]["cs"])
        self.compute_mach = bool(config.get("shifting", {}).get("computeMach", True))
        self.rational = config.get("integration", {}).get("densityUpdate", "reference") != "reference"


def _check_scope(config):
    diff = config.get("diffusion", {})
    if diff.get("velocityScheme", "deltaSPH_inviscid") not in ("deltaSPH_viscid", "deltaSPH_inviscid"):
        raise ValueError("the adjoint covers the deltaSPH_viscid and deltaSPH_inviscid viscosities")
    if config.get("integration", {}).get("scheme", "symplecticEuler") != "symplecticEuler":
        raise ValueError("the adjoint covers the symplecticEuler scheme")
    if config.get("simulation", {}).get("densityScheme", "continuity") != "continuity":
        raise ValueError("the adjoint covers the continuity density")
    sh = config.get("shifting", {})
    if sh.get("scheme", "deltaSPH") != "deltaSPH" or sh.get("freeSurface", False):
        raise ValueError("the adjoint covers the delta+ shift without the free-surface handling")
    if config.get("regions"):
        raise ValueError("the adjoint covers domains without inlet/outlet regions")


def _state(x, u, rho):
    return {"positions": x, "velocities": u, "densities": rho}


def _walls(sol: Solver, densities=None):
    """The solver's wall particles for an upload (None for a fluid-only domain)."""
    if not sol.nB:
        return None
    b = dict(sol.boundary)
    if densities is not None:
        b["densities"] = densities
    return b


def step_stages(sol: Solver, C: _Consts, x, u, rho, shift: bool = True):
    """Stage states of one step from (x, u, rho), evaluated operator by operator with the
    fused step's operation order. Returns (z0, z_half, z_int, z_next, drho_half, rho_b_half)
    with rho_b_half the wall densities of stage 2 (which the shift reads; empty without
    walls)."""
    sol.upload(_state(x, u, rho), _walls(sol))
    r1 = sol.rhs()
    xh = x + u * C.dth
    uh = u + r1["dudt"] * C.dth
    rh = rho + r1["drhodt"] * C.dth
    sol.upload(_state(xh, uh, rh), _walls(sol))
    r2 = sol.rhs()
    rbh = r2["boundary_densities"] if sol.nB else torch.zeros(0, device=x.device)
    u1 = u + r2["dudt"] * C.dt
    x1 = x + (0.5 * (u + u1)) * C.dt
    if C.rational:
        eps = (-C.dt * r2["drhodt"]) / rh
        rho1 = rho * (2.0 - eps) / (2.0 + eps)
    else:
        rho1 = rh.clone()
    if shift:
        sol.upload(_state(x1, u1, rho1), _walls(sol, rbh))
        x2 = x1 + sol.shift()
    else:
        x2 = x1.clone()
    return (x, u, rho), (xh, uh, rh), (x1, u1, rho1), (x2, u1.clone(), rho1.clone()), r2["drhodt"], rbh


def step_vjp(sol: Solver, C: _Consts, stages, xbar2, ubar2, rbar2, shift: bool = True):
    """Adjoint of one step: from the adjoints of z'' to those of z (and of nu)."""
    (x, u, rho), (xh, uh, rh), (x1, u1, rho1), _, drho_h, rbh = stages
    n = x.shape[0]
    dev = x.device
    nu_part = torch.empty(n, device=dev)
    nubar = torch.zeros((), dtype=torch.float64, device=dev)
    walls = sol.nB > 0
    # adjoints of the wall densities of stage 2 (read by the shift too) and of stage 1
    wbar_h = torch.zeros(sol.nB, device=dev) if walls else None
    wbar_0 = torch.zeros(sol.nB, device=dev) if walls else None
    # shift: x'' = x' + dx(x', rho', rho_b(z_h), Ma(u'))
    xbar1 = torch.zeros_like(x)
    rbar1 = rbar2.clone()
    ubar1 = ubar2.clone()
    if shift:
        sol.upload(_state(x1, u1, rho1), _walls(sol, rbh))
        mach = torch.empty(n, device=dev)
        sol.vjp_shift(xbar2, xbar1, rbar1, mach, wbar_h)
        if C.compute_mach:
            # Ma = max|u'| / cs: the adjoint goes to the arg-max particle (no host sync)
            sp = torch.linalg.vector_norm(u1, dim=1)
            k = torch.argmax(sp).view(1)
            scale = mach.sum() / C.cs / sp[k].clamp_min(1e-30)
            ubar1.index_add_(0, k, scale[:, None] * u1[k])
    else:
        xbar1 += xbar2
    # stage 2: u' = u + dt a(z_h); x' = x + dt (u + u')/2; rho' = rho_h or rational(rho, rho_h, drho(z_h))
    ubar1_t = ubar1 + (0.5 * C.dt) * xbar1
    xbar = xbar1.clone()
    ubar = ubar1_t + (0.5 * C.dt) * xbar1
    abar_h = C.dt * ubar1_t
    rbar_h = torch.zeros_like(rho)
    rbar = torch.zeros_like(rho)
    drbar_h = None
    if C.rational:
        eps = (-C.dt * drho_h) / rh
        R = (2.0 - eps) / (2.0 + eps)
        rbar += rbar1 * R
        ebar = rbar1 * rho * (-4.0 / (2.0 + eps) ** 2)
        drbar_h = ebar * (-C.dt / rh)
        rbar_h += ebar * (C.dt * drho_h / rh ** 2)
    else:
        rbar_h += rbar1
    # pass B (and pass A when drho(z_h) has an adjoint) at z_h, then the wall densities of z_h
    sol.upload(_state(xh, uh, rh), _walls(sol))
    xbar_h = torch.zeros_like(x)
    ubar_h = torch.zeros_like(u)
    gbar_h = torch.zeros_like(x) if drbar_h is not None else None
    sol.vjp_rates(abar_h, drbar_h, xbar_h, ubar_h, rbar_h, gbar_h, nu_part, wbar_h)
    nubar += nu_part.double().sum()
    if gbar_h is not None:
        sol.vjp_gradient(gbar_h, xbar_h, rbar_h, wbar_h)
    if walls:
        sol.vjp_walls(wbar_h, xbar_h, rbar_h)
    # stage 1: x_h = x + dt/2 u; u_h = u + dt/2 a(z); rho_h = rho + dt/2 drho(z)
    xbar += xbar_h
    ubar += C.dth * xbar_h + ubar_h
    rbar += rbar_h
    abar0 = C.dth * ubar_h
    drbar0 = C.dth * rbar_h
    sol.upload(_state(x, u, rho), _walls(sol))
    gbar0 = torch.zeros_like(x)
    sol.vjp_rates(abar0, drbar0, xbar, ubar, rbar, gbar0, nu_part, wbar_0)
    nubar += nu_part.double().sum()
    sol.vjp_gradient(gbar0, xbar, rbar, wbar_0)
    if walls:
        sol.vjp_walls(wbar_0, xbar, rbar)
    return xbar, ubar, rbar, nubar


def _with_nu(config, nu):
    cfg = copy.deepcopy(config)
    cfg["diffusion"]["nu"] = float(nu)
    return cfg


def _forward(sol, x0, u0, rho0, n_steps, every, shift, use_graphs=False):
    """Fused forward; returns the final state and the checkpoints {step: (x, u, rho)}."""
    graphed = use_graphs and shift and torch.cuda.current_stream().cuda_stream != 0
    ckpt = {}
    sol.upload(_state(x0, u0, rho0), _walls(sol))
    k = 0
    while k < n_steps:
        got = sol.download()
        ckpt[k] = (got["positions"], got["velocities"], got["densities"])
        m = min(every, n_steps - k)
        if graphed and m >= 2:
            sol.graph_step(m - (m & 1))  # the graph replays an even number of steps
            if m & 1:
                sol.step(1)
        elif shift:
            sol.step(m)
        else:
            for _ in range(m):
                sol.integrate()
        k += m
    sol.check()
    got = sol.download()
    return (got["positions"], got["velocities"], got["densities"]), ckpt


def _flat(st):
    (x, u, rho), (xh, uh, rh), (x1, u1, r1), (x2, u2, r2), dr, rbh = st
    return [x, u, rho, xh, uh, rh, x1, u1, r1, x2, u2, r2, dr, rbh]


_TAPE = 14  # tensors per step in a flat tape


def _unflat(t):
    return (tuple(t[0:3]), tuple(t[3:6]), tuple(t[6:9]), tuple(t[9:12]), t[12], t[13])


class _Replay:
    """A CUDA graph of fn over static input tensors, which each call copies in first.

    Every solver call inside fn re-sorts the particles and swaps the solver's buffer
    pointers on the host; a graph bakes those pointers in, so fn must re-sort an even
    number of times (the callers group steps accordingly)."""

    def __init__(self, fn, inputs):
        self.inputs = [t.clone() for t in inputs]
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            fn(*self.inputs)  # first-call set-up (attributes, tables) outside the capture
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.outputs = fn(*self.inputs)

    def __call__(self, *args):
        for dst, src in zip(self.inputs, args):
            dst.copy_(src)
        self.graph.replay()
        return self.outputs


class _Graphs:
    """Graphed recomputation of stage states (two steps per graph) and graphed step VJPs
    (one step per graph when its re-sort count is even, else two)."""

    def __init__(self, sol, C, shift):
        self.sol, self.C, self.shift = sol, C, shift
        self._rec = None
        self._vjp = None
        sorts = (1 if shift else 0) + 3 + (1 if C.rational else 0) + (2 if sol.nB else 0)
        self.group = 1 if sorts % 2 == 0 else 2

    def two_steps(self, x, u, rho):
        if self._rec is None:
            def fn(x, u, rho):
                a = step_stages(self.sol, self.C, x, u, rho, self.shift)
                b = step_stages(self.sol, self.C, *a[3], self.shift)
                return _flat(a) + _flat(b)
            self._rec = _Replay(fn, [x, u, rho])
        out = [t.clone() for t in self._rec(x, u, rho)]
        return _unflat(out[:_TAPE]), _unflat(out[_TAPE:])

    def vjp(self, tapes, xbar, ubar, rbar):
        if self._vjp is None:
            G = self.group

            def fn(*args):
                xb, ub, rb = args[_TAPE * G:]
                nb = torch.zeros((), dtype=torch.float64, device=xb.device)
                for g in reversed(range(G)):
                    xb, ub, rb, n1 = step_vjp(self.sol, self.C, _unflat(args[_TAPE * g:_TAPE * (g + 1)]), xb, ub, rb,
                                              self.shift)
                    nb = nb + n1
                return xb, ub, rb, nb
            self._vjp = _Replay(fn, [t for st in tapes for t in _flat(st)] + [xbar, ubar, rbar])
        out = self._vjp(*([t for st in tapes for t in _flat(st)] + [xbar, ubar, rbar]))
        return tuple(t.clone() for t in out)


def _backward(sol, C, ckpt, n_steps, every, shift, xbar, ubar, rbar, graphs=None):
    nubar = torch.zeros((), dtype=torch.float64, device=xbar.device)
    for k0 in sorted(ckpt, reverse=True):
        m = min(every, n_steps - k0)
        x, u, rho = ckpt[k0]
        tape = []
        while graphs is not None and m - len(tape) >= 2:
            a, b = graphs.two_steps(x, u, rho)
            tape += [a, b]
            x, u, rho = b[3]
        while len(tape) < m:
            st = step_stages(sol, C, x, u, rho, shift)
            tape.append(st)
            x, u, rho = st[3]
        i = len(tape)
        while graphs is not None and i >= graphs.group:
            xbar, ubar, rbar, nb = graphs.vjp(tape[i - graphs.group:i], xbar, ubar, rbar)
            nubar += nb
            i -= graphs.group
        while i > 0:
            xbar, ubar, rbar, nb = step_vjp(sol, C, tape[i - 1], xbar, ubar, rbar, shift)
            nubar += nb
            i -= 1
    return xbar, ubar, rbar, nubar


class Rollout(torch.autograd.Function):
    """(x0, u0, rho0, nu) -> (x_n, u_n, rho_n) after n_steps full steps; differentiable in
    all four inputs through the VJP kernels with segment checkpointing."""

    @staticmethod
    def forward(ctx, x0, u0, rho0, nu, config, n_steps, every, shift, fluid_extra, use_graphs=True):
        _check_scope(config)
        cfg = _with_nu(config, float(nu))
        fluid = {k: v for k, v in fluid_extra.items() if k != "boundary"}
        fluid.update(_state(x0.detach(), u0.detach(), rho0.detach()))
        sol = Solver(cfg, fluid, fluid_extra.get("boundary"))
        # sort every step, as the stage replay of the backward pass does (same pair order)
        if sol.verlet_reuse:
            sol.set_verlet_reuse(False)
        (x, u, rho), ckpt = _forward(sol, x0.detach(), u0.detach(), rho0.detach(), n_steps, every, shift,
                                     use_graphs)
        ctx.sol, ctx.ckpt, ctx.C = sol, ckpt, _Consts(cfg)
        ctx.n_steps, ctx.every, ctx.shift = n_steps, every, shift
        ctx.use_graphs = use_graphs
        ctx.nu_dtype, ctx.nu_device = nu.dtype, nu.device
        return x, u, rho

    @staticmethod
    def backward(ctx, gx, gu, gr):
        n = ctx.sol.nF
        dev = "cuda"
        xbar = (gx if gx is not None else torch.zeros(n, 2, device=dev)).float().contiguous().clone()
        ubar = (gu if gu is not None else torch.zeros(n, 2, device=dev)).float().contiguous().clone()
        rbar = (gr if gr is not None else torch.zeros(n, device=dev)).float().contiguous().clone()
        graphs = _Graphs(ctx.sol, ctx.C, ctx.shift) if ctx.use_graphs else None
        xbar, ubar, rbar, nubar = _backward(ctx.sol, ctx.C, ctx.ckpt, ctx.n_steps, ctx.every, ctx.shift,
                                            xbar, ubar, rbar, graphs)
        nub = nubar.to(device=ctx.nu_device, dtype=ctx.nu_dtype)
        return xbar, ubar, rbar, nub, None, None, None, None, None, None


def rollout(config, fluid, n_steps, nu=None, checkpoint_every=25, shift=True, x0=None, u0=None, rho0=None,
            use_graphs=True, boundary=None):
    """Differentiable rollout of ``n_steps`` steps. Tensors x0 / u0 / rho0 / nu (defaults:
    the fluid dict's fields and config['diffusion']['nu']) may require grad. ``boundary``:
    the static mDBC wall particles of a walled domain (positions, normals, distances,
    masses, supports). use_graphs replays the forward steps and the backward pass from CUDA
    graphs (same results)."""
    _check_scope(config)
    dev = "cuda"

    def _t(v, ref):
        return (v if v is not None else torch.as_tensor(ref)).to(device=dev, dtype=torch.float32).contiguous()

    x0 = _t(x0, fluid["positions"])
    u0 = _t(u0, fluid["velocities"])
    rho0 = _t(rho0, fluid["densities"])
    if nu is None:
        nu = torch.tensor(float(config["diffusion"]["nu"]), dtype=torch.float64)
    extra = {k: fluid[k] for k in ("masses", "supports") if k in fluid}
    if boundary is not None and config.get("boundary", {}).get("active", True):
        extra["boundary"] = boundary
    return Rollout.apply(x0, u0, rho0, nu, config, int(n_steps), int(checkpoint_every), bool(shift), extra,
                         bool(use_graphs))


def rollout_loss_and_grad(config, fluid, target_u, n_steps, checkpoint_every=25, shift=True, use_graphs=True,
                          boundary=None):
    """Loss = mean((u_n - target)^2) over all velocity components; returns (loss, du0, dnu)."""
    u0 = torch.as_tensor(fluid["velocities"]).to("cuda", torch.float32).clone().requires_grad_(True)
    nu = torch.tensor(float(config["diffusion"]["nu"]), dtype=torch.float64, requires_grad=True)
    _, u, _ = rollout(config, fluid, n_steps, nu=nu, checkpoint_every=checkpoint_every, shift=shift, u0=u0,
                      use_graphs=use_graphs, boundary=boundary)
    tgt = torch.as_tensor(target_u).to("cuda", torch.float32)
    loss = torch.mean((u - tgt) ** 2)
    loss.backward()
    return float(loss.detach()), u0.grad.detach(), float(nu.grad)
