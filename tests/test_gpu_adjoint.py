"""Adjoint kernels against FP64 central finite differences of the oracle.

Each operator VJP of libsph103.so (pass B rates with the pass-A density gradient, the
delta+ shift) and the checkpointed rollout gradient are compared, along random
directions, with central differences (eps = 1e-6) of the FP64 oracle run of the same
scheme. Tolerance: 1e-3 relative to the finite-difference value, checked separately for
the position, velocity, density and nu blocks so that a small block cannot hide behind a
large one.
"""
import copy

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import sph_oracle as O  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402

EPS = 1e-6
RTOL = 1e-3


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _np(t):
    return t.detach().cpu().numpy()


def _fluid64(fl):
    return {k: np.asarray(v, np.float64).copy() for k, v in fl.items()}


def _advanced_state(nx=32, seed=7, steps=5):
    """A jittered periodic Fourier flow advanced a few steps on the GPU (non-uniform
    densities and density gradients), returned as fp32 numpy arrays."""
    from diffsph_gb300.solver import Solver
    cfg, st = scenes.fourier_periodic(nx, seed=seed, jitter=0.2)
    sol = Solver(cfg, st["fluid"])
    sol.step(steps)
    sol.check()
    got = sol.download()
    fl = dict(st["fluid"])
    fl["positions"] = _np(got["positions"])
    fl["velocities"] = _np(got["velocities"])
    fl["densities"] = _np(got["densities"])
    return cfg, fl


def _dirs(cfg, fl, rng):
    n = fl["positions"].shape[0]
    dx = float(cfg["particle"]["dx"])
    umax = float(np.abs(fl["velocities"]).max())
    rvar = float(np.asarray(fl["densities"], np.float64).std()) + 1e-4
    return {
        "positions": rng.standard_normal((n, 2)) * dx,
        "velocities": rng.standard_normal((n, 2)) * umax,
        "densities": rng.standard_normal(n) * rvar,
    }


def _rel(pred, fd):
    return abs(pred - fd) / abs(fd)


@pytest.mark.gpu
def test_rates_vjp_matches_fp64_finite_differences():
    _gpu()
    from diffsph_gb300.solver import Solver
    cfg, fl = _advanced_state()
    rng = np.random.default_rng(11)
    n = fl["positions"].shape[0]
    abar = rng.standard_normal((n, 2)).astype(np.float32)
    drbar = rng.standard_normal(n).astype(np.float32)
    sol = Solver(cfg, fl)
    dev = "cuda"
    xbar = torch.zeros(n, 2, device=dev)
    ubar = torch.zeros(n, 2, device=dev)
    rbar = torch.zeros(n, device=dev)
    gbar = torch.zeros(n, 2, device=dev)
    nup = torch.zeros(n, device=dev)
    sol.vjp_rates(torch.as_tensor(abar, device=dev), torch.as_tensor(drbar, device=dev), xbar, ubar, rbar, gbar, nup)
    sol.vjp_gradient(gbar, xbar, rbar)
    grads = {"positions": _np(xbar), "velocities": _np(ubar), "densities": _np(rbar)}
    f64 = _fluid64(fl)

    def phi(state, c):
        (_, dudt, drho), _ = O.simulation_step({"fluid": state}, c)
        return float(np.sum(abar * dudt) + np.sum(drbar * drho))

    d = _dirs(cfg, fl, rng)
    for key in ("positions", "velocities", "densities"):
        sp, sm = _fluid64(f64), _fluid64(f64)
        sp[key] = sp[key] + EPS * d[key]
        sm[key] = sm[key] - EPS * d[key]
        fd = (phi(sp, cfg) - phi(sm, cfg)) / (2 * EPS)
        pred = float(np.sum(grads[key].astype(np.float64) * d[key]))
        assert _rel(pred, fd) < RTOL, (key, pred, fd)
    nu = float(cfg["diffusion"]["nu"])
    cp, cm = copy.deepcopy(cfg), copy.deepcopy(cfg)
    cp["diffusion"]["nu"] = nu * (1 + EPS)
    cm["diffusion"]["nu"] = nu * (1 - EPS)
    fd = (phi(_fluid64(f64), cp) - phi(_fluid64(f64), cm)) / (2 * EPS * nu)
    pred = float(nup.double().sum())
    assert _rel(pred, fd) < RTOL, ("nu", pred, fd)


@pytest.mark.gpu
def test_shift_vjp_matches_fp64_finite_differences():
    _gpu()
    from diffsph_gb300.solver import Solver
    cfg, fl = _advanced_state(seed=9)
    rng = np.random.default_rng(12)
    n = fl["positions"].shape[0]
    xbn = rng.standard_normal((n, 2)).astype(np.float32)
    sol = Solver(cfg, fl)
    dev = "cuda"
    xbar = torch.zeros(n, 2, device=dev)
    rbar = torch.zeros(n, device=dev)
    mach = torch.zeros(n, device=dev)
    sol.vjp_shift(torch.as_tensor(xbn, device=dev), xbar, rbar, mach)
    u = np.asarray(fl["velocities"], np.float64)
    sp = np.linalg.norm(u, axis=1)
    k = int(np.argmax(sp))
    ubar = np.zeros((n, 2))
    ubar[k] = float(mach.double().sum()) / float(cfg["fluid"]["cs"]) * u[k] / sp[k]
    grads = {"positions": _np(xbar), "velocities": ubar, "densities": _np(rbar)}
    f64 = _fluid64(fl)

    def phi(state):
        dx, _ = O.solve_shifting({"fluid": state}, cfg)
        return float(np.sum(xbn * (state["positions"] + dx)))

    d = _dirs(cfg, fl, rng)
    for key in ("positions", "velocities", "densities"):
        a, b = _fluid64(f64), _fluid64(f64)
        a[key] = a[key] + EPS * d[key]
        b[key] = b[key] - EPS * d[key]
        fd = (phi(a) - phi(b)) / (2 * EPS)
        pred = float(np.sum(np.asarray(grads[key], np.float64) * d[key]))
        assert _rel(pred, fd) < RTOL, (key, pred, fd)


def _oracle_rollout(cfg, fl64, n):
    s = {"fluid": _fluid64(fl64)}
    for _ in range(n):
        s, _ = O.full_step(s, cfg)
    return s["fluid"]


@pytest.mark.gpu
@pytest.mark.parametrize("density_update", ["reference", "rational"])
def test_rollout_gradient_matches_fp64_finite_differences(density_update):
    _gpu()
    from diffsph_gb300.adjoint import rollout
    cfg, st = scenes.fourier_periodic(24, seed=3, jitter=0.1)
    cfg["integration"]["densityUpdate"] = density_update
    fl = st["fluid"]
    n = fl["positions"].shape[0]
    steps = 12
    rng = np.random.default_rng(5)
    target = scenes.fourier_velocity(np.asarray(fl["positions"], np.float64), np.random.default_rng(99))
    dev = "cuda"
    u0 = torch.as_tensor(fl["velocities"], device=dev).clone().requires_grad_(True)
    rho0 = torch.as_tensor(fl["densities"], device=dev).clone().requires_grad_(True)
    x0 = torch.as_tensor(fl["positions"], device=dev).clone().requires_grad_(True)
    nu = torch.tensor(float(cfg["diffusion"]["nu"]), dtype=torch.float64, requires_grad=True)
    _, u, _ = rollout(cfg, fl, steps, nu=nu, checkpoint_every=5, x0=x0, u0=u0, rho0=rho0)
    loss = torch.mean((u - torch.as_tensor(target, dtype=torch.float32, device=dev)) ** 2)
    loss.backward()
    f64 = _fluid64(fl)

    def L(state, c):
        out = _oracle_rollout(c, state, steps)
        return float(np.mean((out["velocities"] - target) ** 2))

    ref64 = L(f64, cfg)
    assert abs(float(loss.detach()) - ref64) <= 1e-4 * ref64
    grads = {"positions": _np(x0.grad), "velocities": _np(u0.grad), "densities": _np(rho0.grad)}
    d = _dirs(cfg, fl, rng)
    for key in ("velocities", "positions", "densities"):
        a, b = _fluid64(f64), _fluid64(f64)
        a[key] = a[key] + EPS * d[key]
        b[key] = b[key] - EPS * d[key]
        fd = (L(a, cfg) - L(b, cfg)) / (2 * EPS)
        pred = float(np.sum(grads[key].astype(np.float64) * d[key]))
        assert _rel(pred, fd) < RTOL, (key, pred, fd)
    nuv = float(cfg["diffusion"]["nu"])
    cp, cm = copy.deepcopy(cfg), copy.deepcopy(cfg)
    cp["diffusion"]["nu"] = nuv * (1 + EPS)
    cm["diffusion"]["nu"] = nuv * (1 - EPS)
    fd = (L(f64, cp) - L(f64, cm)) / (2 * EPS * nuv)
    assert _rel(float(nu.grad), fd) < RTOL, ("nu", float(nu.grad), fd)


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_the_gradient():
    _gpu()
    from diffsph_gb300.adjoint import rollout_loss_and_grad
    cfg, st = scenes.fourier_periodic(32, seed=4, jitter=0.1)
    target = scenes.fourier_velocity(np.asarray(st["fluid"]["positions"], np.float64), np.random.default_rng(1))
    l1, g1, n1 = rollout_loss_and_grad(cfg, st["fluid"], target, 20, checkpoint_every=1)
    l2, g2, n2 = rollout_loss_and_grad(cfg, st["fluid"], target, 20, checkpoint_every=25)
    l3, g3, n3 = rollout_loss_and_grad(cfg, st["fluid"], target, 20, checkpoint_every=7)
    assert l1 == l2 == l3
    for g, nn in ((g2, n2), (g3, n3)):
        assert float((g - g1).abs().max()) <= 1e-4 * float(g1.abs().max())
        assert abs(nn - n1) <= 1e-4 * abs(n1)


def _advanced_dam_break(dx=1.0 / 32, steps=40):
    """The dam break advanced a few steps on the GPU (the column has started to move):
    (config, fluid state as fp32 numpy arrays, static walls)."""
    from diffsph_gb300.solver import Solver
    cfg, st = scenes.dam_break(dx)
    sol = Solver(cfg, st["fluid"], st["boundary"])
    sol.step(steps)
    sol.check()
    got = sol.download()
    fl = dict(st["fluid"])
    for k in ("positions", "velocities", "densities"):
        fl[k] = _np(got[k])
    return cfg, fl, st["boundary"]


def _walled(fl, bd):
    return {"fluid": _fluid64(fl), "boundary": _fluid64(bd)}


@pytest.mark.gpu
def test_walled_rates_vjp_matches_fp64_finite_differences():
    """Pass B + pass A + the mDBC wall densities of a walled domain (inviscid viscosity,
    boundary viscosity, gravity): the VJP chain rates -> gradient -> walls against FP64
    central differences of the oracle's right-hand side, which extrapolates the wall
    densities from the perturbed fluid."""
    _gpu()
    from diffsph_gb300.solver import Solver
    cfg, fl, bd = _advanced_dam_break()
    rng = np.random.default_rng(21)
    n = fl["positions"].shape[0]
    abar = rng.standard_normal((n, 2)).astype(np.float32)
    drbar = rng.standard_normal(n).astype(np.float32)
    sol = Solver(cfg, fl, bd)
    dev = "cuda"
    xbar = torch.zeros(n, 2, device=dev)
    ubar = torch.zeros(n, 2, device=dev)
    rbar = torch.zeros(n, device=dev)
    gbar = torch.zeros(n, 2, device=dev)
    wbar = torch.zeros(sol.nB, device=dev)
    sol.vjp_rates(torch.as_tensor(abar, device=dev), torch.as_tensor(drbar, device=dev), xbar, ubar, rbar, gbar,
                  None, wbar)
    sol.vjp_gradient(gbar, xbar, rbar, wbar)
    assert float(wbar.abs().max()) > 0
    sol.vjp_walls(wbar, xbar, rbar)
    grads = {"positions": _np(xbar), "velocities": _np(ubar), "densities": _np(rbar)}
    base = _walled(fl, bd)

    def phi(state):
        (_, dudt, drho), _ = O.simulation_step(state, cfg)
        return float(np.sum(abar * dudt) + np.sum(drbar * drho))

    d = _dirs(cfg, fl, rng)
    for key in ("positions", "velocities", "densities"):
        sp, sm = copy.deepcopy(base), copy.deepcopy(base)
        sp["fluid"][key] = sp["fluid"][key] + EPS * d[key]
        sm["fluid"][key] = sm["fluid"][key] - EPS * d[key]
        fd = (phi(sp) - phi(sm)) / (2 * EPS)
        pred = float(np.sum(grads[key].astype(np.float64) * d[key]))
        assert _rel(pred, fd) < RTOL, (key, pred, fd)


@pytest.mark.gpu
def test_wall_density_vjp_matches_fp64_finite_differences():
    """sph_solver_vjp_walls alone: sum_b w_b rho_b(fluid) with the mDBC extrapolation
    (fp64 moment solve; Shepard fallback where a ghost has few fluid neighbors)."""
    _gpu()
    from diffsph_gb300.solver import Solver
    cfg, fl, bd = _advanced_dam_break(steps=20)
    rng = np.random.default_rng(22)
    sol = Solver(cfg, fl, bd)
    nB = sol.nB
    w = rng.standard_normal(nB).astype(np.float32)
    n = fl["positions"].shape[0]
    xbar = torch.zeros(n, 2, device="cuda")
    rbar = torch.zeros(n, device="cuda")
    sol.vjp_walls(torch.as_tensor(w, device="cuda"), xbar, rbar)
    grads = {"positions": _np(xbar), "densities": _np(rbar)}
    base = _walled(fl, bd)

    def phi(state):
        rho_b, _, _ = O.mdbc_density(state["boundary"], state["fluid"], cfg)
        return float(np.sum(w * rho_b))

    d = _dirs(cfg, fl, rng)
    for key in ("positions", "densities"):
        sp, sm = copy.deepcopy(base), copy.deepcopy(base)
        sp["fluid"][key] = sp["fluid"][key] + EPS * d[key]
        sm["fluid"][key] = sm["fluid"][key] - EPS * d[key]
        fd = (phi(sp) - phi(sm)) / (2 * EPS)
        pred = float(np.sum(grads[key].astype(np.float64) * d[key]))
        assert _rel(pred, fd) < RTOL, (key, pred, fd)


@pytest.mark.gpu
def test_walled_shift_vjp_matches_fp64_finite_differences():
    """The delta+ shift next to walls: the adjoint of the fluid positions and densities and
    of the wall densities it reads (as uploaded), against the oracle's solveShifting."""
    _gpu()
    from diffsph_gb300.solver import Solver
    cfg, fl, bd = _advanced_dam_break(steps=30)
    rng = np.random.default_rng(23)
    n = fl["positions"].shape[0]
    bdd = dict(bd)
    rho_b, _, _ = O.mdbc_density(_fluid64(bd), _fluid64(fl), cfg)
    bdd["densities"] = rho_b.astype(np.float32)
    sol = Solver(cfg, fl, bdd)
    xbn = rng.standard_normal((n, 2)).astype(np.float32)
    dev = "cuda"
    xbar = torch.zeros(n, 2, device=dev)
    rbar = torch.zeros(n, device=dev)
    mach = torch.zeros(n, device=dev)
    wbar = torch.zeros(sol.nB, device=dev)
    sol.vjp_shift(torch.as_tensor(xbn, device=dev), xbar, rbar, mach, wbar)
    u = np.asarray(fl["velocities"], np.float64)
    sp_ = np.linalg.norm(u, axis=1)
    k = int(np.argmax(sp_))
    ubar = np.zeros((n, 2))
    ubar[k] = float(mach.double().sum()) / float(cfg["fluid"]["cs"]) * u[k] / sp_[k]
    grads = {"positions": _np(xbar), "velocities": ubar, "densities": _np(rbar)}
    base = _walled(fl, bdd)

    def phi(state):
        dx, _ = O.solve_shifting(state, cfg)
        return float(np.sum(xbn * (state["fluid"]["positions"] + dx)))

    d = _dirs(cfg, fl, rng)
    for key in ("positions", "velocities", "densities"):
        a, b = copy.deepcopy(base), copy.deepcopy(base)
        a["fluid"][key] = a["fluid"][key] + EPS * d[key]
        b["fluid"][key] = b["fluid"][key] - EPS * d[key]
        fd = (phi(a) - phi(b)) / (2 * EPS)
        pred = float(np.sum(np.asarray(grads[key], np.float64) * d[key]))
        assert _rel(pred, fd) < RTOL, (key, pred, fd)
    # the wall densities move the shift only (its increments are ~1e-4 of the positions, so
    # the differences take the increments alone, clear of the positions' rounding)
    def phi_dx(state):
        dx, _ = O.solve_shifting(state, cfg)
        return float(np.sum(xbn * dx))

    db = rng.standard_normal(sol.nB)
    a, b = copy.deepcopy(base), copy.deepcopy(base)
    a["boundary"]["densities"] = a["boundary"]["densities"] + EPS * db
    b["boundary"]["densities"] = b["boundary"]["densities"] - EPS * db
    fd = (phi_dx(a) - phi_dx(b)) / (2 * EPS)
    pred = float(np.sum(_np(wbar).astype(np.float64) * db))
    assert _rel(pred, fd) < RTOL, ("wall densities", pred, fd)


@pytest.mark.gpu
def test_walled_rollout_gradient_matches_fp64_finite_differences():
    """A 10-step dam-break rollout (walls, inviscid and boundary viscosity, gravity):
    gradients of a velocity loss with respect to the initial positions, velocities and
    densities against FP64 central differences of the oracle's full steps."""
    _gpu()
    from diffsph_gb300.adjoint import rollout
    cfg, fl, bd = _advanced_dam_break(steps=40)
    steps = 10
    n = fl["positions"].shape[0]
    rng = np.random.default_rng(24)
    target = rng.standard_normal((n, 2)) * 0.1
    dev = "cuda"
    u0 = torch.as_tensor(fl["velocities"], device=dev).clone().requires_grad_(True)
    rho0 = torch.as_tensor(fl["densities"], device=dev).clone().requires_grad_(True)
    x0 = torch.as_tensor(fl["positions"], device=dev).clone().requires_grad_(True)
    _, u, _ = rollout(cfg, fl, steps, checkpoint_every=4, x0=x0, u0=u0, rho0=rho0, boundary=bd)
    loss = torch.mean((u - torch.as_tensor(target, dtype=torch.float32, device=dev)) ** 2)
    loss.backward()

    def L(fluid):
        s = {"fluid": _fluid64(fluid), "boundary": _fluid64(bd)}
        for _ in range(steps):
            s, _ = O.full_step(s, cfg)
        return float(np.mean((s["fluid"]["velocities"] - target) ** 2))

    f64 = _fluid64(fl)
    ref64 = L(f64)
    assert abs(float(loss.detach()) - ref64) <= 1e-4 * ref64
    grads = {"positions": _np(x0.grad), "velocities": _np(u0.grad), "densities": _np(rho0.grad)}
    d = _dirs(cfg, fl, rng)
    for key in ("velocities", "positions", "densities"):
        a, b = _fluid64(f64), _fluid64(f64)
        a[key] = a[key] + EPS * d[key]
        b[key] = b[key] - EPS * d[key]
        fd = (L(a) - L(b)) / (2 * EPS)
        pred = float(np.sum(grads[key].astype(np.float64) * d[key]))
        assert _rel(pred, fd) < RTOL, (key, pred, fd)


@pytest.mark.gpu
def test_vjp_rejects_unsupported_configurations():
    """The summation density has no adjoint; a walled solver needs the wall-density adjoint."""
    _gpu()
    from diffsph_gb300 import _lib
    from diffsph_gb300.solver import Solver
    cfg, st = scenes.dam_break(1.0 / 32)
    sol = Solver(cfg, st["fluid"], st["boundary"])
    n = sol.nF
    z2 = torch.zeros(n, 2, device="cuda")
    z1 = torch.zeros(n, device="cuda")
    with pytest.raises(_lib.SphError) as e:
        sol.vjp_rates(z2, z1, z2, z2, z1)  # no rhob_bar with walls
    assert e.value.code == 1
    cfg2, st2 = scenes.fourier_periodic(24, seed=1)
    cfg2["simulation"]["densityScheme"] = "summation"
    sol2 = Solver(cfg2, st2["fluid"])
    m = sol2.nF
    with pytest.raises(_lib.SphError) as e:
        sol2.vjp_rates(torch.zeros(m, 2, device="cuda"), torch.zeros(m, device="cuda"), torch.zeros(m, 2, device="cuda"),
                       torch.zeros(m, 2, device="cuda"), torch.zeros(m, device="cuda"))
    assert e.value.code == 1


@pytest.mark.parametrize("change", ["summation", "free_surface", "ips", "regions"])
def test_rollout_rejects_out_of_scope_configs(change):
    from diffsph_gb300.adjoint import rollout
    cfg, st = scenes.dam_break(1.0 / 32)
    if change == "summation":
        cfg["simulation"]["densityScheme"] = "summation"
    elif change == "free_surface":
        cfg["shifting"]["freeSurface"] = True
    elif change == "ips":
        cfg["shifting"]["scheme"] = "IPS"
    else:
        cfg["regions"] = [{"type": "outlet"}]
    with pytest.raises(ValueError):
        rollout(cfg, st["fluid"], 2, boundary=st["boundary"])


def _adjoint_fixture(name="fourier24_100"):
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"adjoint_{name}.npz")
    z = np.load(path)
    cfg = json.loads(bytes(z["config_json"]).decode())
    fl = {k.split("/")[-1]: z[k] for k in z.files if k.startswith("in/fluid/")}
    return z, cfg, fl


def test_oracle_rollout_matches_reference_100_steps():
    """The FP64 oracle's 100-step trajectory reproduces the reference's FP64 run (the
    golden fixture made by torch autograd through the reference)."""
    z, cfg, fl = _adjoint_fixture()
    out = _oracle_rollout(cfg, fl, int(z["steps"]))
    u = out["velocities"]
    assert float(np.max(np.abs(u - z["f64/u_final"]))) <= 1e-9 * float(np.max(np.abs(z["f64/u_final"])))
    loss = float(np.mean((u - z["target"]) ** 2))
    assert abs(loss - float(z["f64/loss"])) <= 1e-10 * float(z["f64/loss"])


def _rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["fourier24_100", "fourier128_100"])
def test_rollout_gradient_matches_reference_autograd_100_steps(name):
    """Gradients of the 100-step loss against the reference's own torch-autograd gradient
    (FP64 run): relative L2 error <= 1e-3 for the velocity, position and density blocks
    and relative error <= 1e-3 for nu. The reference's FP32 run is held to the same bar
    as a statement of what FP32 rounding costs. Cases: 24x24 particles, and 128x128 (the
    size of the 128^2 rollout of the adjoint benchmark; its first 100 steps)."""
    _gpu()
    from diffsph_gb300.adjoint import rollout
    z, cfg, fl = _adjoint_fixture(name)
    steps = int(z["steps"])
    dev = "cuda"
    x0 = torch.as_tensor(fl["positions"], device=dev).clone().requires_grad_(True)
    u0 = torch.as_tensor(fl["velocities"], device=dev).clone().requires_grad_(True)
    r0 = torch.as_tensor(fl["densities"], device=dev).clone().requires_grad_(True)
    nu = torch.tensor(float(cfg["diffusion"]["nu"]), dtype=torch.float64, requires_grad=True)
    _, u, _ = rollout(cfg, fl, steps, nu=nu, checkpoint_every=25, x0=x0, u0=u0, rho0=r0)
    loss = torch.mean((u - torch.as_tensor(z["target"], dtype=torch.float32, device=dev)) ** 2)
    loss.backward()
    assert abs(float(loss.detach()) - float(z["f64/loss"])) <= 1e-5 * float(z["f64/loss"])
    for name, g in (("u0", u0.grad), ("x0", x0.grad), ("rho0", r0.grad)):
        assert _rel_l2(z[f"f32/{name}"], z[f"f64/{name}"]) < 1e-3
        assert _rel_l2(_np(g), z[f"f64/{name}"]) < 1e-3, name
    assert abs(float(nu.grad) - float(z["f64/nu"])) <= 1e-3 * abs(float(z["f64/nu"]))


@pytest.mark.gpu
def test_rollout_1000_steps_loss_matches_and_gradient_is_chaotic():
    """The whole 128x128 rollout of the adjoint benchmark (1000 steps, checkpoints every 25)
    against the reference's autograd (tests/golden/adjoint_fourier128_1000.npz). At this
    horizon the gradient with respect to the initial state is chaotic: the reference's own
    fp32 and fp64 gradients are uncorrelated (cosine 0.04 for u0), and moving the initial
    positions by 1e-7 (an fp32 rounding) turns this solver's gradient to cosine 0.19 of
    itself at 1000 steps, 0.76 at 600 and 0.99999 at 300. So only the forward is held to the
    reference here: the loss within 1e-4 of the fp64 run; the gradients are bounded and
    reported (their cosines with the fp64 gradient), and the 100-step checks above are the
    gradient's parity test at this size."""
    _gpu()
    import os
    from diffsph_gb300.adjoint import rollout
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "adjoint_fourier128_1000.npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    z, cfg, fl = _adjoint_fixture("fourier128_1000")
    steps = int(z["steps"])
    dev = "cuda"
    x0 = torch.as_tensor(fl["positions"], device=dev).clone().requires_grad_(True)
    u0 = torch.as_tensor(fl["velocities"], device=dev).clone().requires_grad_(True)
    r0 = torch.as_tensor(fl["densities"], device=dev).clone().requires_grad_(True)
    nu = torch.tensor(float(cfg["diffusion"]["nu"]), dtype=torch.float64, requires_grad=True)
    _, u, _ = rollout(cfg, fl, steps, nu=nu, checkpoint_every=25, x0=x0, u0=u0, rho0=r0)
    loss = torch.mean((u - torch.as_tensor(z["target"], dtype=torch.float32, device=dev)) ** 2)
    loss.backward()
    assert abs(float(loss.detach()) - float(z["f64/loss"])) <= 1e-4 * float(z["f64/loss"])
    report = []
    for name, g in (("u0", u0.grad), ("x0", x0.grad), ("rho0", r0.grad)):
        a = _np(g).astype(np.float64).ravel()
        b = np.asarray(z[f"f64/{name}"], np.float64).ravel()
        c = np.asarray(z[f"f32/{name}"], np.float64).ravel()
        assert np.all(np.isfinite(a)) and np.linalg.norm(a) < 100 * np.linalg.norm(b), name
        report.append(f"{name}: cosine with fp64 {a @ b / np.linalg.norm(a) / np.linalg.norm(b):.3f} "
                      f"(reference fp32 {c @ b / np.linalg.norm(c) / np.linalg.norm(b):.3f})")
    report.append(f"nu: {float(nu.grad):.4f} (reference fp64 {float(z['f64/nu']):.4f}, fp32 {float(z['f32/nu']):.4f})")
    print("; ".join(report))


@pytest.mark.gpu
def test_velocity_gradient_along_32_random_directions():
    """d loss / d u0 along 32 random directions against FP64 central differences
    (eps = 1e-6) of the oracle rollout: 24x24 periodic Fourier flow, 12 steps,
    checkpoints every 25 steps (one segment)."""
    _gpu()
    from diffsph_gb300.adjoint import rollout_loss_and_grad
    cfg, st = scenes.fourier_periodic(24, seed=8, jitter=0.1)
    fl = st["fluid"]
    steps = 12
    target = scenes.fourier_velocity(np.asarray(fl["positions"], np.float64), np.random.default_rng(42))
    loss, gu, _ = rollout_loss_and_grad(cfg, fl, target, steps)
    g = _np(gu).astype(np.float64)
    f64 = _fluid64(fl)
    rng = np.random.default_rng(2024)
    errs = []
    for _ in range(32):
        d = rng.standard_normal(f64["velocities"].shape)
        a, b = _fluid64(f64), _fluid64(f64)
        a["velocities"] += EPS * d
        b["velocities"] -= EPS * d
        la = np.mean((_oracle_rollout(cfg, a, steps)["velocities"] - target) ** 2)
        lb = np.mean((_oracle_rollout(cfg, b, steps)["velocities"] - target) ** 2)
        fd = (la - lb) / (2 * EPS)
        errs.append(_rel(float(np.sum(g * d)), fd))
    assert max(errs) < RTOL, max(errs)


@pytest.mark.gpu
@pytest.mark.parametrize("density_update", ["reference", "rational"])
def test_graph_replay_gives_the_eager_gradient(density_update):
    """The CUDA-graph replay of the recomputation and of the step VJPs (and of the fused
    forward, on a side stream) gives the eager gradient: 23 steps, checkpoints every 9, so
    that segments of odd length exercise the eager remainder too."""
    _gpu()
    from diffsph_gb300.adjoint import rollout_loss_and_grad
    cfg, st = scenes.fourier_periodic(32, seed=6, jitter=0.1)
    cfg["integration"]["densityUpdate"] = density_update
    target = scenes.fourier_velocity(np.asarray(st["fluid"]["positions"], np.float64), np.random.default_rng(3))
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        lg, gg, ng = rollout_loss_and_grad(cfg, st["fluid"], target, 23, checkpoint_every=9, use_graphs=True)
        le, ge, ne = rollout_loss_and_grad(cfg, st["fluid"], target, 23, checkpoint_every=9, use_graphs=False)
    torch.cuda.synchronize()
    assert abs(lg - le) <= 1e-6 * abs(le)
    assert float((gg - ge).abs().max()) <= 1e-5 * float(ge.abs().max())
    assert abs(ng - ne) <= 1e-5 * abs(ne)
