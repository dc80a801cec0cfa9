"""Initial conditions and configuration dictionaries for the benchmark workloads.

The configuration uses the reference's nested keys (``config['particle']['support']``,
``config['fluid']['cs']`` ...) with the values the reference's parser derives
(src/diffSPH/v2/parameters.py:193-245), so the same dict drives the reference, the
oracle and this package. Scenes:

* ``taylor_green``: periodic [-1,1]^2, cell-centred lattice of nx*nx particles
  (src/diffSPH/v2/sampling.py:55-77 convention), u = (-cos(pi x) sin(pi y),
  sin(pi x) cos(pi y)), p0 = -(rho0/4)(cos 2 pi x + cos 2 pi y), rho from the inverse
  stiff Tait EOS, viscid delta-SPH viscosity nu = 0.01.
* ``dam_break``: tank [0,4]x[0,2] with 3 layers of wall particles left, right and
  below (analytic normals pointing into the wall and negative distances, the
  convention of sampling.py:901-930), a water column [0,1]x[0,2], gravity 9.81,
  rho0 = 1000, c0 = 10 sqrt(2 g 2), inviscid artificial viscosity alpha = 0.01.
* ``fourier_periodic``: periodic [-1,1]^2 lattice with uniform jitter and a
  divergence-free velocity from a 16-mode random stream function (|k| <= 4,
  amplitude |k|^-2, uniform phases), normalised to max speed 1.

Support H = 4 dx (targetNeighbors = 16 pi), kernel scale H / (2 dx) = 2, time step
from the acoustic limit CFL H / (c0 kappa) with CFL = 0.3 (timestep.py:18).
"""
from __future__ import annotations

import math

import numpy as np


def _base_config(dx: float, rho0: float, cs: float, minE, maxE, periodic: bool, CFL: float = 0.3):
    support = 4.0 * dx
    kappa = support / (2.0 * dx)
    dt = CFL * support / cs / kappa
    return {
        "domain": {"minExtent": list(minE), "maxExtent": list(maxE), "dim": 2,
                   "periodic": periodic, "periodicity": [periodic, periodic]},
        "particle": {"dx": dx, "support": support},
        "kernel": {"name": "Wendland2", "kernelScale": kappa, "targetNeighbors": 16 * math.pi},
        "fluid": {"rho0": rho0, "cs": cs},
        "EOS": {"type": "stiffTait", "polytropicExponent": 7.0},
        "simulation": {"densityScheme": "continuity"},
        "neighborhood": {"verletScale": 1.5},
        "timestep": {"dt": dt, "active": False},
        "integration": {"scheme": "symplecticEuler"},
        "shifting": {"scheme": "deltaSPH", "R": 0.25, "n": 4, "CFL": 1.5, "computeMach": True,
                     "threshold": 0.05, "maxIterations": 1, "freeSurface": False},
        "gravity": {"active": False, "magnitude": 9.81, "direction": [0.0, -1.0, 0.0]},
        "boundary": {"active": False},
        "compute": {"checkNaN": False},
    }


def _lattice(x0, x1, y0, y1, dx, dtype=np.float32):
    nx = int(round((x1 - x0) / dx))
    ny = int(round((y1 - y0) / dx))
    xs = x0 + dx / 2 + dx * np.arange(nx, dtype=np.float64)
    ys = y0 + dx / 2 + dx * np.arange(ny, dtype=np.float64)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    return np.stack([X.ravel(), Y.ravel()], -1).astype(dtype)


def taylor_green(nx: int = 64, jitter: float = 0.0, seed: int = 0, dtype=np.float32):
    """Plain delta-SPH Taylor-Green vortex on [-1,1]^2 (nx*nx particles)."""
    dx = 2.0 / nx
    rho0, umax = 1.0, 1.0
    cs = 10.0 * umax
    cfg = _base_config(dx, rho0, cs, (-1.0, -1.0), (1.0, 1.0), True)
    cfg["diffusion"] = {"velocityScheme": "deltaSPH_viscid", "nu": 0.01, "alpha": 0.01,
                        "eps": 1e-6, "delta": 0.1, "densityScheme": "deltaSPH", "pi-switch": False}
    cfg["boundaryDiffusion"] = dict(cfg["diffusion"])
    x = _lattice(-1.0, 1.0, -1.0, 1.0, dx, np.float64)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        x = x + rng.uniform(-jitter * dx, jitter * dx, size=x.shape)
    u = np.stack([-np.cos(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1]),
                  np.sin(np.pi * x[:, 0]) * np.cos(np.pi * x[:, 1])], -1)
    gamma = cfg["EOS"]["polytropicExponent"]
    p0 = -(rho0 / 4.0) * (np.cos(2 * np.pi * x[:, 0]) + np.cos(2 * np.pi * x[:, 1]))
    rho = rho0 * (1 + gamma * p0 / (rho0 * cs ** 2)) ** (1.0 / gamma)
    n = x.shape[0]
    fluid = {
        "positions": x.astype(dtype), "velocities": u.astype(dtype), "densities": rho.astype(dtype),
        "masses": np.full(n, dx * dx * rho0, dtype), "supports": np.full(n, cfg["particle"]["support"], dtype),
        "areas": np.full(n, dx * dx, dtype),
    }
    return cfg, {"fluid": fluid}


def _wall_geometry(p, tank_w, tank_h):
    """Depth into the wall and unit normal (pointing into the wall) for a wall particle.

    The fluid region is R = [0, tank_w] x [0, inf); depth = |p - proj_R(p)|."""
    qx = np.clip(p[:, 0], 0.0, tank_w)
    qy = np.maximum(p[:, 1], 0.0)
    d = np.stack([p[:, 0] - qx, p[:, 1] - qy], -1)
    depth = np.linalg.norm(d, axis=-1)
    n = d / depth[:, None]
    return depth, n


def dam_break(dx: float = 1.0 / 256, layers: int = 3, hydrostatic: bool = True, dtype=np.float32,
              tank=(4.0, 2.0), column=(1.0, 2.0)):
    """Dam break with mDBC walls (tank 4x2, water column 1x2 at the left wall)."""
    g = 9.81
    rho0 = 1000.0
    cs = 10.0 * math.sqrt(2 * g * 2.0)
    tw, th = tank
    margin = (layers + 1) * dx
    cfg = _base_config(dx, rho0, cs, (-margin, -margin), (tw + margin, th + 0.5), False)
    cfg["diffusion"] = {"velocityScheme": "deltaSPH_inviscid", "nu": 0.01, "alpha": 0.01,
                        "eps": 1e-6, "delta": 0.1, "densityScheme": "deltaSPH", "pi-switch": False}
    cfg["boundaryDiffusion"] = dict(cfg["diffusion"])
    cfg["gravity"]["active"] = True
    cfg["boundary"] = {"active": True, "type": "mDBC", "static": True}
    xf = _lattice(0.0, column[0], 0.0, column[1], dx, np.float64)
    gamma = cfg["EOS"]["polytropicExponent"]
    if hydrostatic:
        p = rho0 * g * (column[1] - xf[:, 1])
        rho = rho0 * (1 + gamma * p / (rho0 * cs ** 2)) ** (1.0 / gamma)
    else:
        rho = np.full(xf.shape[0], rho0)
    nF = xf.shape[0]
    fluid = {
        "positions": xf.astype(dtype), "velocities": np.zeros((nF, 2), dtype), "densities": rho.astype(dtype),
        "masses": np.full(nF, dx * dx * rho0, dtype), "supports": np.full(nF, cfg["particle"]["support"], dtype),
        "areas": np.full(nF, dx * dx, dtype),
    }
    L = layers * dx
    left = _lattice(-L, 0.0, 0.0, th, dx, np.float64)
    right = _lattice(tw, tw + L, 0.0, th, dx, np.float64)
    bottom = _lattice(-L, tw + L, -L, 0.0, dx, np.float64)
    xb = np.concatenate([bottom, left, right])
    depth, nrm = _wall_geometry(xb, tw, th)
    nB = xb.shape[0]
    boundary = {
        "positions": xb.astype(dtype), "velocities": np.zeros((nB, 2), dtype),
        "densities": np.full(nB, rho0, dtype), "masses": np.full(nB, dx * dx * rho0, dtype),
        "supports": np.full(nB, cfg["particle"]["support"], dtype), "areas": np.full(nB, dx * dx, dtype),
        "normals": nrm.astype(dtype), "distances": (-depth).astype(dtype),
    }
    return cfg, {"fluid": fluid, "boundary": boundary}


def fourier_modes(rng, modes: int = 16, kmax: int = 4):
    """`modes` distinct integer wave vectors with 0 < |k| <= kmax, drawn without replacement;
    k and -k are one mode (sin(-k.x + phi) = -sin(k.x - phi)), so each is drawn as the
    representative with kx > 0, or kx = 0 and ky > 0. Returns (k [modes, 2] int, phases)."""
    cand = [(a, b) for a in range(0, kmax + 1) for b in range(-kmax, kmax + 1)
            if (a > 0 or b > 0) and a * a + b * b <= kmax * kmax]
    if modes > len(cand):
        raise ValueError(f"only {len(cand)} distinct modes have 0 < |k| <= {kmax}")
    pick = rng.choice(len(cand), size=modes, replace=False)
    ks = np.asarray([cand[p] for p in pick], np.int64)
    ph = rng.uniform(0, 2 * np.pi, size=modes)
    return ks, ph


def fourier_velocity(x, rng, modes: int = 16, kmax: int = 4, L: float = 2.0):
    """Divergence-free velocity from the stream function psi = sum |k|^-2 sin(k.x + phi)
    over `modes` distinct modes (fourier_modes): u = d psi / dy, v = -d psi / dx, scaled to a
    maximum speed of 1 over the sampled points."""
    kint, ph = fourier_modes(rng, modes, kmax)
    ks = kint.astype(np.float64) * (2 * np.pi / L)
    amp = 1.0 / np.sum(ks ** 2, axis=1)
    arg = x @ ks.T + ph
    c = np.cos(arg) * amp
    u = c @ ks[:, 1]      # d psi / dy
    v = -(c @ ks[:, 0])   # -d psi / dx
    vel = np.stack([u, v], -1)
    vel /= np.max(np.linalg.norm(vel, axis=-1))
    return vel


def fourier_periodic(nx: int = 128, seed: int = 0, jitter: float = 0.1, dtype=np.float32, L: float = 2.0):
    """Periodic square [-L/2, L/2]^2 of nx*nx particles (dx = L / nx) with a random
    divergence-free Fourier-mode initial field; the Taylor-Green parameters otherwise."""
    cfg, st = taylor_green(nx, 0.0, seed, dtype)
    rng = np.random.default_rng(seed)
    if L != 2.0:
        dx = L / nx
        cfg = _base_config(dx, 1.0, 10.0, (-L / 2, -L / 2), (L / 2, L / 2), True)
        cfg["diffusion"] = {"velocityScheme": "deltaSPH_viscid", "nu": 0.01, "alpha": 0.01,
                            "eps": 1e-6, "delta": 0.1, "densityScheme": "deltaSPH", "pi-switch": False}
        cfg["boundaryDiffusion"] = dict(cfg["diffusion"])
        n = nx * nx
        st = {"fluid": {"masses": np.full(n, dx * dx, dtype), "supports": np.full(n, cfg["particle"]["support"], dtype),
                        "areas": np.full(n, dx * dx, dtype)}}
    dx = cfg["particle"]["dx"]
    x = _lattice(-L / 2, L / 2, -L / 2, L / 2, dx, np.float64)
    x = x + rng.uniform(-jitter * dx, jitter * dx, size=x.shape)
    u = fourier_velocity(x, rng, L=L)
    st["fluid"]["positions"] = x.astype(dtype)
    st["fluid"]["velocities"] = u.astype(dtype)
    st["fluid"]["densities"] = np.full(x.shape[0], cfg["fluid"]["rho0"], dtype)
    return cfg, st


def batched_fourier(n_domains: int = 256, seed: int = 0, n_min: int = 1024, n_max: int = 65536,
                    jitter: float = 0.1, dtype=np.float32):
    """Independent periodic domains on [-1,1]^2 for the batched solver: per domain the particle
    count is drawn log-uniformly in [n_min, n_max] and rounded to a square lattice, positions
    get uniform jitter of 0.1 dx, and the velocity is a random divergence-free Fourier-mode
    field normalised to max speed 1; other parameters as in the Taylor-Green workload.
    Returns a list of (config, state)."""
    rng = np.random.default_rng(seed)
    out = []
    for d in range(n_domains):
        n = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        nx = max(16, int(round(np.sqrt(n))))
        out.append(fourier_periodic(nx, seed=int(rng.integers(0, 2**31 - 1)), jitter=jitter, dtype=dtype))
    return out
