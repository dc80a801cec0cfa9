"""Host wrapper of the fused sm_103a solver (libsph103.so, include/sph103.h).

``Solver`` owns one caller-allocated workspace (a torch uint8 tensor on the GPU) and the
library handle. All device work runs on torch's current CUDA stream. The configuration
is the reference's nested config dict (src/diffSPH/v2/parameters.py keys).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib

VISC_SCHEMES = {"deltaSPH_viscid": 0, "deltaSPH_inviscid": 1}
# simulation.densityScheme (parameters.py:24, deltaPlus.py:193-198)
DENSITY_SCHEMES = {"continuity": 0, "summation": 1}
# kernel.name (parameters.py:37): the kernels evaluate the Wendland C2 kernel only
KERNELS = ("Wendland2",)
# the neighbor passes the autotuner shapes separately, in the C interface's order
TUNED_PASSES = ("pass_a_scan", "pass_a_filter", "pass_b", "shift", "density_sum")
DEFAULT_SKIN = 1.15


def _f(x) -> float:
    if isinstance(x, torch.Tensor):
        return float(x.detach().cpu().reshape(-1)[0])
    if isinstance(x, np.ndarray):
        return float(x.reshape(-1)[0])
    return float(x)


def _pair(x):
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().tolist()
    if isinstance(x, np.ndarray):
        x = x.tolist()
    if isinstance(x, (list, tuple)):
        return [float(v) for v in x][:2]
    return [float(x)] * 2


def _periodic(cfg):
    per = cfg["domain"].get("periodicity", cfg["domain"].get("periodic", False))
    if isinstance(per, torch.Tensor):
        per = per.detach().cpu().tolist()
    if isinstance(per, np.ndarray):
        per = per.tolist()
    if isinstance(per, bool):
        per = [per, per]
    return [bool(per[0]), bool(per[1])]


def domain_struct(cfg) -> _lib.Domain:
    d = _lib.Domain()
    mn, mx = _pair(cfg["domain"]["minExtent"]), _pair(cfg["domain"]["maxExtent"])
    per = _periodic(cfg)
    for a in range(2):
        d.min[a], d.max[a], d.periodic[a] = mn[a], mx[a], int(per[a])
    return d


def default_capacity(skin: float, support: float, dx: float) -> int:
    """Candidate slots per particle: 1.5x the lattice count within skin*H, plus margin."""
    n = math.pi * (skin * support / dx) ** 2
    return int(math.ceil((1.5 * n + 16) / 8.0) * 8)


def _uniform(arr, name):
    a = arr.detach() if isinstance(arr, torch.Tensor) else torch.as_tensor(arr)
    v = a.reshape(-1)
    if v.numel() and not bool((v == v[0]).all()):
        raise ValueError(f"the fused solver needs a uniform particle {name}")
    return float(v[0]) if v.numel() else 0.0


def verlet_scale(cfg) -> float:
    """neighborhood.verletScale (default 1.5, neighborhood.py:603)."""
    return _f(cfg.get("neighborhood", {}).get("verletScale", 1.5))


def wants_verlet_reuse(cfg, params: _lib.Params) -> bool:
    """Verlet reuse of the cell sort and skin list, as the reference reuses its neighbor
    structure while neighborhood.verletScale > 1 (neighborhood.py:505-518), on walled and
    periodic domains alike."""
    return verlet_scale(cfg) > 1.0


def verlet_sort_limit(scale: float, support: float, skin_lim: float) -> float:
    """The displacement since the last sort past which a step sorts again under Verlet
    reuse: the stricter of the reference's rule (a rebuild once 2 max|dx| > (verletScale - 1) h,
    neighborhood.py:509-513) and 0.7 of the skin list's limit (sph_solver_set_verlet_scale)."""
    return min((scale - 1.0) * support / 2.0, 0.7 * skin_lim)


def params_from_config(cfg, mass: float, skin: float = DEFAULT_SKIN, capacity: int | None = None) -> _lib.Params:
    p = _lib.Params()
    p.domain = domain_struct(cfg)
    p.support = _f(cfg["particle"]["support"])
    p.dx = _f(cfg["particle"]["dx"])
    p.mass = mass
    p.rho0 = _f(cfg["fluid"]["rho0"])
    p.cs = _f(cfg["fluid"]["cs"])
    eos = cfg.get("EOS", {})
    if eos.get("type", "stiffTait") != "stiffTait":
        raise ValueError(f"EOS {eos.get('type')} is not implemented by the fused solver (stiffTait is)")
    p.gamma = _f(eos.get("polytropicExponent", 7.0))
    p.kernel_scale = _f(cfg["kernel"]["kernelScale"])
    kname = cfg["kernel"].get("name", "Wendland2")
    if kname not in KERNELS:
        raise ValueError(f"kernel {kname} is not implemented by the fused solver (Wendland2 is)")
    ds = cfg.get("simulation", {}).get("densityScheme", "continuity")
    if ds not in DENSITY_SCHEMES:
        raise ValueError(f"density scheme {ds} is not implemented (continuity, summation are)")
    p.density_scheme = DENSITY_SCHEMES[ds]
    diff = cfg["diffusion"]
    if diff.get("densityScheme", "deltaSPH") != "deltaSPH":
        raise ValueError("only the deltaSPH density diffusion scheme is implemented")
    if diff.get("pi-switch", False):
        raise ValueError("the viscosity pi-switch is not implemented")
    p.delta = _f(diff.get("delta", 0.1))
    vs = diff.get("velocityScheme", "deltaSPH_inviscid")
    if vs not in VISC_SCHEMES:
        raise ValueError(f"viscosity scheme {vs} is not implemented (deltaSPH_viscid, deltaSPH_inviscid are)")
    p.visc_scheme = VISC_SCHEMES[vs]
    p.nu, p.alpha, p.eps = _f(diff.get("nu", 0.01)), _f(diff.get("alpha", 0.01)), _f(diff.get("eps", 1e-6))
    bd = dict(diff)
    bd.update({k: v for k, v in cfg.get("boundaryDiffusion", {}).items() if v is not None})
    bvs = bd.get("velocityScheme", vs)
    if bvs not in VISC_SCHEMES:
        raise ValueError(f"boundary viscosity scheme {bvs} is not implemented")
    p.bvisc_scheme = VISC_SCHEMES[bvs]
    p.b_nu, p.b_alpha, p.b_eps = _f(bd.get("nu", p.nu)), _f(bd.get("alpha", p.alpha)), _f(bd.get("eps", p.eps))
    g = cfg.get("gravity", {})
    p.gravity_on = int(bool(g.get("active", False)))
    if p.gravity_on and g.get("gravityMode", "constant") != "constant":
        raise ValueError("only constant gravity is implemented")
    direction = _pair(g.get("direction", [0.0, -1.0]))
    mag = _f(g.get("magnitude", 9.81))
    p.gravity[0], p.gravity[1] = direction[0] * mag, direction[1] * mag
    p.dt = _f(cfg["timestep"]["dt"])
    if cfg.get("regions"):
        raise ValueError("the fused solver has a fixed particle count and no open-boundary regions; "
                         "diffsph_gb300.regions serves the reference's step for them")
    sh = cfg.get("shifting", {})
    if sh.get("scheme", "deltaSPH") not in ("deltaSPH", "IPS") or int(sh.get("maxIterations", 1)) != 1:
        raise ValueError("only delta+ and implicit (IPS) shifting with one iteration are implemented")
    if sh.get("freeSurface", False) and (sh.get("surfaceDetection", "Barcasco") != "Barcasco"
                                         or sh.get("normalScheme", "lambda") != "lambda"
                                         or sh.get("projectionScheme", "mat") != "mat"
                                         or sh.get("useExtendedMask", False)):
        raise ValueError("free-surface shifting is implemented with surfaceDetection 'Barcasco', normalScheme "
                         "'lambda', projectionScheme 'mat' and useExtendedMask off")
    if sh.get("scheme", "deltaSPH") == "IPS" and (sh.get("summationDensity", False)
                                                  or sh.get("initialization", "zero") != "zero"):
        raise ValueError("implicit shifting is implemented with summationDensity off and a zero initial guess")
    p.shift_on = int(bool(sh.get("active", True)))
    p.shift_R, p.shift_n = _f(sh.get("R", 0.25)), _f(sh.get("n", 4))
    p.shift_CFL, p.shift_threshold = _f(sh.get("CFL", 1.5)), _f(sh.get("threshold", 0.5))
    p.compute_mach = int(bool(sh.get("computeMach", True)))
    p.density_update = 0 if cfg.get("integration", {}).get("densityUpdate", "reference") == "reference" else 1
    if p.density_scheme == 1 and p.density_update != 0:
        raise ValueError("the summation density replaces the integrated one: densityUpdate must be 'reference'")
    p.skin = skin
    p.capacity = capacity or default_capacity(skin, p.support, p.dx)
    return p


def _dev(t, dtype=torch.float32):
    t = torch.as_tensor(t)
    return t.to(device="cuda", dtype=dtype).contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _pinned(t) -> bool:
    """A page-locked float32 contiguous host tensor: the solver's upload and download kernels
    read and write it directly (no staging copy)."""
    return (isinstance(t, torch.Tensor) and not t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
            and t.is_pinned())


def _io(t):
    """The array as the upload kernel reads it: a page-locked host tensor as it is, anything
    else copied to the device."""
    return t if _pinned(t) else _dev(t)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Solver:
    """One fluid (plus optional static mDBC boundary) particle set advanced on the GPU."""

    def __init__(self, config, fluid, boundary=None, skin: float = DEFAULT_SKIN, capacity: int | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("the sph103 solver needs a CUDA device")
        self.lib = _lib.load()
        self.config = config
        use_b = boundary is not None and bool(config.get("boundary", {}).get("active", boundary is not None))
        self.nF = int(torch.as_tensor(fluid["positions"]).shape[0])
        self.nB = int(torch.as_tensor(boundary["positions"]).shape[0]) if use_b else 0
        mass = _uniform(fluid["masses"], "mass")
        if self.nB and abs(_uniform(boundary["masses"], "mass") - mass) > 1e-6 * mass:
            raise ValueError("fluid and boundary particles must share one mass")
        for part in ([fluid, boundary] if self.nB else [fluid]):
            if abs(_uniform(part["supports"], "support") - _f(config["particle"]["support"])) > 1e-6 * _f(config["particle"]["support"]):
                raise ValueError("particle supports must equal config['particle']['support']")
        self.params = params_from_config(config, mass, skin, capacity)
        nbytes = ctypes.c_size_t()
        _lib.check("sph_solver_workspace_bytes",
                   self.lib.sph_solver_workspace_bytes(ctypes.byref(self.params), self.nF, self.nB, ctypes.byref(nbytes)))
        self.workspace = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device="cuda")
        base = self.workspace.data_ptr()
        self._ws_ptr = (base + 255) & ~255
        h = ctypes.c_void_p()
        _lib.check("sph_solver_create", self.lib.sph_solver_create(
            ctypes.byref(self.params), self.nF, self.nB, ctypes.c_void_p(self._ws_ptr), nbytes.value, ctypes.byref(h)))
        self.handle = h
        self.upload(fluid, boundary if self.nB else None)
        # the static wall particles (re-uploads of the fluid state pass them again)
        self.boundary = ({k: _dev(boundary[k]) for k in ("positions", "normals", "distances")}
                         if self.nB else None)
        sh = config.get("shifting", {})
        if sh.get("scheme", "deltaSPH") == "IPS":
            self.set_ips(rtol=float(sh.get("rtol", 1e-4)), max_iter=int(sh.get("maxSolveIter", 64)),
                         solver_threshold=float(sh.get("solverThreshold", -0.5)))
        if sh.get("freeSurface", False):
            sd = config.get("surfaceDetection", {})
            self.set_free_surface(threshold=_f(sd.get("BarecascoThreshold", math.pi / 3)),
                                  expansion=int(sd.get("expansionIterations", 2)),
                                  scaling=_f(sh.get("surfaceScaling", 0.1)))
        self.verlet_reuse = False
        if wants_verlet_reuse(config, self.params):
            self.set_verlet_reuse(True)
            _lib.check("sph_solver_set_verlet_scale",
                       self.lib.sph_solver_set_verlet_scale(self.handle, verlet_scale(config)))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.sph_solver_destroy(h)
            self.handle = None

    # -- state transfer ------------------------------------------------------------------
    def upload(self, fluid, boundary=None):
        """Load a state (original order). Page-locked float32 host tensors are read by the
        upload kernel directly over the host link; other arrays are copied to the device."""
        xf, uf, rf = _io(fluid["positions"]), _io(fluid["velocities"]), _io(fluid["densities"])
        args = [xf, uf, rf, None, None, None, None]
        if self.nB:
            args[3:] = [_io(boundary["positions"]), _io(boundary["normals"]), _io(boundary["distances"]),
                        _io(boundary["densities"]) if "densities" in boundary else None]
        self._keep = args
        _lib.check("sph_solver_upload", self.lib.sph_solver_upload(self.handle, *[_ptr(a) for a in args], _stream()))

    def download(self, out=None):
        """The state in the original order: positions, velocities, densities (and the wall
        densities). ``out``: caller tensors to write into, float32 and contiguous, on the device
        or page-locked on the host (written by the download kernel directly over the host link;
        complete once the current stream has reached this call)."""
        if out is None:
            out = {"positions": torch.empty(self.nF, 2, device="cuda"),
                   "velocities": torch.empty(self.nF, 2, device="cuda"),
                   "densities": torch.empty(self.nF, device="cuda")}
            rb = torch.empty(self.nB, device="cuda") if self.nB else None
        else:
            out = dict(out)
            rb = out.get("boundary_densities") if self.nB else None
            if self.nB and rb is None:
                raise ValueError("out needs boundary_densities for a solver with walls")
            need = {"positions": 2 * self.nF, "velocities": 2 * self.nF, "densities": self.nF,
                    "boundary_densities": self.nB}
            for k, n in need.items():
                t = out.get(k)
                if t is None or (k == "boundary_densities" and not self.nB):
                    continue
                if not (t.dtype == torch.float32 and t.is_contiguous() and (t.is_cuda or _pinned(t))):
                    raise ValueError(f"out[{k!r}] must be float32, contiguous, on the device or page-locked")
                if t.numel() != n:
                    raise ValueError(f"out[{k!r}] holds {t.numel()} values, the state {n}")
        _lib.check("sph_solver_download", self.lib.sph_solver_download(
            self.handle, _ptr(out["positions"]), _ptr(out["velocities"]), _ptr(out["densities"]), _ptr(rb), _stream()))
        if self.nB:
            out["boundary_densities"] = rb
        return out

    # -- compute ---------------------------------------------------------------------------
    def step(self, n: int = 1):
        _lib.check("sph_solver_step", self.lib.sph_solver_step(self.handle, int(n), _stream()))

    def graph_step(self, n: int = 2):
        """n steps replayed from a captured CUDA graph (n even, or any n >= 1 under Verlet
        reuse); needs a non-default stream."""
        if torch.cuda.current_stream().cuda_stream == 0:
            raise RuntimeError("graph_step needs a non-default CUDA stream (torch.cuda.stream(...))")
        _lib.check("sph_solver_graph_step", self.lib.sph_solver_graph_step(self.handle, int(n), _stream()))

    def integrate(self):
        _lib.check("sph_solver_integrate", self.lib.sph_solver_integrate(self.handle, _stream()))

    def shift(self):
        dx = torch.empty(self.nF, 2, device="cuda")
        _lib.check("sph_solver_shift", self.lib.sph_solver_shift(self.handle, _ptr(dx), _stream()))
        return dx

    def set_ips(self, rtol: float = 1e-4, max_iter: int = 64, solver_threshold: float = -0.5):
        """Implicit particle shifting (shifting.scheme 'IPS', src/diffSPH/v2/modules/shifting.py:
        780-880) in place of delta+; the defaults are the reference's (a negative solver
        threshold means dx / 2, parameters.py:238). ``set_ips(None)`` returns to delta+."""
        if rtol is None:
            _lib.check("sph_solver_set_ips", self.lib.sph_solver_set_ips(self.handle, None, None, 0))
            self._ips_ws = None
            return
        nbytes = ctypes.c_size_t()
        _lib.check("sph_solver_ips_workspace_bytes",
                   self.lib.sph_solver_ips_workspace_bytes(self.handle, ctypes.byref(nbytes)))
        self._ips_ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device="cuda")
        ptr = (self._ips_ws.data_ptr() + 255) & ~255
        dx = _f(self.config["particle"]["dx"])
        thr = dx / 2 if solver_threshold < 0 else solver_threshold
        p = _lib.IpsParams(float(rtol), int(max_iter), float(thr))
        _lib.check("sph_solver_set_ips", self.lib.sph_solver_set_ips(self.handle, ctypes.byref(p),
                                                                     ctypes.c_void_p(ptr), nbytes.value))

    def set_free_surface(self, threshold: float | None = math.pi / 3, expansion: int = 2, scaling: float = 0.1):
        """Free-surface handling of the shift (shifting.freeSurface; Barecasco detection,
        'lambda' normals, 'mat' projection; src/diffSPH/v2/modules/shifting.py:882-1019).
        ``set_free_surface(None)`` switches it off."""
        if threshold is None:
            _lib.check("sph_solver_set_free_surface", self.lib.sph_solver_set_free_surface(self.handle, None, None, 0))
            self._fs_ws = None
            return
        nbytes = ctypes.c_size_t()
        _lib.check("sph_solver_free_surface_workspace_bytes",
                   self.lib.sph_solver_free_surface_workspace_bytes(self.handle, ctypes.byref(nbytes)))
        self._fs_ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device="cuda")
        ptr = (self._fs_ws.data_ptr() + 255) & ~255
        p = _lib.FreeSurfaceParams(float(threshold), int(expansion), float(scaling))
        _lib.check("sph_solver_set_free_surface", self.lib.sph_solver_set_free_surface(
            self.handle, ctypes.byref(p), ctypes.c_void_p(ptr), nbytes.value))

    def free_surface_fields(self):
        """Surface flags, expanded mask, Lambdas and normals of the last shift's detection,
        for the fluid particles followed by the walls (original order)."""
        n = self.nF + self.nB
        fs = torch.empty(n, dtype=torch.uint8, device="cuda")
        fsm = torch.empty(n, dtype=torch.uint8, device="cuda")
        lam = torch.empty(n, device="cuda")
        nrm = torch.empty(n, 2, device="cuda")
        _lib.check("sph_solver_free_surface_fields", self.lib.sph_solver_free_surface_fields(
            self.handle, _ptr(fs), _ptr(fsm), _ptr(lam), _ptr(nrm), _stream()))
        return {"freeSurface": fs.bool(), "freeSurfaceMask": fsm.bool(), "Lambdas": lam, "normals": nrm}

    def ips_result(self):
        """(iterations, code) of the last implicit shifting solve; code is bicgstab_shifting's
        second return value."""
        it, code = ctypes.c_int32(), ctypes.c_int32()
        _lib.check("sph_solver_ips_result",
                   self.lib.sph_solver_ips_result(self.handle, ctypes.byref(it), ctypes.byref(code), _stream()))
        return int(it.value), int(code.value)

    def rhs(self, boundary_densities=None):
        """One right-hand side at the current state. ``boundary_densities`` (walls, original
        order) replaces the mDBC extrapolation when given (sph_solver_rhs_walls)."""
        o = {"dudt": torch.empty(self.nF, 2, device="cuda"), "drhodt": torch.empty(self.nF, device="cuda"),
             "gradRho^L": torch.empty(self.nF, 2, device="cuda"), "L": torch.empty(self.nF, 2, 2, device="cuda"),
             "pressures": torch.empty(self.nF, device="cuda"),
             "numNeighbors": torch.empty(self.nF, 2, dtype=torch.int32, device="cuda")}
        if boundary_densities is not None:
            rb = _dev(boundary_densities) if self.nB else None
            if rb is not None and rb.numel() != self.nB:
                raise ValueError("one density per wall particle")
            _lib.check("sph_solver_rhs_walls", self.lib.sph_solver_rhs_walls(
                self.handle, _ptr(rb), _ptr(o["dudt"]), _ptr(o["drhodt"]), _ptr(o["gradRho^L"]), _ptr(o["L"]),
                _ptr(o["pressures"]), _ptr(o["numNeighbors"]), _stream()))
            if self.nB:
                o["boundary_densities"] = rb
            return o
        rb = torch.empty(self.nB, device="cuda") if self.nB else None
        _lib.check("sph_solver_rhs", self.lib.sph_solver_rhs(
            self.handle, _ptr(o["dudt"]), _ptr(o["drhodt"]), _ptr(o["gradRho^L"]), _ptr(o["L"]), _ptr(o["pressures"]),
            _ptr(rb), _ptr(o["numNeighbors"]), _stream()))
        if self.nB:
            o["boundary_densities"] = rb
        return o

    # -- adjoint (fluid-only, viscid) -------------------------------------------------------
    def vjp_rates(self, abar, drbar, xbar, ubar, rbar, gbar=None, nu_part=None, rhob_bar=None):
        """Accumulates the pass-B vector-Jacobian product at the current state (see
        sph_solver_vjp_rates); all arrays are CUDA float32 in the original order. With walls
        the adjoint of the wall densities accumulates into rhob_bar (required)."""
        _lib.check("sph_solver_vjp_rates", self.lib.sph_solver_vjp_rates(
            self.handle, _ptr(abar), _ptr(drbar), _ptr(xbar), _ptr(ubar), _ptr(rbar), _ptr(gbar), _ptr(nu_part),
            _ptr(rhob_bar), _stream()))

    def vjp_gradient(self, gbar, xbar, rbar, rhob_bar=None):
        _lib.check("sph_solver_vjp_gradient", self.lib.sph_solver_vjp_gradient(
            self.handle, _ptr(gbar), _ptr(xbar), _ptr(rbar), _ptr(rhob_bar), _stream()))

    def vjp_shift(self, xbar_new, xbar, rbar, mach_part, rhob_bar=None):
        _lib.check("sph_solver_vjp_shift", self.lib.sph_solver_vjp_shift(
            self.handle, _ptr(xbar_new), _ptr(xbar), _ptr(rbar), _ptr(mach_part), _ptr(rhob_bar), _stream()))

    def vjp_walls(self, rhob_bar, xbar, rbar):
        """Pulls the adjoint of the mDBC wall densities at the current state back to the
        fluid positions and densities (sph_solver_vjp_walls)."""
        _lib.check("sph_solver_vjp_walls", self.lib.sph_solver_vjp_walls(
            self.handle, _ptr(rhob_bar), _ptr(xbar), _ptr(rbar), _stream()))

    def flags(self) -> int:
        f = ctypes.c_uint32()
        _lib.check("sph_solver_flags", self.lib.sph_solver_flags(self.handle, ctypes.byref(f), _stream()))
        return int(f.value)

    def check(self):
        """Raise if the device recorded a capacity overflow, a skin violation or a NaN."""
        f = self.flags()
        if f & _lib.FLAG_CAPACITY:
            raise _lib.SphError("sph_solver_step", 3)
        if f & _lib.FLAG_VERLET:
            raise _lib.SphError("sph_solver_step", 5)
        if f & _lib.FLAG_NONFINITE:
            raise _lib.SphError("sph_solver_step", 6)

    def autotune(self):
        """Pick the fastest launch shape of each neighbor pass for this problem. Returns
        ({pass: shape}, {pass: [ms per shape, -1 where it does not apply]}) with the passes
        named as in TUNED_PASSES."""
        k = self.lib.sph_solver_shapes()
        npass = self.lib.sph_solver_tuned_passes()
        ms = (ctypes.c_float * (k * npass))()
        shapes = (ctypes.c_int32 * npass)()
        _lib.check("sph_solver_autotune", self.lib.sph_solver_autotune(self.handle, shapes, ms, _stream()))
        names = TUNED_PASSES[:npass]
        return ({n: int(shapes[p]) for p, n in enumerate(names)},
                {n: [float(ms[p * k + s]) for s in range(k)] for p, n in enumerate(names)})

    def set_shape(self, shape: int, tuned_pass: str | None = None):
        """Force a launch shape on every neighbor pass, or on one (a name of TUNED_PASSES)."""
        if tuned_pass is None:
            _lib.check("sph_solver_set_shape", self.lib.sph_solver_set_shape(self.handle, int(shape)))
        else:
            p = TUNED_PASSES.index(tuned_pass)
            _lib.check("sph_solver_set_pass_shape", self.lib.sph_solver_set_pass_shape(self.handle, p, int(shape)))

    def shapes(self):
        npass = self.lib.sph_solver_tuned_passes()
        out = (ctypes.c_int32 * npass)()
        _lib.check("sph_solver_pass_shapes", self.lib.sph_solver_pass_shapes(self.handle, out))
        return {n: int(out[p]) for p, n in enumerate(TUNED_PASSES[:npass])}

    def set_verlet_reuse(self, on: bool):
        """Keep the cell sort and the skin list across steps until a particle moved 0.034 h
        (see sph_solver_set_verlet_reuse)."""
        _lib.check("sph_solver_set_verlet_reuse", self.lib.sph_solver_set_verlet_reuse(self.handle, int(bool(on))))
        self.verlet_reuse = bool(on)

    def sort_count(self) -> int:
        """Cell sorts since the last upload."""
        c = ctypes.c_uint32()
        _lib.check("sph_solver_sort_count", self.lib.sph_solver_sort_count(self.handle, ctypes.byref(c), _stream()))
        return int(c.value)

    def launches_per_step(self) -> int:
        return int(self.lib.sph_solver_launches_per_step(self.handle))

    # -- kernel timing -----------------------------------------------------------------------
    def kernel_classes(self):
        return [self.lib.sph_solver_kernel_name(c).decode() for c in range(self.lib.sph_solver_kernel_classes())]

    def set_timing(self, classes):
        names = self.kernel_classes()
        mask = 0
        for c in classes:
            mask |= 1 << names.index(c)
        _lib.check("sph_solver_set_timing", self.lib.sph_solver_set_timing(self.handle, mask))

    def kernel_times(self):
        k = self.lib.sph_solver_kernel_classes()
        ms = (ctypes.c_float * k)()
        cnt = (ctypes.c_int32 * k)()
        _lib.check("sph_solver_kernel_times", self.lib.sph_solver_kernel_times(self.handle, ms, cnt, _stream()))
        names = self.kernel_classes()
        return {names[c]: (float(ms[c]), int(cnt[c])) for c in range(k)}


class BatchSolver(Solver):
    """Many independent periodic fluid domains packed into one set of arrays and stepped by
    the same kernel launches (one solver handle for the whole batch)."""

    def __init__(self, configs, fluids, skin: float = DEFAULT_SKIN, capacity: int | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("the sph103 solver needs a CUDA device")
        if len(configs) != len(fluids) or not configs:
            raise ValueError("one config per domain")
        self.lib = _lib.load()
        self.config = configs[0]
        self.configs = configs
        nd = len(configs)
        counts = [int(torch.as_tensor(f["positions"]).shape[0]) for f in fluids]
        self.counts = counts
        self.nF = sum(counts)
        self.nB = 0
        P = (_lib.Params * nd)()
        for d, (cfg, fl) in enumerate(zip(configs, fluids)):
            if cfg.get("boundary", {}).get("active", False):
                raise ValueError("batched domains are fluid-only")
            P[d] = params_from_config(cfg, _uniform(fl["masses"], "mass"), skin, capacity)
        self.params = P
        n_arr = (ctypes.c_int64 * nd)(*counts)
        nbytes = ctypes.c_size_t()
        _lib.check("sph_batch_workspace_bytes", self.lib.sph_batch_workspace_bytes(P, n_arr, nd, ctypes.byref(nbytes)))
        self.workspace = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device="cuda")
        self._ws_ptr = (self.workspace.data_ptr() + 255) & ~255
        h = ctypes.c_void_p()
        _lib.check("sph_batch_create", self.lib.sph_batch_create(
            P, n_arr, nd, ctypes.c_void_p(self._ws_ptr), nbytes.value, ctypes.byref(h)))
        self.handle = h
        self.upload_domains(fluids)
        # Verlet reuse as for one domain (every domain's verletScale > 1): any domain whose
        # particles moved past its own limit sorts the batch
        self.verlet_reuse = False
        if all(wants_verlet_reuse(c, P[d]) for d, c in enumerate(configs)):
            scales = {verlet_scale(c) for c in configs}
            if len(scales) != 1:
                raise ValueError("the domains of a batch share one neighborhood.verletScale")
            self.set_verlet_reuse(True)
            _lib.check("sph_solver_set_verlet_scale",
                       self.lib.sph_solver_set_verlet_scale(self.handle, scales.pop()))

    def upload_domains(self, fluids):
        cat = {k: torch.cat([torch.as_tensor(f[k]).reshape(torch.as_tensor(f[k]).shape[0], -1).float()
                             for f in fluids]).squeeze(-1) for k in ("positions", "velocities", "densities")}
        self.upload(cat, None)

    def split(self, arr):
        """Split a concatenated per-particle array into the domains."""
        return list(torch.split(arr, self.counts))
