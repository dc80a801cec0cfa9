"""Learned k-step continuous-convolution stepper on the sm_103a kernels.

No reference implementation exists for this part (the reference project has no learned
model). The network stands in for ``k`` plain delta-SPH steps of the periodic fluid-only
solver: from (x, u, rho) at time t it predicts the velocity and density increments over
k dt and a position correction (the shifting), over the same exact neighbor lists the
solver uses (|x_i - x_j| <= H, self included).

Architecture (rotation-aware continuous convolution):
    features h0 = (u, (rho/rho0 - 1) / 0.01, 1, 0 ...)                       [n, 16]
    4 layers    h <- silu(conv(h) + h S + b) (+ h when widths match), width 64
                conv(h)_i = sum_{b, c} E_i[b, c] W[b C + c, :],
                E_i[b, c] = sum_j phi_b(x_i - x_j) g_j[c] / N0,  N0 = pi (H / dx)^2,
                g_j = h_j - h_i in the first layer (the difference form of the SPH
                operators), g_j = h_j in the others; S is the self weight
                phi: 8 radial Chebyshev x 8 angular Fourier terms (libsph103 sph_cconv_aggregate)
    decoder     silu(Linear(64, 64)) -> Linear(64, 5): du (2), drho (1), dx (2), each scaled
                by the spread of the training targets
    update      u' = u + du,  rho' = rho + drho,  x' = x + k dt (u + u') / 2 + dx

The aggregation runs on the tensor cores (per particle E_i = Phi_i^T G_i, a tcgen05 MMA);
its transpose (backward) on the CUDA cores; the basis-weight contraction and both of its
backward products (dE = dy W^T, dW = E^T dy) run on the tcgen05 BF16 GEMM (FP32
accumulation). Weights are kept in FP32 and rounded to BF16 for every product.

``judged_rollout`` keeps the plain solver as fallback and judge: each segment of learned
steps is checked against the solver's own kinetic-energy rate (one right-hand side at the
segment start) and a density-deviation bound; a rejected segment is re-run by the solver.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .solver import Solver, domain_struct

BASIS = 64
WIDTH = 64
IN_CH = 16
OUT_CH = 5


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


_ERR = {}


def _err_word(device):
    key = torch.device(device).index or 0
    if key not in _ERR:
        _ERR[key] = torch.zeros(1, dtype=torch.int32, device=device)
    return _ERR[key]


# bit of the error word: a particle with more neighbors within the learned support than the
# aggregation's 64-edge capacity (its row was truncated to 64 edges)
ROW_OVERFLOW = 8


def check_device_errors():
    """Raise if a tcgen05 kernel recorded a wait that did not complete or a neighbor row
    longer than its capacity (synchronises)."""
    for k, w in _ERR.items():
        v = int(w.item())
        if v:
            w.zero_()
            raise RuntimeError(f"tcgen05 kernel error flags {v:#x} on device {k}")


def take_row_overflow() -> bool:
    """Read and clear the row-capacity flag (synchronises): True when a learned step since the
    last call met a particle with more than 64 neighbors within the learned support, whose
    aggregation was truncated. Any other flag raises as in check_device_errors."""
    hit = False
    for k, w in _ERR.items():
        v = int(w.item())
        if v:
            w.zero_()
            if v & ~ROW_OVERFLOW:
                raise RuntimeError(f"tcgen05 kernel error flags {v:#x} on device {k}")
            hit = True
    return hit


def gemm_tn(A, Bt, out=None, accumulate=False):
    """out[M, N] (+)= A[M, K] @ Bt[N, K]^T with BF16 inputs and FP32 output (tcgen05)."""
    if A.dtype != torch.bfloat16 or Bt.dtype != torch.bfloat16:
        raise TypeError("gemm_tn takes bfloat16 operands")
    if A.stride(1) != 1 or Bt.stride(1) != 1:
        raise ValueError("gemm_tn operands must be row-major")
    M, K = A.shape
    N = Bt.shape[0]
    if Bt.shape[1] != K:
        raise ValueError("inner dimensions differ")
    if out is None:
        out = torch.empty(M, N, device=A.device, dtype=torch.float32)
    lib = _lib.load()
    _lib.check("sph_gemm_bf16_tn", lib.sph_gemm_bf16_tn(
        _p(A), _p(Bt), _p(out), M, N, K, A.stride(0), Bt.stride(0), out.stride(0), int(bool(accumulate)),
        _p(_err_word(A.device)), _stream()))
    return out


def _pad128(n):
    return (n + 127) // 128 * 128


class Graph:
    """Exact neighbor lists (CSR, symmetric) of one or several equal periodic domains."""

    def __init__(self, x, config, n_domains=1):
        x = x.to("cuda", torch.float32).contiguous()
        n = x.shape[0]
        if n % n_domains:
            raise ValueError("particles must split evenly over the domains")
        per = n // n_domains
        H = float(config["particle"]["support"])
        dx = float(config["particle"]["dx"])
        lib = _lib.load()
        dom = domain_struct(config)
        st = _stream()
        hd = torch.full((per,), H, device="cuda")
        nb = ctypes.c_size_t()
        _lib.check("sph_neighbor_workspace_bytes",
                   lib.sph_neighbor_workspace_bytes(per, per, ctypes.byref(dom), H, ctypes.byref(nb)))
        wsb = (int(nb.value) + 255) // 256 * 256
        ws = torch.empty(wsb * n_domains + 256, dtype=torch.uint8, device="cuda")
        ws0 = (ws.data_ptr() + 255) & ~255
        counts = torch.empty(n_domains, per, dtype=torch.int32, device="cuda")
        offs = torch.empty(n_domains, per + 1, dtype=torch.int64, device="cuda")
        # counts and row offsets of every domain, one host synchronisation, then the indices
        for d in range(n_domains):
            xd = x[d * per:(d + 1) * per]
            _lib.check("sph_neighbor_count", lib.sph_neighbor_count(
                _p(xd), per, _p(xd), _p(hd), per, ctypes.byref(dom), H, ctypes.c_void_p(ws0 + d * wsb), wsb,
                _p(counts[d]), _p(offs[d]), st))
        totals = offs[:, -1].cpu()
        base = torch.zeros(n_domains + 1, dtype=torch.int64)
        base[1:] = torch.cumsum(totals, 0)
        self.nbr = torch.empty(int(base[-1]), dtype=torch.int32, device="cuda")
        for d in range(n_domains):
            xd = x[d * per:(d + 1) * per]
            _lib.check("sph_neighbor_fill_csr", lib.sph_neighbor_fill_csr(
                _p(xd), per, _p(xd), _p(hd), per, ctypes.byref(dom), H, ctypes.c_void_p(ws0 + d * wsb), wsb,
                _p(offs[d]), _p(self.nbr[int(base[d]):]), st))
        for d in range(1, n_domains):  # global particle indices of the packed domains
            self.nbr[int(base[d]):int(base[d + 1])] += d * per
        rows = offs[:, :-1] + base[:-1].cuda()[:, None]
        self.offsets = torch.cat([rows.reshape(-1), base[-1:].cuda()]).contiguous()
        self.x = x
        self.n = n
        self.npad = _pad128(n)
        self.H = H
        self.inv_norm = 1.0 / (math.pi * (H / dx) ** 2)
        self.domain = domain_struct(config)


def aggregate(g: Graph, h_bf16, relative=False, tensor_cores=True):
    """E [npad, 64 C] (bf16; rows >= n are zero) of features h [n, C] (bf16). The tensor-core
    kernel rounds the basis values to BF16; the CUDA-core kernel keeps them in FP32."""
    C = h_bf16.shape[1]
    E = torch.empty(g.npad, BASIS * C, dtype=torch.bfloat16, device="cuda")
    if g.npad > g.n:
        E[g.n:].zero_()
    lib = _lib.load()
    if tensor_cores:
        _lib.check("sph_cconv_aggregate_tc", lib.sph_cconv_aggregate_tc(
            _p(g.x), g.n, _p(g.offsets), _p(g.nbr), ctypes.byref(g.domain), g.H, g.inv_norm,
            _p(h_bf16.contiguous()), C, int(bool(relative)), _p(E), _p(_err_word(E.device)), _stream()))
    else:
        _lib.check("sph_cconv_aggregate", lib.sph_cconv_aggregate(
            _p(g.x), g.n, _p(g.offsets), _p(g.nbr), ctypes.byref(g.domain), g.H, g.inv_norm,
            _p(h_bf16.contiguous()), C, int(bool(relative)), _p(E), _stream()))
    return E


def aggregate_t(g: Graph, dE, C, relative=False):
    """dh [n, C] (fp32) = transpose of ``aggregate`` applied to dE [>= n, 64 C] (fp32)."""
    dh = torch.empty(g.n, C, device="cuda")
    _lib.check("sph_cconv_aggregate_t", _lib.load().sph_cconv_aggregate_t(
        _p(g.x), g.n, _p(g.offsets), _p(g.nbr), ctypes.byref(g.domain), g.H, g.inv_norm, _p(dE), dE.stride(0), C,
        int(bool(relative)), _p(dh), _stream()))
    return dh


class ConvFn(torch.autograd.Function):
    """y [n, 64] = aggregate(h) W, with W [64 C, 64] (FP32 master, BF16 products)."""

    @staticmethod
    def forward(ctx, h, W, g, relative=False):
        C = h.shape[1]
        E = aggregate(g, h.to(torch.bfloat16), relative)
        Wt = W.t().contiguous().to(torch.bfloat16)
        y = gemm_tn(E, Wt)
        ctx.save_for_backward(W)
        ctx.E, ctx.g, ctx.C, ctx.rel = E, g, C, relative
        return y[:g.n]

    @staticmethod
    def backward(ctx, dy):
        (W,) = ctx.saved_tensors
        g, E, C = ctx.g, ctx.E, ctx.C
        dyp = torch.zeros(g.npad, WIDTH, dtype=torch.bfloat16, device="cuda")
        dyp[:g.n] = dy
        dE = gemm_tn(dyp, W.to(torch.bfloat16).contiguous())       # [npad, 64 C]
        dh = aggregate_t(g, dE, C, ctx.rel)
        dW = gemm_tn(E.t().contiguous(), dyp.t().contiguous())     # [64 C, 64]
        return dh, dW, None, None


class CConvNet(torch.nn.Module):
    def __init__(self, layers=4, width=WIDTH, in_ch=IN_CH, out_ch=OUT_CH, seed=0):
        super().__init__()
        gen = torch.Generator().manual_seed(seed)
        self.W = torch.nn.ParameterList()
        self.S = torch.nn.ParameterList()
        self.b = torch.nn.ParameterList()
        cin = in_ch
        for _ in range(layers):
            K = BASIS * cin
            self.W.append(torch.nn.Parameter(torch.randn(K, width, generator=gen) * (2.0 / K) ** 0.5))
            self.S.append(torch.nn.Parameter(torch.randn(cin, width, generator=gen) * (1.0 / cin) ** 0.5))
            self.b.append(torch.nn.Parameter(torch.zeros(width)))
            cin = width
        self.dec1 = torch.nn.Linear(width, width)
        self.dec2 = torch.nn.Linear(width, out_ch)
        with torch.no_grad():
            self.dec2.weight.mul_(0.1)
            self.dec2.bias.zero_()
        self.register_buffer("out_scale", torch.ones(out_ch))

    def forward(self, feats, g):
        h = feats
        for layer, (W, S, b) in enumerate(zip(self.W, self.S, self.b)):
            y = ConvFn.apply(h, W, g, layer == 0) + h @ S + b
            hn = torch.nn.functional.silu(y)
            h = hn + h if hn.shape == h.shape else hn
        return self.dec2(torch.nn.functional.silu(self.dec1(h)))


def features(u, rho, rho0):
    n = u.shape[0]
    f = torch.zeros(n, IN_CH, device="cuda")
    f[:, 0:2] = u
    f[:, 2] = (rho / rho0 - 1.0) / 0.01
    f[:, 3] = 1.0
    return f


def _min_image(d, config):
    lo = config["domain"]["minExtent"]
    hi = config["domain"]["maxExtent"]
    out = d.clone()
    for a in range(2):
        ext = float(hi[a]) - float(lo[a])
        out[:, a] = d[:, a] - ext * torch.round(d[:, a] / ext)
    return out


def _wrap(x, config):
    lo = config["domain"]["minExtent"]
    hi = config["domain"]["maxExtent"]
    out = x.clone()
    for a in range(2):
        ext = float(hi[a]) - float(lo[a])
        out[:, a] = torch.remainder(x[:, a] - float(lo[a]), ext) + float(lo[a])
    return out


class LearnedStepper:
    """One learned step = k plain steps of the periodic fluid-only solver."""

    def __init__(self, config, net: CConvNet, k=4, n_domains=1):
        self.config, self.net, self.k, self.n_domains = config, net, k, n_domains
        self.dt = float(config["timestep"]["dt"])
        self.rho0 = float(config["fluid"]["rho0"])

    def predict(self, x, u, rho, g=None):
        g = g or Graph(x, self.config, self.n_domains)
        out = self.net(features(u, rho, self.rho0), g) * self.net.out_scale
        return out, g

    def apply(self, x, u, rho, out):
        u1 = u + out[:, 0:2]
        rho1 = rho + out[:, 2]
        x1 = x + (self.k * self.dt) * 0.5 * (u + u1) + out[:, 3:5]
        return _wrap(x1, self.config), u1, rho1

    @torch.no_grad()
    def step(self, x, u, rho):
        out, _ = self.predict(x, u, rho)
        return self.apply(x, u, rho, out)


def targets(config, k, a, b):
    """Network targets between frames a and b = frame a advanced k plain steps."""
    dt = float(config["timestep"]["dt"])
    du = b[1] - a[1]
    drho = b[2] - a[2]
    dxc = _min_image(b[0] - (a[0] + (k * dt) * 0.5 * (a[1] + b[1])), config)
    return torch.cat([du, drho[:, None], dxc], dim=1)


def generate_trajectories(n_traj, n_frames, nx, seed=0, k=4, jitter=0.1, chunk=256):
    """Solver trajectories of random divergence-free Fourier flows on the periodic square:
    returns (config, [[(x, u, rho) per frame] per trajectory]) with frames every k steps.
    The trajectories are stepped together, up to `chunk` domains packed into one batched
    solver (same kernel launches for all of them, k steps per captured graph replay); the
    batch steps every domain as a solver of its own would, up to the order of each particle's
    pair sums (the batch sorts when any of its domains needs it under Verlet reuse)."""
    from . import scenes
    from .solver import BatchSolver
    rng = np.random.default_rng(seed)
    seeds = [int(rng.integers(0, 2 ** 31 - 1)) for _ in range(n_traj)]
    trajs, cfg = [], None
    stream = torch.cuda.Stream()  # graph replays need a stream of their own
    with torch.cuda.stream(stream):
        for c0 in range(0, n_traj, chunk):
            doms = [scenes.fourier_periodic(nx, seed=s, jitter=jitter) for s in seeds[c0:c0 + chunk]]
            cfg = doms[0][0]
            sol = BatchSolver([c for c, _ in doms], [st["fluid"] for _, st in doms])
            frames = [[] for _ in doms]
            for f in range(n_frames):
                got = sol.download()
                xs, us, rs = (sol.split(got[q]) for q in ("positions", "velocities", "densities"))
                for d in range(len(doms)):
                    frames[d].append((_wrap(xs[d], cfg), us[d].clone(), rs[d].clone()))
                if f + 1 < n_frames:
                    if k % 2 == 0:
                        sol.graph_step(k)
                    else:
                        sol.step(k)
            sol.check()
            trajs.extend(frames)
    torch.cuda.current_stream().wait_stream(stream)
    return cfg, trajs


def fit_scales(config, trajs, k, max_pairs=512, seed=0):
    """Per-output spread of the targets over the frame pairs (a seeded sample of at most
    max_pairs of them for large data sets)."""
    pairs = [(t, i) for t in range(len(trajs)) for i in range(len(trajs[t]) - 1)]
    if len(pairs) > max_pairs:
        pick = np.random.default_rng(seed).choice(len(pairs), size=max_pairs, replace=False)
        pairs = [pairs[p] for p in sorted(pick)]
    t = torch.cat([targets(config, k, trajs[a][i], trajs[a][i + 1]) for a, i in pairs])
    return t.std(dim=0).clamp_min(1e-12)


def train(net, config, trajs, iters, k=4, lr=1e-3, seed=0, log_every=0):
    """Adam on the normalised targets of consecutive frame pairs; returns the loss history."""
    net.out_scale.copy_(fit_scales(config, trajs, k).to(net.out_scale.device))
    pairs = [(t, i) for t in range(len(trajs)) for i in range(len(trajs[t]) - 1)]
    graphs = {}
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, T_max=max(iters, 1), eta_min=lr * 0.05)
    stepper = LearnedStepper(config, net, k)
    rng = np.random.default_rng(seed)
    hist = []
    for it in range(iters):
        t, i = pairs[int(rng.integers(0, len(pairs)))]
        a, b = trajs[t][i], trajs[t][i + 1]
        # (the graphs of small data sets are kept; large ones rebuild each sample's)
        g = graphs.get((t, i))
        if g is None:
            g = Graph(a[0], config)
            if len(pairs) <= 1024:
                graphs[(t, i)] = g
        tgt = targets(config, k, a, b) / net.out_scale
        out = net(features(a[1], a[2], stepper.rho0), g)
        loss = torch.mean((out - tgt) ** 2)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        sched.step()
        hist.append(float(loss.detach()))
        if log_every and (it + 1) % log_every == 0:
            print(f"iter {it + 1}: loss {np.mean(hist[-log_every:]):.4e}")
    check_device_errors()
    return hist


def kinetic_energy(u, m):
    return 0.5 * m * float(torch.sum(u * u))


@torch.no_grad()
def judged_rollout(stepper: LearnedStepper, fluid, n_learned, segment=8, rho_tol=0.02, ke_tol=0.05):
    """Rollout of n_learned learned steps (k plain steps each) with the solver as judge and
    fallback. Each segment of ``segment`` learned steps is accepted when the density stays
    within rho_tol of rho0, the kinetic energy stays within ke_tol (relative) of the
    solver's prediction KE0 + t dKE/dt, dKE/dt = sum m u . a from one right-hand side at the
    segment start, and no particle exceeded the aggregation's 64-neighbor capacity (a
    clustering the learned steps brought about); otherwise the segment is re-run by the
    solver. Returns the final state and the counts of accepted and rejected segments."""
    cfg = stepper.config
    m = float(fluid["masses"][0])
    sol = Solver(cfg, fluid)
    got = sol.download()
    x, u, rho = _wrap(got["positions"], cfg), got["velocities"], got["densities"]
    accepted = rejected = 0
    done = 0
    while done < n_learned:
        nseg = min(segment, n_learned - done)
        sol.upload({"positions": x, "velocities": u, "densities": rho})
        r = sol.rhs()
        ke0 = kinetic_energy(u, m)
        dke = m * float(torch.sum(u * r["dudt"]))
        xs, us, rs = x, u, rho
        take_row_overflow()  # (a flag left by earlier steps is not this segment's)
        for _ in range(nseg):
            xs, us, rs = stepper.step(xs, us, rs)
        T = nseg * stepper.k * stepper.dt
        ke_pred = ke0 + T * dke
        ok = not take_row_overflow()
        ok = ok and bool(torch.isfinite(us).all())
        ok = ok and float(torch.max(torch.abs(rs / stepper.rho0 - 1.0))) <= rho_tol
        ok = ok and abs(kinetic_energy(us, m) - ke_pred) <= ke_tol * max(ke0, 1e-30)
        if ok:
            x, u, rho = xs, us, rs
            accepted += 1
        else:
            sol.upload({"positions": x, "velocities": u, "densities": rho})
            sol.step(nseg * stepper.k)
            sol.check()
            got = sol.download()
            x, u, rho = _wrap(got["positions"], cfg), got["velocities"], got["densities"]
            rejected += 1
        done += nseg
    return (x, u, rho), accepted, rejected
