"""Open-boundary regions: drop-ins for src/diffSPH/v2/modules/inletOutlet.py and for
``LiuLiuConsistent`` (src/diffSPH/v2/sphOps.py:313-341).

The reference describes a region by a signed distance function (a Python callable, negative
inside) and a type: 'mirror' outlets get ghost particles mirrored across the region's
boundary, whose consistent interpolation of the fluid replaces the densities and velocities
of the fluid particles inside (deltaPlus.py:188-235); 'outlet' regions remove particles,
'forcing' regions impose a velocity and the rest density, and emitters insert particles
where no fluid particle is closer than dx (the runner calls these between steps).

Here the neighbor searches run on the GPU (``diffsph_gb300.neighborhood.neighborSearch``)
and the consistent interpolation is the sm_103a kernel ``sph_liuliu_consistent``; the
region functions themselves are the callers' Python callables, evaluated on the tensors.
The fused ``Solver`` has a fixed particle count and no region support: it rejects configs
with regions, and these functions serve the reference's own step with the drop-in
neighbor search.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .neighborhood import neighborSearch


def _dev(t, dtype=torch.float32):
    return torch.as_tensor(t).to(device="cuda", dtype=dtype).contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def LiuLiuConsistent(ghostState, fluidState, q):
    """First-order consistent interpolation of the fluid quantity q at the ghost particles
    (sphOps.py:313-341) over ghostState['neighborhood'] (reference format). Returns
    (solution [n, 3] = value and gradient, M [n, 3, 3], b [n, 3]) like the reference."""
    nb = ghostState["neighborhood"]
    n = int(torch.as_tensor(ghostState["positions"]).shape[0])
    dev = torch.as_tensor(q).device
    sol = torch.empty(n, 3, device="cuda")
    M = torch.empty(n, 3, 3, device="cuda")
    b = torch.empty(n, 3, device="cuda")
    keep = [_dev(nb["neighborOffsets"], torch.int32), _dev(nb["numNeighbors"], torch.int32),
            _dev(nb["indices"][1], torch.int64), _dev(nb["distances"]), _dev(nb["vectors"]), _dev(nb["supports"]),
            _dev(nb["kernels"]), _dev(nb["gradients"]), _dev(fluidState["masses"]), _dev(fluidState["densities"]),
            _dev(q)]
    _lib.check("sph_liuliu_consistent", _lib.load().sph_liuliu_consistent(
        n, *[_ptr(t) for t in keep], _ptr(sol), _ptr(M), _ptr(b), _stream()))
    return sol.to(dev), M.to(dev), b.to(dev)


def _periodic_image(x, config):
    """Positions wrapped into the domain on its periodic axes (inletOutlet.py:6-12)."""
    d = config["domain"]
    per = d.get("periodicity", d.get("periodic", [False, False]))
    if isinstance(per, bool):
        per = [per, per]
    cols = []
    for a in range(x.shape[1]):
        if bool(per[a]):
            lo, hi = float(d["minExtent"][a]), float(d["maxExtent"][a])
            cols.append(torch.remainder(x[:, a] - lo, hi - lo) + lo)
        else:
            cols.append(x[:, a])
    return torch.stack(cols, dim=1)


def _sdf_gradient(sdf, p, h):
    """The reference's central-difference gradient of a region's distance function
    (continuousGradient with centralDifferenceStencil(1, 2), finiteDifference.py:3-6,214-232):
    the stencil weights (-1/2, 0, 1/2) also serve as the offsets (in units of h), and the
    function is evaluated on the CPU."""
    w = torch.tensor([-0.5, 0.0, 0.5])
    out = []
    for a in range(p.shape[1]):
        off = torch.zeros(3, p.shape[1])
        off[:, a] = w
        probe = (p[:, None, :].cpu() + off[None] * h).reshape(-1, p.shape[1])
        f = torch.as_tensor(sdf(probe)).reshape(p.shape[0], 3)
        out.append(torch.sum(w * f, dim=-1) / h)
    return torch.stack(out, dim=-1).to(p.device)


def buildOutletGhostParticles(regions, perennialState, config):
    """Ghosts of the fluid particles inside 'mirror' regions (inletOutlet.py:67-147):
    x_ghost = x - 2 d(x) n(x) with n the normalised distance gradient, rest density and the
    uniform support and mass, with their neighborhood over the fluid. None without any."""
    fl = perennialState["fluid"]
    x = torch.as_tensor(fl["positions"])
    parts = []
    for region in regions:
        if region["type"] != "mirror":
            continue
        inside = torch.nonzero(torch.as_tensor(region["sdf"](x)) < 0).flatten()
        if inside.numel() == 0:
            continue
        p = x[inside]
        dist = torch.as_tensor(region["sdf"](_periodic_image(p, config)))
        g = _sdf_gradient(region["sdf"], p, float(config["particle"]["support"]) * 0.01)
        g = g / (torch.linalg.norm(g, dim=1, keepdim=True) + 1e-7)
        parts.append((inside, p - 2 * dist[:, None] * g, dist, g))
    if not parts:
        return None
    pos = torch.cat([q[1] for q in parts])
    n = pos.shape[0]
    h = float(config["particle"]["support"])
    rho0 = float(config["fluid"]["rho0"])
    ghost = {
        "positions": pos, "velocities": torch.zeros_like(pos),
        "supports": torch.full((n,), h, device=pos.device),
        "densities": torch.full((n,), rho0, device=pos.device),
        "masses": torch.full((n,), float(config["particle"]["volume"]) * rho0, device=pos.device),
        "index": torch.cat([torch.arange(q[0].numel(), device=pos.device) for q in parts]),
        "fluidIndex": torch.cat([q[0] for q in parts]), "numParticles": n,
        "sdf_dist": torch.cat([q[2] for q in parts]), "sdf_grad": torch.cat([q[3] for q in parts]),
    }
    search = {"domain": config["domain"], "simulation": {"supportScheme": "scatter"},
              "neighborhood": {"algorithm": "compact", "scheme": "compact", "verletScale": 1.0},
              "kernel": config["kernel"]}
    _, ghost["neighborhood"] = neighborSearch(ghost, fl, search, computeKernels=True)
    ghost["numNeighbors"] = ghost["neighborhood"]["numNeighbors"]
    return ghost


def processOutlet(region, config, perennialState):
    """Removes the fluid particles inside an outlet region (inletOutlet.py:14-33)."""
    fl = perennialState["fluid"]
    outside = torch.as_tensor(region["sdf"](fl["positions"])) >= 0
    if bool(outside.all()):
        return
    keep = torch.nonzero(outside).flatten()
    for k, v in list(fl.items()):
        if isinstance(v, torch.Tensor):
            fl[k] = v[keep]
    fl["numParticles"] = fl["positions"].shape[0]


def processForcing(region, config, perennialState):
    """Imposes the region's velocity and the rest density inside it (inletOutlet.py:35-48)."""
    fl = perennialState["fluid"]
    inside = torch.nonzero(torch.as_tensor(region["sdf"](fl["positions"])) < 0).flatten()
    if inside.numel() == 0:
        return
    fl["velocities"][inside, 0] = region["velocity"][0]
    fl["velocities"][inside, 1] = region["velocity"][1]
    fl["densities"][inside] = config["fluid"]["rho0"]


def _append(state, new):
    """Concatenates new particles to a state; fields the new particles lack are zero
    (mergeStates, inletOutlet.py:51-66)."""
    m = int(new["numParticles"])
    for k, v in list(state.items()):
        if not isinstance(v, torch.Tensor):
            continue
        add = new[k] if k in new else v.new_zeros((m, *v.shape[1:]))
        state[k] = torch.cat([v, add.to(v.device, v.dtype)], dim=0)
    state["numParticles"] = state["positions"].shape[0]
    return state


def processInlet(perennialState, config, emitter):
    """Inserts the emitter particles that have no fluid particle closer than dx
    (inletOutlet.py:150-189): their smallest fluid distance (in units of h, 1 when they have
    no neighbor) comes from the GPU neighbor search."""
    fl = perennialState["fluid"]
    em = emitter["particles"]
    _, nb = neighborSearch(em, fl, config, computeKernels=False)
    n = int(torch.as_tensor(em["positions"]).shape[0])
    i = nb["indices"][0]
    closest = torch.ones(n, device=nb["distances"].device, dtype=nb["distances"].dtype)
    closest = closest.index_reduce_(0, i, nb["distances"], "amin", include_self=False)
    free = closest >= float(config["particle"]["dx"]) / float(config["particle"]["support"])
    dev = torch.as_tensor(fl["positions"]).device
    x = torch.as_tensor(em["positions"]).to(dev)[free.to(dev)]
    m = x.shape[0]
    dt = torch.as_tensor(fl["positions"]).dtype
    vol, rho0, h = float(config["particle"]["volume"]), float(config["fluid"]["rho0"]), float(config["particle"]["support"])
    ones = torch.ones(m, dtype=dt, device=dev)
    new = {"numParticles": m, "positions": x, "areas": ones * vol, "masses": ones * vol * rho0,
           "densities": ones * rho0, "supports": ones * h, "pressures": ones * 0, "divergence": ones * 0,
           "velocities": torch.zeros_like(x), "accelerations": torch.zeros_like(x),
           "index": torch.arange(m, dtype=torch.int32, device=dev) + int(perennialState["uidCounter"])}
    new["velocities"][:, 0] = emitter["velocity"][0]
    new["velocities"][:, 1] = emitter["velocity"][1]
    if "initialPositions" in fl:
        new["initialPositions"] = x.clone()
    perennialState["uidCounter"] += m
    perennialState["fluid"] = _append(fl, new)
