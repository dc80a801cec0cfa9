"""Import harness for the reference diffSPH v2 torch code (fixture generation only).

This module is test infrastructure. It is used in the development container to
import the reference package from its source tree and run its own torch
functions on CPU, so that golden input/output vectors can be written under
``tests/golden/``. It never runs on the GPU machine and nothing in the product
imports it.

What it has to work around (all read from the reference sources):

* plotting / IO packages imported at module import time (matplotlib, seaborn,
  h5py, skimage, tomli, ipywidgets) are replaced by inert stub modules; the
  compute path never calls them;
* ``diffSPH.v2.compiler.compileSourceFiles`` JIT-builds ``cppSrc/mDBC.cpp`` at
  import (``src/diffSPH/v2/modules/mDBC.py:43-47``); the CPU-only build cannot
  load, and the Python mDBC path does not use it, so it is replaced by a stub;
* ``diffSPH.v2.modules`` must be imported before the simulation schemes to
  avoid a circular import (``incompressible.py:367``);
* ``torchCompactRadius`` (external pip package, unpinned, absent here) is
  provided by a small cell-list shim. The reference re-filters every
  candidate pair with its own code (``src/diffSPH/v2/modules/neighborhood.py:433-460``),
  so the final neighbor set only requires the shim to return a superset of all
  pairs within the exact radius; the shim returns all pairs with
  ``|x_i - x_j| <= verletScale * h_j`` (plus a small margin), in (i, j)
  lexicographic order.
"""
import importlib.machinery
import os
import sys
import types

import numpy as np
import torch

# The reference's ``src`` directory (the one holding the ``diffSPH`` package). The fixture
# generators take it from this variable, e.g.
#     DIFFSPH_REF_SRC=<reference checkout>/src python tests/golden/make_golden.py
REF_SRC = os.environ.get("DIFFSPH_REF_SRC")


class _Stub(types.ModuleType):
    """Module stub whose every attribute is another callable stub."""

    def __init__(self, name):
        super().__init__(name)
        # a spec, so that importlib.util.find_spec (used by torch's tracing rules) accepts it
        self.__spec__ = importlib.machinery.ModuleSpec(name, None)

    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        sub = _Stub(f"{self.__name__}.{name}")
        setattr(self, name, sub)
        return sub

    def __call__(self, *args, **kwargs):
        # decorators used as @stub or @stub(...) return the function unchanged
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return _Stub(self.__name__ + "()")

    def __iter__(self):
        return iter(())

    def __mro_entries__(self, bases):
        return (object,)


def _install_stubs():
    names = [
        "matplotlib", "matplotlib.pyplot", "matplotlib.colors", "matplotlib.patches",
        "matplotlib.ticker", "matplotlib.path", "matplotlib.cm", "matplotlib.animation",
        "mpl_toolkits", "mpl_toolkits.axes_grid1",
        "seaborn", "h5py", "skimage", "skimage.measure", "skimage.draw", "tomli",
        "ipywidgets", "IPython", "IPython.display", "numba", "pandas",
        "tqdm.autonotebook",
    ]
    for n in names:
        if n not in sys.modules:
            sys.modules[n] = _Stub(n)
    try:
        import tqdm as _tq
        sys.modules["tqdm.autonotebook"].tqdm = _tq.tqdm
        sys.modules["tqdm.autonotebook"].trange = _tq.trange
    except ImportError:
        pass


def _periodic_delta(d, ext, periodic):
    for a in range(d.shape[-1]):
        if bool(periodic[a]):
            da = d[..., a]
            d[..., a] = da - torch.round(da / ext[a]) * ext[a]
    return d


def _candidate_pairs_brute(q, r, rsup, ext, periodic, scale):
    out_i, out_j = [], []
    chunk = max(1, int(2e7 // max(1, r.shape[0])))
    for s in range(0, q.shape[0], chunk):
        d = _periodic_delta(q[s:s + chunk, None, :] - r[None, :, :], ext, periodic)
        dist = torch.linalg.norm(d, dim=-1)
        m = dist <= (scale * rsup.double()[None, :] * 1.001 + 1e-9)
        ii, jj = torch.nonzero(m, as_tuple=True)
        out_i.append(ii + s)
        out_j.append(jj)
    return torch.cat(out_i).to(torch.int64), torch.cat(out_j).to(torch.int64)


def _candidate_pairs(qpos, qsup, rpos, rsup, minD, maxD, periodic, scale):
    """Candidate superset: all (i, j) with periodic |x_i-x_j| <= scale*h_j (plus a margin),
    in (i, j) lexicographic order. Cells of the largest such radius bin the reference points
    and every query tests the 3^dim cells around its own; with fewer than 3 cells on an axis
    every pair is tested instead."""
    q = qpos.double()
    r = rpos.double()
    dim = q.shape[1]
    minD = torch.as_tensor(minD, dtype=torch.float64).reshape(-1).expand(dim)
    maxD = torch.as_tensor(maxD, dtype=torch.float64).reshape(-1).expand(dim)
    periodic = torch.as_tensor(periodic).reshape(-1).expand(dim)
    ext = maxD - minD
    if r.shape[0] == 0 or q.shape[0] == 0:
        e = torch.zeros(0, dtype=torch.int64)
        return e, e
    rad = float((scale * rsup.double() * 1.001 + 1e-9).max())
    lo = torch.minimum(q.min(0).values, r.min(0).values)
    hi = torch.maximum(q.max(0).values, r.max(0).values)
    ncell, origin = [], []
    for a in range(dim):
        if bool(periodic[a]):
            n = int(torch.floor(ext[a] / rad))
            origin.append(float(minD[a]))
        else:
            n = int(torch.floor((hi[a] - lo[a]) / rad)) + 1
            origin.append(float(lo[a]))
        ncell.append(n)
    if min(ncell) < 3 or r.shape[0] * q.shape[0] < 4e6:
        return _candidate_pairs_brute(q, r, rsup, ext, periodic, scale)
    csize = [float(ext[a]) / ncell[a] if bool(periodic[a]) else rad for a in range(dim)]

    def cells(p):
        c = []
        for a in range(dim):
            ca = torch.floor((p[:, a] - origin[a]) / csize[a]).to(torch.int64)
            c.append(torch.remainder(ca, ncell[a]) if bool(periodic[a]) else ca.clamp(0, ncell[a] - 1))
        return c

    def flat(c):
        f = torch.zeros_like(c[0])
        for a in range(dim):
            f = f * ncell[a] + c[a]
        return f

    rc = flat(cells(r))
    order = torch.argsort(rc, stable=True)
    total = 1
    for n in ncell:
        total *= n
    counts = torch.bincount(rc, minlength=total)
    start = torch.cumsum(counts, 0) - counts
    qc = cells(q)
    out_i, out_j = [], []
    offsets = torch.cartesian_prod(*[torch.tensor([-1, 0, 1])] * dim).reshape(-1, dim)
    qidx = torch.arange(q.shape[0])
    for off in offsets:
        c, ok = [], torch.ones(q.shape[0], dtype=torch.bool)
        for a in range(dim):
            ca = qc[a] + int(off[a])
            if bool(periodic[a]):
                ca = torch.remainder(ca, ncell[a])
            else:
                ok &= (ca >= 0) & (ca < ncell[a])
                ca = ca.clamp(0, ncell[a] - 1)
            c.append(ca)
        cid = flat(c)
        cnt = torch.where(ok, counts[cid], torch.zeros_like(cid))
        ii = torch.repeat_interleave(qidx, cnt)
        first = torch.repeat_interleave(start[cid], cnt)
        base = torch.repeat_interleave(torch.cumsum(cnt, 0) - cnt, cnt)
        jj = order[first + torch.arange(ii.shape[0]) - base]
        d = _periodic_delta(q[ii] - r[jj], ext, periodic)
        keep = torch.linalg.norm(d, dim=-1) <= (scale * rsup.double()[jj] * 1.001 + 1e-9)
        out_i.append(ii[keep])
        out_j.append(jj[keep])
    i = torch.cat(out_i)
    j = torch.cat(out_j)
    key = torch.argsort(i * r.shape[0] + j)
    return i[key].to(torch.int64), j[key].to(torch.int64)


def _install_compact_radius_shim():
    mod = types.ModuleType("torchCompactRadius")
    nb = types.ModuleType("torchCompactRadius.neighborhood")

    def buildDataStructure(positions, supports, hmax, minD, maxD, periodic, N, verbose=False):
        return {
            "referencePositions": positions.clone(),
            "referenceSupports": supports.clone(),
            "sortIndex": torch.arange(positions.shape[0], device=positions.device),
            "sortedPositions": positions.clone(),
            "sortedSupports": supports.clone(),
            "minD": minD, "maxD": maxD, "periodic": periodic,
        }

    def neighborSearchExisting(qpos, qsup, ds, mode, a, b):
        # the data structure holds supports already scaled by verletScale
        return _candidate_pairs(qpos, qsup, ds["sortedPositions"], ds["sortedSupports"],
                                ds["minD"], ds["maxD"], ds["periodic"], 1.0)

    def _unused(*args, **kwargs):
        raise RuntimeError("not used on the v2 live path")

    nb.buildDataStructure = buildDataStructure
    nb.neighborSearchExisting = neighborSearchExisting
    nb.neighborSearch = _unused
    nb.radiusSearch = _unused
    mod.neighborhood = nb
    mod.radiusSearch = _unused
    mod.neighborSearch = _unused
    sys.modules["torchCompactRadius"] = mod
    sys.modules["torchCompactRadius.neighborhood"] = nb


_LOADED = None


def load_reference():
    """Import the reference v2 package and return a namespace of its hot-path functions."""
    global _LOADED
    if _LOADED is not None:
        return _LOADED
    if not REF_SRC or not os.path.isdir(os.path.join(REF_SRC, "diffSPH")):
        raise RuntimeError("set DIFFSPH_REF_SRC to the reference's src directory (the one holding diffSPH/)")
    _install_stubs()
    _install_compact_radius_shim()
    if not torch.cuda.is_available():
        # the summation-density branch synchronises the CUDA device (deltaPlus.py:198); on a
        # host without one that call is a no-op here
        torch.cuda.synchronize = lambda *a, **k: None
    if REF_SRC not in sys.path:
        sys.path.insert(0, REF_SRC)
    import diffSPH.v2.compiler as comp

    comp.compileSourceFiles = lambda *a, **k: types.SimpleNamespace(
        mDBC=None, computeNeighborhood=None, viscosityKernel=None)
    import diffSPH.v2.modules  # noqa: F401  (must precede the schemes)
    import diffSPH.v2.simulationSchemes.deltaPlus as deltaPlus
    import diffSPH.v2.modules.neighborhood as neighborhood
    import diffSPH.v2.modules.integration as integration
    import diffSPH.v2.modules.shifting as shifting
    import diffSPH.v2.modules.timestep as timestep
    import diffSPH.v2.modules.mDBC as mDBC
    import diffSPH.v2.parameters as parameters
    import diffSPH.v2.sampling as sampling
    import diffSPH.v2.math as rmath
    import diffSPH.v2.sphOps as sphOps
    import diffSPH.kernels as kernels

    _LOADED = types.SimpleNamespace(
        deltaPlus=deltaPlus, neighborhood=neighborhood, integration=integration,
        shifting=shifting, timestep=timestep, mDBC=mDBC, parameters=parameters,
        sampling=sampling, math=rmath, sphOps=sphOps, kernels=kernels)
    return _LOADED
