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
  provided by a small brute-force shim. The reference re-filters every
  candidate pair with its own code (``src/diffSPH/v2/modules/neighborhood.py:433-460``),
  so the final neighbor set only requires the shim to return a superset of all
  pairs within the exact radius; the shim returns all pairs with
  ``|x_i - x_j| <= verletScale * h_j`` (plus a small margin), in (i, j)
  lexicographic order.
"""
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


def _candidate_pairs(qpos, qsup, rpos, rsup, minD, maxD, periodic, scale):
    """Brute-force candidate superset: all (i, j) with periodic |x_i-x_j| <= scale*h_j."""
    q = qpos.double()
    r = rpos.double()
    out_i, out_j = [], []
    dim = q.shape[1]
    minD = torch.as_tensor(minD, dtype=torch.float64).reshape(-1).expand(dim)
    maxD = torch.as_tensor(maxD, dtype=torch.float64).reshape(-1).expand(dim)
    periodic = torch.as_tensor(periodic).reshape(-1).expand(dim)
    ext = maxD - minD
    chunk = max(1, int(2e7 // max(1, r.shape[0])))
    for s in range(0, q.shape[0], chunk):
        d = q[s:s + chunk, None, :] - r[None, :, :]
        for a in range(d.shape[-1]):
            if bool(periodic[a]):
                da = d[..., a]
                d[..., a] = da - torch.round(da / ext[a]) * ext[a]
        dist = torch.linalg.norm(d, dim=-1)
        m = dist <= (scale * rsup.double()[None, :] * 1.001 + 1e-9)
        ii, jj = torch.nonzero(m, as_tuple=True)
        out_i.append(ii + s)
        out_j.append(jj)
    i = torch.cat(out_i).to(torch.int64)
    j = torch.cat(out_j).to(torch.int64)
    return i, j


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
