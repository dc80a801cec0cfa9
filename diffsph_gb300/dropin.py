"""Installs the sm_103a drop-ins into an imported diffSPH v2 package.

This does the swap of the reference's call sites that a maintainer would otherwise write
by hand. Several modules of the reference import these functions by name, so each copy is
replaced where it lives:
- ``neighborSearch``: neighborhood.py:491, imported by name in deltaPlus.py:27, mDBC.py:4,
  inletOutlet.py:4 and shifting.py:172;
- ``integrate`` and ``solveShifting``: imported by name in runner.py:5,7;
- ``LiuLiuConsistent``: imported by name in deltaPlus.py:104, inletOutlet.py:148 and
  boundaryViscosity.py:259;
- ``buildOutletGhostParticles``: imported by name in deltaPlus.py:128;
- the module functions of the right-hand side, each imported by name in deltaPlus.py:13-34
  and 111-129.

``install('fused')`` routes the step to the fused solver: integrate, solveShifting,
simulationStep, the neighbor search and the pressure switch. ``install('regions')`` is for
configs with open-boundary regions, which keep the reference's own simulationStep (the
fused solver has a fixed particle count). It installs the neighbor search, the pressure
switch, the consistent interpolation and the region functions. ``install('operators')``
keeps the reference's own simulationStep and integrate and replaces the pair operators it
calls: the neighbor search, computeDensity, computeCovarianceMatrices, the density
gradients, computeDensityDeltaTerm, computeMomentumEquation, computePressureAccel (and the
switch), computeViscosity(_Boundary), computeGravity and mDBCDensity (diffsph_gb300.ops).
The generic sphOperation / sphOperationStates of diffsph_gb300.ops are left for direct
calls: the reference's own modules use them in combinations (3D fields, the naive
laplacian) the GPU operator does not take. Every mode returns the replaced functions;
``uninstall`` puts them back. The reference package must already be importable; its
functions are not called here.
"""
from __future__ import annotations

import importlib

from . import neighborhood, ops, regions, scheme

_SEARCH = [
    ("diffSPH.v2.modules.neighborhood", "neighborSearch", neighborhood.neighborSearch),
    ("diffSPH.v2.simulationSchemes.deltaPlus", "neighborSearch", neighborhood.neighborSearch),
    ("diffSPH.v2.modules.mDBC", "neighborSearch", neighborhood.neighborSearch),
    ("diffSPH.v2.modules.inletOutlet", "neighborSearch", neighborhood.neighborSearch),
    ("diffSPH.v2.modules.shifting", "neighborSearch", neighborhood.neighborSearch),
    ("diffSPH.v2.modules.pressureForce", "computePressureAccelSwitch", scheme.computePressureAccelSwitch),
    ("diffSPH.v2.simulationSchemes.deltaPlus", "computePressureAccelSwitch", scheme.computePressureAccelSwitch),
]

_FUSED = [
    ("diffSPH.v2.modules.integration", "integrate", scheme.integrate),
    ("diffSPH.v2.runner", "integrate", scheme.integrate),
    ("diffSPH.v2.modules.shifting", "solveShifting", scheme.solveShifting),
    ("diffSPH.v2.runner", "solveShifting", scheme.solveShifting),
    ("diffSPH.v2.simulationSchemes.deltaPlus", "simulationStep", scheme.simulationStep),
]

_REGIONS = [
    ("diffSPH.v2.sphOps", "LiuLiuConsistent", regions.LiuLiuConsistent),
    ("diffSPH.v2.simulationSchemes.deltaPlus", "LiuLiuConsistent", regions.LiuLiuConsistent),
    ("diffSPH.v2.modules.inletOutlet", "LiuLiuConsistent", regions.LiuLiuConsistent),
    ("diffSPH.v2.modules.boundaryViscosity", "LiuLiuConsistent", regions.LiuLiuConsistent),
    ("diffSPH.v2.modules.mDBC", "LiuLiuConsistent", regions.LiuLiuConsistent),
    ("diffSPH.v2.modules.inletOutlet", "buildOutletGhostParticles", regions.buildOutletGhostParticles),
    ("diffSPH.v2.simulationSchemes.deltaPlus", "buildOutletGhostParticles", regions.buildOutletGhostParticles),
    ("diffSPH.v2.modules.inletOutlet", "processOutlet", regions.processOutlet),
    ("diffSPH.v2.modules.inletOutlet", "processForcing", regions.processForcing),
    ("diffSPH.v2.modules.inletOutlet", "processInlet", regions.processInlet),
]


_DP = "diffSPH.v2.simulationSchemes.deltaPlus"
_OPERATORS = [
    (mod, name, fn)
    for home, name, fn in [
        ("diffSPH.v2.modules.density", "computeDensity", ops.computeDensity),
        ("diffSPH.v2.modules.normalizationMatrices", "computeCovarianceMatrices", ops.computeCovarianceMatrices),
        ("diffSPH.v2.modules.densityDiffusion", "renormalizedDensityGradient", ops.renormalizedDensityGradient),
        ("diffSPH.v2.modules.densityDiffusion", "densityGradient", ops.densityGradient),
        ("diffSPH.v2.modules.densityDiffusion", "computeDensityDeltaTerm", ops.computeDensityDeltaTerm),
        ("diffSPH.v2.modules.momentumEquation", "computeMomentumEquation", ops.computeMomentumEquation),
        ("diffSPH.v2.modules.pressureForce", "computePressureAccel", ops.computePressureAccel),
        ("diffSPH.v2.modules.viscosity", "computeViscosity", ops.computeViscosity),
        ("diffSPH.v2.modules.boundaryViscosity", "computeViscosity_Boundary", ops.computeViscosity_Boundary),
        ("diffSPH.v2.modules.gravity", "computeGravity", ops.computeGravity),
        ("diffSPH.v2.modules.mDBC", "mDBCDensity", ops.mDBCDensity),
    ]
    for mod in (home, _DP)
]


# Reference modules that import some of these functions by name but are not on the delta-SPH
# step this package replaces; their copies are left alone on purpose.
LEFT_ALONE = {
    "diffSPH.v2.plotting": "plotting of a state, not a simulation step",
    "diffSPH.v2.sampling": "scene construction (initial particle sampling), run once before any step",
    "diffSPH.v2.simulationSchemes.dfsph": "the divergence-free (DFSPH) scheme, not implemented by the kernels",
    "diffSPH.v2.modules.incompressible": "the incompressible (DFSPH) pressure solve, not implemented by the kernels",
}


def targets(mode: str = "fused"):
    """(module name, attribute, replacement) for the mode ('fused', 'regions' or 'operators')."""
    if mode == "fused":
        return _SEARCH + _FUSED
    if mode == "regions":
        return _SEARCH + _REGIONS
    if mode == "operators":
        return _SEARCH + _OPERATORS
    raise ValueError(f"unknown drop-in mode {mode!r} (use 'fused', 'regions' or 'operators')")


def install(mode: str = "fused"):
    """Replaces the reference's functions with the drop-ins. Returns [(module, attribute,
    original)] for ``uninstall``. Raises if a reference module or attribute is missing,
    before anything is replaced."""
    plan = []
    for mod_name, attr, new in targets(mode):
        mod = importlib.import_module(mod_name)
        if not hasattr(mod, attr):
            raise AttributeError(f"{mod_name} has no attribute {attr}: not the diffSPH v2 layout expected")
        plan.append((mod, attr, getattr(mod, attr), new))
    for mod, attr, _, new in plan:
        setattr(mod, attr, new)
    return [(mod, attr, old) for mod, attr, old, _ in plan]


def uninstall(replaced):
    """Puts back what ``install`` replaced."""
    for mod, attr, old in reversed(replaced):
        setattr(mod, attr, old)
