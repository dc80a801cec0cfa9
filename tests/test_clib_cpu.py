"""The C-ABI library loads and exports every entry point include/sph103.h declares.

Runs without a GPU: only host-side queries (workspace sizes, parameter validation) are
called here; compute calls are covered by the gpu-marked tests.
"""
import copy
import ctypes
import os
import re

import pytest

from diffsph_gb300 import _lib, build, scenes
from diffsph_gb300.solver import default_capacity, domain_struct, params_from_config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    try:
        build.build()
    except RuntimeError as e:  # no nvcc on this machine
        pytest.skip(str(e))
    return _lib.load()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "sph103.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sph_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(_lib.EXPORTS) == names


def test_solver_workspace_query(lib):
    cfg, st = scenes.taylor_green(64)
    p = params_from_config(cfg, float(st["fluid"]["masses"][0]))
    nbytes = ctypes.c_size_t()
    assert lib.sph_solver_workspace_bytes(ctypes.byref(p), 4096, 0, ctypes.byref(nbytes)) == 0
    # state: raw positions (2x8 B), four float4 position/density and four velocity buffers
    # (8x16 B), ids, sort keys (4x4 B) plus the cell tables
    assert nbytes.value > 4096 * (16 + 128 + 16)
    assert nbytes.value < 4096 * 1024


def test_solver_rejects_bad_parameters(lib):
    cfg, st = scenes.taylor_green(16)
    p = params_from_config(cfg, float(st["fluid"]["masses"][0]))
    nbytes = ctypes.c_size_t()
    bad = _lib.Params.from_buffer_copy(p)
    bad.skin = 0.9
    assert lib.sph_solver_workspace_bytes(ctypes.byref(bad), 256, 0, ctypes.byref(nbytes)) == 1
    bad = _lib.Params.from_buffer_copy(p)
    bad.support = -1
    assert lib.sph_solver_workspace_bytes(ctypes.byref(bad), 256, 0, ctypes.byref(nbytes)) == 1
    assert lib.sph_solver_workspace_bytes(ctypes.byref(p), 0, 0, ctypes.byref(nbytes)) == 1
    # creating over a too-small workspace fails cleanly, before touching the device
    h = ctypes.c_void_p()
    assert lib.sph_solver_create(ctypes.byref(p), 256, 0, ctypes.c_void_p(256), 16, ctypes.byref(h)) == 2


def test_neighbor_workspace_query(lib):
    cfg, _ = scenes.dam_break(dx=1.0 / 64)
    d = domain_struct(cfg)
    nbytes = ctypes.c_size_t()
    assert lib.sph_neighbor_workspace_bytes(1000, 2000, ctypes.byref(d), cfg["particle"]["support"],
                                            ctypes.byref(nbytes)) == 0
    assert nbytes.value > 2000 * 8
    assert lib.sph_neighbor_workspace_bytes(10, 10, ctypes.byref(d), -1.0, ctypes.byref(nbytes)) == 1


def test_kernel_classes(lib):
    k = lib.sph_solver_kernel_classes()
    names = [lib.sph_solver_kernel_name(c).decode() for c in range(k)]
    assert "pass_b_rates" in names and "cell_sort" in names
    assert lib.sph_solver_kernel_name(k) is None


def test_params_from_reference_config_keys():
    cfg, st = scenes.dam_break(dx=1.0 / 64)
    p = params_from_config(cfg, float(st["fluid"]["masses"][0]))
    assert p.visc_scheme == 1 and p.bvisc_scheme == 1 and p.gravity_on == 1
    assert abs(p.gravity[1] + 9.81) < 1e-12
    assert p.capacity == default_capacity(1.15, p.support, p.dx)
    cfg["diffusion"]["velocityScheme"] = "Monaghan1992"
    with pytest.raises(ValueError):
        params_from_config(cfg, 1.0)


def test_params_accept_the_implicit_shifting_scheme():
    cfg, st = scenes.fourier_periodic(16, seed=1)
    cfg["shifting"]["scheme"] = "IPS"
    params_from_config(cfg, float(st["fluid"]["masses"][0]))
    cfg["shifting"]["initialization"] = "deltaPlus"
    with pytest.raises(ValueError):
        params_from_config(cfg, 1.0)
    cfg["shifting"]["initialization"] = "zero"
    cfg["shifting"]["freeSurface"] = True
    params_from_config(cfg, 1.0)
    cfg["shifting"]["surfaceDetection"] = "Maronne"
    with pytest.raises(ValueError):
        params_from_config(cfg, 1.0)


def test_free_surface_params_struct_layout():
    from diffsph_gb300 import _lib
    assert ctypes.sizeof(_lib.FreeSurfaceParams) == 24
    assert _lib.FreeSurfaceParams.surface_scaling.offset == 16


def test_ips_params_struct_layout():
    from diffsph_gb300 import _lib
    assert ctypes.sizeof(_lib.IpsParams) == 24
    assert _lib.IpsParams.solver_threshold.offset == 16


def test_params_reject_open_boundary_regions():
    cfg, st = scenes.fourier_periodic(16, seed=1)
    cfg["regions"] = [{"type": "outlet", "sdf": lambda p: p[:, 0]}]
    with pytest.raises(ValueError):
        params_from_config(cfg, 1.0)


def test_handle_entry_points_reject_null_handles(lib):
    """Host-side argument checks of the handle-based entry points, before any device work."""
    u32 = ctypes.c_uint32()
    assert lib.sph_solver_set_verlet_reuse(None, 1) == 1
    assert lib.sph_solver_sort_count(None, ctypes.byref(u32), None) == 1
    assert lib.sph_solver_flags(None, ctypes.byref(u32), None) == 1
    assert lib.sph_solver_graph_step(None, 2, None) == 1
    assert lib.sph_solver_step(None, 1, None) == 1
    assert lib.sph_solver_launches_per_step(None) == -1
    assert lib.sph_solver_set_verlet_scale(None, 1.5) == 1


def test_verlet_reuse_follows_the_reference_verlet_scale():
    from diffsph_gb300.solver import wants_verlet_reuse
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    p = params_from_config(cfg, float(st["fluid"]["masses"][0]))
    assert wants_verlet_reuse(cfg, p)                  # verletScale 1.5, walls
    cfg["neighborhood"]["verletScale"] = 1.0
    assert not wants_verlet_reuse(cfg, p)              # the reference rebuilds every step
    del cfg["neighborhood"]
    assert wants_verlet_reuse(cfg, p)                  # the reference's default, 1.5
    cfg, st = scenes.taylor_green(16)
    p = params_from_config(cfg, float(st["fluid"]["masses"][0]))
    assert wants_verlet_reuse(cfg, p)                  # periodic domains reuse too
    cfg["neighborhood"]["verletScale"] = 1.0
    assert not wants_verlet_reuse(cfg, p)


def test_params_reject_what_the_kernels_do_not_implement():
    """The fused solver raises instead of silently stepping another scheme: kernel.name
    (parameters.py:37) other than Wendland2, simulation.densityScheme (parameters.py:24) other
    than continuity / summation, and the summation density with the rational density update."""
    cfg, st = scenes.dam_break(dx=1.0 / 64)
    m = float(st["fluid"]["masses"][0])
    assert params_from_config(cfg, m).density_scheme == 0
    c = copy.deepcopy(cfg)
    c["kernel"]["name"] = "CubicSpline"
    with pytest.raises(ValueError):
        params_from_config(c, m)
    c = copy.deepcopy(cfg)
    c["simulation"]["densityScheme"] = "shepard"
    with pytest.raises(ValueError):
        params_from_config(c, m)
    c = copy.deepcopy(cfg)
    c["simulation"]["densityScheme"] = "summation"
    assert params_from_config(c, m).density_scheme == 1
    c.setdefault("integration", {})["densityUpdate"] = "rational"
    with pytest.raises(ValueError):
        params_from_config(c, m)


def test_solver_rejects_summation_with_rational_update(lib):
    """The C ABI's own check (sph_solver_workspace_bytes validates the parameters)."""
    cfg, st = scenes.dam_break(dx=1.0 / 64)
    p = params_from_config(cfg, float(st["fluid"]["masses"][0]))
    nbytes = ctypes.c_size_t()
    nF, nB = st["fluid"]["positions"].shape[0], st["boundary"]["positions"].shape[0]
    assert lib.sph_solver_workspace_bytes(ctypes.byref(p), nF, nB, ctypes.byref(nbytes)) == 0
    p.density_scheme = 1
    assert lib.sph_solver_workspace_bytes(ctypes.byref(p), nF, nB, ctypes.byref(nbytes)) == 0
    p.density_update = 1
    assert lib.sph_solver_workspace_bytes(ctypes.byref(p), nF, nB, ctypes.byref(nbytes)) == 1
    p.density_update, p.density_scheme = 0, 2
    assert lib.sph_solver_workspace_bytes(ctypes.byref(p), nF, nB, ctypes.byref(nbytes)) == 1


def test_verlet_sort_limit_is_the_stricter_of_the_reference_rule_and_the_skin_limit():
    """The reference rebuilds once 2 max|dx| > (verletScale - 1) h (neighborhood.py:509-513);
    the solver keeps its skin list complete only up to 0.049 h, so it sorts at the smaller of
    (verletScale - 1) h / 2 and 0.7 x 0.049 h."""
    from diffsph_gb300.solver import verlet_sort_limit
    h = 4.0 / 1024
    skin_lim = 0.5 * 0.1 * h * 0.98
    assert verlet_sort_limit(1.5, h, skin_lim) == 0.7 * skin_lim        # default scale: the skin limit
    assert abs(verlet_sort_limit(1.02, h, skin_lim) - 0.02 * h / 2) < 1e-15  # a tight scale: the reference's rule
    assert verlet_sort_limit(1.0686, h, skin_lim) < 0.7 * skin_lim + 1e-12
