"""sph_neighbor_count_static: the neighbor count on a fixed file-scope scratch array.

Collected last so that it also runs after every other test has used the library on the
device. The GPU tests call both entry points through the C ABI on the same inputs and
require identical counts and offsets (integer outputs: bit-exact), on calls in a row that
reuse the one static array with different problem sizes.
"""
import ctypes

import numpy as np
import pytest

from diffsph_gb300 import _lib, build, scenes
from diffsph_gb300.solver import domain_struct

LIMIT = 24 << 20  # SPH_NEIGHBOR_STATIC_SCRATCH_BYTES
STATIC_LIMIT = 7  # SPH_ERR_STATIC_LIMIT


@pytest.fixture(scope="module")
def lib():
    try:
        build.build()
    except RuntimeError as e:  # no nvcc on this machine
        pytest.skip(str(e))
    return _lib.load()


def _workspace_bytes(lib, n, cfg, h):
    dom = domain_struct(cfg)
    nb = ctypes.c_size_t()
    _lib.check("sph_neighbor_workspace_bytes",
               lib.sph_neighbor_workspace_bytes(n, n, ctypes.byref(dom), h, ctypes.byref(nb)))
    return nb.value


def test_limit_is_checked_before_any_device_work(lib):
    # 1024^2 particles need more than the static array: rejected on the host (null device
    # pointers are never touched), with its own status
    cfg, _ = scenes.taylor_green(1024)
    h = cfg["particle"]["support"]
    n = 1024 * 1024
    assert _workspace_bytes(lib, n, cfg, h) > LIMIT
    dom = domain_struct(cfg)
    code = lib.sph_neighbor_count_static(None, n, None, None, n, ctypes.byref(dom), h, None, None, None)
    assert code == STATIC_LIMIT
    with pytest.raises(_lib.SphError, match="static scratch"):
        _lib.check("sph_neighbor_count_static", code)


def test_stated_capacity(lib):
    # the header states about 400k particles in a square periodic domain
    for nx, fits in ((512, True), (632, True), (720, False)):
        cfg, _ = scenes.taylor_green(nx)
        assert (_workspace_bytes(lib, nx * nx, cfg, cfg["particle"]["support"]) <= LIMIT) == fits, nx


def _cases():
    cfg1, st1 = scenes.fourier_periodic(96, seed=3, jitter=0.2)
    cfg2, st2 = scenes.dam_break(1.0 / 64)
    cfg3, st3 = scenes.fourier_periodic(48, seed=5, jitter=0.4)
    x2 = np.concatenate([st2["fluid"]["positions"], st2["boundary"]["positions"]])
    h2 = np.concatenate([st2["fluid"]["supports"], st2["boundary"]["supports"]])
    return [
        ("fourier96_periodic", cfg1, st1["fluid"]["positions"], st1["fluid"]["positions"], st1["fluid"]["supports"]),
        ("dambreak64_fluid_vs_all", cfg2, st2["fluid"]["positions"], x2, h2),
        ("fourier48_periodic", cfg3, st3["fluid"]["positions"], st3["fluid"]["positions"], st3["fluid"]["supports"]),
    ]


@pytest.mark.gpu
def test_static_count_matches_workspace_count(lib):
    import torch

    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for rep in range(2):
        for name, cfg, xq_np, xr_np, hr_np in _cases():
            xq = torch.as_tensor(xq_np, dtype=torch.float32, device="cuda").contiguous()
            xr = torch.as_tensor(xr_np, dtype=torch.float32, device="cuda").contiguous()
            hr = torch.as_tensor(hr_np, dtype=torch.float32, device="cuda").contiguous()
            nq, nr = xq.shape[0], xr.shape[0]
            hmax = float(hr.max())
            dom = domain_struct(cfg)
            need = _workspace_bytes(lib, nq, cfg, hmax) if nq == nr else None
            nbytes = ctypes.c_size_t()
            _lib.check("sph_neighbor_workspace_bytes",
                       lib.sph_neighbor_workspace_bytes(nq, nr, ctypes.byref(dom), hmax, ctypes.byref(nbytes)))
            assert nbytes.value <= LIMIT and (need is None or need == nbytes.value)
            ws = torch.empty(nbytes.value + 256, dtype=torch.uint8, device="cuda")
            wsp = (ws.data_ptr() + 255) & ~255
            c_ref = torch.full((nq,), -1, dtype=torch.int32, device="cuda")
            o_ref = torch.full((nq + 1,), -1, dtype=torch.int64, device="cuda")
            c_st = torch.full((nq,), -2, dtype=torch.int32, device="cuda")
            o_st = torch.full((nq + 1,), -2, dtype=torch.int64, device="cuda")
            _lib.check("sph_neighbor_count", lib.sph_neighbor_count(
                xq.data_ptr(), nq, xr.data_ptr(), hr.data_ptr(), nr, ctypes.byref(dom), hmax,
                ctypes.c_void_p(wsp), nbytes.value, c_ref.data_ptr(), o_ref.data_ptr(), stream))
            _lib.check("sph_neighbor_count_static", lib.sph_neighbor_count_static(
                xq.data_ptr(), nq, xr.data_ptr(), hr.data_ptr(), nr, ctypes.byref(dom), hmax,
                c_st.data_ptr(), o_st.data_ptr(), stream))
            torch.cuda.synchronize()
            assert int(c_ref.min()) > 0, name
            assert torch.equal(c_st, c_ref), (rep, name)
            assert torch.equal(o_st, o_ref), (rep, name)
            assert int(o_st[-1]) == int(c_ref.sum()), (rep, name)
