"""ctypes binding of libsph103.so (declarations in include/sph103.h).

The library is the only compute path of this package: if it is missing or cannot load,
every entry point raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsph103.so")

STATUS = {
    0: "ok", 1: "invalid argument", 2: "workspace too small", 3: "neighbor list capacity exceeded",
    4: "CUDA launch or copy failed", 5: "particles moved farther than the neighbor-list skin allows",
    6: "non-finite value in the state",
    7: "problem exceeds the fixed static scratch of sph_neighbor_count_static",
}
FLAG_CAPACITY, FLAG_VERLET, FLAG_NONFINITE = 1, 2, 4


class SphError(RuntimeError):
    def __init__(self, fn, code):
        super().__init__(f"{fn}: {STATUS.get(code, 'unknown status')} (status {code})")
        self.code = code


class Domain(ctypes.Structure):
    _fields_ = [("min", ctypes.c_double * 2), ("max", ctypes.c_double * 2), ("periodic", ctypes.c_int32 * 2)]


class Params(ctypes.Structure):
    _fields_ = [
        ("domain", Domain),
        ("support", ctypes.c_double), ("dx", ctypes.c_double), ("mass", ctypes.c_double),
        ("rho0", ctypes.c_double), ("cs", ctypes.c_double), ("gamma", ctypes.c_double),
        ("kernel_scale", ctypes.c_double), ("delta", ctypes.c_double),
        ("visc_scheme", ctypes.c_int32), ("nu", ctypes.c_double), ("alpha", ctypes.c_double), ("eps", ctypes.c_double),
        ("bvisc_scheme", ctypes.c_int32), ("b_nu", ctypes.c_double), ("b_alpha", ctypes.c_double),
        ("b_eps", ctypes.c_double),
        ("gravity_on", ctypes.c_int32), ("gravity", ctypes.c_double * 2),
        ("dt", ctypes.c_double),
        ("shift_on", ctypes.c_int32), ("shift_R", ctypes.c_double), ("shift_n", ctypes.c_double),
        ("shift_CFL", ctypes.c_double), ("shift_threshold", ctypes.c_double),
        ("compute_mach", ctypes.c_int32), ("density_update", ctypes.c_int32),
        ("skin", ctypes.c_double), ("capacity", ctypes.c_int32), ("density_scheme", ctypes.c_int32),
    ]


class FreeSurfaceParams(ctypes.Structure):
    """sph_free_surface_params_t (free-surface handling of the shift)."""
    _fields_ = [("barecasco_threshold", ctypes.c_double), ("expansion_iterations", ctypes.c_int32),
                ("surface_scaling", ctypes.c_double)]


class Pairs(ctypes.Structure):
    """sph_pairs_t: a neighborhood in the reference's format (device pointers)."""
    _fields_ = [("n_query", ctypes.c_int64), ("offsets", ctypes.c_void_p), ("counts", ctypes.c_void_p),
                ("pair_j", ctypes.c_void_p), ("distances", ctypes.c_void_p), ("vectors", ctypes.c_void_p),
                ("supports", ctypes.c_void_p), ("kernels", ctypes.c_void_p), ("gradients", ctypes.c_void_p)]


class ViscosityParams(ctypes.Structure):
    """sph_viscosity_params_t (the deltaSPH viscosity schemes)."""
    _fields_ = [("scheme", ctypes.c_int32), ("wall_volume", ctypes.c_int32), ("pi_switch", ctypes.c_int32),
                ("nu", ctypes.c_double), ("alpha", ctypes.c_double), ("eps", ctypes.c_double),
                ("cs", ctypes.c_double), ("rho0", ctypes.c_double)]


class IpsParams(ctypes.Structure):
    """sph_ips_params_t (implicit particle shifting)."""
    _fields_ = [("rtol", ctypes.c_double), ("max_iter", ctypes.c_int32), ("solver_threshold", ctypes.c_double)]


EXPORTS = [
    "sph_neighbor_workspace_bytes", "sph_neighbor_count", "sph_neighbor_fill",
    "sph_solver_workspace_bytes", "sph_solver_create", "sph_solver_destroy", "sph_solver_upload",
    "sph_solver_step", "sph_solver_integrate", "sph_solver_shift", "sph_solver_rhs", "sph_solver_download", "sph_solver_flags",
    "sph_solver_launches_per_step", "sph_solver_kernel_classes", "sph_solver_kernel_name",
    "sph_solver_set_timing", "sph_solver_kernel_times", "sph_solver_autotune", "sph_solver_shapes",
    "sph_solver_set_shape", "sph_solver_tuned_passes", "sph_solver_set_pass_shape", "sph_solver_pass_shapes",
    "sph_batch_workspace_bytes", "sph_batch_create", "sph_solver_graph_step",
    "sph_neighbor_count_static", "sph_solver_vjp_rates", "sph_solver_vjp_gradient", "sph_solver_vjp_shift",
    "sph_solver_vjp_walls",
    "sph_gemm_bf16_tn", "sph_cconv_aggregate", "sph_cconv_aggregate_t", "sph_cconv_aggregate_tc",
    "sph_neighbor_fill_csr", "sph_solver_ips_workspace_bytes", "sph_solver_set_ips", "sph_solver_ips_result",
    "sph_solver_free_surface_workspace_bytes", "sph_solver_set_free_surface", "sph_solver_free_surface_fields",
    "sph_pressure_switch", "sph_liuliu_consistent", "sph_solver_set_verlet_reuse", "sph_solver_sort_count",
    "sph_solver_rhs_walls", "sph_operation", "sph_covariance", "sph_density_gradient", "sph_delta_term",
    "sph_momentum", "sph_pressure_accel", "sph_viscosity", "sph_mdbc_density", "sph_set_gemm_wait_limit",
    "sph_solver_set_verlet_scale",
]

_lib = None


def load(build_if_missing: bool = False):
    """Load libsph103.so (building it first when asked and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _build
            _build.build()
        else:
            raise RuntimeError(f"libsph103.so is not built ({LIB_PATH}); run diffsph_gb300.build.build()")
    lib = ctypes.CDLL(LIB_PATH)
    P, I64, I32, SZ = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_size_t
    DP = ctypes.POINTER(Domain)
    PP = ctypes.POINTER(Params)
    sig = {
        "sph_neighbor_workspace_bytes": ([I64, I64, DP, ctypes.c_double, ctypes.POINTER(SZ)], ctypes.c_int),
        "sph_neighbor_count": ([P, I64, P, P, I64, DP, ctypes.c_double, P, SZ, P, P, P], ctypes.c_int),
        "sph_neighbor_fill": ([P, I64, P, P, I64, DP, ctypes.c_double, P, SZ, P, I64, P, P, P, P, P, P, P, P],
                              ctypes.c_int),
        "sph_solver_vjp_rates": ([P, P, P, P, P, P, P, P, P, P], ctypes.c_int),
        "sph_solver_vjp_gradient": ([P, P, P, P, P, P], ctypes.c_int),
        "sph_solver_vjp_shift": ([P, P, P, P, P, P, P], ctypes.c_int),
        "sph_solver_vjp_walls": ([P, P, P, P, P], ctypes.c_int),
        "sph_gemm_bf16_tn": ([P, P, P, I64, I64, I64, I64, I64, I64, I32, P, P], ctypes.c_int),
        "sph_cconv_aggregate": ([P, I64, P, P, DP, ctypes.c_double, ctypes.c_double, P, I32, I32, P, P],
                                ctypes.c_int),
        "sph_cconv_aggregate_tc": ([P, I64, P, P, DP, ctypes.c_double, ctypes.c_double, P, I32, I32, P, P, P],
                                   ctypes.c_int),
        "sph_cconv_aggregate_t": ([P, I64, P, P, DP, ctypes.c_double, ctypes.c_double, P, I64, I32, I32, P, P],
                                  ctypes.c_int),
        "sph_neighbor_fill_csr": ([P, I64, P, P, I64, DP, ctypes.c_double, P, SZ, P, P, P], ctypes.c_int),
        "sph_neighbor_count_static": ([P, I64, P, P, I64, DP, ctypes.c_double, P, P, P], ctypes.c_int),
        "sph_solver_workspace_bytes": ([PP, I64, I64, ctypes.POINTER(SZ)], ctypes.c_int),
        "sph_solver_create": ([PP, I64, I64, P, SZ, ctypes.POINTER(P)], ctypes.c_int),
        "sph_solver_destroy": ([P], None),
        "sph_solver_upload": ([P, P, P, P, P, P, P, P, P], ctypes.c_int),
        "sph_solver_step": ([P, I32, P], ctypes.c_int),
        "sph_solver_integrate": ([P, P], ctypes.c_int),
        "sph_solver_shift": ([P, P, P], ctypes.c_int),
        "sph_solver_rhs": ([P, P, P, P, P, P, P, P, P], ctypes.c_int),
        "sph_solver_rhs_walls": ([P, P, P, P, P, P, P, P, P], ctypes.c_int),
        "sph_solver_download": ([P, P, P, P, P, P], ctypes.c_int),
        "sph_solver_flags": ([P, ctypes.POINTER(ctypes.c_uint32), P], ctypes.c_int),
        "sph_solver_launches_per_step": ([P], ctypes.c_int),
        "sph_solver_kernel_classes": ([], ctypes.c_int),
        "sph_solver_kernel_name": ([ctypes.c_int], ctypes.c_char_p),
        "sph_solver_set_timing": ([P, I32], ctypes.c_int),
        "sph_solver_autotune": ([P, ctypes.POINTER(I32), ctypes.POINTER(ctypes.c_float), P], ctypes.c_int),
        "sph_solver_shapes": ([], ctypes.c_int),
        "sph_solver_set_shape": ([P, I32], ctypes.c_int),
        "sph_solver_tuned_passes": ([], ctypes.c_int),
        "sph_solver_set_pass_shape": ([P, I32, I32], ctypes.c_int),
        "sph_solver_pass_shapes": ([P, ctypes.POINTER(I32)], ctypes.c_int),
        "sph_solver_set_verlet_reuse": ([P, I32], ctypes.c_int),
        "sph_solver_set_verlet_scale": ([P, ctypes.c_double], ctypes.c_int),
        "sph_solver_sort_count": ([P, ctypes.POINTER(ctypes.c_uint32), P], ctypes.c_int),
        "sph_batch_workspace_bytes": ([PP, ctypes.POINTER(I64), I32, ctypes.POINTER(SZ)], ctypes.c_int),
        "sph_batch_create": ([PP, ctypes.POINTER(I64), I32, P, SZ, ctypes.POINTER(P)], ctypes.c_int),
        "sph_solver_graph_step": ([P, I32, P], ctypes.c_int),
        "sph_solver_kernel_times": ([P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(I32), P], ctypes.c_int),
        "sph_solver_ips_workspace_bytes": ([P, ctypes.POINTER(SZ)], ctypes.c_int),
        "sph_solver_set_ips": ([P, ctypes.POINTER(IpsParams), P, SZ], ctypes.c_int),
        "sph_solver_ips_result": ([P, ctypes.POINTER(I32), ctypes.POINTER(I32), P], ctypes.c_int),
        "sph_solver_free_surface_workspace_bytes": ([P, ctypes.POINTER(SZ)], ctypes.c_int),
        "sph_solver_set_free_surface": ([P, ctypes.POINTER(FreeSurfaceParams), P, SZ], ctypes.c_int),
        "sph_solver_free_surface_fields": ([P, P, P, P, P, P], ctypes.c_int),
        "sph_pressure_switch": ([I64, P, P, P, P, P, P, P, P, P, P, P, P], ctypes.c_int),
        "sph_liuliu_consistent": ([I64] + [P] * 15, ctypes.c_int),
        "sph_operation": ([ctypes.POINTER(Pairs), I32, I32, I32, I32] + [P] * 8, ctypes.c_int),
        "sph_covariance": ([ctypes.POINTER(Pairs), P, P, P, P], ctypes.c_int),
        "sph_density_gradient": ([ctypes.POINTER(Pairs), P, P, P, P, P, P], ctypes.c_int),
        "sph_delta_term": ([ctypes.POINTER(Pairs)] + [P] * 6 + [ctypes.c_double] * 3 + [P, P], ctypes.c_int),
        "sph_momentum": ([ctypes.POINTER(Pairs)] + [P] * 7, ctypes.c_int),
        "sph_pressure_accel": ([ctypes.POINTER(Pairs)] + [P] * 7, ctypes.c_int),
        "sph_viscosity": ([ctypes.POINTER(Pairs)] + [P] * 6 + [ctypes.POINTER(ViscosityParams), P, P], ctypes.c_int),
        "sph_mdbc_density": ([ctypes.POINTER(Pairs), P, P, P, P, ctypes.c_double, ctypes.c_double, P, P, P],
                             ctypes.c_int),
        "sph_set_gemm_wait_limit": ([ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(fn_name: str, code: int):
    if code != 0:
        raise SphError(fn_name, code)


def call(fn_name: str, *args):
    code = getattr(load(), fn_name)(*args)
    check(fn_name, code)
    return code
