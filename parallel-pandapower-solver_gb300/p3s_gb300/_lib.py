"""ctypes binding of the C ABI in include/gbpf.h (libgbpf.so, built in-tree).

The library is the product path: there is no CPU fallback. Loading fails loudly when the
library is missing or no CUDA device is visible.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
_bp = C.POINTER(C.c_uint8)


class Params(C.Structure):
    _fields_ = [
        ("max_iter", C.c_int),
        ("tol", C.c_double),
        ("line_search", C.c_int),
        ("precision", C.c_int),
        ("mixed_switch", C.c_double),
        ("check_v0", C.c_int),
        ("pivot_ratio_double", C.c_double),
        ("pivot_ratio_single", C.c_double),
        ("vote_rule", C.c_int),
        ("polish", C.c_double),
        ("vtol", C.c_double),
        ("chord_tol", C.c_double),
        ("shared_start", C.c_int),
        ("phase_timers", C.c_int),
        ("eager_jacobian", C.c_int),
    ]


class Info(C.Structure):
    _fields_ = [
        ("n_bus", C.c_int),
        ("nnz_ybus", C.c_int),
        ("n_var_bus", C.c_int),
        ("n_blocks", C.c_int),
        ("n_levels", C.c_int),
        ("n_back_levels", C.c_int),
        ("cases_per_cta", C.c_int),
        ("threads_per_cta", C.c_int),
        ("workers", C.c_int),
        ("factor_pairs", C.c_longlong),
        ("forward_pairs", C.c_longlong),
        ("backward_pairs", C.c_longlong),
        ("rcond0", C.c_double),
        ("jinv_norm", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("single_factorizations", C.c_ulonglong),
        ("double_factorizations", C.c_ulonglong),
        ("single_rejected", C.c_ulonglong),
        ("double_rejected", C.c_ulonglong),
        ("macro_steps", C.c_ulonglong),
        ("grid", C.c_int),
        ("cases_per_cta", C.c_int),
        ("kernel_ms", C.c_double),
        ("call_ms", C.c_double),
        ("threads_per_cta", C.c_int),
        ("chord_steps", C.c_ulonglong),
        ("first_steps", C.c_ulonglong),
        ("phase_cycles", C.c_ulonglong * 6),
        ("lazy_jacobians", C.c_ulonglong),
        ("jacobian_sweeps", C.c_ulonglong),
    ]


class Job(C.Structure):
    """struct gbpf_job (one topology's cases in a group launch)."""

    _fields_ = [
        ("solver", _vp),
        ("n_cases", C.c_int),
        ("S", _vp),
        ("s_per_col", C.c_int),
        ("V0", _vp),
        ("v0_per_col", C.c_int),
        ("pin", _vp),
        ("st_ptr", _vp),
        ("st_k", _vp),
        ("st_val", _vp),
        ("V", _vp),
        ("iterations", _vp),
        ("converged", _vp),
        ("cases_per_cta", C.c_int),
        ("out_ptr", _vp),
        ("out_idx", _vp),
        ("reslack", C.c_int),
        ("served", _vp),
        ("precision", C.c_int),
    ]


# exported symbols and their signatures (restype, argtypes)
SIGNATURES = {
    "gbpf_last_error": (C.c_char_p, []),
    "gbpf_version": (C.c_int, []),
    "gbpf_device_count": (C.c_int, []),
    "gbpf_create": (_vp, [C.c_int, _ip, _ip, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_int]),
    "gbpf_create_ex": (_vp, [C.c_int, _ip, _ip, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_int, C.c_int]),
    "gbpf_destroy": (None, [_vp]),
    "gbpf_update_Y": (C.c_int, [_vp, _dp, C.c_int]),
    "gbpf_get_info": (C.c_int, [_vp, C.POINTER(Info)]),
    "gbpf_get_stats": (C.c_int, [_vp, C.POINTER(Stats)]),
    "gbpf_get_posmap": (C.c_int, [_vp, _ip]),
    "gbpf_get_Y": (C.c_int, [_vp, _dp]),
    "gbpf_get_shape": (C.c_int, [_vp, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "gbpf_set_shape": (C.c_int, [_vp, C.c_longlong, C.c_int, C.c_int]),
    "gbpf_prepare_shapes": (C.c_int, [_vp, C.c_int]),
    "gbpf_get_row_of_bus": (C.c_int, [_vp, _ip]),
    "gbpf_solve_batch": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _dp, C.c_int, C.POINTER(Params), _dp, _ip, _bp]),
    "gbpf_solve_batch_device": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _vp, C.c_int, C.POINTER(Params), _vp, _vp,
                                          _vp]),
    "gbpf_solve_lanes": (C.c_int, [_vp, C.c_int, _dp, _dp, C.c_int, _lp, C.POINTER(Params), _dp, _ip, _bp]),
    "gbpf_solve_lanes_device": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int, _vp, C.POINTER(Params), _vp, _vp, _vp]),
    "gbpf_solve_lanes_async": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp, C.c_int, _lp, C.POINTER(Params), _dp,
                                         _ip, _bp]),
    "gbpf_solve_wait": (C.c_int, [_vp, C.c_int]),
    "gbpf_solve_contingency": (C.c_int, [_vp, C.c_int, _dp, _dp, _bp, _dp, _ip, _ip, _dp, C.POINTER(Params), _dp,
                                         _ip, _bp]),
    "gbpf_dc_start": (C.c_int, [_vp, _dp, _dp, _dp]),
    "gbpf_dc_start_batch": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp, _dp, _bp]),
    "gbpf_eval_jacobian": (C.c_int, [_vp, _dp, _dp, _bp, _dp, _dp]),
    "gbpf_selftest_conversions": (C.c_int, [_dp, C.c_int, C.POINTER(C.c_float), _dp, C.POINTER(C.c_float)]),
    "gbpf_get_mismatch": (C.c_int, [_vp, _dp, C.c_longlong]),
    "gbpf_selftest_math": (C.c_int, [_dp, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "gbpf_host_alloc": (_vp, [C.c_size_t]),
    "gbpf_host_free": (None, [_vp]),
    "gbpf_plan_selftest": (C.c_int, [C.c_int, _ip, _ip, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_int, _dp, _dp,
                                     _dp, _dp, _ip, C.c_char_p, C.c_int, C.c_double]),
    "gbpf_set_chain_cap": (C.c_int, [_vp, C.c_double]),
    "gbpf_islands": (C.c_int, [C.c_int, C.c_int, _ip, _ip, _bp, C.c_int, _ip, _ip, _bp, _dp, C.c_int, _ip, _bp,
                               _ip, _ip]),
    "gbpf_group_create": (_vp, []),
    "gbpf_group_destroy": (None, [_vp]),
    "gbpf_group_solve": (C.c_int, [_vp, C.c_int, C.POINTER(Job), C.POINTER(Params)]),
    "gbpf_stream_create": (_vp, [C.c_int, C.c_size_t, C.c_int, C.c_int, C.c_int]),
    "gbpf_stream_destroy": (None, [_vp]),
    "gbpf_stream_start": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), C.POINTER(Params), C.c_double]),
    "gbpf_stream_submit": (C.c_int, [_vp, C.POINTER(Job)]),
    "gbpf_stream_flags": (C.POINTER(C.c_int), [_vp]),
    "gbpf_stream_done": (C.c_int, [_vp, C.c_int]),
    "gbpf_stream_alive": (C.c_int, [_vp]),
    "gbpf_stream_stop": (C.c_int, [_vp]),
    "gbpf_group_solve_device": (C.c_int, [_vp, C.c_int, C.POINTER(Job), C.POINTER(Params)]),
    "gbpf_group_stats": (C.c_int, [_vp, C.POINTER(Stats)]),
    "gbpf_group_set_shape": (C.c_int, [_vp, C.c_int, C.c_int]),
    "gbpf_build_sbus": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _lp, _ip, _dp, _dp, _bp, _dp, _dp]),
    "gbpf_build_sbus_device": (C.c_int, [C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbpf_branch_flows": (C.c_int, [C.c_int, C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _bp, C.c_double, _dp,
                                    _bp, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp]),
    "gbpf_branch_flows_device": (C.c_int, [C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_double, _vp,
                                           _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbpf_branch_stamps": (C.c_int, [C.c_int, _dp, _dp, _dp, _dp, _dp, _bp, _bp, _bp, _dp]),
    "gbpf_branch_stamps_device": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbpf_update_Y_from_branches": (C.c_int, [_vp, _dp, _dp]),
    "gbpf_set_branches": (C.c_int, [_vp, C.c_int, _ip, _ip, _ip, _dp, _bp, _dp]),
    "gbpf_solver_islands": (C.c_int, [_vp, C.c_int, _ip, _ip, _bp, C.c_int, _ip, _ip, _bp, _dp, C.c_int, _ip, _bp,
                                      _ip, _ip]),
    "gbpf_islands_device_static": (C.c_int, [C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, _vp, _vp, C.c_int, _vp,
                                             _vp, C.c_int, _vp, _vp, _vp, _vp, _vp]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """The loaded library (built first if missing and a CUDA toolkit is present)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path) or (build_if_missing and not _build.up_to_date()):
        if not build_if_missing:
            raise RuntimeError(f"libgbpf.so not built ({path}); run p3s_gb300.build.build()")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def require_device():
    L = load()
    if L.gbpf_device_count() <= 0:
        raise RuntimeError("p3s_gb300: no CUDA device visible; the GPU solver has no CPU fallback")
    return L


def last_error() -> str:
    return load().gbpf_last_error().decode(errors="replace")


def check(rc: int, what: str = ""):
    if rc != 0:
        msg = last_error()
        raise RuntimeError(msg if msg else f"{what} failed ({rc})")


PHASES = ("load", "factor_forward", "backward", "step", "eval", "decide")


def stats_dict(o: Stats) -> dict:
    """gbpf_stats as a dict; phase_cycles as {phase: SM cycles summed over CTAs}."""
    out = {f: getattr(o, f) for f, _ in o._fields_ if f != "phase_cycles"}
    out["phase_cycles"] = dict(zip(PHASES, (int(x) for x in o.phase_cycles)))
    return out


def d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def i32(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def i64(a: np.ndarray):
    return a.ctypes.data_as(_lp)


def u8(a: np.ndarray):
    return a.ctypes.data_as(_bp)


def cview(a: np.ndarray):
    """complex128 array as its interleaved float64 pointer"""
    return a.view(np.float64).ctypes.data_as(_dp)
