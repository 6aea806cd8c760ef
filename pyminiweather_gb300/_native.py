"""ctypes binding of libminiweather_gb300.so (declarations in include/miniweather_gb300.h).

The library is the only compute path: if it cannot be loaded, every entry
point raises.  Tensors are passed as raw device pointers together with the
current CUDA stream of PyTorch.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import build as _build

_lock = threading.Lock()
_lib = None

MW_OK = 0
MW_DIR_X, MW_DIR_Z = 0, 1
MW_F64_NATIVE, MW_F64_SPLIT, MW_F64_IEEE = 0, 1, 2
MW_FLAG_WRITE_HALO = 1
MW_FLAG_INDEX64 = 2
MW_FLAG_CHECK_FINITE = 4
MW_FLAG_PAIRS_OUT = 8
MW_FLAG_PAIRS_IN = 16
MW_BG_CONST_THETA, MW_BG_BVFREQ = 0, 1
MW_MAX_BUBBLES = 8

F64_MODES = {"native": MW_F64_NATIVE, "split": MW_F64_SPLIT, "fp64": MW_F64_IEEE}

_i, _u, _d, _P, _sz = ctypes.c_int, ctypes.c_uint, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t

# name -> argtypes (all return int unless listed in _RESTYPES)
_SIGNATURES = {
    "mw_dirstage_f64": [_i, _i, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _d, _i, _i, _u, _P],
    "mw_dirstage_f32": [_i, _i, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _d, _i, _u, _P],
    "mw_step_f64": [_i, _i, _d, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i, ctypes.POINTER(_i), _i, _u, _P],
    "mw_step_f64_host": [_i, _i, _d, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(_i), _i,
                         _u, _i, _P],
    "mw_step_f32": [_i, _i, _d, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i, ctypes.POINTER(_i), _u, _P],
    "mw_step_f64_noalloc": [_i, _i, _d, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _i, ctypes.POINTER(_i), _i, _u,
                            _P],
    "mw_ensemble_plan_info": [_i, _P, _i, _P],
    "mw_ensemble_plan": [_i, _P, _i, _P, _sz, _P, _P],
    "mw_ensemble_step_f64": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i, ctypes.POINTER(_i), _i, _u, _i, _i, _P],
    "mw_ensemble_step_f32": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i, ctypes.POINTER(_i), _u, _i, _i, _P],
    "mw_ensemble_occupancy": [_i, _i, ctypes.POINTER(_i)],
    "mw_dirstage_vjp_workspace_bytes": [_i, _i],
    "mw_dirstage_vjp_f64": [_i, _i, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i, _P, _d, _i, _i, _P, _sz, _P],
    "mw_step_record_f64": [_i, _i, _d, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i, _i, _P],
    "mw_step_vjp_f64": [_i, _i, _d, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i, _i, _P, _sz, _P],
    "mw_init_f64": [_i, _i, _d, _d, _i, _d, _i, _P, _P, _P, _P, _P, _P, _P, _P],
    "mw_init_f32": [_i, _i, _d, _d, _i, _d, _i, _P, _P, _P, _P, _P, _P, _P, _P],
    "mw_gravity_source_f64": [_i, _i, _d, _d, _P, _P, _P],
    "mw_stats_workspace_bytes": [_i, _i],
    "mw_stats_f64": [_i, _i, _d, _d, _P, _P, _P, _P, _sz, _P, _P],
    "mw_stats_f32": [_i, _i, _d, _d, _P, _P, _P, _P, _sz, _P, _P],
    "mw_solution_variables_f64": [_i, _i, _P, _P, _P, _P, _P],
    "mw_count_nonfinite_f64": [_i, _i, _P, _P, _P],
    "mw_debug_oob_count": [_P, _i],
    "mw_debug_oob_selftest": [_P],
    "mw_debug_wait_timeouts": [_P, _i],
    "mw_fp64_throughput": [_i, _i, _P, _P],
    "mw_count_nonfinite_f32": [_i, _i, _P, _P, _P],
    "mw_savetxt_f64": [_P, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_char_p, _i, _i],
    "mw_set_bc_f64": [_i, _i, _P, _P, _i, _P],
    "mw_interpolate_f64": [_i, _i, _P, _P, _P, _i, _P],
    "mw_flux_f64": [_i, _i, _d, _d, _d, _P, _P, _P, _P, _P, _P, _P, _P, _i, _P],
    "mw_tend_f64": [_i, _i, _d, _d, _P, _P, _P, _P, _i, _P],
    "mw_add_source_f64": [_i, _i, _P, _P, _P],
    "mw_update_f64": [_i, _i, _P, _P, _P, _d, _P],
    "mw_last_error": [],
    "mw_status_string": [_i],
    "mw_abi_version": [],
}
_RESTYPES = {"mw_last_error": ctypes.c_char_p, "mw_status_string": ctypes.c_char_p,
             "mw_stats_workspace_bytes": _sz, "mw_dirstage_vjp_workspace_bytes": _sz}


class EnsMember(ctypes.Structure):
    """mw_ens_member of include/miniweather_gb300.h."""
    _fields_ = [("nx", ctypes.c_int), ("nz", ctypes.c_int), ("dx", ctypes.c_double), ("dz", ctypes.c_double),
                ("dt", ctypes.c_double), ("state_off", ctypes.c_longlong), ("cell_off", ctypes.c_longlong),
                ("int_off", ctypes.c_longlong)]


class EnsPlanInfo(ctypes.Structure):
    """mw_ens_plan_info of include/miniweather_gb300.h."""
    _fields_ = [("n_members", ctypes.c_int), ("n_x_items", ctypes.c_int), ("n_z_items", ctypes.c_int),
                ("z_tile", ctypes.c_int), ("members_off", ctypes.c_size_t), ("x_items_off", ctypes.c_size_t),
                ("z_items_off", ctypes.c_size_t), ("bytes", ctypes.c_size_t), ("xrows_off", ctypes.c_size_t),
                ("n_xrows", ctypes.c_longlong)]


class MiniWeatherError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn: str, status: int, message: str):
        super().__init__("%s failed (%d: %s): %s" % (fn, status, status_string(status), message))
        self.status = status


def library_path() -> str:
    return _build.LIB_PATH


def load():
    """Load (building first if needed) the CUDA library; raises if that fails."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            if not os.path.exists(path):
                raise RuntimeError("libminiweather_gb300.so missing at %s" % path)
            L = ctypes.CDLL(path)
            for name, args in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = _RESTYPES.get(name, _i)
            _lib = L
    return _lib


def status_string(st: int) -> str:
    return load().mw_status_string(int(st)).decode()


def call(name: str, *args):
    """Call an int-returning entry point and raise MiniWeatherError on failure."""
    L = load()
    st = getattr(L, name)(*args)
    if st != MW_OK:
        raise MiniWeatherError(name, st, L.mw_last_error().decode())
    return st


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def require_cuda(t: torch.Tensor, name: str, dtype=None, shape=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError("%s must be a torch.Tensor, got %s" % (name, type(t).__name__))
    if not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor (this package has no CPU path)" % name)
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    if dtype is not None and t.dtype != dtype:
        raise TypeError("%s must have dtype %s, got %s" % (name, dtype, t.dtype))
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError("%s must have shape %s, got %s" % (name, tuple(shape), tuple(t.shape)))
    return t
