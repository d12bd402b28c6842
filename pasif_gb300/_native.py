"""ctypes binding of libpasif_gb300.so (the C ABI of include/pasif_gb300.h).

The shared library is built in-tree (pasif_gb300/build.py).  There is no
Python or CPU fallback: if the library is missing, importing this module
raises, and every solve runs the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpasif_gb300.so")

PASIF_OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_NVRTC = 3
ERR_MEMORY = 4
ERR_STATE = 5
ERR_LENGTH = 6

FP64, FP32, FP32_KAHAN, FP32_EXT = 0, 1, 2, 3
HOST, DEVICE = 0, 1
KERNEL_NONE, KERNEL_GENERIC, KERNEL_SPECIALISED = 0, 1, 2
PLAN_GENERIC_ONLY = 1
PLAN_NO_LITERALS = 2
PLAN_WARP_SLICED = 4
PLAN_NO_WARP_SLICED = 8
PLAN_FAST = 16

PRECISIONS = {"fp64": FP64, "fp32": FP32, "fp32_kahan": FP32_KAHAN, "fp32_ext": FP32_EXT}

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint)
_llp = C.POINTER(C.c_longlong)


class PatternC(C.Structure):
    _fields_ = [("n", C.c_int), ("n_sp", C.c_int),
                ("k_nnz", C.c_int), ("k_ptr", _ip), ("k_col", _ip),
                ("g_nnz", C.c_int), ("g_idx", _ip),
                ("l_nnz", C.c_int), ("l_idx", _ip),
                ("p_nnz", C.c_int), ("p_idx", _ip),
                ("f_nnz", C.c_int), ("f_idx", _ip)]


class ReducersC(C.Structure):
    _fields_ = [("n_max", C.c_int), ("max_comp", _ip), ("max_start", C.c_int),
                ("n_sq", C.c_int), ("sq_comp", _ip), ("sq_start", C.c_int)]


class PasifError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"pasif_gb300 error {code}: {msg}")
        self.code = code


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    return C.CDLL(LIB_PATH)


lib = _load()

_vp = C.c_void_p
_SIGS = {
    "pasif_last_error": (C.c_char_p, []),
    "pasif_version": (C.c_int, []),
    "pasif_device_count": (C.c_int, []),
    "pasif_driver_create": (C.c_int, [C.POINTER(_vp), C.POINTER(_dp), _llp, C.c_int, C.c_uint, C.c_uint,
                                      C.c_int, C.c_int, C.c_int, C.c_uint]),
    "pasif_driver_destroy": (C.c_int, [_vp]),
    "pasif_driver_set_precision": (C.c_int, [_vp, C.c_int]),
    "pasif_driver_set_fwd_k": (C.c_int, [_vp, C.c_uint, C.c_uint, _dp, _up, _up, C.c_longlong]),
    "pasif_driver_set_bwd_k": (C.c_int, [_vp, C.c_uint, C.c_uint, _dp, _up, _up, C.c_longlong]),
    "pasif_driver_set_fwd_gamma": (C.c_int, [_vp, _up, _dp, _up, C.c_longlong]),
    "pasif_driver_set_bwd_gamma": (C.c_int, [_vp, _up, _dp, _up, C.c_longlong]),
    "pasif_driver_set_fwd_lambda": (C.c_int, [_vp, _up, _dp, _up, C.c_longlong]),
    "pasif_driver_set_bwd_lambda": (C.c_int, [_vp, _up, _dp, _up, C.c_longlong]),
    "pasif_driver_set_fwd_psi": (C.c_int, [_vp, _up, _dp, _up, C.c_longlong]),
    "pasif_driver_set_bwd_psi": (C.c_int, [_vp, _up, _dp, _up, C.c_longlong]),
    "pasif_driver_set_fwd_force_pattern": (C.c_int, [_vp, _dp, C.c_longlong]),
    "pasif_driver_set_bwd_force_pattern": (C.c_int, [_vp, _dp, C.c_longlong]),
    "pasif_driver_set_fwd_initial_conditions": (C.c_int, [_vp, _dp, C.c_longlong]),
    "pasif_driver_set_bwd_initial_conditions": (C.c_int, [_vp, _dp, C.c_longlong]),
    "pasif_driver_allocate_system": (C.c_int, [_vp]),
    "pasif_driver_allocate_adjoint": (C.c_int, [_vp]),
    "pasif_driver_load_excitations": (C.c_int, [_vp, C.POINTER(_dp), _llp, C.c_int, C.c_uint]),
    "pasif_driver_set_interpolation_matrix": (C.c_int, [_vp, _dp, C.c_longlong, C.c_uint]),
    "pasif_driver_set_modulation_buffer": (C.c_int, [_vp, _dp, C.c_longlong]),
    "pasif_driver_get_amplitudes": (C.c_int, [_vp, _dp, C.c_longlong, _llp]),
    "pasif_driver_get_trajectory": (C.c_int, [_vp, C.c_uint, _dp, C.c_longlong, _llp]),
    "pasif_driver_get_gradient": (C.c_int, [_vp, C.c_uint, _dp, C.c_longlong, _llp]),
    "pasif_driver_last_kernel": (C.c_int, [_vp, _ip]),
    "pasif_plan_create": (C.c_int, [C.POINTER(_vp), C.POINTER(PatternC), C.c_int, C.c_int]),
    "pasif_plan_destroy": (C.c_int, [_vp]),
    "pasif_signals_create": (C.c_int, [C.POINTER(_vp), _dp, C.c_int, C.c_int, C.c_int, _dp, C.c_int, C.c_int, _vp]),
    "pasif_signals_destroy": (C.c_int, [_vp]),
    "pasif_signals_update": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    "pasif_batch_resize": (C.c_int, [_vp, C.c_int]),
    "pasif_batch_reserve": (C.c_int, [_vp, C.c_int, C.c_int]),
    "pasif_batch_set_adjoint_storage": (C.c_int, [_vp, C.c_longlong]),
    "pasif_batch_create": (C.c_int, [C.POINTER(_vp), _vp, C.c_int]),
    "pasif_batch_destroy": (C.c_int, [_vp]),
    "pasif_batch_set": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, _vp]),
    "pasif_batch_forward": (C.c_int, [_vp, _vp, C.c_double, C.c_int, C.c_int, C.POINTER(ReducersC), _vp]),
    "pasif_batch_get": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, _vp]),
    "pasif_batch_adjoint": (C.c_int, [_vp, _vp, C.c_double, C.c_int, C.POINTER(ReducersC), _vp, _vp, _vp, _vp,
                                      C.c_int, _vp]),
    "pasif_batch_kernel_info": (C.c_int, [_vp, _ip, _ip]),
    "pasif_plan_jit_report": (C.c_int, [_vp, _dp, C.c_int, C.c_ulonglong, C.c_ulonglong, C.c_int, _dp,
                                        C.c_char_p, C.c_longlong, _llp]),
    "pasif_plan_jit_report_adjoint": (C.c_int, [_vp, _dp, C.c_int, C.c_ulonglong, C.c_char_p, C.c_longlong, _llp]),
    "pasif_batch_adjoint_kernel": (C.c_int, [_vp, _ip]),
    "pasif_pool_create": (C.c_int, [C.POINTER(_vp), C.POINTER(PatternC), C.c_int, C.c_int, _dp, C.c_double,
                                    C.POINTER(ReducersC), C.c_int, C.c_longlong, C.c_int, C.c_int]),
    "pasif_pool_destroy": (C.c_int, [_vp]),
    "pasif_pool_admit": (C.c_int, [_vp, C.c_int, _dp, _dp, _ip, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   _ip]),
    "pasif_pool_launch": (C.c_int, [_vp]),
    "pasif_pool_poll": (C.c_int, [_vp, _ip, C.c_int, _ip]),
    "pasif_pool_harvest": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp]),
    "pasif_pool_info": (C.c_int, [_vp, _ip, _llp, _ip]),
    "pasif_plan_jit_report_pool": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(ReducersC), C.c_char_p, C.c_longlong,
                                             _llp]),
    "pasif_fma_peak": (C.c_int, [C.c_int, _dp]),
    "pasif_forward_noalloc": (C.c_int, [C.POINTER(PatternC), C.c_int, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int,
                                        _vp, C.c_double, C.c_int, C.c_int, _vp, _vp]),
    "pasif_forward_noalloc_status": (C.c_int, [_ip, _ip, _vp]),
    "pasif_driver_set_memory_budget": (C.c_int, [_vp, C.c_longlong]),
    "pasif_driver_last_chunks": (C.c_int, [_vp, _ip]),
    "pasif_sweep_chunk": (C.c_int, [C.c_longlong, C.c_longlong, C.c_longlong, _llp]),
    "pasif_forward": (C.c_int, [C.POINTER(PatternC), C.c_int, C.c_int, _dp, _dp, _ip, _dp, C.c_int, C.c_int,
                                C.c_int, _dp, C.c_double, C.c_int, C.c_int, C.POINTER(ReducersC), _dp, _dp, _dp]),
}

for _name, (_res, _args) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

EXPORTED = tuple(_SIGS)


def last_error() -> str:
    return lib.pasif_last_error().decode(errors="replace")


def check(rc: int) -> None:
    if rc != PASIF_OK:
        raise PasifError(rc, last_error())


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def uptr(a: np.ndarray):
    return a.ctypes.data_as(_up)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def u32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def device_count() -> int:
    return int(lib.pasif_device_count())
