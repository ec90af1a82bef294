"""ctypes binding of the C ABI in include/paliwa_gb300.h.

The shared library is built in tree by ``paliwa_gb300.build``. There is no
CPU fallback: if the library is missing or cannot be loaded, every transform
raises, so a GPU run can never pass on a silent substitute.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

OK = 0
INVALID_ARGUMENT = 1
RUNTIME_ERROR = 2
OUT_OF_RANGE = 3
CUDA_ERROR = 4
TIMEOUT = 5

F64 = 0
F32 = 1
F32C = 2

HAT = 0
BIORTHOGONAL = 1
FULLWEIGHTING = 2

# Every exported entry point: name -> (restype, argtypes).
_vp = ctypes.c_void_p
_i = ctypes.c_int
_pi64 = ctypes.POINTER(ctypes.c_int64)
_pi32 = ctypes.POINTER(ctypes.c_int32)
_pd = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "paliwa_gb_last_error": (ctypes.c_char_p, []),
    "paliwa_gb_version": (_i, []),
    "paliwa_gb_synchronize": (_i, [_vp]),
    "paliwa_gb_wavelet_id": (_i, [ctypes.c_char_p, ctypes.POINTER(_i)]),
    "paliwa_gb_wavelet_filters": (_i, [_i, _i, ctypes.POINTER(_i), _pi32, _pd]),
    "paliwa_gb_transform_in": (
        _i, [_vp, _i, _i, _pi64, _pi64, _i, _pi64, _i, _pi32, _pd, _i, _vp]),
    "paliwa_gb_transform_in_window": (
        _i, [_vp, _i, _i, _pi64, _pi64, _pi64, _pi64, _i, _pi64, _i, _pi32,
             _pd, _i, _vp]),
    "paliwa_gb_hierarchize_in": (
        _i, [_vp, _i, _i, _pi64, _pi64, _pi64, _i, _i, _vp]),
    "paliwa_gb_dehierarchize_in": (
        _i, [_vp, _i, _i, _pi64, _pi64, _pi64, _i, _i, _vp]),
    "paliwa_gb_hierarchize": (_i, [_vp, _i, _i, _pi64, _pi64, _pi64, _i, _vp]),
    "paliwa_gb_dehierarchize": (_i, [_vp, _i, _i, _pi64, _pi64, _pi64, _i, _vp]),
    "paliwa_gb_transform_bounds": (
        _i, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
             _pi64, _i, _pi32, _i, _pi64, _pi64]),
    "paliwa_gb_transform_outputs": (
        _i, [_vp, _i, _i, _pi64, _pi64, _pi64, _pi64, _i, _pi64, _i, _pi32,
             _pd, _i, _pi64, _pi64, _pi64, _vp]),
    "paliwa_gb_dump_to_binary_file": (
        _i, [_vp, ctypes.c_int64, ctypes.c_char_p, _vp]),
    "paliwa_gb_transform_noalloc": (
        _i, [_vp, _i, _i, _pi64, _pi64, _pi64, _i, _i, _vp]),
    "paliwa_gb_batch_use_slabs": (_i, [_vp, _i]),
    "paliwa_gb_batch_status": (_i, [_vp]),
    "paliwa_gb_batch_set_ctas_per_sm": (_i, [_vp, _i]),
    "paliwa_gb_batch_use_tma": (_i, [_vp, _i]),
    "paliwa_gb_batch_create": (
        _i, [_i, _i, _pi64, _pi64, _pi64, _i, _i, ctypes.POINTER(_vp),
             ctypes.POINTER(_vp)]),
    "paliwa_gb_batch_hierarchize": (_i, [_vp, _vp]),
    "paliwa_gb_batch_dehierarchize": (_i, [_vp, _vp]),
    "paliwa_gb_batch_use_graphs": (_i, [_vp, _i]),
    "paliwa_gb_batch_set_groups": (_i, [_vp, _i]),
    "paliwa_gb_batch_info": (_i, [_vp, _pi64, _pi64, _pi64]),
    "paliwa_gb_batch_profile": (
        _i, [_vp, _i, _vp, _i, ctypes.POINTER(_i),
             ctypes.POINTER(ctypes.c_float), _pi64,
             ctypes.POINTER(ctypes.c_int32)]),
    "paliwa_gb_batch_autotune": (_i, [_vp, _vp, _i, ctypes.POINTER(_i)]),
    "paliwa_gb_batch_tuning": (
        _i, [_vp, _i, _i, ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_int32),
             ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "paliwa_gb_batch_set_tuning": (
        _i, [_vp, _i, _i, ctypes.POINTER(ctypes.c_int32),
             ctypes.POINTER(ctypes.c_int32)]),
    "paliwa_gb_batch_destroy": (None, [_vp]),
    "paliwa_gb_ct_create": (
        _i, [_i, _i, _pi64, _pd, _pi64, _i, ctypes.POINTER(_vp), _i,
             ctypes.POINTER(_vp)]),
    "paliwa_gb_ct_info": (_i, [_vp, _pi64, _pi64]),
    "paliwa_gb_ct_subspaces": (_i, [_vp, _pi64, _pi64]),
    "paliwa_gb_ct_combine": (_i, [_vp, _vp, _vp]),
    "paliwa_gb_ct_restrict": (_i, [_vp, _vp, _vp]),
    "paliwa_gb_ct_scatter": (_i, [_vp, _vp, _vp, _vp]),
    "paliwa_gb_ct_destroy": (None, [_vp]),
}


class PaliwaError(RuntimeError):
    """Base class of errors returned by the C ABI."""


class InvalidArgument(PaliwaError, ValueError):
    """std::invalid_argument in the reference (or a failed assert)."""


class OutOfRange(PaliwaError, KeyError):
    """std::out_of_range in the reference (unknown wavelet name)."""

    def __str__(self):  # KeyError quotes its message otherwise
        return RuntimeError.__str__(self)


class CudaError(PaliwaError):
    """A CUDA call inside the library failed."""


class DeviceTimeout(PaliwaError):
    """A bounded device-side wait gave up."""


_ERRORS = {
    INVALID_ARGUMENT: InvalidArgument,
    RUNTIME_ERROR: PaliwaError,
    OUT_OF_RANGE: OutOfRange,
    CUDA_ERROR: CudaError,
    TIMEOUT: DeviceTimeout,
}

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise ImportError(f"paliwa_gb300 CUDA library not built: {path}")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc == OK:
        return
    msg = load().paliwa_gb_last_error().decode()
    raise _ERRORS.get(rc, PaliwaError)(msg)


def i64(values):
    values = [int(v) for v in values]
    return (ctypes.c_int64 * max(1, len(values)))(*values)


def i32(values):
    values = [int(v) for v in values]
    return (ctypes.c_int32 * max(1, len(values)))(*values)


def f64(values):
    values = [float(v) for v in values]
    return (ctypes.c_double * max(1, len(values)))(*values)
