"""ctypes binding of libtt_gb300.so (the C ABI in include/tracetransform.h).

The library is built in-tree by ``python -m tracetransform_gb300.build``.  There
is no fallback: if the library is missing or cannot be loaded, every entry
point raises, so a machine without the CUDA engine never silently computes
something else.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtt_gb300.so")

TT_OK = 0
STATUS_NAMES = {0: "TT_OK", 1: "TT_ERR_INVALID_ARG", 2: "TT_ERR_UNSUPPORTED", 3: "TT_ERR_CUDA",
                4: "TT_ERR_TIMEOUT", 5: "TT_ERR_OOM"}

# every symbol include/tracetransform.h declares
EXPORTS = (
    "tt_plan_create", "tt_plan_destroy", "tt_plan_synchronize", "tt_last_error", "tt_version",
    "tt_pad_geometry", "tt_ortho_size", "tt_angles_from_step", "tt_sinograms", "tt_circus",
    "tt_zscore", "tt_rotate", "tt_resize", "tt_transform", "tt_sinograms_device", "tt_circus_device", "tt_zscore_device",
    "tt_circus_zscore_noalloc", "tt_transform_batch", "tt_transform_batch_device",
    "tt_circus_backward_device", "tt_sinograms_backward_device", "tt_sinograms_f64_device",
    "tt_circus_f64_device", "tt_circus_backward_f64_device", "tt_sinograms_backward_f64_device",
    "tt_circus_orthonormal_device", "tt_nos", "tt_transform_batch_sinograms_device",
    "tt_transform_batch_stage_ms", "tt_transform_extended", "tt_transform_batch_tile",
    "tt_debug_fail_allocations",
)


class TTError(RuntimeError):
    """A failed engine call: .status is the tt_status code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class InvalidArgument(TTError, ValueError):
    pass


class PFunctionalC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("order", ctypes.c_int32), ("center", ctypes.c_int32)]


_lib = None
_F = ctypes.POINTER(ctypes.c_float)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_P = ctypes.c_void_p
_int = ctypes.c_int


def lib():
    """The loaded engine library (raises if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                           "`python -m tracetransform_gb300.build` (needs nvcc)")
    l = ctypes.CDLL(LIB_PATH)
    st = ctypes.c_int
    sig = {
        "tt_plan_create": [ctypes.POINTER(_P), _int],
        "tt_plan_destroy": [_P],
        "tt_plan_synchronize": [_P],
        "tt_pad_geometry": [_int, _int, ctypes.POINTER(_int), ctypes.POINTER(_int), ctypes.POINTER(_int)],
        "tt_ortho_size": [ctypes.c_uint, ctypes.POINTER(_int)],
        "tt_angles_from_step": [ctypes.c_uint, _F, _int, ctypes.POINTER(_int)],
        "tt_sinograms": [_P, _F, _int, _int, ctypes.c_uint, _I32, _int, _F],
        "tt_circus": [_P, _F, _int, _int, ctypes.POINTER(PFunctionalC), _int, _F],
        "tt_zscore": [_P, _F, _int, _int, _F],
        "tt_rotate": [_P, _F, _int, _int, ctypes.c_float, _F],
        "tt_resize": [_P, _F, _int, _int, _int, _int, _F],
        "tt_transform": [_P, _F, _int, _int, ctypes.c_uint, _I32, _int, ctypes.POINTER(PFunctionalC),
                         _int, _F, _F],
        "tt_sinograms_device": [_P, _P, _int, _int, _int, _int, _int, _int, _F, _int, _I32, _int,
                                _P, _P, _P],
        "tt_circus_device": [_P, _P, _int, _int, _int, ctypes.POINTER(PFunctionalC), _int, _I32,
                             _P, _P],
        "tt_zscore_device": [_P, _P, _int, _int, _P, _P],
        "tt_circus_zscore_noalloc": [_P, _int, _int, _int, ctypes.POINTER(PFunctionalC), _int,
                                     _P, _P],
        "tt_transform_batch": [_P, _F, _I64, _I32, _I32, _I32, _int, _I32, _int,
                               ctypes.POINTER(PFunctionalC), _int, _F, _F],
        "tt_transform_batch_device": [_P, _P, _I64, _I32, _I32, _I32, _int, _I32, _int,
                                      ctypes.POINTER(PFunctionalC), _int, _P, _P, _P],
        "tt_circus_backward_device": [_P, _P, _int, _int, _int, ctypes.POINTER(PFunctionalC),
                                      _int, _P, _P, _P],
        "tt_circus_backward_f64_device": [_P, _P, _int, _int, _int,
                                          ctypes.POINTER(PFunctionalC), _int, _P, _P, _P],
        "tt_sinograms_backward_device": [_P, _int, _int, _int, _int, _int, _int, _F, _int, _I32,
                                         _int, _P, _P, _P, _P],
        "tt_sinograms_backward_f64_device": [_P, _int, _int, _int, _int, _int, _int, _F, _int,
                                             _I32, _int, _P, _P, _P, _P],
        "tt_sinograms_f64_device": [_P, _P, _int, _int, _F, _int, _I32, _int, _P, _P, _P],
        "tt_circus_f64_device": [_P, _P, _int, _int, _int, ctypes.POINTER(PFunctionalC), _int,
                                 _P, _P],
        "tt_circus_orthonormal_device": [_P, _P, _int, _int, _int, ctypes.POINTER(PFunctionalC),
                                         _int, _P, _I32, _I32, _P],
        "tt_nos": [_P, _F, _int, _int, _F, _I32, _I32],
        "tt_transform_batch_sinograms_device": [_P, _P, ctypes.c_int64, _I64, _P],
        "tt_transform_batch_stage_ms": [_P, _F],
        "tt_transform_batch_tile": [_P, _I32, ctypes.c_int32],
        "tt_debug_fail_allocations": [_int],
        "tt_transform_extended": [_P, _F, _int, _int, _F, _int, _I32, _int,
                                  ctypes.POINTER(PFunctionalC), _int, _I32, _int, _F, _F, _F,
                                  _F, _I32],
    }
    for name, args in sig.items():
        fn = getattr(l, name)
        fn.argtypes = args
        fn.restype = st
    l.tt_last_error.restype = ctypes.c_char_p
    l.tt_last_error.argtypes = []
    l.tt_version.restype = ctypes.c_char_p
    l.tt_version.argtypes = []
    _lib = l
    return l


def check(status: int) -> None:
    if status != TT_OK:
        msg = lib().tt_last_error().decode(errors="replace")
        if status == 1:
            raise InvalidArgument(status, msg)
        raise TTError(status, msg)


def fptr(a):
    return a.ctypes.data_as(_F)


def iptr(a):
    return a.ctypes.data_as(_I32)
