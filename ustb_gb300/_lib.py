"""ctypes binding of the in-tree CUDA library ``libustb_gb300.so``.

The library is the product's only compute path: if it is missing, importing
the compute entry points raises instead of falling back to anything else.
Signatures mirror ``include/ustb_gb300.h``.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libustb_gb300.so")

_lock = threading.Lock()
_lib = None

i32, i64, f32, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_double
vp = ctypes.c_void_p

# name -> (restype, argtypes); every exported symbol of include/ustb_gb300.h
SIGNATURES = {
    "ustb_last_error": (ctypes.c_char_p, []),
    "ustb_abi_version": (ctypes.c_int, []),
    "ustb_das_table_f32": (ctypes.c_int, [vp, i32, i64, i64, i64, i64, f32, f32, vp, vp, vp, vp,
                                          i64, f32, i32, vp, vp]),
    "ustb_das_table_f32_host": (ctypes.c_int, [vp, i32, i64, i64, i64, i64, f32, f32, vp, vp, vp,
                                               vp, i64, f32, i32, vp, i32]),
    "ustb_das_table_f32_host_noalloc": (ctypes.c_int, [vp, i32, i64, i64, i64, i64, f32, f32, vp,
                                                       vp, vp, vp, i64, f32, i32, vp, i32]),
    "ustb_apply_pixel_phase": (ctypes.c_int, [vp, i64, i64, vp, vp]),
    "ustb_das_fast": (ctypes.c_int, [vp, i32, i32, i64, i64, i64, i64, vp, i32, i32, vp, vp, vp]),
    "ustb_das_fast_batch": (ctypes.c_int, [vp, i32, vp, vp]),
    "ustb_entries_bytes": (i64, [i64, i64, i64, i64, i32]),
    "ustb_build_entries": (ctypes.c_int, [vp, i32, i32, i64, i64, i64, i64, vp, vp]),
    "ustb_das_fast_entries": (ctypes.c_int, [vp, i32, i64, i64, i64, i64, vp, i32, i32, vp, vp, vp]),
    "ustb_das_fast_workspace_bytes": (i64, [vp, i32]),
    "ustb_das_fast_batch_ws": (ctypes.c_int, [vp, i32, vp, vp, i64, vp]),
    "ustb_das_fast_batch_ex": (ctypes.c_int, [vp, i32, vp, vp, i64, i32, vp]),
    "ustb_convert_channels": (ctypes.c_int, [vp, i32, vp, i32, i64, f32, vp]),
    "ustb_plan_create": (ctypes.c_int, [vp, vp]),
    "ustb_plan_destroy": (ctypes.c_int, [vp]),
    "ustb_plan_tiles": (i64, [vp]),
    "ustb_plan_tiles_host": (i64, [vp, vp, i64]),
    "ustb_plan_execute": (ctypes.c_int, [vp, vp, vp, vp, vp]),
    "ustb_serve_create": (ctypes.c_int, [i64, i32, i64, vp]),
    "ustb_serve_create_ex": (ctypes.c_int, [i64, i32, i64, i32, vp]),
    "ustb_serve_submit": (ctypes.c_int, [vp, vp, vp, vp, vp]),
    "ustb_serve_wait": (ctypes.c_int, [vp, ctypes.c_uint64, i32, vp]),
    "ustb_serve_destroy": (ctypes.c_int, [vp]),
    "ustb_demodulate": (ctypes.c_int, [vp, i32, vp, i32, i64, i64, f64, f64, f64, i32, vp, i32, f32, vp]),
    "ustb_demodulate_filtfilt": (ctypes.c_int, [vp, i32, vp, i32, i64, i64, f64, f64, f64, i32, vp, i32, f32, vp]),
    "ustb_scan_convert": (ctypes.c_int, [vp, i32, i32, i64, i64, i64, vp, vp, vp, vp, i64, i64, f32, f32, f32, f32,
                                         vp]),
    "ustb_phase_coherence": (ctypes.c_int, [vp, i64, i64, i64, vp, f32, f32, vp, vp, vp, vp]),
    "ustb_generalized_coherence": (ctypes.c_int, [vp, i64, i64, i64, i32, vp, vp, vp]),
    "ustb_capon": (ctypes.c_int, [vp, vp, i64, i64, i64, i64, f32, i32, f32, f32, i32, vp, vp]),
    "ustb_coherence_factor": (ctypes.c_int, [vp, i64, i64, i64, i64, i32, vp, vp, vp, vp]),
    "ustb_fir_depth": (ctypes.c_int, [vp, vp, i64, i64, vp, i32, i32, vp]),
}

STATUS = {0: "USTB_OK", 1: "USTB_E_ARG", 2: "USTB_E_SHAPE", 3: "USTB_E_DTYPE", 4: "USTB_E_CUDA",
          5: "USTB_E_OOM", 6: "USTB_E_TIMEOUT", 7: "USTB_E_OVERFLOW", 8: "USTB_E_BUSY"}


class UstbError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code


def lib():
    """Load (once) and return the CUDA library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.isfile(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build it with `python -m ustb_gb300.build` "
                    "(the GB300 beamformer has no CPU fallback)")
            h = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(h, name)
                fn.restype = res
                fn.argtypes = args
            _lib = h
    return _lib


def check(rc: int) -> None:
    if rc != 0:
        msg = lib().ustb_last_error()
        raise UstbError(rc, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
