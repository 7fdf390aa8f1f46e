"""ctypes binding of libswe_gpu.so (include/swe_gpu.h).

This is the binding a Python caller of the C ABI writes (a Fortran caller
binds the same symbols through iso_c_binding).  Loading fails loudly when the
library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

FIELD_H32 = 16
SWE_OK, SWE_ERR_NEG_H, SWE_ERR_DELTA, SWE_ERR_NAN, SWE_ERR_TIMEOUT, SWE_ERR_CUDA, SWE_ERR_ARG, SWE_ERR_MESH = range(8)
ERROR_NAMES = {1: "NEG_H", 2: "DELTA", 3: "NAN", 4: "TIMEOUT", 5: "CUDA", 6: "ARG", 7: "MESH"}


class swe_params(ctypes.Structure):
    _fields_ = [
        ("gravity", ctypes.c_double), ("dt", ctypes.c_double), ("cfl", ctypes.c_double),
        ("htiny", ctypes.c_double), ("mannings", ctypes.c_double), ("lambda_sgn", ctypes.c_double),
        ("max_water_h", ctypes.c_double),
        ("type_test", ctypes.c_int), ("syst_size", ctypes.c_int), ("viscosity_type", ctypes.c_int),
        ("viscous_type", ctypes.c_int), ("if_alpha_limit", ctypes.c_int), ("if_lumped", ctypes.c_int),
        ("if_roundoff_fix", ctypes.c_int), ("precision", ctypes.c_int),
    ]


# every symbol include/swe_gpu.h declares
EXPORTS = [
    "swe_create", "swe_create_batch", "swe_destroy", "swe_last_error", "swe_set_params", "swe_set_bath",
    "swe_set_dirichlet",
    "swe_sizes", "swe_get_matrices", "swe_compute_dij", "swe_euler", "swe_euler_intermediates",
    "swe_fct_positivity", "swe_fct_generic", "swe_gauss_points", "swe_norms", "swe_upload", "swe_download", "swe_upload_device", "swe_download_device",
    "swe_set_time", "swe_rk3_steps", "swe_mass", "swe_last_launch_count", "swe_tuning",
    "swe_last_device_ms", "swe_profile_kernels", "swe_fct_positivity_noalloc", "swe_autotune",
    "swe_write_vtk_2d", "swe_frame_fields", "swe_frame_async", "swe_frames_wait", "swe_gauges_set",
    "swe_gauges_read", "swe_get_time", "swe_set_tuning", "swe_set_dirichlet_anal",
    "swe_rk3_steps_host",
]
NOALLOC_MAX_NODES = 1 << 20   # SWE_NOALLOC_MAX_NODES
KERNEL_KINDS = ("dt", "node", "low", "fct", "update")

_lib = None


class SweError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"SWE_ERR_{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


def library_path() -> Path:
    return _build.LIB


def load(build: bool = True):
    """Load (building first if needed) the native library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not Path(path).exists():
        raise OSError(f"native library {path} is missing; run the build")
    L = ctypes.CDLL(str(path))
    vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    pp = ctypes.POINTER(swe_params)
    sig = {
        "swe_create": ([ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ip, dp, dp, pp], ctypes.c_int),
        "swe_create_batch": ([ctypes.POINTER(vp), ctypes.c_int, ip, ip, ip, dp, dp, pp], ctypes.c_int),
        "swe_destroy": ([vp], None),
        "swe_last_error": ([vp], ctypes.c_char_p),
        "swe_set_params": ([vp, ctypes.c_int, pp], ctypes.c_int),
        "swe_set_bath": ([vp, ctypes.c_int, dp], ctypes.c_int),
        "swe_set_dirichlet": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, dp], ctypes.c_int),
        "swe_set_dirichlet_anal": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip], ctypes.c_int),
        "swe_sizes": ([vp, ctypes.c_int, ip, ip], ctypes.c_int),
        "swe_get_matrices": ([vp, ctypes.c_int, ip, ip, dp, dp, ip, dp, dp], ctypes.c_int),
        "swe_compute_dij": ([vp, ctypes.c_int, dp, dp, dp], ctypes.c_int),
        "swe_euler": ([vp, ctypes.c_int, dp, dp], ctypes.c_int),
        "swe_euler_intermediates": ([vp, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp], ctypes.c_int),
        "swe_fct_positivity": ([vp, ctypes.c_int, dp, dp, dp], ctypes.c_int),
        "swe_fct_generic": ([vp, ctypes.c_int, dp, dp, dp, dp, dp], ctypes.c_int),
        "swe_gauss_points": ([vp, ctypes.c_int, dp, dp], ctypes.c_int),
        "swe_norms": ([vp, ctypes.c_int, ctypes.c_int, dp, dp, dp], ctypes.c_int),
        "swe_upload": ([vp, dp], ctypes.c_int),
        "swe_download": ([vp, dp], ctypes.c_int),
        "swe_upload_device": ([vp, ctypes.c_void_p], ctypes.c_int),
        "swe_download_device": ([vp, ctypes.c_void_p], ctypes.c_int),
        "swe_set_time": ([vp, dp, dp], ctypes.c_int),
        "swe_get_time": ([vp, dp, dp, dp], ctypes.c_int),
        "swe_rk3_steps": ([vp, ctypes.c_int, dp, dp, ip], ctypes.c_int),
        "swe_rk3_steps_host": ([vp, dp, dp, ctypes.c_int, dp, dp, ip], ctypes.c_int),
        "swe_mass": ([vp, dp], ctypes.c_int),
        "swe_last_launch_count": ([vp], ctypes.c_longlong),
        "swe_tuning": ([vp], ctypes.c_char_p),
        "swe_last_device_ms": ([vp], ctypes.c_double),
        "swe_autotune": ([vp], ctypes.c_int),
        "swe_set_tuning": ([vp, ctypes.c_char_p], ctypes.c_int),
        "swe_profile_kernels": ([vp, ctypes.c_int, dp], ctypes.c_int),
        "swe_fct_positivity_noalloc": ([ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p],
                                       ctypes.c_int),
        "swe_write_vtk_2d": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ip, dp, dp],
                             ctypes.c_int),
        "swe_frame_fields": ([vp, ctypes.c_int, ctypes.c_double, dp, dp], ctypes.c_int),
        "swe_frame_async": ([vp, ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_char_p], ctypes.c_int),
        "swe_frames_wait": ([vp], ctypes.c_int),
        "swe_gauges_set": ([vp, ctypes.c_int, ip, dp, ip], ctypes.c_int),
        "swe_gauges_read": ([vp, ctypes.c_int, dp, ip, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None else None
