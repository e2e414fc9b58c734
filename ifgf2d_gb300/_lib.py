"""ctypes binding of libifgf2d.so (declared in include/ifgf2d.h).

The library is built in-tree (ifgf2d_gb300/_build/libifgf2d.so).  There is no CPU fallback:
if the library cannot be built or loaded, importing the bindings raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

IFGF2D_OK = 0
STATUS = {
    0: "OK", 1: "ERR_ARG", 2: "ERR_GEOMETRY", 3: "ERR_NEIGHBORHOOD", 4: "ERR_NLEVELS",
    5: "ERR_CUDA", 6: "ERR_STATE", 7: "ERR_NONFINITE", 8: "ERR_NOCONV",
}
APPLY_DIRECT, APPLY_IFGF, APPLY_IFGF_MIXED = 0, 1, 2
PRECOND_NET, PRECOND_SPECTRAL = 1, 2
SPECTRAL_DEFAULT_SCALE = 0.25   # IFGF2D_SPECTRAL_DEFAULT_SCALE
CURVE_CIRCLE, CURVE_KITE, CURVE_LINE, CURVE_STAR = 0, 1, 2, 3

# every symbol include/ifgf2d.h declares
EXPORTS = [
    "ifgf2d_create", "ifgf2d_destroy", "ifgf2d_last_error", "ifgf2d_num_unknowns", "ifgf2d_num_patches",
    "ifgf2d_get_points", "ifgf2d_get_patches", "ifgf2d_get_near_singular", "ifgf2d_precompute",
    "ifgf2d_get_precomputations", "ifgf2d_setup", "ifgf2d_get_nlevels", "ifgf2d_get_sorting", "ifgf2d_apply",
    "ifgf2d_apply_device", "ifgf2d_ifgf_far", "ifgf2d_solve", "ifgf2d_propagate", "ifgf2d_hankel",
    "ifgf2d_stream", "ifgf2d_work_counts", "ifgf2d_last_refinements", "ifgf2d_apply_timed", "ifgf2d_measure_fp64_peak",
    "ifgf2d_apply_direct_noalloc", "ifgf2d_apply_batch", "ifgf2d_apply_batch_device", "ifgf2d_solve_batch",
    "ifgf2d_set_host_threads", "ifgf2d_prepare", "ifgf2d_net_num_params", "ifgf2d_net_create", "ifgf2d_net_destroy",
    "ifgf2d_net_last_error", "ifgf2d_net_get_params", "ifgf2d_net_set_params", "ifgf2d_net_gradient",
    "ifgf2d_net_train_step", "ifgf2d_net_apply", "ifgf2d_get_geometry_features", "ifgf2d_solve_precond",
    "ifgf2d_tuning_size", "ifgf2d_autotune", "ifgf2d_get_tuning", "ifgf2d_set_tuning", "ifgf2d_eval_offsurface_setup", "ifgf2d_eval_offsurface", "ifgf2d_eval_offsurface_counts",
    "ifgf2d_group_create", "ifgf2d_group_destroy", "ifgf2d_group_last_error", "ifgf2d_group_num_unknowns",
    "ifgf2d_group_offsets", "ifgf2d_group_apply", "ifgf2d_group_solve",
    "ifgf2d_spectral_setup", "ifgf2d_spectral_apply", "ifgf2d_solve_flexible", "ifgf2d_solve_batch_flexible",
    "ifgf2d_group_solve_flexible", "ifgf2d_spectral_symbol", "ifgf2d_net_set_output_weighting",
    "ifgf2d_net_output_weighting",
]


class Curve(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("closed", ctypes.c_int), ("tlim1", ctypes.c_double),
                ("tlim2", ctypes.c_double), ("params", ctypes.c_double * 16)]


class Junction(ctypes.Structure):
    _fields_ = [("curve", ctypes.c_int), ("touching_curve", ctypes.c_int), ("t1_touches_t1", ctypes.c_int)]


class Options(ctypes.Structure):
    _fields_ = [("Np", ctypes.c_int), ("delta", ctypes.c_double), ("wavelengths_per_patch", ctypes.c_double),
                ("patch_split_wavenumber", ctypes.c_double), ("p", ctypes.c_double),
                ("patches_per_curve", ctypes.c_int), ("Ps", ctypes.c_int), ("Pang", ctypes.c_int),
                ("formulation", ctypes.c_int), ("coupling", ctypes.c_double), ("device_geometry", ctypes.c_int)]
SINGLE_LAYER, COMBINED = 0, 2


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libifgf2d.so, building it first if needed (raises when that is impossible)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"libifgf2d.so not found at {path}; build it with ifgf2d_gb300/build.py")
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        I64 = ctypes.POINTER(ctypes.c_longlong)
        L.ifgf2d_create.argtypes = [ctypes.POINTER(Curve), ctypes.c_int, ctypes.POINTER(Junction), ctypes.c_int,
                                    ctypes.POINTER(Options), ctypes.POINTER(P)]
        L.ifgf2d_destroy.argtypes = [P]
        L.ifgf2d_last_error.argtypes = [P]; L.ifgf2d_last_error.restype = ctypes.c_char_p
        L.ifgf2d_num_unknowns.argtypes = [P]; L.ifgf2d_num_unknowns.restype = ctypes.c_longlong
        L.ifgf2d_num_patches.argtypes = [P]; L.ifgf2d_num_patches.restype = ctypes.c_longlong
        L.ifgf2d_get_points.argtypes = [P, D, D, D, D]
        L.ifgf2d_get_patches.argtypes = [P, D, I64]
        L.ifgf2d_get_near_singular.argtypes = [P, I64, D]
        L.ifgf2d_precompute.argtypes = [P, ctypes.c_double]
        L.ifgf2d_get_precomputations.argtypes = [P, ctypes.c_longlong, D]
        L.ifgf2d_setup.argtypes = [P, ctypes.c_double, ctypes.c_int]
        L.ifgf2d_get_nlevels.argtypes = [P]
        L.ifgf2d_get_sorting.argtypes = [P, I64]
        L.ifgf2d_apply.argtypes = [P, D, D, ctypes.c_int]
        L.ifgf2d_apply_device.argtypes = [P, P, P, ctypes.c_int]
        L.ifgf2d_ifgf_far.argtypes = [P, D, D]
        L.ifgf2d_solve.argtypes = [P, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int), D]
        L.ifgf2d_propagate.argtypes = [P, ctypes.c_longlong, D, D, D, D]
        L.ifgf2d_hankel.argtypes = [ctypes.c_int, ctypes.c_longlong, D, D]
        L.ifgf2d_stream.argtypes = [P]; L.ifgf2d_stream.restype = ctypes.c_void_p
        L.ifgf2d_work_counts.argtypes = [P, I64]
        L.ifgf2d_last_refinements.argtypes = [P]
        L.ifgf2d_apply_timed.argtypes = [P, P, P, ctypes.c_int, D]
        L.ifgf2d_measure_fp64_peak.argtypes = [D]
        L.ifgf2d_apply_direct_noalloc.argtypes = [P, P, P]
        L.ifgf2d_set_host_threads.argtypes = [ctypes.c_int]
        L.ifgf2d_prepare.argtypes = [P, ctypes.c_double, ctypes.c_int]
        F = ctypes.POINTER(ctypes.c_float)
        IP = ctypes.POINTER(ctypes.c_int)
        L.ifgf2d_net_num_params.restype = ctypes.c_longlong
        L.ifgf2d_net_create.argtypes = [ctypes.c_ulonglong, ctypes.POINTER(P)]
        L.ifgf2d_net_destroy.argtypes = [P]
        L.ifgf2d_net_last_error.argtypes = [P]; L.ifgf2d_net_last_error.restype = ctypes.c_char_p
        L.ifgf2d_net_get_params.argtypes = [P, F]
        L.ifgf2d_net_set_params.argtypes = [P, F]
        L.ifgf2d_net_gradient.argtypes = [P, ctypes.c_int, IP, D, D, D, D, D, F]
        L.ifgf2d_net_train_step.argtypes = [P, ctypes.c_int, IP, D, D, D, D, ctypes.c_float, ctypes.c_float, D]
        L.ifgf2d_net_apply.argtypes = [P, ctypes.c_int, IP, D, D, D, D, F]
        L.ifgf2d_get_geometry_features.argtypes = [P, D]
        L.ifgf2d_autotune.argtypes = [P, ctypes.c_int, IP]
        L.ifgf2d_get_tuning.argtypes = [P, IP]
        L.ifgf2d_set_tuning.argtypes = [P, IP]
        L.ifgf2d_solve_precond.argtypes = [P, P, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int), D]
        L.ifgf2d_spectral_setup.argtypes = [P, ctypes.c_double]
        L.ifgf2d_spectral_apply.argtypes = [P, D, D]
        L.ifgf2d_spectral_symbol.argtypes = [P, ctypes.c_int, D, D]
        L.ifgf2d_net_set_output_weighting.argtypes = [P, ctypes.c_int]
        L.ifgf2d_net_output_weighting.argtypes = [P]
        L.ifgf2d_solve_flexible.argtypes = [P, P, ctypes.c_int, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int), D]
        L.ifgf2d_group_solve_flexible.argtypes = [P, ctypes.c_int, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_int), D]
        L.ifgf2d_solve_batch_flexible.argtypes = [P, ctypes.c_int, D, D, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                  ctypes.c_int, ctypes.POINTER(ctypes.c_int), D]
        L.ifgf2d_eval_offsurface_setup.argtypes = [P, ctypes.c_longlong, D, D]
        L.ifgf2d_eval_offsurface.argtypes = [P, D, D]
        L.ifgf2d_eval_offsurface_counts.argtypes = [P, I64]
        L.ifgf2d_apply_batch.argtypes = [P, D, D, ctypes.c_int, ctypes.c_int]
        L.ifgf2d_apply_batch_device.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int]
        L.ifgf2d_solve_batch.argtypes = [P, D, D, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int), D]
        L.ifgf2d_group_create.argtypes = [ctypes.POINTER(P), ctypes.c_int, ctypes.POINTER(P)]
        L.ifgf2d_group_destroy.argtypes = [P]
        L.ifgf2d_group_last_error.argtypes = [P]; L.ifgf2d_group_last_error.restype = ctypes.c_char_p
        L.ifgf2d_group_num_unknowns.argtypes = [P]; L.ifgf2d_group_num_unknowns.restype = ctypes.c_longlong
        L.ifgf2d_group_offsets.argtypes = [P, I64]
        L.ifgf2d_group_apply.argtypes = [P, D, D, ctypes.c_int]
        L.ifgf2d_group_solve.argtypes = [P, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int), D]
        _lib = L
        return L
