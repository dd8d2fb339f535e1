"""ctypes binding of libskewt_gb300.so (the C ABI declared in include/skewt.h).

The library is required: there is no CPU fallback. ``load()`` raises if the in-tree build is
missing (call ``skewtcloudsim_gb300.build.build()`` first).
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

c_float_p = ctypes.POINTER(ctypes.c_float)


class GridDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("voxel", ctypes.c_float)]


class SolverCfg(ctypes.Structure):
    _fields_ = [("semantics", ctypes.c_int), ("diffuse_sweeps", ctypes.c_int), ("pcg_tol", ctypes.c_float),
                ("pcg_max_iter", ctypes.c_int), ("max_substeps", ctypes.c_int), ("precision", ctypes.c_int),
                ("refine_tol", ctypes.c_float), ("inner_max_iter", ctypes.c_int), ("inner_rtol", ctypes.c_float),
                ("use_graph", ctypes.c_int), ("mg_half", ctypes.c_int), ("pcg_fused", ctypes.c_int)]


class Sounding(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("altitude", c_float_p), ("pressure", c_float_p), ("temperature", c_float_p),
                ("dew_point", c_float_p), ("wind_speed", c_float_p), ("wind_dir", c_float_p)]


# long long (*)(void* ctx, const char* name, char* buf, size_t cap)
ARCHIVE_READ_FN = ctypes.CFUNCTYPE(ctypes.c_longlong, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t)


class StepStats(ctypes.Structure):
    _fields_ = [("pcg_iters", ctypes.c_int), ("pcg_residual", ctypes.c_float), ("pcg_converged", ctypes.c_int),
                ("nsub", ctypes.c_int * 10), ("outer_iters", ctypes.c_int), ("sim_time", ctypes.c_double),
                ("kernel_launches", ctypes.c_longlong), ("gpu_ms", ctypes.c_float)]


# every symbol include/skewt.h declares, with its ctypes signature
SIGNATURES = {
    "skt_default_config": (None, [ctypes.POINTER(SolverCfg)]),
    "skt_create": (ctypes.c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(SolverCfg), ctypes.POINTER(ctypes.c_void_p)]),
    "skt_destroy": (None, [ctypes.c_void_p]),
    "skt_init": (ctypes.c_int, [ctypes.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p,
                                c_float_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_uint32, ctypes.c_uint32]),
    "skt_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_int]),
    "skt_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "skt_step_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_int]),
    "skt_step_ensemble": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, c_float_p, ctypes.c_float, c_float_p,
                                         ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "skt_read_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_float_p, ctypes.c_size_t]),
    "skt_read_fields_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(c_float_p), ctypes.c_size_t]),
    "skt_read_wait": (ctypes.c_int, [ctypes.c_void_p]),
    "skt_write_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_float_p, ctypes.c_size_t]),
    "skt_field_device_ptr": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(c_float_p)]),
    "skt_read_ground": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p, ctypes.c_size_t]),
    "skt_write_ground": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p, ctypes.c_size_t]),
    "skt_read_column": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p, ctypes.c_size_t]),
    "skt_write_column": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p, ctypes.c_size_t]),
    "skt_set_clock": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_int]),
    "skt_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StepStats)]),
    "skt_run_stage": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                     ctypes.POINTER(StepStats)]),
    "skt_profile_enable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "skt_profile_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "skt_diffuse_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                           ctypes.c_float, ctypes.c_int, c_float_p, c_float_p,
                                           ctypes.POINTER(ctypes.c_int32), c_float_p, c_float_p, c_float_p, c_float_p,
                                           ctypes.c_void_p]),
    "skt_set_rate_region": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int)]),
    "skt_read_rates": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_size_t]),
    "skt_set_diagnostics": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "skt_apply_brush": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.POINTER(ctypes.c_int), ctypes.c_float,
                                       ctypes.c_float, ctypes.c_float, ctypes.c_float, c_float_p, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int)]),
    "skt_apply_selection": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                           ctypes.c_float, c_float_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "skt_reset_parameter": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "skt_read_ground_height": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_size_t]),
    "skt_read_neighbours": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t]),
    "skt_sounding_read_knmi": (ctypes.c_int, [ARCHIVE_READ_FN, ctypes.c_void_p, ctypes.POINTER(Sounding)]),
    "skt_sounding_read_dwd": (ctypes.c_int, [ctypes.c_char_p, ARCHIVE_READ_FN, ctypes.c_void_p, ctypes.POINTER(Sounding)]),
    "skt_sounding_free": (None, [ctypes.POINTER(Sounding)]),
    "skt_sounding_to_init": (ctypes.c_int, [ctypes.POINTER(Sounding), ctypes.POINTER(GridDesc), c_float_p, c_float_p,
                                            c_float_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "skt_view_volume": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_int), c_float_p, ctypes.POINTER(ctypes.c_uint8),
                                       ctypes.c_size_t]),
    "skt_export_bricks": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_int, ctypes.POINTER(ctypes.c_uint32), ctypes.c_void_p, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_size_t)]),
    "skt_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "skt_version": (ctypes.c_char_p, []),
}

class Tuning(ctypes.Structure):
    _fields_ = [("diffuse_depth", ctypes.c_int), ("diffuse_rows", ctypes.c_int), ("diffuse_bps", ctypes.c_int),
                ("diffuse2_bps", ctypes.c_int), ("ppm_x_bps", ctypes.c_int), ("ppm_y_bps", ctypes.c_int),
                ("ppm_z_bps", ctypes.c_int), ("from_cache", ctypes.c_int), ("diffuse_ms", ctypes.c_float),
                ("advect_ms", ctypes.c_float)]


SIGNATURES.update({
    "skt_get_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tuning)]),
    "skt_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tuning)]),
    "skt_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(Tuning)]),
    "skt_ensemble_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "skt_ensemble_destroy": (None, [ctypes.c_void_p]),
    "skt_ensemble_step": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_float, c_float_p, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int)]),
})

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(path: str | None = None):
    """Load the library (once). Raises FileNotFoundError when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or lib_path()
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is missing: build it with skewtcloudsim_gb300.build.build() "
                                "(there is no CPU fallback)")
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L
