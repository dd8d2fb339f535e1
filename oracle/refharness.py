"""ORACLE — test infrastructure only.

Runs the reference's own CUDA kernels (cubins built by oracle/build_ref.py from the reference
checkout) through oracle/ref_harness.cpp, starting from an ``OracleState``'s arrays, which it
updates in place. Needs a GPU.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_ref
from . import OcState, OracleState

_lib = None


def available_grids():
    return [(X, Y, Z) for (X, Y, Z, _v) in build_ref.GRIDS if os.path.exists(build_ref.cubin_path(X, Y, Z))]


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build_ref.build_harness())
        L.rh_run.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.POINTER(OcState),
                             ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.rh_run.restype = ctypes.c_int
        L.rh_stage.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.POINTER(OcState),
                               ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_int)]
        L.rh_stage.restype = ctypes.c_int
        L.rh_neighbours.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.POINTER(OcState),
                                    ctypes.POINTER(ctypes.c_uint8)]
        L.rh_neighbours.restype = ctypes.c_int
        L.rh_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def run_reference(st: OracleState, dt: float, speed: float, nsteps: int, pcg_tol: float = 1e-5, pcg_max: int = 200):
    """Advance ``st`` (float32) by nsteps with the reference kernels; returns diagnostics."""
    assert st.dtype == np.float32
    cub = build_ref.cubin_path(st.X, st.Y, st.Z)
    if not os.path.exists(cub):
        raise FileNotFoundError(cub)
    c = st._cstate()
    iters = (ctypes.c_int * nsteps)()
    nsub = (ctypes.c_int * (10 * nsteps))()
    rc = lib().rh_run(cub.encode(), st.X, st.Y, st.Z, st.voxel, ctypes.byref(c), dt, speed, nsteps, pcg_tol, pcg_max, iters, nsub)
    if rc != 0:
        raise RuntimeError("reference harness: " + lib().rh_last_error().decode())
    st.sim_time = c.sim_time
    return {"pcg_iters": list(iters), "nsub": [list(nsub[10 * i:10 * i + 10]) for i in range(nsteps)]}


def _cubin(st):
    assert st.dtype == np.float32
    cub = build_ref.cubin_path(st.X, st.Y, st.Z)
    if not os.path.exists(cub):
        raise FileNotFoundError(cub)
    return cub


def run_stage_reference(st: OracleState, stage: int, arg: int, dt: float, speed: float = 1.0, pcg_tol: float = 1e-5,
                        pcg_max: int = 200):
    """One stage of the reference's step (the numbering of skt_run_stage) on ``st`` (float32), in
    place; returns {"pcg_iters", "nsub"}."""
    cub = _cubin(st)
    c = st._cstate()
    diag = (ctypes.c_int * 2)()
    rc = lib().rh_stage(cub.encode(), st.X, st.Y, st.Z, st.voxel, ctypes.byref(c), stage, arg, dt, speed, pcg_tol, pcg_max, diag)
    if rc != 0:
        raise RuntimeError("reference harness: " + lib().rh_last_error().decode())
    return {"pcg_iters": diag[0], "nsub": diag[1]}


def neighbours(st: OracleState) -> np.ndarray:
    """computeNeighbourGPU's Neigh records for ``st``'s heightfield: uint8 (n, 6, 2)."""
    cub = _cubin(st)
    c = st._cstate()
    out = np.empty(st.X * st.Y * st.Z * 12, np.uint8)
    rc = lib().rh_neighbours(cub.encode(), st.X, st.Y, st.Z, st.voxel, ctypes.byref(c),
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    if rc != 0:
        raise RuntimeError("reference harness: " + lib().rh_last_error().decode())
    return out.reshape(-1, 6, 2)
