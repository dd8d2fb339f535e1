"""ORACLE — test infrastructure only.

CPU restatement of skewTCloudSim's atmosphere step (skt_oracle.cpp), loaded through ctypes.
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this module; the
product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libskt_oracle.so")

SKY_FIELDS = ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p", "rho")
GROUND_FIELDS = ("Qrs", "Qgr", "Qgs", "Qgi", "Pg", "tg", "Tg")
COLUMN_FIELDS = ("isenT", "isenQv", "defU", "defW")


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-ffp-contract=off so x86 and Arm give the same bits)."""
    src = os.path.join(HERE, "skt_oracle.cpp")
    hdr = os.path.join(HERE, "skt_oracle_physics.hpp")
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    newest = max(os.path.getmtime(src), os.path.getmtime(hdr))
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class OcConfig(ctypes.Structure):
    _fields_ = [("semantics", ctypes.c_int), ("diffuse_sweeps", ctypes.c_int), ("pcg_tol", ctypes.c_float),
                ("pcg_max_iter", ctypes.c_int), ("max_substeps", ctypes.c_int), ("voxel", ctypes.c_float)]


class OcState(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_void_p) for n in SKY_FIELDS + GROUND_FIELDS + COLUMN_FIELDS] +
                [("gh", ctypes.c_void_p), ("sim_time", ctypes.c_double), ("day", ctypes.c_int),
                 ("longitude", ctypes.c_float), ("sun", ctypes.c_float), ("pause", ctypes.c_int)])


class OcDiag(ctypes.Structure):
    _fields_ = [("pcg_iters", ctypes.c_int), ("pcg_residual", ctypes.c_double),
                ("nsub", ctypes.c_int * 10), ("converged", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        for suf in ("f32", "f64"):
            f = getattr(L, f"oc_step_{suf}")
            f.argtypes = [ctypes.POINTER(OcConfig), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                          ctypes.POINTER(OcState), ctypes.c_float, ctypes.c_float, ctypes.POINTER(OcDiag)]
            f.restype = ctypes.c_int
            g = getattr(L, f"oc_init_{suf}")
            g.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OcState), ctypes.c_int]
            g.restype = ctypes.c_int
        for suf in ("f32", "f64"):
            f = getattr(L, f"oc_stage_{suf}")
            f.argtypes = [ctypes.POINTER(OcConfig), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                          ctypes.POINTER(OcState), ctypes.c_int, ctypes.c_int, ctypes.c_float,
                          ctypes.c_float, ctypes.POINTER(OcDiag)]
            f.restype = ctypes.c_int
        L.oc_micro_rates_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OcState), ctypes.c_float,
                                         ctypes.c_float, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
        L.oc_micro_rates_f32.restype = ctypes.c_int
        L.oc_buoyancy_dbg_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OcState), ctypes.c_float,
                                          ctypes.POINTER(ctypes.c_float)]
        L.oc_buoyancy_dbg_f32.restype = ctypes.c_int
        FP, IP = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
        L.oc_brush_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OcState), ctypes.c_int, ctypes.c_float, IP,
                                   ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, FP, ctypes.c_int, FP]
        L.oc_brush_f32.restype = ctypes.c_int
        L.oc_selection_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OcState), ctypes.c_int, IP, IP,
                                       ctypes.c_float, FP, ctypes.c_int, FP]
        L.oc_selection_f32.restype = ctypes.c_int
        L.oc_reset_parameter_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OcState), ctypes.c_int, FP]
        L.oc_reset_parameter_f32.restype = ctypes.c_int
        L.oc_editor_block_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OcState)]
        L.oc_editor_block_f32.restype = ctypes.c_int
        L.oc_projection_residual_f32.argtypes = [ctypes.POINTER(OcConfig), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(OcState), FP, ctypes.c_float, ctypes.POINTER(ctypes.c_double)]
        L.oc_projection_residual_f32.restype = ctypes.c_int
        L.oc_irradiance.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_float]
        L.oc_irradiance.restype = ctypes.c_float
        L.oc_num_threads.restype = ctypes.c_int
        L.oc_set_threads.argtypes = [ctypes.c_int]
        L.oc_set_threads.restype = None
        _lib = L
    return _lib


@dataclass
class Config:
    semantics: int = 0          # 0 reference, 1 textbook
    diffuse_sweeps: int = 20
    pcg_tol: float = 1e-5
    pcg_max_iter: int = 200
    max_substeps: int = 100

    def c(self, voxel):
        return OcConfig(self.semantics, self.diffuse_sweeps, self.pcg_tol, self.pcg_max_iter,
                        self.max_substeps, voxel)


class OracleState:
    """All prognostic arrays of one environment, in float32 or float64."""

    def __init__(self, init, dtype=np.float32, noise: bool = True):
        self.dtype = np.dtype(dtype)
        self.X, self.Y, self.Z = init.nx, init.ny, init.nz
        self.voxel = init.voxel
        n, ng = self.X * self.Y * self.Z, self.X * self.Z
        vel = init.vel.reshape(n, 3)
        a = {}
        a["th"] = init.theta.astype(dtype).copy()
        a["qv"] = init.qv.astype(dtype).copy()
        for k in ("qw", "qc", "qr", "qs", "qi", "rho"):
            a[k] = np.zeros(n, dtype)
        a["u"] = vel[:, 0].astype(dtype).copy()
        a["v"] = vel[:, 1].astype(dtype).copy()
        a["w"] = vel[:, 2].astype(dtype).copy()
        a["p"] = init.p3d.astype(dtype).copy()
        a["Qrs"] = np.full(ng, 0.001, dtype)
        for k in ("Qgr", "Qgs", "Qgi", "tg"):
            a[k] = np.zeros(ng, dtype)
        a["Pg"] = init.ground_p.astype(dtype).copy()
        a["Tg"] = init.ground_T.astype(dtype).copy()
        for k in COLUMN_FIELDS:
            a[k] = np.zeros(self.Y, dtype)
        self.a = a
        self.gh = np.ascontiguousarray(init.ground_height, np.int32).copy()
        self.sim_time = 43200.0
        self.day, self.longitude, self.sun, self.pause = 130, 52.37, 1.0, 0
        # the reference's m_groundChanged after the init pass: set by ground edits, it runs
        # editorDataGPU's ground block after the edit and at the start of the next step
        self.ground_changed = False
        st = self._cstate()
        fn = lib().oc_init_f32 if self.dtype == np.float32 else lib().oc_init_f64
        fn(self.X, self.Y, self.Z, ctypes.byref(st), int(noise))

    def _cstate(self):
        st = OcState()
        for k, v in self.a.items():
            setattr(st, k, v.ctypes.data)
        st.gh = self.gh.ctypes.data
        st.sim_time, st.day, st.longitude, st.sun, st.pause = self.sim_time, self.day, self.longitude, self.sun, self.pause
        return st

    def _editor_block(self):
        assert self.dtype == np.float32
        st = self._cstate()
        lib().oc_editor_block_f32(self.X, self.Y, self.Z, ctypes.byref(st))

    def step(self, cfg: Config, dt: float, speed: float = 1.0):
        if self.ground_changed:
            self._editor_block()
        st = self._cstate()
        d = OcDiag()
        fn = lib().oc_step_f32 if self.dtype == np.float32 else lib().oc_step_f64
        c = cfg.c(self.voxel)
        rc = fn(ctypes.byref(c), self.X, self.Y, self.Z, ctypes.byref(st), dt, speed, ctypes.byref(d))
        if rc != 0:
            raise RuntimeError(f"oracle step failed: {rc}")
        self.sim_time = st.sim_time
        self.ground_changed = False
        return {"pcg_iters": d.pcg_iters, "pcg_residual": d.pcg_residual, "nsub": list(d.nsub),
                "converged": bool(d.converged)}

    def stage(self, cfg: Config, stage: int, arg: int = 0, dt: float = 0.5, speed: float = 1.0):
        st = self._cstate()
        d = OcDiag()
        c = cfg.c(self.voxel)
        fn = lib().oc_stage_f32 if self.dtype == np.float32 else lib().oc_stage_f64
        rc = fn(ctypes.byref(c), self.X, self.Y, self.Z, ctypes.byref(st), stage, arg, dt, speed,
                                ctypes.byref(d))
        if rc != 0:
            raise RuntimeError(f"oracle stage failed: {rc}")
        return {"pcg_iters": d.pcg_iters, "pcg_residual": d.pcg_residual, "nsub": d.nsub[0]}

    def projection_residual(self, cfg: Config, pp, dt: float):
        """For a pressure correction ``pp`` (FP32), the residual of the projection's linear system
        built from this (FP32) state as the projection stage builds it: (max |r - A pp|,
        ||r - A pp||_2, max |r|, ||r||_2) over sky cells. The state is not changed."""
        assert self.dtype == np.float32
        st = self._cstate()
        p = np.ascontiguousarray(pp, np.float32)
        out = (ctypes.c_double * 4)()
        c = cfg.c(self.voxel)
        lib().oc_projection_residual_f32(ctypes.byref(c), self.X, self.Y, self.Z, ctypes.byref(st),
                                         p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), dt, out)
        return tuple(out[:])

    def micro_rates(self, dt: float, speed: float, lo, hi):
        """The microphysics stage (FP32 state) and the 33 region-summed process amounts."""
        assert self.dtype == np.float32
        st = self._cstate()
        reg = (ctypes.c_int * 6)(*lo, *hi)
        out = (ctypes.c_double * 33)()
        lib().oc_micro_rates_f32(self.X, self.Y, self.Z, ctypes.byref(st), dt, speed, reg, out)
        return np.array(out[:], np.float64)

    def buoyancy_debug(self, dt: float):
        """The buoyancy stage (FP32 state) and its per-cell velocity change (0 in ground cells)."""
        assert self.dtype == np.float32
        dbg = np.zeros(self.X * self.Y * self.Z, np.float32)
        st = self._cstate()
        lib().oc_buoyancy_dbg_f32(self.X, self.Y, self.Z, ctypes.byref(st), dt, dbg.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return dbg

    # -- editing (prepareBrushGPU / prepareSelectionGPU / resetParameterGPU) --------------------
    def brush(self, param, size, pos, smooth, dt, intensity, value, direction=(1.0, 0.0, 0.0), erase=False, p_column=None):
        st = self._cstate()
        pc = np.ascontiguousarray(p_column, np.float32)
        r = lib().oc_brush_f32(self.X, self.Y, self.Z, ctypes.byref(st), int(param), size, (ctypes.c_int * 3)(*pos), smooth, dt,
                               intensity, value, (ctypes.c_float * 3)(*direction), int(erase),
                               pc.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        if r < 0:
            raise ValueError("bad parameter")
        self.ground_changed |= bool(r)
        if self.ground_changed:
            self._editor_block()
        return bool(r)

    def selection(self, param, lo, hi, value, direction=(1.0, 0.0, 0.0), erase=False, p_column=None):
        st = self._cstate()
        pc = np.ascontiguousarray(p_column, np.float32)
        r = lib().oc_selection_f32(self.X, self.Y, self.Z, ctypes.byref(st), int(param), (ctypes.c_int * 3)(*lo),
                                   (ctypes.c_int * 3)(*hi), value, (ctypes.c_float * 3)(*direction), int(erase),
                                   pc.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        if r < 0:
            raise ValueError("bad parameter")
        self.ground_changed |= bool(r)
        if self.ground_changed:
            self._editor_block()
        return bool(r)

    def reset_parameter(self, param, p_column=None):
        st = self._cstate()
        pc = np.ascontiguousarray(p_column, np.float32)
        lib().oc_reset_parameter_f32(self.X, self.Y, self.Z, ctypes.byref(st), int(param), pc.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    def sky_mask(self):
        y = np.arange(self.Y)[None, :, None]
        gh = self.gh.reshape(self.Z, self.X)[:, None, :]
        return (y > gh).reshape(-1)

    def field(self, name):
        return self.a[name]
