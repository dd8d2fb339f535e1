"""Python mirror of the reference's ``environmentGPU`` (Game/environment.cuh:9-183).

Same operations, names and argument meaning as the reference class: ``init`` takes the host
arrays of environmentGPU::init (Game/environment.cu:249), ``update_gpu(dt, speed)`` is
environmentGPU::updateGPU (:391), ``get_param_array(parameter, direction)`` returns the device
pointer of a field (:1076). Field readback, which the reference does every step through
editor::GPUSetEnv (Game/editor.cpp:226-260), is explicit here (``read``). Every call goes
through the C ABI of libskewt_gb300; errors raise ``SktError`` carrying the skt_status.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from enum import IntEnum
from typing import Optional

import numpy as np

from . import _lib


class Status(IntEnum):
    OK = 0
    INVALID_ARG = 1
    CUDA_ERROR = 2
    NOT_CONVERGED = 3
    NAN_DETECTED = 4
    TIMEOUT = 5
    OUT_OF_MEMORY = 6
    NOT_INITIALIZED = 7
    COURANT_LIMIT = 8


class Parameter(IntEnum):  # Game/config.h:62-65
    POTTEMP = 0
    QV = 1
    QW = 2
    QC = 3
    QR = 4
    QS = 5
    QI = 6
    WIND = 7
    PGROUND = 8
    PRESSURE = 9
    DEBUG1 = 10
    DEBUG2 = 11
    DEBUG3 = 12
    DENSITY = 100


class Direction(IntEnum):  # Game/config.h:36-39
    LEFT = 0
    RIGHT = 1
    UP = 2
    DOWN = 3
    FORWARD = 4
    BACKWARD = 5


class Ground(IntEnum):
    QRS = 0
    QGR = 1
    QGS = 2
    QGI = 3
    P = 4
    TIME_WET = 5
    T = 6
    CLOUD_COVER = 7


class Column(IntEnum):
    ISEN_T = 0
    ISEN_QV = 1
    DEF_U = 2
    DEF_W = 3
    PRESSURE = 4


class SktError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{Status(status).name}: {msg}")
        self.status = Status(status)


# name -> (parameter, direction) for read/write
FIELDS = {
    "th": (Parameter.POTTEMP, 0), "qv": (Parameter.QV, 0), "qw": (Parameter.QW, 0), "qc": (Parameter.QC, 0),
    "qr": (Parameter.QR, 0), "qs": (Parameter.QS, 0), "qi": (Parameter.QI, 0),
    "u": (Parameter.WIND, Direction.RIGHT), "v": (Parameter.WIND, Direction.UP), "w": (Parameter.WIND, Direction.FORWARD),
    "p": (Parameter.PRESSURE, 0), "rho": (Parameter.DENSITY, 0),
    # the reference's editor debug views: DEBUG1 never written (zeros), DEBUG2 the buoyancy velocity
    # change (needs set_diagnostics(DIAG_BUOYANCY)), DEBUG3 the projection's pressure correction
    "debug1": (Parameter.DEBUG1, 0), "debug2": (Parameter.DEBUG2, 0), "debug3": (Parameter.DEBUG3, 0),
}
DIAG_BUOYANCY = 1
# the 33 region-summed microphysics amounts (microPhysicsParams order, Game/microPhysics.cuh:7-21)
RATE_NAMES = ("PVCON", "PVDEP", "PIMLT", "PIDW", "PIHOM", "PIACR", "PRACI", "PRAUT", "PRACW", "PREVP", "PRACS", "PSACW",
              "PSACR", "PSACI", "PSAUT", "PSFW", "PSFI", "PSDEP", "PSSUB", "PSMLT", "PGAUT", "PGFR", "PGACW", "PGACI",
              "PGACR", "PGDRY", "PGACS", "PGSUB", "PGMLT", "PGWET", "PGACR1", "PVVAP", "PVSUB")
GROUND_FIELDS = {"Qrs": Ground.QRS, "Qgr": Ground.QGR, "Qgs": Ground.QGS, "Qgi": Ground.QGI, "Pg": Ground.P,
                 "tg": Ground.TIME_WET, "Tg": Ground.T, "cover": Ground.CLOUD_COVER}
COLUMNS = {"isenT": Column.ISEN_T, "isenQv": Column.ISEN_QV, "defU": Column.DEF_U, "defW": Column.DEF_W,
           "pcol": Column.PRESSURE}


@dataclass
class SolverConfig:
    semantics: int = 0          # 0 reference quirks, 1 textbook
    diffuse_sweeps: int = 20
    pcg_tol: float = 1e-5
    pcg_max_iter: int = 200
    max_substeps: int = 100
    precision: int = 0          # 0 plain, 1 mixed
    refine_tol: float = 1e-8
    inner_max_iter: int = 60
    inner_rtol: float = 1e-4
    use_graph: int = 0          # 1: each step is one launch of a captured CUDA graph
    mg_half: int = 1            # mixed: FP16 finest-level coefficients inside the V-cycle
    pcg_fused: int = 1          # plain: search step and pressure update fused into the operator

    def c(self):
        return _lib.SolverCfg(self.semantics, self.diffuse_sweeps, self.pcg_tol, self.pcg_max_iter, self.max_substeps,
                              self.precision, self.refine_tol, self.inner_max_iter, self.inner_rtol, self.use_graph,
                              self.mg_half, self.pcg_fused)


def _fp(a):
    return a.ctypes.data_as(_lib.c_float_p)


class Environment:
    """One simulated atmosphere on the current CUDA device."""

    def __init__(self, nx: int, ny: int, nz: int, voxel: float, cfg: Optional[SolverConfig] = None):
        self._L = _lib.load()
        self.nx, self.ny, self.nz, self.voxel = nx, ny, nz, float(voxel)
        self.n = nx * ny * nz
        self.ng = nx * nz
        self.cfg = cfg or SolverConfig()
        g = _lib.GridDesc(nx, ny, nz, self.voxel)
        c = self.cfg.c()
        h = ctypes.c_void_p()
        st = self._L.skt_create(ctypes.byref(g), ctypes.byref(c), ctypes.byref(h))
        if st != 0:
            raise SktError(st, self._L.skt_last_error(None).decode())
        self._h = h
        self._clock = dict(day=130, longitude=52.37, sun=1.0, pause=0)

    # -- lifetime --------------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.skt_destroy(self._h)  # waits for pending readback copies first
            self._h = None
        self._pending_reads = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, allow=()):
        if st != 0 and st not in allow:
            raise SktError(st, self._L.skt_last_error(self._h).decode())
        return Status(st)

    # -- environmentGPU API ----------------------------------------------------------------
    def init(self, theta, vel_aos, qv, ground_T, ground_p, p3d, p_column, ground_height, noise=True, noise_seed=100):
        """environmentGPU::init (Game/environment.cu:249-389)."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in (theta, vel_aos, qv, ground_T, ground_p, p3d, p_column)]
        gh = np.ascontiguousarray(ground_height, np.int32)
        self._gh = gh.copy()
        st = self._L.skt_init(self._h, *[_fp(a) for a in arrs], gh.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                              1 if noise else 0, noise_seed)
        self._check(st)

    def init_from(self, state, noise=True, noise_seed=100):
        """init() from a ``sounding.InitialState``."""
        self.init(state.theta, state.vel, state.qv, state.ground_T, state.ground_p, state.p3d, state.p_column,
                  state.ground_height, noise=noise, noise_seed=noise_seed)

    def update_gpu(self, dt: float, speed: float = 1.0, nsteps: int = 1) -> Status:
        """environmentGPU::updateGPU (Game/environment.cu:391-555); NOT_CONVERGED is returned, not raised."""
        return self._check(self._L.skt_step(self._h, dt, speed, nsteps), allow=(Status.NOT_CONVERGED,))

    def update_gpu_async(self, dt: float, speed: float = 1.0, nsteps: int = 1) -> Status:
        """skt_step_async: queues the steps (graph mode) and returns; sync() collects them."""
        return self._check(self._L.skt_step_async(self._h, dt, speed, nsteps), allow=(Status.NOT_CONVERGED,))

    def sync(self) -> Status:
        """skt_sync: waits; after update_gpu_async, the queued steps' status (NOT_CONVERGED is returned, not raised)."""
        return self._check(self._L.skt_sync(self._h), allow=(Status.NOT_CONVERGED,))

    def get_param_array(self, parameter: int, direction: int = Direction.RIGHT) -> int:
        """environmentGPU::getParamArray: device address of the field (int)."""
        p = _lib.c_float_p()
        self._check(self._L.skt_field_device_ptr(self._h, int(parameter), int(direction), ctypes.byref(p)))
        return ctypes.cast(p, ctypes.c_void_p).value

    # -- readback / injection --------------------------------------------------------------
    def read(self, name: str) -> np.ndarray:
        if name in FIELDS:
            prm, d = FIELDS[name]
            out = np.empty(self.n, np.float32)
            self._check(self._L.skt_read_field(self._h, int(prm), int(d), _fp(out), out.size))
        elif name in GROUND_FIELDS:
            out = np.empty(self.ng, np.float32)
            self._check(self._L.skt_read_ground(self._h, int(GROUND_FIELDS[name]), _fp(out), out.size))
        elif name in COLUMNS:
            out = np.empty(self.ny, np.float32)
            self._check(self._L.skt_read_column(self._h, int(COLUMNS[name]), _fp(out), out.size))
        else:
            raise KeyError(name)
        return out

    def read_async(self, outs: dict):
        """skt_read_fields_async: queue the readback of the fields named in ``outs`` (name -> float32
        array of n values, ideally pinned) as they stand after the queued work; returns at once.
        The arrays of every call are kept alive here until ``read_wait``."""
        names = list(outs)
        prm = (ctypes.c_int * len(names))(*[int(FIELDS[k][0]) for k in names])
        drs = (ctypes.c_int * len(names))(*[int(FIELDS[k][1]) for k in names])
        for k in names:
            a = outs[k]
            if a.dtype != np.float32 or a.size != self.n or not a.flags.c_contiguous:
                raise ValueError(f"{k}: need a contiguous float32 array of {self.n} values")
        dst = (_lib.c_float_p * len(names))(*[_fp(outs[k]) for k in names])
        if getattr(self, "_pending_reads", None) is None:
            self._pending_reads = []
        self._pending_reads.append(outs)  # the device may still write them after this call returns
        self._check(self._L.skt_read_fields_async(self._h, len(names), prm, drs, dst, self.n))

    def read_wait(self):
        self._check(self._L.skt_read_wait(self._h))
        self._pending_reads = None

    def write(self, name: str, a):
        a = np.ascontiguousarray(a, np.float32)
        if name in FIELDS:
            prm, d = FIELDS[name]
            self._check(self._L.skt_write_field(self._h, int(prm), int(d), _fp(a), a.size))
        elif name in GROUND_FIELDS:
            self._check(self._L.skt_write_ground(self._h, int(GROUND_FIELDS[name]), _fp(a), a.size))
        elif name in COLUMNS:
            self._check(self._L.skt_write_column(self._h, int(COLUMNS[name]), _fp(a), a.size))
        else:
            raise KeyError(name)

    # -- diagnostics (the reference's data graph and debug views) ----------------------------
    def set_rate_region(self, lo=None, hi=None, enable: bool = True):
        """Sum the microphysics process amounts over lo <= (x, y, z) <= hi (reference layout, y
        vertical, inclusive) every step; enable=False turns it off."""
        lo3 = (ctypes.c_int * 3)(*(lo or (0, 0, 0)))
        hi3 = (ctypes.c_int * 3)(*(hi or (self.nx - 1, self.ny - 1, self.nz - 1)))
        self._check(self._L.skt_set_rate_region(self._h, 1 if enable else 0, lo3, hi3))

    def read_rates(self) -> dict:
        out = np.empty(len(RATE_NAMES), np.float32)
        self._check(self._L.skt_read_rates(self._h, _fp(out), out.size))
        return dict(zip(RATE_NAMES, out.tolist()))

    def set_diagnostics(self, flags: int):
        self._check(self._L.skt_set_diagnostics(self._h, int(flags)))

    def set_clock(self, sim_time=43200.0, day=130, longitude=52.37, sun=1.0, pause=0):
        self._check(self._L.skt_set_clock(self._h, sim_time, day, longitude, sun, pause))
        self._clock = dict(day=day, longitude=longitude, sun=sun, pause=pause)

    # -- headless view, volume export, checkpoints (skewtcloudsim_gb300.volume) ----------------
    def view(self, sky: int = Parameter.POTTEMP, ground: int = -1, lo=None, hi=None):
        """The editor's voxel view: (rgb (n, 3) float32, kind (n,) uint8); see volume.view_volume."""
        from . import volume
        return volume.view_volume(self, sky, ground, lo, hi)

    def export_bricks(self, name: str, threshold: float = 0.0, background: float = 0.0, half: bool = False):
        from . import volume
        return volume.export_bricks(self, name, threshold, background, half)

    def save_checkpoint(self, path):
        from . import volume
        volume.save_checkpoint(self, path)

    def stats(self) -> dict:
        s = _lib.StepStats()
        self._check(self._L.skt_stats(self._h, ctypes.byref(s)))
        return {"pcg_iters": s.pcg_iters, "pcg_residual": s.pcg_residual, "converged": bool(s.pcg_converged),
                "nsub": list(s.nsub), "outer_iters": s.outer_iters, "sim_time": s.sim_time,
                "kernel_launches": s.kernel_launches, "gpu_ms": s.gpu_ms}

    def profile(self, on: bool = True):
        self._check(self._L.skt_profile_enable(self._h, 1 if on else 0))

    def profile_read(self) -> dict:
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._L.skt_profile_read(self._h, buf, len(buf)))
        return {k: {"ms": v[0], "kernels": v[1], "scopes": v[2]} for k, v in json.loads(buf.value.decode()).items()}

    def run_stage(self, stage: int, arg: int = 0, dt: float = 0.5, speed: float = 1.0) -> dict:
        s = _lib.StepStats()
        self._check(self._L.skt_run_stage(self._h, stage, arg, dt, speed, ctypes.byref(s)))
        return {"pcg_iters": s.pcg_iters, "pcg_residual": s.pcg_residual, "converged": bool(s.pcg_converged),
                "nsub": s.nsub[0]}

    def sky_mask(self, ground_height=None) -> np.ndarray:
        gh = self.read_ground_height() if ground_height is None else np.asarray(ground_height)
        y = np.arange(self.ny)[None, :, None]
        return (y > gh.reshape(self.nz, self.nx)[:, None, :]).reshape(-1)

    def read_ground_height(self):
        out = np.empty(self.ng, np.int32)
        self._check(self._L.skt_read_ground_height(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), out.size))
        return out

    # -- launch-shape tuning ---------------------------------------------------------------------
    TUNING_FIELDS = ("diffuse_depth", "diffuse_rows", "diffuse_bps", "diffuse2_bps", "ppm_x_bps", "ppm_y_bps", "ppm_z_bps")

    def get_tuning(self) -> dict:
        t = _lib.Tuning()
        self._check(self._L.skt_get_tuning(self._h, ctypes.byref(t)))
        return {k: getattr(t, k) for k in self.TUNING_FIELDS}

    def set_tuning(self, **kw):
        """Changes some launch shapes (keys of get_tuning()); the others stay."""
        cur = self.get_tuning()
        unknown = set(kw) - set(cur)
        if unknown:
            raise ValueError(f"unknown tuning keys {sorted(unknown)}")
        cur.update(kw)
        t = _lib.Tuning(*[int(cur[k]) for k in self.TUNING_FIELDS])
        self._check(self._L.skt_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, cache_path=None, force=False) -> dict:
        """skt_autotune: the launch shapes for this grid, from the cache file or measured."""
        t = _lib.Tuning()
        path = os.fsencode(cache_path) if cache_path else None
        self._check(self._L.skt_autotune(self._h, path, 1 if force else 0, ctypes.byref(t)))
        d = {k: getattr(t, k) for k in self.TUNING_FIELDS}
        d.update(from_cache=bool(t.from_cache), diffuse_ms=t.diffuse_ms, advect_ms=t.advect_ms)
        return d

    def read_neighbours(self) -> np.ndarray:
        """The Neigh records of every cell (computeNeighbourGPU's layout): uint8 (n, 6, 2) of
        (outside, type) for left, right, up, down, forward, backward; type 1 = ground."""
        out = np.empty(self.n * 12, np.uint8)
        self._check(self._L.skt_read_neighbours(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), self.n))
        return out.reshape(self.n, 6, 2)

    # -- editing between steps (the reference's editor tools) -------------------------------
    def apply_brush(self, param, size, pos, smoothness, dt, intensity, value, direction=(1.0, 0.0, 0.0), erase=False) -> bool:
        """prepareBrushGPU: returns whether the heightfield changed."""
        ch = ctypes.c_int(0)
        d = np.asarray(direction, np.float32)
        self._check(self._L.skt_apply_brush(self._h, int(param), size, (ctypes.c_int * 3)(*pos), smoothness, dt, intensity, value,
                                            _fp(d), int(erase), ctypes.byref(ch)))
        return bool(ch.value)

    def apply_selection(self, param, lo, hi, value, direction=(1.0, 0.0, 0.0), erase=False) -> bool:
        """prepareSelectionGPU: returns whether the heightfield changed."""
        ch = ctypes.c_int(0)
        d = np.asarray(direction, np.float32)
        self._check(self._L.skt_apply_selection(self._h, int(param), (ctypes.c_int * 3)(*lo), (ctypes.c_int * 3)(*hi), value, _fp(d),
                                                int(erase), ctypes.byref(ch)))
        return bool(ch.value)

    def reset_parameter(self, param):
        """resetParameterGPU."""
        self._check(self._L.skt_reset_parameter(self._h, int(param)))


def step_ensemble(envs, dt, speed=1.0, nsteps: int = 1, threads: int = 0):
    """skt_step_ensemble: advance every Environment in ``envs`` by ``nsteps`` steps at once (a
    host thread per member drives its own stream). ``dt`` and ``speed`` are scalars or one value
    per member. Returns the members' statuses; raises on the first failing member."""
    L = _lib.load()
    n = len(envs)
    hs = (ctypes.c_void_p * n)(*[e._h.value if hasattr(e._h, "value") else e._h for e in envs])
    dts = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float32), (n,)))
    sps = np.ascontiguousarray(np.broadcast_to(np.asarray(speed, np.float32), (n,)))
    st = (ctypes.c_int * n)()
    rc = L.skt_step_ensemble(hs, n, _fp(dts), 0.0, _fp(sps), int(nsteps), int(threads), st)
    if rc != 0:
        raise SktError(rc, L.skt_last_error(None).decode())
    return [Status(v) for v in st]


class Ensemble:
    """skt_ensemble_*: members advanced together by one CUDA graph launch per step (every member's
    whole step an independent branch of the graph). The members must stay open while it exists."""

    def __init__(self, envs):
        self._L = _lib.load()
        self.envs = list(envs)
        n = len(self.envs)
        hs = (ctypes.c_void_p * n)(*[e._h.value if hasattr(e._h, "value") else e._h for e in self.envs])
        self._h = ctypes.c_void_p()
        rc = self._L.skt_ensemble_create(hs, n, ctypes.byref(self._h))
        if rc != 0:
            raise SktError(rc, self._L.skt_last_error(None).decode())

    def step(self, dt, speed=1.0, nsteps: int = 1):
        """Advances every member; returns their statuses, raises on the first failing member."""
        n = len(self.envs)
        dts = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float32), (n,)))
        sps = np.ascontiguousarray(np.broadcast_to(np.asarray(speed, np.float32), (n,)))
        st = (ctypes.c_int * n)()
        rc = self._L.skt_ensemble_step(self._h, _fp(dts), 0.0, _fp(sps), int(nsteps), st)
        if rc not in (0, int(Status.NOT_CONVERGED)):
            raise SktError(rc, self._L.skt_last_error(None).decode())
        return [Status(v) for v in st]

    def close(self):
        if self._h:
            self._L.skt_ensemble_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

