"""Shared helpers of the parity tests: state transfer between the oracle and the GPU
environment, and the error measures."""
import numpy as np

import oracle
from skewtcloudsim_gb300 import Environment, SolverConfig, FIELDS, GROUND_FIELDS, COLUMNS, sounding

SKY = ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p", "rho")
GROUND = ("Qrs", "Qgr", "Qgs", "Qgi", "Pg", "tg", "Tg")


def small_case(shape=(32, 32, 32), name="plain-64x64x32", seed=None):
    """(x, y, z) with z vertical, as the workloads are named."""
    init, dt, speed = sounding.workload(name, seed=seed, scale=shape)
    return init, dt, speed


def oracle_cfg(sem=0, **kw):
    return oracle.Config(semantics=sem, **kw)


def gpu_cfg(sem=0, **kw):
    return SolverConfig(semantics=sem, **kw)


def make_env(init, cfg=None, noise=True):
    env = Environment(init.nx, init.ny, init.nz, init.voxel, cfg or SolverConfig())
    env.init_from(init, noise=noise)
    return env


def push_oracle_to_env(st: oracle.OracleState, env: Environment):
    for k in SKY:
        env.write(k, st.a[k].astype(np.float32))
    for k in GROUND:
        env.write(k, st.a[k].astype(np.float32))
    for k in COLUMNS:
        if k in st.a:  # the oracle holds no copy of the init pressure column
            env.write(k, st.a[k].astype(np.float32))
    env.set_clock(st.sim_time, st.day, st.longitude, st.sun, st.pause)


def rel_l2(a, b, mask):
    a = a[mask].astype(np.float64)
    b = b[mask].astype(np.float64)
    nb = np.linalg.norm(b)
    d = np.linalg.norm(a - b)
    if nb == 0.0:
        return 0.0 if d == 0.0 else np.inf
    return d / nb


def rel_max(a, b, mask):
    a = a[mask].astype(np.float64)
    b = b[mask].astype(np.float64)
    s = np.max(np.abs(b))
    d = np.max(np.abs(a - b)) if a.size else 0.0
    if s == 0.0:
        return 0.0 if d == 0.0 else np.inf
    return d / s


def compare(env: Environment, st: oracle.OracleState, names=SKY, ground=GROUND):
    m = st.sky_mask()
    out = {}
    for k in names:
        out[k] = (rel_l2(env.read(k), st.a[k], m), rel_max(env.read(k), st.a[k], m))
    full = np.ones(st.X * st.Z, bool)
    for k in ground:
        out[k] = (rel_l2(env.read(k), st.a[k], full), rel_max(env.read(k), st.a[k], full))
    return out
