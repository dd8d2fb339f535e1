"""GPU parity on grids wide enough for the code paths of the 512-cell-wide benchmark.

The vectorised kernels put four cells of a row on each lane, so a warp covers 128 cells of x.
At x = 260 a row takes 65 lanes: two full warps and a third with one active lane. That runs what
a 32- or 64-wide grid never does: the x neighbours that cross from lane 31 of one warp to lane 0
of the next (diffusion, the fused PCG operator, the V-cycle kernels), the interior warp-boundary
flux of the PPM x pass, and the right-edge lane falling in a later warp. The vertical size 48
gives three 16-row blocks and two PPM y runs of 26 rows; the horizontal z size 32 gives several
z runs per column. The state is the precision-512x512x256 workload's sounding (five bubbles,
westerly shear), scaled to this grid and developed for two steps, with a wind of both signs
injected for the advection stages.

The stage and step tolerances are those of test_gpu_parity.py: stages max-norm relative 2e-5 on
sky cells, whole steps relative L2 1e-5 per field, Courant substep counts equal, PCG iteration
counts within one. The mixed-precision projection is held to 1e-6 of the FP64 oracle solved to
1e-13, as in test_gpu_mixed.py.
"""
import copy

import numpy as np
import pytest

import oracle
from helpers import GROUND, compare, gpu_cfg, make_env, oracle_cfg, push_oracle_to_env, rel_l2, small_case

pytestmark = pytest.mark.gpu

WIDE = (260, 32, 48)      # (x, y, z), z vertical -> reference layout X=260, Y=48, Z=32
WIDE_MG = (264, 32, 48)   # halves to 33x6x4: the mixed solve's hierarchy exists
WORKLOAD = "precision-512x512x256"
STAGE_TOL = 2e-5
STEP_TOL = 1e-5


def _clone(st):
    c = copy.copy(st)
    c.a = {k: v.copy() for k, v in st.a.items()}
    c.gh = st.gh.copy()
    return c


def _developed(shape, sem=0):
    init, dt, speed = small_case(shape, name=WORKLOAD)
    st = oracle.OracleState(init, np.float32)
    for _ in range(2):
        st.step(oracle_cfg(sem), dt, speed)
    return init, dt, speed, st


@pytest.fixture(scope="module")
def developed():
    return _developed(WIDE)


def _swirl(st, amp=6.0):
    """Winds of both signs in every direction, up to `amp` m/s, on sky cells (MAC faces)."""
    X, Y, Z = st.X, st.Y, st.Z
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    m = st.sky_mask()
    u = amp * np.sin(2 * np.pi * x / 37.0) * np.cos(2 * np.pi * z / 11.0)
    v = 0.5 * amp * np.sin(2 * np.pi * y / 13.0) * np.sin(2 * np.pi * x / 29.0)
    w = -amp * np.cos(2 * np.pi * z / 9.0) * np.sin(2 * np.pi * x / 53.0)
    for k, a in (("u", u), ("v", v), ("w", w)):
        st.a[k][m] = a.reshape(-1)[m].astype(np.float32)


def _stage(init, st0, stage, arg, dt, speed=None, sem=0, mutate=None):
    st = _clone(st0)
    if mutate:
        mutate(st)
    env = make_env(init, gpu_cfg(sem))
    push_oracle_to_env(st, env)
    if speed is None:
        g = env.run_stage(stage, arg, dt)
        o = st.stage(oracle_cfg(sem), stage, arg, dt)
    else:
        g = env.run_stage(stage, arg, dt, speed)
        o = st.stage(oracle_cfg(sem), stage, arg, dt, speed)
    return env, st, g, o


@pytest.mark.parametrize("ftype", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("dts", [None, 2.0e5])
def test_wide_diffusion_stage(gpu_lib, developed, ftype, dts):
    """All six boundary types; at dt*speed = 2e5 s (k = 0.1) every neighbour term matters."""
    init, dt, speed, st0 = developed
    env, st, _, _ = _stage(init, st0, 0, ftype, dts if dts else dt * speed)
    name = ["th", "qv", "u", "v", "w", "qw"][ftype]
    l2, mx = compare(env, st, names=(name,), ground=())[name]
    env.close()
    assert mx <= STAGE_TOL, (name, l2, mx)


@pytest.mark.parametrize("field", [0, 1, 2, 3, 4, 5])
def test_wide_advection_stage(gpu_lib, developed, field):
    """Every PPM pass with winds of both signs, at dt*speed = 25 s (Courant numbers above 1, so
    several substeps)."""
    init, dt, speed, st0 = developed
    env, st, g, o = _stage(init, st0, 1, field, 25.0, mutate=_swirl)
    name = ["th", "u", "v", "w", "qv", "qw"][field]
    l2, mx = compare(env, st, names=(name,), ground=())[name]
    env.close()
    assert g["nsub"] == o["nsub"] and o["nsub"] > 1, (g, o)
    assert mx <= STAGE_TOL, (name, l2, mx)


def test_wide_buoyancy_stage(gpu_lib, developed):
    init, dt, speed, st0 = developed
    env, st, _, _ = _stage(init, st0, 2, 0, dt * speed)
    l2, mx = compare(env, st, names=("v",), ground=())["v"]
    env.close()
    assert mx <= STAGE_TOL, (l2, mx)


@pytest.mark.parametrize("sem", [0, 1])
def test_wide_projection_stage(gpu_lib, developed, sem):
    init, dt, speed, st0 = developed
    env, st, g, o = _stage(init, st0, 3, 0, dt * speed, sem=sem, mutate=_swirl)
    res = compare(env, st, names=("u", "v", "w", "p", "rho"), ground=())
    env.close()
    assert abs(g["pcg_iters"] - o["pcg_iters"]) <= 1, (g, o)
    for k, (l2, mx) in res.items():
        assert l2 <= STEP_TOL, (k, l2, mx)


def _condensate(st):
    rng = np.random.default_rng(7)
    m = st.sky_mask()
    for k, s in (("qw", 2e-3), ("qc", 1e-3), ("qr", 1e-3), ("qs", 5e-4), ("qi", 5e-4)):
        st.a[k][m] = rng.uniform(0, s, m.sum()).astype(np.float32)


def test_wide_microphysics_stage(gpu_lib, developed):
    init, dt, speed, st0 = developed
    env, st, _, _ = _stage(init, st0, 4, 0, dt, speed, mutate=_condensate)
    res = compare(env, st, names=("th", "qv", "qw", "qc", "qr", "qs", "qi"), ground=())
    env.close()
    for k, (l2, mx) in res.items():
        assert mx <= 1e-4 and l2 <= STEP_TOL, (k, l2, mx)


@pytest.mark.parametrize("ptype", [0, 1, 2])
def test_wide_sedimentation_stage(gpu_lib, developed, ptype):
    init, dt, speed, st0 = developed
    env, st, _, _ = _stage(init, st0, 5, ptype, dt * speed, mutate=_condensate)
    name = ["qr", "qs", "qi"][ptype]
    l2, mx = compare(env, st, names=(name,), ground=())[name]
    env.close()
    assert mx <= STAGE_TOL, (l2, mx)


def test_wide_ground_stage(gpu_lib, developed):
    init, dt, speed, st0 = developed
    env, st, _, _ = _stage(init, st0, 6, 0, dt, speed, mutate=_condensate)
    res = compare(env, st, names=("th", "qv", "qr", "qs", "qi"), ground=GROUND)
    env.close()
    for k, (l2, mx) in res.items():
        assert mx <= 1e-4 and l2 <= STEP_TOL, (k, l2, mx)


@pytest.mark.parametrize("sem", [0, 1])
def test_wide_full_step_parity(gpu_lib, sem):
    """Two whole steps, each from the oracle's state: relative L2 <= 1e-5 on every field."""
    init, dt, speed = small_case(WIDE, name=WORKLOAD)
    st = oracle.OracleState(init, np.float32)
    env = make_env(init, gpu_cfg(sem))
    cfg = oracle_cfg(sem)
    for step in range(2):
        od = st.step(cfg, dt, speed)
        env.update_gpu(dt, speed)
        gd = env.stats()
        assert gd["nsub"] == od["nsub"], (step, gd, od)
        assert abs(gd["pcg_iters"] - od["pcg_iters"]) <= 1, (step, gd, od)
        res = compare(env, st)
        bad = {k: v for k, v in res.items() if v[0] > STEP_TOL}
        assert not bad, (step, bad)
        push_oracle_to_env(st, env)
    env.close()


def test_wide_mixed_projection_matches_fp64(gpu_lib):
    """The mixed-precision projection at x = 264 (finest rows of 66 lanes, coarse levels of 132,
    66 and 33 cells) against the FP64 oracle of the same textbook system."""
    from test_gpu_mixed import _check_projection, _developed as mixed_developed
    init, dt, speed, st32 = mixed_developed(WIDE_MG)
    _check_projection(init, dt, speed, st32, gpu_cfg(1, precision=1, refine_tol=1e-8), 60)


def test_c2_one_step(gpu_lib):
    """One whole step of the plain-256x256x128 workload at full size (8.4M cells; the oracle
    takes about a minute on 16 cores): relative L2 <= 1e-5 on every field, equal substep counts,
    PCG iteration counts within one."""
    init, dt, speed = small_case((256, 256, 128), name="plain-256x256x128")
    st = oracle.OracleState(init, np.float32)
    env = make_env(init)
    od = st.step(oracle_cfg(), dt, speed)
    env.update_gpu(dt, speed)
    gd = env.stats()
    res = compare(env, st)
    env.close()
    assert gd["nsub"] == od["nsub"], (gd, od)
    assert abs(gd["pcg_iters"] - od["pcg_iters"]) <= 1, (gd, od)
    bad = {k: v for k, v in res.items() if v[0] > STEP_TOL}
    assert not bad, bad


def test_c3_one_step_benchmarked_configuration(gpu_lib):
    """One whole step of the precision-512x512x256 workload at its full size (67.1M cells), in the
    configuration the benchmark runs (the step as one graph launch, two-sweep diffusion passes of
    14-row tiles with 4 blocks per SM, the tuned PPM run lengths) against the oracle on the host
    cores (about a minute on 16 cores): relative L2 <= 1e-5 on every field, equal substep counts,
    PCG iteration counts within one."""
    from skewtcloudsim_gb300 import SolverConfig
    init, dt, speed = small_case((512, 512, 256), name=WORKLOAD)
    env = make_env(init, SolverConfig(use_graph=1))
    env.set_tuning(diffuse_depth=2, diffuse_rows=14, diffuse2_bps=4, ppm_x_bps=8, ppm_y_bps=32, ppm_z_bps=8)
    env.update_gpu(dt, speed)
    gd = env.stats()
    st = oracle.OracleState(init, np.float32)
    od = st.step(oracle_cfg(), dt, speed)
    res = compare(env, st)
    env.close()
    assert gd["nsub"] == od["nsub"], (gd, od)
    assert abs(gd["pcg_iters"] - od["pcg_iters"]) <= 1, (gd, od)
    bad = {k: v for k, v in res.items() if v[0] > STEP_TOL}
    assert not bad, bad
