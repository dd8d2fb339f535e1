"""Correctness bars beyond per-field parity: the water budget and the projection's residual.

Water. The model's water lives in the six sky mixing ratios (qv, qw, qc, qr, qs, qi) and the
four ground stores (Qrs, Qgr, Qgs, Qgi), all in kg/kg of the cell above the ground, and every
transfer between them moves the same number out of one and into another: the microphysics
(Game/microPhysics.cu:1319-1353) within a cell, sedimentation (Game/kernelSky.cu:576-657) down a
column, precipitation reaching the ground (Game/microPhysics.cu:1544-1636) and the ground
processes (:1419-1542) between the first sky cell and the stores. Water leaves only through the
lateral boundaries (Dirichlet or default-column faces of diffusion and advection), by
sedimentation out of the lowest sky cell, and by the advection's density companion differing from
one. The bars (sums in FP64 over the FP32 fields):
* microphysics: every cell's total is unchanged within 2e-6 relative (FP32 rounding of the
  species updates);
* sedimentation: with the two lowest sky cells empty (one substep moves water one cell), every
  column's total is unchanged within 1e-6 relative;
* ground stage: the sum over the grid of the first sky cells' qv, qr, qs, qi and the ground stores
  is unchanged within 1e-6 relative;
* whole steps: W = sum of all sky mixing ratios and ground stores changes by at most 2e-5 of
  itself over 10 steps of the 32^3 plain workload with condensate in the middle of the domain
  (measured: the FP64 oracle's W changes by +2.0e-6, the FP32 oracle's by -7.5e-6, the difference
  being the FP32 rounding of the vapour field's small diffusion and advection increments), and the
  GPU's W agrees with the FP32 oracle's within 1e-6 of W after every step.

Projection. The projection solves A p = r (r the divergence of calculateDivergenceGPU, A the
matrix of initAMatrix; Game/kernelSky.cu:780-860,1320-1393). The velocity correction that follows
(applyPresProjGPU) divides by face densities that A does not use, so the divergence recomputed
after it is not the solver's residual; the bar is the residual of the system itself: for the
pressure correction the GPU leaves (the third debug field), max |r - A p| evaluated by the oracle
in FP64 over A and r built in FP32 from the same state must lie below the PCG tolerance 1e-5, in
the mixed-precision mode and in the plain textbook mode run to convergence; the mixed mode also
holds the relative L2 residual below 1e-6 (refine_tol 1e-8 before the solution is rounded to FP32).
"""
import copy

import numpy as np
import pytest

import oracle
from helpers import GROUND, make_env, oracle_cfg, push_oracle_to_env, small_case
from skewtcloudsim_gb300 import SolverConfig

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 32)
MOIST = ("qv", "qw", "qc", "qr", "qs", "qi")
STORES = ("Qrs", "Qgr", "Qgs", "Qgi")


def _clone(st):
    c = copy.copy(st)
    c.a = {k: v.copy() for k, v in st.a.items()}
    c.gh = st.gh.copy()
    return c


@pytest.fixture(scope="module")
def developed():
    init, dt, speed = small_case(SHAPE)
    st = oracle.OracleState(init, np.float32)
    st.step(oracle_cfg(), dt, speed)
    return init, dt, speed, st


def _blob(st, lo_y=3, hi_y=12, seed=7):
    """Condensate of every species in a cylinder in the middle of the domain, from row lo_y up."""
    X, Y, Z = st.X, st.Y, st.Z
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    blob = ((((x - X // 2) ** 2 + (z - Z // 2) ** 2) < 36) & (y >= lo_y) & (y < hi_y)).reshape(-1)
    rng = np.random.default_rng(seed)
    for k, s in (("qw", 2e-3), ("qc", 1e-3), ("qr", 1e-3), ("qs", 5e-4), ("qi", 5e-4)):
        st.a[k][:] = 0.0
        st.a[k][blob] = rng.uniform(0, s, blob.sum()).astype(np.float32)
    rng2 = np.random.default_rng(seed + 1)
    for k in ("Qgr", "Qgs", "Qgi"):
        st.a[k][:] = rng2.uniform(0, 5e-4, st.a[k].size).astype(np.float32)


def _cell_total(get, m):
    return sum(get(k).astype(np.float64) for k in MOIST)[m]


def test_microphysics_conserves_water_per_cell(gpu_lib, developed):
    init, dt, speed, st0 = developed
    st = _clone(st0)
    _blob(st)
    m = st.sky_mask()
    before = _cell_total(lambda k: st.a[k], m)
    env = make_env(init)
    push_oracle_to_env(st, env)
    env.run_stage(4, 0, dt, speed)
    after_gpu = _cell_total(env.read, m)
    env.close()
    st.stage(oracle_cfg(), 4, 0, dt, speed)
    after_orc = _cell_total(lambda k: st.a[k], m)
    for after in (after_gpu, after_orc):
        rel = np.abs(after - before) / np.maximum(before, 1e-30)
        assert rel.max() <= 2e-6, rel.max()


@pytest.mark.parametrize("ptype", [0, 1, 2])
def test_sedimentation_conserves_water_per_column(gpu_lib, developed, ptype):
    init, dt, speed, st0 = developed
    st = _clone(st0)
    _blob(st, lo_y=3)  # rows 1 and 2 (the lowest sky cells) hold no condensate
    name = ["qr", "qs", "qi"][ptype]
    X, Y, Z = st.X, st.Y, st.Z
    col = lambda a: a.astype(np.float64).reshape(Z, Y, X).sum(axis=1)
    field0 = st.a[name].copy()
    before = col(field0)
    env = make_env(init)
    push_oracle_to_env(st, env)
    env.run_stage(5, ptype, dt * speed)
    field_gpu = env.read(name)
    after_gpu = col(field_gpu)
    env.close()
    st.stage(oracle_cfg(), 5, ptype, dt * speed)
    after_orc = col(st.a[name])
    scale = max(before.max(), 1e-30)
    assert np.abs(field_gpu.astype(np.float64) - field0).max() > 0.0  # the species did fall
    assert np.abs(after_gpu - before).max() <= 1e-6 * scale
    assert np.abs(after_orc - before).max() <= 1e-6 * scale
    assert np.abs(after_gpu - after_orc).max() <= 1e-6 * scale


def test_ground_stage_conserves_water(gpu_lib, developed):
    init, dt, speed, st0 = developed
    st = _clone(st0)
    _blob(st, lo_y=1)  # condensate down to the first sky cell, so precipitation reaches the ground
    X, Y, Z = st.X, st.Y, st.Z

    def total(get):
        first = lambda k: get(k).astype(np.float64).reshape(Z, Y, X)[:, 1, :].sum()  # flat ground: row 1
        return sum(first(k) for k in ("qv", "qr", "qs", "qi")) + sum(get(k).astype(np.float64).sum() for k in STORES)

    before = total(lambda k: st.a[k])
    env = make_env(init)
    push_oracle_to_env(st, env)
    env.run_stage(6, 0, dt, speed)
    after_gpu = total(env.read)
    moved = np.abs(env.read("Qgr").astype(np.float64) - st.a["Qgr"]).sum()
    env.close()
    st.stage(oracle_cfg(), 6, 0, dt, speed)
    after_orc = total(lambda k: st.a[k])
    assert moved > 0.0  # precipitation did reach the ground
    assert abs(after_gpu - before) <= 1e-6 * before, (after_gpu, before)
    assert abs(after_orc - before) <= 1e-6 * before, (after_orc, before)


def test_whole_step_water_budget(gpu_lib, developed):
    init, dt, speed, st0 = developed
    st = _clone(st0)
    _blob(st)
    m = st.sky_mask()

    def W(get):
        return sum(get(k).astype(np.float64)[m].sum() for k in MOIST) + sum(get(k).astype(np.float64).sum() for k in STORES)

    w0 = W(lambda k: st.a[k])
    env = make_env(init)
    push_oracle_to_env(st, env)
    for step in range(10):
        st.step(oracle_cfg(), dt, speed)
        env.update_gpu(dt, speed)
        wg, wo = W(env.read), W(lambda k: st.a[k])
        assert abs(wg - wo) <= 1e-6 * w0, (step, wg, wo)
        assert abs(wg - w0) <= 2e-5 * w0, (step, wg, w0)
    env.close()


@pytest.mark.parametrize("mode", ["mixed", "textbook"])
def test_projection_residual_below_pcg_tolerance(gpu_lib, mode):
    init, dt, speed = small_case(SHAPE)
    st = oracle.OracleState(init, np.float32)
    for _ in range(2):
        st.step(oracle_cfg(1), dt, speed)
    cfg = (SolverConfig(precision=1, refine_tol=1e-8) if mode == "mixed"
           else SolverConfig(semantics=1, pcg_tol=1e-5, pcg_max_iter=20000))
    env = make_env(init, cfg)
    push_oracle_to_env(st, env)
    env.run_stage(3, 0, dt * speed)
    assert env.stats()["converged"]
    pp = env.read("debug3")
    env.close()
    mx, l2, bmx, bl2 = st.projection_residual(oracle_cfg(1), pp, dt * speed)
    assert bmx > 1e-3  # there was a divergence to remove
    assert mx <= 1e-5, (mx, l2, bmx, bl2)
    if mode == "mixed":
        assert l2 <= 1e-6 * bl2, (mx, l2, bmx, bl2)
