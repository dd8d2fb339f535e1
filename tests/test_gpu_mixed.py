"""Mixed-precision projection (FP32 multigrid-preconditioned CG inside FP64 iterative
refinement) against the FP64 oracle of the same (textbook) method solved to a tight tolerance.

The FP64 oracle runs the projection with Jacobi-PCG in double precision until the max residual
is below 1e-13; the GPU solves the same symmetric system to a relative FP64 residual of 1e-8.
Tolerances: relative L2 <= 1e-6 on u, v, w, p, rho after one projection (v: or 1.5x the FP32
oracle's own distance on the same projection, whichever is larger); <= 1e-5 on every field
after each of three whole steps started from identical inputs, except the vertical wind v: its
FP32 rounding alone (buoyancy differences of ~300 K virtual temperatures, and v is an order of
magnitude smaller than u and w) gives ~1.4e-5, which the FP32 oracle shows too, so v must stay
within 1.5x of the FP32 oracle's own distance from the FP64 oracle.
"""
import numpy as np
import pytest

import oracle
from helpers import SKY, make_env, push_oracle_to_env, rel_l2, small_case
from skewtcloudsim_gb300 import SolverConfig

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 32)


def _to64(st32, init):
    st = oracle.OracleState(init, np.float64, noise=False)
    for k, v in st32.a.items():
        st.a[k][:] = v.astype(np.float64)
    st.gh[:] = st32.gh
    st.sim_time = st32.sim_time
    return st


def _to32(st64, init):
    st = oracle.OracleState(init, np.float32, noise=False)
    for k, v in st64.a.items():
        st.a[k][:] = v.astype(np.float32)
    st.gh[:] = st64.gh
    st.sim_time = st64.sim_time
    return st


FP64_CFG = dict(semantics=1, pcg_tol=1e-13, pcg_max_iter=20000)


@pytest.fixture(scope="module")
def developed():
    return _developed(SHAPE)


def _developed(shape):
    init, dt, speed = small_case(shape)
    st = oracle.OracleState(init, np.float32)
    for _ in range(2):
        st.step(oracle.Config(semantics=1), dt, speed)
    return init, dt, speed, st


def _check_projection(init, dt, speed, st32, cfg, max_inner=None):
    ref = _to64(st32, init)
    f32 = _to32(ref, init)  # the same projection by the FP32 oracle: v's own FP32 floor
    f32.stage(oracle.Config(semantics=1, pcg_tol=1e-9, pcg_max_iter=5000), 3, 0, dt * speed)
    env = make_env(init, cfg)
    push_oracle_to_env(st32, env)
    g = env.run_stage(3, 0, dt * speed)
    o = ref.stage(oracle.Config(**FP64_CFG), 3, 0, dt * speed)
    assert o["pcg_iters"] < 20000
    st = env.stats()
    assert st["converged"] and st["pcg_residual"] <= 1e-8, st
    assert st["outer_iters"] >= 1
    if max_inner is not None:
        assert st["pcg_iters"] <= max_inner, st
    m = ref.sky_mask()
    for k in ("u", "v", "w", "p", "rho"):
        e = rel_l2(env.read(k), ref.a[k], m)
        limit = 1e-6 if k != "v" else max(1e-6, 1.5 * rel_l2(f32.a[k], ref.a[k], m))
        assert e <= limit, (k, e, limit, g, st)
    env.close()


@pytest.mark.parametrize("mg_half", [1, 0])
def test_mixed_projection_matches_fp64(gpu_lib, developed, mg_half):
    """32^3: the fused float4 V-cycle on the finest level, FP16 or FP32 smoother coefficients."""
    init, dt, speed, st32 = developed
    _check_projection(init, dt, speed, st32, SolverConfig(precision=1, refine_tol=1e-8, mg_half=mg_half))


@pytest.mark.parametrize("shape,max_inner", [((64, 64, 32), 40), ((30, 20, 20), 60), ((36, 28, 24), 60), ((16, 16, 8), 60)])
def test_mixed_projection_hierarchies(gpu_lib, shape, max_inner):
    """64x64x32 runs two vector coarse levels; x = 30 runs the scalar finest level with the
    unfused CG; 36x28x24 a vector finest level over a coarsest level of odd x size; 16x16x8 (2048
    cells) has no coarse level, so the one-block coarsest solve preconditions the finest level
    itself and the unfused residual kernel sets the inner tolerance from its max |r|."""
    init, dt, speed, st32 = _developed(shape)
    _check_projection(init, dt, speed, st32, SolverConfig(precision=1, refine_tol=1e-8), max_inner)


def test_mixed_projection_c2_matches_fp64(gpu_lib):
    """The plain-256x256x128 workload at its full size (8.4M cells: a vector finest level and
    vector coarse levels of 128x64x128 .. 16x8x16), after one oracle step: the projection against
    the FP64 oracle solved to 1e-13 (about half a minute on 16 cores)."""
    init, dt, speed = small_case((256, 256, 128), name="plain-256x256x128")
    st = oracle.OracleState(init, np.float32)
    st.step(oracle.Config(semantics=1), dt, speed)
    _check_projection(init, dt, speed, st, SolverConfig(precision=1, refine_tol=1e-8), 60)


def test_mixed_steps_match_fp64(gpu_lib):
    init, dt, speed = small_case(SHAPE)
    ref = oracle.OracleState(init, np.float64)
    env = make_env(init, SolverConfig(precision=1, refine_tol=1e-8))
    for step in range(3):
        start = _to32(ref, init)
        push_oracle_to_env(start, env)
        f32 = _to32(ref, init)
        f32.step(oracle.Config(semantics=1, pcg_tol=1e-9, pcg_max_iter=5000), dt, speed)
        ref.step(oracle.Config(**FP64_CFG), dt, speed)
        env.update_gpu(dt, speed)
        assert env.stats()["converged"]
        m = ref.sky_mask()
        bad = {}
        for k in SKY:
            e = rel_l2(env.read(k), ref.a[k], m)
            limit = 1e-5 if k != "v" else max(1e-5, 1.5 * rel_l2(f32.a[k], ref.a[k], m))
            if e > limit:
                bad[k] = (e, limit)
        assert not bad, (step, bad)
    env.close()


def test_mixed_rejects_odd_grids(gpu_lib):
    from skewtcloudsim_gb300 import Environment, SktError
    with pytest.raises(SktError):
        Environment(33, 33, 33, 100.0, SolverConfig(precision=1))
