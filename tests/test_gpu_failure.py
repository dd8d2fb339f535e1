"""Failure detection without a GPU fault: a NaN, an Inf or a zero-density cell written into the
state through the C ABI (skt_write_field) must make skt_step return SKT_NAN_DETECTED with a
message, stop stepping after the step that met it, and leave the context usable: the same
environment, given a valid state again, steps normally. The reference has no such check (it
traps on CUDA errors only, Game/environment.cu:394-403, and carries NaNs on); the oracle shows
that each injected fault turns every sky field non-finite within one step, so a step that
returned OK here would hand back garbage.

The faults are host-side writes of ordinary float values; no kernel is made to fault, trap or
wait.
"""
import numpy as np
import pytest

import oracle
from helpers import SKY, compare, make_env, oracle_cfg, push_oracle_to_env, small_case
from skewtcloudsim_gb300 import SolverConfig, SktError
from skewtcloudsim_gb300.environment import Status

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 32)


@pytest.fixture(scope="module")
def developed():
    init, dt, speed = small_case(SHAPE)
    st = oracle.OracleState(init, np.float32)
    st.step(oracle_cfg(), dt, speed)
    return init, dt, speed, st


def _cell(st):
    return 16 + 10 * st.X + 16 * st.X * st.Y  # a sky cell mid-domain


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("field,value", [("th", np.nan), ("u", np.inf), ("v", -np.inf), ("qr", np.nan), ("p", 0.0)])
def test_injected_fault_is_reported(gpu_lib, developed, precision, field, value):
    init, dt, speed, st = developed
    env = make_env(init, SolverConfig(precision=precision))
    push_oracle_to_env(st, env)
    a = st.a[field].copy()
    a[_cell(st)] = value
    env.write(field, a)
    t0 = env.stats()["sim_time"]
    with pytest.raises(SktError) as ei:
        env.update_gpu(dt, speed, nsteps=3)
    assert ei.value.status == Status.NAN_DETECTED, ei.value
    assert "NaN or Inf" in str(ei.value)
    # the call stopped after the first step
    assert env.stats()["sim_time"] == pytest.approx(t0 + dt * speed)
    # the context is usable and the status was cleared: a valid state steps normally and matches
    # the oracle's step from the same state
    push_oracle_to_env(st, env)
    ref = oracle.OracleState(init, np.float32, noise=False)
    for k, v in st.a.items():
        ref.a[k][:] = v
    ref.gh[:] = st.gh
    ref.sim_time = st.sim_time
    status = env.update_gpu(dt, speed)
    assert status in (Status.OK, Status.NOT_CONVERGED)
    if precision == 0:
        ref.step(oracle_cfg(), dt, speed)
        res = compare(env, ref, names=SKY, ground=())
        bad = {k: v for k, v in res.items() if v[0] > 1e-5}
        assert not bad, bad
    else:
        for k in SKY:
            assert np.isfinite(env.read(k)[env.sky_mask()]).all(), k
    env.close()


def test_projection_stage_reports_zero_density(gpu_lib, developed):
    """The projection alone (skt_run_stage) on a state whose density is zero in one sky cell:
    the build divides by that density, and the solver's dot products turn non-finite."""
    init, dt, speed, st = developed
    env = make_env(init)
    push_oracle_to_env(st, env)
    p = st.a["p"].copy()
    p[_cell(st)] = 0.0
    env.write("p", p)
    with pytest.raises(SktError) as ei:
        env.run_stage(3, 0, dt * speed)
    assert ei.value.status == Status.NAN_DETECTED, ei.value
    env.close()
