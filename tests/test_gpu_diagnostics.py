"""Diagnostics of the step against the oracle: the region-summed microphysics process amounts
(the reference's data graph, Game/microPhysics.cu:1356-1413) and the debug fields of the
reference's editor (Game/editor.cpp:190-224).

Tolerances. Rates: each of the 33 sums within 1e-3 relative, plus an absolute floor of 1e-6 of
the largest sum (per-cell FP32 rates with CUDA vs libm transcendentals, summed in a different
order; a rate whose regime test flips in one cell moves by that cell's amount). Buoyancy change:
max-norm relative 2e-5 over sky cells, as the buoyancy stage itself. Pressure correction: the
step leaves p - pp/100 in p, so pp is recovered from p before and after to two FP32 ulps of p
(~1000 hPa) times 100.
"""
import numpy as np
import pytest

import oracle
from helpers import make_env, oracle_cfg, push_oracle_to_env, small_case
from skewtcloudsim_gb300 import DIAG_BUOYANCY, RATE_NAMES, SktError

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 32)  # (x, y, z), z vertical -> reference layout X=32, Y=32, Z=32


@pytest.fixture(scope="module")
def developed():
    init, dt, speed = small_case(SHAPE)
    st = oracle.OracleState(init, np.float32)
    for _ in range(2):
        st.step(oracle_cfg(), dt, speed)
    # condensate everywhere and a cold upper region, so both temperature regimes add to the sums
    rng = np.random.default_rng(3)
    m = st.sky_mask()
    for k, s in (("qw", 2e-3), ("qc", 1e-3), ("qr", 1e-3), ("qs", 5e-4), ("qi", 5e-4)):
        st.a[k][m] = rng.uniform(0, s, m.sum()).astype(np.float32)
    y = (np.arange(st.X * st.Y * st.Z) // st.X) % st.Y
    cold = m & (y >= st.Y // 2)
    st.a["th"][cold] -= np.float32(45.0)
    return init, dt, speed, st


def _clone(st):
    import copy
    c = copy.copy(st)
    c.a = {k: v.copy() for k, v in st.a.items()}
    c.gh = st.gh.copy()
    return c


@pytest.mark.parametrize("box", [((0, 0, 0), (31, 31, 31)), ((4, 3, 5), (20, 25, 27)), ((7, 16, 0), (7, 16, 31))])
def test_rate_region_matches_oracle(gpu_lib, developed, box):
    init, dt, speed, st0 = developed
    lo, hi = box
    ref = _clone(st0)
    want = ref.micro_rates(dt, speed, lo, hi)
    env = make_env(init)
    push_oracle_to_env(st0, env)
    env.set_rate_region(lo, hi)
    env.run_stage(4, 0, dt, speed)
    got = env.read_rates()
    env.close()
    g = np.array([got[k] for k in RATE_NAMES], np.float64)
    # the reference's unlimited PSFW of a cell at or above 0 C is NaN (it never reaches the state,
    # but enters the region sum): NaN on both sides is agreement
    np.testing.assert_array_equal(np.isnan(g), np.isnan(want))
    fin = ~np.isnan(want)
    assert np.count_nonzero(want[fin]) >= 15, want  # most processes take part
    floor = 1e-6 * np.abs(want[fin]).max()
    bad = {RATE_NAMES[i]: (g[i], want[i]) for i in np.flatnonzero(fin) if abs(g[i] - want[i]) > 1e-3 * abs(want[i]) + floor}
    assert not bad, bad


def test_rate_region_off_and_errors(gpu_lib, developed):
    init, dt, speed, st0 = developed
    env = make_env(init)
    with pytest.raises(SktError):
        env.read_rates()  # never enabled
    env.set_rate_region((0, 0, 0), (3, 3, 3))
    env.run_stage(4, 0, dt, speed)
    first = env.read_rates()
    env.set_rate_region(enable=False)
    env.run_stage(4, 0, dt, speed)
    again = env.read_rates()
    assert all(a == b or (a != a and b != b) for a, b in zip(again.values(), first.values()))  # not recomputed while off
    with pytest.raises(SktError):
        env.read("debug2")  # debug fields need set_diagnostics
    env.close()


def test_debug_fields(gpu_lib, developed):
    init, dt, speed, st0 = developed
    ref = _clone(st0)
    want = ref.buoyancy_debug(dt * speed)
    env = make_env(init)
    push_oracle_to_env(st0, env)
    env.set_diagnostics(DIAG_BUOYANCY)
    env.run_stage(2, 0, dt * speed)
    m = st0.sky_mask()
    got = env.read("debug2")
    scale = np.abs(want[m]).max()
    assert scale > 0
    assert np.abs(got[m] - want[m]).max() <= 2e-5 * scale
    np.testing.assert_array_equal(env.read("debug1"), 0.0)
    # the pressure correction of a projection
    p0 = env.read("p")
    env.run_stage(3, 0, dt * speed)
    p1 = env.read("p")
    pp = env.read("debug3")
    rec = (p0 - p1) * 100.0
    assert np.abs(pp[m]).max() > 0
    # p ~ 1000 hPa in FP32: recovering pp = 100 (p0 - p1) is good to about two ulps of p, times 100
    tol = 200.0 * np.spacing(np.abs(p0[m]).astype(np.float32))
    assert np.all(np.abs(pp[m] - rec[m]) <= tol)
    env.close()
