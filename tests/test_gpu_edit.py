"""Editing between steps (the reference's brush, box selection and parameter reset; heightfield
edits with the reset of freed cells and the ground temperature) against the oracle.

Both start from the same state (pushed in full, ground cells included), so every cell is compared:
the edits are element-wise, the only arithmetic difference is CUDA's powf against libm's in the
brush profile (relative 1e-6). Heightfields must match exactly.
"""
import numpy as np
import pytest

import oracle
from helpers import SKY, GROUND, make_env, oracle_cfg, push_oracle_to_env, rel_l2, small_case
from skewtcloudsim_gb300 import Parameter, SktError

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 32)  # (x, y, z), z vertical -> reference layout X=32, Y=32, Z=32
PGROUND, WIND = int(Parameter.PGROUND), int(Parameter.WIND)


@pytest.fixture(scope="module")
def developed():
    init, dt, speed = small_case(SHAPE)
    st = oracle.OracleState(init, np.float32)
    st.step(oracle_cfg(), dt, speed)
    return init, dt, speed, st


def _clone(st):
    import copy
    c = copy.copy(st)
    c.a = {k: v.copy() for k, v in st.a.items()}
    c.gh = st.gh.copy()
    return c


def _same(env, st, names=SKY + GROUND):
    np.testing.assert_array_equal(env.read_ground_height(), st.gh)
    for k in names:
        np.testing.assert_allclose(env.read(k), st.a[k], rtol=1e-6, atol=1e-7, err_msg=k)


def _pair(developed):
    init, dt, speed, st0 = developed
    st = _clone(st0)
    env = make_env(init)
    push_oracle_to_env(st, env)
    return init, st, env


@pytest.mark.parametrize("param,pos,size", [(0, (10, 8, 12), 3.5), (1, (20, 20, 4), 2.0), (WIND, (3, 12, 28), 4.25),
                                            (4, (31, 31, 31), 3.0), (0, (0, 1, 0), 6.0)])
def test_brush(gpu_lib, developed, param, pos, size):
    init, st, env = _pair(developed)
    d = (0.8, -0.4, 0.25)
    ch_o = st.brush(param, size, pos, 2.0, 0.5, 1.5, 4.0, d, p_column=init.p_column)
    ch_g = env.apply_brush(param, size, pos, 2.0, 0.5, 1.5, 4.0, d)
    assert ch_o is False and ch_g is False
    _same(env, st)
    env.close()


@pytest.mark.parametrize("param,lo,hi", [(0, (4, 2, 5), (12, 9, 20)), (WIND, (0, 1, 0), (31, 3, 31)), (6, (10, 5, 3), (8, 7, 9)),
                                         (2, (-3, 25, 28), (40, 40, 40))])
def test_selection(gpu_lib, developed, param, lo, hi):
    init, st, env = _pair(developed)
    d = (0.5, 0.25, -1.0)
    st.selection(param, lo, hi, 3.25, d, p_column=init.p_column)
    env.apply_selection(param, lo, hi, 3.25, d)
    _same(env, st)
    env.close()


def test_ground_edits_then_step(gpu_lib, developed):
    init, dt, speed, _ = developed
    _, st, env = _pair(developed)
    # raise terrain with the brush, lower part of it with a box erase, then take a step on it
    assert st.brush(PGROUND, 3.5, (12, 4, 14), 1.0, 0.5, 1.0, 1.0, p_column=init.p_column)
    assert env.apply_brush(PGROUND, 3.5, (12, 4, 14), 1.0, 0.5, 1.0, 1.0)
    _same(env, st)
    assert st.gh.max() > 0
    assert st.selection(PGROUND, (11, 1, 13), (13, 2, 15), 0.0, erase=True, p_column=init.p_column)
    assert env.apply_selection(PGROUND, (11, 1, 13), (13, 2, 15), 0.0, erase=True)
    _same(env, st)
    # a brush on the new terrain leaves the ground alone
    st.brush(0, 4.0, (12, 3, 14), 1.0, 0.5, 1.0, 2.0, p_column=init.p_column)
    env.apply_brush(0, 4.0, (12, 3, 14), 1.0, 0.5, 1.0, 2.0)
    _same(env, st)
    st.step(oracle_cfg(), dt, speed)
    env.update_gpu(dt, speed)
    m = st.sky_mask()
    bad = {k: rel_l2(env.read(k), st.a[k], m) for k in SKY if rel_l2(env.read(k), st.a[k], m) > 1e-5}
    assert not bad, bad
    env.close()


@pytest.mark.parametrize("param", [0, 1, 2, 5, WIND, int(Parameter.PRESSURE), PGROUND])
def test_reset_parameter(gpu_lib, developed, param):
    init, st, env = _pair(developed)
    # some terrain first, so the per-column stop at the first ground cell matters
    st.selection(PGROUND, (3, 2, 4), (9, 3, 6), 0.0, p_column=init.p_column)
    env.apply_selection(PGROUND, (3, 2, 4), (9, 3, 6), 0.0)
    st.reset_parameter(param, p_column=init.p_column)
    env.reset_parameter(param)
    _same(env, st)
    env.close()


def test_edit_rejects(gpu_lib, developed):
    init, st, env = _pair(developed)
    with pytest.raises(SktError):
        env.apply_brush(int(Parameter.PRESSURE), 2.0, (4, 4, 4), 1.0, 0.5, 1.0, 1.0)
    with pytest.raises(SktError):
        env.apply_selection(12, (0, 0, 0), (1, 1, 1), 1.0)
    env.close()
