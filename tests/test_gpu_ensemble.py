"""The batched ensemble (skt_step_ensemble): members of uneven sizes, each with its own seeded
sounding and bubble, advanced together (a host thread per member, each on its own stream).

Stepping the ensemble must give the same bits as stepping the members one after another (the
kernels are deterministic and the members share nothing), and every member must match the oracle
after a step (relative L2 <= 1e-5 per sky field, as the whole-step parity tests).
"""
import numpy as np
import pytest

import oracle
from helpers import SKY, compare, oracle_cfg

pytestmark = pytest.mark.gpu


def _members(n, precision):
    from skewtcloudsim_gb300 import Environment, SolverConfig, sounding
    out = []
    for st, dt, speed in sounding.ensemble_members(n, scale=0.2):
        env = Environment(st.nx, st.ny, st.nz, st.voxel, SolverConfig(precision=precision))
        env.init_from(st)
        out.append((env, st, dt, speed))
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_ensemble_equals_members_stepped_alone(gpu_lib, precision):
    from skewtcloudsim_gb300 import step_ensemble
    a = _members(6, precision)
    b = _members(6, precision)
    assert len({(m[1].nx, m[1].ny, m[1].nz) for m in a}) >= 2  # uneven sizes
    st = step_ensemble([m[0] for m in a], [m[2] for m in a], 1.0, nsteps=2, threads=6)
    assert len(st) == 6
    for env, _, dt, speed in b:
        env.update_gpu(dt, speed, nsteps=2)
    for (ea, *_), (eb, *_) in zip(a, b):
        m = ea.sky_mask()
        for k in SKY:
            assert np.isfinite(ea.read(k)[m]).all(), k  # equal bits of two NaN states would also pass
            np.testing.assert_array_equal(ea.read(k).view(np.uint32), eb.read(k).view(np.uint32), err_msg=k)
        assert ea.stats()["nsub"] == eb.stats()["nsub"]
    for m in a + b:
        m[0].close()


def test_ensemble_members_match_oracle(gpu_lib):
    from skewtcloudsim_gb300 import step_ensemble
    ms = _members(4, 0)
    step_ensemble([m[0] for m in ms], [m[2] for m in ms], 1.0, nsteps=1)
    for env, init, dt, speed in ms:
        o = oracle.OracleState(init, np.float32)
        o.step(oracle_cfg(), dt, speed)
        bad = {k: v for k, v in compare(env, o).items() if v[0] > 1e-5}
        assert not bad, ((init.nx, init.ny, init.nz), bad)
        env.close()


def test_ensemble_errors(gpu_lib):
    from skewtcloudsim_gb300 import Environment, SktError, step_ensemble
    env = Environment(8, 8, 8, 100.0)  # never initialised
    with pytest.raises(SktError, match="member 0"):
        step_ensemble([env], 0.5)
    env.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_ensemble_equals_members_stepped_alone(gpu_lib, precision):
    """skt_ensemble_step (one graph launch per step for all members) against the members stepped
    one by one, stream-ordered: the same bits, the same substep and iteration counts; the
    ensemble steps again after one member was stepped alone (its trip counters stay consistent)."""
    from skewtcloudsim_gb300 import Ensemble
    a = _members(6, precision)
    b = _members(6, precision)
    ens = Ensemble([m[0] for m in a])
    ens.step([m[2] for m in a], 1.0, nsteps=2)
    for env, _, dt, speed in b:
        env.update_gpu(dt, speed, nsteps=2)
    a[0][0].update_gpu(a[0][2], 1.0)  # one member alone, between ensemble steps
    b[0][0].update_gpu(b[0][2], 1.0)
    st = ens.step([m[2] for m in a], 1.0)
    for env, _, dt, speed in b:
        env.update_gpu(dt, speed)
    assert len(st) == 6
    for (ea, *_), (eb, *_) in zip(a, b):
        m = ea.sky_mask()
        for k in SKY:
            assert np.isfinite(ea.read(k)[m]).all(), k
            np.testing.assert_array_equal(ea.read(k).view(np.uint32), eb.read(k).view(np.uint32), err_msg=k)
        sa, sb = ea.stats(), eb.stats()
        assert sa["nsub"] == sb["nsub"] and sa["pcg_iters"] == sb["pcg_iters"], (sa, sb)
        assert sa["kernel_launches"] > 0
    ens.close()
    for m in a + b:
        m[0].close()

