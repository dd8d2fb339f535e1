"""A radiosonde archive drives the GPU step: readTable's readDWDFile / readKNMIFile and
initEnvironment (host code of libskewt_gb300), then environmentGPU::init and updateGPU on the
device, against the oracle started from the same interpolated state.

The synthetic ascents (tests/sounding_files.py) change wind direction from row to row, so the
initial wind has strong shear: a harder start than the analytic workloads. Tolerances as the
whole-step parity tests: relative L2 <= 1e-5 per sky field after each step, Courant substep
counts equal; the state is carried forward from the oracle between steps.
"""
import io

import numpy as np
import pytest

import oracle
import sounding_files as sf
from helpers import compare, oracle_cfg, push_oracle_to_env, small_case

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5


@pytest.mark.parametrize("kind,case,shape", [("dwd", "mid", (24, 32, 20)), ("knmi", "fine", (32, 24, 16))])
def test_sounding_drives_the_step(gpu_lib, kind, case, shape):
    from skewtcloudsim_gb300 import Environment, SolverConfig, radiosonde
    X, Y, Z = shape
    t = radiosonde.ReadTable()
    if kind == "dwd":
        t.data = radiosonde.read_dwd(io.BytesIO(sf.dwd_archive(case, 7)), archive_name=sf.DWD_ARCHIVE)
    else:
        t.data = radiosonde.read_knmi(io.BytesIO(sf.knmi_archive(case, 3)))
    env = Environment(X, Y, Z, 64.0, SolverConfig())
    init = t.init_environment(env)  # environmentGPU::init with the reference's init noise
    st = oracle.OracleState(init, np.float32)
    res = compare(env, st)
    assert all(mx <= 1e-6 for _, mx in res.values()), res
    _, dt, speed = small_case((16, 16, 16))
    for step in range(2):
        od = st.step(oracle_cfg(), dt, speed)
        env.update_gpu(dt, speed)
        assert env.stats()["nsub"] == od["nsub"], step
        res = compare(env, st)
        bad = {k: v for k, v in res.items() if v[0] > STEP_TOL}
        assert not bad, (step, bad)
        push_oracle_to_env(st, env)
    env.close()
