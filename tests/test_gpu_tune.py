"""Launch-shape tuning (skt_set_tuning / skt_autotune) and the two-sweep diffusion kernel.

The tuned shapes must not change a single bit: the two-sweep passes (temporal blocking of depth
2, input planes streamed through shared memory by TMA: k_diffuse_pair4 with four-cell lanes and
6 or 14 rows per block, k_diffuse2 with one-cell lanes and 4 or 8 rows per warp) compute each
intermediate cell with the arithmetic of the one-sweep kernel from the same neighbour values, its
ghost values included, so every diffusion boundary table, even and odd sweep counts, every tile
height and several run lengths (down to one plane per run) are compared bit for bit with the
default one-sweep passes, on a 32^3 grid and on a wide one (x = 260: three blocks along x, the
last with one active lane, ragged row tiles, several z runs). k = 0.1
(dt*speed = 2e5 s) makes every neighbour term count. The autotuner is checked to write its cache,
to read it back for a second environment of the same grid, and to leave a whole step's results
unchanged.
"""
import json

import numpy as np
import pytest

from helpers import GROUND, SKY, gpu_cfg, make_env, small_case

pytestmark = pytest.mark.gpu

NAMES = ["th", "qv", "u", "v", "w", "qw"]


def _developed_env(shape, cfg):
    init, dt, speed = small_case(shape, name="precision-512x512x256")
    env = make_env(init, cfg)
    env.update_gpu(dt, speed)
    return init, dt, speed, env


@pytest.mark.parametrize("shape", [(32, 32, 32), (260, 32, 48)])
@pytest.mark.parametrize("sweeps", [20, 7, 2, 1])
def test_two_sweep_diffusion_is_bit_identical(gpu_lib, shape, sweeps):
    init, dt, speed, ref = _developed_env(shape, gpu_cfg(0, diffuse_sweeps=sweeps))
    state = {k: ref.read(k) for k in SKY + GROUND}  # theta's ground faces read the ground T and p
    variants = [dict(diffuse_depth=2, diffuse_rows=14, diffuse2_bps=2), dict(diffuse_depth=2, diffuse_rows=14, diffuse2_bps=64),
                dict(diffuse_depth=2, diffuse_rows=6, diffuse2_bps=4), dict(diffuse_depth=2, diffuse_rows=6, diffuse2_bps=256),
                dict(diffuse_depth=2, diffuse_rows=4, diffuse2_bps=8), dict(diffuse_depth=2, diffuse_rows=8, diffuse2_bps=2),
                dict(diffuse_depth=2, diffuse_rows=4, diffuse2_bps=64), dict(diffuse_depth=1, diffuse_bps=7)]
    envs = []
    for v in variants:
        e = make_env(init, gpu_cfg(0, diffuse_sweeps=sweeps))
        e.set_tuning(**v)
        envs.append(e)
    for ftype in range(6):
        for dts in (dt * speed, 2.0e5):
            for k, a in state.items():
                ref.write(k, a)
            ref.run_stage(0, ftype, dts)
            want = ref.read(NAMES[ftype])
            for v, e in zip(variants, envs):
                for k, a in state.items():
                    e.write(k, a)
                e.run_stage(0, ftype, dts)
                got = e.read(NAMES[ftype])
                bad = np.nonzero(got.view(np.uint32) != want.view(np.uint32))[0]
                assert bad.size == 0, (v, ftype, dts, bad[:8], got[bad[:4]], want[bad[:4]])
    for e in envs + [ref]:
        e.close()


def test_autotune_cache_and_unchanged_step(gpu_lib, tmp_path):
    cache = str(tmp_path / "tuning.json")
    init, dt, speed = small_case((64, 64, 32), name="precision-512x512x256")
    a = make_env(init)
    t1 = a.autotune(cache)
    assert not t1["from_cache"] and t1["diffuse_ms"] > 0
    with open(cache) as f:
        entries = json.load(f)
    assert len(entries) == 1
    b = make_env(init)
    t2 = b.autotune(cache)
    assert t2["from_cache"]
    assert {k: t2[k] for k in b.TUNING_FIELDS} == {k: t1[k] for k in a.TUNING_FIELDS}
    assert b.get_tuning() == {k: t1[k] for k in b.TUNING_FIELDS}
    c = make_env(init)  # default shapes
    for env in (a, c):
        env.update_gpu(dt, speed, nsteps=2)
    for k in SKY:
        np.testing.assert_array_equal(a.read(k).view(np.uint32), c.read(k).view(np.uint32), err_msg=k)
    # a second grid gets its own entry; forcing re-measures the first
    d_init, _, _ = small_case((32, 32, 32))
    d = make_env(d_init)
    assert not d.autotune(cache)["from_cache"]
    assert not a.autotune(cache, force=True)["from_cache"]
    with open(cache) as f:
        assert len(json.load(f)) == 2
    for env in (a, b, c, d):
        env.close()


def test_set_tuning_rejects_bad_values(gpu_lib):
    from skewtcloudsim_gb300 import SktError
    init, dt, speed = small_case((32, 32, 32))
    env = make_env(init)
    with pytest.raises(SktError):
        env.set_tuning(diffuse_depth=3)
    with pytest.raises(SktError):
        env.set_tuning(diffuse_rows=5)
    with pytest.raises(SktError):
        env.set_tuning(diffuse_rows=12)
    with pytest.raises(SktError):
        env.set_tuning(ppm_x_bps=0)
    env.close()
