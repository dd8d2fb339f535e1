"""Headless view and volume export on the GPU.

* The voxel view (``skt_view_volume``) against the oracle's restatement of editor::viewSky /
  viewGround (oracle/view.py) on the device's own fields: voxel kinds exactly, colours bit for bit
  (every operation of getColor is rounded on its own on both sides) except the temperature view:
  CUDA's powf differs from libm's by up to 2 ulp, a few ulp of T ~ 290 K (3e-5 K each), and the
  temperature scheme turns 10 K into one colour unit, so colours agree within 2e-5.
* Brick export: the bricks written are exactly those with a cell off the background by more than
  the threshold, and their values are the field's (float32 bit for bit, float16 as numpy rounds).
* Checkpoints: a state saved, loaded into a new environment and stepped gives the same bits as
  the original run.
"""
import numpy as np
import pytest

from helpers import make_env, small_case
from oracle import view as ov

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 24)  # (x, y, z), z vertical -> reference layout X=32, Y=24, Z=32


@pytest.fixture(scope="module")
def state(gpu_lib):
    from skewtcloudsim_gb300 import DIAG_BUOYANCY, Parameter
    init, dt, speed = small_case(SHAPE)
    env = make_env(init)
    env.set_diagnostics(DIAG_BUOYANCY)
    for _ in range(2):
        env.update_gpu(dt, speed)
    env.apply_selection(int(Parameter.PGROUND), (3, 1, 4), (9, 3, 8), 0.0)  # a block of terrain
    env.update_gpu(dt, speed)
    # condensate in half the cells after the last step, so every mixing-ratio view has colours
    rng = np.random.default_rng(5)
    for k, s in (("qw", 2e-3), ("qc", 1e-3), ("qr", 1e-3), ("qs", 5e-4), ("qi", 5e-4)):
        a = env.read(k)
        m = rng.random(a.size) < 0.5
        a[m] = rng.uniform(0, s, m.sum()).astype(np.float32)
        env.write(k, a)
    yield env
    env.close()


def _host_view(env, sky, ground, lo=None, hi=None):
    f = {k: env.read(k) for k in ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p", "debug2", "debug3")}
    g = {"T": env.read("Tg"), "Qrs": env.read("Qrs"), "Qgr": env.read("Qgr"), "Qgs": env.read("Qgs"),
         "Qgi": env.read("Qgi"), "P": env.read("Pg")}
    return ov.view(f, g, env.read_ground_height(), (env.nx, env.ny, env.nz), sky, ground, lo, hi)


@pytest.mark.parametrize("sky,ground", [(0, 0), (1, -1), (2, 1), (3, 2), (4, 3), (5, 4), (6, -1), (7, 0), (9, -1),
                                        (10, 1), (11, -1), (12, 2)])
def test_view_matches_oracle(state, sky, ground):
    env = state
    rgb, kind = env.view(sky, ground)
    want_rgb, want_kind = _host_view(env, sky, ground)
    np.testing.assert_array_equal(kind, want_kind)
    assert (kind == 1).sum() > 0 and ((kind == 3).sum() > 0) == (ground >= 0) and (kind == 2).sum() > 0
    if sky == 0:
        assert np.abs(rgb - want_rgb).max() <= 2e-5
    else:
        np.testing.assert_array_equal(rgb.view(np.uint32), want_rgb.view(np.uint32))
    assert len(np.unique(rgb[kind == 1], axis=0)) > 3  # the view is not one flat colour


def test_view_slice_and_errors(state):
    from skewtcloudsim_gb300 import SktError
    env = state
    lo, hi = (5, 0, 7), (6, env.ny, 20)
    rgb, kind = env.view(3, 1, lo, hi)
    want_rgb, want_kind = _host_view(env, 3, 1, lo, hi)
    np.testing.assert_array_equal(kind, want_kind)
    np.testing.assert_array_equal(rgb.view(np.uint32), want_rgb.view(np.uint32))
    k = kind.reshape(env.nz, env.ny, env.nx)
    assert (k[:, 1:, 4] != 1).all() and (k[7:20, 6:, 5] == 1).all()
    with pytest.raises(SktError):
        env.view(8)  # PGROUND has no sky view
    with pytest.raises(SktError):
        env.view(3, 7)


def _active(a, shape, bg, thr):
    X, Y, Z = shape
    nb = [(-(-s // 8)) for s in shape]
    pad = np.full((nb[2] * 8, nb[1] * 8, nb[0] * 8), bg, np.float32)
    pad[:Z, :Y, :X] = a.reshape(Z, Y, X)
    off = ~(np.abs(pad - np.float32(bg)) <= np.float32(thr))
    return off.reshape(nb[2], 8, nb[1], 8, nb[0], 8).any(axis=(1, 3, 5))  # [bz, by, bx]


@pytest.mark.parametrize("name,thr,bg,half", [("qc", 1e-6, 0.0, False), ("th", -1.0, 0.0, False), ("u", 0.5, 0.0, True),
                                              ("qv", 0.0, 0.0, False), ("p", 2.0, 900.0, False)])
def test_brick_export_exact(state, name, thr, bg, half):
    env = state
    a = env.read(name)
    bf = env.export_bricks(name, threshold=thr, background=bg, half=half)
    want = _active(a, (env.nx, env.ny, env.nz), bg, thr)
    got = np.zeros_like(want)
    got[bf.coords[:, 2], bf.coords[:, 1], bf.coords[:, 0]] = True
    np.testing.assert_array_equal(got, want)
    order = bf.coords[:, 0] + want.shape[2] * (bf.coords[:, 1] + want.shape[1] * bf.coords[:, 2].astype(np.int64))
    assert np.all(np.diff(order) > 0)  # brick order, x fastest
    dense = bf.dense()
    cell_active = np.repeat(np.repeat(np.repeat(want, 8, 0), 8, 1), 8, 2)[:env.nz, :env.ny, :env.nx].reshape(-1)
    if half:
        np.testing.assert_array_equal(dense[cell_active].view(np.uint16), a[cell_active].astype(np.float16).view(np.uint16))
    else:
        np.testing.assert_array_equal(dense[cell_active].view(np.uint32), a[cell_active].view(np.uint32))
    assert np.all(dense[~cell_active] == np.float32(bg))
    if thr < 0:
        assert bf.count == want.size


@pytest.mark.parametrize("precision", [0, 1])
def test_checkpoint_resume_is_bit_identical(gpu_lib, tmp_path, precision):
    from skewtcloudsim_gb300 import SolverConfig, volume
    init, dt, speed = small_case((24, 24, 16))
    cfg = SolverConfig(precision=precision)
    env = make_env(init, cfg)
    env.set_clock(43200.0, day=170, longitude=4.9, sun=0.9, pause=0)
    for _ in range(2):
        env.update_gpu(dt, speed)
    path = tmp_path / "state.npz"
    env.save_checkpoint(path)
    names = ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p", "rho", "Tg", "Qrs", "Qgr", "tg", "cover")
    for _ in range(2):
        env.update_gpu(dt, speed)
    want = {k: env.read(k) for k in names}
    want_t = env.stats()["sim_time"]
    env.close()
    env2 = volume.load_checkpoint(path)
    assert env2.cfg.precision == precision
    for _ in range(2):
        env2.update_gpu(dt, speed)
    for k in names:
        np.testing.assert_array_equal(env2.read(k).view(np.uint32), want[k].view(np.uint32), err_msg=k)
    assert env2.stats()["sim_time"] == want_t
    env2.close()
