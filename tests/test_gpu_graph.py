"""The step captured as a CUDA graph (use_graph = 1) against the stream-ordered step.

A graph step runs the same kernels with the same arguments in the same order: the loops whose trip
counts the host reads back in the stream-ordered form (advection substeps, PCG iteration chunks,
the mixed refinement and its inner CG) are conditional WHILE nodes whose conditions the kernels set
on the device, and kernels of iterations past a solver's stop return at once in both forms. So the
fields must agree bit for bit, and the substep and iteration counts exactly, for both semantics,
the mixed-precision solve, a wide grid (several warps and tiles), a change of dt (a new capture),
an edit between steps (the ground block runs outside the graph) and several steps per call. A NaN
written into the state is reported as in the stream-ordered form.
"""
import numpy as np
import pytest

from helpers import SKY, gpu_cfg, make_env, small_case
from skewtcloudsim_gb300 import SolverConfig, SktError
from skewtcloudsim_gb300.environment import Status

pytestmark = pytest.mark.gpu


def _pair(shape, cfg_kw, name="plain-64x64x32"):
    init, dt, speed = small_case(shape, name=name)
    a = make_env(init, SolverConfig(**cfg_kw))
    b = make_env(init, SolverConfig(use_graph=1, **cfg_kw))
    return init, dt, speed, a, b


def _same(a, b, what):
    for k in SKY:
        x, y = a.read(k), b.read(k)
        bad = np.nonzero(x.view(np.uint32) != y.view(np.uint32))[0]
        assert bad.size == 0, (what, k, bad.size, bad[:5], x[bad[:3]], y[bad[:3]])
    sa, sb = a.stats(), b.stats()
    assert sa["nsub"] == sb["nsub"], (what, sa, sb)
    assert sa["pcg_iters"] == sb["pcg_iters"] and sa["converged"] == sb["converged"], (what, sa, sb)
    assert sa["outer_iters"] == sb["outer_iters"], (what, sa, sb)
    assert sa["sim_time"] == sb["sim_time"]


@pytest.mark.parametrize("cfg_kw", [dict(semantics=0), dict(semantics=1), dict(precision=1),
                                    dict(semantics=0, pcg_fused=0)], ids=["reference", "textbook", "mixed", "three-launch"])
def test_graph_step_equals_stream_ordered(gpu_lib, cfg_kw):
    init, dt, speed, a, b = _pair((32, 32, 32), cfg_kw)
    for step in range(3):
        a.update_gpu(dt, speed)
        b.update_gpu(dt, speed)
        _same(a, b, step)
    assert b.stats()["kernel_launches"] > 0
    a.close()
    b.close()


def test_graph_wide_grid_and_several_steps_per_call(gpu_lib):
    init, dt, speed, a, b = _pair((260, 32, 48), dict(semantics=0), name="precision-512x512x256")
    a.update_gpu(dt, speed, nsteps=2)
    b.update_gpu(dt, speed, nsteps=2)
    _same(a, b, "two steps")
    a.close()
    b.close()


def test_graph_recaptures_on_new_dt_and_after_an_edit(gpu_lib):
    init, dt, speed, a, b = _pair((32, 32, 32), dict(semantics=0))
    for env in (a, b):
        env.update_gpu(dt, speed)
        env.update_gpu(2 * dt, speed)  # a new dt: a new capture
    _same(a, b, "new dt")
    for env in (a, b):  # raise the ground under a brush: non-flat terrain (a new capture), and the
        # editor's ground block runs before the next step
        env.apply_brush(8, 3.0, (16, 2, 16), 1.0, dt, 1.0, 1.0)
        env.update_gpu(dt, speed)
    _same(a, b, "after an edit")
    a.close()
    b.close()


def test_graph_reports_nan(gpu_lib):
    init, dt, speed = small_case((32, 32, 32))
    env = make_env(init, gpu_cfg(0, use_graph=1))
    env.update_gpu(dt, speed)
    u = env.read("u")
    u[16 + 10 * 32 + 16 * 32 * 32] = np.inf
    env.write("u", u)
    with pytest.raises(SktError) as ei:
        env.update_gpu(dt, speed)
    assert ei.value.status == Status.NAN_DETECTED
    env.close()


def test_async_steps_equal_synchronous_steps(gpu_lib):
    """skt_step_async queues graph steps without waiting and skt_sync collects them: three queued
    single steps give the fields, counts, clock and status of one three-step skt_step; a new dt
    between queued calls captures again after collecting what the old graph queued; a synchronous
    step after queued ones collects them first; a NaN met by a queued step is reported by skt_sync."""
    init, dt, speed, a, c = _pair((32, 32, 32), dict(semantics=0))
    ra = a.update_gpu(dt, speed, nsteps=3)
    for _ in range(3):
        assert c.update_gpu_async(dt, speed) == Status.OK
    assert c.sync() == ra
    _same(a, c, "three queued steps")
    a.update_gpu(2 * dt, speed)
    a.update_gpu(dt, speed)
    c.update_gpu_async(dt * 2, speed)  # a new dt: a new capture
    c.update_gpu(dt, speed)            # synchronous, after a queued step of another dt
    _same(a, c, "new dt, then a synchronous step")
    u = c.read("u")
    u[16 + 10 * 32 + 16 * 32 * 32] = np.nan
    c.write("u", u)
    assert c.update_gpu_async(dt, speed) == Status.OK  # queued: nothing is known yet
    with pytest.raises(SktError) as ei:
        c.sync()
    assert ei.value.status == Status.NAN_DETECTED
    a.close()
    c.close()
