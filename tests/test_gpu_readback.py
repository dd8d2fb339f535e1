"""Asynchronous readback (skt_read_fields_async / skt_read_wait): the fields arrive as they stood
when the call was made, even though the next step is already running on the device, and match
the synchronous skt_read_field bit for bit, into pageable (copy engine) and pinned (a kernel
storing through the mapped address) host buffers."""
import numpy as np
import pytest

from helpers import make_env, small_case

pytestmark = pytest.mark.gpu

NAMES = ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p")


def _host_buffers(n, pinned, keep):
    """Pinned buffers take the kernel path (stores through the mapped address), pageable ones the
    copy engine."""
    if not pinned:
        return {k: np.empty(n, np.float32) for k in NAMES}
    torch = pytest.importorskip("torch")
    out = {}
    for k in NAMES:
        t = torch.empty(n, dtype=torch.float32).pin_memory()
        keep.append(t)
        out[k] = t.numpy()
    return out


@pytest.mark.parametrize("precision,pinned", [(0, False), (1, False), (0, True), (1, True)])
def test_async_readback_is_the_snapshot(gpu_lib, precision, pinned):
    from skewtcloudsim_gb300 import SolverConfig
    init, dt, speed = small_case((32, 32, 24))
    cfg = SolverConfig(precision=precision)
    a = make_env(init, cfg)
    b = make_env(init, cfg)
    want = []
    for _ in range(3):
        a.update_gpu(dt, speed)
        want.append({k: a.read(k) for k in NAMES})
    keep = []
    bufs = [_host_buffers(b.n, pinned, keep) for _ in range(3)]
    for i in range(3):
        b.update_gpu(dt, speed)
        b.read_async(bufs[i])  # queued behind step i, copied out while step i+1 runs
        if i:
            b.read_wait()
            for k in NAMES:
                np.testing.assert_array_equal(bufs[i - 1][k].view(np.uint32), want[i - 1][k].view(np.uint32),
                                              err_msg=f"step {i - 1} {k}")
    b.read_wait()
    for k in NAMES:
        np.testing.assert_array_equal(bufs[2][k].view(np.uint32), want[2][k].view(np.uint32), err_msg=k)
        np.testing.assert_array_equal(b.read(k).view(np.uint32), want[2][k].view(np.uint32), err_msg=k)
    a.close()
    b.close()


def test_async_readback_errors_and_growth(gpu_lib):
    from skewtcloudsim_gb300 import SktError
    init, dt, speed = small_case((16, 16, 16))
    env = make_env(init)
    env.update_gpu(dt, speed)
    with pytest.raises(ValueError):
        env.read_async({"th": np.empty(env.n - 1, np.float32)})
    with pytest.raises(ValueError):
        env.read_async({"th": np.empty(env.n, np.float64)})
    # two fields, then more: the snapshot grows and the copies stay right
    small = {k: np.empty(env.n, np.float32) for k in ("th", "p")}
    env.read_async(small)
    env.read_wait()
    big = {k: np.empty(env.n, np.float32) for k in NAMES}
    env.read_async(big)
    env.read_wait()
    for k in NAMES:
        np.testing.assert_array_equal(big[k], env.read(k))
    np.testing.assert_array_equal(small["th"], env.read("th"))
    env.read_wait()  # nothing pending: returns at once
    lib, h = env._L, env._h
    import ctypes
    sel = (ctypes.c_int * 1)(999)
    d = (ctypes.c_int * 1)(0)
    out = np.empty(env.n, np.float32)
    ptrs = (ctypes.POINTER(ctypes.c_float) * 1)(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    assert lib.skt_read_fields_async(h, 1, sel, d, ptrs, env.n) != 0
    with pytest.raises(SktError):
        env._check(lib.skt_read_fields_async(h, 1, sel, d, ptrs, env.n))
    env.close()
