"""skt_diffuse_noalloc: diffusion of caller-owned device buffers with no allocation in the call.

For callers that cannot allocate device memory themselves (a host framework that owns the whole
device memory pool, or a loop where an allocation would stall the device), the library keeps
the one intermediate buffer the sweeps need in a static device array. This test drives the entry
point through the C ABI on buffers the test allocates with torch, twice in a row (theta, then
u), and checks each result against the existing stage entry point (skt_run_stage, which uses
skt_create's buffers) within the stage tolerance of the other parity tests. It also checks that
a grid above the array's capacity is rejected with a clear message.
"""
import ctypes

import numpy as np
import pytest

from helpers import make_env, rel_max, small_case

pytestmark = pytest.mark.gpu

STAGE_TOL = 2e-5


def _dev(torch, a, dtype=None):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _call(L, torch, env, ftype, dt, src, out, gh, col, p, Tg, Pg):
    fn = L.skt_diffuse_noalloc
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = fn(env.nx, env.ny, env.nz, ctypes.c_float(env.voxel), ftype, ctypes.c_float(dt), 20,
            ctypes.cast(_ptr(src), ctypes.POINTER(ctypes.c_float)), ctypes.cast(_ptr(out), ctypes.POINTER(ctypes.c_float)),
            ctypes.cast(_ptr(gh), ctypes.POINTER(ctypes.c_int32)),
            ctypes.cast(_ptr(col), ctypes.POINTER(ctypes.c_float)) if col is not None else None,
            ctypes.cast(_ptr(p), ctypes.POINTER(ctypes.c_float)), ctypes.cast(_ptr(Tg), ctypes.POINTER(ctypes.c_float)),
            ctypes.cast(_ptr(Pg), ctypes.POINTER(ctypes.c_float)), stream)
    torch.cuda.synchronize()
    return st


def test_noalloc_diffusion_matches_stage_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    L = gpu_lib
    init, dt, speed = small_case((32, 32, 32))
    env = make_env(init)
    env.update_gpu(dt, speed)  # a developed state
    mask = env.sky_mask()
    gh = _dev(torch, init.ground_height.astype(np.int32))
    p = _dev(torch, env.read("p"))
    Tg = _dev(torch, env.read("Tg"))
    Pg = _dev(torch, env.read("Pg"))
    for ftype, name, col_name in ((0, "th", "isenT"), (2, "u", "defU")):
        before = env.read(name)
        src = _dev(torch, before)
        out = torch.empty_like(src)
        col = _dev(torch, env.read(col_name))
        st = _call(L, torch, env, ftype, dt * speed, src, out, gh, col, p, Tg, Pg)
        assert st == 0, L.skt_last_error(None)
        got = out.cpu().numpy()
        env.run_stage(0, ftype, dt * speed)
        want = env.read(name)
        assert rel_max(got, want, mask) <= STAGE_TOL, (name, rel_max(got, want, mask))
        np.testing.assert_array_equal(got[~mask], before[~mask])  # ground cells are passed through
    env.close()


def test_noalloc_rejects_grids_beyond_capacity(gpu_lib):
    L = gpu_lib
    st = L.skt_diffuse_noalloc(256, 128, 256, ctypes.c_float(100.0), 5, ctypes.c_float(0.5), 20, None, None, None,
                               None, None, None, None, None)
    assert st == 1  # SKT_INVALID_ARG
    assert b"SKT_NOALLOC_MAX_CELLS" in L.skt_last_error(None)
