"""skt_diffuse_noalloc: diffusion of caller-owned device buffers with no allocation in the call.

For callers that cannot allocate device memory themselves (a host framework that owns the whole
device memory pool, or a loop where an allocation would stall the device), the library keeps
the one intermediate buffer the sweeps need in a static device array. This test drives the entry
point through the C ABI on buffers the test allocates with torch, three calls in a row (theta,
u, v) for an even and an odd sweep count (the odd count starts the ping-pong in the output
buffer), and checks each result against the existing stage entry point (skt_run_stage, which uses
skt_create's buffers) and against the oracle, within the stage tolerance of the other parity
tests. The u and v calls use k = 0.1 (dt*speed = 2e5 s), where every neighbour term matters. It
also checks that grids above the array's capacity and beyond the launch limits are rejected with
a clear message.
"""
import copy
import ctypes

import numpy as np
import pytest

import oracle
from helpers import gpu_cfg, make_env, oracle_cfg, push_oracle_to_env, rel_max, small_case

pytestmark = pytest.mark.gpu

STAGE_TOL = 2e-5


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _fptr(t):
    return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctypes.c_float))


def _call(L, torch, env, ftype, dts, sweeps, src, out, gh, col, p, Tg, Pg):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = L.skt_diffuse_noalloc(env.nx, env.ny, env.nz, ctypes.c_float(env.voxel), ftype, ctypes.c_float(dts), sweeps,
                               _fptr(src), _fptr(out), ctypes.cast(ctypes.c_void_p(gh.data_ptr()), ctypes.POINTER(ctypes.c_int32)),
                               _fptr(col) if col is not None else None, _fptr(p), _fptr(Tg), _fptr(Pg), stream)
    torch.cuda.synchronize()
    return st


@pytest.mark.parametrize("sweeps", [20, 7])
def test_noalloc_diffusion_matches_stage_entry_point_and_oracle(gpu_lib, sweeps):
    torch = pytest.importorskip("torch")
    L = gpu_lib
    init, dt, speed = small_case((32, 32, 32))
    st0 = oracle.OracleState(init, np.float32)
    st0.step(oracle_cfg(), dt, speed)  # a developed state
    env = make_env(init, gpu_cfg(0, diffuse_sweeps=sweeps))
    push_oracle_to_env(st0, env)
    mask = env.sky_mask()
    gh = _dev(torch, init.ground_height.astype(np.int32))
    p = _dev(torch, st0.a["p"])
    Tg = _dev(torch, st0.a["Tg"])
    Pg = _dev(torch, st0.a["Pg"])
    for ftype, name, col_name, dts in ((0, "th", "isenT", dt * speed), (2, "u", "defU", 2.0e5), (3, "v", None, 2.0e5)):
        before = st0.a[name].copy()
        src = _dev(torch, before)
        out = torch.full_like(src, float("nan"))
        col = _dev(torch, st0.a[col_name]) if col_name else None
        st = _call(L, torch, env, ftype, dts, sweeps, src, out, gh, col, p, Tg, Pg)
        assert st == 0, L.skt_last_error(None)
        got = out.cpu().numpy()
        # the existing entry point on the library's own buffers
        push_oracle_to_env(st0, env)
        env.run_stage(0, ftype, dts)
        want = env.read(name)
        assert rel_max(got, want, mask) <= STAGE_TOL, (name, sweeps, rel_max(got, want, mask))
        # the oracle
        ost = copy.copy(st0)
        ost.a = {k: v.copy() for k, v in st0.a.items()}
        ost.gh = st0.gh.copy()
        ost.stage(oracle_cfg(diffuse_sweeps=sweeps), 0, ftype, dts)
        assert rel_max(got, ost.a[name], mask) <= STAGE_TOL, (name, sweeps, rel_max(got, ost.a[name], mask))
        np.testing.assert_array_equal(got[~mask], before[~mask])  # ground cells are passed through
    env.close()


def test_noalloc_rejects_grids_beyond_capacity(gpu_lib):
    L = gpu_lib
    st = L.skt_diffuse_noalloc(256, 128, 256, ctypes.c_float(100.0), 5, ctypes.c_float(0.5), 20, None, None, None,
                               None, None, None, None, None)
    assert st == 1  # SKT_INVALID_ARG
    assert b"SKT_NOALLOC_MAX_CELLS" in L.skt_last_error(None)
    # within the cell cap, but nz above the launch grid's z limit: rejected before any launch
    st = L.skt_diffuse_noalloc(1, 2, 70000, ctypes.c_float(100.0), 5, ctypes.c_float(0.5), 20, None, None, None,
                               None, None, None, None, None)
    assert st == 1
    assert b"65535" in L.skt_last_error(None)
