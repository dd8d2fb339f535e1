"""The oracle and the GPU library against the reference's OWN kernels, run live.

The reference kernels are compiled unmodified from the reference sources into
oracle/_ref/ref_<X>x<Y>x<Z>.cubin (oracle/build_ref.py) and driven by oracle/ref_harness.cpp.

Whole steps: each step starts all three implementations from the reference's state after the
previous step, so every comparison is one step from identical inputs. Tolerance: relative L2
<= 1e-5 per sky field per step, and equal Courant substep counts. On grids wider than 16 cells in
x or z the reference's advectGroundWaterGPU reads uninitialised shared memory at the interior
edges of its 16x16 tiles (Game/kernelSky.cu:141-164 fills halos only at the domain edge); the
garbage can reach the sky fields within a few steps, as non-finite values or as finite but wrong
ones. A step is compared only while the reference's own output is sound: finite, and within
relative L2 1e-5 of the oracle (which otherwise agrees with it to ~1e-6). The 16x32x16 grid has no
interior tile edge and must be sound on every step; a grid where no step is sound is reported as
an expected failure with that reason instead of passing without a comparison.

Stages: every stage of the step except the ground stage runs alone from the same developed state
in the reference kernels (rh_stage), the oracle and the library (skt_run_stage), on every grid,
including 64x32x64 where whole steps cannot be compared. Tolerances as the stage tests of
test_gpu_parity.py: relative L2 <= 1e-5 and max-norm relative <= 2e-5 on the fields the stage
writes, equal substep counts, PCG iteration counts within one. The ground stage is compared on
16x32x16 only, for the reason above.

Boundary masks: the Neigh records of computeNeighbourGPU (Game/kernelSky.cu:1284-1316) against
the classes the library's kernels derive from the heightfield (skt_read_neighbours), bit for bit,
on flat ground and on a heightfield with interior hills and ground at the domain edges.

Step time: the reference's kernels as its updateGPU drives them (the harness synchronises the
context after launches as the reference does) against this library, each step one launch of its
captured graph, on the same grids from the same initial state: the reference GPU baseline.
"""
import copy
import json
import os
import time

import numpy as np
import pytest

import oracle
from helpers import GROUND, SKY, make_env, oracle_cfg, push_oracle_to_env, rel_l2, rel_max, small_case
from skewtcloudsim_gb300 import SolverConfig

pytestmark = pytest.mark.gpu

refh = pytest.importorskip("oracle.refharness")

STEP_TOL = 1e-5
STAGE_TOL = 2e-5


def _clone(st):
    c = copy.copy(st)
    c.a = {k: v.copy() for k, v in st.a.items()}
    c.gh = st.gh.copy()
    return c


def _grids():
    try:
        return refh.available_grids()
    except Exception:
        return []


GRIDS = _grids() or [pytest.param(None, marks=pytest.mark.skip("no reference cubins"))]


def _record(name, data):
    """Writes a report (per-step distances, step times) to $SKT_REPORT_DIR/refparity_<name>.json when that folder is set."""
    d = os.environ.get("SKT_REPORT_DIR", "")
    if d and os.path.isdir(d):
        with open(os.path.join(d, f"refparity_{name}.json"), "w") as f:
            json.dump(data, f, indent=1)


@pytest.mark.parametrize("grid", GRIDS)
def test_step_against_reference_kernels(gpu_lib, grid):
    X, Y, Z = grid
    init, dt, speed = small_case((X, Z, Y))
    ref = oracle.OracleState(init, np.float32)
    env = make_env(init)
    cfg = oracle.Config()
    report = []
    for step in range(3):
        m = ref.sky_mask()
        if step > 0 and not all(np.isfinite(ref.a[k][m]).all() for k in SKY):
            break  # the reference's own state went non-finite: no later step starts from valid inputs
        orc = _clone(ref)
        push_oracle_to_env(ref, env)
        rd = refh.run_reference(ref, dt, speed, 1)
        od = orc.step(cfg, dt, speed)
        env.update_gpu(dt, speed)
        gd = env.stats()
        m = ref.sky_mask()
        finite = all(np.isfinite(ref.a[k][m]).all() for k in SKY)
        # the reference reads uninitialised shared memory at interior ground-tile edges (grids
        # wider than 16): its state turns NaN, or stays finite but wrong, by anything from a few
        # 1e-5 to O(1) and differently from run to run; the independent oracle tells the two apart
        # (it agrees with the reference to ~1e-6 whenever the reference is sound)
        sound = finite and all(rel_l2(orc.a[k], ref.a[k], m) <= STEP_TOL for k in SKY)
        row = {"ref_finite": bool(finite), "ref_sound": bool(sound), "step": step + 1, "ref_pcg": rd["pcg_iters"][0],
               "oracle_pcg": od["pcg_iters"], "gpu_pcg": gd["pcg_iters"], "nsub_ref": rd["nsub"][0], "nsub_gpu": gd["nsub"]}
        for k in SKY:
            row[f"oracle_{k}"] = rel_l2(orc.a[k], ref.a[k], m)
            row[f"gpu_{k}"] = rel_l2(env.read(k), ref.a[k], m)
        report.append(row)
    _record(f"{X}x{Y}x{Z}", report)
    env.close()
    if (X, Y, Z) == (16, 32, 16):
        assert all(r["ref_sound"] for r in report)
    if not report[0]["ref_sound"]:
        pytest.xfail(f"{X}x{Y}x{Z}: the reference's own first step is unsound (advectGroundWaterGPU reads uninitialised "
                     "shared memory at interior 16x16 tile edges); compared stage by stage instead")
    for row in report:
        if not row["ref_sound"]:
            break  # the reference's uninitialised ground-tile halos; later steps start from its corrupted state
        assert row["nsub_ref"] == row["nsub_gpu"], row
        bad = {k: v for k, v in row.items() if (k.startswith("oracle_") or k.startswith("gpu_"))
               and not k.endswith("_pcg") and v > STEP_TOL}
        assert not bad, (row["step"], bad)


# ---- stage by stage ------------------------------------------------------------------------

_developed_cache = {}


def _developed(grid):
    if grid not in _developed_cache:
        X, Y, Z = grid
        init, dt, speed = small_case((X, Z, Y))
        st = oracle.OracleState(init, np.float32)
        for _ in range(2):
            st.step(oracle_cfg(), dt, speed)
        _developed_cache[grid] = (init, dt, speed, st)
    return _developed_cache[grid]


def _condensate(st):
    rng = np.random.default_rng(7)
    m = st.sky_mask()
    for k, s in (("qw", 2e-3), ("qc", 1e-3), ("qr", 1e-3), ("qs", 5e-4), ("qi", 5e-4)):
        st.a[k][m] = rng.uniform(0, s, m.sum()).astype(np.float32)


def _swirl(st, amp=6.0):
    X, Y, Z = st.X, st.Y, st.Z
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    m = st.sky_mask()
    u = amp * np.sin(2 * np.pi * x / 13.0) * np.cos(2 * np.pi * z / 11.0)
    v = 0.5 * amp * np.sin(2 * np.pi * y / 9.0) * np.sin(2 * np.pi * x / 7.0)
    w = -amp * np.cos(2 * np.pi * z / 9.0) * np.sin(2 * np.pi * x / 15.0)
    for k, a in (("u", u), ("v", v), ("w", w)):
        st.a[k][m] = a.reshape(-1)[m].astype(np.float32)


# (stage, arg, dt or dt*speed, speed, fields written, state change)
STAGES = (
    [(0, t, None, None, (["th", "qv", "u", "v", "w", "qw"][t],), None) for t in range(6)]
    + [(0, t, 2.0e5, None, (["th", "qv", "u", "v", "w", "qw"][t],), None) for t in (0, 2, 3)]
    + [(1, f, 25.0, None, (["th", "u", "v", "w", "qv", "qw"][f],), _swirl) for f in range(6)]
    + [(2, 0, None, None, ("v",), None),
       (3, 0, None, None, ("u", "v", "w", "p", "rho"), None),
       (4, 0, None, 1.0, ("th", "qv", "qw", "qc", "qr", "qs", "qi"), _condensate)]
    + [(5, t, None, None, (["qr", "qs", "qi"][t],), _condensate) for t in range(3)]
    + [(6, 0, None, 1.0, ("th", "qv", "qr", "qs", "qi") + GROUND, _condensate)]
)


def _stage_id(s):
    stage, arg, dts, *_ = s
    return f"s{stage}a{arg}" + (f"dt{dts:g}" if dts else "")


@pytest.mark.parametrize("grid", GRIDS)
@pytest.mark.parametrize("spec", STAGES, ids=[_stage_id(s) for s in STAGES])
def test_stage_against_reference_kernels(gpu_lib, grid, spec):
    stage, arg, dts, speed, names, mutate = spec
    X, Y, Z = grid
    if stage == 6 and max(X, Z) > 16:
        pytest.skip("the reference's advectGroundWaterGPU reads uninitialised shared memory at interior 16x16 tile edges "
                    "(Game/kernelSky.cu:141-164): its ground stage is unsound on grids wider than 16")
    init, dt, sp, st0 = _developed(grid)
    st = _clone(st0)
    if mutate:
        mutate(st)
    if speed is None:  # stages that take dt*speed
        a, b = (dts if dts else dt * sp), 1.0
    else:  # stages that take dt and speed apart
        a, b = dt, sp
    ref = _clone(st)
    orc = _clone(st)
    env = make_env(init)
    push_oracle_to_env(st, env)
    rd = refh.run_stage_reference(ref, stage, arg, a, b)
    od = orc.stage(oracle_cfg(), stage, arg, a, b)
    gd = env.run_stage(stage, arg, a, b)
    m = st.sky_mask()
    full = np.ones(st.X * st.Z, bool)
    bad = {}
    for k in names:
        mask = full if k in GROUND else m
        g = env.read(k)
        for who, val in (("gpu", g), ("oracle", orc.a[k])):
            l2, mx = rel_l2(val, ref.a[k], mask), rel_max(val, ref.a[k], mask)
            if l2 > STEP_TOL or mx > STAGE_TOL:
                bad[f"{who}_{k}"] = (l2, mx)
    env.close()
    assert not bad, bad
    if stage == 1:
        assert gd["nsub"] == rd["nsub"] == od["nsub"], (gd, rd, od)
    if stage == 3:
        assert abs(gd["pcg_iters"] - rd["pcg_iters"]) <= 1, (gd, rd)


# ---- boundary masks ---------------------------------------------------------------------------

def _heightfield(X, Z):
    xx, zz = np.meshgrid(np.arange(X), np.arange(Z))
    gh = np.clip(np.round(3.0 * np.exp(-((xx - X // 3) ** 2 + (zz - Z // 2) ** 2) / 20.0)), 0, 3).astype(np.int32)
    gh[:, 0] = np.maximum(gh[:, 0], 2)       # ground along the x = 0 edge
    gh[Z - 1, :] = np.maximum(gh[Z - 1, :], 1)  # and along the last z row
    gh[0, X - 1] = 4                          # a corner column
    return gh.reshape(-1)


@pytest.mark.parametrize("grid", GRIDS)
@pytest.mark.parametrize("terrain", [False, True])
def test_boundary_masks_bit_exact(gpu_lib, grid, terrain):
    X, Y, Z = grid
    init, dt, speed = small_case((X, Z, Y))
    if terrain:
        init.ground_height = _heightfield(X, Z)
    st = oracle.OracleState(init, np.float32)
    want = refh.neighbours(st)
    env = make_env(init)
    got = env.read_neighbours()
    env.close()
    assert want.shape == got.shape
    diff = np.nonzero((want != got).any(axis=(1, 2)))[0]
    assert diff.size == 0, (diff[:10], want[diff[:3]], got[diff[:3]])
    if terrain:
        assert (want[:, :, 1] == 1).sum() > 0  # the masks do see ground neighbours


@pytest.mark.parametrize("grid", GRIDS)
def test_step_time_against_reference_kernels(gpu_lib, grid):
    """Wall time per step (device synchronised) over ten steps: the reference's kernels through the
    harness, the per-call upload and readback taken out as (T(10 steps) - T(1 step)) / 9, against
    the library in graph mode. Both start from the same initial state; the PCG iteration counts
    are recorded beside the times (the reference's state turns unsound on grids wider than 16, and
    its PCG then runs to the cap). Written to $SKT_REPORT_DIR/refparity_time_<grid>.json when set."""
    X, Y, Z = grid
    init, dt, speed = small_case((X, Z, Y))
    n = 10
    ref = oracle.OracleState(init, np.float32)
    refh.run_reference(ref, dt, speed, 1)  # module load and first allocations
    t0 = time.perf_counter()
    refh.run_reference(ref, dt, speed, 1)
    t1 = time.perf_counter()
    rn = refh.run_reference(ref, dt, speed, n)
    t2 = time.perf_counter()
    ref_ms = ((t2 - t1) - (t1 - t0)) / (n - 1) * 1e3
    env = make_env(init, SolverConfig(use_graph=1))
    env.update_gpu(dt, speed)  # capture
    env.sync()
    t3 = time.perf_counter()
    env.update_gpu(dt, speed, nsteps=n)
    env.sync()
    ours_ms = (time.perf_counter() - t3) / n * 1e3
    st = env.stats()
    env.close()
    _record(f"time_{X}x{Y}x{Z}", {"grid_ref_layout": [X, Y, Z], "steps": n, "reference_ms_per_step": ref_ms,
                                  "library_ms_per_step": ours_ms, "speedup": ref_ms / ours_ms,
                                  "reference_pcg_iters": rn["pcg_iters"], "library_pcg_iters_last_step": st["pcg_iters"],
                                  "library_kernel_launches": st["kernel_launches"]})
    assert ours_ms < ref_ms, (ours_ms, ref_ms)
