"""Error growth of the GPU step against the FP64 oracle of the same method, free running.

Both runs start from the same state and are never re-synchronised. After N steps (50 by default,
SKT_ERR_STEPS overrides; the grid is 32x32x32, SKT_ERR_SHAPE=x,y,z (z vertical) overrides; run with
-s to print the per-field table) every sky field's relative L2
distance from the FP64 oracle is compared with that of the FP32 oracle (the same method in FP32):
FP32 storage of the fields alone makes the two FP64 and FP32 trajectories drift apart (theta by
~1.4e-6 per step: the diffusion increments k*dtheta ~ 1e-7 K are below one ulp of theta ~ 300 K),
so the bound is the FP32 oracle's own distance, with a factor 2 for the GPU's different rounding
(FMA contraction, CUDA transcendentals, reciprocal multiplies, reduction order) and an absolute
floor of 1e-6.

Two methods: plain (reference semantics: the reference's Jacobi-PCG with its quirks, 200
iterations or max residual 1e-5) against the FP64 oracle of reference semantics, and mixed
(textbook operator, multigrid-preconditioned FP32 CG in float-float refinement to 1e-8) against
the FP64 oracle of the textbook method solved to a max residual of 1e-13.
"""
import os

import numpy as np
import pytest

import oracle
from helpers import SKY, make_env, rel_l2, small_case
from skewtcloudsim_gb300 import SolverConfig

pytestmark = pytest.mark.gpu

SHAPE = tuple(int(v) for v in os.environ.get("SKT_ERR_SHAPE", "32,32,32").split(","))
STEPS = int(os.environ.get("SKT_ERR_STEPS", "50"))
REPORT = sorted({1, 10, STEPS // 2, STEPS} - {0})


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_error_growth_vs_fp64(gpu_lib, mode):
    init, dt, speed = small_case(SHAPE)
    if mode == "plain":
        c64 = oracle.Config(semantics=0)
        c32 = oracle.Config(semantics=0)
        cfg = SolverConfig(semantics=0)
    else:
        c64 = oracle.Config(semantics=1, pcg_tol=1e-13, pcg_max_iter=20000)
        c32 = oracle.Config(semantics=1, pcg_tol=1e-9, pcg_max_iter=5000)
        cfg = SolverConfig(precision=1, refine_tol=1e-8)
    s64 = oracle.OracleState(init, np.float64)
    s32 = oracle.OracleState(init, np.float32)
    env = make_env(init, cfg)
    m = s64.sky_mask()
    rows = []
    for step in range(1, STEPS + 1):
        s64.step(c64, dt, speed)
        s32.step(c32, dt, speed)
        env.update_gpu(dt, speed)
        if step in REPORT:
            gpu = {k: rel_l2(env.read(k), s64.a[k], m) for k in SKY}
            f32 = {k: rel_l2(s32.a[k], s64.a[k], m) for k in SKY}
            rows.append((step, gpu, f32))
    env.close()
    print(f"\n{mode}: relative L2 vs the FP64 oracle (GPU / FP32 oracle), {SHAPE} (x,y,z), dt={dt}")
    for step, gpu, f32 in rows:
        print(f"  step {step:4d}: " + "  ".join(f"{k}={gpu[k]:.1e}/{f32[k]:.1e}" for k in SKY))
    step, gpu, f32 = rows[-1]
    bad = {k: (gpu[k], f32[k]) for k in SKY if gpu[k] > max(2.0 * f32[k], 1e-6)}
    assert not bad, (step, bad)
