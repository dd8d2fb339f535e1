"""The oracle and the GPU library against the reference's OWN kernels, run live.

The reference kernels are compiled unmodified from the reference sources into
oracle/_ref/ref_<X>x<Y>x<Z>.cubin (oracle/build_ref.py) and driven by oracle/ref_harness.cpp.
Each step starts all three implementations from the reference's state after the previous step,
so every comparison is one step from identical inputs. Tolerance: relative L2 <= 1e-5 per sky
field per step, and equal Courant substep counts.

On grids wider than 16 cells in x or z the reference's advectGroundWaterGPU reads
uninitialised shared memory at the interior edges of its 16x16 tiles
(Game/kernelSky.cu:141-164 fills halos only at the domain edge); the garbage can reach the
sky fields within a few steps, as non-finite values or as finite but wrong ones. A step is
compared only while the reference's own output is sound: finite, and within 1e-3 of the oracle
(which otherwise agrees with it to ~1e-6). The 16x32x16 grid has no interior tile edge and is
compared on every step.
"""
import json
import os

import numpy as np
import pytest

import oracle
from helpers import SKY, make_env, push_oracle_to_env, rel_l2, small_case

pytestmark = pytest.mark.gpu

refh = pytest.importorskip("oracle.refharness")


def _clone(st):
    import copy
    c = copy.copy(st)
    c.a = {k: v.copy() for k, v in st.a.items()}
    c.gh = st.gh.copy()
    return c


def _grids():
    try:
        return refh.available_grids()
    except Exception:
        return []


def _record(name, data):
    """Writes the per-step distances to $SKT_REPORT_DIR/refparity_<grid>.json when that folder is set."""
    d = os.environ.get("SKT_REPORT_DIR", "")
    if d and os.path.isdir(d):
        with open(os.path.join(d, f"refparity_{name}.json"), "w") as f:
            json.dump(data, f, indent=1)


@pytest.mark.parametrize("grid", _grids() or [pytest.param(None, marks=pytest.mark.skip("no reference cubins"))])
def test_step_against_reference_kernels(gpu_lib, grid):
    X, Y, Z = grid
    init, dt, speed = small_case((X, Z, Y))
    ref = oracle.OracleState(init, np.float32)
    env = make_env(init)
    cfg = oracle.Config()
    report = []
    for step in range(3):
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
        sound = finite and all(rel_l2(orc.a[k], ref.a[k], m) <= 1e-5 for k in SKY)
        row = {"ref_finite": bool(finite), "ref_sound": bool(sound), "step": step + 1, "ref_pcg": rd["pcg_iters"][0], "oracle_pcg": od["pcg_iters"], "gpu_pcg": gd["pcg_iters"],
               "nsub_ref": rd["nsub"][0], "nsub_gpu": gd["nsub"]}
        for k in SKY:
            row[f"oracle_{k}"] = rel_l2(orc.a[k], ref.a[k], m)
            row[f"gpu_{k}"] = rel_l2(env.read(k), ref.a[k], m)
        report.append(row)
    _record(f"{X}x{Y}x{Z}", report)
    env.close()
    if (X, Y, Z) == (16, 32, 16):
        assert all(r["ref_sound"] for r in report)
    assert report[0]["ref_sound"] or max(X, Z) > 16
    for row in report:
        if not row["ref_sound"]:
            break  # the reference's uninitialised ground-tile halos; later steps start from its corrupted state
        assert row["nsub_ref"] == row["nsub_gpu"], row
        bad = {k: v for k, v in row.items() if (k.startswith("oracle_") or k.startswith("gpu_"))
               and not k.endswith("_pcg") and v > 1e-5}
        assert not bad, (row["step"], bad)
