"""Generates tests/golden/ref_16x32x16.npz on a GPU machine.

The reference's own kernels (oracle/_ref/ref_16x32x16.cubin, built from the reference sources by
oracle/build_ref.py) advance the plain 64x64x32 workload profile scaled to 16x16x32 (x,y,z; z
vertical; reference layout X=16, Y=32, Z=16; 100 m cells, dt 0.5 s) for three steps from the
oracle's initial state (reference init noise on). The file holds that initial state, the sky and
ground fields after steps 1 and 3, and the per-step PCG iteration and substep counts.

    python -c "import __graft_entry__ as g; g.build()"   # builds the harness next to the cubin
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import refharness  # noqa: E402
from skewtcloudsim_gb300 import sounding  # noqa: E402

SKY = ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p", "rho")
GROUND = ("Qrs", "Qgr", "Qgs", "Qgi", "Pg", "tg", "Tg")
COLS = ("isenT", "isenQv", "defU", "defW")


def main():
    init, dt, speed = sounding.workload("plain-64x64x32", scale=(16, 16, 32))
    st = oracle.OracleState(init, np.float32)
    out = {"dt": np.float32(dt), "speed": np.float32(speed), "voxel": np.float32(init.voxel),
           "shape": np.array([st.X, st.Y, st.Z], np.int32), "gh": st.gh.copy(), "sim_time0": np.float64(st.sim_time)}
    for k in SKY + GROUND + COLS:
        out["init_" + k] = st.a[k].copy()
    d1 = refharness.run_reference(st, dt, speed, 1)
    for k in SKY + GROUND:
        out["step1_" + k] = st.a[k].copy()
    d2 = refharness.run_reference(st, dt, speed, 2)
    for k in SKY + GROUND:
        out["step3_" + k] = st.a[k].copy()
    out["pcg_iters"] = np.array(d1["pcg_iters"] + d2["pcg_iters"], np.int32)
    out["nsub"] = np.array(d1["nsub"] + d2["nsub"], np.int32)
    path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_16x32x16.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes; pcg iters", out["pcg_iters"].tolist())


if __name__ == "__main__":
    main()
