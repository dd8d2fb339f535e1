"""bench.py's reference arm runs on the host alone (the oracle port on all host threads) and
prints the contract's JSON line; the byte model of the step is the documented one."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["unit"] == "cell-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["config"]["workload"] == "precision-512x512x256"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "sub-box" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    full = d["full_size_run"]
    assert full["workload"] == "plain-64x64x32" and full["same_config"] is True and full["value"] > 0


def test_step_byte_model():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.step_bytes("plain", 200, 0) == 2534.0 + 60.0 * 200
    assert bench.step_bytes("plain", 200, 0, diffuse_depth=2) == 2534.0 - 800.0 + 60.0 * 200  # two sweeps per pass
    assert bench.STAGE_BYTES["pcg_matvec"] + bench.STAGE_BYTES["pcg_update"] == 60.0
    assert 40.0 < bench.MEASURED_TRAFFIC_PER_CELL["pcg_matvec"] < 41.0
    # the scope table's model of the same step: 2558 B of stages + 52 B per matrix-free iteration
    assert bench.scope_step_bytes("plain", 200, 0) == 2558.0 + 52.0 * 200
