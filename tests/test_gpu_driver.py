"""The skt_run driver (host C++ over the C ABI) steps the same atmosphere as the Python path: the
same KNMI sounding, grid and solver settings give the same 11 prognostic fields, bit for bit,
after a few steps, in both projection modes; and the driver's fast path (each step one graph
launch, the autotuner's launch shapes) gives the same bits as the Python path's default one."""
import json
import subprocess
import zipfile

import numpy as np
import pytest

import sounding_files as sf

pytestmark = pytest.mark.gpu

NAMES = ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p")


@pytest.mark.parametrize("mixed,fast", [(False, False), (True, False), (False, True)], ids=["plain", "mixed", "graph-tuned"])
def test_driver_matches_python_path(gpu_lib, tmp_path, mixed, fast):
    from skewtcloudsim_gb300 import Environment, SolverConfig, build, radiosonde
    driver = build.build_driver()
    path = sf.write_knmi(str(tmp_path), "fine", 3)
    members = tmp_path / "members"
    with zipfile.ZipFile(path) as zf:
        zf.extractall(members)
    out = tmp_path / "raw"
    out.mkdir()
    nx, ny, nz, steps = 32, 24, 32, 3
    args = [driver, "--knmi", str(members), "--grid", f"{nx},{ny},{nz}", "--steps", str(steps), "--dt", "0.5",
            "--raw", str(out)] + (["--mixed"] if mixed else []) + (["--graph", "--tune", str(tmp_path / "tune.json")] if fast else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(s) for s in r.stdout.strip().splitlines()]
    if fast:
        assert "tuning" in lines[1] and not lines[1]["tuning"]["from_cache"]
        lines = lines[:1] + lines[2:]
    assert lines[0]["grid"] == [nx, ny, nz] and len(lines) == steps + 2
    assert all(l["pcg_iters"] > 0 for l in lines[1:-1]) and lines[-1]["cell_steps_per_s"] > 0

    table = radiosonde.ReadTable()
    table.read_knmi_file(path)
    env = Environment(nx, ny, nz, 100.0, SolverConfig(precision=1 if mixed else 0))
    table.init_environment(env, noise=True, noise_seed=100)
    for _ in range(steps):
        env.update_gpu(0.5, 1.0)
    for k in NAMES:
        got = np.fromfile(out / f"{k}.f32", np.float32)
        np.testing.assert_array_equal(got.view(np.uint32), env.read(k).view(np.uint32), err_msg=k)
    env.close()
