"""The skt_run driver (host C++ over the C ABI and the environmentGPU-shaped adapter) on the CPU:
it reads unpacked KNMI and DWD archives into the same rows as the Python readers (both go
through the library's parser), and rejects bad arguments and missing members with an error
(the GPU side, stepping, is tests/test_gpu_driver.py)."""
import json
import os
import subprocess
import zipfile

import numpy as np
import pytest

import sounding_files as sf
from skewtcloudsim_gb300 import radiosonde


@pytest.fixture(scope="module")
def driver():
    from skewtcloudsim_gb300 import build
    return build.build_driver()


def _unpack(archive_path, directory):
    with zipfile.ZipFile(archive_path) as zf:
        zf.extractall(directory)
    return str(directory)


def _rows(driver, *args):
    out = subprocess.run([driver, *args, "--parse-only"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    d = json.loads(out.stdout, parse_int=float)  # "-0" stays a negative zero
    return np.asarray(d["rows"], np.float64).reshape(-1, 6).astype(np.float32), d["sounding_rows"]


def _want(snd):
    return np.stack([snd.altitude, snd.pressure, snd.temperature, snd.dew_point, snd.wind_speed, snd.wind_dir], axis=1)


@pytest.mark.parametrize("case", sf.KNMI_CASES)
def test_driver_reads_knmi_like_python(driver, tmp_path, case):
    path = sf.write_knmi(str(tmp_path), case, 11)
    rows, n = _rows(driver, "--knmi", _unpack(path, tmp_path / "members"))
    want = _want(radiosonde.read_knmi(path))
    assert n == len(want) > 0
    np.testing.assert_array_equal(rows.view(np.uint32), want.astype(np.float32).view(np.uint32))


@pytest.mark.parametrize("case", ["mid", "first", "tail", "crlf"])
def test_driver_reads_dwd_like_python(driver, tmp_path, case):
    name = sf.write_dwd(str(tmp_path), case, 7)
    path = os.path.join(str(tmp_path), name)
    rows, n = _rows(driver, "--dwd", name, "--dir", _unpack(path, tmp_path / "members"))
    want = _want(radiosonde.read_dwd(path, archive_name=name))
    assert n == len(want) > 0
    np.testing.assert_array_equal(rows.view(np.uint32), want.astype(np.float32).view(np.uint32))


def test_driver_errors(driver, tmp_path):
    r = subprocess.run([driver], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "exactly one of --knmi and --dwd" in r.stderr
    r = subprocess.run([driver, "--knmi", str(tmp_path), "--grid", "8,8"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "--grid" in r.stderr
    r = subprocess.run([driver, "--knmi", str(tmp_path / "none"), "--parse-only"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "SynchronizedSoundingData.xml" in r.stderr
    r = subprocess.run([driver, "--dwd", "x_y_01303_z.zip", "--dir", str(tmp_path), "--parse-only"], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "Metadaten_Sekunde_Aero_01303.txt" in r.stderr
