"""CPU tests: the oracle itself (runs here, no GPU), the sounding generator, and the C ABI
library's exports (loaded, never called for compute without a GPU)."""
import ctypes
import os

import numpy as np
import pytest

import oracle
from helpers import small_case


def test_sounding_profile_is_hydrostatic_and_saturation_bounded():
    init, dt, speed = small_case((16, 16, 48))
    p = init.p_column.astype(np.float64)
    assert np.all(np.diff(p) < 0)
    assert abs(p[0] - 1000.0) < 1e-3
    from skewtcloudsim_gb300.sounding import ws
    th = init.theta.reshape(init.nz, init.ny, init.nx)[0, :, 0].astype(np.float64)
    T = th * (p / 1000.0) ** (287.0528 / 1003.5)
    qs = ws(T - 273.15, p)
    qv = init.qv.reshape(init.nz, init.ny, init.nx)[0, :, 0]
    assert np.all(qv <= qs * 1.0001)


def test_oracle_step_runs_and_is_finite():
    init, dt, speed = small_case((16, 16, 16))
    st = oracle.OracleState(init, np.float32)
    d = st.step(oracle.Config(), dt, speed)
    m = st.sky_mask()
    for k in ("th", "qv", "u", "v", "w", "p", "rho"):
        assert np.all(np.isfinite(st.a[k][m])), k
    assert d["nsub"] == [1] * 10
    assert d["pcg_iters"] >= 1


def test_oracle_float_and_double_agree():
    """The FP32 oracle against the FP64 oracle of the same method, one step."""
    init, dt, speed = small_case((16, 16, 16))
    a = oracle.OracleState(init, np.float32)
    b = oracle.OracleState(init, np.float64)
    cfg = oracle.Config(semantics=1, pcg_tol=1e-7, pcg_max_iter=400)
    a.step(cfg, dt, speed)
    b.step(cfg, dt, speed)
    m = a.sky_mask()
    for k in ("th", "qv", "p", "rho"):
        err = np.linalg.norm(a.a[k][m] - b.a[k][m]) / np.linalg.norm(b.a[k][m])
        assert err < 1e-5, (k, err)


def test_irradiance_matches_formula():
    L = oracle.lib()
    v = L.oc_irradiance(43200.0, 130, 52.37, 1.0)
    import math
    lat = 52.37 * math.pi / 180
    sd = 0.409 * math.sin(2 * math.pi / 365 * (130 - 81))
    rd = 1 + 0.034 * math.cos(2 * math.pi * 130 / 365)
    sr = (12 - 13) * math.pi / 12
    ref = 1361 * rd * (math.sin(lat) * math.sin(sd) + math.cos(lat) * math.cos(sd) * math.cos(sr))
    assert abs(v - ref) / ref < 1e-5


def test_library_exports_every_declared_symbol():
    """libskewt_gb300.so loads without a GPU and exports every function of include/skewt.h."""
    from skewtcloudsim_gb300 import build, _lib
    path = build.build()
    lib = ctypes.CDLL(path)
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "skewt.h")).read()
    import re
    names = set(re.findall(r"\b(skt_[a-z_0-9]+)\s*\(", hdr))
    assert names, "no declarations parsed"
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert set(_lib.SIGNATURES) == names
    L = _lib.load(path)
    assert L.skt_version().startswith(b"skewt-gb300")


def test_cpp_adapter_compiles_and_links(tmp_path):
    """include/skewt_env.hpp (the environmentGPU-shaped C++ adapter) compiles against skewt.h and
    links libskewt_gb300.so; the program only queries the version (no GPU work)."""
    import subprocess
    from skewtcloudsim_gb300 import build
    lib = build.build()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "use_env.cpp"
    src.write_text('#include "skewt_env.hpp"\n#include <cstdio>\n'
                   'int main() { std::printf("%s\\n", skt_version()); skt_solver_cfg c; skt_default_config(&c);'
                   ' return c.pcg_max_iter == 200 ? 0 : 1; }\n')
    exe = tmp_path / "use_env"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", str(src), "-I", os.path.join(root, "include"), "-L", libdir, "-lskewt_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("skewt-gb300")


def test_c_header_compiles_as_strict_c(tmp_path):
    """include/skewt.h is a C header: a C11 program (-Wall -Wextra -pedantic -Werror) includes it,
    links libskewt_gb300.so and reads the default configuration (no GPU work)."""
    import subprocess
    from skewtcloudsim_gb300 import build
    lib = build.build()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "use_abi.c"
    src.write_text('#include "skewt.h"\n#include <stdio.h>\n'
                   'int main(void) { skt_solver_cfg c; skt_default_config(&c);'
                   ' printf("%s %d\\n", skt_version(), c.pcg_fused); return c.pcg_max_iter == 200 ? 0 : 1; }\n')
    exe = tmp_path / "use_abi"
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", str(src), "-I", os.path.join(root, "include"),
                    "-L", libdir, "-lskewt_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("skewt-gb300") and out.stdout.strip().endswith("1")
