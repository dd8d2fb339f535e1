"""Sounding ingestion (the reference's readTable: KNMI and DWD readers, initEnvironment) on the CPU.

The readers and the column interpolation are host code of libskewt_gb300 (no GPU needed). Both
the library and the oracle restatement are compared bit for bit with the reference itself: the
golden file tests/golden/sounding_ref.npz holds what the reference's Game/readTable.cpp,
compiled unmodified, read from the synthetic archives of tests/sounding_files.py and what its
initEnvironment handed to init on three compile-time grids. Further seeds and run-time grids
compare the library with the oracle.
"""
import ctypes
import hashlib
import io
import os
import subprocess
import zipfile

import numpy as np
import pytest

import sounding_files as sf
from oracle import radiosonde as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = np.load(os.path.join(ROOT, "tests", "golden", "sounding_ref.npz"))
SEED = {"knmi": 3, "dwd": 7}
CASES = [("knmi", c) for c in sf.KNMI_CASES] + [("dwd", c) for c in sf.DWD_CASES]
GRIDS = [tuple(g) for g in GOLDEN["grids"]]


@pytest.fixture(scope="module")
def rs():
    from skewtcloudsim_gb300 import build
    build.build()
    from skewtcloudsim_gb300 import radiosonde
    return radiosonde


def _archive(kind, case, seed=None):
    seed = SEED[kind] if seed is None else seed
    return sf.knmi_archive(case, seed) if kind == "knmi" else sf.dwd_archive(case, seed)


def _members(blob):
    with zipfile.ZipFile(io.BytesIO(blob)) as zf:
        return {m: zf.read(m) for m in zf.namelist()}


def _oracle_read(kind, blob):
    m = _members(blob)
    if kind == "knmi":
        return orc.read_knmi(m["SynchronizedSoundingData.xml"])
    return orc.read_dwd(sf.DWD_ARCHIVE, m)


def _lib_read(rs, kind, blob):
    if kind == "knmi":
        return rs.read_knmi(io.BytesIO(blob))
    return rs.read_dwd(io.BytesIO(blob), archive_name=sf.DWD_ARCHIVE)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _same(a, b, what):
    assert np.array_equal(_bits(a), _bits(b)), f"{what}: max diff {np.nanmax(np.abs(np.float64(a) - np.float64(b)))}"


@pytest.mark.parametrize("kind,case", CASES)
def test_archives_regenerate_the_golden_bytes(kind, case):
    blob = _archive(kind, case)
    for m, data in _members(blob).items():
        want = GOLDEN[f"{kind}/{case}/sha256/{m}"].tobytes()
        assert hashlib.sha256(data).digest() == want, m


@pytest.mark.parametrize("kind,case", CASES)
def test_oracle_reader_matches_reference(kind, case):
    n = int(GOLDEN[f"{kind}/{case}/n"])
    blob = _archive(kind, case)
    if n == 0:
        with pytest.raises(orc.ReadError):
            _oracle_read(kind, blob)
        return
    got = _oracle_read(kind, blob)
    for k in orc.COLUMNS:
        _same(got[k], GOLDEN[f"{kind}/{case}/{k}"], k)


@pytest.mark.parametrize("kind,case", CASES)
def test_library_reader_matches_reference(rs, kind, case):
    from skewtcloudsim_gb300 import SktError
    n = int(GOLDEN[f"{kind}/{case}/n"])
    blob = _archive(kind, case)
    if n == 0:
        with pytest.raises(SktError):
            _lib_read(rs, kind, blob)
        return
    got = _lib_read(rs, kind, blob)
    assert got.n == n
    for k in orc.COLUMNS:
        _same(getattr(got, k), GOLDEN[f"{kind}/{case}/{k}"], k)


def _golden_init(kind, case, grid):
    X, Y, Z, vox = grid
    gk = f"{kind}/{case}/init/{int(X)}x{int(Y)}x{int(Z)}_{vox:g}"
    if f"{gk}/theta" not in GOLDEN:
        return None
    return {k: GOLDEN[f"{gk}/{k}"] for k in ("theta", "qv", "p3d", "u", "v", "w", "ground_T", "ground_p", "p_column")}


def _check_init(arr, want, X, Y, Z):
    col = lambda a: np.ascontiguousarray(a, np.float32).reshape(Z, Y, X)
    for k in ("theta", "qv", "p3d"):
        _same(col(arr[k]), np.broadcast_to(want[k][None, :, None], (Z, Y, X)), k)
    vel = np.ascontiguousarray(arr["vel"], np.float32).reshape(Z, Y, X, 3)
    for c, k in enumerate("uvw"):
        _same(vel[..., c], np.broadcast_to(want[k][None, :, None], (Z, Y, X)), k)
    for k in ("ground_T", "ground_p"):
        _same(arr[k], np.full(X * Z, want[k][0], np.float32), k)
    _same(arr["p_column"], want["p_column"], "p_column")


INIT_CASES = [(kind, case, g) for kind, case in CASES for g in GRIDS if _golden_init(kind, case, g) is not None]


def test_golden_covers_every_grid():
    assert len(INIT_CASES) >= 20
    assert {g for _, _, g in INIT_CASES} == set(GRIDS)


@pytest.mark.parametrize("kind,case,grid", INIT_CASES)
def test_init_environment_matches_reference(rs, kind, case, grid):
    X, Y, Z, vox = int(grid[0]), int(grid[1]), int(grid[2]), float(grid[3])
    want = _golden_init(kind, case, grid)
    cols = _oracle_read(kind, _archive(kind, case))
    _check_init(orc.init_environment(cols, X, Y, Z, vox), want, X, Y, Z)
    snd = rs.SoundingData.from_arrays(**cols)
    st = rs.initial_state(snd, X, Y, Z, vox)
    _check_init(dict(theta=st.theta, qv=st.qv, p3d=st.p3d, vel=st.vel, ground_T=st.ground_T, ground_p=st.ground_p,
                     p_column=st.p_column), want, X, Y, Z)
    assert st.ground_height.shape == (X * Z,) and not st.ground_height.any()


@pytest.mark.parametrize("kind,case,seed,grid", [
    ("knmi", "fine", 11, (7, 50, 3, 80.0)), ("knmi", "coarse", 12, (3, 28, 5, 45.3)),
    ("knmi", "burst", 13, (4, 17, 4, 250.0)), ("dwd", "mid", 14, (5, 64, 2, 31.25)),
    ("dwd", "crlf", 15, (2, 40, 6, 99.9)), ("dwd", "first", 16, (3, 90, 3, 47.0)),
])
def test_library_matches_oracle_more_seeds(rs, kind, case, seed, grid):
    X, Y, Z, vox = grid
    blob = _archive(kind, case, seed)
    want = _oracle_read(kind, blob)
    got = _lib_read(rs, kind, blob)
    for k in orc.COLUMNS:
        _same(getattr(got, k), want[k], k)
    ref = orc.init_environment(want, X, Y, Z, vox)
    st = rs.initial_state(got, X, Y, Z, vox)
    for k in ("theta", "vel", "qv", "ground_T", "ground_p", "p3d", "p_column"):
        _same(getattr(st, k), ref[k], k)


def test_errors(rs):
    from skewtcloudsim_gb300 import SktError
    empty = io.BytesIO()
    zipfile.ZipFile(empty, "w").close()
    with pytest.raises(SktError, match="SynchronizedSoundingData"):
        rs.read_knmi(io.BytesIO(empty.getvalue()))
    with pytest.raises(SktError, match="Metadaten_Sekunde_Aero_04711"):
        rs.read_dwd(io.BytesIO(empty.getvalue()), archive_name=sf.DWD_ARCHIVE)
    blob = sf.dwd_archive("mid", SEED["dwd"])
    with pytest.raises(SktError, match="Metadaten_Sekunde_Aero_.txt"):  # no station field in the name
        rs.read_dwd(io.BytesIO(blob), archive_name="ascents.zip")
    with pytest.raises(SktError, match="could not find date"):
        rs.read_dwd(io.BytesIO(sf.dwd_archive("missing", SEED["dwd"])), archive_name=sf.DWD_ARCHIVE)
    snd = rs.read_knmi(io.BytesIO(sf.knmi_archive("coarse", SEED["knmi"])))
    top = float(snd.altitude.max() - snd.altitude[0])
    with pytest.raises(SktError, match="below the grid top"):
        rs.initial_state(snd, 2, int(top // 100) + 2, 2, 100.0)
    # a short attribute token: the reference would read past its end
    bad = io.BytesIO()
    with zipfile.ZipFile(bad, "w") as zf:
        zf.writestr("SynchronizedSoundingData.xml", "<x>\n<Row a b c P=\"1\" T=\"2\" H=\"3\" D=\"4\" S=\"5\" />\n</x>\n")
    with pytest.raises(SktError, match="unreadable value"):
        rs.read_knmi(io.BytesIO(bad.getvalue()))
    with pytest.raises(orc.ReadError):
        orc.read_knmi(_members(bad.getvalue())["SynchronizedSoundingData.xml"])


def test_read_table_mirror_feeds_init(rs):
    """ReadTable.init_environment hands the interpolated arrays to Environment.init_from."""
    class FakeEnv:
        nx, ny, nz, voxel = 4, 20, 3, 100.0

        def init_from(self, state, noise=True, noise_seed=100):
            self.state, self.noise = state, noise

    env = FakeEnv()
    t = rs.ReadTable()
    with pytest.raises(RuntimeError):
        t.init_environment(env)
    t.data = rs.read_knmi(io.BytesIO(sf.knmi_archive("fine", SEED["knmi"])))
    st = t.init_environment(env, noise=False)
    assert env.state is st and env.noise is False
    ref = orc.init_environment({k: getattr(t.data, k) for k in orc.COLUMNS}, 4, 20, 3, 100.0)
    _same(st.theta, ref["theta"], "theta")
    assert np.all(np.isfinite(st.theta)) and np.all(st.qv > 0)


def test_stream_emulation_matches_libstdcxx(tmp_path):
    """The oracle's std::stringstream model (getline at EOF, seekg past either end, tellg after
    EOF, clear) against libstdc++ on the same operation script."""
    from skewtcloudsim_gb300 import build  # noqa: F401  (g++ is what this needs)
    data = b"head\nline one\nline two;x\n\nlast"
    ops = [("g",), ("s", 7), ("g",), ("t",), ("s", -100), ("t",), ("c",), ("s", 3), ("g",), ("g",), ("g",), ("t",),
           ("g",), ("g",), ("t",), ("s", -5), ("t",), ("c",), ("s", -5), ("g",), ("t",), ("s", 1000), ("g",), ("t",)]
    src = tmp_path / "stream.cpp"
    body = []
    for op in ops:
        if op[0] == "g":
            body.append('{ bool ok = (bool)std::getline(s, line); std::printf("g %d %s|\\n", ok, line.c_str()); }')
        elif op[0] == "s":
            body.append(f's.seekg({op[1]}, std::ios::cur); std::printf("s %d\\n", (int)s.fail());')
        elif op[0] == "t":
            body.append('std::printf("t %ld\\n", (long)s.tellg());')
        else:
            body.append('s.clear(); std::printf("c\\n");')
    lit = data.decode().replace("\n", "\\n")
    src.write_text('#include <cstdio>\n#include <sstream>\n#include <string>\nint main() {\n'
                   f'std::stringstream s(std::string("{lit}")); std::string line;\n' + "\n".join(body) + "\nreturn 0; }\n")
    exe = tmp_path / "stream"
    subprocess.run(["g++", "-std=c++17", str(src), "-o", str(exe)], check=True)
    want = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    s, line, got = orc.Stream(data), b"", []
    for op in ops:
        if op[0] == "g":
            ok, line = s.getline(line)
            got.append(f"g {int(ok)} {line.decode()}|")
        elif op[0] == "s":
            s.seekg(op[1])
            got.append(f"s {int(s.fail)}")
        elif op[0] == "t":
            got.append(f"t {s.tellg()}")
        else:
            s.clear()
            got.append("c")
    assert got == want


def test_cpp_read_table_adapter(tmp_path, rs):
    """include/skewt_env.hpp's ReadTable reads a KNMI text through a member-read callback and
    interpolates it (host code only), matching the Python path."""
    from skewtcloudsim_gb300 import build
    lib = build.build()
    xml = sf.knmi_text("fine", 21)
    (tmp_path / "snd.xml").write_text(xml)
    src = tmp_path / "use_table.cpp"
    src.write_text(r'''
#include "skewt_env.hpp"
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
static std::string g_xml;
static long long rd(void*, const char* name, char* buf, size_t cap) {
    if (std::strcmp(name, "SynchronizedSoundingData.xml") != 0) return -1;
    if (buf && cap >= g_xml.size()) std::memcpy(buf, g_xml.data(), g_xml.size());
    return (long long)g_xml.size();
}
int main(int argc, char** argv) {
    std::ifstream f(argv[1]); std::stringstream ss; ss << f.rdbuf(); g_xml = ss.str();
    skewt::ReadTable t;
    t.readKNMIFile(rd, nullptr);
    skt_grid_desc g{3, 12, 2, 75.0f};
    std::vector<float> th(72), vel(216), qv(72), gT(6), gp(6), p3d(72), pc(12);
    if (skt_sounding_to_init(&t.data(), &g, th.data(), vel.data(), qv.data(), gT.data(), gp.data(), p3d.data(), pc.data()))
        return 2;
    std::printf("%zu", t.data().n);
    for (int y = 0; y < 12; y++) std::printf(" %a", th[y * 3]);
    std::printf("\n");
    return 0;
}
''')
    exe = tmp_path / "use_table"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", str(src), "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lskewt_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path / "snd.xml")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    fields = out.stdout.split()
    snd = rs.read_knmi(io.BytesIO(sf.knmi_archive("fine", 21)))
    st = rs.initial_state(snd, 3, 12, 2, 75.0)
    assert int(fields[0]) == snd.n
    np.testing.assert_array_equal(np.array([float.fromhex(v) for v in fields[1:]], np.float32), st.theta.reshape(2, 12, 3)[0, :, 0])
