"""Generates tests/golden/sounding_ref.npz from the reference's own sounding reader.

The reference's Game/readTable.cpp (readKNMIFile, readDWDFile, initEnvironment), compiled
unmodified for three compile-time grids by oracle/build_ref.py (build_readtable), reads the
synthetic archives of tests/sounding_files.py (every KNMI and DWD case, written to a scratch
directory beside this script and removed afterwards). The file holds, per case, the SHA-256 of each archive member (so a test knows it
regenerated the same bytes), the rows read (six float32 columns; none where the reference found
no rows), and for each grid the per-level columns initEnvironment hands to init. The reference
output is checked to be horizontally uniform (every column a copy) before only one column is
stored.

    python -c "from oracle import build_ref; build_ref.build_readtable()"
    python tests/golden/make_sounding_golden.py
"""
import contextlib
import ctypes
import hashlib
import os
import shutil
import sys
import tempfile
import zipfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build_ref  # noqa: E402
import sounding_files as sf  # noqa: E402

COLUMNS = ("altitude", "pressure", "temperature", "dew_point", "wind_speed", "wind_dir")
SEED_KNMI, SEED_DWD = 3, 7


@contextlib.contextmanager
def _quiet():
    """The reference prints progress with printf: keep it off this script's stdout."""
    sys.stdout.flush()
    fd = os.dup(1)
    with open(os.devnull, "w") as dn:
        os.dup2(dn.fileno(), 1)
        try:
            yield
        finally:
            libc = ctypes.CDLL(None)
            libc.fflush(None)
            os.dup2(fd, 1)
            os.close(fd)


def _lib(grid):
    L = ctypes.CDLL(build_ref.readtable_path(*grid))
    L.ref_read.restype = ctypes.c_long
    L.ref_read.argtypes = [ctypes.c_int, ctypes.c_char_p]
    return L


def main():
    grids = build_ref.build_readtable()
    if not grids:
        raise SystemExit("the reference checkout is needed")
    libs = {g: _lib(g) for g in build_ref.READTABLE_GRIDS}
    out = {"grids": np.array(build_ref.READTABLE_GRIDS, np.float64)}
    tmp = tempfile.mkdtemp(dir=HERE)  # scratch beside this script, removed below
    cwd = os.getcwd()
    os.chdir(tmp)  # the DWD reader takes the station from the path string: pass a bare file name
    try:
        cases = [("knmi", c, SEED_KNMI) for c in sf.KNMI_CASES] + [("dwd", c, SEED_DWD) for c in sf.DWD_CASES]
        for kind, case, seed in cases:
            name = sf.write_dwd(tmp, case, seed) if kind == "dwd" else os.path.basename(sf.write_knmi(tmp, case, seed))
            key = f"{kind}/{case}"
            with zipfile.ZipFile(name) as zf:
                for m in sorted(zf.namelist()):
                    out[f"{key}/sha256/{m}"] = np.frombuffer(hashlib.sha256(zf.read(m)).digest(), np.uint8)
            for g, L in libs.items():
                with _quiet():
                    n = L.ref_read(0 if kind == "knmi" else 1, name.encode())
                X, Y, Z, vox = g
                cols = [np.empty(n, np.float32) for _ in COLUMNS]
                if n:
                    L.ref_rows(*[c.ctypes.data_as(ctypes.c_void_p) for c in cols])
                if g == build_ref.READTABLE_GRIDS[0]:
                    out[f"{key}/n"] = np.int64(n)
                    for k, c in zip(COLUMNS, cols):
                        out[f"{key}/{k}"] = c
                else:  # the reader does not depend on the grid
                    for k, c in zip(COLUMNS, cols):
                        assert np.array_equal(out[f"{key}/{k}"].view(np.uint32), c.view(np.uint32))
                if n == 0 or cols[0].max() < cols[0][0] + Y * vox + vox:
                    continue  # no rows, or the ascent ends below the grid top (the reference reads out of bounds)
                N, G = X * Y * Z, X * Z
                arr = dict(theta=np.empty(N, np.float32), vel=np.empty(3 * N, np.float32), qv=np.empty(N, np.float32),
                           ground_T=np.empty(G, np.float32), ground_p=np.empty(G, np.float32),
                           p3d=np.empty(N, np.float32), p_column=np.empty(Y, np.float32))
                calls = L.ref_init_environment(*[arr[k].ctypes.data_as(ctypes.c_void_p) for k in
                                                 ("theta", "vel", "qv", "ground_T", "ground_p", "p3d", "p_column")])
                assert calls == 1
                gk = f"{key}/init/{X}x{Y}x{Z}_{vox:g}"
                vel = arr["vel"].reshape(Z, Y, X, 3)
                for name_, a in (("theta", arr["theta"].reshape(Z, Y, X)), ("qv", arr["qv"].reshape(Z, Y, X)),
                                 ("p3d", arr["p3d"].reshape(Z, Y, X)), ("u", vel[..., 0]), ("v", vel[..., 1]),
                                 ("w", vel[..., 2])):
                    col = a[0, :, 0]
                    assert np.array_equal(a.view(np.uint32), np.broadcast_to(col[None, :, None], a.shape).view(np.uint32)), name_
                    out[f"{gk}/{name_}"] = col.copy()
                for name_ in ("ground_T", "ground_p"):
                    assert np.all(arr[name_].view(np.uint32) == arr[name_][:1].view(np.uint32))
                    out[f"{gk}/{name_}"] = arr[name_][:1].copy()
                out[f"{gk}/p_column"] = arr["p_column"]
            print(f"{key}: {int(out[f'{key}/n'])} rows")
    finally:
        os.chdir(cwd)
        shutil.rmtree(tmp)
    path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "sounding_ref.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
