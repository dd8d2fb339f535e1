"""Headless view and volume export on the CPU: the oracle's colour-scheme evaluation against
the reference's own bee::colorScheme::getColor (Engine/source/rendering/colors.cpp:28-67) filled by
its own editor::setColors (Game/editor.cpp:53-112), both compiled here from the reference sources
(oracle/build_ref.py build_colors; the test is skipped where the reference checkout is absent),
and against hand-computed known answers; the voxel kinds of viewSky / viewGround on a grid with
terrain and a slice, and the brick, VTK and checkpoint file formats (round trips; the GPU side is
tests/test_gpu_volume.py)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import view as ov
from skewtcloudsim_gb300 import volume

f32 = np.float32


def _reference_colors():
    from oracle import build_ref
    so = build_ref.colors_path()
    if not os.path.exists(so):
        try:
            so = build_ref.build_colors()
        except Exception as exc:  # a build failure is a failure, not a skip
            pytest.fail(f"reference colour schemes did not build: {exc}")
    if not so or not os.path.exists(so):
        pytest.skip("the reference checkout is not available to build its colour schemes")
    L = ctypes.CDLL(so)
    L.rc_get_color.argtypes = [ctypes.c_char_p, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
    L.rc_get_color.restype = ctypes.c_int
    return L


@pytest.mark.parametrize("name", sorted(ov.SCHEMES))
def test_schemes_match_the_reference_getcolor(name):
    """Every colour the view can give, bit for bit: each key, its float neighbours on both sides,
    a dense sweep through and beyond the scheme's range, random values, and NaN/Inf."""
    L = _reference_colors()
    keys = ov.SCHEMES[name][0].astype(np.float32)
    lo, hi = float(keys.min()), float(keys.max())
    span = hi - lo
    rng = np.random.default_rng(11)
    vals = np.concatenate([keys, np.nextafter(keys, np.float32(np.inf)), np.nextafter(keys, np.float32(-np.inf)),
                           np.linspace(lo - 0.1 * span, hi + 0.1 * span, 4001, dtype=np.float32),
                           rng.uniform(lo, hi, 4000).astype(np.float32),
                           np.geomspace(1e-6, max(hi, 1e-3), 500).astype(np.float32),
                           np.float32([np.nan, np.inf, -np.inf, 0.0, -0.0])]).astype(np.float32)
    want = np.empty((vals.size, 3), np.float32)
    buf = (ctypes.c_float * 3)()
    for i, v in enumerate(vals):
        assert L.rc_get_color(name.encode(), ctypes.c_float(v), buf) >= 0
        want[i] = buf[:]
    got = ov.get_color(name, vals)
    bad = np.nonzero((got.view(np.uint32) != want.view(np.uint32)).any(axis=1))[0]
    assert bad.size == 0, [(float(vals[i]), got[i].tolist(), want[i].tolist()) for i in bad[:5]]


def test_scheme_known_answers():
    c = ov.get_color
    np.testing.assert_array_equal(c("mixingRatio", [0.0, 0.0005, 0.001, 0.01, 1.0, 5.0, -1.0]),
                                  [[0, 0, 1], [0, 1, 1], [0, 1, 0], [1, 1, 0], [1, 0, 0], [1, 0, 0], [0, 0, 1]])
    # halfway between Blue at 0 and Cyan at 0.0005: green is t = 0.00025 / 0.0005 in float32
    t = (f32(0.00025) - f32(0)) / (f32(0.0005) - f32(0))
    np.testing.assert_array_equal(c("mixingRatio", [0.00025])[0], [0, t, (f32(1) - t) + t])
    # the two keys at -0.01 keep their order: the value itself takes Purple (the first), values
    # between -0.01 and -0.001 blend Blue (the second) into DodgerBlue
    np.testing.assert_array_equal(c("debugColor", [-0.01])[0], f32([0.55, 0, 0.65]))
    mid = c("debugColor", [-0.0055])[0]
    assert mid[0] == 0 and 0.2 < mid[1] < 0.3 and mid[2] == 1
    below = c("debugColor", [-0.5])[0]  # between Purple * 0.2 at -1 and Purple at -0.01
    assert 0.11 < below[0] < 0.55 and below[1] == 0
    first = ov.SCHEMES["debugColor"][1][0]  # Purple * 0.2 in float32
    np.testing.assert_array_equal(first, [f32(0.55) * f32(0.2), 0, f32(0.65) * f32(0.2)])
    np.testing.assert_array_equal(c("debugColor", [np.nan, -2.0, 2.0]), [first, first, [1, 1, 1]])
    # temperature keys are -40 + 273.15f etc. in float32
    np.testing.assert_array_equal(c("TemperatureSky", [f32(-10) + f32(273.15)])[0], [0, 1, 1])
    p = c("pressure", [950.0, 962.5])
    np.testing.assert_array_equal(p[0], f32([1.0, 0.6, 0.6]))
    np.testing.assert_allclose(p[1], [0.8, 0.55, 0.55], atol=1e-6)


def test_view_kinds_with_terrain_and_slice():
    X, Y, Z = 6, 7, 5
    n = X * Y * Z
    rng = np.random.default_rng(0)
    gh = np.zeros(X * Z, np.int32)
    gh[3] = 3  # one column of terrain at x = 3, z = 0
    fields = {k: rng.uniform(0, 2e-3, n).astype(np.float32) for k in ("qv", "qw", "qc", "qr", "qs", "qi")}
    ground = {k: rng.uniform(0, 1e-3, X * Z).astype(np.float32) for k in ("Qrs", "Qgr", "Qgs", "Qgi")}
    ground["T"] = np.full(X * Z, 290.0, np.float32)
    rgb, kind = ov.view(fields, ground, gh, (X, Y, Z), sky=3, ground_view=1)
    k = kind.reshape(Z, Y, X)
    assert (k[:, 0, :][gh.reshape(Z, X) == 0] == 3).all()           # the surface of flat columns
    assert list(k[0, :, 3]) == [2, 2, 2, 3, 1, 1, 1]                 # brown below, surface, sky
    assert (k[:, 1:, :][np.broadcast_to(gh.reshape(Z, 1, X) == 0, (Z, Y - 1, X))] == 1).all()
    # a slice hides the sky outside it, never the ground surface
    _, ks = ov.view(fields, ground, gh, (X, Y, Z), sky=3, ground_view=0, lo=(2, 0, 0), hi=(3, Y, Z))
    ks = ks.reshape(Z, Y, X)
    assert (ks[:, 1:, 2] == 1).all() and (ks[:, 1:, 4] == 0).all()
    assert (ks[:, 0, :][gh.reshape(Z, X) == 0] == 3).all() and ks[0, 3, 3] == 3
    assert (ks[0, :3, 3] == 0).all()  # ground below the surface outside the slice is not drawn
    # the realistic view hides faint cells (total condensate below 1e-4, compared in double)
    for q in ("qw", "qc", "qr", "qs", "qi"):
        fields[q][:] = 0
    fields["qc"][::2] = 2e-5
    fields["qc"][1::2] = 2e-4
    _, kr = ov.view(fields, ground, gh, (X, Y, Z), sky=10)
    sky = (np.arange(n) // X) % Y > gh[(np.arange(n) % X) + (np.arange(n) // (X * Y)) * X]
    assert (kr[sky & (np.arange(n) % 2 == 0)] == 0).all() and (kr[sky & (np.arange(n) % 2 == 1)] == 1).all()


def _bricks(shape, half, rng):
    nbx, nby, nbz = (-(-s // 8) for s in shape)
    sel = rng.random(nbx * nby * nbz) < 0.4
    idx = np.flatnonzero(sel)
    coords = np.stack([idx % nbx, (idx // nbx) % nby, idx // (nbx * nby)], axis=1).astype(np.uint32)
    vals = rng.normal(size=(idx.size, 8, 8, 8)).astype(np.float16 if half else np.float32)
    return volume.BrickField("qc", shape, coords, vals, 0.0, 1e-6)


@pytest.mark.parametrize("half,compress", [(False, True), (True, False), (True, True)])
def test_brick_file_round_trip(tmp_path, half, compress):
    rng = np.random.default_rng(1)
    shape = (19, 12, 9)  # not multiples of 8: edge bricks are partial
    a = _bricks(shape, half, rng)
    b = _bricks(shape, half, rng)
    b.name = "th"
    path = tmp_path / "v.sktb"
    volume.write_bricks(path, {"qc": a, "th": b}, voxel=100.0, sim_time=43210.5, compress=compress)
    fields, meta = volume.read_bricks(path)
    assert meta == {"shape": shape, "voxel": 100.0, "sim_time": 43210.5}
    for want in (a, b):
        got = fields[want.name]
        np.testing.assert_array_equal(got.coords, want.coords)
        assert got.values.dtype == want.values.dtype
        np.testing.assert_array_equal(got.values.view(np.uint16 if half else np.uint32),
                                      want.values.view(np.uint16 if half else np.uint32))
        d = got.dense()
        assert d.shape == (shape[0] * shape[1] * shape[2],)
    # dense() places brick (bx, by, bz) cell (dx, dy, dz) at x = 8 bx + dx, ...
    d = a.dense().reshape(shape[2], shape[1], shape[0])
    i = 0
    bx, by, bz = a.coords[i]
    for dz, dy, dx in ((0, 0, 0), (1, 2, 3), (7, 0, 5)):
        x, y, z = 8 * bx + dx, 8 * by + dy, 8 * bz + dz
        if x < shape[0] and y < shape[1] and z < shape[2]:
            assert d[z, y, x] == a.values[i, dz, dy, dx]


@pytest.mark.parametrize("compress", [True, False])
def test_vti_round_trip(tmp_path, compress):
    rng = np.random.default_rng(2)
    shape = (7, 5, 4)
    n = 7 * 5 * 4
    data = {"th": rng.normal(300, 5, n).astype(np.float32), "rgb": rng.random((n, 3)).astype(np.float32),
            "kind": rng.integers(0, 4, n).astype(np.uint8)}
    path = tmp_path / "v.vti"
    volume.write_vti(path, shape, 64.0, data, compress=compress, block=100)
    got_shape, spacing, got = volume.read_vti(path)
    assert got_shape == shape and spacing == [64.0] * 3
    for k, v in data.items():
        np.testing.assert_array_equal(got[k], v)
    text = path.read_bytes()
    assert text.startswith(b'<?xml version="1.0"?>\n<VTKFile type="ImageData"')
    assert (b'compressor="vtkZLibDataCompressor"' in text) == compress
