"""ORACLE — test infrastructure only: a numpy restatement of the reference editor's voxel view,
editor::viewSky and editor::viewGround (Game/editor.cpp:1041-1171), with the colour schemes of
editor::setColors (Game/editor.cpp:53-112) evaluated as bee::colorScheme::getColor does
(Engine/source/rendering/colors.cpp:28-67; Lerp, Engine/include/math/math.hpp:11-15), and the
cell-centred wind of environment::getUV (Game/environment.cpp:2083-2095). Float32 arithmetic
operation by operation (numpy float32 arrays, no fused multiply-add).

The colour-scheme evaluation is pinned to the reference itself: tests/test_cpu_volume.py compares
get_color bit for bit with the reference's own getColor and setColors, compiled from the reference
sources (oracle/build_ref.py build_colors, oracle/ref_colors.cpp). The per-voxel choices of
viewSky/viewGround (which field feeds which scheme, the hidden and ground voxels) are restated from
the source: the reference evaluates them only while drawing through OpenGL.
"""
import numpy as np

f32 = np.float32

# bee::Colors (Engine/include/rendering/colors.hpp:34-47) as RGB
BLACK, WHITE, RED, GREEN, BLUE = (0, 0, 0), (1, 1, 1), (1, 0, 0), (0, 1, 0), (0, 0, 1)
DODGER, ORANGE, CYAN, YELLOW, PURPLE = (0, 0.5, 1), (1, 0.66, 0), (0, 1, 1), (1, 1, 0), (0.55, 0, 0.65)


def _scheme(pairs):
    """(keys, colours) in the order getColor sees them: std::sort of fewer than 16 entries is an
    insertion sort, so equal keys keep the order in which they were added."""
    order = sorted(range(len(pairs)), key=lambda i: (np.float32(pairs[i][0]), i))
    keys = np.array([pairs[i][0] for i in order], np.float32)
    cols = np.array([pairs[i][1] for i in order], np.float32)
    return keys, cols


def _k(v):
    return f32(v)


SCHEMES = {
    "TemperatureSky": _scheme([(_k(-40) + f32(273.15), BLUE), (_k(40) + f32(273.15), RED), (_k(-10) + f32(273.15), CYAN),
                               (_k(10) + f32(273.15), GREEN), (_k(20) + f32(273.15), YELLOW)]),
    "mixingRatio": _scheme([(0.0, BLUE), (1.0, RED), (0.0005, CYAN), (0.001, GREEN), (0.01, YELLOW)]),
    "velField": _scheme([(0, BLUE), (100, RED), (10, CYAN), (25, GREEN), (50, YELLOW)]),
    "debugColor": _scheme([(-1, tuple(f32(c) * f32(0.2) for c in PURPLE)), (1, WHITE), (-0.01, PURPLE), (-0.01, BLUE),
                           (-0.001, DODGER), (-0.0001, CYAN), (0.0, GREEN), (0.0001, YELLOW), (0.001, ORANGE),
                           (0.01, RED), (0.1, (1.0, 0.8, 0.72))]),
    "realistic": _scheme([(0.0, BLUE), (1.0, BLACK), (0.0005, (0.6, 0.9, 1.0)), (0.001, WHITE), (0.005, (0.8, 0.8, 0.8)),
                          (0.01, (0.4, 0.4, 0.4))]),
    "pressure": _scheme([(0.0, PURPLE), (1050.0, WHITE), (100.0, (0.3, 0.0, 0.75)), (200.0, (0.1, 0.8, 0.9)),
                         (300.0, (0.0, 0.8, 1.0)), (400.0, (0.0, 0.4, 1.0)), (600.0, (0.0, 0.8, 0.8)),
                         (700.0, (0.0, 1.0, 0.0)), (800.0, (0.4, 0.8, 0.0)), (900.0, (0.8, 0.0, 0.0)),
                         (950.0, (1.0, 0.6, 0.6)), (975.0, (0.6, 0.5, 0.5)), (1000.0, (0.2, 0.2, 0.2))]),
}


def get_color(name, v):
    """bee::colorScheme::getColor for an array of values: (n, 3) float32."""
    keys, cols = SCHEMES[name]
    v = np.asarray(v, np.float32)
    n = keys.size
    it = np.searchsorted(keys, v, side="left")  # lower_bound
    it = np.where(np.isnan(v), 0, it)           # no key compares below NaN
    out = np.empty(v.shape + (3,), np.float32)
    end = it == n
    itc = np.minimum(it, n - 1)
    exact = ~end & ((it == 0) | (keys[itc] == v))
    lo = np.maximum(it - 1, 0)
    prev = ~end & ~exact & (v == keys[lo])
    mid = ~(end | exact | prev)
    out[end] = cols[n - 1]
    out[exact] = cols[itc[exact]]
    out[prev] = cols[lo[prev]]
    if mid.any():
        a, b, vm = keys[lo[mid]], keys[itc[mid]], v[mid]
        t = (vm - a) / (b - a)
        t = np.where(f32(1.0) < t, f32(1.0), t)
        t = np.where(f32(0.0) < t, t, f32(0.0)).astype(np.float32)
        s = (f32(1.0) - t).astype(np.float32)
        out[mid] = cols[lo[mid]] * s[:, None] + cols[itc[mid]] * t[:, None]
    return out


def view(fields, ground, gh, shape, sky, ground_view=-1, lo=None, hi=None):
    """editor::viewSky + viewGround: (rgb (n, 3), kind (n,)). ``fields`` holds th, qv..qi, u, v,
    w, p and debug2/debug3 as needed (flat, idx = x + y*X + z*X*Y); ``ground`` holds T, Qrs, Qgr,
    Qgs, Qgi, P (X*Z); sky is the reference's parameter number (0 POTTEMP .. 12 DEBUG3)."""
    X, Y, Z = shape
    n = X * Y * Z
    idx = np.arange(n)
    x, y, z = idx % X, (idx // X) % Y, idx // (X * Y)
    cg = x + z * X
    g = np.asarray(gh)[cg]
    lo = lo if lo is not None else (0, 0, 0)
    hi = hi if hi is not None else (X, Y, Z)
    box = (x >= lo[0]) & (x < hi[0]) & (y >= lo[1]) & (y < hi[1]) & (z >= lo[2]) & (z < hi[2])
    rgb = np.zeros((n, 3), np.float32)
    kind = np.zeros(n, np.uint8)
    surf = y == g
    below = box & (y < g) & ~surf
    sky_m = box & (y > g)
    if ground_view >= 0:
        gname = ["T", "Qrs", "Qgr", "Qgs", "Qgi"][ground_view]
        rgb[surf] = get_color("TemperatureSky" if ground_view == 0 else "mixingRatio", np.asarray(ground[gname])[cg[surf]])
        kind[surf] = 3
    rgb[below] = np.array([0.5, 0.3, 0.0], np.float32)
    kind[below] = 2
    f = {k: np.asarray(v, np.float32) for k, v in fields.items()}
    m = sky_m
    kind[m] = 1
    if sky == 0:  # temperature: potentialTemp(theta - 273.15, ground P, p) + 273.15
        tz = f["th"][m] - f32(273.15)
        kappa = f32(287.0528) / f32(1003.5)
        fac = np.power(f["p"][m] / np.asarray(ground["P"], np.float32)[cg[m]], kappa).astype(np.float32)
        t = ((tz + f32(273.15)) * fac - f32(273.15)) + f32(273.15)
        rgb[m] = get_color("TemperatureSky", t)
    elif sky in (1, 2, 3, 4, 5, 6):
        rgb[m] = get_color("mixingRatio", f[["qv", "qw", "qc", "qr", "qs", "qi"][sky - 1]][m])
    elif sky == 7:  # |getUV|: the z term pairs w with the v of the cell behind
        u, v, w = f["u"], f["v"], f["w"]
        ii = idx[m]
        pu = np.where(x[m] == 0, u[ii], u[np.maximum(ii - 1, 0)])
        pv = np.where(y[m] == 0, f32(0), v[np.maximum(ii - X, 0)])
        pw = np.where(z[m] == 0, f32(0), v[np.maximum(ii - X * Y, 0)])
        cx = (pu + u[ii]) / f32(2)
        cy = (pv + v[ii]) / f32(2)
        cz = (pw + w[ii]) / f32(2)
        rgb[m] = get_color("velField", np.sqrt((cx * cx + cy * cy) + cz * cz))
    elif sky == 9:
        rgb[m] = get_color("pressure", f["p"][m])
    elif sky == 10:  # the "realistic" view; cells below 1e-4 (a double compare) are not drawn
        s = (((f["qw"] + f["qc"]) + f["qr"]) + f["qs"]) + f["qi"]
        rgb[m] = get_color("realistic", s[m])
        faint = m & (s.astype(np.float64) < 0.0001)
        rgb[faint] = 0
        kind[faint] = 0
    elif sky in (11, 12):
        rgb[m] = get_color("debugColor", f["debug2" if sky == 11 else "debug3"][m])
    else:
        raise ValueError("no view for this parameter")
    return rgb, kind
