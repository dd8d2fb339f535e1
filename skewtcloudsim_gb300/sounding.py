"""Synthetic soundings and warm bubbles: the scenario ingest that feeds ``init``.

The reference builds its initial state from a DWD radiosonde file
(Game/readTable.cpp:364-474): level ``y`` sits at height ``y * voxel`` (the ground layer is
y = 0), every column is a copy of the interpolated sounding, potential temperature is taken
relative to the *surface* pressure (Engine/source/math/meteoformulas.cpp:184-188 called with
Pt = surface pressure, Game/readTable.cpp:402), vapour is ``ws(dewpoint, p)`` and the wind is
averaged onto MAC faces (Game/readTable.cpp:443-460). No radiosonde file ships with the
reference, so this module generates the same arrays from an analytic sounding:

* temperature ``T(h) = Ts - lapse*h`` up to the tropopause, isothermal above;
* hydrostatic dry pressure from the surface pressure with g = 9.8076, Rsd = 287.0528
  (Game/environment.cu:31,34);
* ``Qv = RH(h) * ws(T, p)`` with the Magnus form of Game/meteoformulas.cuh:16-45;
* ``theta = T * (ps / p)^(Rsd/Cpd)``;
* a horizontal wind profile (``u`` along x, ``w`` along z), zero vertical wind;
* Gaussian warm bubbles ``+dT * exp(-r^2/R^2)`` added to theta.

All arrays use the reference layout ``idx = x + y*X + z*X*Y`` (y vertical) and are float32.
Everything is computed in float64 and rounded once, so the same seed gives the same bytes on
any host.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

G = 9.8076
RSD = 287.0528
CPD = 1003.5
EPS = 287.0528 / 461.5
KAPPA = RSD / CPD


def es_hpa(t_c):
    """Saturation vapour pressure over water in hPa (Game/meteoformulas.cuh:16-20)."""
    return 0.61078 * np.exp((17.27 * t_c) / (t_c + 237.3)) * 10.0


def ws(t_c, p_hpa):
    """Saturation mixing ratio in kg/kg (Game/meteoformulas.cuh:41-45)."""
    e = es_hpa(t_c)
    return EPS * e / (p_hpa - e)


@dataclass
class Bubble:
    x: float  # metres from the x=0 face of cell 0
    h: float  # metres above the ground layer
    z: float
    radius: float
    dT: float


@dataclass
class Sounding:
    Ts: float = 300.0            # surface temperature, K
    lapse: float = 6.5e-3        # K/m
    tropopause: float = 11000.0  # m
    ps: float = 1000.0           # surface pressure, hPa
    rh: Callable[[np.ndarray], np.ndarray] = None   # relative humidity (0..1) vs height
    wind_u: Callable[[np.ndarray], np.ndarray] = None
    wind_w: Callable[[np.ndarray], np.ndarray] = None

    def profile(self, h):
        h = np.asarray(h, dtype=np.float64)
        ht = self.tropopause
        Tt = self.Ts - self.lapse * ht
        T = np.where(h < ht, self.Ts - self.lapse * h, Tt)
        expo = G / (RSD * self.lapse)
        p_lin = self.ps * (np.maximum(self.Ts - self.lapse * np.minimum(h, ht), 1.0) / self.Ts) ** expo
        pt = self.ps * (Tt / self.Ts) ** expo
        p = np.where(h < ht, p_lin, pt * np.exp(-G * (h - ht) / (RSD * Tt)))
        rh = self.rh(h) if self.rh is not None else np.zeros_like(h)
        qv = rh * ws(T - 273.15, p)
        theta = T * (self.ps / p) ** KAPPA
        u = self.wind_u(h) if self.wind_u is not None else np.zeros_like(h)
        w = self.wind_w(h) if self.wind_w is not None else np.zeros_like(h)
        return T, p, qv, theta, u, w


def rh_piecewise(low_rh, low_top, high_rh=0.30, high_h=6000.0):
    """RH ``low_rh`` below ``low_top`` metres, decaying linearly to ``high_rh`` at ``high_h``."""
    def f(h):
        h = np.asarray(h, dtype=np.float64)
        frac = np.clip((h - low_top) / max(high_h - low_top, 1.0), 0.0, 1.0)
        return np.where(h <= low_top, low_rh, low_rh + (high_rh - low_rh) * frac)
    return f


def shear(u_top, depth):
    def f(h):
        return u_top * np.clip(np.asarray(h, dtype=np.float64) / depth, 0.0, 1.0)
    return f


@dataclass
class InitialState:
    """Host arrays for ``init`` (same meaning and units as environmentGPU::init)."""
    nx: int
    ny: int
    nz: int
    voxel: float
    theta: np.ndarray       # K, X*Y*Z
    vel: np.ndarray         # AoS (u, v, w) per cell on MAC faces, X*Y*Z*3
    qv: np.ndarray          # kg/kg
    ground_T: np.ndarray    # K, X*Z
    ground_p: np.ndarray    # hPa, X*Z
    p3d: np.ndarray         # hPa
    p_column: np.ndarray    # hPa, Y
    ground_height: np.ndarray  # int32, X*Z (index of the highest ground cell)

    @property
    def n(self):
        return self.nx * self.ny * self.nz


def make_initial_state(nx: int, ny: int, nz: int, voxel: float, snd: Sounding,
                       bubbles: Sequence[Bubble] = (), wind_noise: float = 0.0,
                       seed: int = 0, ground_height: Optional[np.ndarray] = None) -> InitialState:
    """Build the init arrays. ``ny`` is the vertical size (reference layout)."""
    rng = np.random.default_rng(seed)
    h = np.arange(ny, dtype=np.float64) * voxel
    T, p, qv, theta, u, w = snd.profile(h)
    shape = (nz, ny, nx)  # C order == x + y*X + z*X*Y
    th3 = np.broadcast_to(theta[None, :, None], shape).copy()
    qv3 = np.broadcast_to(qv[None, :, None], shape).copy()
    p3 = np.broadcast_to(p[None, :, None], shape).copy()
    u3 = np.broadcast_to(u[None, :, None], shape).copy()
    w3 = np.broadcast_to(w[None, :, None], shape).copy()
    v3 = np.zeros(shape)
    if bubbles:
        xc = (np.arange(nx) + 0.5) * voxel
        zc = (np.arange(nz) + 0.5) * voxel
        Z3, H3, X3 = np.meshgrid(zc, h, xc, indexing="ij")
        for b in bubbles:
            r2 = (X3 - b.x) ** 2 + (H3 - b.h) ** 2 + (Z3 - b.z) ** 2
            th3 += b.dT * np.exp(-r2 / (b.radius ** 2))
    if wind_noise > 0:
        u3 += rng.uniform(0.0, wind_noise, shape)
        v3 += rng.uniform(0.0, wind_noise, shape)
        w3 += rng.uniform(0.0, wind_noise, shape)
    vel = np.stack([u3, v3, w3], axis=-1).astype(np.float32).reshape(-1)
    gh = np.zeros(nx * nz, np.int32) if ground_height is None else np.asarray(ground_height, np.int32).reshape(-1)
    return InitialState(
        nx=nx, ny=ny, nz=nz, voxel=float(voxel),
        theta=th3.astype(np.float32).reshape(-1),
        vel=vel,
        qv=qv3.astype(np.float32).reshape(-1),
        ground_T=np.full(nx * nz, snd.Ts, np.float32),
        ground_p=np.full(nx * nz, snd.ps, np.float32),
        p3d=p3.astype(np.float32).reshape(-1),
        p_column=p.astype(np.float32),
        ground_height=gh,
    )


# --------------------------------------------------------------------------------------------
# Named workloads: (x, y, z) with z vertical map to the reference layout X = x, Y = z, Z = y.
# --------------------------------------------------------------------------------------------

def workload(name: str, seed: Optional[int] = None, scale: Optional[tuple] = None) -> tuple:
    """Return ``(InitialState, dt, speed)`` for a named workload.

    ``plain-64x64x32``     : 64x64x32, 100 m, dt 0.5 s, one +2 K bubble (R 500 m, 500 m up),
                             RH 85 % below 1.5 km -> 30 % at 6 km, wind U(0, 0.01) noise.
    ``plain-256x256x128``  : 256x256x128, three +1.5..3 K bubbles, westerly shear 0->10 m/s
                             over 3 km.
    ``precision-512x512x256`` : 512x512x256, RH 95 % below 2 km, five bubbles.
    ``scale`` overrides the (x, y, z) size while keeping the profile (tests use small copies).
    """
    cfgs = {
        "plain-64x64x32": (64, 64, 32, 1),
        "plain-256x256x128": (256, 256, 128, 2),
        "precision-512x512x256": (512, 512, 256, 3),
        "stress-1024x1024x256": (1024, 1024, 256, 5),
    }
    gx, gy, gz, cid = cfgs[name]
    if scale is not None:
        gx, gy, gz = scale
    if seed is None:
        seed = 1000 * cid
    rng = np.random.default_rng(seed)
    vox = 100.0
    dt = 0.5
    X, Y, Z = gx, gz, gy
    if cid == 1:
        snd = Sounding(Ts=300.0, lapse=6.5e-3, tropopause=11000.0, ps=1000.0,
                       rh=rh_piecewise(0.85, 1500.0))
        bubbles = [Bubble(X * vox / 2, 500.0, Z * vox / 2, 500.0, 2.0)]
        noise = 0.01
    elif cid == 2:
        snd = Sounding(Ts=300.0, lapse=6.5e-3, tropopause=11000.0, ps=1000.0,
                       rh=rh_piecewise(0.85, 1500.0), wind_u=shear(10.0, 3000.0))
        bubbles = [Bubble(rng.uniform(0.15, 0.85) * X * vox, 500.0, rng.uniform(0.15, 0.85) * Z * vox,
                          500.0, rng.uniform(1.5, 3.0)) for _ in range(3)]
        noise = 0.01
    elif cid == 3:
        snd = Sounding(Ts=300.0, lapse=6.5e-3, tropopause=11000.0, ps=1000.0,
                       rh=rh_piecewise(0.95, 2000.0), wind_u=shear(10.0, 3000.0))
        bubbles = [Bubble(rng.uniform(0.15, 0.85) * X * vox, 500.0, rng.uniform(0.15, 0.85) * Z * vox,
                          500.0, rng.uniform(1.5, 3.0)) for _ in range(5)]
        noise = 0.01
    else:
        vox = 100.0
        dt = 0.4
        snd = Sounding(Ts=303.0, lapse=6.5e-3, tropopause=15000.0, ps=1000.0,
                       rh=rh_piecewise(0.90, 3000.0), wind_u=shear(15.0, 3000.0))
        bubbles = [Bubble(rng.uniform(0.1, 0.9) * X * vox, 500.0, rng.uniform(0.1, 0.9) * Z * vox,
                          500.0, rng.uniform(1.5, 3.0)) for _ in range(12)]
        noise = 0.01
    st = make_initial_state(X, Y, Z, vox, snd, bubbles, wind_noise=noise, seed=seed + 1)
    return st, dt, 1.0


# --------------------------------------------------------------------------------------------
# The batched ensemble: members of uneven sizes, each with its own sounding and bubble.
# --------------------------------------------------------------------------------------------

ENSEMBLE_SIZES = ((64, 64, 32), (96, 96, 64), (128, 128, 64), (192, 192, 96))  # (x, y, z), z vertical


def ensemble_members(n: int = 48, seed: int = 4000, sizes=ENSEMBLE_SIZES, scale: Optional[float] = None) -> list:
    """``n`` members ``(InitialState, dt, speed)``: a size drawn uniformly from ``sizes``, surface
    temperature U[290, 305] K, lapse rate U[5.5, 8] K/km to an 11 km tropopause, RH U[60, 95] %
    below 1.5 km falling to 30 % at 6 km, one bubble of +1.5..3 K (R 500 m, 500 m up) at a random
    horizontal position; 100 m cells, dt 0.5 s. Member m is seeded with ``seed + m``. ``scale``
    shrinks every size by that factor (tests), to multiples of 8 cells (at least 8), which the
    mixed solver's multigrid hierarchy can halve."""
    out = []
    for m in range(n):
        rng = np.random.default_rng(seed + m)
        gx, gy, gz = sizes[int(rng.integers(len(sizes)))]
        if scale is not None:
            gx, gy, gz = (max(8, int(round(v * scale / 8)) * 8) for v in (gx, gy, gz))
        X, Y, Z = gx, gz, gy
        vox = 100.0
        snd = Sounding(Ts=float(rng.uniform(290.0, 305.0)), lapse=float(rng.uniform(5.5e-3, 8e-3)), tropopause=11000.0,
                       ps=1000.0, rh=rh_piecewise(float(rng.uniform(0.60, 0.95)), 1500.0))
        bubble = Bubble(float(rng.uniform(0.2, 0.8)) * X * vox, 500.0, float(rng.uniform(0.2, 0.8)) * Z * vox, 500.0,
                        float(rng.uniform(1.5, 3.0)))
        st = make_initial_state(X, Y, Z, vox, snd, [bubble], wind_noise=0.01, seed=seed + m + 100000)
        out.append((st, 0.5, 1.0))
    return out
