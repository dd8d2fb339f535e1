"""ORACLE — test infrastructure only: a plain-Python restatement of the reference's radiosonde
readers and column interpolation, readTable (Game/readTable.cpp), with the formulas of
Engine/source/math/meteoformulas.cpp it calls. Only the tests and the golden-vector script use it.

Pinned against the reference itself: tests/golden/make_sounding_golden.py runs the reference's
Game/readTable.cpp, compiled unmodified (oracle/build_ref.py: build_readtable), on synthetic
archives and stores what it read and what initEnvironment handed to init.

Arithmetic follows the reference operation by operation in IEEE float32 (numpy float32 scalars,
no fused multiply-add), with the C library's expf, powf, sinf and cosf called through ctypes, and
std::stof restated as correct rounding of the decimal prefix. The DWD reader's search runs on an
emulation of std::stringstream (getline, seekg, tellg and the stream state bits) because the
reference's 100000-byte probes decide which rows are read.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import re
from fractions import Fraction

import numpy as np

f32 = np.float32

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _n in ("expf", "sinf", "cosf"):
    getattr(_libm, _n).restype = ctypes.c_float
    getattr(_libm, _n).argtypes = [ctypes.c_float]
_libm.powf.restype = ctypes.c_float
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]


def expf(x):
    return f32(_libm.expf(float(x)))


def powf(x, y):
    return f32(_libm.powf(float(x), float(y)))


def sinf(x):
    return f32(_libm.sinf(float(x)))


def cosf(x):
    return f32(_libm.cosf(float(x)))


# Engine/include/math/constants.hpp:9,10,11,15,32
RSD = f32(287.0528)
RSW = f32(461.5)
E = RSD / RSW
CPD = f32(1003.5)
PI = f32(3.14159265359)
PROBE = 100000  # Game/readTable.cpp:228,235

COLUMNS = ("altitude", "pressure", "temperature", "dew_point", "wind_speed", "wind_dir")


class ReadError(Exception):
    """Where the reference prints an error and reads nothing, or would read out of bounds."""


_NUM = re.compile(rb"[ \t\n\v\f\r]*([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)")
_SPECIAL = re.compile(rb"[ \t\n\v\f\r]*([+-]?)(inf(?:inity)?|nan)", re.I)
_F32_MAX = Fraction(2) ** 127 * (2 - Fraction(1, 2 ** 23))


def _round_f32(fr: Fraction) -> np.float32:
    """The float32 nearest to an exact rational (ties to even), as strtof rounds."""
    c = f32(float(fr))  # within one float32 step of the answer
    best = None
    for cand in (np.nextafter(c, f32(-np.inf)), c, np.nextafter(c, f32(np.inf))):
        if not np.isfinite(cand):
            continue
        d = abs(Fraction(float(cand)) - fr)
        key = (d, int(np.frombuffer(cand.tobytes(), np.uint32)[0]) & 1)
        if best is None or key < best[0]:
            best = (key, cand)
    return best[1]


def stof(b: bytes):
    """std::stof (strtof): the longest decimal prefix after white space; None where it throws."""
    m = _NUM.match(b)
    if m:
        fr = Fraction(m.group(1).decode())
        if fr == 0:
            return f32(-0.0) if m.group(1).startswith(b"-") else f32(0.0)
        v = _round_f32(fr)
        if abs(fr) > _F32_MAX or not np.isfinite(v) or v == 0 or abs(v) < np.finfo(np.float32).tiny:
            return None  # ERANGE: std::stof throws out_of_range
        return v
    m = _SPECIAL.match(b)
    if m:
        v = f32(np.inf) if m.group(2).lower().startswith(b"inf") else f32(np.nan)
        return -v if m.group(1) == b"-" else v
    return None


class Stream:
    """std::stringstream over bytes, the calls readTable makes: getline, seekg(off, cur), tellg,
    clear, and the eof/fail bits (C++11 semantics: seekg first clears eofbit; tellg and seekg
    construct a sentry, which fails a stream that is not good)."""

    def __init__(self, data: bytes):
        self.d, self.pos, self.eof, self.fail = data, 0, False, False

    def good(self):
        return not (self.eof or self.fail)

    def getline(self, line, delim=b"\n"):
        """Returns (ok, line): ``line`` is kept when the sentry fails, as std::getline leaves it."""
        if not self.good():
            self.fail = True
            return False, line
        j = self.d.find(delim, self.pos)
        if j < 0:
            out = self.d[self.pos:]
            self.pos = len(self.d)
            self.eof = True
            if not out:
                self.fail = True
            return not self.fail, out
        out = self.d[self.pos:j]
        self.pos = j + 1
        return True, out

    def seekg(self, off):
        self.eof = False
        if self.fail:
            return
        p = self.pos + off
        if p < 0 or p > len(self.d):
            self.fail = True
            return
        self.pos = p

    def tellg(self):
        if not self.good():
            self.fail = True
            return -1
        return self.pos

    def clear(self):
        self.eof = self.fail = False


def _fields(line: bytes, sep: bytes):
    """The words `while (std::getline(ss, word, sep))` yields."""
    parts = line.split(sep)
    return parts[:-1] if parts[-1] == b"" else parts


def _lines(text: bytes):
    """The lines `while (std::getline(s, line))` yields."""
    s, out, line = Stream(text), [], b""
    while True:
        ok, line = s.getline(line)
        if not ok:
            return out
        out.append(line)


def _attr(word: bytes, prefix: int):
    if len(word) <= prefix:
        raise ReadError(f"short token {word!r}")
    v = stof(word[prefix:-1])
    if v is None:
        raise ReadError(f"unreadable value {word!r}")
    return v


def _publish(cols, n):
    if any(len(cols[k]) < n for k in COLUMNS):
        raise ReadError("sounding columns of unequal length")
    if n <= 0:
        raise ReadError("no rows")
    return {k: np.array(cols[k][:n], np.float32) for k in COLUMNS}


def read_knmi(xml: bytes):
    """readTable::readKNMIFile (Game/readTable.cpp:27-132) on SynchronizedSoundingData.xml."""
    cols = {k: [] for k in COLUMNS}
    lines = _lines(xml)[1:]  # the first line is skipped
    for row, line in enumerate(lines):
        for tok, w in enumerate(line.split()):
            if tok == 4:
                cols["pressure"].append(_attr(w, 10))
            elif tok == 5:
                cols["temperature"].append(_attr(w, 13) - f32(273.15))
            elif tok == 6:
                rh = _attr(w, 10)
                if row >= len(cols["temperature"]):
                    raise ReadError("humidity before its temperature")
                t = cols["temperature"][row]
                cols["dew_point"].append(t - ((f32(100) - rh) * f32(0.2)) * ((t + f32(273.15)) * f32(0.01)))
            elif tok == 7:
                cols["wind_dir"].append(_attr(w, 9))
            elif tok == 8:
                cols["wind_speed"].append(_attr(w, 11))
            elif w[:8] == b"Altitude":
                cols["altitude"].append(_attr(w, 10))
    return _publish(cols, len(lines) - 1)


def read_dwd(archive_name: str, members: dict):
    """readTable::readDWDFile (Game/readTable.cpp:134-354). ``members`` maps member names to bytes."""
    parts = archive_name.encode().split(b"_")
    station = parts[2] if len(parts) > 2 else b""
    meta_name = b"Metadaten_Sekunde_Aero_" + station + b".txt"
    if meta_name.decode() not in members:
        raise ReadError("no metadata member")
    dates = []
    for line in _lines(members[meta_name.decode()])[1:]:
        for k, w in enumerate(_fields(line, b";")):
            if k == 1:
                if len(w) < 2:
                    raise ReadError("short date field")
                dates.append(w[:-2])
            elif k == 8:
                if stof(w) is None:
                    raise ReadError("unreadable ground temperature")
                break
    if len(dates) < 162:
        raise ReadError("fewer than 162 ascents")
    target = dates[161] + b"12"
    prod_name = (b"produkt_sec_aero_" + dates[0] + b"_" + dates[-1] + b"_" + station + b".txt").decode()
    if prod_name not in members:
        raise ReadError("no product member")
    s = Stream(members[prod_name])
    line = b""
    hit = False
    while not hit:
        _, line = s.getline(line)
        _, line = s.getline(line)
        for k, w in enumerate(_fields(line, b";")):
            if k != 1:
                continue
            if w == target:
                s.seekg(-PROBE)
                if s.fail:
                    s.clear()
                hit = True
                _, line = s.getline(line)
            else:
                s.seekg(PROBE)
            break
        if s.tellg() == -1:
            raise ReadError("could not find date")
    cols = {k: [] for k in COLUMNS}
    slot = {6: "altitude", 7: "pressure", 8: "temperature", 10: "dew_point", 11: "wind_speed", 12: "wind_dir"}
    rows, in_block, done = 0, False, False
    while True:
        ok, line = s.getline(line)
        if not ok or done:
            break
        k = 0
        for w in _fields(line, b";"):
            if not in_block:
                if k == 1 and w == target:
                    in_block = True
                    k -= 1
                k += 1
            if in_block:
                if k == 1:
                    if w != target:
                        in_block, done = False, True
                elif k in slot:
                    v = stof(w)
                    if v is None:
                        raise ReadError(f"unreadable field {k}: {w!r}")
                    cols[slot[k]].append(v)
                k += 1
        if in_block:
            rows += 1
        if s.tellg() == -1:
            raise ReadError("could not find date")
    return _publish(cols, rows)


def _lerp(h1, h2, hc, v1, v2):
    """lerpEnvValue (Game/readTable.cpp:356-362)."""
    if hc == h1:
        return v1
    if hc == h2:
        return v2
    t = (hc - h1) / (h2 - h1)
    return v1 + t * (v2 - v1)


def _ws(t, p):
    """meteoformulas::ws with es (Engine/source/math/meteoformulas.cpp:8-22)."""
    es = f32(0.61078) * expf((f32(17.27) * t) / (t + f32(237.3))) * f32(10.0)
    return (E * es) / (p - es)


def init_environment(cols, X: int, Y: int, Z: int, voxel: float):
    """readTable::initEnvironment (Game/readTable.cpp:364-474) for an X*Y*Z grid (Y vertical):
    dict of theta, vel (AoS u,v,w), qv, ground_T, ground_p, p3d, p_column, float32."""
    alt = [f32(a) for a in cols["altitude"]]
    P = [f32(a) for a in cols["pressure"]]
    T = [f32(a) for a in cols["temperature"]]
    D = [f32(a) for a in cols["dew_point"]]
    S = [f32(a) for a in cols["wind_speed"]]
    W = [f32(a) for a in cols["wind_dir"]]
    n, vox, h0 = len(alt), f32(voxel), alt[0]
    rowi, p_lev, t_lev = [0] * Y, [f32(0)] * Y, [f32(0)] * Y
    y, j, top = f32(0), 0, f32(Y) * vox
    while y < top and j < Y:
        h = y + h0
        i = next((k for k in range(n) if h <= alt[k]), -1)
        if i < 0:
            raise ReadError("the sounding ends below the grid top")
        pi = 0 if i == 0 else i - 1
        p_lev[j] = _lerp(alt[pi] - h0, alt[i] - h0, y, P[pi], P[i])
        t_lev[j] = _lerp(alt[pi] - h0, alt[i] - h0, y, T[pi], T[i])
        rowi[j] = i
        y = y + vox
        j += 1
    if j < Y:
        raise ReadError("levels reach the grid top early")
    p0 = P[0]
    kappa = RSD / CPD
    th = [((t_lev[k] + f32(273.15)) * powf(p0 / p_lev[k], kappa) - f32(273.15)) + f32(273.15) for k in range(Y)]
    u, w, ps, qv = [], [], [], []
    for k in range(Y):
        i = rowi[k]
        pi = 0 if i == 0 else i - 1
        pk = 0 if k == 0 else k - 1
        ang = (W[i] - f32(180.0)) * (PI / f32(180.0))
        u.append(sinf(ang) * S[i])
        w.append(cosf(ang) * S[i])
        hk = f32(k) * vox
        ps.append(_lerp(alt[pi] - h0, alt[i] - h0, hk, p_lev[pk], p_lev[k]))
        qv.append(_ws(_lerp(alt[pi] - h0, alt[i] - h0, hk, D[pi], D[i]), ps[k]))
    # MAC faces: the average with the next cell (clamped); columns are uniform
    uf = [(a + a) / f32(2.0) for a in u]
    wf = [(a + a) / f32(2.0) for a in w]
    col = lambda v: np.broadcast_to(np.array(v, np.float32)[None, :, None], (Z, Y, X)).reshape(-1).copy()
    vel = np.stack([col(uf), col([f32(0)] * Y), col(wf)], axis=-1).reshape(-1)
    G = X * Z
    return dict(theta=col(th), vel=vel, qv=col(qv), ground_T=np.full(G, T[0] + f32(273.15), np.float32),
                ground_p=np.full(G, p0, np.float32), p3d=col(ps), p_column=np.array(p_lev, np.float32))
