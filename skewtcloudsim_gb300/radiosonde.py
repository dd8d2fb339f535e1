"""Radiosonde ingestion: the reference's readTable (Game/readTable.cpp) over the C ABI.

* ``read_knmi(path)``: readTable::readKNMIFile (Game/readTable.cpp:27-132), a KNMI ``.mwx``
  archive (its member SynchronizedSoundingData.xml).
* ``read_dwd(path)``: readTable::readDWDFile (Game/readTable.cpp:134-354), a DWD
  "sekundenwerte aero" archive. As in the reference the station number is the third
  ``_``-separated field of the path string as given (``assets/input/DWD/sekundenwerte_aero_01303_akt.zip``
  gives 01303), so pass a path whose directories hold no ``_``, or give ``archive_name``.
* ``initial_state(sounding, nx, ny, nz, voxel)``: readTable::initEnvironment
  (Game/readTable.cpp:364-474) on a run-time grid (``ny`` vertical), returning the
  ``sounding.InitialState`` that ``Environment.init_from`` uploads.
* ``ReadTable``: the same three calls under the reference's method names.

The parsing and interpolation run in libskewt_gb300 (``skt_sounding_*``); this module only opens
the zip container (the reference's miniz ``zip_file``) and hands members to the library.
"""
from __future__ import annotations

import ctypes
import zipfile
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from .environment import SktError
from .sounding import InitialState

COLUMNS = ("altitude", "pressure", "temperature", "dew_point", "wind_speed", "wind_dir")


@dataclass
class SoundingData:
    """radioSondeData (Game/readTable.h:9-47): float32 columns of one ascent, bottom up."""
    altitude: np.ndarray     # m above sea level
    pressure: np.ndarray     # hPa
    temperature: np.ndarray  # deg C
    dew_point: np.ndarray    # deg C
    wind_speed: np.ndarray   # m/s
    wind_dir: np.ndarray     # degrees (where the wind comes from)

    @property
    def n(self) -> int:
        return int(self.altitude.size)

    @classmethod
    def from_arrays(cls, **cols) -> "SoundingData":
        return cls(**{k: np.ascontiguousarray(cols[k], np.float32) for k in COLUMNS})


def _reader(zf: zipfile.ZipFile):
    """The skt_archive_read_fn for an open archive: member size (-1 if absent), bytes on request."""
    cache = {}

    def read(ctx, name, buf, cap):
        try:
            key = name.decode("utf-8", "surrogateescape")
            data = cache.get(key)
            if data is None:
                data = cache[key] = zf.read(key)
        except KeyError:
            return -1
        except Exception:  # an unreadable member reads as a missing one: never raise through C
            return -1
        if buf and cap >= len(data):
            ctypes.memmove(buf, data, len(data))
        return len(data)

    return _lib.ARCHIVE_READ_FN(read)


def _take(L, snd: "_lib.Sounding") -> SoundingData:
    try:
        cols = {k: np.ctypeslib.as_array(getattr(snd, k), (snd.n,)).copy() for k in COLUMNS}
    finally:
        L.skt_sounding_free(ctypes.byref(snd))
    return SoundingData(**cols)


def _err(L, st):
    raise SktError(st, L.skt_last_error(None).decode())


def read_knmi(path: str) -> SoundingData:
    """readTable::readKNMIFile: the rows of a KNMI .mwx archive."""
    L = _lib.load()
    snd = _lib.Sounding()
    with zipfile.ZipFile(path) as zf:
        cb = _reader(zf)
        st = L.skt_sounding_read_knmi(cb, None, ctypes.byref(snd))
    if st:
        _err(L, st)
    return _take(L, snd)


def read_dwd(path: str, archive_name: Optional[str] = None) -> SoundingData:
    """readTable::readDWDFile: ascent 161 (12 UTC) of a DWD archive. ``archive_name`` (default:
    ``path`` as given) is the string the station number is taken from."""
    L = _lib.load()
    snd = _lib.Sounding()
    name = (path if archive_name is None else archive_name).encode()
    with zipfile.ZipFile(path) as zf:
        cb = _reader(zf)
        st = L.skt_sounding_read_dwd(name, cb, None, ctypes.byref(snd))
    if st:
        _err(L, st)
    return _take(L, snd)


def initial_state(snd: SoundingData, nx: int, ny: int, nz: int, voxel: float,
                  ground_height: Optional[np.ndarray] = None) -> InitialState:
    """readTable::initEnvironment: the init arrays for an nx*ny*nz grid (ny vertical)."""
    L = _lib.load()
    cols = {k: np.ascontiguousarray(getattr(snd, k), np.float32) for k in COLUMNS}
    n = cols["altitude"].size
    if any(c.size != n for c in cols.values()):
        raise ValueError("sounding columns differ in length")
    s = _lib.Sounding(n, *(cols[k].ctypes.data_as(_lib.c_float_p) for k in COLUMNS))
    N, G = nx * ny * nz, nx * nz
    out = dict(theta=np.empty(N, np.float32), vel=np.empty(3 * N, np.float32), qv=np.empty(N, np.float32),
               ground_T=np.empty(G, np.float32), ground_p=np.empty(G, np.float32), p3d=np.empty(N, np.float32),
               p_column=np.empty(ny, np.float32))
    g = _lib.GridDesc(nx, ny, nz, float(voxel))
    p = [out[k].ctypes.data_as(_lib.c_float_p) for k in ("theta", "vel", "qv", "ground_T", "ground_p", "p3d", "p_column")]
    st = L.skt_sounding_to_init(ctypes.byref(s), ctypes.byref(g), *p)
    if st:
        _err(L, st)
    gh = np.zeros(G, np.int32) if ground_height is None else np.asarray(ground_height, np.int32).reshape(-1)
    return InitialState(nx=nx, ny=ny, nz=nz, voxel=float(voxel), ground_height=gh, **out)


class ReadTable:
    """The reference's readTable (Game/readTable.h:50-92), reading side: one sounding, then
    ``init_environment`` on an Environment (environmentGPU::init with its arrays)."""

    def __init__(self):
        self.data: Optional[SoundingData] = None

    def read_knmi_file(self, path: str) -> SoundingData:
        self.data = read_knmi(path)
        return self.data

    def read_dwd_file(self, path: str) -> SoundingData:
        self.data = read_dwd(path)
        return self.data

    def init_environment(self, env, noise: bool = True, noise_seed: int = 100) -> InitialState:
        if self.data is None:
            raise RuntimeError("no sounding read")
        state = initial_state(self.data, env.nx, env.ny, env.nz, env.voxel)
        env.init_from(state, noise=noise, noise_seed=noise_seed)
        return state
