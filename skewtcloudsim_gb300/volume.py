"""Headless view and volume export: what the reference's editor shows in its OpenGL voxel view
(editor::viewSky / viewGround, Game/editor.cpp:1041-1171), without a renderer, and files for
external viewers.

* ``view_volume(env, sky, ground, lo, hi)``: per cell the RGB colour and voxel kind the editor's
  view gives it (``skt_view_volume``, computed on the device).
* ``export_bricks(env, name, threshold)``: a field as sparse 8x8x8 bricks, only those holding a
  value off the background (``skt_export_bricks``, compacted on the device); ``BrickField.dense()``
  rebuilds the array. ``write_bricks`` / ``read_bricks``: a small file format for several such
  fields (a VDB-style leaf layout, optionally zlib-compressed).
* ``write_vti`` / ``read_vti``: VTK XML ImageData (cell data, zlib-compressed appended blocks),
  the format volume viewers such as ParaView open.
* ``save_checkpoint`` / ``load_checkpoint``: the whole prognostic state of an Environment (sky,
  ground, default columns, heightfield, clock, solver settings) in one ``.npz``; a loaded
  environment continues bit-identically.

Layout as everywhere: cell (x, y, z), y vertical, idx = x + y*nx + z*nx*ny.
"""
from __future__ import annotations

import ctypes
import json
import struct
import xml.etree.ElementTree as ET
import zlib
from dataclasses import asdict, dataclass
from typing import Dict, Optional

import numpy as np

from . import _lib
from .environment import (COLUMNS, FIELDS, GROUND_FIELDS, Environment, Parameter, SolverConfig)

BRICK = 8
VOXEL_HIDDEN, VOXEL_SKY, VOXEL_GROUND, VOXEL_GROUND_SURFACE = 0, 1, 2, 3
GROUND_VIEWS = {"T": 0, "Qrs": 1, "Qgr": 2, "Qgs": 3, "Qgi": 4}


def view_volume(env: Environment, sky: int = Parameter.POTTEMP, ground: int = -1, lo=None, hi=None):
    """editor::viewSky (+ viewGround when ``ground`` is 0..4): (rgb (n, 3) float32 in 0..1,
    kind (n,) uint8: 0 hidden, 1 sky, 2 ground below the surface, 3 ground surface)."""
    rgb = np.empty((env.n, 3), np.float32)
    kind = np.empty(env.n, np.uint8)
    lo3 = (ctypes.c_int * 3)(*lo) if lo is not None else None
    hi3 = (ctypes.c_int * 3)(*hi) if hi is not None else None
    env._check(env._L.skt_view_volume(env._h, int(sky), int(ground), lo3, hi3, rgb.ctypes.data_as(_lib.c_float_p),
                                      kind.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), env.n))
    return rgb, kind


@dataclass
class BrickField:
    """A field as sparse bricks: ``coords`` (n, 3) uint32 brick indices (bx, by, bz), ``values``
    (n, 8, 8, 8) indexed [dz, dy, dx] (x fastest in memory)."""
    name: str
    shape: tuple            # (nx, ny, nz)
    coords: np.ndarray
    values: np.ndarray
    background: float = 0.0
    threshold: float = 0.0

    @property
    def count(self) -> int:
        return int(self.coords.shape[0])

    def dense(self) -> np.ndarray:
        """The flat array (idx = x + y*nx + z*nx*ny); cells of absent bricks hold the background."""
        nx, ny, nz = self.shape
        nbx, nby, nbz = (-(-nx // BRICK), -(-ny // BRICK), -(-nz // BRICK))
        pad = np.full((nbz, nby, nbx, BRICK, BRICK, BRICK), self.background, self.values.dtype)
        if self.count:
            c = self.coords.astype(np.int64)
            pad[c[:, 2], c[:, 1], c[:, 0]] = self.values
        full = pad.transpose(0, 3, 1, 4, 2, 5).reshape(nbz * BRICK, nby * BRICK, nbx * BRICK)
        return np.ascontiguousarray(full[:nz, :ny, :nx]).reshape(-1)


def export_bricks(env: Environment, name: str, threshold: float = 0.0, background: float = 0.0,
                  half: bool = False) -> BrickField:
    prm, d = FIELDS[name]
    count = ctypes.c_size_t(0)
    L, h = env._L, env._h
    env._check(L.skt_export_bricks(h, int(prm), int(d), background, threshold, int(half), None, None, 0,
                                   ctypes.byref(count)))
    n = count.value
    dt = np.float16 if half else np.float32
    coords = np.empty((n, 3), np.uint32)
    values = np.empty((n, BRICK, BRICK, BRICK), dt)
    if n:
        env._check(L.skt_export_bricks(h, int(prm), int(d), background, threshold, int(half),
                                       coords.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                       values.ctypes.data_as(ctypes.c_void_p), n, ctypes.byref(count)))
        if count.value != n:
            raise RuntimeError("brick count changed between the two export calls")
    return BrickField(name, (env.nx, env.ny, env.nz), coords, values, float(background), float(threshold))


# ---- brick files --------------------------------------------------------------------------
# header: b"SKTB", u32 version, u32 fields, u32 nx, ny, nz, f32 voxel, u32 brick edge, f64 time
# per field: 32-byte name, u32 dtype (0 float32, 1 float16), u32 codec (0 raw, 1 zlib),
#   f32 background, f32 threshold, u64 bricks, u64 stored bytes, then the coordinates (u32 x 3
#   per brick) and values (512 per brick), together zlib-compressed when codec is 1.
_MAGIC, _VERSION = b"SKTB", 1
_HEAD = struct.Struct("<4sIIIIIfId")
_FIELD = struct.Struct("<32sIIffQQ")


def write_bricks(path, fields: Dict[str, BrickField], voxel: float, sim_time: float = 0.0, compress: bool = True):
    fields = list(fields.values())
    if not fields:
        raise ValueError("no fields")
    shape = fields[0].shape
    if any(f.shape != shape for f in fields):
        raise ValueError("fields of different grids")
    with open(path, "wb") as out:
        out.write(_HEAD.pack(_MAGIC, _VERSION, len(fields), *shape, float(voxel), BRICK, float(sim_time)))
        for f in fields:
            blob = np.ascontiguousarray(f.coords, "<u4").tobytes() + np.ascontiguousarray(
                f.values, "<f2" if f.values.dtype == np.float16 else "<f4").tobytes()
            if compress:
                blob = zlib.compress(blob, 6)
            out.write(_FIELD.pack(f.name.encode()[:32], 1 if f.values.dtype == np.float16 else 0, 1 if compress else 0,
                                  f.background, f.threshold, f.count, len(blob)))
            out.write(blob)


def read_bricks(path):
    """(fields: dict name -> BrickField, meta: dict with shape, voxel, sim_time)."""
    with open(path, "rb") as src:
        data = src.read()
    magic, ver, nf, nx, ny, nz, voxel, edge, t = _HEAD.unpack_from(data, 0)
    if magic != _MAGIC or ver != _VERSION or edge != BRICK:
        raise ValueError("not a brick file of this version")
    off, fields = _HEAD.size, {}
    for _ in range(nf):
        name, dtype, codec, bg, thr, n, nbytes = _FIELD.unpack_from(data, off)
        off += _FIELD.size
        blob = data[off:off + nbytes]
        off += nbytes
        if codec == 1:
            blob = zlib.decompress(blob)
        dt = np.dtype("<f2") if dtype == 1 else np.dtype("<f4")
        coords = np.frombuffer(blob, "<u4", 3 * n).reshape(n, 3).astype(np.uint32)
        values = np.frombuffer(blob, dt, n * BRICK ** 3, offset=12 * n).reshape(n, BRICK, BRICK, BRICK)
        nm = name.rstrip(b"\0").decode()
        fields[nm] = BrickField(nm, (nx, ny, nz), coords, values.astype(dt.newbyteorder("=")), bg, thr)
    return fields, {"shape": (nx, ny, nz), "voxel": voxel, "sim_time": t}


# ---- VTK XML ImageData --------------------------------------------------------------------
_VTK_TYPES = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64", np.dtype(np.uint8): "UInt8",
              np.dtype(np.int32): "Int32", np.dtype(np.float16): None}


def write_vti(path, shape, voxel: float, cell_data: Dict[str, np.ndarray], origin=(0.0, 0.0, 0.0),
              compress: bool = True, block: int = 1 << 20):
    """Cell data on an nx*ny*nz image (cells of edge ``voxel``; arrays of n or (n, k) values in
    the grid's cell order, which is VTK's: x fastest, then y, then z)."""
    nx, ny, nz = shape
    n = nx * ny * nz
    root = ET.Element("VTKFile", type="ImageData", version="1.0", byte_order="LittleEndian", header_type="UInt64")
    if compress:
        root.set("compressor", "vtkZLibDataCompressor")
    img = ET.SubElement(root, "ImageData", WholeExtent=f"0 {nx} 0 {ny} 0 {nz}",
                        Origin=" ".join(str(float(o)) for o in origin), Spacing=f"{voxel} {voxel} {voxel}")
    piece = ET.SubElement(img, "Piece", Extent=f"0 {nx} 0 {ny} 0 {nz}")
    cd = ET.SubElement(piece, "CellData")
    blobs, off = [], 0
    for name, a in cell_data.items():
        a = np.asarray(a)
        if a.dtype == np.float16:
            a = a.astype(np.float32)
        comps = 1 if a.ndim == 1 else a.shape[1]
        if a.shape[0] != n or _VTK_TYPES.get(a.dtype) is None:
            raise ValueError(f"{name}: need {n} cells of float32/float64/uint8/int32")
        raw = np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<")).tobytes()
        if compress:
            parts = [raw[i:i + block] for i in range(0, len(raw), block)] or [b""]
            comp = [zlib.compress(p, 6) for p in parts]
            head = np.array([len(parts), block, len(parts[-1])] + [len(c) for c in comp], "<u8").tobytes()
            blob = head + b"".join(comp)
        else:
            blob = np.array([len(raw)], "<u8").tobytes() + raw
        ET.SubElement(cd, "DataArray", type=_VTK_TYPES[a.dtype], Name=name, NumberOfComponents=str(comps),
                      format="appended", offset=str(off))
        blobs.append(blob)
        off += len(blob)
    ET.SubElement(root, "AppendedData", encoding="raw").text = "@@"
    text = ET.tostring(root, encoding="unicode")
    head, tail = text.split("@@")
    with open(path, "wb") as out:
        out.write(b'<?xml version="1.0"?>\n' + head.encode() + b"_" + b"".join(blobs) + tail.encode())


def read_vti(path):
    """(shape, spacing, cell_data dict) of a file written by ``write_vti``."""
    with open(path, "rb") as src:
        data = src.read()
    start = data.index(b'<AppendedData encoding="raw">') + len(b'<AppendedData encoding="raw">')
    us = data.index(b"_", start) + 1
    root = ET.fromstring(data[:us - 1] + b"</AppendedData></VTKFile>")
    compressed = root.get("compressor") == "vtkZLibDataCompressor"
    img = root.find("ImageData")
    ext = [int(v) for v in img.get("WholeExtent").split()]
    shape = (ext[1] - ext[0], ext[3] - ext[2], ext[5] - ext[4])
    n = shape[0] * shape[1] * shape[2]
    rev = {v: k for k, v in _VTK_TYPES.items() if v}
    out = {}
    for da in img.find("Piece").find("CellData"):
        pos = us + int(da.get("offset"))
        dt = rev[da.get("type")].newbyteorder("<")
        comps = int(da.get("NumberOfComponents", "1"))
        if compressed:
            nb = int(np.frombuffer(data, "<u8", 1, pos)[0])
            head = np.frombuffer(data, "<u8", 3 + nb, pos)
            p = pos + 8 * (3 + nb)
            raw = b""
            for c in head[3:]:
                raw += zlib.decompress(data[p:p + int(c)])
                p += int(c)
        else:
            nbytes = int(np.frombuffer(data, "<u8", 1, pos)[0])
            raw = data[pos + 8:pos + 8 + nbytes]
        a = np.frombuffer(raw, dt).astype(dt.newbyteorder("="))
        out[da.get("Name")] = a.reshape(n, comps) if comps > 1 else a
    return shape, [float(v) for v in img.get("Spacing").split()], out


# ---- checkpoints --------------------------------------------------------------------------
_STATE_FIELDS = ("th", "qv", "qw", "qc", "qr", "qs", "qi", "u", "v", "w", "p", "rho")


def save_checkpoint(env: Environment, path):
    """Every array a step reads from the last one, plus heightfield, clock and solver settings."""
    arrs = {f"sky/{k}": env.read(k) for k in _STATE_FIELDS}
    arrs.update({f"ground/{k}": env.read(k) for k in GROUND_FIELDS})
    arrs.update({f"column/{k}": env.read(k) for k in COLUMNS})
    arrs["gh"] = env.read_ground_height()
    meta = {"grid": [env.nx, env.ny, env.nz, env.voxel], "sim_time": env.stats()["sim_time"], "clock": env._clock,
            "cfg": asdict(env.cfg), "format": 1}
    arrs["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    np.savez(path, **arrs)


def load_checkpoint(path, cfg: Optional[SolverConfig] = None) -> Environment:
    """A new Environment holding the saved state (solver settings from the file unless given)."""
    z = np.load(path)
    meta = json.loads(z["meta"].tobytes().decode())
    nx, ny, nz, voxel = meta["grid"]
    env = Environment(nx, ny, nz, voxel, cfg or SolverConfig(**meta["cfg"]))
    vel = np.stack([z["sky/u"], z["sky/v"], z["sky/w"]], axis=-1).reshape(-1)
    # init sets up the environment (heightfield, flat-terrain flag, derived columns); every array
    # is then overwritten with the saved one
    env.init(z["sky/th"], vel, z["sky/qv"], z["ground/Tg"], z["ground/Pg"], z["sky/p"], z["column/pcol"], z["gh"],
             noise=False)
    for k in _STATE_FIELDS:
        env.write(k, z[f"sky/{k}"])
    for k in GROUND_FIELDS:
        env.write(k, z[f"ground/{k}"])
    for k in COLUMNS:
        env.write(k, z[f"column/{k}"])
    env.set_clock(meta["sim_time"], **meta["clock"])
    return env
