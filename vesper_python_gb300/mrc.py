"""MRC2014 density-map reader/writer.

The reference reads maps with the third-party ``mrcfile`` package
(VESPER_1_prob_new.py:21-56, ``mrcfile.open``).  That package is not a
dependency here, so this module reads and writes the format directly with the
same observable behaviour the reference relies on:

* ``data`` is returned in file order ``(nz, ny, nx)`` (section, row, column),
  ignoring MAPC/MAPR/MAPS exactly as ``mrcfile.open(...).data`` does;
* ``voxel_size`` is ``cella / (mx, my, mz)`` as float32;
* ``origin`` is header words 50-52 as float32.
"""
from __future__ import annotations

import dataclasses
import os
import struct

import numpy as np

__all__ = ["MrcMap", "read_mrc", "write_mrc", "MrcFormatError"]

_MODE_DTYPES = {0: np.int8, 1: np.int16, 2: np.float32, 6: np.uint16, 12: np.float16}


class MrcFormatError(ValueError):
    pass


@dataclasses.dataclass
class MrcMap:
    data: np.ndarray          # (nz, ny, nx)
    nx: int
    ny: int
    nz: int
    voxel_size: np.ndarray    # float32 (x, y, z)
    origin: np.ndarray        # float32 (x, y, z)


def _endian(hdr: bytes) -> str:
    machst = hdr[212:216]
    if machst[0] == 0x11:
        return ">"
    if machst[0] in (0x44, 0x41):
        return "<"
    # fall back on a plausibility check of the mode word
    mode_le = struct.unpack("<i", hdr[12:16])[0]
    return "<" if mode_le in _MODE_DTYPES else ">"


def read_mrc(path: str | os.PathLike) -> MrcMap:
    with open(path, "rb") as f:
        hdr = f.read(1024)
        if len(hdr) != 1024:
            raise MrcFormatError(f"{path}: file shorter than the 1024-byte MRC header")
        e = _endian(hdr)
        nx, ny, nz, mode = struct.unpack(e + "4i", hdr[0:16])
        mx, my, mz = struct.unpack(e + "3i", hdr[28:40])
        cella = np.array(struct.unpack(e + "3f", hdr[40:52]), np.float32)
        nsymbt = struct.unpack(e + "i", hdr[92:96])[0]
        origin = np.array(struct.unpack(e + "3f", hdr[196:208]), np.float32)
        if mode not in _MODE_DTYPES:
            raise MrcFormatError(f"{path}: unsupported MRC mode {mode}")
        if nx <= 0 or ny <= 0 or nz <= 0:
            raise MrcFormatError(f"{path}: bad dimensions {nx}x{ny}x{nz}")
        if nsymbt < 0:
            raise MrcFormatError(f"{path}: negative extended-header size {nsymbt}")
        f.seek(1024 + nsymbt)
        dt = np.dtype(_MODE_DTYPES[mode]).newbyteorder(e)
        count = nx * ny * nz
        raw = np.fromfile(f, dtype=dt, count=count)
        if raw.size != count:
            raise MrcFormatError(f"{path}: data block truncated ({raw.size} of {count} values)")
    data = raw.astype(dt.newbyteorder("="), copy=False).reshape(nz, ny, nx)
    with np.errstate(divide="ignore", invalid="ignore"):
        mxyz = np.array([mx, my, mz], np.float32)
        vs = np.where(mxyz != 0, cella / np.where(mxyz != 0, mxyz, 1), 0).astype(np.float32)
    return MrcMap(data, int(nx), int(ny), int(nz), vs, origin)


def write_mrc(path: str | os.PathLike, data_zyx: np.ndarray, voxel_size: float = 1.0, origin=(0.0, 0.0, 0.0)):
    """Write a float32 MRC2014 file; ``data_zyx`` is in file order (nz, ny, nx)."""
    a = np.ascontiguousarray(data_zyx, dtype="<f4")
    nz, ny, nx = a.shape
    hdr = bytearray(1024)
    struct.pack_into("<4i", hdr, 0, nx, ny, nz, 2)
    struct.pack_into("<3i", hdr, 16, 0, 0, 0)
    struct.pack_into("<3i", hdr, 28, nx, ny, nz)
    struct.pack_into("<3f", hdr, 40, nx * voxel_size, ny * voxel_size, nz * voxel_size)
    struct.pack_into("<3f", hdr, 52, 90.0, 90.0, 90.0)
    struct.pack_into("<3i", hdr, 64, 1, 2, 3)
    struct.pack_into("<3f", hdr, 76, float(a.min()), float(a.max()), float(a.mean()))
    struct.pack_into("<2i", hdr, 88, 1, 0)
    struct.pack_into("<i", hdr, 108, 20140)
    struct.pack_into("<3f", hdr, 196, *[float(o) for o in origin])
    hdr[208:212] = b"MAP "
    hdr[212:216] = bytes([0x44, 0x44, 0x00, 0x00])
    struct.pack_into("<f", hdr, 216, float(a.std()))
    with open(path, "wb") as f:
        f.write(bytes(hdr))
        f.write(a.tobytes())
