"""Reader/writer of the coarse dump format asph_tXXXXXXs.bin.

Format (asph_h100.cu:743-747, 1106-1120; consumer tools/make_viz.py:17-37):
68-byte little-endian header `<2I10i5f`: magic 0x41535048, version 3,
nx, ny, nz, cx, cy, cz, sx, sy, sz, nfields=6, t_sim, dt, lx, ly, lz;
then float32[cx*cy*cz*6] of per-coarse-cell means [theta, qv, qc, u, v, w],
coarse index idx = cxx + cx*(cyy + cy*czz).  The files themselves are
written by the C ABI (asph_dump); this module reads them back.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = 0x41535048
VERSION = 3
HEADER = struct.Struct("<2I10i5f")
FIELDS = ("theta", "qv", "qc", "u", "v", "w")


def read(path: str) -> dict:
    with open(path, "rb") as f:
        raw = f.read()
    return parse(raw)


def parse(raw: bytes) -> dict:
    h = HEADER.unpack(raw[:HEADER.size])
    magic, version, nx, ny, nz, cx, cy, cz, sx, sy, sz, nf, t, dt, lx, ly, lz = h
    if magic != MAGIC:
        raise ValueError("bad magic 0x%08x" % magic)
    data = np.frombuffer(raw, np.float32, count=cx * cy * cz * nf, offset=HEADER.size)
    if len(raw) != HEADER.size + 4 * cx * cy * cz * nf:
        raise ValueError("size mismatch")
    return dict(version=version, nx=nx, ny=ny, nz=nz, cx=cx, cy=cy, cz=cz, sx=sx, sy=sy, sz=sz, nfields=nf,
                t_sim=t, dt=dt, lx=lx, ly=ly, lz=lz, data=data.reshape(cz, cy, cx, nf))


def write(path: str, d: dict) -> None:
    hdr = HEADER.pack(MAGIC, d.get("version", VERSION), d["nx"], d["ny"], d["nz"], d["cx"], d["cy"], d["cz"],
                      d["sx"], d["sy"], d["sz"], d["nfields"], d["t_sim"], d["dt"], d["lx"], d["ly"], d["lz"])
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(np.ascontiguousarray(d["data"], np.float32).tobytes())
