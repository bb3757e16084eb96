"""Dump format (asph_h100.cu:743-747, 1106-1120; read by tools/make_viz.py)."""
import os
import struct

import numpy as np

from sph_cuda_gb300 import dumpfmt
from conftest import GOLDEN


def test_reference_dump_fixture_parses_and_roundtrips(tmp_path):
    src = os.path.join(GOLDEN, "ref_dump_t300.bin")
    d = dumpfmt.read(src)
    assert (d["nx"], d["ny"], d["nz"]) == (128, 128, 64)
    assert (d["cx"], d["cy"], d["cz"]) == (13, 13, 22)
    assert (d["sx"], d["sy"], d["sz"], d["nfields"]) == (10, 10, 3, 6)
    assert abs(d["t_sim"] - 300.03) < 0.01
    out = tmp_path / "copy.bin"
    dumpfmt.write(str(out), d)
    assert open(out, "rb").read() == open(src, "rb").read()


def test_make_viz_struct_layout():
    # make_viz.py unpacks '<2I10i5f' from the first 68 bytes (make_viz.py:19)
    assert struct.calcsize("<2I10i5f") == 68 == dumpfmt.HEADER.size
    raw = open(os.path.join(GOLDEN, "ref_dump_t300.bin"), "rb").read()
    h = struct.unpack("<2I10i5f", raw[:68])
    assert h[0] == 0x41535048 and h[1] == 3
    vals = np.frombuffer(raw[68:], np.float32)
    assert vals.size == h[5] * h[6] * h[7] * h[11]
