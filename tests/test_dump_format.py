"""Dump format (asph_h100.cu:743-747, 1106-1120; read by tools/make_viz.py)."""
import os
import struct
import sys

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


def _make_viz():
    """tools/make_viz.py of the reference checkout (ASPH_REFERENCE_SRC),
    imported by path; skips where the checkout is not present."""
    import pytest
    sys.path.insert(0, GOLDEN)
    from make_golden import load_make_viz
    mv = load_make_viz()
    if mv is None:
        pytest.skip("reference checkout not present (ASPH_REFERENCE_SRC unset)")
    return mv


def test_our_reader_equals_make_viz_on_a_dump_this_library_wrote():
    """What the reference's own reader, make_viz.load() (make_viz.py:16-37),
    returned for the dump our command-line driver wrote on a GB300
    (tests/golden/make_viz_ours.npz, made by make_golden.py viz) equals our
    reader's parse of the same file, value for value; runs everywhere."""
    fx = os.path.join(GOLDEN, "ours_cli_dump.bin")
    v = np.load(os.path.join(GOLDEN, "make_viz_ours.npz"))
    d = dumpfmt.read(fx)
    assert list(v["head"]) == [d["nx"], d["ny"], d["nz"], d["cx"], d["cy"], d["cz"]]
    assert v["dims"][0] == np.float32(d["t_sim"])
    assert tuple(v["dims"][1:]) == (d["lx"], d["ly"], d["lz"])
    for c, name in enumerate(("theta", "qv", "ql", "u", "v", "w")):
        assert np.array_equal(v[name], d["data"][..., c]), name


def test_make_viz_loads_a_dump_this_library_wrote():
    """The consumer contract run for real: the reference's own reader,
    make_viz.load() (make_viz.py:16-37), parses a dump written on a GB300 by
    this library's command-line driver (fixture from make_golden.py dump),
    and every value equals our reader's."""
    import pytest
    fx = os.path.join(GOLDEN, "ours_cli_dump.bin")
    if not os.path.exists(fx):
        pytest.skip("fixture not generated (make_golden.py dump)")
    mv = _make_viz()
    v = mv.load(fx)
    d = dumpfmt.read(fx)
    assert (v["nx"], v["ny"], v["nz"], v["cx"], v["cy"], v["cz"]) == (d["nx"], d["ny"], d["nz"], d["cx"], d["cy"],
                                                                      d["cz"])
    assert v["t"] == d["t_sim"] and (v["lx"], v["ly"], v["lz"]) == (d["lx"], d["ly"], d["lz"])
    for c, name in enumerate(("theta", "qv", "ql", "u", "v", "w")):
        assert np.array_equal(np.asarray(v["fields"][name], np.float32), d["data"][..., c]), name
    assert np.all(d["data"][..., 0][d["data"][..., 0] != 0] > 250.0)   # theta of non-empty cells


def test_make_viz_loads_the_reference_dump_fixture():
    mv = _make_viz()
    src = os.path.join(GOLDEN, "ref_dump_t300.bin")
    v, d = mv.load(src), dumpfmt.read(src)
    assert np.array_equal(np.asarray(v["fields"]["w"], np.float32), d["data"][..., 5])
