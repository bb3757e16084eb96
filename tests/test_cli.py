"""The command-line driver (the reference's executable boundary).

CPU: flag parsing, --help, the Morton grid limit and bad flags give the
reference's exit codes without touching a GPU.  GPU: a short run writes the
reference's dump files, and its dumps are byte-identical to dumps taken
through the library API after the same number of steps.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from sph_cuda_gb300 import Asph, preset, _build
from sph_cuda_gb300 import dumpfmt


@pytest.fixture(scope="module")
def cli():
    path = _build.build_cli()
    assert path and os.path.exists(path)
    return path


def _run(cli, *args, cwd=None, timeout=600):
    return subprocess.run([cli, *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=timeout)


def test_help(cli):
    r = _run(cli, "--help")
    assert r.returncode == 0
    for flag in ("--nx", "--dt", "--cfl", "--cfl-interval", "--max-trip", "--strict-cfl", "--dump-every",
                 "--sim-hours", "--dump-stride", "--outdir", "--noise", "--validate", "--quick"):
        assert flag in r.stdout


def test_morton_limit_exits_1(cli):
    r = _run(cli, "--nx", 2000)
    assert r.returncode == 1
    assert "1024 cells/axis" in r.stderr


@pytest.mark.parametrize("args", [["--nx"], ["--dump-stride", "3"], ["--bogus", "1"], ["--preset", "nope"], ["x"]])
def test_bad_arguments_exit_1(cli, args):
    r = _run(cli, *args)
    assert r.returncode == 1
    assert "ERROR" in r.stderr


def test_grid_too_small_is_a_config_error(cli):
    r = _run(cli, "--nx", 2, "--ny", 8, "--nz", 8)
    assert r.returncode == 1
    assert "invalid configuration" in r.stderr


DUMP_LINE = re.compile(r"^(\d+)\s+\+(\d+)\s*s\s+\S+\s+(\S+)\s+CFL")


@pytest.mark.gpu
@pytest.mark.parametrize("validate", [True, False])
def test_cli_dumps_match_library(cli, tmp_path, validate):
    """With --validate the dump is synchronous (the audit reads its state);
    without, the dump's copy and file write overlap the next steps."""
    out = tmp_path / "dumps"
    r = _run(cli, "--nx", 16, "--ny", 16, "--nz", 16, "--dump-every", 30, "--sim-hours", 0.02,
             *(["--validate"] if validate else []), "--dump-stride", 4, 4, "--outdir", out, "--report", 50)
    assert r.returncode == 0, r.stderr
    assert "=== DONE" in r.stdout
    assert ("AUDIT" in r.stdout and "DRIFT" in r.stdout) == validate
    lines = [DUMP_LINE.match(l) for l in r.stdout.splitlines()]
    dumps = [(int(m.group(1)), int(m.group(2))) for m in lines if m]
    files = sorted(os.listdir(out))
    assert len(dumps) == 2 and len(files) == 2
    # the same run through the library: the dump after the same step count is identical
    p = preset("reference", 16, 16, 16)
    p.dump_sx = p.dump_sy = 4
    p.dump_sz = 4
    sim = Asph(p)
    sim.init()
    done = 0
    for (step, t), fn in zip(dumps, files):
        assert fn == "asph_t%06ds.bin" % t
        sim.step(step - done)
        done = step
        mine = sim.dump(str(tmp_path / "lib"))
        assert os.path.basename(mine) == fn
        assert open(out / fn, "rb").read() == open(mine, "rb").read()
        d = dumpfmt.read(str(out / fn))
        assert (d["nx"], d["cx"], d["cz"], d["sx"], d["sz"]) == (16, 4, 4, 4, 4)
    sim.close()


@pytest.mark.gpu
def test_cli_dump_reproduces_the_make_viz_fixture(cli, tmp_path):
    """The committed fixture tests/golden/ours_cli_dump.bin (read by the
    reference's own tools/make_viz.py load() in test_dump_format.py) is the
    last dump of this run: the run still writes a file of the same layout
    and the same fields.  The layout must match exactly; the time and the
    field means are compared to a tolerance, because the 60 s run (about
    250 steps with the closed-loop dt) amplifies any rounding change in the
    step over its course."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_golden import DUMP_FIXTURE_ARGS
    fx = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ours_cli_dump.bin")
    if not os.path.exists(fx):
        pytest.skip("fixture not generated (make_golden.py dump)")
    out = tmp_path / "d"
    r = _run(cli, *DUMP_FIXTURE_ARGS, "--outdir", out)
    assert r.returncode == 0, r.stderr
    last = sorted(os.listdir(out))[-1]
    a, b = dumpfmt.read(str(out / last)), dumpfmt.read(fx)
    for k in ("version", "nx", "ny", "nz", "cx", "cy", "cz", "sx", "sy", "sz", "nfields", "lx", "ly", "lz"):
        assert a[k] == b[k], k
    assert a["t_sim"] == pytest.approx(b["t_sim"], rel=1e-3) and a["dt"] == pytest.approx(b["dt"], rel=1e-2)
    for c, tol in ((0, 1e-4), (1, 1e-2)):   # theta and qv means per coarse cell
        assert np.allclose(a["data"][..., c], b["data"][..., c], rtol=tol, atol=0), c
    assert np.max(np.abs(a["data"][..., 3:6] - b["data"][..., 3:6])) < 0.5   # wind means [m/s]
