"""Parity at the benchmark configurations (through the C ABI).

* The FP64 conservation audit (asph_h100.cu:650-668) against the oracle's
  on an identical state: 1e-10 relative per total.
* The config-mode initial state (jittered lattice, seeded bubbles, Gaussian
  noise, RH sounding, then the initial sort and forces, asph_h100.cu:885-921)
  against the oracle's restatement: keys, cell table and positions bit for
  bit; the float fields within the single-step bound of 1e-5 normwise.
* Every stage at the cell geometries the benchmarks run: the 2,097,152-
  particle moist bubble (150.4 x 150.4 x 40 m cells) in a developed,
  clustered state, and the 8:1 cells (160 x 160 x 20 m) of the large
  anisotropic run, checked with the oracle's cell-scaled metric
  (asph_h100.cu:315-320) at 1e-5 normwise.
"""
import numpy as np
import pytest

from sph_cuda_gb300 import Asph, preset
from oracle import oracle
from conftest import normwise
from test_gpu_parity import _stages

pytestmark = pytest.mark.gpu
TOL = 1e-5
FIELDS = ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az", "prs", "dthdt")


def _audit_gate(gpu, orc, s, pmass):
    """Totals 0-3 and 5 are sums of positive terms: relative error.  p_z
    (total 4) is a sum of signed terms: error relative to the sum of the
    magnitudes."""
    for k in (0, 1, 2, 3, 5):
        assert abs(gpu[k] - orc[k]) <= 1e-10 * abs(orc[k]), (k, gpu[k], orc[k])
    scale = pmass * np.sum(np.abs(np.asarray(s["w"], np.float64)))
    assert abs(gpu[4] - orc[4]) <= 1e-10 * max(scale, 1e-300), (gpu[4], orc[4], scale)


@pytest.mark.parametrize("name", ["small65k", "reference"])
def test_audit_matches_oracle(name):
    p = preset(name, 24, 24, 16) if name == "reference" else preset(name)
    sim = Asph(p)
    sim.init()
    for nsteps in (0, 7):
        sim.step(nsteps) if nsteps else None
        s = sim.get_state()
        gpu = sim.audit()
        orc = oracle.audit(p, {k: s[k].astype(np.float64) for k in s})
        _audit_gate(gpu, orc, s, oracle.derived(p)["pmass"])
    sim.close()


def _init_vs_oracle(p):
    sim = Asph(p)
    sim.init()
    st = sim.get_state(FIELDS)
    gs = sim.get_sort()
    o = oracle.initial_state(p)
    assert np.array_equal(gs["keys_sorted"], o["keys_sorted"])
    assert np.array_equal(gs["cell_range"], o["cell_range"])
    for k in ("x", "y", "z"):
        assert np.array_equal(st[k], np.asarray(o[k], np.float32)), k
    for k in ("th", "qv", "qc", "rho", "prs", "ax", "ay", "az"):
        e = normwise(st[k], o[k])
        assert e < TOL, (k, e)
    sim.close()


def test_config_init_matches_oracle_moist_bubble_2m():
    """The 2,097,152-particle moist bubble: 128^3 jittered lattice, three
    seeded bubbles, 80% RH."""
    _init_vs_oracle(preset("bubble2m"))


def test_config_init_matches_oracle_large_run_physics():
    """The large run's physics (95% RH below 1 km, theta noise 0.2 K, 8:1
    cells of 160 x 160 x 20 m) on a 10 x 10 x 10 km box of 1,048,576
    particles, 62 x 62 x 500 cells."""
    p = preset("large16m")
    big = preset("large16m")
    p.nx = p.ny = 62
    p.dx = p.dy = np.float32(10000.0) / np.float32(62)
    p.lat_nx = p.lat_ny = 64
    p.n_particles = 64 * 64 * 256
    assert p.dz == big.dz and p.nz == big.nz
    _init_vs_oracle(p)


def test_stages_at_moist_bubble_2m_developed_state():
    """Every stage on the 2,097,152-particle moist bubble's own state after
    300 steps (clustered updrafts), at its 133 x 133 x 200 cells."""
    p = preset("bubble2m")
    sim = Asph(p)
    sim.init()
    sim.step(300)
    s = sim.get_state(FIELDS)
    assert sim.control()["aborted"] == 0
    sim.close()
    _stages(p, s)


@pytest.mark.parametrize("path", [0, 1])
def test_stages_at_large_run_8to1_cells(path):
    """Every stage at the large run's 8:1 cells (the cell-scaled metric with
    h_xy/h_z = 8), on its physics in a 10 x 10 x 10 km box, after 50 steps;
    brick path and per-target path."""
    p = preset("large16m")
    p.nx = p.ny = 62
    p.dx = p.dy = np.float32(10000.0) / np.float32(62)
    p.lat_nx = p.lat_ny = 64
    p.n_particles = 64 * 64 * 256
    assert p.dx / p.dz == pytest.approx(8.0, rel=0.01)
    sim = Asph(p)
    sim.init()
    sim.step(50)
    s = sim.get_state(FIELDS)
    sim.close()
    _stages(p, s, global_path=path)
