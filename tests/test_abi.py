"""C ABI: the library loads, exports every symbol include/asph.h declares,
and its parameter layout, presets and validation behave (no GPU needed)."""
import ctypes
import os
import re

import pytest

from sph_cuda_gb300 import abi, preset, check_params, AsphError
from oracle import oracle
from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "asph.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(asph_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = abi.load_library()
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
        assert n in abi.SIGNATURES, "ctypes signature missing for %s" % n


def test_layout_and_version():
    lib = abi.load_library()
    assert lib.asph_abi_version() == 2
    assert lib.asph_params_size() == ctypes.sizeof(abi.AsphParams)
    assert lib.asph_status_string(3) == b"CFL trip limit exceeded"


@pytest.mark.parametrize("name", ["reference", "small65k", "bubble2m", "large16m", "adjoint262k"])
def test_presets_are_valid(name):
    p = preset(name, 16, 16, 8) if name == "reference" else preset(name)
    check_params(p)
    d = oracle.derived(p)
    assert d["pmass"] > 0 and d["dt_cap"] <= d["dt_static"] + 1e-12


def test_bubble2m_geometry():
    p = preset("bubble2m")
    assert (p.nx, p.ny, p.nz) == (133, 133, 200)
    assert p.n_particles == 128 ** 3 == 2097152
    assert abs(p.dx - 20000.0 / 133) < 1e-3 and p.dz == 40.0
    assert p.sort_every == 1 and p.n_bubbles == 3
    d = oracle.derived(p)
    # the reference clamps the requested dt to its static CFL bound (asph_h100.cu:794-795)
    assert abs(d["dt_cap"] - 0.2) < 1e-6
    assert d["key_bits"] == 24


def test_reference_preset_matches_constexpr():
    p = preset("reference", 128, 128, 64)
    assert (p.dx, p.dy, p.dz, p.th0, p.cs) == (1000.0, 1000.0, 100.0, 300.0, 80.0)
    d = oracle.derived(p)
    rho0 = 1e5 / (287.05 * 300.0)
    assert abs(d["pmass"] / (rho0 * 1e8) - 1) < 1e-6   # PMASS = RHO0*V_CELL (asph_h100.cu:76)
    assert abs(d["mm"] / rho0 - 1) < 1e-6               # mm = PMASS/V_CELL (asph_h100.cu:497)
    assert abs(d["dt_static"] - 0.5) < 1e-7
    assert d["key_bits"] == 21


def test_morton_limit_rejected():
    p = preset("reference", 1025, 8, 8)
    with pytest.raises(AsphError) as e:
        check_params(p)
    assert e.value.status == abi.ASPH_ERR_CONFIG
    assert "1024" in str(e.value)


def test_bad_lattice_rejected():
    p = preset("small65k")
    p.lat_nx = 31
    with pytest.raises(AsphError):
        check_params(p)


def test_oracle_params_struct_is_the_library_layout():
    from oracle import params as op
    assert ctypes.sizeof(op.AsphParams) == ctypes.sizeof(abi.AsphParams)
    ours = [(n, getattr(abi.AsphParams, n).offset, getattr(abi.AsphParams, n).size) for n, _ in abi.AsphParams._fields_]
    theirs = [(n, getattr(op.AsphParams, n).offset, getattr(op.AsphParams, n).size) for n, _ in op.AsphParams._fields_]
    assert ours == theirs


@pytest.mark.parametrize("name,grid", [("reference", (0, 0, 0)), ("reference", (128, 128, 128)),
                                       ("small65k", (0, 0, 0)), ("bubble2m", (0, 0, 0)), ("large16m", (0, 0, 0)),
                                       ("adjoint262k", (0, 0, 0)), ("bubble2m", (66, 66, 0))])
def test_oracle_presets_equal_the_library_presets(name, grid):
    """The CPU benchmark legs build their parameters from the oracle's own
    preset table; it must give the library's parameters bit for bit."""
    from oracle import params as op
    a = preset(name, *grid)
    b = op.preset(name, *grid)
    assert bytes(a) == bytes(b), [k for k in a.as_dict() if a.as_dict()[k] != b.as_dict()[k]]


def test_oracle_workloads_equal_the_bench_workloads():
    import bench
    from oracle import params as op
    for w in ("bubble2m", "bubble524k", "reference128", "large16m"):
        assert bytes(bench.workload_params(w)) == bytes(op.workload(w)), w
