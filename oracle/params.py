"""Run parameters on the oracle side (TEST INFRASTRUCTURE ONLY).

A ctypes copy of the AsphParams struct of include/asph.h and the named
presets, filled by the oracle's own C restatement of the preset table
(or_params_preset in asph_oracle.c).  The CPU legs of the benchmark and
the oracle itself use this module so that they never import the product
package or load the CUDA library; tests/test_oracle.py holds the struct
layout and every preset equal to the library's, field by field.
"""
from __future__ import annotations

import ctypes as C

MAX_BUBBLES = 8
PRESETS = {"reference": 0, "small65k": 1, "bubble2m": 2, "large16m": 3, "adjoint262k": 4}

_f = C.c_float
_i = C.c_int32
_B = _f * MAX_BUBBLES


class AsphParams(C.Structure):
    """Field-for-field copy of `AsphParams` (include/asph.h)."""
    _fields_ = [
        ("nx", _i), ("ny", _i), ("nz", _i),
        ("dx", _f), ("dy", _f), ("dz", _f),
        ("n_particles", _i), ("init_mode", _i), ("lat_nx", _i), ("lat_ny", _i), ("lat_nz", _i),
        ("jitter", _f), ("seed", C.c_uint32), ("noise", _f),
        ("n_bubbles", _i),
        ("bubble_x", _B), ("bubble_y", _B), ("bubble_z", _B), ("bubble_r", _B), ("bubble_amp", _B),
        ("th0", _f), ("n2", _f), ("cs", _f),
        ("qv_mode", _i), ("qv0", _f), ("rh", _f), ("rh_bl", _f), ("z_bl", _f),
        ("alpha_av", _f), ("beta_av", _f), ("h_av", _f),
        ("sponge_sigma", _f), ("sponge_frac", _f), ("dthdt_cap", _f),
        ("surface_flux", _i), ("c_h", _f), ("c_e", _f), ("beta_moist", _f), ("v_bg", _f), ("dts_skin", _f),
        ("ramp", _f),
        ("qc_auto", _f), ("rate_auto", _f), ("v_rain", _f), ("theta_cap", _f), ("qv_cap", _f),
        ("accretion", _i), ("rain_evap", _i), ("k_accr", _f),
        ("dt_request", _f), ("cfl", _f), ("max_trip", _i), ("strict_cfl", _i), ("adaptive_dt", _i),
        ("sort_every", _i), ("permute_acc", _i), ("pmass", _f),
        ("dump_sx", _i), ("dump_sy", _i), ("dump_sz", _i),
        ("reserved", _i * 16),
    ]

    def copy(self) -> "AsphParams":
        p = AsphParams()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(AsphParams))
        return p

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


def as_pointer(p) -> C.c_void_p:
    """Address of a params struct of either side (this copy or the product
    package's), after checking that it has this layout's size."""
    if C.sizeof(p) != C.sizeof(AsphParams):
        raise TypeError("params struct of %d bytes, expected %d" % (C.sizeof(p), C.sizeof(AsphParams)))
    return C.c_void_p(C.addressof(p))


def preset(name: str = "bubble2m", nx: int = 0, ny: int = 0, nz: int = 0, **overrides) -> AsphParams:
    """A named preset from the oracle's table, then field overrides."""
    from . import oracle
    p = AsphParams()
    st = oracle.lib().or_params_preset(as_pointer(p), PRESETS[name], nx, ny, nz)
    if st != 0:
        raise ValueError("unknown preset %r" % name)
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def workload(name: str) -> AsphParams:
    """The benchmark workloads (the same definitions as bench.py's)."""
    if name == "large16m":
        return preset("large16m")
    if name == "reference128":
        p = preset("reference", 128, 128, 128)
        p.sort_every = 1
        p.dt_request = 0.25
        return p
    p = preset("bubble2m")
    if name == "bubble524k":
        p.nx = p.ny = 66
        p.lat_nx = p.lat_ny = 64
        p.n_particles = 64 * 64 * 128
        for b in range(p.n_bubbles):
            p.bubble_x[b] *= 66 / 133.0
            p.bubble_y[b] *= 66 / 133.0
    return p
