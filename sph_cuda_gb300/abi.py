"""ctypes mirror of include/asph.h (structs, constants, signatures)."""
from __future__ import annotations

import ctypes as C
import os

ASPH_OK = 0
ASPH_ERR_CUDA = 1
ASPH_ERR_CONFIG = 2
ASPH_ERR_CFL_ABORT = 3
ASPH_ERR_TIMEOUT = 4
ASPH_ERR_ARG = 5
ASPH_ERR_NOMEM = 6
ASPH_ERR_IO = 7
ASPH_ERR_STATE = 8
ASPH_ERR_NONFINITE = 9
ASPH_ERR_DENSE = 10
MAX_CANDIDATES = 65536

PRESET_REFERENCE = 0
PRESET_SMALL_65K = 1
PRESET_BUBBLE_2M = 2
PRESET_LARGE_16M = 3
PRESET_ADJOINT_262K = 4

INIT_REFERENCE = 0
INIT_LATTICE = 1
QV_REFERENCE = 0
QV_RH = 1
MAX_BUBBLES = 8
NPHASES = 6
OPT_PAIR_PATH = 1
OPT_PAIR_SHAPE = 2
OPT_SORT_EVERY = 3
OPT_TARGETS_PER_THREAD = 4
OPT_SORT_AHEAD = 5
NOALLOC_MAX_KEYS = 524288
NBR_CAP = 192
PHASES = ("table_clear", "sort", "gather_kick_drift", "density_eos", "momentum_integrate", "step")

_f = C.c_float
_i = C.c_int32
_B = _f * MAX_BUBBLES


class AsphParams(C.Structure):
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


_FP = C.POINTER(C.c_float)


class AsphHostState(C.Structure):
    _fields_ = [(n, _FP) for n in ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho",
                                   "ax", "ay", "az", "prs", "dthdt")]


STATE_FIELDS = ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az", "prs", "dthdt")


class AsphControl(C.Structure):
    _fields_ = [
        ("simt", C.c_double), ("since_sort", C.c_double),
        ("dt", _f), ("dt_cap", _f), ("dt_floor", _f), ("dt_static", _f), ("dt_required", _f), ("sort_dt", _f),
        ("umax", _f), ("vmax", _f), ("wmax", _f),
        ("step", _i), ("trips", _i), ("sort_count", _i), ("aborted", _i), ("clamp_pending", _i),
        ("do_sort", _i), ("error", _i), ("surf_count", _i), ("deferred", _i),
        ("split_regions", _i),
    ]


# Every entry point of include/asph.h: name -> (restype, argtypes)
_P = C.c_void_p
SIGNATURES = {
    "asph_abi_version": (C.c_int, []),
    "asph_params_size": (C.c_int, []),
    "asph_last_error": (C.c_char_p, []),
    "asph_status_string": (C.c_char_p, [C.c_int]),
    "asph_params_preset": (C.c_int, [C.POINTER(AsphParams), C.c_int, C.c_int, C.c_int, C.c_int]),
    "asph_params_check": (C.c_int, [C.POINTER(AsphParams)]),
    "asph_create": (C.c_int, [C.POINTER(AsphParams), _P, C.POINTER(_P)]),
    "asph_destroy": (C.c_int, [_P]),
    "asph_init": (C.c_int, [_P]),
    "asph_set_state": (C.c_int, [_P, C.POINTER(AsphHostState)]),
    "asph_get_state": (C.c_int, [_P, C.POINTER(AsphHostState)]),
    "asph_get_rain": (C.c_int, [_P, _FP, _FP]),
    "asph_set_rain": (C.c_int, [_P, _FP, _FP]),
    "asph_get_control": (C.c_int, [_P, C.POINTER(AsphControl)]),
    "asph_set_time": (C.c_int, [_P, C.c_double, C.c_float, C.c_int]),
    "asph_sort_build": (C.c_int, [_P]),
    "asph_get_sort": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "asph_kick_drift_flux": (C.c_int, [_P]),
    "asph_density_eos": (C.c_int, [_P]),
    "asph_momentum": (C.c_int, [_P, C.c_int]),
    "asph_rain": (C.c_int, [_P]),
    "asph_cfl": (C.c_int, [_P]),
    "asph_step": (C.c_int, [_P, C.c_int]),
    "asph_step_async": (C.c_int, [_P, C.c_int]),
    "asph_step_kernels": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "asph_sync": (C.c_int, [_P]),
    "asph_step_profiled": (C.c_int, [_P, C.c_int, _FP]),
    "asph_set_option": (C.c_int, [_P, C.c_int, C.c_int]),
    "asph_get_option": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int)]),
    "asph_audit": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "asph_dump": (C.c_int, [_P, C.c_char_p, C.c_char_p, C.c_int]),
    "asph_column_diag": (C.c_int, [_P, _FP]),
    "asph_sort_keys_noalloc": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, _P]),
    "asph_get_neighbours": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "asph_snapshot_create": (C.c_int, [_P, C.POINTER(_P)]),
    "asph_snapshot_save": (C.c_int, [_P, _P]),
    "asph_snapshot_restore": (C.c_int, [_P, _P]),
    "asph_snapshot_destroy": (C.c_int, [_P]),
    "asph_checkpoint_write": (C.c_int, [_P, C.c_char_p]),
    "asph_checkpoint_read": (C.c_int, [_P, C.c_char_p]),
    "asph_ens_create": (C.c_int, [C.POINTER(AsphParams), C.c_int, _P, C.POINTER(_P)]),
    "asph_ens_destroy": (C.c_int, [_P]),
    "asph_ens_size": (C.c_int, [_P]),
    "asph_ens_member": (C.c_int, [_P, C.c_int, C.POINTER(_P)]),
    "asph_ens_init": (C.c_int, [_P]),
    "asph_ens_step": (C.c_int, [_P, C.c_int]),
    "asph_ens_step_async": (C.c_int, [_P, C.c_int]),
    "asph_ens_sync": (C.c_int, [_P]),
    "asph_ens_tune": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int)]),
    "asph_adj_create": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(_P)]),
    "asph_adj_forward": (C.c_int, [_P]),
    "asph_adj_backward": (C.c_int, [_P, _FP, _FP, _FP, _FP, C.POINTER(C.c_double)]),
    "asph_adj_destroy": (C.c_int, [_P]),
    "asph_set_viscosity": (C.c_int, [_P, C.c_float, C.c_float]),
    "asph_dump_begin": (C.c_int, [_P]),
    "asph_dump_finish": (C.c_int, [_P, C.c_char_p, C.c_char_p, C.c_int, _FP]),
    "asph_source_enable": (C.c_int, [_P, C.c_int]),
    "asph_source_set": (C.c_int, [_P, _FP, _FP, _FP]),
    "asph_source_set_device": (C.c_int, [_P, _P]),
    "asph_state_device": (C.c_int, [_P, _P, _P, _P]),
}

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(ROOT, "sph_cuda_gb300", "_build", "libasph.so")
HEADER_PATH = os.path.join(ROOT, "include", "asph.h")

_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load libasph.so (built by sph_cuda_gb300._build).  Raises if absent:
    there is no CPU fallback for any entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libasph.so not built (%s); run __graft_entry__.build()" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.asph_params_size() != C.sizeof(AsphParams):
        raise RuntimeError("AsphParams layout mismatch: library %d bytes, Python %d bytes"
                           % (lib.asph_params_size(), C.sizeof(AsphParams)))
    if path is None:
        _lib = lib
    return lib
