"""ctypes wrapper of the FP64 CPU oracle (asph_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the product package.
Each function restates one block of asph_h100.cu (cited in the C file).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from oracle.params import AsphParams, as_pointer as _p  # noqa: E402

LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None

_D = C.POINTER(C.c_double)
_U32 = C.POINTER(C.c_uint32)
_I32 = C.POINTER(C.c_int32)
_U8 = C.POINTER(C.c_uint8)
_PP = C.c_void_p   # an AsphParams of either side, by address


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from . import build_oracle  # type: ignore
            build_oracle.build_oracle()
        _lib = C.CDLL(LIB)
        sig = {
            "or_num_threads": (C.c_int, []),
            "or_set_threads": (None, [C.c_int]),
            "or_key_bits": (C.c_int, [_PP]),
            "or_init_reference": (C.c_int, [_PP, _D, _D, _D, _D, _D, _D]),
            "or_init_lattice": (C.c_int, [_PP, _D, _D, _D, _D, _D, _D]),
            "or_keys": (C.c_int, [_PP, _D, _D, _D, _U32]),
            "or_stable_sort": (C.c_int, [C.c_int, C.c_int, _U32, _U32, _U32]),
            "or_cell_table": (C.c_int, [_PP, _D, _D, _D, _I32]),
            "or_surface": (C.c_int, [_PP, _D, _U8]),
            "or_kick_drift_flux": (C.c_int, [_PP, C.c_double, C.c_double, C.c_int, _U8, _D, _D, _D, _D, _D, _D,
                                             _D, _D, _D, _D, _D]),
            "or_density_eos": (C.c_int, [_PP, C.c_double, _D, _D, _D, _D, _I32, _D, _D, _D, _D, _D, _D, _D]),
            "or_momentum": (C.c_int, [_PP, C.c_double, C.c_int, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _I32,
                                      _D, _D, _D, _D]),
            "or_rain": (C.c_int, [_PP, C.c_double, _D, _D, _D, _D]),
            "or_cfl": (C.c_int, [_PP, _D, _D]),
            "or_audit": (C.c_int, [_PP, _D, _D, _D, _D, _D, _D, _D, _D]),
            "or_helpers": (C.c_int, [_PP, C.c_int, _D, _D]),
            "or_hash_noise": (C.c_int, [C.c_int, _I32, C.POINTER(C.c_float)]),
            "or_derived": (C.c_int, [_PP, _D]),
            "or_params_preset": (C.c_int, [_PP, C.c_int, C.c_int, C.c_int, C.c_int]),
            "or_run": (C.c_int, [_PP, C.c_int, C.POINTER(_D), _D, _D, _D]),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def _d(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _pd(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _chk(st: int) -> None:
    if st != 0:
        raise RuntimeError("oracle status %d" % st)


def threads() -> int:
    return lib().or_num_threads()


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def key_bits(p: AsphParams) -> int:
    return lib().or_key_bits(_p(p))


def derived(p: AsphParams) -> dict:
    out = np.zeros(12)
    lib().or_derived(_p(p), _pd(out))
    names = ["pmass", "mm", "dt_static", "dt_cap", "dt_floor", "lx", "ly", "lz", "key_bits", "h_av", "a_exner",
             "v_cell"]
    return dict(zip(names, out.tolist()))


def init_reference(p: AsphParams) -> dict:
    N = p.n_particles
    out = {k: np.zeros(N) for k in ("x", "y", "z", "th", "qv", "rho")}
    _chk(lib().or_init_reference(_p(p), *[_pd(out[k]) for k in ("x", "y", "z", "th", "qv", "rho")]))
    return out


def init_lattice(p: AsphParams) -> dict:
    N = p.n_particles
    out = {k: np.zeros(N) for k in ("x", "y", "z", "th", "qv", "rho")}
    _chk(lib().or_init_lattice(_p(p), *[_pd(out[k]) for k in ("x", "y", "z", "th", "qv", "rho")]))
    return out


def init_state(p: AsphParams) -> dict:
    """Full initial state (positions, sounding, bubbles; zero velocity,
    cloud water and acceleration) for either init mode."""
    s = init_reference(p) if p.init_mode == 0 else init_lattice(p)
    N = p.n_particles
    for k in ("u", "v", "w", "qc", "ax", "ay", "az", "prs", "dthdt"):
        s[k] = np.zeros(N)
    return s


def initial_state(p: AsphParams) -> dict:
    """The state the library's asph_init leaves, restated: initial state,
    initial sort, density/EOS/microphysics and the forces without
    integration (asph_h100.cu:885-921).  Fields are in sorted order;
    `rain` holds the rain grid after the initial autoconversion."""
    s = init_state(p)
    # the library holds the initial density as float32 (rho_ref rounded once)
    s["rho"] = np.asarray(s["rho"], np.float32).astype(np.float64)
    ob = sort_build(p, s)
    g = ob["gathered"]
    dt = derived(p)["dt_cap"]
    de = density_eos(p, g, g["rho"], ob["cell_range"], dt)
    st = dict(g)
    for k in ("rho", "prs", "th", "qv", "qc"):
        st[k] = de[k]
    mo = momentum(p, st, ob["cell_range"], dt, integrate=False)
    for k in ("ax", "ay", "az", "dthdt"):
        st[k] = mo[k]
    st["rain"] = de["rain_dep"]
    st["keys_sorted"] = ob["keys_sorted"]
    st["cell_range"] = ob["cell_range"]
    return st


def keys(p: AsphParams, x, y, z) -> np.ndarray:
    k = np.zeros(p.n_particles, np.uint32)
    x, y, z = _d(x), _d(y), _d(z)
    _chk(lib().or_keys(_p(p), _pd(x), _pd(y), _pd(z), k.ctypes.data_as(_U32)))
    return k


def stable_sort(k: np.ndarray, nbits: int):
    k = np.ascontiguousarray(k, np.uint32)
    perm = np.zeros(k.size, np.uint32)
    srt = np.zeros(k.size, np.uint32)
    _chk(lib().or_stable_sort(k.size, nbits, k.ctypes.data_as(_U32), perm.ctypes.data_as(_U32),
                              srt.ctypes.data_as(_U32)))
    return perm, srt


def cell_table(p: AsphParams, x, y, z) -> np.ndarray:
    r = np.zeros(2 * p.nx * p.ny * p.nz, np.int32)
    x, y, z = _d(x), _d(y), _d(z)
    _chk(lib().or_cell_table(_p(p), _pd(x), _pd(y), _pd(z), r.ctypes.data_as(_I32)))
    return r.reshape(-1, 2)


def surface(p: AsphParams, z) -> np.ndarray:
    f = np.zeros(p.n_particles, np.uint8)
    z = _d(z)
    _chk(lib().or_surface(_p(p), _pd(z), f.ctypes.data_as(_U8)))
    return f


def sort_build(p: AsphParams, s: dict) -> dict:
    """keys -> stable sort -> gather -> table + surface (asph_h100.cu:963-977)."""
    k = keys(p, s["x"], s["y"], s["z"])
    perm, srt = stable_sort(k, key_bits(p))
    g = {name: np.asarray(v)[perm] for name, v in s.items()}
    rng = cell_table(p, g["x"], g["y"], g["z"])
    surf = surface(p, g["z"])
    return {"keys_in": k, "perm": perm, "keys_sorted": srt, "gathered": g, "cell_range": rng, "surf": surf}


def kick_drift_flux(p: AsphParams, s: dict, simt: float, dt: float, surf, clamp: bool = False) -> dict:
    o = {k: _d(s[k]).copy() for k in ("x", "y", "z", "u", "v", "w", "th", "qv")}
    ax, ay, az = _d(s["ax"]), _d(s["ay"]), _d(s["az"])
    sf = np.ascontiguousarray(surf, np.uint8)
    _chk(lib().or_kick_drift_flux(_p(p), simt, dt, int(clamp), sf.ctypes.data_as(_U8),
                                  *[_pd(o[k]) for k in ("x", "y", "z", "u", "v", "w", "th", "qv")],
                                  _pd(ax), _pd(ay), _pd(az)))
    return o


def density_eos(p: AsphParams, s: dict, rho_old, cell_range, dt: float, rain_cur=None) -> dict:
    N = p.n_particles
    ncell = p.nx * p.ny * p.nz
    x, y, z = _d(s["x"]), _d(s["y"]), _d(s["z"])
    ro = _d(rho_old)
    rng = np.ascontiguousarray(cell_range, np.int32).reshape(-1)
    rain = _d(rain_cur if rain_cur is not None else np.zeros(ncell))
    th, qv, qc = _d(s["th"]).copy(), _d(s["qv"]).copy(), _d(s["qc"]).copy()
    rho, prs, dep = np.zeros(N), np.zeros(N), np.zeros(ncell)
    _chk(lib().or_density_eos(_p(p), dt, _pd(x), _pd(y), _pd(z), _pd(ro), rng.ctypes.data_as(_I32),
                              _pd(rain), _pd(th), _pd(qv), _pd(qc), _pd(rho), _pd(prs), _pd(dep)))
    return {"th": th, "qv": qv, "qc": qc, "rho": rho, "prs": prs, "rain_dep": dep}


def momentum(p: AsphParams, s: dict, cell_range, dt: float, integrate: bool) -> dict:
    N = p.n_particles
    x, y, z = _d(s["x"]), _d(s["y"]), _d(s["z"])
    u, v, w, th = _d(s["u"]).copy(), _d(s["v"]).copy(), _d(s["w"]).copy(), _d(s["th"]).copy()
    qv, qc, rho, prs = _d(s["qv"]), _d(s["qc"]), _d(s["rho"]), _d(s["prs"])
    rng = np.ascontiguousarray(cell_range, np.int32).reshape(-1)
    ax, ay, az, dth = np.zeros(N), np.zeros(N), np.zeros(N), np.zeros(N)
    _chk(lib().or_momentum(_p(p), dt, int(integrate), _pd(x), _pd(y), _pd(z), _pd(u), _pd(v), _pd(w),
                           _pd(th), _pd(qv), _pd(qc), _pd(rho), _pd(prs), rng.ctypes.data_as(_I32),
                           _pd(ax), _pd(ay), _pd(az), _pd(dth)))
    return {"ax": ax, "ay": ay, "az": az, "dthdt": dth, "u": u, "v": v, "w": w, "th": th}


def rain(p: AsphParams, rain_in, dt: float, delta=None, precip=None):
    ncell = p.nx * p.ny * p.nz
    rin = _d(rain_in)
    dl = None if delta is None else _d(delta)
    out = np.zeros(ncell)
    pr = np.zeros(p.nx * p.ny) if precip is None else _d(precip).copy()
    _chk(lib().or_rain(_p(p), dt, _pd(rin), _pd(dl) if dl is not None else None, _pd(out), _pd(pr)))
    return out, pr


def cfl(p: AsphParams, umax, dt: float, trips: int) -> dict:
    um = _d(umax)
    ctl = np.array([dt, trips, 0, 0, 0, 0], np.float64)
    st = lib().or_cfl(_p(p), _pd(um), _pd(ctl))
    return {"status": st, "dt": ctl[0], "trips": int(ctl[1]), "clamp": bool(ctl[2]), "abort": bool(ctl[3]),
            "sort_dt": ctl[4], "dt_required": ctl[5]}


def audit(p: AsphParams, s: dict) -> np.ndarray:
    out = np.zeros(6)
    arrs = [_d(s[k]) for k in ("z", "u", "v", "w", "th", "qv", "qc")]
    _chk(lib().or_audit(_p(p), *[_pd(a) for a in arrs], _pd(out)))
    return out


def helpers(p: AsphParams, z, T, pr, q) -> np.ndarray:
    """Columns: theta_ref, exner_ref, pres_ref, rho_ref, qv_ref (at z); esat,
    qsat, dqsdT (at T, pr); w3, dw3 (at q)."""
    a = np.ascontiguousarray(np.stack([_d(z), _d(T), _d(pr), _d(q)], 1))
    out = np.zeros((a.shape[0], 10))
    _chk(lib().or_helpers(_p(p), a.shape[0], _pd(a), _pd(out)))
    return out


def hash_noise(ijk) -> np.ndarray:
    a = np.ascontiguousarray(ijk, np.int32).reshape(-1, 3)
    out = np.zeros(a.shape[0], np.float32)
    _chk(lib().or_hash_noise(a.shape[0], a.ctypes.data_as(_I32), out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


RUN_FIELDS = ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az", "prs", "dthdt")


def run(p: AsphParams, state: dict, nsteps: int, rain_grid=None, precip=None, ctl=None):
    """nsteps full FP64 steps in place (the CPU baseline)."""
    N = p.n_particles
    f = [_d(state.get(k, np.zeros(N))).copy() for k in RUN_FIELDS]
    arr = (_D * 15)(*[_pd(a) for a in f])
    ncell = p.nx * p.ny * p.nz
    rg = _d(rain_grid if rain_grid is not None else np.zeros(ncell)).copy()
    pr = _d(precip if precip is not None else np.zeros(p.nx * p.ny)).copy()
    c = np.array(ctl if ctl is not None else [0.0, derived(p)["dt_cap"], 1e9, 0.5, 0, 0, 1, 0, 0], np.float64)
    st = lib().or_run(_p(p), int(nsteps), arr, _pd(rg), _pd(pr), _pd(c))
    return dict(zip(RUN_FIELDS, f)), rg, pr, c, st


# ---- adjoint window (FP64 host reference; adjoint_host.cpp) -----------------
ADJ_FIELDS = ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az")
_adj = None


def adj_lib() -> C.CDLL:
    global _adj
    if _adj is None:
        from . import build_oracle
        _adj = C.CDLL(build_oracle.build_adjoint_host())
        P = C.c_void_p
        _adj.adj_host_loss.argtypes = [P, _D, _D, C.c_double, C.c_double, C.c_int, _D, _D, C.c_int, _D, _D]
        _adj.adj_host_loss.restype = C.c_int
        _adj.adj_host_grad.argtypes = [P, _D, _D, C.c_double, C.c_double, C.c_int, _D, _D, C.c_int, _D, _D, _D]
        _adj.adj_host_grad.restype = C.c_long
    return _adj


def _adj_args(p, state, rain, alpha_beta, gauss):
    st = np.ascontiguousarray(np.stack([_d(state[k]) for k in ADJ_FIELDS]))
    rg = np.ascontiguousarray(_d(rain))
    ab = np.ascontiguousarray(_d(alpha_beta))
    g = np.ascontiguousarray(_d(gauss).reshape(-1, 6))
    return st, rg, ab, g


def adj_loss(p: AsphParams, state: dict, rain, simt: float, dt: float, nsteps: int, alpha_beta, gauss,
             final: bool = False):
    """FP64 window forward: loss (1/N) sum (qc - T(x))^2 after nsteps (and the final state)."""
    st, rg, ab, g = _adj_args(p, state, rain, alpha_beta, gauss)
    L = np.zeros(1)
    fin = np.zeros_like(st) if final else None
    _chk(adj_lib().adj_host_loss(_p(p), _pd(st), _pd(rg), float(simt), float(dt), int(nsteps), _pd(ab),
                                 _pd(g), g.shape[0], _pd(L), _pd(fin) if final else None))
    if final:
        return float(L[0]), dict(zip(ADJ_FIELDS, fin))
    return float(L[0])


def adj_grad(p: AsphParams, state: dict, rain, simt: float, dt: float, nsteps: int, alpha_beta, gauss):
    """FP64 host adjoint (reverse-mode over the FP64 window): (L, dL/dtheta0[N], dL/dalpha, dL/dbeta)."""
    st, rg, ab, g = _adj_args(p, state, rain, alpha_beta, gauss)
    L = np.zeros(1)
    dth = np.zeros(p.n_particles)
    dab = np.zeros(2)
    n = adj_lib().adj_host_grad(_p(p), _pd(st), _pd(rg), float(simt), float(dt), int(nsteps), _pd(ab), _pd(g),
                                g.shape[0], _pd(L), _pd(dth), _pd(dab))
    if n <= 0:
        raise RuntimeError("adj_host_grad failed")
    return float(L[0]), dth, float(dab[0]), float(dab[1])
