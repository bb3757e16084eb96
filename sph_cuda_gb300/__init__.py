"""GB300 anisotropic-SPH warm-rain step (Forbu/sph_cuda asph_h100.cu hot path).

Python host mirror of the C ABI in include/asph.h.  Every method is one C
call into libasph.so; there is no Python or CPU implementation of any step,
so a missing or unloadable library raises immediately.

    p = sph_cuda_gb300.preset("bubble2m")
    sim = sph_cuda_gb300.Asph(p)
    sim.init()
    sim.step(500)
    state = sim.get_state()
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .abi import (AsphControl, AsphHostState, AsphParams, STATE_FIELDS, load_library)

__all__ = ["Asph", "AsphError", "AsphParams", "Ensemble", "Snapshot", "ensemble_members", "preset", "library",
           "STATE_FIELDS"]

PRESETS = {
    "reference": abi.PRESET_REFERENCE,
    "small65k": abi.PRESET_SMALL_65K,
    "bubble2m": abi.PRESET_BUBBLE_2M,
    "large16m": abi.PRESET_LARGE_16M,
    "adjoint262k": abi.PRESET_ADJOINT_262K,
}


class AsphError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("asph status %d: %s" % (status, msg))
        self.status = status


def library() -> C.CDLL:
    return load_library()


def _check(st: int) -> None:
    if st != abi.ASPH_OK:
        lib = library()
        raise AsphError(st, (lib.asph_last_error() or b"").decode(errors="replace")
                        or lib.asph_status_string(st).decode())


def preset(name: str = "bubble2m", nx: int = 0, ny: int = 0, nz: int = 0, **overrides) -> AsphParams:
    """Fill AsphParams from a named preset, then apply field overrides."""
    p = AsphParams()
    _check(library().asph_params_preset(C.byref(p), PRESETS[name], nx, ny, nz))
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def check_params(p: AsphParams) -> None:
    _check(library().asph_params_check(C.byref(p)))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Asph:
    """One simulation context (device buffers, stream, captured graphs)."""

    def __init__(self, params: AsphParams, stream: int | None = None, _borrowed=None):
        self.lib = library()
        self.params = params.copy()
        self._ctx = C.c_void_p()
        self._owner = _borrowed   # an Ensemble that owns the context, or None
        if _borrowed is None:
            _check(self.lib.asph_create(C.byref(self.params), C.c_void_p(stream or 0), C.byref(self._ctx)))
        self.N = int(self.params.n_particles)
        self.ncell = int(self.params.nx * self.params.ny * self.params.nz)

    def close(self) -> None:
        if self._ctx and self._owner is None:
            self.lib.asph_destroy(self._ctx)
        self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- state --------------------------------------------------------------
    def init(self) -> None:
        _check(self.lib.asph_init(self._ctx))

    def set_state(self, fields: dict) -> None:
        hs = AsphHostState()
        keep = []
        for name in STATE_FIELDS:
            if name in fields and fields[name] is not None:
                a = np.ascontiguousarray(fields[name], dtype=np.float32)
                if a.shape != (self.N,):
                    raise ValueError("field %s has shape %s, expected (%d,)" % (name, a.shape, self.N))
                keep.append(a)
                setattr(hs, name, _fptr(a))
        _check(self.lib.asph_set_state(self._ctx, C.byref(hs)))

    def get_state(self, fields=STATE_FIELDS, out: dict | None = None) -> dict:
        hs = AsphHostState()
        res = {}
        for name in fields:
            a = out[name] if out is not None and name in out else np.empty(self.N, np.float32)
            res[name] = a
            setattr(hs, name, _fptr(a))
        _check(self.lib.asph_get_state(self._ctx, C.byref(hs)))
        return res

    def get_rain(self):
        rain = np.empty(self.ncell, np.float32)
        precip = np.empty(self.params.nx * self.params.ny, np.float32)
        _check(self.lib.asph_get_rain(self._ctx, _fptr(rain), _fptr(precip)))
        return rain, precip

    def set_rain(self, rain=None, precip=None) -> None:
        r = None if rain is None else np.ascontiguousarray(rain, np.float32)
        q = None if precip is None else np.ascontiguousarray(precip, np.float32)
        _check(self.lib.asph_set_rain(self._ctx, _fptr(r) if r is not None else None,
                                      _fptr(q) if q is not None else None))

    def control(self) -> dict:
        c = AsphControl()
        _check(self.lib.asph_get_control(self._ctx, C.byref(c)))
        return {n: getattr(c, n) for n, _ in AsphControl._fields_}

    def set_time(self, simt: float, dt: float = 0.0, do_sort: bool = True) -> None:
        _check(self.lib.asph_set_time(self._ctx, float(simt), float(dt), int(bool(do_sort))))

    # ---- granular blocks ----------------------------------------------------------
    def sort_build(self) -> None:
        _check(self.lib.asph_sort_build(self._ctx))

    def get_sort(self) -> dict:
        N = self.N
        kin = np.empty(N, np.uint32)
        ks = np.empty(N, np.uint32)
        perm = np.empty(N, np.uint32)
        rng = np.empty(2 * self.ncell, np.int32)
        surf = np.empty(N, np.int32)
        cnt = C.c_int32()
        u32 = C.POINTER(C.c_uint32)
        i32 = C.POINTER(C.c_int32)
        _check(self.lib.asph_get_sort(self._ctx, kin.ctypes.data_as(u32), ks.ctypes.data_as(u32),
                                      perm.ctypes.data_as(u32), rng.ctypes.data_as(i32),
                                      surf.ctypes.data_as(i32), C.byref(cnt)))
        return {"keys_in": kin, "keys_sorted": ks, "perm": perm, "cell_range": rng.reshape(-1, 2),
                "surf_list": surf[:cnt.value].copy(), "surf_count": cnt.value}

    def neighbours(self):
        """(count[N], list[NBR_CAP][N]) of the last density pass."""
        cnt = np.empty(self.N, np.int32)
        lst = np.empty((abi.NBR_CAP, self.N), np.int32)
        i32 = C.POINTER(C.c_int32)
        _check(self.lib.asph_get_neighbours(self._ctx, cnt.ctypes.data_as(i32), lst.ctypes.data_as(i32)))
        return cnt, lst

    def kick_drift_flux(self) -> None:
        _check(self.lib.asph_kick_drift_flux(self._ctx))

    def density_eos(self) -> None:
        _check(self.lib.asph_density_eos(self._ctx))

    def momentum(self, integrate: bool = True) -> None:
        _check(self.lib.asph_momentum(self._ctx, int(bool(integrate))))

    def rain(self) -> None:
        _check(self.lib.asph_rain(self._ctx))

    def cfl(self) -> None:
        _check(self.lib.asph_cfl(self._ctx))

    # ---- fused step --------------------------------------------------------------------
    def step(self, nsteps: int = 1) -> None:
        _check(self.lib.asph_step(self._ctx, int(nsteps)))

    def step_async(self, nsteps: int = 1) -> None:
        _check(self.lib.asph_step_async(self._ctx, int(nsteps)))

    def step_kernels(self) -> int:
        """Kernel launches of one step (kernel nodes of the step's CUDA graph)."""
        n = C.c_int(0)
        _check(self.lib.asph_step_kernels(self._ctx, C.byref(n)))
        return int(n.value)

    def step_profiled(self, nsteps: int = 1) -> dict:
        """Per-phase device milliseconds summed over nsteps (non-graph launches)."""
        out = np.zeros(abi.NPHASES, np.float32)
        _check(self.lib.asph_step_profiled(self._ctx, int(nsteps), _fptr(out)))
        return dict(zip(abi.PHASES, out.tolist()))

    def set_pair_path(self, global_path) -> None:
        """Pair path: False/0 automatic, True/1 the per-target global path,
        2 density with one warp per target."""
        _check(self.lib.asph_set_option(self._ctx, abi.OPT_PAIR_PATH, int(global_path)))

    def pair_shape(self) -> int:
        v = C.c_int()
        _check(self.lib.asph_get_option(self._ctx, abi.OPT_PAIR_SHAPE, C.byref(v)))
        return v.value

    def set_pair_shape(self, shape: int) -> None:
        """Brick shape of the density pass (0..3), -1 for automatic."""
        _check(self.lib.asph_set_option(self._ctx, abi.OPT_PAIR_SHAPE, int(shape)))

    def set_viscosity(self, alpha: float, beta: float) -> None:
        """Artificial-viscosity coefficients alpha and beta of the running context."""
        _check(self.lib.asph_set_viscosity(self._ctx, float(alpha), float(beta)))
        self.params.alpha_av, self.params.beta_av = float(alpha), float(beta)

    def sort_every(self) -> int:
        v = C.c_int()
        _check(self.lib.asph_get_option(self._ctx, abi.OPT_SORT_EVERY, C.byref(v)))
        return v.value

    def set_sort_every(self, k: int) -> None:
        _check(self.lib.asph_set_option(self._ctx, abi.OPT_SORT_EVERY, int(k)))

    def targets_per_thread(self) -> int:
        v = C.c_int()
        _check(self.lib.asph_get_option(self._ctx, abi.OPT_TARGETS_PER_THREAD, C.byref(v)))
        return v.value

    def set_targets_per_thread(self, k: int) -> None:
        """Momentum-pass targets per thread: 1, 2 or 4 (a warp covers 32 k targets)."""
        _check(self.lib.asph_set_option(self._ctx, abi.OPT_TARGETS_PER_THREAD, int(k)))

    def sort_ahead(self) -> bool:
        v = C.c_int()
        _check(self.lib.asph_get_option(self._ctx, abi.OPT_SORT_AHEAD, C.byref(v)))
        return bool(v.value)

    def set_sort_ahead(self, on: bool) -> None:
        """With a sort every step, runs of several steps sort the next step's
        keys beside the current step's pair passes (on by default); results
        are bit-identical either way."""
        _check(self.lib.asph_set_option(self._ctx, abi.OPT_SORT_AHEAD, int(bool(on))))

    # ---- source-term hook ---------------------------------------------------------
    def enable_source(self, on: bool = True) -> None:
        """Per-particle additive tendencies of theta, qv, qc applied in every
        step's theta update (zero after enabling)."""
        _check(self.lib.asph_source_enable(self._ctx, int(bool(on))))

    def set_source(self, dtheta=None, dqv=None, dqc=None) -> None:
        """Tendencies [K/s, 1/s, 1/s] in the current particle order."""
        keep = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (dtheta, dqv, dqc)]
        for a in keep:
            if a is not None and a.shape != (self.N,):
                raise ValueError("tendency arrays must have shape (%d,)" % self.N)
        _check(self.lib.asph_source_set(self._ctx, *[None if a is None else _fptr(a) for a in keep]))

    def set_source_device(self, tendencies) -> None:
        """Tendencies from a CUDA tensor of shape (N, 4) float32 {S_theta, S_qv, S_qc, -}."""
        if tuple(tendencies.shape) != (self.N, 4) or not tendencies.is_contiguous():
            raise ValueError("need a contiguous (N, 4) tensor")
        import torch
        torch.cuda.synchronize()   # the tensor's producer may run on another stream
        _check(self.lib.asph_source_set_device(self._ctx, C.c_void_p(tendencies.data_ptr())))
        self.sync()

    def state_device(self, pos=None, vel=None, thq=None) -> None:
        """Copy the current state into CUDA tensors of shape (N, 4) float32
        (pos: x, y, z, rho_old; vel: u, v, w, -; thq: theta, qv, qc, -)."""
        ptrs = []
        for t in (pos, vel, thq):
            if t is not None and (tuple(t.shape) != (self.N, 4) or not t.is_contiguous()):
                raise ValueError("need contiguous (N, 4) tensors")
            ptrs.append(None if t is None else C.c_void_p(t.data_ptr()))
        _check(self.lib.asph_state_device(self._ctx, *ptrs))
        self.sync()   # the tensors are read on torch's streams

    # ---- snapshots and restart files --------------------------------------------
    def snapshot(self) -> "Snapshot":
        """A device-resident copy of the full state (see restore)."""
        s = Snapshot(self)
        _check(self.lib.asph_snapshot_save(self._ctx, s._h))
        return s

    def save_snapshot(self, snap: "Snapshot") -> None:
        _check(self.lib.asph_snapshot_save(self._ctx, snap._h))

    def restore(self, snap: "Snapshot") -> None:
        _check(self.lib.asph_snapshot_restore(self._ctx, snap._h))

    def checkpoint_write(self, path: str) -> None:
        _check(self.lib.asph_checkpoint_write(self._ctx, str(path).encode()))

    def checkpoint_read(self, path: str) -> None:
        _check(self.lib.asph_checkpoint_read(self._ctx, str(path).encode()))

    def sync(self) -> None:
        _check(self.lib.asph_sync(self._ctx))

    # ---- diagnostics ---------------------------------------------------------------------
    def audit(self) -> np.ndarray:
        out = np.zeros(6, np.float64)
        _check(self.lib.asph_audit(self._ctx, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def dump(self, outdir: str) -> str:
        buf = C.create_string_buffer(1024)
        os.makedirs(outdir, exist_ok=True)
        _check(self.lib.asph_dump(self._ctx, outdir.encode(), buf, 1024))
        return buf.value.decode()

    def dump_begin(self) -> None:
        """Queue a dump of the current state (asynchronous device-to-host copy)."""
        _check(self.lib.asph_dump_begin(self._ctx))

    def dump_finish(self, outdir: str):
        """Write the dump queued by dump_begin; returns (path, column diagnostics)."""
        buf = C.create_string_buffer(1024)
        diag = np.zeros(4, np.float32)
        os.makedirs(outdir, exist_ok=True)
        _check(self.lib.asph_dump_finish(self._ctx, outdir.encode(), buf, 1024, _fptr(diag)))
        return buf.value.decode(), {"cloud_pct": float(diag[0]), "ql_max": float(diag[1]),
                                    "w_max": float(diag[2]), "precip_mm": float(diag[3])}

    def column_diag(self) -> dict:
        out = np.zeros(4, np.float32)
        _check(self.lib.asph_column_diag(self._ctx, _fptr(out)))
        return {"cloud_pct": float(out[0]), "ql_max": float(out[1]), "w_max": float(out[2]),
                "precip_mm": float(out[3])}


class Snapshot:
    """Device memory holding one full state of a context."""

    def __init__(self, sim: Asph):
        self.lib = sim.lib
        self._h = C.c_void_p()
        _check(self.lib.asph_snapshot_create(sim._ctx, C.byref(self._h)))

    def close(self) -> None:
        if self._h:
            self.lib.asph_snapshot_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Many independent simulations stepped together: one CUDA graph launch
    per ensemble step forks into every member's step."""

    def __init__(self, members: list, stream: int | None = None):
        self.lib = library()
        self.params = [p.copy() for p in members]
        arr = (AsphParams * len(members))(*self.params)
        self._h = C.c_void_p()
        _check(self.lib.asph_ens_create(arr, len(members), C.c_void_p(stream or 0), C.byref(self._h)))
        self._members = {}

    def __len__(self) -> int:
        return len(self.params)

    @property
    def n_particles(self) -> int:
        return sum(int(p.n_particles) for p in self.params)

    def close(self) -> None:
        for m in self._members.values():
            m._ctx = C.c_void_p()
        self._members.clear()
        if self._h:
            self.lib.asph_ens_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self) -> None:
        _check(self.lib.asph_ens_init(self._h))

    def step(self, nsteps: int = 1) -> None:
        _check(self.lib.asph_ens_step(self._h, int(nsteps)))

    def step_async(self, nsteps: int = 1) -> None:
        _check(self.lib.asph_ens_step_async(self._h, int(nsteps)))

    def sync(self) -> None:
        _check(self.lib.asph_ens_sync(self._h))

    def member(self, k: int) -> Asph:
        """The k-th member as an Asph view (state, audit, dump, options);
        the ensemble owns it."""
        ctx = C.c_void_p()
        _check(self.lib.asph_ens_member(self._h, int(k), C.byref(ctx)))
        m = self._members.get(k)
        if m is None:
            m = Asph(self.params[k], _borrowed=self)
            self._members[k] = m
        m._ctx = ctx
        return m

    def tune(self, trial_steps: int = 5, sort_choices=()) -> list:
        """Per member (brick shape, sort cadence, momentum targets per
        thread) picked by timing; the state is kept."""
        n = len(self.params)
        chosen = (C.c_int * (3 * n))()
        sc = (C.c_int * max(1, len(sort_choices)))(*sort_choices)
        _check(self.lib.asph_ens_tune(self._h, int(trial_steps), sc, len(sort_choices), chosen))
        return [(chosen[3 * k], chosen[3 * k + 1], chosen[3 * k + 2]) for k in range(n)]


def ensemble_members(count: int = 64, seed: int = 7, lo: int = 16384, hi: int = 524288,
                     theta_sigma: float = 0.1, dt: float = 0.5) -> list:
    """Members of uneven size: particle counts log-uniform in [lo, hi]
    (seeded), each the 65,536-particle small-box atmosphere (h 200 x 200 x 50 m,
    lattice spacing 312.5 x 312.5 x 78.125 m, +2 K bubble of 1 km radius at
    1 km height) on an (n, n, 2n) lattice, n = round((N/2)^(1/3)), in a box
    scaled with n so that the particle spacing and particles per cell stay
    those of the small box; initial theta noise sigma [K]; member k seeds its
    noise with k."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    out = []
    for k, nm in enumerate(counts):
        n = int(round((nm / 2.0) ** (1.0 / 3.0)))
        p = preset("small65k")
        lx, lz = n * 312.5, 2 * n * 78.125
        p.nx = p.ny = int(lx // 200.0)
        p.nz = int(lz // 50.0)
        p.dx = p.dy = lx / p.nx
        p.dz = lz / p.nz
        p.lat_nx = p.lat_ny = n
        p.lat_nz = 2 * n
        p.n_particles = 2 * n ** 3
        p.bubble_x[0] = p.bubble_y[0] = lx / 2
        p.noise = theta_sigma
        p.seed = k
        p.dt_request = dt
        out.append(p)
    return out
