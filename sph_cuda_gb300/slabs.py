"""Slab decomposition of the plain step over several processes, one GPU each.

The reference runs on one GPU (asph_h100.cu:799).  Its step shards by slabs
of cell layers in z: rank r owns the particles whose cell layer at the start
of a step (the layer the step's sort bins them into, asph_h100.cu:229-240)
lies in [lo_r, hi_r), and the rain cells of those layers.  Every step:

1. Halo exchange.  Each rank sends copies of its particles within HALO
   layers of another rank's slab, and the rain of those layers.  HALO = 6:
   a target's search window reaches 2 layers around its current cell, which
   is at most one layer from the cell it was sorted into (3 layers), and the
   density and pressure of every particle in that window need their own
   windows covered as well (3 more).
2. The local step.  The rank's engine runs one full step (sort every step,
   kick/drift/flux, density/EOS/microphysics, momentum/integration, rain)
   on its own particles plus the halo copies, at the global dt.  Owned
   particles, and the rain of owned cells, come out exactly as in a single-
   domain step: every pair they see, and every rain deposit into their
   cells, is computed from complete neighbourhoods.  The halo results are
   dropped.
3. Migration.  Owned particles whose cell layer left the slab go to the
   rank that owns their new layer.
4. Reductions.  The velocity maxima of owned particles are reduced with MAX
   over ranks, and every rank runs the same closed-loop CFL control on them
   (asph_h100.cu:1040-1078), so all ranks keep one dt.  The conservation
   audit (asph_h100.cu:650-668) is an FP64 SUM over ranks.

Surface precipitation falls out of layer 0 and is kept by the rank that
owns it.  The exchanges use torch.distributed object collectives (gloo on
CPU, NCCL on GPUs); no device memory is shared between processes and no
kernel waits on another process.

The engine is any callable `engine(p, state, rain, precip, simt, dt)` that
runs one step and returns (state, rain, precip, perm): the state comes back
in the order of the sort that begins the step, perm[i] being the input
index of output particle i; AsphEngine runs it on the rank's GPU through
the library.  Slabs need a sort every step (the local
particle set changes every step), as the moist-bubble workload does.
"""
from __future__ import annotations

import numpy as np

from .abi import STATE_FIELDS

HALO = 6


def cell_layer(p, z) -> np.ndarray:
    """Cell layer of each particle: the float32 product z * (1/dz), truncated
    and clamped (asph_h100.cu:193-198, 236-238)."""
    inv = np.float32(1.0) / np.float32(p.dz)
    s = np.asarray(z, np.float32) * inv
    return np.clip(np.trunc(s), 0, p.nz - 1).astype(np.int64)


class SlabPlan:
    """Layer ranges of `world` z-slabs: [bounds[r], bounds[r + 1])."""

    def __init__(self, p, world: int, halo: int = HALO, bounds=None):
        if world < 1:
            raise ValueError("world must be >= 1")
        self.nz, self.world, self.halo = int(p.nz), int(world), int(halo)
        if bounds is None:
            bounds = [round(r * self.nz / world) for r in range(world + 1)]
        self.bounds = np.asarray(bounds, np.int64)
        if self.bounds[0] != 0 or self.bounds[-1] != self.nz or np.any(np.diff(self.bounds) < 1):
            raise ValueError("slab bounds must rise from 0 to nz with at least one layer per slab")

    def slab(self, r: int):
        return int(self.bounds[r]), int(self.bounds[r + 1])

    def owner(self, layer) -> np.ndarray:
        return np.searchsorted(self.bounds, np.asarray(layer), side="right") - 1

    def halo_range(self, r: int):
        """Layers whose particles rank r needs copies of (its slab +- halo)."""
        lo, hi = self.slab(r)
        return max(lo - self.halo, 0), min(hi + self.halo, self.nz)


def cfl_control(p, umax, dt: float, trips: int):
    """The library's closed-loop CFL control (asph_h100.cu:1040-1078) on the
    host, in float32: returns (dt_next, trips, clamp, abort)."""
    f = np.float32
    cfl, cs = f(p.cfl), f(p.cs)
    dt_static = cfl * min(min(f(p.dx), f(p.dy)), f(p.dz)) / cs
    dt_cap = min(f(p.dt_request), dt_static) if p.dt_request > 0 else dt_static
    dt_floor = f(0.05) * dt_cap
    ux, uy, uz = (f(u) for u in umax)
    req = cfl * min(min(f(p.dx) / (cs + ux), f(p.dy) / (cs + uy)), f(p.dz) / (cs + uz)) * f(0.9)
    adopt = min(dt_cap, req)
    clamp = False
    if adopt < dt_floor:
        trips += 1
        if p.strict_cfl or trips > p.max_trip:
            return float(dt), trips, False, True
        clamp = True
        adopt = max(dt_floor, cfl * min(min(f(p.dx), f(p.dy)), f(p.dz)) / (f(1.5) * cs) * f(0.9))
    elif adopt < f(0.98) * f(dt):
        trips = 0
    return float(adopt if p.adaptive_dt else f(dt)), trips, clamp, False


def clamp_velocities(p, s: dict) -> None:
    """The emergency clamp |v| <= cs/2 after a CFL trip (asph_h100.cu:669-675)."""
    vmax = np.float32(0.5) * np.float32(p.cs)
    u, v, w = (np.asarray(s[k], np.float32) for k in ("u", "v", "w"))
    s2 = u * u + v * v + w * w
    m = s2 > vmax * vmax
    if np.any(m):
        fac = vmax / np.sqrt(s2[m])
        for k in ("u", "v", "w"):
            a = np.array(s[k], copy=True)
            a[m] = a[m] * fac.astype(a.dtype)
            s[k] = a


class SlabRank:
    """One rank of a slab-decomposed run: its owned particles (with global
    ids), the rain of its layers, the shared dt and CFL state."""

    def __init__(self, p, plan: SlabPlan, rank: int, dist, engine, controller=cfl_control):
        self.p, self.plan, self.rank, self.dist = p, plan, int(rank), dist
        self.engine, self.controller = engine, controller
        self.lo, self.hi = plan.slab(self.rank)
        self.ids = np.zeros(0, np.int64)
        self.f = {}
        self.rain = np.zeros((self.hi - self.lo, p.ny, p.nx))
        self.precip = np.zeros(p.nx * p.ny)
        self.simt, self.dt, self.trips, self.clamp, self.aborted = 0.0, 0.0, 0, False, False
        self.n_total = 0

    # ---- set-up ---------------------------------------------------------------
    def scatter(self, state: dict, rain=None, precip=None, dt: float = 0.0, simt: float = 0.0) -> None:
        """Take this rank's share of a global state (every rank passes the
        same one); particle ids are the global indices."""
        z = np.asarray(state["z"])
        mine = np.nonzero(self.plan.owner(cell_layer(self.p, z)) == self.rank)[0]
        self.ids = mine.astype(np.int64)
        self.f = {k: np.asarray(state[k])[mine].copy() for k in STATE_FIELDS if k in state}
        self.n_total = int(z.size)
        g = np.zeros(self.p.nz * self.p.ny * self.p.nx) if rain is None else np.asarray(rain, np.float64)
        self.rain = g.reshape(self.p.nz, self.p.ny, self.p.nx)[self.lo:self.hi].copy()
        if precip is not None and self.lo == 0:
            self.precip = np.asarray(precip, np.float64).copy()
        self.dt, self.simt = float(dt), float(simt)

    # ---- exchanges ------------------------------------------------------------
    def _all_to_all(self, outbox: dict) -> list:
        """Every rank's outbox {dest: payload}; returns the payloads sent to
        this rank, in rank order."""
        boxes = [None] * self.plan.world
        self.dist.all_gather_object(boxes, outbox)
        return [b[self.rank] for b in boxes if self.rank in b]

    def _halo_in(self):
        layer = cell_layer(self.p, self.f["z"])
        out = {}
        for q in range(self.plan.world):
            if q == self.rank:
                continue
            a, b = self.plan.halo_range(q)
            sel = np.nonzero((layer >= a) & (layer < b))[0]
            ra, rb = max(a, self.lo), min(b, self.hi)
            rain = (ra, self.rain[ra - self.lo:rb - self.lo].copy()) if rb > ra else None
            if sel.size or rain is not None:
                out[q] = (self.ids[sel], {k: v[sel] for k, v in self.f.items()}, rain)
        return self._all_to_all(out)

    def _migrate(self) -> None:
        layer = cell_layer(self.p, self.f["z"])
        dest = self.plan.owner(layer)
        out = {}
        for q in np.unique(dest):
            if q == self.rank:
                continue
            sel = np.nonzero(dest == q)[0]
            out[int(q)] = (self.ids[sel], {k: v[sel] for k, v in self.f.items()})
        keep = np.nonzero(dest == self.rank)[0]
        ids, f = [self.ids[keep]], {k: [v[keep]] for k, v in self.f.items()}
        for rid, rf in self._all_to_all(out):
            ids.append(rid)
            for k in f:
                f[k].append(rf[k])
        self.ids = np.concatenate(ids)
        order = np.argsort(self.ids, kind="stable")
        self.ids = self.ids[order]
        self.f = {k: np.concatenate(v)[order] for k, v in f.items()}

    # ---- one step -------------------------------------------------------------
    def step(self) -> None:
        if self.aborted:
            raise RuntimeError("run stopped by the CFL trip limit")
        if self.clamp:
            clamp_velocities(self.p, self.f)
        got = self._halo_in()
        ids = [self.ids] + [g[0] for g in got]
        f = {k: [v] + [g[1][k] for g in got] for k, v in self.f.items()}
        loc_ids = np.concatenate(ids)
        order = np.argsort(loc_ids, kind="stable")   # a deterministic local order: global ids
        loc_ids = loc_ids[order]
        local = {k: np.concatenate(v)[order] for k, v in f.items()}
        rain = np.zeros((self.p.nz, self.p.ny, self.p.nx))
        rain[self.lo:self.hi] = self.rain
        for g in got:
            if g[2] is not None:
                a, r = g[2]
                rain[a:a + r.shape[0]] = r
        out, rain_out, precip_out, perm = self.engine(self.p, local, rain.reshape(-1), self.precip, self.simt,
                                                      self.dt)
        out_ids = loc_ids[np.asarray(perm, np.int64)]
        own = np.nonzero(np.isin(out_ids, self.ids, assume_unique=True))[0]
        order = own[np.argsort(out_ids[own], kind="stable")]
        self.f = {k: np.asarray(out[k])[order] for k in self.f}
        self.rain = np.asarray(rain_out, np.float64).reshape(self.p.nz, self.p.ny, self.p.nx)[self.lo:self.hi].copy()
        if self.lo == 0:
            self.precip = np.asarray(precip_out, np.float64).copy()
        self.simt += self.dt
        umax = self._reduce_max([np.abs(self.f[k]).max() if self.f[k].size else 0.0 for k in ("u", "v", "w")])
        self.dt, self.trips, self.clamp, self.aborted = self.controller(self.p, umax, self.dt, self.trips)
        self._migrate()

    def _reduce_max(self, vals):
        import torch
        t = torch.tensor([float(v) for v in vals], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return t.tolist()

    # ---- diagnostics ------------------------------------------------------------
    def audit(self, pmass: float) -> np.ndarray:
        """FP64 totals KE, PE, IE, water, p_z, mass over all ranks
        (asph_h100.cu:650-668); Exner from the reference sounding."""
        import torch
        p = self.p
        g, rd, cp, p0 = 9.80665, 287.05, 1004.0, 100000.0
        th0, n2 = float(np.float32(p.th0)), float(np.float32(p.n2))
        a = g * g / (cp * th0 * n2)
        z = np.asarray(self.f["z"], np.float64)
        ex = 1.0 - a * (1.0 - np.exp(-n2 * z / g))
        pi = (np.maximum(p0 * ex ** (cp / rd), 1.0) / p0) ** (rd / cp)
        u, v, w = (np.asarray(self.f[k], np.float64) for k in ("u", "v", "w"))
        loc = [0.5 * np.sum(u * u + v * v + w * w), g * np.sum(z),
               cp * np.sum(np.asarray(self.f["th"], np.float64) * pi),
               np.sum(np.asarray(self.f["qv"], np.float64) + np.asarray(self.f["qc"], np.float64)), np.sum(w)]
        t = torch.tensor(loc, dtype=torch.float64)
        self.dist.all_reduce(t)
        return np.array(t.tolist() + [self.n_total]) * pmass

    def gather(self):
        """The whole state in global-id order (for checks and dumps)."""
        parts = [None] * self.plan.world
        self.dist.all_gather_object(parts, (self.ids, self.f))
        ids = np.concatenate([q[0] for q in parts])
        order = np.argsort(ids)
        return ids[order], {k: np.concatenate([q[1][k] for q in parts])[order] for k in self.f}

    def gather_rain(self):
        parts = [None] * self.plan.world
        self.dist.all_gather_object(parts, (self.lo, self.rain))
        g = np.zeros((self.p.nz, self.p.ny, self.p.nx))
        for lo, r in parts:
            g[lo:lo + r.shape[0]] = r
        return g.reshape(-1)


class AsphEngine:
    """One rank's step on its GPU through the C ABI: a context for the local
    particle set (a new one whenever the count changes; a step's own CFL
    decision is not used, the ranks share dt through cfl_control)."""

    def __init__(self, pmass: float, stream=None):
        self.pmass = float(pmass)
        self.stream = stream
        self.sim = None
        self.n = -1

    def __call__(self, p, local, rain, precip, simt, dt):
        from . import Asph, abi
        n = int(local["x"].size)
        if self.sim is None or n != self.n:
            if self.sim is not None:
                self.sim.close()
            q = p.copy()
            q.n_particles = n
            q.init_mode = abi.INIT_LATTICE
            q.lat_nx, q.lat_ny, q.lat_nz = n, 1, 1
            q.pmass = self.pmass           # the global mass per particle
            q.sort_every = 1
            # The shared controller decides dt, trips and clamps: the local
            # context's own control (whose maxima include the halo copies)
            # must never trip, so its cap (and with it its floor) is made
            # tiny; each step runs at the dt given by set_time.
            q.dt_request = 1e-6
            self.sim = Asph(q, stream=self.stream)
            self.n = n
        self.sim.set_state({k: np.asarray(v, np.float32) for k, v in local.items()})
        self.sim.set_rain(np.asarray(rain, np.float32), np.asarray(precip, np.float32))
        self.sim.set_time(simt, dt, True)
        self.sim.step(1)
        st = self.sim.get_state()
        r, pr = self.sim.get_rain()
        return st, r, pr, self.sim.get_sort()["perm"]

    def close(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None
