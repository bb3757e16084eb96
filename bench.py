"""Benchmark: particle-steps/s of the full SPH warm-rain step.

Workload: the 2,097,152-particle moist-bubble configuration (128^3 jittered lattice in a 20 x 20 x 8 km box, cells 150.4 x 150.4 x 40 m,
three seeded warm bubbles, warm rain with accretion and evaporation, Morton
re-sort every step).  Synthetic, seeded initial state; no dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours: K fused steps (sort + gather/kick/drift/flux + density/EOS/micro +
momentum/integrate/rain/CFL, one CUDA graph per step) timed with CUDA events
on the simulation stream; one JSON line on rank 0.  --impl reference times
the CPU restatement of the reference (FP64, all host cores) on a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (plain step, 2,097,152 particles)"
UNIT = "particle-steps/s"
L2_BYTES = 129e6


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def algorithmic_bytes(N: int, C: int) -> dict:
    """Minimum compulsory traffic of the reference dataflow per step with a
    sort every step (bytes): keygen 16 + sort 16 + gather 108 + table 4 +
    8 per cell + kick/drift 60 + density/EOS/micro 48 + momentum/integrate
    72 + rain 12 per cell (per particle unless noted)."""
    per_particle = 16 + 16 + 108 + 4 + 60 + 48 + 72
    return {"step": per_particle * N + 20 * C,
            "momentum_integrate": 72 * N + 12 * C,
            "density_eos": 48 * N,
            "gather_kick_drift": (108 + 60 + 16) * N,
            "sort": 16 * N,
            "table_clear": 8 * C}


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def job_rate(units: float, seconds_local: float, dist=None, device="cpu"):
    """Whole-job throughput of independent replicas: every rank processes
    `units` inside its own timed region and the job time is the maximum over
    ranks.  Returns (units/s over all ranks, job seconds)."""
    import torch
    t = torch.tensor([seconds_local], dtype=torch.float64, device=device)
    ws = 1
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ws = dist.get_world_size()
    sec = float(t.item())
    return ws * units / sec, sec


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_sample_params():
    """The moist-bubble physics on a quarter-width box: 32 x 32 x 128 lattice (131,072
    particles), 33 x 33 x 200 cells of the same 150.4 x 150.4 x 40 m size, so
    the per-particle neighbour work equals the full workload's."""
    import sph_cuda_gb300 as sph
    p = sph.preset("bubble2m")
    p.nx = p.ny = 33
    p.lat_nx = p.lat_ny = 32
    p.n_particles = 32 * 32 * 128
    for b in range(p.n_bubbles):
        p.bubble_x[b] *= 33 / 133.0
        p.bubble_y[b] *= 33 / 133.0
    return p


def time_oracle(p, state, nsteps: int):
    from oracle import oracle
    t0 = time.perf_counter()
    _, _, _, ctl, st = oracle.run(p, state, nsteps)
    dt = time.perf_counter() - t0
    return dt, oracle.threads(), st


def oracle_initial_state(p):
    """Initial state of the CPU runs from the oracle's own init."""
    from oracle import oracle
    return oracle.init_state(p)


def workload_string(name: str) -> str:
    return {"bubble2m": "moist bubble, 2,097,152 particles, 133x133x200 cells, sort every step",
            "bubble524k": "moist bubble, 524,288 particles, 66x66x200 cells, sort every step",
            "reference128": "the reference's own geometry and init, 128x128x128 cells, dt 0.25 s, "
                            "sort every step",
            "large16m": "large anisotropic run, 16,777,216 particles, 250x250x500 cells (h 160 m x 20 m), "
                        "95% RH boundary layer, theta noise 0.2 K, sort every step"}[name]


def metric_for(p) -> str:
    return "particle-steps/s (plain step, {:,} particles)".format(int(p.n_particles))


def run_reference(args):
    """The reference's CPU path (the FP64 oracle port, all host threads) on a
    bounded sample of the workload: each step is one full step of the
    131,072-particle box with the workload's cells and physics."""
    ws, rank, local = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle
    p = cpu_sample_params()
    state = oracle_initial_state(p)
    oracle.run(p, state, max(args.warmup, 1))   # warm-up: page in, thread pool
    t, cores, _ = time_oracle(p, state, args.steps)
    value = p.n_particles * args.steps / t
    sample = ("%d consecutive FP64 steps of the 131,072-particle moist-bubble box "
              "(same cells and physics, 5 x 5 km footprint)" % args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload_string(args.workload), "sample": sample,
                   "sample_particles": p.n_particles, "sample_cells": p.nx * p.ny * p.nz},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_params(name: str):
    """bubble2m: the headline 2,097,152-particle moist-bubble workload.
    bubble524k: the same physics, cell size and density on a 10 x 10 x 8 km box
    (64 x 64 x 128 lattice, 66 x 66 x 200 cells) for profiler captures.
    reference128: the reference's own configuration at --nx --ny --nz 128 and
    --dt 0.25 with a sort every step (what oracle/time_reference.py native runs).
    large16m: the 16,777,216-particle anisotropic run (40 x 40 x 10 km, 8:1)."""
    import sph_cuda_gb300 as sph
    if name == "large16m":
        return sph.preset("large16m")
    if name == "reference128":
        p = sph.preset("reference", 128, 128, 128)
        p.sort_every = 1
        p.dt_request = 0.25
        return p
    p = sph.preset("bubble2m")
    if name == "bubble524k":
        p.nx = p.ny = 66
        p.lat_nx = p.lat_ny = 64
        p.n_particles = 64 * 64 * 128
        for b in range(p.n_bubbles):
            p.bubble_x[b] *= 66 / 133.0
            p.bubble_y[b] *= 66 / 133.0
    return p


def run_ours(args):
    import torch
    import sph_cuda_gb300 as sph

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    p = workload_params(args.workload)
    N, C = p.n_particles, p.nx * p.ny * p.nz
    sim = sph.Asph(p, stream=stream.cuda_stream)
    sim.init()
    if args.advance > 0:   # untimed steps first: measure the developed state
        sim.step(args.advance)
    sim.step(max(args.warmup, 1))
    per_step = sim.step_kernels()   # kernel nodes of the step's CUDA graph

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step_async(args.steps)
    e1.record(stream)
    e1.synchronize()
    sim.sync()
    clk = clocks.stop()
    barrier()
    value, sec = job_rate(N * args.steps, e0.elapsed_time(e1) / 1e3, dist, "cuda")
    ms = sec * 1e3

    # per-kernel device times of the same step (non-graph launches, events
    # between the kernels on the simulation stream)
    prof_steps = max(3, min(args.steps, 20))
    ph = sim.step_profiled(prof_steps)
    ph_ms = {k: v / prof_steps for k, v in ph.items()}
    algo = algorithmic_bytes(N, C)
    kernels = ["table_clear", "sort", "gather_kick_drift", "density_eos", "momentum_integrate"]
    dom = max(kernels, key=lambda k: ph_ms[k])
    hbm, src = peaks()
    achieved = algo[dom] / (ph_ms[dom] / 1e3) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic_%s.txt" % args.workload)
    if os.path.exists(tfile):
        try:
            traffic = json.load(open(tfile)).get(dom)
        except Exception:
            traffic = None
    # the pair kernels are bound by instruction issue and load latency, not
    # HBM: their pipe utilisation from the committed ncu capture goes beside
    # the HBM fraction
    companion = None
    pfile = os.path.join(ROOT, "profiles", "pipes_bubble2m.txt")
    if os.path.exists(pfile):
        try:
            d = json.load(open(pfile))
            companion = dict(d.get(dom, {}), source=d.get("source"))
        except Exception:
            companion = None

    # end to end through the C ABI with pinned host buffers: per step the
    # persistent state goes host->device, one step runs, the state comes back
    fields = ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az")
    host = {k: torch.empty(N, dtype=torch.float32, pin_memory=True).numpy() for k in fields}
    sim.get_state(fields, out=host)
    e2e_steps = max(3, min(args.steps, 20))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.set_state(host)
        sim.step(1)
        sim.get_state(fields, out=host)
    e2e, _ = job_rate(N * e2e_steps, time.perf_counter() - t0, dist, "cuda")
    nbytes = len(fields) * 4 * N

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu and args.workload == "bubble2m":
        ps = cpu_sample_params()
        st = oracle_initial_state(ps)
        nsteps = args.cpu_steps
        if nsteps <= 0:   # size the sample to about 12 s of CPU work
            t1, _, _ = time_oracle(ps, st, 1)
            nsteps = int(min(400, max(3, round(12.0 / max(t1, 1e-3)))))
        tc, cores, _ = time_oracle(ps, st, nsteps)
        cpu = {"value": ps.n_particles * nsteps / tc, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d consecutive FP64 steps of the 131,072-particle moist-bubble box "
                         "(same cells and physics, 5 x 5 km footprint) in %.1f s" % (nsteps, tc)}

    ctl = sim.control()
    if rank == 0:
        line = {
            "metric": metric_for(p), "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_string(args.workload),
                       "particles": N, "cells": C, "dt_s": ctl["dt"], "advance_steps": args.advance,
                       "l2": "working set %.0f MB > 129 MB L2 (no flush needed)" % ((N * 164 + C * 20) / 1e6),
                       "parallelism": "replicas x%d" % ws},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_source": src, "traffic": traffic,
                         "companion": companion,
                         "step_achieved": algo["step"] / (ph_ms["step"] / 1e3) / 1e9,
                         "kernel_ms": ph_ms},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "steps": e2e_steps, "api": "asph_set_state + asph_step(1) + asph_get_state, pinned host SoA"},
            "gpu_launches": per_step * args.steps,
            "clocks": clk,
            "state": {"simt": ctl["simt"], "steps_done": ctl["step"], "aborted": ctl["aborted"],
                      "wmax": ctl["wmax"], "deferred_targets_last_step": ctl["deferred"]},
        }
        print(json.dumps(line))
    sim.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_ensemble(args):
    """64 members of uneven size stepped together (one graph launch per
    ensemble step) against the same members stepped one after another
    through the plain step, with the same tuned options."""
    import torch
    import sph_cuda_gb300 as sph

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    members = sph.ensemble_members(64, seed=7)
    total = sum(int(p.n_particles) for p in members)
    ens = sph.Ensemble(members, stream=stream.cuda_stream)
    ens.init()
    t0 = time.perf_counter()
    chosen = ens.tune(trial_steps=3, sort_choices=(0, 1, 2)) if not args.no_tune else []
    t_tune = time.perf_counter() - t0
    ens.step(args.warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    e0.record(stream)
    ens.step_async(args.steps)
    e1.record(stream)
    e1.synchronize()
    ens.sync()
    clk = clocks.stop()
    ms_ens = e0.elapsed_time(e1)
    # the same members one after another, each through its own captured plain step
    views = [ens.member(k) for k in range(len(members))]
    for v in views:
        v.step(1)
    member_kernels = sum(v.step_kernels() for v in views)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for v in views:
        v.step_async(args.steps)
    for v in views:
        v.sync()
    ms_seq = (time.perf_counter() - t0) * 1e3
    line = {
        "metric": "aggregate particle-steps/s (64-member ensemble)", "value": total * args.steps / (ms_ens / 1e3),
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_ens / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ensemble of 64 members, particle counts log-uniform in [16384, 524288] (seed 7), "
                               "small-box atmosphere at fixed spacing, theta noise 0.1 K",
                   "members": len(members), "particles_total": total,
                   "particles_min": min(int(p.n_particles) for p in members),
                   "particles_max": max(int(p.n_particles) for p in members)},
        "sequential": {"value": total * args.steps / (ms_seq / 1e3), "ms_per_step": ms_seq / args.steps,
                       "how": "each member's own graph-launched plain step, members one after another"},
        "speedup_vs_sequential": ms_seq / ms_ens,
        "tuning": {"seconds": t_tune, "chosen_shape_counts": {str(s): sum(1 for c in chosen if c[0] == s)
                                                               for s in sorted(set(c[0] for c in chosen))},
                   "chosen_sort_counts": {str(s): sum(1 for c in chosen if c[1] == s)
                                          for s in sorted(set(c[1] for c in chosen))}},
        "gpu_launches": args.steps * member_kernels,
        "clocks": clk,
    }
    print(json.dumps(line))
    ens.close()
    return 0


def run_adjoint(args):
    """Adjoint window on the 262,144-particle small-box workload: K plain
    steps against one window of K steps (forward with checkpoints every 10
    steps, backward with recompute) of the final cloud-water misfit."""
    import torch
    import sph_cuda_gb300 as sph
    from sph_cuda_gb300.adjoint import AdjointWindow, misfit, seeded_gaussians

    torch.cuda.set_device(0)
    p = sph.preset("adjoint262k")
    sim = sph.Asph(p)
    sim.init()
    start = sim.snapshot()
    K = args.steps
    sim.step(max(args.warmup, 1))
    # the plain steps from the window's start, three times; the fastest is the
    # denominator (the conservative choice for the ratio)
    t_plain = float("inf")
    for _ in range(3):
        sim.restore(start)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.step(K)
        t_plain = min(t_plain, (time.perf_counter() - t0) / K)
    sim.restore(start)
    sim.sync()
    win = AdjointWindow(sim, K, 10)
    gauss = seeded_gaussians(p.nx * p.dx, p.ny * p.dy, p.nz * p.dz, n=4, seed=0)
    fin = win.forward()                      # warm: allocations, first launches
    L, dqc, dxyz = misfit(fin, gauss)
    win.backward(dL_dqc=dqc, dL_dxyz=dxyz)
    t0 = time.perf_counter()
    fin = win.forward()
    t_fwd = time.perf_counter() - t0
    L, dqc, dxyz = misfit(fin, gauss)
    t0 = time.perf_counter()
    dth, da, db = win.backward(dL_dqc=dqc, dL_dxyz=dxyz)
    t_bwd = time.perf_counter() - t0
    ratio = (t_fwd + t_bwd) / K / t_plain
    line = {
        "metric": "adjoint step time / forward step time (262,144 particles)", "value": ratio, "unit": "x",
        "higher_is_better": False, "n_gpus": 1, "steps": K, "warmup": args.warmup, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "small-box atmosphere, 64 x 64 x 64 lattice, 50 x 50 x 100 cells, "
                               "checkpoints every 10 steps, misfit of final cloud water to 4 seeded Gaussians",
                   "particles": int(p.n_particles)},
        "plain_ms_per_step": t_plain * 1e3, "window_forward_ms_per_step": t_fwd * 1e3 / K,
        "backward_ms_per_step": t_bwd * 1e3 / K,
        "loss": L, "grad": {"max_abs_dtheta0": float(np.abs(dth).max()), "dalpha": da, "dbeta": db},
    }
    print(json.dumps(line))
    win.close()
    sim.close()
    return 0


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)   # the moist bubble's 500 steps
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=0, help="0: about 12 s of oracle steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--advance", type=int, default=0,
                    help="untimed steps after init, before warm-up (profile a developed state)")
    ap.add_argument("--workload", default="bubble2m",
                    choices=["bubble2m", "bubble524k", "reference128", "large16m", "ensemble64", "adjoint262k"])
    ap.add_argument("--no-tune", action="store_true", help="ensemble64: skip the autotuner")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    return args


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble64":
        return run_ensemble(args)
    if args.workload == "adjoint262k":
        return run_adjoint(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
