"""Benchmark: particle-steps/s of the full SPH warm-rain step.

Workload: the 2,097,152-particle moist-bubble configuration (128^3 jittered lattice in a 20 x 20 x 8 km box, cells 150.4 x 150.4 x 40 m,
three seeded warm bubbles, warm rain with accretion and evaporation, Morton
re-sort every step).  Synthetic, seeded initial state; no dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours: K fused steps (sort + gather/kick/drift/flux + density/EOS/micro +
momentum/integrate/rain/CFL, one CUDA graph per step) timed with CUDA events
on the simulation stream; one JSON line on rank 0.  Beside it: the per-kernel
times over the same K states, the reference's own kernels on this GPU
(`reference_gpu`) and the FP64 CPU port (`cpu_baseline`), both from the same
initial state, and the two other forms at their own configurations
(`forms`: the 64-member ensemble against its members run one after another,
the adjoint step against the plain step).  --impl reference times the CPU
restatement of the reference (FP64, all host cores) on the full
configuration.
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


def oracle_timed(p, warmup: int, steps: int = 0, budget_s: float = 12.0):
    """FP64 oracle steps (all host threads) of the full configuration, from
    the state the library's init leaves (restated by the oracle): `warmup`
    untimed steps, then `steps` timed steps, or, with steps = 0, as many as
    fill about `budget_s` seconds.  Returns (seconds, steps, threads)."""
    from oracle import oracle
    s = oracle.initial_state(p)
    rain = s["rain"]
    st, rg, pr, ctl, _ = oracle.run(p, s, max(warmup, 1), rain)
    if steps <= 0:
        t0 = time.perf_counter()
        st, rg, pr, ctl, _ = oracle.run(p, st, 1, rg, pr, ctl)
        t1 = time.perf_counter() - t0
        steps = int(min(400, max(3, round(budget_s / max(t1, 1e-3)))))
    t0 = time.perf_counter()
    oracle.run(p, st, steps, rg, pr, ctl)
    return time.perf_counter() - t0, steps, oracle.threads()


def workload_string(name: str) -> str:
    return {"bubble2m": "moist bubble, 2,097,152 particles, 133x133x200 cells, sort every step",
            "bubble524k": "moist bubble, 524,288 particles, 66x66x200 cells, sort every step",
            "reference128": "the reference's own geometry and init, 128x128x128 cells, dt 0.25 s, "
                            "sort every step",
            "large2m": "the large run's 8:1 cells and physics on a 20 x 20 x 5 km box, 2,097,152 particles, "
                       "125x125x250 cells (h 160 m x 20 m), sort every step",
            "large16m": "large anisotropic run, 16,777,216 particles, 250x250x500 cells (h 160 m x 20 m), "
                        "95% RH boundary layer, theta noise 0.2 K, sort every step"}[name]


def metric_for(p) -> str:
    return "particle-steps/s (plain step, {:,} particles)".format(int(p.n_particles))


def run_reference(args):
    """The reference's CPU path: the FP64 oracle port (the reference has no
    CPU implementation of its step) with all host threads, on the full
    configuration of the workload: init, W warm-up steps, K timed steps.
    Parameters come from the oracle's own preset table, so this arm neither
    imports the product package nor loads the CUDA library."""
    ws, rank, local = dist_setup()
    if rank != 0:
        return 0
    from oracle import params
    if args.workload not in ("bubble2m", "bubble524k", "reference128", "large16m"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no form of the %s workload"
                          % args.workload}))
        return 0
    p = params.workload(args.workload)
    t, steps, cores = oracle_timed(p, args.warmup, args.steps)
    value = p.n_particles * steps / t
    sample = ("the full configuration (%d particles, %d cells): %d FP64 steps after init and %d warm-up steps"
              % (p.n_particles, p.nx * p.ny * p.nz, steps, max(args.warmup, 1)))
    line = {
        "impl": "reference", "metric": metric_for(p), "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload_string(args.workload), "particles": p.n_particles,
                   "cells": p.nx * p.ny * p.nz},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def reference_gpu(args, ours_value: float):
    """The reference's own kernels (asph_h100.cu compiled for sm_103a with
    the workload's cell sizes) in its host step loop on this GPU, from the
    same initial state, W untimed steps then K timed: the comparator of the
    plain step.  Runs after our timed region, in a child process."""
    if args.workload not in ("bubble2m", "reference128"):
        return None
    script = os.path.join(ROOT, "oracle", "time_reference.py")
    mode = "bubble2m" if args.workload == "bubble2m" else "native"
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    try:
        r = subprocess.run([sys.executable, script, mode, str(args.steps), str(max(args.warmup, 1))],
                           capture_output=True, text=True, timeout=900)
    except Exception as e:   # the harness is test infrastructure: report, do not fail the bench
        clocks.stop()
        return {"unavailable": "reference kernels did not run: %s" % str(e).splitlines()[0]}
    clk = clocks.stop()
    line = None
    for ln in r.stdout.splitlines():
        if ln.startswith("{") and "reference-gpu" in ln:
            line = json.loads(ln)
    if r.returncode != 0 or line is None:
        tail = (r.stderr or r.stdout or "").strip().splitlines()[-1:] or ["no output"]
        return {"unavailable": "reference kernels exited %d: %s" % (r.returncode, tail[0])}
    return {"ms_per_step": line["ms_per_step"], "particle_steps_per_s": line["particle_steps_per_s"],
            "steps": line["steps"], "warmup": line.get("warmup"), "speedup": ours_value / line["particle_steps_per_s"],
            "how": "asph_h100.cu's kernels (cubin built from the reference source with its own flags, cell sizes "
                   "of the workload) in its step loop: CUB sort every step, host CFL read-back per step",
            "clocks": clk}


def traffic_record(workload: str, steps_before: int, steps: int, kernel: str):
    """DRAM bytes of one launch of `kernel` captured by ncu in the state the
    line's per-kernel times cover: profiles/traffic_<workload>.json holds
    captures keyed by the number of steps completed before the captured
    launch, each standing for a timed region of at most `max_steps` steps
    from there.  No capture for this state: None (the line says so)."""
    path = os.path.join(ROOT, "profiles", "traffic_%s.json" % workload)
    if not os.path.exists(path):
        return None
    try:
        d = json.load(open(path))
    except Exception:
        return None
    for rec in d.get("captures", []):
        if (rec.get("steps_before") == steps_before and steps <= rec.get("max_steps", 1)
                and kernel in rec.get("bytes", {})):
            return {"bytes": rec["bytes"][kernel], "source": "profiles/traffic_%s.json" % workload,
                    "command": rec.get("command"), "steps_before": steps_before,
                    "companion": rec.get("companion", {}).get(kernel)}
    return None


def workload_params(name: str):
    """bubble2m: the headline 2,097,152-particle moist-bubble workload.
    bubble524k: the same physics, cell size and density on a 10 x 10 x 8 km box
    (64 x 64 x 128 lattice, 66 x 66 x 200 cells) for profiler captures.
    reference128: the reference's own configuration at --nx --ny --nz 128 and
    --dt 0.25 with a sort every step (what oracle/time_reference.py native runs).
    large16m: the 16,777,216-particle anisotropic run (40 x 40 x 10 km, 8:1).
    large2m: its cells, lattice spacing and physics at 2,097,152 particles (a
    20 x 20 x 5 km box: 128^3 lattice, 125 x 125 x 250 cells) for profiler
    captures of the 8:1 kernels."""
    import sph_cuda_gb300 as sph
    if name == "large16m":
        return sph.preset("large16m")
    if name == "large2m":
        p = sph.preset("large16m")
        p.nx = p.ny = 125
        p.nz = 250
        p.lat_nx = p.lat_ny = p.lat_nz = 128
        p.n_particles = 128 ** 3
        return p
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
    steps_before = int(sim.control()["step"])   # steps completed when the timed region starts
    start = sim.snapshot()          # the timed region's first state, replayed for the per-kernel times

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
    ctl = sim.control()

    # per-kernel device times over the very states of the timed region: the
    # same K steps again from the snapshot (results are deterministic), with
    # events between the phases on the simulation stream
    sim.restore(start)
    ph = sim.step_profiled(args.steps)
    ph_ms = {k: v / args.steps for k, v in ph.items()}
    start.close()
    algo = algorithmic_bytes(N, C)
    kernels = ["table_clear", "sort", "gather_kick_drift", "density_eos", "momentum_integrate"]
    dom = max(kernels, key=lambda k: ph_ms[k])
    hbm, src = peaks()
    achieved = algo[dom] / (ph_ms[dom] / 1e3) / 1e9
    # DRAM traffic of the dominant kernel from an ncu capture of the first
    # timed step of this same command (profiles/traffic_<workload>.json)
    trec = traffic_record(args.workload, steps_before, args.steps, dom)

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
    sim.close()

    cpu, ref_gpu, forms = None, None, None
    if rank == 0 and ws == 1:
        if not args.no_reference_gpu:
            ref_gpu = reference_gpu(args, value)
        if not args.no_forms and args.workload == "bubble2m":
            forms = measure_forms()
        if not args.no_cpu:
            tc, nsteps, cores = oracle_timed(p, args.warmup, args.cpu_steps)
            cpu = {"value": N * nsteps / tc, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": "%d FP64 steps of the full configuration after init and %d warm-up steps, in %.1f s"
                             % (nsteps, max(args.warmup, 1), tc)}

    if rank == 0:
        line = {
            "metric": metric_for(p), "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_string(args.workload),
                       "particles": N, "cells": C, "dt_s": ctl["dt"], "advance_steps": args.advance,
                       "steps_before_timed": steps_before,
                       "l2": "working set %.0f MB > 129 MB L2 (no flush needed)" % ((N * 164 + C * 20) / 1e6),
                       "parallelism": "replicas x%d" % ws},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_source": src,
                         "traffic": None if trec is None else trec["bytes"],
                         "traffic_source": ("no ncu capture of steps %d-%d of this workload"
                                            % (steps_before + 1, steps_before + args.steps))
                         if trec is None else "%s: one launch of step %d (%s)" % (trec["source"], steps_before + 1,
                                                                                 trec["command"]),
                         "traffic_over_algorithmic": None if trec is None else trec["bytes"] / algo[dom],
                         "companion": None if trec is None else trec["companion"],
                         "kernel_ms": ph_ms, "kernel_ms_over": "the timed region's %d steps, replayed from a "
                                                               "snapshot with events between phases" % args.steps,
                         "frac_step": algo["step"] / N * (value / ws) / 1e9 / hbm,
                         "step_bytes_per_particle": algo["step"] / N},
            "cpu_baseline": cpu,
            "reference_gpu": ref_gpu,
            "forms": forms,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "steps": e2e_steps, "api": "asph_set_state + asph_step(1) + asph_get_state, pinned host SoA"},
            "gpu_launches": per_step * args.steps,
            "clocks": clk,
            "state": {"simt": ctl["simt"], "steps_done": ctl["step"], "aborted": ctl["aborted"],
                      "wmax": ctl["wmax"], "deferred_targets_last_step": ctl["deferred"]},
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_ensemble(args):
    import torch
    torch.cuda.set_device(0)
    line = measure_ensemble(args.steps, args.warmup, tune=not args.no_tune)
    print(json.dumps(line))
    return 0


def measure_ensemble(steps: int, warmup: int, tune: bool = True) -> dict:
    """64 members of uneven size stepped together (one graph launch per
    ensemble step) against the same members stepped one after another
    through the plain step, with the same tuned options."""
    import torch
    import sph_cuda_gb300 as sph

    stream = torch.cuda.Stream()
    members = sph.ensemble_members(64, seed=7)
    total = sum(int(p.n_particles) for p in members)
    ens = sph.Ensemble(members, stream=stream.cuda_stream)
    ens.init()
    t0 = time.perf_counter()
    chosen = ens.tune(trial_steps=3, sort_choices=(0, 1, 2)) if tune else []
    t_tune = time.perf_counter() - t0
    ens.step(warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    e0.record(stream)
    ens.step_async(steps)
    e1.record(stream)
    e1.synchronize()
    ens.sync()
    clk = clocks.stop()
    ms_ens = e0.elapsed_time(e1)
    # the same members run sequentially through the plain step: member k
    # runs its K graph-launched steps to completion before member k + 1
    # starts (same tuned options, each member continuing from its state)
    views = [ens.member(k) for k in range(len(members))]
    for v in views:
        v.step(1)
    member_kernels = sum(v.step_kernels() for v in views)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for v in views:
        v.step(steps)   # returns when the member's steps are done
    ms_seq = (time.perf_counter() - t0) * 1e3
    line = {
        "metric": "aggregate particle-steps/s (64-member ensemble)", "value": total * steps / (ms_ens / 1e3),
        "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": ms_ens / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ensemble of 64 members, particle counts log-uniform in [16384, 524288] (seed 7), "
                               "small-box atmosphere at fixed spacing, theta noise 0.1 K",
                   "members": len(members), "particles_total": total,
                   "particles_min": min(int(p.n_particles) for p in members),
                   "particles_max": max(int(p.n_particles) for p in members)},
        "sequential": {"value": total * steps / (ms_seq / 1e3), "ms_per_step": ms_seq / steps,
                       "how": "each member's own graph-launched plain step; member k runs its K steps to "
                              "completion before member k+1 starts"},
        "speedup_vs_sequential": ms_seq / ms_ens,
        "tuning": {"seconds": t_tune, "chosen_shape_counts": {str(s): sum(1 for c in chosen if c[0] == s)
                                                               for s in sorted(set(c[0] for c in chosen))},
                   "chosen_sort_counts": {str(s): sum(1 for c in chosen if c[1] == s)
                                          for s in sorted(set(c[1] for c in chosen))},
                   "chosen_targets_per_thread_counts": {str(s): sum(1 for c in chosen if c[2] == s)
                                                        for s in sorted(set(c[2] for c in chosen))}},
        "gpu_launches": steps * member_kernels,
        "clocks": clk,
    }
    ens.close()
    return line


def run_adjoint(args):
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(measure_adjoint(args.steps, args.warmup)))
    return 0


def measure_adjoint(K: int, warmup: int) -> dict:
    """Adjoint window on the 262,144-particle small-box workload: K plain
    steps against one window of K steps (forward with checkpoints every 10
    steps, backward with recompute) of the final cloud-water misfit."""
    import torch
    import sph_cuda_gb300 as sph
    from sph_cuda_gb300.adjoint import AdjointWindow, misfit, seeded_gaussians

    p = sph.preset("adjoint262k")
    sim = sph.Asph(p)
    sim.init()
    start = sim.snapshot()
    sim.step(max(warmup, 1))
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
        "higher_is_better": False, "n_gpus": 1, "steps": K, "warmup": warmup, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "small-box atmosphere, 64 x 64 x 64 lattice, 50 x 50 x 100 cells, "
                               "checkpoints every 10 steps, misfit of final cloud water to 4 seeded Gaussians",
                   "particles": int(p.n_particles)},
        "plain_ms_per_step": t_plain * 1e3, "window_forward_ms_per_step": t_fwd * 1e3 / K,
        "backward_ms_per_step": t_bwd * 1e3 / K,
        "loss": L, "grad": {"max_abs_dtheta0": float(np.abs(dth).max()), "dalpha": da, "dbeta": db},
    }
    win.close()
    start.close()
    sim.close()
    return line


FORM_STEPS = {"ensemble64": 100, "adjoint262k": 100}


def measure_forms() -> dict:
    """The two other forms at their own configurations, after the headline's
    timed region: the 64-member ensemble against its members run one after
    another through the plain step, and the adjoint step against the plain
    step (100-step window, checkpoints every 10 steps)."""
    out = {}
    e = measure_ensemble(FORM_STEPS["ensemble64"], 5)
    out["ensemble64"] = {"value": e["value"], "unit": UNIT, "ms_per_step": e["ms_per_step"], "steps": e["steps"],
                         "sequential_value": e["sequential"]["value"],
                         "speedup_vs_sequential": e["speedup_vs_sequential"],
                         "particles_total": e["config"]["particles_total"], "members": e["config"]["members"],
                         "tuning_s": e["tuning"]["seconds"], "clocks": e["clocks"],
                         "run": "python bench.py --workload ensemble64 --steps 100"}
    a = measure_adjoint(FORM_STEPS["adjoint262k"], 5)
    out["adjoint262k"] = {"adjoint_over_forward": a["value"], "plain_ms_per_step": a["plain_ms_per_step"],
                          "window_forward_ms_per_step": a["window_forward_ms_per_step"],
                          "backward_ms_per_step": a["backward_ms_per_step"], "steps": a["steps"],
                          "run": "python bench.py --workload adjoint262k --steps 100"}
    return out


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)   # the moist bubble's 500 steps
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=0, help="0: about 12 s of oracle steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true", help="skip the reference-kernel comparator")
    ap.add_argument("--advance", type=int, default=0,
                    help="untimed steps after init, before warm-up (profile a developed state)")
    ap.add_argument("--workload", default="bubble2m",
                    choices=["bubble2m", "bubble524k", "reference128", "large16m", "large2m", "ensemble64",
                             "adjoint262k"])
    ap.add_argument("--no-tune", action="store_true", help="ensemble64: skip the autotuner")
    ap.add_argument("--no-forms", action="store_true",
                    help="bubble2m: skip the ensemble and adjoint measurements after the headline")
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
