"""Slab decomposition (sph_cuda_gb300.slabs) on CPU ranks (gloo).

Each rank steps its slab with the FP64 oracle as the step engine; after K
steps, the owned particles of all ranks (in global-id order), the rain grid,
the surface precipitation, the dt sequence and the FP64 audit equal a
single-domain oracle run of the same K steps to 1e-12 normwise (the sums
inside a cell may run in another particle order).  This checks the halo
width, the halo and rain exchange, the migration and the reductions; the
engine on a GPU rank is the library (AsphEngine).
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

K = 4


def _config():
    from statebuild import small_config
    from oracle import oracle
    p = small_config(lat=(16, 16, 16), grid=(20, 20, 40), box=(4000.0, 4000.0, 2000.0), sort_every=1)
    # an explicit particle mass: a rank's engine runs a subset of the
    # particles and must use the global mass per particle (a float field)
    p.pmass = oracle.derived(p)["pmass"]
    return p


def _initial(p):
    from statebuild import random_state
    s = random_state(p, 31, "uniform", speed=30.0, shuffle=True)
    s = {k: np.asarray(v, np.float64) for k, v in s.items()}
    N = p.n_particles
    s["prs"] = np.zeros(N)
    s["dthdt"] = np.zeros(N)
    rng = np.random.default_rng(5)
    C = p.nx * p.ny * p.nz
    rain = np.where(rng.uniform(size=C) < .3, rng.uniform(0, 3e4, C), 0.0)
    return s, rain


def _oracle_engine(pmass):
    from oracle import oracle

    def engine(p, local, rain, precip, simt, dt):
        q = p.copy()
        q.n_particles = int(local["x"].size)
        q.pmass = pmass
        ctl = [simt, dt, 1e9, 0.5, 0, 0, 1, 0, 0]
        perm, _ = oracle.stable_sort(oracle.keys(q, local["x"], local["y"], local["z"]), oracle.key_bits(q))
        st, rg, pr, _, rc = oracle.run(q, local, 1, rain, precip, ctl)
        assert rc == 0
        return st, rg, pr, perm
    return engine


def _oracle_controller(p, umax, dt, trips):
    from oracle import oracle
    c = oracle.cfl(p, umax, dt, trips)
    return c["dt"], c["trips"], c["clamp"], c["abort"]


def _global_run(p, s, rain):
    """K single-domain oracle steps, tracking each particle's global id
    through the stable sort that begins every step."""
    from oracle import oracle
    ids = np.arange(p.n_particles)
    st = {k: v.copy() for k, v in s.items()}
    rg, pr = rain.copy(), np.zeros(p.nx * p.ny)
    ctl = [0.0, oracle.derived(p)["dt_cap"], 1e9, 0.5, 0, 0, 1, 0, 0]
    dts = []
    for _ in range(K):
        perm, _ = oracle.stable_sort(oracle.keys(p, st["x"], st["y"], st["z"]), oracle.key_bits(p))
        ids = ids[perm]
        dts.append(ctl[1])
        st, rg, pr, ctl, rc = oracle.run(p, st, 1, rg, pr, list(ctl))
        assert rc == 0
    order = np.argsort(ids)
    return {k: v[order] for k, v in st.items()}, rg, pr, dts, ctl


def _rank_main(rank, world, port, out, halo):
    import torch.distributed as dist
    from oracle import oracle
    from sph_cuda_gb300 import slabs
    oracle.set_threads(2)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p = _config()
        s, rain = _initial(p)
        pmass = oracle.derived(p)["pmass"]
        plan = slabs.SlabPlan(p, world, halo=halo)
        r = slabs.SlabRank(p, plan, rank, dist, _oracle_engine(pmass), _oracle_controller)
        r.scatter(s, rain, dt=oracle.derived(p)["dt_cap"])
        own0 = r.ids.copy()
        dts = []
        for _ in range(K):
            dts.append(r.dt)
            r.step()
        ids, f = r.gather()
        g_rain = r.gather_rain()
        audit = r.audit(pmass)
        out.put((rank, own0, r.ids.copy(), ids, f, g_rain, r.precip if rank == 0 else None, dts, r.dt, audit))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_slab_plan_and_layers():
    from sph_cuda_gb300 import slabs
    p = _config()
    plan = slabs.SlabPlan(p, 3)
    assert list(plan.bounds) == [0, 13, 27, 40]
    assert list(plan.owner([0, 12, 13, 26, 27, 39])) == [0, 0, 1, 1, 2, 2]
    assert plan.halo_range(0) == (0, 19) and plan.halo_range(1) == (7, 33) and plan.halo_range(2) == (21, 40)
    z = np.array([0.0, 49.999, 50.0, 1999.9, 2000.0, 2500.0], np.float32)
    assert list(slabs.cell_layer(p, z)) == [0, 0, 1, 39, 39, 39]
    with pytest.raises(ValueError):
        slabs.SlabPlan(p, 2, bounds=[0, 40, 40])


def test_host_cfl_control_matches_oracle():
    from oracle import oracle
    from sph_cuda_gb300 import slabs
    p = _config()
    dt = oracle.derived(p)["dt_cap"]
    for umax in ([1.0, 2.0, 3.0], [40.0, 30.0, 90.0], [5.0, 5.0, 1500.0]):
        a = slabs.cfl_control(p, umax, dt, 0)
        b = oracle.cfl(p, umax, dt, 0)
        assert a[0] == pytest.approx(b["dt"], rel=1e-6) and a[1] == b["trips"] and a[2] == b["clamp"]


def _run_slabs(world, halo):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q, halo)) for r in range(world)]
    for pr in procs:
        pr.start()
    res = sorted([q.get(timeout=300) for _ in procs], key=lambda t: t[0])
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    return res


def _nw(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_a_halo_narrower_than_two_windows_is_caught():
    """With 2 layers of halo the pressure force on particles next to a
    slab boundary misses neighbours' contributions: the check sees it."""
    p = _config()
    s, rain = _initial(p)
    ref = _global_run(p, s, rain)[0]
    f = _run_slabs(2, 2)[0][4]
    assert _nw(f["ax"], ref["ax"]) > 1e-6


@pytest.mark.parametrize("world", [2, 3])
def test_slabs_equal_the_single_domain_step(world):
    from oracle import oracle
    from sph_cuda_gb300 import slabs
    p = _config()
    s, rain = _initial(p)
    ref, ref_rain, ref_precip, ref_dts, ref_ctl = _global_run(p, s, rain)
    res = _run_slabs(world, slabs.HALO)
    _, _, _, ids, f, g_rain, precip, dts, dt_next, audit = res[0]
    assert np.array_equal(ids, np.arange(p.n_particles))
    assert sum(t[2].size for t in res) == p.n_particles
    assert all(t[1].size > 0 for t in res)
    # particles changed slabs during the run (the migration was exercised)
    moved = sum(np.setdiff1d(t[2], t[1]).size for t in res)
    assert moved > 0

    for k in ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az", "prs", "dthdt"):
        assert _nw(f[k], ref[k]) < 1e-12, (k, _nw(f[k], ref[k]))
    assert _nw(g_rain, ref_rain) < 1e-12
    assert _nw(precip, ref_precip) < 1e-12
    assert np.allclose(dts, ref_dts, rtol=1e-12, atol=0) and dt_next == pytest.approx(ref_ctl[1], rel=1e-12)
    aud = oracle.audit(p, ref)
    for k in range(6):
        assert audit[k] == pytest.approx(aud[k], rel=1e-12, abs=1e-12 * abs(aud[1]))
    for t in res[1:]:
        assert np.array_equal(t[3], ids) and np.allclose(t[9], audit, rtol=0, atol=0)


def _gpu_rank_main(rank, world, port, out):
    import torch.distributed as dist
    from sph_cuda_gb300 import slabs
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p = _config()
        s, rain = _initial(p)
        s = {k: np.asarray(v, np.float32) for k, v in s.items()}
        eng = slabs.AsphEngine(p.pmass)
        r = slabs.SlabRank(p, slabs.SlabPlan(p, world), rank, dist, eng)
        dt0 = float(np.float32(_dt_cap(p)))
        r.scatter(s, rain, dt=dt0)
        dts = []
        for _ in range(KG):
            dts.append(r.dt)
            r.step()
        ids, f = r.gather()
        g_rain = r.gather_rain()
        eng.close()
        out.put((rank, ids, {k: np.asarray(v, np.float32) for k, v in f.items()}, g_rain, dts))
    finally:
        dist.destroy_process_group()


KG = 3


def _dt_cap(p):
    from sph_cuda_gb300 import slabs
    return slabs.cfl_control(p, [0.0, 0.0, 0.0], 1e9, 0)[0]


@pytest.mark.gpu
def test_slabs_on_the_gpu_equal_the_single_domain_gpu_step():
    """Two ranks, each stepping its slab on the GPU through the library
    (AsphEngine), against one context stepping the whole domain: the same
    particles to 1e-5 normwise after 3 steps (float32 sums inside a cell run
    in another particle order on the two sides)."""
    import torch.multiprocessing as mp
    from sph_cuda_gb300 import Asph
    p = _config()
    s, rain = _initial(p)
    s32 = {k: np.asarray(v, np.float32) for k, v in s.items()}
    sim = Asph(p)
    sim.set_state(s32)
    sim.set_rain(np.asarray(rain, np.float32))
    sim.set_time(0.0, float(np.float32(_dt_cap(p))), True)
    ids = np.arange(p.n_particles)
    for _ in range(KG):
        sim.step(1)
        ids = ids[sim.get_sort()["perm"]]
    ref = sim.get_state()
    ref = {k: v[np.argsort(ids)] for k, v in ref.items()}
    ref_rain = sim.get_rain()[0]
    sim.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gpu_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted([q.get(timeout=600) for _ in procs], key=lambda t: t[0])
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    _, gids, f, g_rain, dts = res[0]
    assert np.array_equal(gids, np.arange(p.n_particles))
    for k in ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az"):
        assert _nw(f[k], ref[k]) < 1e-5, (k, _nw(f[k], ref[k]))
    assert _nw(g_rain, ref_rain) < 1e-5
