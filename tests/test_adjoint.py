"""Adjoint window: the CUDA reverse against the FP64 host adjoint and against
central finite differences of the FP64 host forward.

Tolerances: the FP64 host adjoint is pinned against finite differences to
1e-6 normwise (CPU).  The CUDA adjoint runs an FP32 forward and an FP32
reverse; its gradients must match the FP64 host adjoint and finite
differences to 1e-3 relative (normwise over the checked particles), the
bar for the adjoint.
"""
import numpy as np
import pytest

from oracle import oracle
from sph_cuda_gb300 import Asph
from sph_cuda_gb300.adjoint import AdjointWindow, misfit, seeded_gaussians, window_function
from statebuild import random_state, small_config

GRAD_TOL = 1e-3
DT = 0.25   # the static CFL bound of these cells (0.4 x 50 m / 80 m/s)


def _case(seed=3, lat=(8, 8, 16), grid=(12, 12, 30), box=(2400.0, 2400.0, 1500.0), speed=3.0):
    p = small_config(lat=lat, grid=grid, box=box)
    s = random_state(p, seed=seed, speed=speed)
    g = seeded_gaussians(*box, n=4, seed=seed)
    return p, s, g


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _fd(p, s, rain, simt, dt, nsteps, ab, g, idx, eps=1e-3):
    out = []
    for i in idx:
        sp = {k: np.asarray(v, np.float64).copy() for k, v in s.items()}
        sm = {k: np.asarray(v, np.float64).copy() for k, v in s.items()}
        sp["th"][i] += eps
        sm["th"][i] -= eps
        out.append((oracle.adj_loss(p, sp, rain, simt, dt, nsteps, ab, g) -
                    oracle.adj_loss(p, sm, rain, simt, dt, nsteps, ab, g)) / (2 * eps))
    return np.array(out)


# ---- CPU: pin the FP64 host adjoint -------------------------------------------
def test_host_adjoint_matches_finite_differences():
    p, s, g = _case()
    rain = np.zeros(p.nx * p.ny * p.nz)
    ab = (p.alpha_av, 0.1)
    L, dth, da, db = oracle.adj_grad(p, s, rain, 0.0, 0.5, 4, ab, g)
    assert L > 0
    rng = np.random.default_rng(5)
    # the particles that matter: largest gradients, plus random ones
    idx = np.concatenate([np.argsort(-np.abs(dth))[:6], rng.choice(p.n_particles, 4, replace=False)])
    fd = _fd(p, s, rain, 0.0, 0.5, 4, ab, g, idx)
    assert _rel(dth[idx], fd) < 1e-6
    for k, e in ((0, 1e-4), (1, 1e-3)):
        a1, a2 = list(ab), list(ab)
        a1[k] += e
        a2[k] -= e
        f = (oracle.adj_loss(p, s, rain, 0.0, 0.5, 4, a1, g) - oracle.adj_loss(p, s, rain, 0.0, 0.5, 4, a2, g)) / (2 * e)
        assert abs((da, db)[k] - f) <= 1e-6 * abs(f)


def test_seeded_gaussians_and_misfit_gradient():
    g = seeded_gaussians(1000.0, 1000.0, 500.0, seed=1)
    assert g.shape == (4, 6) and np.all(g[:, 5] == 1e-4)
    rng = np.random.default_rng(0)
    fin = {"x": rng.uniform(0, 1000, 50), "y": rng.uniform(0, 1000, 50), "z": rng.uniform(0, 500, 50),
           "qc": rng.uniform(0, 1e-3, 50)}
    L, dqc, dxyz = misfit(fin, g)
    e = 1e-3
    for k, name in enumerate(("x", "y", "z")):
        fp = dict(fin); fp[name] = fin[name].copy(); fp[name][7] += e
        fm = dict(fin); fm[name] = fin[name].copy(); fm[name][7] -= e
        fd = (misfit(fp, g)[0] - misfit(fm, g)[0]) / (2 * e)
        assert abs(dxyz[k * 50 + 7] - fd) <= 1e-6 * max(abs(fd), 1e-30) + 1e-20


# ---- GPU --------------------------------------------------------------------------
def _gpu_window(p, s, nsteps, every, alpha=None, beta=0.1):
    sim = Asph(p)
    sim.set_state(s)
    sim.sort_build()            # fresh surface flags; the window starts in this order
    sim.set_time(0.0, DT, True)
    start = sim.get_state()
    win = AdjointWindow(sim, nsteps, every)
    return sim, win, start


def _gpu_grad(p, s, g, nsteps, every, beta=0.1):
    sim, win, start = _gpu_window(p, s, nsteps, every)
    fin = win.forward(alpha=p.alpha_av, beta=beta)
    L, dqc, dxyz = misfit(fin, g)
    dth, da, db = win.backward(dL_dqc=dqc, dL_dxyz=dxyz)
    return sim, win, start, fin, L, dth, da, db


@pytest.mark.gpu
def test_window_forward_matches_fp64_host():
    p, s, g = _case()
    sim, win, start = _gpu_window(p, s, 4, 2)
    rain0 = np.zeros(p.nx * p.ny * p.nz)
    fin = win.forward(alpha=p.alpha_av, beta=0.1)
    L_gpu = misfit(fin, g)[0]
    L_host, hfin = oracle.adj_loss(p, start, rain0, 0.0, DT, 4, (p.alpha_av, 0.1), g, final=True)
    assert abs(L_gpu - L_host) <= 1e-4 * L_host
    # same particles, different order: compare sorted values
    for k in ("th", "qv", "z"):
        assert _rel(np.sort(fin[k]), np.sort(hfin[k])) < 1e-5, k
    sim.close()


@pytest.mark.gpu
def test_gpu_adjoint_matches_fp64_host_adjoint():
    p, s, g = _case()
    sim, win, start, fin, L, dth, da, db = _gpu_grad(p, s, g, 4, 2)
    rain0 = np.zeros(p.nx * p.ny * p.nz)
    Lh, dth_h, da_h, db_h = oracle.adj_grad(p, start, rain0, 0.0, DT, 4, (p.alpha_av, 0.1), g)
    assert _rel(dth, dth_h) < GRAD_TOL
    assert abs(da - da_h) <= GRAD_TOL * abs(da_h)
    assert abs(db - db_h) <= GRAD_TOL * abs(db_h)
    sim.close()


@pytest.mark.gpu
def test_gpu_adjoint_matches_finite_differences_on_32_particles():
    p, s, g = _case(seed=7, lat=(10, 10, 20), grid=(14, 14, 36), box=(2800.0, 2800.0, 1800.0))
    sim, win, start, fin, L, dth, da, db = _gpu_grad(p, s, g, 6, 3)
    rain0 = np.zeros(p.nx * p.ny * p.nz)
    rng = np.random.default_rng(7)
    idx = np.concatenate([np.argsort(-np.abs(dth))[:16], rng.choice(p.n_particles, 16, replace=False)])
    fd = _fd(p, start, rain0, 0.0, DT, 6, (p.alpha_av, 0.1), g, idx)
    assert _rel(dth[idx], fd) < GRAD_TOL
    sim.close()


def _dry(s, p):
    """No cloud and vapour well below saturation: the microphysics is idle
    and the gradient flows through the dynamics alone."""
    d = dict(s)
    h = oracle.helpers(p, np.asarray(s["z"], np.float64), np.full(p.n_particles, 280.0),
                       np.full(p.n_particles, 9e4), np.zeros(p.n_particles))
    d["qv"] = (0.5 * h[:, 4]).astype(np.float32)
    d["qc"] = np.zeros(p.n_particles, np.float32)
    return d


@pytest.mark.gpu
def test_gpu_adjoint_dry_dynamics_matches_fp64_host_adjoint():
    """Positions carry the loss (a target of 2e-3 against zero cloud water),
    so every dynamic path of the reverse is exercised over 6 steps."""
    p, s, _ = _case(seed=5, speed=4.0)
    s = _dry(s, p)
    g = seeded_gaussians(2400.0, 2400.0, 1500.0, n=4, seed=5, amplitude=2e-3)
    g[:, 3] *= 0.5
    g[:, 4] *= 0.5
    sim, win, start, fin, L, dth, da, db = _gpu_grad(p, s, g, 6, 3)
    rain0 = np.zeros(p.nx * p.ny * p.nz)
    Lh, dth_h, da_h, db_h = oracle.adj_grad(p, start, rain0, 0.0, DT, 6, (p.alpha_av, 0.1), g)
    assert abs(L - Lh) <= 1e-4 * Lh
    assert np.max(np.abs(dth_h)) > 0
    assert _rel(dth, dth_h) < GRAD_TOL
    assert abs(da - da_h) <= GRAD_TOL * abs(da_h)
    assert abs(db - db_h) <= 1e-2 * abs(db_h)
    sim.close()


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_the_gradient():
    p, s, g = _case()
    res = []
    for every in (1, 2, 4):
        sim, win, start, fin, L, dth, da, db = _gpu_grad(p, s, g, 4, every)
        res.append((dth, da, db))
        sim.close()
    for dth, da, db in res[1:]:
        assert _rel(dth, res[0][0]) < 1e-5
        assert abs(da - res[0][1]) <= 1e-5 * abs(res[0][1])


@pytest.mark.gpu
def test_backward_leaves_the_end_of_window_state():
    p, s, g = _case()
    sim, win, start = _gpu_window(p, s, 4, 2)
    fin = win.forward()
    L, dqc, dxyz = misfit(fin, g)
    win.backward(dL_dqc=dqc, dL_dxyz=dxyz)
    after = sim.get_state()
    for k in ("x", "th", "qc", "u"):
        assert np.array_equal(after[k], fin[k]), k
    sim.close()


@pytest.mark.gpu
def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    p, s, g = _case()
    sim, win, start = _gpu_window(p, s, 4, 2)
    F = window_function()
    th0 = torch.tensor(start["th"], dtype=torch.float32, requires_grad=True)
    alpha = torch.tensor(float(p.alpha_av), dtype=torch.float64, requires_grad=True)
    beta = torch.tensor(0.1, dtype=torch.float64, requires_grad=True)
    qc, xyz = F.apply(th0, alpha, beta, win)
    gt = torch.from_numpy(seeded_gaussians(2400.0, 2400.0, 1500.0, n=4, seed=3))
    x, y, z = xyz.double()
    T = torch.zeros_like(x)
    for cx, cy, cz, sg, sz, a in gt:
        T = T + a * torch.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sg * sg) - (z - cz) ** 2 / (2 * sz * sz))
    loss = ((qc.double() - T) ** 2).mean()
    loss.backward()
    fin = win.forward(start["th"], p.alpha_av, 0.1)
    L, dqc, dxyz = misfit(fin, g)
    dth, da, db = win.backward(dL_dqc=dqc, dL_dxyz=dxyz)
    assert _rel(th0.grad.numpy(), dth) < 1e-4
    assert abs(alpha.grad.item() - da) <= 1e-4 * abs(da)
    sim.close()
