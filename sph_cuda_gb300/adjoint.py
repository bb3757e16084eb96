"""Adjoint window: gradients of a loss of the final state with respect to the
initial theta of every particle and the viscosity coefficients.

    win = AdjointWindow(sim, nsteps=100, every=10)     # window starts at sim's state
    fin = win.forward(theta0)                          # final state (dict of arrays)
    dth0, dalpha, dbeta = win.backward(dL_dqc=..., dL_dxyz=...)

`window_function()` wraps the pair as a torch.autograd.Function:
forward(theta0, alpha, beta) -> (qc_final, xyz_final); backward gives the
gradients of theta0, alpha and beta.  Every call is one C-ABI call into
libasph.so (asph_adj_*); there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import Asph, _check, _fptr


class AdjointWindow:
    def __init__(self, sim: Asph, nsteps: int, every: int = 10):
        self.sim = sim
        self.lib = sim.lib
        self.nsteps = int(nsteps)
        self.every = int(every)
        self._h = C.c_void_p()
        _check(self.lib.asph_adj_create(sim._ctx, self.nsteps, self.every, C.byref(self._h)))
        self.start = sim.snapshot()   # the window's initial state, restored by every forward

    def close(self) -> None:
        if self._h:
            self.lib.asph_adj_destroy(self._h)
            self._h = C.c_void_p()
        if self.start is not None:
            self.start.close()
            self.start = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def start_state(self) -> dict:
        self.sim.restore(self.start)
        return self.sim.get_state()

    def forward(self, theta0=None, alpha: float | None = None, beta: float | None = None) -> dict:
        """Run the window from its initial state (theta replaced by theta0
        when given, in the initial state's order); returns the final state."""
        self.sim.restore(self.start)
        if theta0 is not None:
            st = self.sim.get_state()
            st["th"] = np.ascontiguousarray(theta0, np.float32)
            self.sim.set_state(st)
        if alpha is not None or beta is not None:
            self.sim.set_viscosity(self.sim.params.alpha_av if alpha is None else alpha,
                                   self.sim.params.beta_av if beta is None else beta)
        _check(self.lib.asph_adj_forward(self._h))
        return self.sim.get_state()

    def backward(self, dL_dqc=None, dL_dtheta=None, dL_dxyz=None):
        """dL/d(final qc, theta, positions) in the final state's order ->
        (dL/dtheta0[N] in the initial order, dL/dalpha, dL/dbeta)."""
        N = self.sim.N
        keep = []

        def arr(a, n):
            if a is None:
                return None
            b = np.ascontiguousarray(a, np.float32).reshape(n)
            keep.append(b)
            return _fptr(b)

        out = np.empty(N, np.float32)
        ab = np.zeros(2, np.float64)
        _check(self.lib.asph_adj_backward(self._h, arr(dL_dqc, N), arr(dL_dtheta, N), arr(dL_dxyz, 3 * N),
                                          _fptr(out), ab.ctypes.data_as(C.POINTER(C.c_double))))
        return out, float(ab[0]), float(ab[1])


def gaussian_target(gauss, x, y, z):
    """T(x) = sum_k a_k exp(-((x-cx)^2 + (y-cy)^2) / (2 s^2) - (z-cz)^2 / (2 sz^2)),
    rows of gauss = (cx, cy, cz, s, sz, a); returns (T, dT/dx, dT/dy, dT/dz)."""
    x, y, z = (np.asarray(a, np.float64) for a in (x, y, z))
    T = np.zeros_like(x)
    gx, gy, gz = np.zeros_like(x), np.zeros_like(x), np.zeros_like(x)
    for cx, cy, cz, s, sz, a in np.asarray(gauss, np.float64).reshape(-1, 6):
        e = a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s) - (z - cz) ** 2 / (2 * sz * sz))
        T += e
        gx += -e * (x - cx) / (s * s)
        gy += -e * (y - cy) / (s * s)
        gz += -e * (z - cz) / (sz * sz)
    return T, gx, gy, gz


def seeded_gaussians(lx: float, ly: float, lz: float, n: int = 4, seed: int = 0, amplitude: float = 1e-4):
    """n smooth target bumps inside the box (widths a quarter of the box)."""
    rng = np.random.default_rng(seed)
    g = np.zeros((n, 6))
    g[:, 0] = rng.uniform(0.2, 0.8, n) * lx
    g[:, 1] = rng.uniform(0.2, 0.8, n) * ly
    g[:, 2] = rng.uniform(0.1, 0.5, n) * lz
    g[:, 3] = 0.25 * min(lx, ly)
    g[:, 4] = 0.15 * lz
    g[:, 5] = amplitude
    return g


def misfit(final: dict, gauss):
    """L = mean (qc - T(x))^2 and its gradient with respect to the final qc and positions."""
    T, gx, gy, gz = gaussian_target(gauss, final["x"], final["y"], final["z"])
    d = np.asarray(final["qc"], np.float64) - T
    N = d.size
    L = float(np.mean(d * d))
    dqc = 2.0 * d / N
    dxyz = np.concatenate([-dqc * gx, -dqc * gy, -dqc * gz])
    return L, dqc, dxyz


def window_function():
    """torch.autograd.Function over an AdjointWindow:
    apply(theta0, alpha, beta, window) -> (qc_final, xyz_final[3, N])."""
    import torch

    class WindowFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta0, alpha, beta, window):
            fin = window.forward(theta0.detach().cpu().numpy(), float(alpha), float(beta))
            ctx.window = window
            qc = torch.from_numpy(np.asarray(fin["qc"], np.float32).copy())
            xyz = torch.from_numpy(np.stack([fin["x"], fin["y"], fin["z"]]).astype(np.float32))
            return qc, xyz

        @staticmethod
        def backward(ctx, g_qc, g_xyz):
            dth, da, db = ctx.window.backward(
                None if g_qc is None else g_qc.detach().cpu().numpy(), None,
                None if g_xyz is None else g_xyz.detach().cpu().numpy().reshape(-1))
            return (torch.from_numpy(dth), torch.tensor(da, dtype=torch.float64),
                    torch.tensor(db, dtype=torch.float64), None)

    return WindowFunction
