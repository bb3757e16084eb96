"""Seeded synthetic particle states for the parity tests."""
import numpy as np

from oracle import oracle
from sph_cuda_gb300 import preset


def small_config(lat=(16, 16, 16), grid=(20, 20, 40), box=(4000.0, 4000.0, 2000.0), **kw):
    """Config-mode physics (4 K/km, RH profile, warm rain with accretion and
    evaporation) on a small box: the 200 m x 50 m cells of the 65,536-particle preset."""
    p = preset("small65k")
    p.nx, p.ny, p.nz = grid
    p.dx, p.dy, p.dz = box[0] / grid[0], box[1] / grid[1], box[2] / grid[2]
    p.lat_nx, p.lat_ny, p.lat_nz = lat
    p.n_particles = lat[0] * lat[1] * lat[2]
    p.bubble_x[0], p.bubble_y[0], p.bubble_z[0], p.bubble_r[0] = box[0] / 2, box[1] / 2, 500.0, 600.0
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def reference_geometry(nx, ny, nz, **kw):
    p = preset("reference", nx, ny, nz)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def random_state(p, seed=0, layout="jitter", speed=6.0, shuffle=True):
    """A physically plausible state: positions (jittered lattice, uniform,
    clustered, one cell), velocities, theta near the sounding, vapour near
    saturation, some cloud water, density perturbed about rho_ref."""
    rng = np.random.default_rng(seed)
    N = int(p.n_particles)
    Lx, Ly, Lz = p.nx * p.dx, p.ny * p.dy, p.nz * p.dz
    if layout == "jitter":
        n3 = (p.lat_nx, p.lat_ny, p.lat_nz) if p.lat_nx * p.lat_ny * p.lat_nz == N else (p.nx, p.ny, N // (p.nx * p.ny))
        i = np.arange(N)
        ix, iy, iz = i % n3[0], (i // n3[0]) % n3[1], i // (n3[0] * n3[1])
        x = (ix + 0.5 + rng.uniform(-.3, .3, N)) * Lx / n3[0]
        y = (iy + 0.5 + rng.uniform(-.3, .3, N)) * Ly / n3[1]
        z = (iz + 0.5 + rng.uniform(-.3, .3, N)) * Lz / n3[2]
    elif layout == "uniform":
        x, y, z = rng.uniform(0, Lx, N), rng.uniform(0, Ly, N), rng.uniform(0, Lz, N)
    elif layout == "cluster":
        c = rng.uniform([.1, .1, .1], [.9, .9, .9], (5, 3)) * [Lx, Ly, Lz]
        k = rng.integers(0, 5, N)
        x = np.mod(c[k, 0] + rng.normal(0, 1.5 * p.dx, N), Lx)
        y = np.mod(c[k, 1] + rng.normal(0, 1.5 * p.dy, N), Ly)
        z = np.clip(np.abs(c[k, 2] + rng.normal(0, 2 * p.dz, N)), 0, Lz)
    elif layout == "onecell":
        x = (3 + rng.uniform(0.01, 0.99, N)) * p.dx
        y = (2 + rng.uniform(0.01, 0.99, N)) * p.dy
        z = (1 + rng.uniform(0.01, 0.99, N)) * p.dz
    else:
        raise ValueError(layout)
    if shuffle:
        o = rng.permutation(N)
        x, y, z = x[o], y[o], z[o]
    x, y, z = (np.asarray(a, np.float32) for a in (x, y, z))
    h = oracle.helpers(p, z.astype(np.float64), np.full(N, 280.0), np.full(N, 9e4), np.zeros(N))
    th_r, rho_r, qv_r = h[:, 0], h[:, 3], h[:, 4]
    f = lambda a: np.asarray(a, np.float32)
    s = dict(x=x, y=y, z=z,
             u=f(rng.normal(0, speed, N)), v=f(rng.normal(0, speed, N)), w=f(rng.normal(0, speed / 2, N)),
             th=f(th_r + rng.normal(0, .6, N)), qv=f(qv_r * rng.uniform(.85, 1.25, N)),
             qc=f(np.where(rng.uniform(size=N) < .3, rng.uniform(0, 2.5e-3, N), 0.0)),
             rho=f(rho_r * (1 + .03 * rng.normal(size=N))),
             ax=f(rng.normal(0, .05, N)), ay=f(rng.normal(0, .05, N)), az=f(rng.normal(0, .05, N)))
    return s


def as64(s):
    return {k: np.asarray(v, np.float64) for k, v in s.items()}
