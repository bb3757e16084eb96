"""Pin the CPU oracle to the reference.

The reference ships no tests or vectors; the fixtures under tests/golden
were produced by running the reference's own code (tests/golden/
make_golden.py): its host helpers compiled from asph_h100.cu, and its
kernels run on a GB300 through oracle/refgpu.  These tests run on the CPU.
"""
import numpy as np
import pytest

from oracle import oracle
from sph_cuda_gb300 import preset
from conftest import golden, normwise

TOL = 1e-5          # normwise single-step tolerance


def test_helpers_match_reference_host_code():
    g = golden("ref_helpers.npz")
    p = preset("reference", 8, 8, 8)
    q = np.linspace(0, 2.2, g["z"].size)
    h = oracle.helpers(p, g["z"], g["T"], g["p"], q)
    for k, name in enumerate(["theta_ref", "exner_ref", "pres_ref", "rho_ref", "qv_ref", "esat", "qsat", "dqsdT"]):
        ref = g[name].astype(np.float64)
        rel = np.max(np.abs(h[:, k] - ref) / np.maximum(np.abs(ref), 1e-30))
        assert rel < 3e-6, (name, rel)


def test_spline_kernel_properties():
    p = preset("reference", 8, 8, 8)
    q = np.linspace(0, 2.5, 2001)
    h = oracle.helpers(p, np.zeros_like(q), np.full_like(q, 280.0), np.full_like(q, 9e4), q)
    w, dw = h[:, 8], h[:, 9]
    assert w[0] == pytest.approx(1 / np.pi) and np.all(w[q >= 2] == 0) and np.all(dw[q >= 2] == 0)
    # normalisation: 4 pi int_0^2 q^2 W dq = 1 (sigma = 1/pi, asph_h100.cu:56)
    m = q <= 2
    assert 4 * np.pi * np.trapezoid(q[m] ** 2 * w[m], q[m]) == pytest.approx(1.0, rel=1e-5)
    assert np.max(np.abs(np.gradient(w, q)[5:-5] - dw[5:-5])[q[5:-5] < 1.99]) < 2e-3


def _np_keys(p, x, y, z):
    def cell(a, d, n):
        s = np.float32(a) * np.float32(np.float32(1.0) / np.float32(d))
        return np.clip(s.astype(np.int64), 0, n - 1).astype(np.uint32)

    def spread(v):
        v = v & 0x3FF
        v = (v ^ (v << 16)) & 0xFF0000FF
        v = (v ^ (v << 8)) & 0x0300F00F
        v = (v ^ (v << 4)) & 0x030C30C3
        v = (v ^ (v << 2)) & 0x09249249
        return v

    ix, iy, iz = cell(x, p.dx, p.nx), cell(y, p.dy, p.ny), cell(z, p.dz, p.nz)
    return (spread(ix) | (spread(iy) << 1) | (spread(iz) << 2)).astype(np.uint32)


def test_keys_sort_table_properties():
    p = preset("small65k")
    rng = np.random.default_rng(3)
    N = p.n_particles
    x = rng.uniform(0, p.nx * p.dx, N).astype(np.float32)
    y = rng.uniform(0, p.ny * p.dy, N).astype(np.float32)
    z = rng.uniform(0, p.nz * p.dz, N).astype(np.float32)
    x[:5] = [0.0, np.nextafter(np.float32(p.nx * p.dx), 0, dtype=np.float32), p.dx, p.dx * 3 - 1e-3, 1e-30]
    z[:3] = [p.nz * p.dz, 0.0, p.dz]
    k = oracle.keys(p, x, y, z)
    assert np.array_equal(k, _np_keys(p, x, y, z))
    perm, srt = oracle.stable_sort(k, oracle.key_bits(p))
    assert np.array_equal(perm, np.argsort(k, kind="stable"))
    assert np.array_equal(srt, k[perm])
    rng_tab = oracle.cell_table(p, x[perm], y[perm], z[perm])
    cnt = rng_tab[:, 1] - rng_tab[:, 0]
    assert cnt.sum() == N and np.all(cnt >= 0)
    empty = cnt == 0
    assert np.all(rng_tab[empty] == 0)


def test_density_eos_conserves_water_and_theta_l():
    p = preset("reference", 10, 10, 10)
    rng = np.random.default_rng(5)
    N = p.n_particles
    i = np.arange(N)
    s = {"x": ((i % 10) + 0.5 + rng.uniform(-.3, .3, N)) * 1000.0,
         "y": (((i // 10) % 10) + 0.5 + rng.uniform(-.3, .3, N)) * 1000.0,
         "z": ((i // 100) + 0.5 + rng.uniform(-.3, .3, N)) * 100.0}
    s = {k: v.astype(np.float32) for k, v in s.items()}
    h = oracle.helpers(p, s["z"], np.full(N, 280.0), np.full(N, 9e4), np.zeros(N))
    s["th"] = h[:, 0] + rng.normal(0, .5, N)
    s["qv"] = h[:, 4] * rng.uniform(0.9, 1.4, N)
    s["qc"] = np.where(rng.uniform(size=N) < .3, rng.uniform(0, 3e-3, N), 0.0)
    sb = oracle.sort_build(p, s)
    g = sb["gathered"]
    out = oracle.density_eos(p, g, h[:, 3][sb["perm"]], sb["cell_range"], 0.5)
    pm = oracle.derived(p)["pmass"]
    w0 = np.sum(g["qv"] + g["qc"]) * pm
    w1 = np.sum(out["qv"] + out["qc"]) * pm + out["rain_dep"].sum()
    assert abs(w1 - w0) / w0 < 1e-12
    assert np.any(out["rain_dep"] > 0)


def test_rain_mass_balance():
    p = preset("reference", 6, 5, 9)
    rng = np.random.default_rng(1)
    r = rng.uniform(0, 1e5, p.nx * p.ny * p.nz)
    out, pr = oracle.rain(p, r, 0.5)
    assert out.sum() + pr.sum() * p.dx * p.dy == pytest.approx(r.sum(), rel=1e-13)


def test_cfl_control_paths():
    p = preset("reference", 16, 16, 8)
    d = oracle.derived(p)
    ok = oracle.cfl(p, [5.0, 5.0, 1.0], d["dt_cap"], 0)
    assert not ok["clamp"] and not ok["abort"] and ok["dt"] <= d["dt_cap"]
    trip = oracle.cfl(p, [1e4, 1e4, 1e4], d["dt_cap"], 0)
    assert trip["clamp"] and trip["trips"] == 1 and trip["dt"] >= d["dt_floor"]
    ab = oracle.cfl(p, [1e4, 1e4, 1e4], d["dt_cap"], p.max_trip)
    assert ab["abort"] and ab["status"] == 3


# ---------------------------------------------------------------------------
# oracle vs the reference's kernels (fixtures made on a GB300)
# ---------------------------------------------------------------------------
def _ref_state(g, pre):
    N = int(g["in_N"])
    if pre == "in":
        return {k: g["in_" + k].astype(np.float64) for k in
                ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "ax", "ay", "az")}
    raise ValueError(pre)


@pytest.mark.parametrize("case", ["jitter", "cluster"])
def test_oracle_matches_reference_stages(case):
    g = golden("ref_stages_%s.npz" % case)
    nx, ny, nz = int(g["in_nx"]), int(g["in_ny"]), int(g["in_nz"])
    p = preset("reference", nx, ny, nz)
    dt, simt = float(g["in_dt"]), float(g["in_simt"])
    s = _ref_state(g, "in")
    # sort block: bit exact
    sb = oracle.sort_build(p, s)
    assert np.array_equal(sb["keys_in"], g["out_keys_in"])
    assert np.array_equal(sb["perm"], g["out_perm"])
    assert np.array_equal(sb["keys_sorted"], g["out_keys_sorted"])
    assert np.array_equal(sb["cell_range"], g["out_cell_range"])
    assert np.array_equal(np.nonzero(sb["surf"])[0], g["out_surf_list"])
    gp = sb["gathered"]
    assert np.array_equal(gp["x"].astype(np.float32), g["out_g_pos"][:, 0])
    # kick + drift + flux; the reference kicks with acc in its pre-sort
    # order (kernel_gather does not permute acc, asph_h100.cu:245-256)
    st = dict(gp, ax=s["ax"], ay=s["ay"], az=s["az"])
    kd = oracle.kick_drift_flux(p, st, simt, dt, sb["surf"])
    assert normwise(kd["x"], g["out_kd_pos"][:, 0]) < 1e-6
    assert normwise(kd["z"], g["out_kd_pos"][:, 2]) < 1e-6
    assert normwise(kd["w"], g["out_kd_vel"][:, 2]) < 1e-6
    assert normwise(kd["th"], g["out_flux_thq"][:, 0]) < 1e-6
    assert normwise(kd["qv"], g["out_flux_thq"][:, 1]) < 1e-6
    # density + EOS + micro, from the reference's own post-drift state
    pos = g["out_kd_pos"].astype(np.float64)
    thq = g["out_flux_thq"].astype(np.float64)
    sd = {"x": pos[:, 0], "y": pos[:, 1], "z": pos[:, 2], "th": thq[:, 0], "qv": thq[:, 1], "qc": thq[:, 2]}
    de = oracle.density_eos(p, sd, g["out_g_rho"], g["out_cell_range"], dt)
    assert normwise(de["rho"], g["out_d_rho"]) < 1e-6
    # p' = c_s^2 (rho - rho_ref) amplifies the reference's FP32 rounding of
    # rho by rho/|rho - rho_ref| (~30 here): its own p' carries ~3e-5
    # normwise error against FP64, so p' pins the oracle only to 1e-4;
    # rho, from which p' follows, pins it to 1e-6 above.
    assert normwise(de["prs"], g["out_e_prs"]) < 1e-4
    for k, c in (("th", 0), ("qv", 1)):
        assert normwise(de[k], g["out_e_thq"][:, c]) < TOL, k
    # cloud water after saturation adjustment is qv_total - qsat(T, p): the
    # same cancellation, under the reference's fast-math esat
    assert normwise(de["qc"], g["out_e_thq"][:, 2]) < 1e-4
    assert normwise(g["in_rain"] + de["rain_dep"], g["out_e_rain"]) < 1e-4
    # momentum + theta update + kick + sponge
    vel = g["out_kd_vel"].astype(np.float64)
    eth = g["out_e_thq"].astype(np.float64)
    sm = {"x": pos[:, 0], "y": pos[:, 1], "z": pos[:, 2], "u": vel[:, 0], "v": vel[:, 1], "w": vel[:, 2],
          "th": eth[:, 0], "qv": eth[:, 1], "qc": eth[:, 2], "rho": g["out_d_rho"], "prs": g["out_e_prs"]}
    mo = oracle.momentum(p, sm, g["out_cell_range"], dt, integrate=True)
    for k, c in (("ax", 0), ("ay", 1), ("az", 2)):
        assert normwise(mo[k], g["out_m_acc"][:, c]) < TOL, k
    assert normwise(mo["dthdt"], g["out_m_dthdt"]) < TOL
    assert normwise(mo["th"], g["out_i_thq"][:, 0]) < TOL
    for k, c in (("u", 0), ("v", 1), ("w", 2)):
        assert normwise(mo[k], g["out_i_vel"][:, c]) < TOL, k
    # rain
    rr, pr = oracle.rain(p, g["out_e_rain"], dt)
    assert normwise(rr, g["out_r_rain"]) < 1e-6
    assert normwise(pr, g["out_r_precip"]) < 1e-6
    assert np.array_equal(np.abs(g["out_i_vel"][:, :3]).max(0), g["out_gmax"])
    # audit of the end-of-step state
    iv = g["out_i_vel"].astype(np.float64)
    it = g["out_i_thq"].astype(np.float64)
    au = oracle.audit(p, {"z": pos[:, 2], "u": iv[:, 0], "v": iv[:, 1], "w": iv[:, 2], "th": it[:, 0],
                          "qv": it[:, 1], "qc": it[:, 2]})
    for k in (1, 2, 3):
        assert abs(au[k] / g["out_audit"][k] - 1) < 1e-6, k
    # the reference adds PMASS once per thread of its 1024 x 256 audit grid
    # (asph_h100.cu:667), so its "mass" is 262144 PMASS whatever N is; the
    # oracle and the CUDA path report N PMASS
    assert abs(g["out_audit"][5] / (262144 * au[5] / p.n_particles) - 1) < 1e-6
    assert abs(au[0] - g["out_audit"][0]) <= 1e-5 * abs(g["out_audit"][0])


def test_oracle_matches_reference_init():
    g = golden("ref_init.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    p = preset("reference", nx, ny, nz, noise=float(g["noise"]))
    ini = oracle.init_reference(p)
    s = {k: ini[k] for k in ("x", "y", "z", "th", "qv", "rho")}
    N = p.n_particles
    for k in ("u", "v", "w", "qc", "ax", "ay", "az"):
        s[k] = np.zeros(N)
    sb = oracle.sort_build(p, s)
    gp = sb["gathered"]
    assert np.array_equal(sb["perm"], g["perm"])
    assert np.array_equal(sb["cell_range"], g["cell_range"])
    assert np.array_equal(gp["x"].astype(np.float32), g["pos"][:, 0])
    assert np.array_equal(gp["z"].astype(np.float32), g["pos"][:, 2])
    dt = oracle.derived(p)["dt_cap"]
    de = oracle.density_eos(p, gp, gp["rho"], sb["cell_range"], dt)
    assert normwise(de["rho"], g["rho"]) < TOL
    assert normwise(de["th"], g["thq"][:, 0]) < TOL
    assert normwise(de["qv"], g["thq"][:, 1]) < TOL
    sm = dict(gp, th=de["th"], qv=de["qv"], qc=de["qc"], rho=de["rho"], prs=de["prs"])
    mo = oracle.momentum(p, sm, sb["cell_range"], dt, integrate=False)
    # On the hydrostatic cell-centre lattice the acceleration is a small
    # residual of cancelling pressure-gradient terms; the reference's FP32
    # (fast-math) evaluation of it carries ~3e-4 normwise error, so the
    # pinning bound here is looser than the 1e-5 single-step gate.
    assert normwise(mo["az"], g["acc"][:, 2]) < 1e-3
