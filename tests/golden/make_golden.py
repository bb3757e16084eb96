"""Generate the golden fixtures that pin the oracle to the reference.

The reference (asph_h100.cu) ships no tests or known-answer vectors, so the
fixtures are produced by running the reference's own code:

  python tests/golden/make_golden.py helpers
      Compiles tests/golden/ref_helpers_host.cu, which #includes the
      reference file itself, for the host, and tabulates its host-callable
      helpers (asph_h100.cu:136-171).  Needs the reference checkout
      (ASPH_REFERENCE_SRC = the path of its asph_h100.cu) and nvcc.
      Writes tests/golden/ref_helpers.npz.

  python tests/golden/make_golden.py gpu <outdir>
      On a GB300: runs the reference's kernels (oracle/_ref/asph_ref.cubin,
      built from the reference checkout by oracle/build_oracle.py) through
      oracle/refgpu on seeded synthetic states, one full reference step with
      every stage saved, plus the reference's own initial state.  Writes
      ref_stages_<case>.npz and ref_init.npz into outdir; they are then
      committed under tests/golden/.

  python tests/golden/make_golden.py dump <outdir>
      On a GB300: runs this library's command-line driver on the small
      reference-geometry case of tests/test_cli.py (DUMP_FIXTURE_ARGS) and
      copies its last dump to <outdir>/ours_cli_dump.bin, the fixture that
      the reference's own reader, tools/make_viz.py load(), is run on.

  python tests/golden/make_golden.py viz
      Runs the reference's own reader, tools/make_viz.py load() (next to
      ASPH_REFERENCE_SRC in the checkout), on tests/golden/ours_cli_dump.bin
      and saves what it returns as tests/golden/make_viz_ours.npz, so that
      machines without the checkout still compare our reader with it.

All inputs are seeded synthetic states in the reference geometry
(1000 m x 1000 m x 100 m cells, one particle per cell on average).
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

DX, DY, DZ = 1000.0, 1000.0, 100.0


def make_helpers() -> None:
    from oracle import build_oracle
    ref = build_oracle.reference_src()
    if not ref or not os.path.exists(ref):
        raise SystemExit("reference checkout not found (set ASPH_REFERENCE_SRC)")
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "refhelpers")
        out = os.path.join(td, "h.bin")
        subprocess.check_call(["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                               '-DREFSRC="%s"' % ref, "-o", exe, os.path.join(HERE, "ref_helpers_host.cu")])
        subprocess.check_call([exe, out])
        a = np.fromfile(out, np.float32).reshape(-1, 11)
    np.savez_compressed(os.path.join(HERE, "ref_helpers.npz"), z=a[:, 0], theta_ref=a[:, 1], exner_ref=a[:, 2],
                        pres_ref=a[:, 3], rho_ref=a[:, 4], qv_ref=a[:, 5], esat=a[:, 6], qsat=a[:, 7],
                        dqsdT=a[:, 8], T=a[:, 9], p=a[:, 10])
    print("wrote", os.path.join(HERE, "ref_helpers.npz"))


# ---------------------------------------------------------------------------
# synthetic reference-geometry states
# ---------------------------------------------------------------------------
def _profiles(z):
    """Reference sounding in double (asph_h100.cu:136-153) for building inputs."""
    g, cp, rd, th0, n2 = 9.80665, 1004.0, 287.05, 300.0, 6.0e-5
    th = th0 * np.exp(n2 * z / g)
    ex = 1.0 - g * g / (cp * th0 * n2) * (1.0 - np.exp(-n2 * z / g))
    p = 1e5 * ex ** (cp / rd)
    rho = p / (rd * th * ex)
    qv = 0.016 * np.exp(-z / 2500.0) * np.exp(-np.maximum(z - 5000.0, 0.0) / 1000.0)
    return th, ex, p, rho, qv


def make_state(case: str, seed: int) -> dict:
    rng = np.random.default_rng(seed)
    if case == "jitter":
        nx, ny, nz = 12, 12, 10
        N = nx * ny * nz
        i = np.arange(N)
        ix, iy, iz = i % nx, (i // nx) % ny, i // (nx * ny)
        x = (ix + 0.5 + rng.uniform(-0.3, 0.3, N)) * DX
        y = (iy + 0.5 + rng.uniform(-0.3, 0.3, N)) * DY
        z = (iz + 0.5 + rng.uniform(-0.3, 0.3, N)) * DZ
        order = rng.permutation(N)
        x, y, z = x[order], y[order], z[order]
    elif case == "cluster":
        nx, ny, nz = 10, 12, 8
        N = nx * ny * nz
        centres = rng.uniform([0.1, 0.1, 0.1], [0.9, 0.9, 0.9], size=(6, 3)) * [nx * DX, ny * DY, nz * DZ]
        k = rng.integers(0, 6, N)
        x = centres[k, 0] + rng.normal(0, 1.2 * DX, N)
        y = centres[k, 1] + rng.normal(0, 1.2 * DY, N)
        z = centres[k, 2] + rng.normal(0, 1.5 * DZ, N)
        x = np.mod(x, nx * DX)
        y = np.mod(y, ny * DY)
        z = np.clip(np.abs(z), 0.0, nz * DZ)
    else:
        raise ValueError(case)
    x = x.astype(np.float32); y = y.astype(np.float32); z = z.astype(np.float32)
    zd = z.astype(np.float64)
    th_r, ex, p, rho_r, qv_r = _profiles(zd)
    u = rng.normal(0, 6.0, N); v = rng.normal(0, 6.0, N); w = rng.normal(0, 2.5, N)
    # a few fast particles near the x/y seams so the drift wraps them
    edge = np.where(x < 0.3 * DX)[0][:6]
    u[edge] = -rng.uniform(40, 60, edge.size)
    th = th_r + rng.normal(0, 0.6, N)
    qv = qv_r * rng.uniform(0.85, 1.25, N)
    qc = np.where(rng.uniform(size=N) < 0.3, rng.uniform(0, 2.5e-3, N), 0.0)
    rho = rho_r * (1.0 + 0.03 * rng.normal(size=N))
    ax = rng.normal(0, 0.05, N); ay = rng.normal(0, 0.05, N); az = rng.normal(0, 0.05, N)
    C = nx * ny * nz
    rain = np.where(rng.uniform(size=C) < 0.2, rng.uniform(0, 5e4, C), 0.0)
    f32 = lambda a: np.asarray(a, np.float32)
    return dict(nx=nx, ny=ny, nz=nz, N=N, x=x, y=y, z=z, u=f32(u), v=f32(v), w=f32(w), th=f32(th), qv=f32(qv),
                qc=f32(qc), rho=f32(rho), ax=f32(ax), ay=f32(ay), az=f32(az), rain=f32(rain),
                precip=np.zeros(nx * ny, np.float32), simt=1234.5, dt=np.float32(0.5), do_sort=1, clamp=0)


def _write_input(path: str, s: dict) -> None:
    N = s["N"]
    z4 = np.zeros(N, np.float32)
    pos = np.stack([s["x"], s["y"], s["z"], z4], 1)
    vel = np.stack([s["u"], s["v"], s["w"], z4], 1)
    thq = np.stack([s["th"], s["qv"], s["qc"], z4], 1)
    acc = np.stack([s["ax"], s["ay"], s["az"], z4], 1)
    with open(path, "wb") as f:
        f.write(struct.pack("<8i", 0x41535048, s["nx"], s["ny"], s["nz"], N, s["do_sort"], s["clamp"], 0))
        f.write(struct.pack("<d", s["simt"]))
        f.write(struct.pack("<f", float(s["dt"])))
        for a in (pos, vel, thq, s["rho"], acc, s["rain"], s["precip"]):
            f.write(np.ascontiguousarray(a, np.float32).tobytes())


def _refgpu():
    from oracle import build_oracle
    build_oracle.build_refgpu()
    if not os.path.exists(build_oracle.CUBIN):
        raise RuntimeError("reference cubin missing: %s" % build_oracle.CUBIN)
    return build_oracle.REFGPU, build_oracle.CUBIN


def make_gpu(outdir: str) -> None:
    exe, cubin = _refgpu()
    os.makedirs(outdir, exist_ok=True)
    for case, seed in (("jitter", 11), ("cluster", 12)):
        s = make_state(case, seed)
        with tempfile.TemporaryDirectory() as td:
            inp = os.path.join(td, "in.bin")
            _write_input(inp, s)
            subprocess.check_call([exe, cubin, "stages", inp, td])
            N, C = s["N"], s["nx"] * s["ny"] * s["nz"]
            out = {}
            for name, dt, shape in (
                    ("keys_in", np.uint32, (N,)), ("keys_sorted", np.uint32, (N,)), ("perm", np.uint32, (N,)),
                    ("g_pos", np.float32, (N, 4)), ("g_vel", np.float32, (N, 4)), ("g_thq", np.float32, (N, 4)),
                    ("g_rho", np.float32, (N,)), ("cell_range", np.int32, (C, 2)), ("surf_count", np.int32, (1,)),
                    ("surf_list", np.int32, (2 * s["nx"] * s["ny"],)),
                    ("kd_pos", np.float32, (N, 4)), ("kd_vel", np.float32, (N, 4)), ("flux_thq", np.float32, (N, 4)),
                    ("d_rho", np.float32, (N,)), ("e_thq", np.float32, (N, 4)), ("e_prs", np.float32, (N,)),
                    ("e_rain", np.float32, (C,)), ("m_acc", np.float32, (N, 4)), ("m_dthdt", np.float32, (N,)),
                    ("i_thq", np.float32, (N, 4)), ("i_vel", np.float32, (N, 4)), ("r_rain", np.float32, (C,)),
                    ("r_precip", np.float32, (s["nx"] * s["ny"],)), ("gmax", np.float32, (3,)),
                    ("audit", np.float64, (6,))):
                out["out_" + name] = np.fromfile(os.path.join(td, name + ".bin"), dt).reshape(shape)
        cnt = int(out["out_surf_count"][0])
        out["out_surf_list"] = np.sort(out["out_surf_list"][:min(cnt, 2 * s["nx"] * s["ny"])])
        inputs = {"in_" + k: np.asarray(v) for k, v in s.items()}
        np.savez_compressed(os.path.join(outdir, "ref_stages_%s.npz" % case), **inputs, **out)
        print("wrote", case, N)
    # the reference's own initial state
    nx, ny, nz = 14, 12, 10
    with tempfile.TemporaryDirectory() as td:
        subprocess.check_call([exe, cubin, "init", str(nx), str(ny), str(nz), "0.1", td])
        N, C = nx * ny * nz, nx * ny * nz
        out = {"nx": nx, "ny": ny, "nz": nz, "noise": 0.1}
        for name, dt, shape in (("pos", np.float32, (N, 4)), ("vel", np.float32, (N, 4)),
                                ("thq", np.float32, (N, 4)), ("rho", np.float32, (N,)), ("prs", np.float32, (N,)),
                                ("acc", np.float32, (N, 4)), ("dthdt", np.float32, (N,)),
                                ("rain", np.float32, (C,)), ("cell_range", np.int32, (C, 2)),
                                ("perm", np.uint32, (N,))):
            out[name] = np.fromfile(os.path.join(td, name + ".bin"), dt).reshape(shape)
        np.savez_compressed(os.path.join(outdir, "ref_init.npz"), **out)
        print("wrote init", N)


# The command-line run whose last dump is the make_viz fixture: the
# reference physics on a 16^3 grid, 0.02 h, dumps every 30 s, strides 4.
DUMP_FIXTURE_ARGS = ["--nx", "16", "--ny", "16", "--nz", "16", "--dump-every", "30", "--sim-hours", "0.02",
                     "--dump-stride", "4", "4", "--report", "50"]


def make_dump(outdir: str) -> None:
    import shutil
    from sph_cuda_gb300 import _build
    cli = _build.build_cli()
    os.makedirs(outdir, exist_ok=True)
    with tempfile.TemporaryDirectory() as td:
        subprocess.check_call([cli, *DUMP_FIXTURE_ARGS, "--outdir", td], stdout=subprocess.DEVNULL)
        last = sorted(f for f in os.listdir(td) if f.startswith("asph_t"))[-1]
        shutil.copy(os.path.join(td, last), os.path.join(outdir, "ours_cli_dump.bin"))
    print("wrote", os.path.join(outdir, "ours_cli_dump.bin"), "from", last)


def load_make_viz():
    """tools/make_viz.py of the reference checkout (next to the file that
    ASPH_REFERENCE_SRC names), imported by path: its main() only runs as a
    script.  None when the checkout is not present."""
    import importlib.util
    from oracle import build_oracle
    ref = build_oracle.reference_src()
    path = os.path.join(os.path.dirname(ref), "tools", "make_viz.py") if ref else ""
    if not path or not os.path.exists(path):
        return None
    spec = importlib.util.spec_from_file_location("make_viz", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


VIZ_FIELDS = ("theta", "qv", "ql", "u", "v", "w")


def make_viz() -> None:
    mv = load_make_viz()
    if mv is None:
        raise SystemExit("reference checkout not found (set ASPH_REFERENCE_SRC)")
    v = mv.load(os.path.join(HERE, "ours_cli_dump.bin"))
    head = np.array([v["nx"], v["ny"], v["nz"], v["cx"], v["cy"], v["cz"]], np.int64)
    dims = np.array([v["t"], v["lx"], v["ly"], v["lz"]], np.float64)
    fields = {k: np.asarray(v["fields"][k], np.float32) for k in VIZ_FIELDS}
    np.savez_compressed(os.path.join(HERE, "make_viz_ours.npz"), head=head, dims=dims, **fields)
    print("wrote", os.path.join(HERE, "make_viz_ours.npz"))


if __name__ == "__main__":
    usage = "usage: make_golden.py helpers | viz | gpu <outdir> | dump <outdir>"
    cmd = sys.argv[1] if len(sys.argv) > 1 else "helpers"
    if cmd == "helpers":
        make_helpers()
    elif cmd == "viz":
        make_viz()
    elif cmd in ("gpu", "dump"):
        if len(sys.argv) < 3:
            raise SystemExit(usage)
        (make_gpu if cmd == "gpu" else make_dump)(sys.argv[2])
    else:
        raise SystemExit(usage)
