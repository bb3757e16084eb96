"""Time the reference's own kernels on the GPU (test infrastructure only).

  python oracle/time_reference.py native   [steps]            reference geometry 128^3, its own init
  python oracle/time_reference.py bubble2m [steps] [warmup]   the 2,097,152-particle moist-bubble state

`native` runs the unmodified reference cubin with the reference's own init
and step loop, a sort every step.  `bubble2m` runs the reference's kernels
compiled with the moist-bubble cell sizes (oracle/build_oracle.py) on the
moist-bubble initial state restated by the oracle (jittered 128^3 lattice,
three bubbles, initial sort and forces), a sort every step, starting at
dt = 0.2 s (the reference's static CFL bound for 40 m cells) under the
reference's closed-loop dt control: `warmup` untimed steps, then `steps`
timed ones.  Prints the refgpu JSON line.
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build_oracle, oracle  # noqa: E402


def write_state(path: str, p, s: dict, dt: float, simt: float = 0.0) -> None:
    N = p.n_particles
    z4 = np.zeros(N, np.float32)
    f = lambda k: np.asarray(s[k], np.float32)
    pos = np.stack([f("x"), f("y"), f("z"), z4], 1)
    vel = np.stack([f("u"), f("v"), f("w"), z4], 1)
    thq = np.stack([f("th"), f("qv"), f("qc"), z4], 1)
    acc = np.stack([f("ax"), f("ay"), f("az"), z4], 1)
    C = p.nx * p.ny * p.nz
    with open(path, "wb") as fh:
        fh.write(struct.pack("<8i", 0x41535048, p.nx, p.ny, p.nz, N, 1, 0, 0))
        fh.write(struct.pack("<d", simt))
        fh.write(struct.pack("<f", dt))
        for a in (pos, vel, thq, f("rho"), acc, np.zeros(C, np.float32), np.zeros(p.nx * p.ny, np.float32)):
            fh.write(np.ascontiguousarray(a, np.float32).tobytes())


def main() -> int:
    mode = sys.argv[1] if len(sys.argv) > 1 else "bubble2m"
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 50
    warmup = int(sys.argv[3]) if len(sys.argv) > 3 else 3
    exe = build_oracle.build_refgpu()
    if mode == "native":
        return subprocess.call([exe, build_oracle.CUBIN, "run", "128", "128", "128", str(steps), "0.25", "1"])
    from oracle import params
    p = params.preset("bubble2m")
    s = oracle.initial_state(p)
    dt = float(np.float32(oracle.derived(p)["dt_cap"]))
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "state.bin")
        write_state(path, p, s, dt)
        return subprocess.call([exe, build_oracle.BUBBLE2M_CUBIN, "runstate", path, str(steps), str(warmup),
                                repr(float(p.dx)), repr(float(p.dy)), repr(float(p.dz))])


if __name__ == "__main__":
    sys.exit(main())
