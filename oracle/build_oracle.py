"""Build recipe for the oracle (test infrastructure only).

* liboracle.so  — the FP64 C restatement (asph_oracle.c), gcc + OpenMP.
* libadjhost.so — the FP64 host reference of the adjoint window
  (adjoint_host.cpp): forward loss and reverse-mode gradient, g++.
* _ref/asph_ref.cubin — the reference's device code compiled UNMODIFIED
  from the reference checkout with its own documented flags
  (asph_h100.cu:23-25: -O3 -use_fast_math -std=c++17), retargeted to
  sm_103a.  Built only where the reference checkout exists; the cubin is
  architecture-neutral for the host, so it travels to the GPU machine.
* refgpu — host program that loads that cubin and replays the reference
  step (refgpu.cu); compiled wherever nvcc and libcuda are available.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")


def reference_src() -> str:
    """Path of the reference's asph_h100.cu, from ASPH_REFERENCE_SRC; empty
    when it is unset (the recipes that need the checkout then skip)."""
    return os.environ.get("ASPH_REFERENCE_SRC", "")

LIBORACLE = os.path.join(BUILD, "liboracle.so")
LIBADJHOST = os.path.join(BUILD, "libadjhost.so")
CUBIN = os.path.join(REF_OUT, "asph_ref.cubin")
REFGPU = os.path.join(BUILD, "refgpu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "asph_oracle.c")
    hdr = os.path.join(os.path.dirname(HERE), "include", "asph.h")
    if force or _stale(LIBORACLE, [src, hdr]):
        _run(["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
              "-o", LIBORACLE, src, "-lm"])
    return LIBORACLE


def build_adjoint_host(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "adjoint_host.cpp")
    hdr = os.path.join(os.path.dirname(HERE), "include", "asph.h")
    if force or _stale(LIBADJHOST, [src, hdr]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", LIBADJHOST, src])
    return LIBADJHOST


def build_ref_cubin(force: bool = False) -> str:
    """Compile the reference's kernels into a cubin (needs the checkout)."""
    src = reference_src()
    if not src or not os.path.exists(src):
        return CUBIN if os.path.exists(CUBIN) else ""
    os.makedirs(REF_OUT, exist_ok=True)
    if force or _stale(CUBIN, [src]):
        _run([_nvcc(), "-cubin", "-O3", "-use_fast_math", "-std=c++17", *ARCH, "-o", CUBIN, src])
    return CUBIN


# The reference's run parameters are constexpr (asph_h100.cu:48-72).  To time
# its kernels on the 2,097,152-particle moist-bubble geometry (cells of
# 20 km/133 x 20 km/133 x 40 m, theta rising 4 K/km) they are compiled from a
# copy whose two constexpr lines carry those values; the copy lives in a
# temporary directory and only the cubin is kept.
BUBBLE2M_CUBIN = os.path.join(REF_OUT, "asph_ref_bubble2m.cubin")
_GEOMETRY_LINES = {
    "constexpr float DX = 1000.0f, DY = 1000.0f, DZ = 100.0f;":
        "constexpr float DX = 150.37594f, DY = 150.37594f, DZ = 40.0f;",
    "constexpr float N2   = 6.0e-5f;": "constexpr float N2   = 1.3075533e-4f;",
}


def build_ref_cubin_bubble2m(force: bool = False) -> str:
    src = reference_src()
    if not src or not os.path.exists(src):
        return BUBBLE2M_CUBIN if os.path.exists(BUBBLE2M_CUBIN) else ""
    os.makedirs(REF_OUT, exist_ok=True)
    if force or _stale(BUBBLE2M_CUBIN, [src]):
        import tempfile
        text = open(src).read()
        for old, new in _GEOMETRY_LINES.items():
            if old not in text:
                raise RuntimeError("reference constexpr line not found: " + old)
            text = text.replace(old, new)
        with tempfile.TemporaryDirectory() as td:
            src = os.path.join(td, "asph_bubble2m.cu")
            with open(src, "w") as f:
                f.write(text)
            _run([_nvcc(), "-cubin", "-O3", "-use_fast_math", "-std=c++17", *ARCH, "-o", BUBBLE2M_CUBIN, src])
    return BUBBLE2M_CUBIN


def build_refgpu(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "refgpu.cu")
    if force or _stale(REFGPU, [src]):
        stubs = "/usr/local/cuda/lib64/stubs"
        _run([_nvcc(), "-O2", "-std=c++17", *ARCH, "-o", REFGPU, src, "-lcuda", "-L", stubs])
    return REFGPU


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_adjoint_host(force)
    build_ref_cubin(force)
    build_ref_cubin_bubble2m(force)
    build_refgpu(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIBORACLE, CUBIN, REFGPU)
