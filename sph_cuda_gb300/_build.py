"""Build the CUDA library (libasph.so), the CLI driver and the oracle.

Everything is compiled in-tree with plain nvcc/gcc invocations, in
parallel, for sm_103a only.  No cmake, no torch extension machinery: the
library has a C ABI (include/asph.h) and is loaded with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sph_cuda_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libasph.so")
CLI = os.path.join(BUILD, "asph")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CU_SOURCES = ["asph_sort.cu", "asph_kernels.cu", "asph_pairs.cu", "asph_capi.cu", "asph_noalloc.cu",
              "asph_ensemble.cu", "asph_adjoint.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if os.environ.get("ASPH_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, extra: list[str] | None = None) -> str:
    """Compile csrc/*.cu into _build/libasph.so (sm_103a)."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "asph.h"))
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *(extra or []), "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


def build_cli(force: bool = False) -> str:
    """Compile the command-line driver (csrc/asph_cli.cpp) against libasph.so."""
    src = os.path.join(CSRC, "asph_cli.cpp")
    if not os.path.exists(src):
        return ""
    if force or _stale(CLI, [src, LIB, os.path.join(ROOT, "include", "asph.h")]):
        cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"),
              "-I", os.path.join(cuda, "include"), src, "-o", CLI,
              "-L", BUILD, "-lasph", "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN"])
    return CLI


def build_all(force: bool = False) -> None:
    build_library(force)
    build_cli(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
