"""Builds libgpusteer.so (the sm_103a kernels and the C ABI) in-tree.

nvcc compiles each translation unit for sm_103a only, in parallel, and links
a shared library into gpusteer_gb300/_build/.  -fmad=false keeps every
binary32 expression unfused (the arithmetic contract of the oracle and the
reference sources); division and square root stay IEEE (no fast math).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libgpusteer.so"
SOURCES = ["gs_kernels.cu", "gs_step.cu", "gs_capi.cu", "gs_noalloc.cu", "gs_adjoint.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "gpusteer.h"]
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    relinked = False
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "--cudart", "static", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        relinked = True
    build_headless(force or relinked, verbose)
    return LIB


HEADLESS_SRC = PKG / "plugins" / "headless.cpp"
HEADLESS = BUILD / "gs_headless"


def build_headless(force: bool = False, verbose: bool = False) -> Path:
    """The headless plugin driver: C++ plugins on include/GroupSteerLibrary.h,
    linked against libgpusteer.so (found next to it at run time)."""
    inc = PKG.parent / "include"
    deps = [HEADLESS_SRC, LIB, inc / "GroupSteerLibrary.h", inc / "PlugIn.h", inc / "gpusteer.h",
            inc / "SimulationParams.h"]
    if not force and not _stale(HEADLESS, deps):
        return HEADLESS
    cuda = Path(nvcc()).resolve().parent.parent
    # The plugins make their own CUDA runtime calls (cudaMemset on the device
    # arrays), as the reference's do: the static runtime needs no library path.
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-ffp-contract=off",
           "-I", str(inc), "-I", str(cuda / "include"), str(HEADLESS_SRC), "-o", str(HEADLESS),
           "-L", str(BUILD), "-lgpusteer", "-Wl,-rpath,$ORIGIN", "-L", str(cuda / "lib64"),
           "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("headless driver build failed")
    return HEADLESS


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
