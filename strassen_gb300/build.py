"""Builds libbsgpu.so (all CUDA sources in csrc/) for sm_103a with nvcc.

Translation units compile in parallel; the library links into this package
directory (in-tree, git-ignored).  Host and device code are built without
floating-point contraction (-ffp-contract=off, -fmad=false): the FP64 form
spells out every fused multiply-add it performs, which is what makes it
bit-identical to the reference on the deterministic BLAS definition.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbsgpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def flags():
    return ["-O3", "-std=c++17", ARCH, "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp", "-I" + os.path.join(os.path.dirname(HERE), "include")]


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + flags() + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc(), ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", LIB] + objs + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


DRIVERS = os.path.join(HERE, "drivers")


def build_drivers(verbose=False):
    """The reference's three drivers rebuilt against the C++ facade
    (include/bsgpu.hpp), linked to the in-tree library."""
    out = os.path.join(DRIVERS, "bin")
    os.makedirs(out, exist_ok=True)
    inc = os.path.join(os.path.dirname(HERE), "include")
    gxx = shutil.which("g++") or "g++"
    built = []
    for src in sorted(glob.glob(os.path.join(DRIVERS, "*.cpp"))):
        exe = os.path.join(out, os.path.splitext(os.path.basename(src))[0])
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(src), os.path.getmtime(LIB),
                                                               os.path.getmtime(os.path.join(inc, "bsgpu.hpp"))):
            built.append(exe)
            continue
        cmd = [gxx, "-O2", "-std=c++17", "-I" + inc, src, "-o", exe, "-L" + HERE, "-lbsgpu",
               "-Wl,-rpath,$ORIGIN/../.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed for {src}:\n{r.stdout}\n{r.stderr}")
        built.append(exe)
    if verbose:
        print("built", built)
    return built


if __name__ == "__main__":
    build(verbose=True)
    build_drivers(verbose=True)
    sys.exit(0)
