"""Builds the native library libemoo.so in-tree (nvcc for sm_103a, g++ for host code).

Each CUDA translation unit is compiled separately, in parallel, with the flags it
needs: the FP64 parity kernels and the sampler with --fmad=false (every multiply
and add separately rounded, as in the reference's x86-64 build), the mixed-precision
kernels with contraction allowed.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libemoo.so")
DRIVER = os.path.join(HERE, "emoopic_gpu")  # the reference-style driver (emoopic_main.cpp)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]

# (source, extra nvcc flags)
CUDA_UNITS = [
    ("fields_f64.cu", ["--fmad=false"]),
    ("multigrid.cu", []),
    ("particles_f64.cu", ["--fmad=false"]),
    ("loader.cu", ["--fmad=false"]),
    ("sort.cu", []),
    ("particles_mixed.cu", ["--fmad=true"]),
    ("adjoint_f64.cu", ["--fmad=false"]),
    ("adjoint_mixed.cu", []),
]
HOST_UNITS = ["api.cpp", "loader_host.cpp", "input_parser.cpp", "io.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "emoo.h"))
    jobs = []
    objs = []
    for src, extra in CUDA_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s, __file__] + headers):
            flags = list(extra)
            if ptxas_info:
                flags += ["-Xptxas", "-v"]
            jobs.append([nvcc, "-c", s, "-o", o] + ARCH + NVCC_COMMON + flags)
    for src in HOST_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s, __file__] + headers):
            jobs.append(["g++", "-c", s, "-o", o, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         "-Wall", "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(_cuda_home(nvcc), "include")])
    outs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
    if jobs or not os.path.exists(LIB):
        link = [nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
        outs.append(_run(link))
    drv_src = os.path.join(CSRC, "emoopic_main.cpp")
    if _stale(DRIVER, [drv_src, LIB, os.path.join(INCLUDE, "emoopic.hpp"), os.path.join(INCLUDE, "emoo.h")]):
        outs.append(_run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, drv_src, "-o", DRIVER, "-L" + HERE,
                          "-lemoo", "-Wl,-rpath,$ORIGIN"]))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
