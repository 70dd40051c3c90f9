"""Builds the native library ffip_gb300/_lib/libffip_gb300.so in-tree:
CUDA sources with nvcc for sm_103a, host C++ with g++, linked by nvcc.
Translation units compile in parallel."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libffip_gb300.so")
CLI = os.path.join(LIBDIR, "run_sim_json")

CUDA_SOURCES = ["kernels.cu", "adjoint.cu", "surrogate.cu", "raster.cu"]
# raster.cu rounds its double arithmetic like the host's media code (no
# contraction into fused multiply-adds), so that both give the same tables
CUDA_FLAGS = {"raster.cu": ["-fmad=false"]}
CXX_SOURCES = ["plan.cpp", "engine.cpp", "capi.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _deps_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def build(force: bool = False, verbose: bool = False, defines=(), libdir: str | None = None) -> str:
    """Builds the library (and the run_sim_json driver beside it).  defines /
    libdir: a tuning build with extra -D macros for the CUDA sources (the
    FFIP_FUSED_* switches of fused.cuh), placed in its own directory."""
    lib = LIB if libdir is None else os.path.join(libdir, "libffip_gb300.so")
    cli = CLI if libdir is None else os.path.join(libdir, "run_sim_json")
    bdir = BUILD if libdir is None else os.path.join(libdir, "_build")
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _deps_mtime():
        return lib
    os.makedirs(bdir, exist_ok=True)
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    dflags = ["-D" + d for d in defines]
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        o = os.path.join(bdir, s + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-Xptxas", "-warn-spills", *CUDA_FLAGS.get(s, []), *dflags, *inc, "-c", os.path.join(CSRC, s), "-o", o])
    for s in CXX_SOURCES:
        o = os.path.join(bdir, s + ".o")
        objs.append(o)
        jobs.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function", *dflags, *inc,
                     "-I", "/usr/local/cuda/include", "-c", os.path.join(CSRC, s), "-o", o])
    cli_obj = os.path.join(bdir, "run_sim_json.cpp.o")
    jobs.append(["g++", "-O2", "-std=c++17", "-Wall", *inc, "-c", os.path.join(CSRC, "run_sim_json.cpp"), "-o", cli_obj])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append((j, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n\n".join(" ".join(j) + "\n" + out for j, out in failed)
        raise RuntimeError("native build failed:\n" + msg)
    tmp = lib + ".tmp%d" % os.getpid()
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("native link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, lib)
    # the run_sim_json command-line driver, next to the library it loads
    r = subprocess.run(["g++", "-o", cli, cli_obj, "-L", os.path.dirname(lib), "-lffip_gb300", "-Wl,-rpath,$ORIGIN"],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("run_sim_json link failed:\n" + r.stdout.decode(errors="replace"))
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
