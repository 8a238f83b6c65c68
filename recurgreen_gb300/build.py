"""Builds librecurgreen_gb300.so (the C ABI of include/recurgreen.h) in-tree,
and the host programs bin/recurgreen and bin/plothisto on top of it.

nvcc compiles every CUDA translation unit for sm_103a only (one -gencode), in
parallel, then links a shared library with the CUDA runtime linked
statically, so the library has no run-time dependency beyond the driver.
The host programs are plain C++17 (g++), linked against the library with an
rpath to it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librecurgreen_gb300.so")
HOST = os.path.join(PKG, "host")
BIN = os.path.join(PKG, "bin")
HOST_SOURCES = ["driver.cpp"]
PROGRAMS = {"recurgreen": "recurgreen_main.cpp", "plothisto": "plothisto_main.cpp",
            "waveguide_test": "waveguide_test_main.cpp"}
SOURCES = ["rg_sweep.cu", "rg_sweep_sym.cu", "rg_sweep_large.cu", "rg_sweep_large_sym.cu", "rg_adjoint.cu",
           "rg_waveguide.cpp", "rg_noalloc.cu", "rg_green.cu", "rg_green.cpp", "rg_probe.cu", "rg_ozaki.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, "rg_internal.h"), os.path.join(CSRC, "rg_device.cuh"),
               os.path.join(CSRC, "rg_ozaki.cuh"),
               os.path.join(ROOT, "include", "recurgreen.h")]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc()] + ARCH + FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0 or verbose or ptxas_info:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart=static", "-o", LIB] + objs
        run(cmd)
    build_programs(force, run)
    return LIB


def cxx() -> str:
    cand = shutil.which("g++") or shutil.which("c++")
    if not cand:
        raise RuntimeError("g++ not found")
    return cand


def build_programs(force: bool, run) -> None:
    """bin/recurgreen, bin/plothisto and bin/waveguide_test (host C++ over
    include/recurgreen.hpp)."""
    os.makedirs(BIN, exist_ok=True)
    hdrs = [os.path.join(ROOT, "include", "recurgreen.h"), os.path.join(ROOT, "include", "recurgreen.hpp"),
            os.path.join(HOST, "driver.hpp")]
    flags = ["-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include")]
    objs = []
    for src in HOST_SOURCES:
        s, o = os.path.join(HOST, src), os.path.join(OBJ, "host_" + src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            run([cxx()] + flags + ["-c", s, "-o", o])
    for prog, src in PROGRAMS.items():
        s, exe = os.path.join(HOST, src), os.path.join(BIN, prog)
        if force or _stale(exe, [s, LIB] + objs + hdrs):
            run([cxx()] + flags + [s] + objs + ["-o", exe, "-L", PKG, "-lrecurgreen_gb300",
                                                "-Wl,-rpath,$ORIGIN/.."])


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
