"""Build recipe of the cpfem_gb300 shared library (sm_103a only).

Compiles the CUDA sources with nvcc and the host pattern builder with g++ in parallel,
then links ``libcpfem_gb300.so`` next to this file.  Run ``python build.py`` or call
``build()``.  Rebuilds only when a source is newer than the library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcpfem_gb300.so")

CUDA_SOURCES = ["assembly.cu", "krylov.cu", "adjoint.cu", "probe.cu"]
CXX_SOURCES = ["pattern.cpp"]
HEADERS = ["cpfem_common.cuh", "gp_update.cuh", "gp_adjoint.cuh", "reduce.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(home, "bin", "nvcc")
    return p if os.path.exists(p) else "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "cpfem_gb300.h")]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nvcc_path(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", INCLUDE, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-I", INCLUDE, "-c", s, "-o", o])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        logs.append(_run([nvcc_path(), *ARCH, "-shared", "-o", LIB, *objs]))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
