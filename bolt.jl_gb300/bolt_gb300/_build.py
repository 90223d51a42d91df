"""Builds libbolt_gb300.so in-tree with nvcc for sm_103a.

The translation units compile in parallel; the result lands in
``bolt_gb300/_lib/``.  No CMake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # bolt.jl_gb300/
CSRC = os.path.join(ROOT, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libbolt_gb300.so")
OBJ_DIR = os.path.join(ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-diag-suppress", "177"]
CU_SOURCES = ["solver.cu", "los.cu", "capi.cu", "probe.cu", "noalloc.cu", "engine.cu", "moments.cu"]
CXX_SOURCES = ["host_cosmo.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, s) for s in CU_SOURCES + CXX_SOURCES] + [
        os.path.join(CSRC, "bolt_dev.cuh"), os.path.join(CSRC, "host_cosmo.hpp"), os.path.join(CSRC, "tuner.hpp"),
        os.path.join(CSRC, "chains.cuh"), os.path.join(CSRC, "tangent.cuh"), os.path.join(CSRC, "adjoint.cuh"),
        os.path.join(os.path.dirname(ROOT), "include", "bolt_gb300.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for s in CU_SOURCES:
        obj = os.path.join(OBJ_DIR, s.replace(".cu", ".o"))
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, s), "-o", obj])
    for s in CXX_SOURCES:
        obj = os.path.join(OBJ_DIR, s.replace(".cpp", ".o"))
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, s), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(OBJ_DIR, s.rsplit(".", 1)[0] + ".o") for s in CU_SOURCES + CXX_SOURCES]
    tmp = LIB + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
