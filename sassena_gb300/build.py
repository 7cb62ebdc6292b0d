"""Build recipe for the sassena_gb300 native libraries (nvcc, sm_103a, in-tree).

Outputs (git-ignored, rebuilt on every machine):
  sassena_gb300/_lib/libsassena_gb300.so   CUDA kernels + C ABI (include/sassena_gb300.h)
  sassena_gb300/_lib/libsassena_host.so    C++ host devices (XML, database, DCD, writer)
  sassena_gb300/_lib/sassena-gpu            driver executable (scatter.xml -> signal.h5)

Translation units compile in parallel; only stale objects are rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")
INCLUDE = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without FP contraction (the reference's x86-64 build has no fused multiply-add,
# and the Arm compiler would contract by default)
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I" + INCLUDE, "-Xptxas", "-warn-spills"]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", "-I" + INCLUDE, "-I" + HOST]

CUDA_SOURCES = [
    "capi.cu", "engine.cu", "phase_sum.cu", "phase_rec.cu", "correlate.cu", "peaks.cu", "noalloc.cu", "mlp.cu",
    "cv.cu", "multipole.cu", "align.cu", "corr_long.cu",
]
HOST_SOURCES = []  # filled when the host layer exists (see host_sources())

LIB = os.path.join(OUT, "libsassena_gb300.so")
HOST_LIB = os.path.join(OUT, "libsassena_host.so")
DRIVER = os.path.join(OUT, "sassena-gpu")


def host_sources():
    if not os.path.isdir(HOST):
        return []
    return sorted(f for f in os.listdir(HOST) if f.endswith(".cpp") and f != "sassena_gpu.cpp")


def _deps(src):
    d = os.path.dirname(src)
    return [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh", ".hpp"))] + [
        os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _compile_cu(name, verbose):
    src = os.path.join(CSRC, name)
    obj = os.path.join(OBJ, name + ".o")
    if _stale(obj, [src] + _deps(src)):
        flags = NVCC_FLAGS + (["-Xptxas", "-v"] if verbose else [])
        log = _run([NVCC] + flags + ["-c", src, "-o", obj])
        return obj, log
    return obj, ""


def _compile_cpp(name):
    src = os.path.join(HOST, name)
    obj = os.path.join(OBJ, "host_" + name + ".o")
    if _stale(obj, [src] + _deps(src)):
        _run([CXX] + CXX_FLAGS + ["-c", src, "-o", obj])
    return obj


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    jobs = jobs or min(8, os.cpu_count() or 4)
    logs = []
    with cf.ThreadPoolExecutor(jobs) as ex:
        cu = list(ex.map(lambda n: _compile_cu(n, verbose), CUDA_SOURCES))
        hs = list(ex.map(_compile_cpp, host_sources()))
    objs = [o for o, _ in cu]
    logs = [l for _, l in cu if l]
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    if hs:
        if _stale(HOST_LIB, hs + [LIB]):
            _run([CXX, "-shared", "-o", HOST_LIB] + hs + ["-L" + OUT, "-lsassena_gb300",
                                                         "-Wl,-rpath,$ORIGIN", "-pthread"])
        drv_src = os.path.join(HOST, "sassena_gpu.cpp")
        if os.path.exists(drv_src) and _stale(DRIVER, [drv_src, HOST_LIB, LIB] + _deps(drv_src)):
            _run([CXX] + CXX_FLAGS + [drv_src, "-o", DRIVER, "-L" + OUT, "-lsassena_host",
                                      "-lsassena_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"])
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
