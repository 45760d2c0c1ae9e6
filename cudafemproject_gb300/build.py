"""In-tree build of the sm_103a library (nvcc, no cmake).

    python -m cudafemproject_gb300.build

Produces ``cudafemproject_gb300/_lib/libcfem_gb300.so`` (C-ABI of include/cfem.h)
and ``cudafemproject_gb300/_lib/cfem_run`` (command-line driver that mirrors
the reference's main.cpp with argv). Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libcfem_gb300.so")
EXE = os.path.join(OUT, "cfem_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off on host code: the float arithmetic that mirrors the
# reference (wavelets, load factors) must round alike on x86 and aarch64.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                  "-Xcompiler", "-ffp-contract=off",
                  "-I", os.path.join(REPO, "include")]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-I", os.path.join(REPO, "include")]

CU_SOURCES = ["context.cu", "context_dyn.cu", "context_multi.cu", "context_batch.cu"]
CXX_SOURCES = ["prep.cpp", "femfunc.cpp", "kfile.cpp"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cudafemproject_gb300")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    return hs + [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc] + NVFLAGS + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["g++"] + CXXFLAGS + ["-I", "/usr/local/cuda/include", "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if r.returncode != 0:
                    raise RuntimeError(f"compile failed: {' '.join(j)}\n{r.stdout}\n{r.stderr}")
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout, r.stderr, file=sys.stderr)
    if force or _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    main_src = os.path.join(CSRC, "cfem_main.cpp")
    if os.path.exists(main_src) and (force or _stale(EXE, [main_src, LIB] + hdrs)):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(REPO, "include"), main_src, "-o", EXE,
               "-L", OUT, "-lcfem_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
