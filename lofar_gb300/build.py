"""Builds lofar_gb300/libwstack_gb300.so with nvcc for sm_103a (GB300).

Each translation unit in csrc/ is compiled in parallel, then linked into one
shared library against the CUDA runtime and cuFFT.  No cmake, no torch
extension machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwstack_gb300.so")

SOURCES = ["bin.cu", "grid.cu", "degrid.cu", "wcorrect.cu", "fft.cu", "fft64.cu", "capi.cu",
           "batch.cu", "noalloc.cu", "binms.cu", "driver.cu", "sector.cu"]
# the reference's executable (main.c) over the library: wstack_gb300_run PARAMFILE ...
RUNNER_SRC = "wstack_run.cpp"
RUNNER = os.path.join(HERE, "wstack_gb300_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwstack_gb300.so")
    return cand


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _flags() -> list[str]:
    return ["-O3", "-lineinfo", "-std=c++17", *ARCH, "-Xcompiler", "-fPIC,-O2,-fvisibility=hidden",
            f"-I{INCLUDE}", f"-I{CSRC}", "--expt-relaxed-constexpr"]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(INCLUDE, "wstack_gb300.h"))
    headers.append(os.path.join(INCLUDE, "wstack_gb300_io.h"))
    headers.append(os.path.abspath(__file__))
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([nvcc, *_flags(), "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        cuda_lib = os.path.join(_cuda_home(nvcc), "lib64")
        link = [nvcc, *ARCH, "-shared", "-cudart", "shared", *objs, "-o", LIB,
                f"-L{cuda_lib}", "-lcufft", "-Xlinker", f"-rpath={cuda_lib}"]
        run(link)
    runner_src = os.path.join(CSRC, RUNNER_SRC)
    if force or _stale(RUNNER, [runner_src, LIB, *headers]):
        run(["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", runner_src, "-o", RUNNER, f"-L{HERE}",
             "-lwstack_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
