"""In-tree build of the GB300 library, the emd_gb300 executable and nothing else.

    python -m examinimd_gb300.build          # or examinimd_gb300.build.build()

CUDA sources are compiled for sm_103a only.  Files holding FP64 drop-in
kernels are compiled with -fmad=false so no multiply-add pair is fused and
results round like the serial reference; mixed-precision files keep FMA.
Host C++ uses -ffp-contract=off for the same reason on every host
architecture.  Outputs: examinimd_gb300/libemd_gb300.so, examinimd_gb300/emd_gb300.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libemd_gb300.so")
EXE = os.path.join(HERE, "emd_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# kernels whose FP64 results must round exactly like the serial reference
FMAD_OFF = {"ctx", "integrate", "comm", "binning", "neighbor", "lj", "snap"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    out = []
    for d in (CSRC, HOST, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                out.append(os.path.join(d, f))
    return out


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    jobs = jobs or max(2, min(16, os.cpu_count() or 2))
    tasks = []
    objs = []
    for f in sorted(os.listdir(CSRC)):
        if not f.endswith(".cu"):
            continue
        stem = f[:-3]
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, stem + ".cu.o")
        objs.append(obj)
        flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                 "-diag-suppress", "177"]
        if stem in FMAD_OFF:
            flags.append("-fmad=false")
        if not _newer(obj, [src] + headers):
            tasks.append([nvcc] + ARCH + flags + ["-c", src, "-o", obj])
    host_objs = []
    for f in sorted(os.listdir(HOST)):
        if not f.endswith(".cpp"):
            continue
        src = os.path.join(HOST, f)
        obj = os.path.join(BUILD, f[:-4] + ".cpp.o")
        (host_objs if f != "main.cpp" else []).append(obj)
        if not _newer(obj, [src] + headers):
            tasks.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-result",
                          "-I", os.path.join(cuda, "include"), "-c", src, "-o", obj])
    if tasks:
        with ThreadPoolExecutor(jobs) as ex:
            for t in tasks:
                if verbose:
                    print(" ".join(t), flush=True)
            list(ex.map(_run, tasks))
    all_objs = objs + host_objs
    if not _newer(LIB, all_objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + all_objs + ["-lcudart"])
    main_obj = os.path.join(BUILD, "main.cpp.o")
    if not _newer(EXE, [main_obj, LIB]):
        _run(["g++", "-o", EXE, main_obj, "-L", HERE, "-lemd_gb300", "-Wl,-rpath,$ORIGIN",
              "-L", os.path.join(cuda, "lib64"), "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
