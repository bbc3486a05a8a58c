"""Builds the oracle -- TEST INFRASTRUCTURE ONLY.

* oracle/_build/liboracle.so: the C++ restatement (emd_oracle.cpp), built
  with -ffp-contract=off and OpenMP on any host (x86-64 or aarch64).
* oracle/_ref/ref_examinimd and ref_probe: ExaMiniMD's own sources compiled
  against the serial Kokkos shim (oracle/Makefile.ref), only where the
  ExaMiniMD source tree is present (it is not on the GPU machines).

The ExaMiniMD tree is taken from the EXAMINIMD_SRC environment variable;
without it this recipe looks in the one place the tree is mounted read-only
on the machine that generates the golden fixtures.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SRC_ENV = "EXAMINIMD_SRC"
_MOUNTED_REF_SRC = "/root/reference"


def reference_source() -> str:
    """The ExaMiniMD source tree this recipe compiles."""
    return os.environ.get(REF_SRC_ENV) or _MOUNTED_REF_SRC


def build_oracle() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "emd_oracle.cpp")
    hdr = os.path.join(HERE, "emd_oracle.h")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
           "-o", LIB, src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def build_reference(ref_src: str | None = None) -> str | None:
    """Compiles ExaMiniMD's sources against the shim when they are present."""
    ref_src = ref_src or reference_source()
    if not os.path.isdir(os.path.join(ref_src, "src")):
        return None
    cmd = ["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), f"REF={ref_src}", f"-j{os.cpu_count() or 4}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    return os.path.join(REF_DIR, "ref_examinimd")


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference())
