"""The C ABI library (CPU-side checks: no kernel launches).

* every function declared in include/*.h is exported by libemd_gb300.so;
* without a usable GPU, context creation fails with an error status
  instead of falling back to anything.
"""
import ctypes
import os
import re
import subprocess

import pytest

from tests.conftest import ROOT, gpu_available

HEADERS = [os.path.join(ROOT, "include", f) for f in ("emd_gpu.h", "emd_driver.h", "emd_batch.h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(emd_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib_path():
    from examinimd_gb300 import build
    return build.build()


def test_headers_declare_the_module_api():
    names = declared_functions()
    for required in ("emd_create", "emd_nve_initial", "emd_comm_exchange_halo", "emd_binning_create",
                     "emd_neigh_create", "emd_lj_compute", "emd_snap_compute", "emd_md_create", "emd_md_run"):
        assert required in names


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(lib_path)
    for n in declared_functions():
        getattr(lib, n)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_no_gpu_fails_loudly(lib_path):
    from examinimd_gb300 import Context, EmdError, MD
    with pytest.raises(EmdError):
        Context(0)
    with pytest.raises(EmdError, match="CUDA"):
        MD(["-il", "/nonexistent"])
