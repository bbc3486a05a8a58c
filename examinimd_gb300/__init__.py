"""GB300 (sm_103a) implementation of ExaMiniMD's per-timestep hot path.

The compute lives in ``libemd_gb300.so`` (CUDA kernels behind the C ABI in
``include/emd_gpu.h``) and the ExaMiniMD driver re-hosted on those kernels
(``include/emd_driver.h``).  This package only loads that library through
ctypes; there is no Python or CPU fallback for any kernel.
"""
from __future__ import annotations

from ._lib import (EMD_ERR_ARG, EMD_ERR_BOUNDS, EMD_ERR_CUDA, EMD_ERR_NOMEM, EMD_ERR_OVERFLOW_GHOST,
                   EMD_ERR_OVERFLOW_NEIGH, EMD_ERR_STATE, EMD_ERR_TIMEOUT, EMD_NEIGH_2D, EMD_NEIGH_CSR, EMD_OK,
                   EMD_PREC_FP64, EMD_PREC_MIXED, MD, Batch, Context, EmdError, library_path, load_library)

__all__ = ["Batch", "Context", "MD", "EmdError", "load_library", "library_path", "EMD_PREC_FP64", "EMD_PREC_MIXED",
           "EMD_NEIGH_CSR", "EMD_NEIGH_2D", "EMD_OK", "EMD_ERR_OVERFLOW_GHOST", "EMD_ERR_OVERFLOW_NEIGH",
           "EMD_ERR_TIMEOUT", "EMD_ERR_BOUNDS", "EMD_ERR_CUDA", "EMD_ERR_ARG", "EMD_ERR_STATE", "EMD_ERR_NOMEM"]
