"""GB300-native critical-curve and caustic finder (drop-in for weisluke/ccf).

The computation lives in the native library built from ``ccf_gb300/csrc``
(CUDA kernels for sm_103a behind the C ABI of ``include/ccf_gb300.h``);
this package is a thin Python front end over that ABI.
"""
from .ccf import CCF, BatchJob, CCFError, Server, derive_params, pinned_empty, run_batch, submit_batch  # noqa: F401

__all__ = ["CCF", "BatchJob", "CCFError", "Server", "derive_params", "pinned_empty", "run_batch", "submit_batch"]
