"""numrs_gb300: NumRS2's `kernels` dispatch layer (GEMM, reductions,
elementwise ufuncs) as hand-written sm_103a CUDA behind a C ABI
(include/numrs_gpu.h).

`numrs_gb300.kernels` is the reference-shaped host API; `numrs_gb300._lib`
is the raw ctypes binding. The compiled library is loaded on first use and
its absence raises: there is no CPU fallback.
"""
from ._lib import (DeviceTimeout, DimensionMismatch, InvalidOperation, NumRs2Error,  # noqa: F401
                   ShapeMismatch)
