"""CPU oracle for the NumRS2 `kernels` hot path -- test infrastructure only.

The oracle restates the reference's CPU kernels (see ``oracle.c`` for the
per-function citations). Only the test suite, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may load it; the CUDA library and the
``numrs_gb300`` package never do.
"""
from .oracle import Oracle, build, load  # noqa: F401
