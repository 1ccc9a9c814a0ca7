"""The C-ABI library loads and exports every symbol include/numrs_gpu.h
declares; host-side logic that needs no GPU (CPU only)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "numrs_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nrs_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    assert "nrs_reduce" in names and "nrs_gemm" in names and "nrs_ufunc" in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = C.CDLL(lib_path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header():
    from numrs_gb300 import _lib as L
    missing = [n for n in _declared() if n not in L.SIGNATURES]
    assert not missing, missing


def test_status_strings_and_version(lib_path):
    from numrs_gb300 import _lib as L
    lib = L.load()
    assert lib.nrs_abi_version() == 3
    for s in range(0, -12, -1):
        assert lib.nrs_status_string(s)
    # Null handles are rejected on the host, before any CUDA call.
    assert lib.nrs_reduce(None, 0, 0, 0, None, None, 0, 0, None, None) == L.ERR_INVALID
    assert lib.nrs_gemm(None, 0, 1, 1, 1, None, 1, None, 1, None, 1, 0, 0) == L.ERR_INVALID


def test_error_kinds_map_to_reference_errors():
    from numrs_gb300 import _lib as L
    with pytest.raises(L.DimensionMismatch):
        L.check(L.ERR_AXIS)
    with pytest.raises(L.InvalidOperation):
        L.check(L.ERR_EMPTY)
    with pytest.raises(L.ShapeMismatch):
        L.check(L.ERR_SHAPE)


def test_expr_program_compiles_to_postfix():
    import torch
    from numrs_gb300 import _lib as L
    from numrs_gb300.kernels import Expr
    x = torch.zeros(4)
    e = (Expr.leaf(x) * 0.5 + (-0.25)).exp()
    assert [k for k, _ in e.prog] == ["in", "sc", "op", "sc", "op", "op"]
    assert e.prog[2][1] == L.OP_MUL and e.prog[4][1] == L.OP_ADD and e.prog[5][1] == L.OP_EXP
