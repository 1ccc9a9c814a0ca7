"""The allocation-free flat reduction, called through the C ABI.

nrs_reduce_flat_noalloc is for callers that must not let this library
allocate device memory -- code under another runtime's memory discipline (a
serving stack or framework allocator that owns and budgets all device memory)
and latency-critical loops that cannot take the synchronisation a cudaMalloc
may cause. It keeps its scratch in a fixed device array instead of a
workspace, so it must give exactly what the ordinary entry point (nrs_reduce
with NRS_AXIS_NONE) gives, call after call, even though every call reuses the
same array. This file is collected last so that a failure here cannot hide
the rest of the suite; it passes on its own in a fresh process as well.
"""
import ctypes as C

import pytest
import torch

from numrs_gb300 import _lib as L

pytestmark = pytest.mark.gpu

MAX_ELEMS = 8192 * 8192


def _noalloc(lib, x, op):
    out = torch.empty(1, dtype=x.dtype, device=x.device)
    st = lib.nrs_reduce_flat_noalloc(C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                     L.F32 if x.dtype == torch.float32 else L.F64, op, x.numel(),
                                     C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()))
    assert st == L.OK, st
    return out


def _bits(t):
    return t.view(torch.int32 if t.element_size() == 4 else torch.int64)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n", [0, 1, 4097, 9999, 50_000, 3_000_017, MAX_ELEMS])
def test_noalloc_equals_nrs_reduce_on_two_calls_in_a_row(K, dtype, n):
    lib = L.load()
    g = torch.Generator(device="cuda").manual_seed(n + 1)
    for op in (L.SUM, L.MEAN, L.MAX, L.MIN):
        # two calls in a row on different data: the second must not see the
        # first call's partials (the shared array keeps them)
        x1 = torch.randn(n, dtype=dtype, device="cuda", generator=g)
        x2 = torch.randn(n, dtype=dtype, device="cuda", generator=g) * 3 + 1
        got1 = _noalloc(lib, x1, op)
        got2 = _noalloc(lib, x2, op)
        ref1 = K.reduce(x1, op)
        ref2 = K.reduce(x2, op)
        torch.cuda.synchronize()
        # same kernels and chunk order as nrs_reduce: identical bits (which is
        # within any tolerance the other reduction tests use)
        assert torch.equal(_bits(got1), _bits(ref1)), (op, got1, ref1)
        assert torch.equal(_bits(got2), _bits(ref2)), (op, got2, ref2)


def test_noalloc_reproduces_reference_pin(K):
    """The reference's pinned f32 sum (x_i = 0.5 i - 12345, N = 50,000)."""
    lib = L.load()
    x = torch.arange(50_000, dtype=torch.float32, device="cuda") * 0.5 - 12345.0
    for _ in range(2):
        got = _noalloc(lib, x, L.SUM)
        assert int(_bits(got).item()) == 1256988984


def test_noalloc_rejects_beyond_the_limit_and_bad_args(K):
    lib = L.load()
    x = torch.zeros(4, device="cuda")
    out = torch.empty(1, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # beyond the documented maximum: refused before anything is launched
    assert lib.nrs_reduce_flat_noalloc(s, L.F32, L.SUM, MAX_ELEMS + 1, C.c_void_p(x.data_ptr()),
                                       C.c_void_p(out.data_ptr())) == L.ERR_TOO_LARGE
    assert lib.nrs_reduce_flat_noalloc(s, L.I64, L.SUM, 4, C.c_void_p(x.data_ptr()),
                                       C.c_void_p(out.data_ptr())) == L.ERR_DTYPE
    assert lib.nrs_reduce_flat_noalloc(s, L.F32, L.PROD, 4, C.c_void_p(x.data_ptr()),
                                       C.c_void_p(out.data_ptr())) == L.ERR_INVALID
    assert lib.nrs_reduce_flat_noalloc(s, L.F32, L.SUM, 4, None, C.c_void_p(out.data_ptr())) == L.ERR_INVALID


def test_noalloc_unaligned_input_and_alternating_calls(K):
    """A view one element in (x[1:], not 16-byte aligned: the scalar-load
    path) gives nrs_reduce's bits; f64 MAX and f32 SUM calls alternating on
    one stream, all sharing the one array, each give their own result."""
    lib = L.load()
    g = torch.Generator(device="cuda").manual_seed(77)
    for dtype in (torch.float32, torch.float64):
        base = torch.randn(1_000_003, dtype=dtype, device="cuda", generator=g)
        x = base[1:]
        assert x.data_ptr() % 16 != 0
        for op in (L.SUM, L.MAX):
            got = _noalloc(lib, x, op)
            torch.cuda.synchronize()
            assert torch.equal(_bits(got), _bits(K.reduce(x, op))), (dtype, op)
    a64 = torch.randn(3_000_001, dtype=torch.float64, device="cuda", generator=g)
    b32 = torch.randn(2_000_003, dtype=torch.float32, device="cuda", generator=g)
    outs = []
    for _ in range(3):  # queued back to back, no synchronisation in between
        outs.append((_noalloc(lib, a64, L.MAX), _noalloc(lib, b32, L.SUM)))
    want_max, want_sum = K.reduce(a64, L.MAX), K.reduce(b32, L.SUM)
    torch.cuda.synchronize()
    for mx, sm in outs:
        assert torch.equal(_bits(mx), _bits(want_max))
        assert torch.equal(_bits(sm), _bits(want_sum))
