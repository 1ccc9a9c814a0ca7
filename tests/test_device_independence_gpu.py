"""Results do not depend on how many SMs the grids are sized for.

The reference's GEMM splits rows only, so its result is the same for any
thread count (src/kernels/gemm.rs:364-381, tested at :784-807). Here every
plan that decides a rounding order -- a DMMA GEMM's k split, a flattened
scan's segments, the flat reductions' chunk grouping -- is fixed by the
problem's sizes, while grids follow the handle's SM budget. Each case runs
with the full device and with budgets of 100 and 37 SMs and must give the
same bits.
"""
import numpy as np
import pytest
import torch

from numrs_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _cases(K):
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.rand((512, 700), dtype=torch.float64, device="cuda", generator=g) - 0.5
    B = torch.rand((700, 384), dtype=torch.float64, device="cuda", generator=g) - 0.5
    Ab = torch.rand((2048, 2048), dtype=torch.float64, device="cuda", generator=g) - 0.5
    x = torch.randn(12_345_679, device="cuda", generator=g)
    xd = torch.randn(3_000_001, dtype=torch.float64, device="cuda", generator=g)
    m = torch.randn((4096, 3000), device="cuda", generator=g)
    return [
        ("dmma 512x700x384", lambda: K.matmul(A, B, variant=L.GEMM_DMMA)),
        ("dmma 2048^3 (k split)", lambda: K.matmul(Ab, Ab, variant=L.GEMM_DMMA)),
        ("f32 simt", lambda: K.matmul(A.float(), B.float())),
        ("ozaki auto", lambda: K.gemm_ozaki(A, B)[0]),
        ("flat sum f32", lambda: K.sum(x)),
        ("flat var f64", lambda: K.var(xd)),
        ("flat max f32", lambda: K.max(x)),
        ("flat argmax", lambda: K.argmax(x)),
        ("cumsum flat f32", lambda: K.cumsum(x)),
        ("cumprod flat f64", lambda: K.cumprod(1.0 + 1e-7 * xd)),
        ("axis sums", lambda: torch.cat([K.sum(m, 0), K.sum(m, 1), K.mean(m.t(), 0)])),
        ("exp affine", lambda: K.exp_affine(x, 0.5, -0.25)),
    ]


def _bits(t):
    t = t.contiguous()
    return t.view({1: torch.uint8, 2: torch.int16, 4: torch.int32, 8: torch.int64}[t.element_size()])


def test_results_independent_of_sm_budget(K):
    cases = _cases(K)
    full = [fn() for _, fn in cases]
    for sms in (100, 37):
        with K.sm_budget(sms):
            got = [fn() for _, fn in cases]
        torch.cuda.synchronize()
        for (name, _), a, b in zip(cases, full, got):
            assert torch.equal(_bits(a), _bits(b)), (name, sms)


def test_sm_budget_arguments(K):
    lib = L.load()
    h = K.handle()
    assert lib.nrs_set_sm_budget(h, -1) == L.ERR_INVALID
    assert lib.nrs_set_sm_budget(h, 10_000) == L.OK  # clamped to the device
    assert lib.nrs_set_sm_budget(h, 0) == L.OK
