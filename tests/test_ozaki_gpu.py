"""Split-precision (Ozaki) f64 GEMM on tcgen05 vs the double-double oracle.

Known answers first: small-integer operands make every slice product exact,
so the result must equal the exact integer product bit for bit. Then random
operands against max |C - C_dd| / (|A||B|)_ij, compared with the native FP64
DMMA GEMM's own error on the same inputs.
"""
import numpy as np
import pytest
import torch

from numrs_gb300 import _lib as L
from tests.conftest import to_np

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _err(C, Cdd, ab):
    return float(np.max(np.where(ab > 0, np.abs(C - Cdd) / np.where(ab > 0, ab, 1), 0), initial=0))


@pytest.mark.parametrize("mkn", [(128, 64, 256), (128, 128, 256), (200, 100, 300), (256, 1000, 512),
                                 (1, 7, 1), (129, 65, 257)])
def test_ozaki_integer_known_answer(K, mkn):
    m, k, n = mkn
    r = np.random.default_rng(1)
    A = r.integers(-3, 4, (m, k)).astype(np.float64)
    B = r.integers(-3, 4, (k, n)).astype(np.float64)
    C, info = K.gemm_ozaki(_dev(A), _dev(B), slices=2)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    np.testing.assert_array_equal(to_np(C), exact)
    assert info["products"] == 3


@pytest.mark.parametrize("mkn", [(128, 256, 256), (300, 500, 200), (512, 512, 512), (1024, 4096, 768)])
def test_ozaki_f64_accuracy(K, ora, mkn):
    m, k, n = mkn
    A = ora.gen_uniform_pm1(5, m * k).reshape(m, k)
    B = ora.gen_uniform_pm1(6, k * n).reshape(k, n)
    C, info = K.gemm_ozaki(_dev(A), _dev(B))
    Cdd, ab = ora.gemm_dd(A, B)
    e_oz = _err(to_np(C), Cdd, ab)
    Cd = K.matmul(_dev(A), _dev(B), variant=L.GEMM_DMMA)
    e_dmma = _err(to_np(Cd), Cdd, ab)
    assert e_oz <= 1e-14, (e_oz, e_dmma, info)
    assert e_oz <= max(3 * e_dmma, 5e-16), (e_oz, e_dmma)


def test_ozaki_dynamic_range(K, ora):
    """Entries U(-0.5,0.5)*exp(phi*N(0,1)), phi = 1: more slices shrink the error."""
    m = k = n = 256
    A = torch.empty((m, k), dtype=torch.float64, device="cuda")
    B = torch.empty((k, n), dtype=torch.float64, device="cuda")
    K.fill_random(A, L.RNG_OZAKI, 5, 1.0, 0.0)
    K.fill_random(B, L.RNG_OZAKI, 6, 1.0, 0.0)
    Cdd, ab = ora.gemm_dd(to_np(A), to_np(B))
    errs = []
    for s in (6, 9, 12):
        C, _ = K.gemm_ozaki(A, B, slices=s)
        errs.append(_err(to_np(C), Cdd, ab))
    assert errs[0] >= errs[1] >= errs[2]
    assert errs[2] <= 1e-14


def test_ozaki_zero_and_errors(K):
    import numrs_gb300 as N
    A = torch.zeros((64, 32), dtype=torch.float64, device="cuda")
    B = torch.zeros((32, 300), dtype=torch.float64, device="cuda")
    C, _ = K.gemm_ozaki(A, B)
    assert torch.all(C == 0)
    with pytest.raises(N.NumRs2Error):
        K.gemm_ozaki(A, B, slices=17)
    Z = torch.zeros((64, 0), dtype=torch.float64, device="cuda")
    C, _ = K.gemm_ozaki(Z, torch.zeros((0, 8), dtype=torch.float64, device="cuda"))
    assert torch.all(C == 0)


@pytest.mark.parametrize("k,bits", [(2048, 8), (20000, 7)])
def test_ozaki_digit_width_follows_k(K, ora, k, bits):
    """The widest digits whose int32 diagonal sums stay exact: 8-bit digits
    (1024-wide exact FP32 chunks) while ceil(k / 1024) * S < 128, else 7-bit
    (4096-wide chunks); both at the FP64 error level."""
    m = n = 128
    A = ora.gen_uniform_pm1(7, m * k).reshape(m, k)
    B = ora.gen_uniform_pm1(8, k * n).reshape(k, n)
    C, info = K.gemm_ozaki(_dev(A), _dev(B))
    assert info["slice_bits"] == bits, info
    assert info["k_chunk"] == 1 << (26 - 2 * bits)
    Cdd, ab = ora.gemm_dd(A, B)
    e_oz = _err(to_np(C), Cdd, ab)
    e_dmma = _err(to_np(K.matmul(_dev(A), _dev(B), variant=L.GEMM_DMMA)), Cdd, ab)
    assert e_oz <= 1e-14 and e_oz <= max(3 * e_dmma, 5e-16), (e_oz, e_dmma, info)
