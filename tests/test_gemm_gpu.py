"""Plain GEMM on the GPU vs the double-double oracle and numrs2's restated
CPU GEMM.

f64 (DMMA and SIMT): max |C - C_dd| / (|A||B|)_ij <= 1e-14, the north-star
tolerance normalised componentwise. f32: <= 1e-5 (K <= 4096). Integers:
bit-exact. Size grid, overwrite-garbage and k = 0 cases follow
src/kernels/gemm.rs:499-721.
"""
import numpy as np
import pytest
import torch

from numrs_gb300 import _lib as L
from tests.conftest import to_np

pytestmark = pytest.mark.gpu

SIZE_GRID = [(1, 1, 1), (2, 2, 2), (31, 31, 31), (32, 32, 32), (33, 33, 33), (63, 63, 63),
             (64, 64, 64), (65, 65, 65), (127, 127, 127), (128, 128, 128), (0, 5, 4), (5, 0, 4),
             (5, 4, 0), (7, 300, 129), (200, 17, 333)]


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _err(C, Cdd, ab):
    return float(np.max(np.where(ab > 0, np.abs(C - Cdd) / np.where(ab > 0, ab, 1), 0), initial=0))


@pytest.mark.parametrize("variant", [L.GEMM_AUTO, L.GEMM_DMMA, L.GEMM_SIMT, L.GEMM_GENERIC])
@pytest.mark.parametrize("mkn", SIZE_GRID)
def test_gemm_f64_size_grid(K, ora, mkn, variant):
    m, k, n = mkn
    A = ora.gen_uniform_pm1(1, m * k).reshape(m, k)
    B = ora.gen_uniform_pm1(2, k * n).reshape(k, n)
    C = torch.full((m, n), float("nan"), dtype=torch.float64, device="cuda")  # garbage
    K.gemm_2d(m, k, n, _dev(A), _dev(B), C, variant=variant)
    Cg = to_np(C)
    Cdd, ab = ora.gemm_dd(A, B)
    if m * n:
        assert not np.any(np.isnan(Cg))
        assert _err(Cg, Cdd, ab) <= 1e-14
        if k == 0:
            assert np.all(Cg == 0)


def test_gemm_f64_512_config(K, ora):
    """The plain f64 GEMM workload: 512^3, U(-1,1) from SplitMix64 seeds 1/2."""
    A = torch.empty((512, 512), dtype=torch.float64, device="cuda")
    B = torch.empty_like(A)
    K.fill_random(A, L.RNG_UNIFORM, 1, -1.0, 1.0)
    K.fill_random(B, L.RNG_UNIFORM, 2, -1.0, 1.0)
    C = K.matmul(A, B, variant=L.GEMM_DMMA)
    An, Bn = to_np(A), to_np(B)
    np.testing.assert_array_equal(An.ravel(), ora.gen_uniform_pm1(1, 512 * 512))
    Cdd, ab = ora.gemm_dd(An, Bn)
    assert _err(to_np(C), Cdd, ab) <= 1e-14
    Cr = ora.gemm(An, Bn)  # numrs2's own CPU result (restated)
    assert _err(Cr, Cdd, ab) <= 1e-14
    assert np.max(np.abs(to_np(C) - Cr) / ab) <= 2e-14


@pytest.mark.parametrize("variant", [L.GEMM_AUTO, L.GEMM_SIMT, L.GEMM_SIMT_SMALL, L.GEMM_GENERIC])
@pytest.mark.parametrize("mkn", [(1, 1, 1), (33, 65, 31), (128, 128, 128), (300, 1000, 257), (1024, 512, 1024)])
def test_gemm_f32(K, ora, mkn, variant):
    m, k, n = mkn
    r = np.random.default_rng(5)
    A = r.uniform(-1, 1, (m, k)).astype(np.float32)
    B = r.uniform(-1, 1, (k, n)).astype(np.float32)
    C = torch.full((m, n), float("nan"), device="cuda")
    K.gemm_2d(m, k, n, _dev(A), _dev(B), C, variant=variant)
    Cdd, ab = ora.gemm_dd(A.astype(np.float64), B.astype(np.float64))
    assert _err(to_np(C).astype(np.float64), Cdd, ab) <= 1e-5


def test_gemm_i64_exact(K, ora):
    r = np.random.default_rng(6)
    A = r.integers(-1000, 1000, (37, 129)).astype(np.int64)
    B = r.integers(-1000, 1000, (129, 65)).astype(np.int64)
    C = torch.zeros((37, 65), dtype=torch.int64, device="cuda")
    K.gemm_2d(37, 129, 65, _dev(A), _dev(B), C)
    np.testing.assert_array_equal(to_np(C), ora.gemm(A, B))


def test_transposed_and_accumulate(K, ora):
    r = np.random.default_rng(8)
    A = r.uniform(-1, 1, (90, 70))
    B = r.uniform(-1, 1, (110, 90))
    At, Bt = _dev(A).t(), _dev(B).t()  # (70, 90) @ (90, 110) via transposed views
    C = K.matmul(At, Bt)
    Cdd, ab = ora.gemm_dd(A.T.copy(), B.T.copy())
    assert _err(to_np(C), Cdd, ab) <= 1e-14
    out = torch.ones((70, 110), dtype=torch.float64, device="cuda")
    K.matmul_to(At, Bt, out)
    assert np.max(np.abs(to_np(out) - (Cdd + 1.0))) <= 1e-12


def test_matmul_batched_and_promotion(K, ora):
    """Broadcast batch axes and 1-D promotion against the oracle's
    Array::matmul restatement (more of the reference's cases in
    tests/test_matmul_nd.py)."""
    r = np.random.default_rng(12)
    a = r.uniform(-1, 1, (3, 1, 20, 30))
    b = r.uniform(-1, 1, (4, 30, 10))
    c = to_np(K.matmul(_dev(a), _dev(b)))
    want = ora.matmul(a, b)
    assert c.shape == want.shape == (3, 4, 20, 10)
    for i in range(3):
        for j in range(4):
            Cdd, ab = ora.gemm_dd(a[i, 0], b[j])
            assert _err(c[i, j], Cdd, ab) <= 1e-14
    v = r.uniform(-1, 1, 30)
    c = to_np(K.matmul(_dev(a[0, 0]), _dev(v)))
    assert c.shape == ora.matmul(a[0, 0], v).shape == (20, 1)


def test_gemm_errors(K):
    import numrs_gb300 as N
    a = torch.ones((3, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(N.ShapeMismatch):
        K.matmul(a, a)
    with pytest.raises(N.ShapeMismatch):
        K.gemm_2d(3, 4, 5, a, a, a)
