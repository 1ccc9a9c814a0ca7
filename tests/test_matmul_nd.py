"""N-D batched / broadcast Array::matmul, pinned to the reference's own cases.

The cases are those of the reference's tests/test_matmul_dispatch.rs:368-540
(3-D batched grid, a 4-D batch that must equal its 3-D flattening bit for
bit, the batched generic integer tier, broadcast panel pairing, rank
mismatch, identity and associativity, rejected inner dimensions) on its
seq_f64 / seq_i32 data (:113-123). The CPU part checks the oracle's
restatement of Array::matmul (src/array/linalg.rs:153-266, batched_gemm
:56-136) against naive loops with the reference's 1e-9 relative bar; the
GPU part runs numrs_gb300's matmul through the C ABI against that oracle,
with f64 results held to the componentwise double-double bar
max |C - C_dd| / (|A||B|)_ij <= 1e-14 and integers exact.
"""
import numpy as np
import pytest

BATCH_GRID = [(1, 4, 5, 3), (3, 8, 7, 6), (8, 16, 16, 16), (64, 16, 16, 16), (5, 33, 65, 31)]


def seq_f64(n, scale, offset):
    return np.arange(n, dtype=np.float64) * scale + offset


def seq_i32(n, modulus, offset):
    return (np.arange(n, dtype=np.int64) % modulus + offset).astype(np.int64)


def naive(a, b):
    """Per-panel triple loop in f64 (the reference tests' naive_gemm_f64)."""
    return np.einsum("...ik,...kj->...ij", a, b)


def _close(got, want, tol):
    scale = np.maximum(np.abs(want), 1.0)
    return float(np.max(np.abs(got - want) / scale, initial=0.0)) <= tol


# ---------------------------------------------------------------- oracle (CPU)
@pytest.mark.parametrize("bmkn", BATCH_GRID)
def test_oracle_batched_matches_naive(ora, bmkn):
    batch, m, k, n = bmkn
    a = seq_f64(batch * m * k, 0.0625, -1.25).reshape(batch, m, k)
    b = seq_f64(batch * k * n, -0.03125, 2.5).reshape(batch, k, n)
    c = ora.matmul(a, b)
    assert c.shape == (batch, m, n)
    assert _close(c, naive(a, b), 1e-9)


def test_oracle_4d_equals_3d_and_broadcast_pairing(ora):
    b0, b1, m, k, n = 2, 3, 6, 5, 4
    ad = seq_f64(6 * m * k, 0.1, -0.5)
    bd = seq_f64(6 * k * n, -0.2, 1.0)
    c4 = ora.matmul(ad.reshape(b0, b1, m, k), bd.reshape(b0, b1, k, n))
    c3 = ora.matmul(ad.reshape(6, m, k), bd.reshape(6, k, n))
    assert c4.shape == (b0, b1, m, n)
    np.testing.assert_array_equal(c4.reshape(6, m, n), c3)
    # [2,1,m,k] x [1,3,k,n] -> [2,3,m,n]: panel (i, j) pairs a_i with b_j
    m, k, n = 4, 3, 5
    a = seq_f64(2 * m * k, 0.25, -1.0).reshape(2, 1, m, k)
    b = seq_f64(3 * k * n, -0.5, 2.0).reshape(1, 3, k, n)
    c = ora.matmul(a, b)
    assert c.shape == (2, 3, m, n)
    for i in range(2):
        for j in range(3):
            assert _close(c[i, j], naive(a[i, 0], b[0, j]), 1e-9)
    # rank mismatch: [3,m,k] x [2,3,k,n]: a panel j pairs with b panel (i, j)
    m, k, n = 3, 4, 2
    a = seq_f64(3 * m * k, 0.5, -2.0).reshape(3, m, k)
    b = seq_f64(6 * k * n, -0.25, 1.0).reshape(2, 3, k, n)
    c = ora.matmul(a, b)
    assert c.shape == (2, 3, m, n)
    for i in range(2):
        for j in range(3):
            assert _close(c[i, j], naive(a[j], b[i, j]), 1e-9)


def test_oracle_promotion_keeps_unit_axes_and_errors(ora):
    a = seq_f64(12, 1.0, 0.0).reshape(3, 4)
    v = seq_f64(4, 0.5, -1.0)
    assert ora.matmul(v, a.T).shape == (1, 3)       # [1,4] x [4,3]
    assert ora.matmul(a, v).shape == (3, 1)         # [3,4] x [4,1]
    assert ora.matmul(v, v).shape == (1, 1)
    assert ora.matmul(np.stack([a, a]), v).shape == (2, 3, 1)
    with pytest.raises(ValueError, match="shape"):
        ora.matmul(seq_f64(6, 1, 0).reshape(2, 3), seq_f64(8, 1, 0).reshape(4, 2))
    with pytest.raises(ValueError, match="shape"):
        ora.matmul(seq_f64(12, 1, 0).reshape(2, 2, 3), seq_f64(16, 1, 0).reshape(2, 4, 2))
    with pytest.raises(ValueError, match="shape"):
        ora.matmul(np.zeros((2, 3, 4)), np.zeros((3, 4, 5)))   # batch 2 vs 3
    with pytest.raises(ValueError, match="dimension"):
        ora.matmul(np.float64(2.0), a)


def test_oracle_batched_integer_exact(ora):
    batch, m, k, n = 4, 5, 3, 6
    a = seq_i32(batch * m * k, 7, -3).reshape(batch, m, k)
    b = seq_i32(batch * k * n, 5, -2).reshape(batch, k, n)
    np.testing.assert_array_equal(ora.matmul(a, b), naive(a, b))


# ------------------------------------------------------------------- GPU
def _dd_err(ora, c, a, b):
    """max |C - C_dd| / (|A||B|)_ij over the broadcast panels."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    batch = np.broadcast_shapes(a.shape[:-2], b.shape[:-2])
    af = np.broadcast_to(a, batch + a.shape[-2:]).reshape(-1, *a.shape[-2:])
    bf = np.broadcast_to(b, batch + b.shape[-2:]).reshape(-1, *b.shape[-2:])
    cf = np.asarray(c, dtype=np.float64).reshape(-1, c.shape[-2], c.shape[-1])
    worst = 0.0
    for t in range(af.shape[0]):
        cdd, ab = ora.gemm_dd(af[t], bf[t])
        d = np.abs(cf[t] - cdd)
        worst = max(worst, float(np.max(np.where(ab > 0, d / np.where(ab > 0, ab, 1), d), initial=0.0)))
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("bmkn", BATCH_GRID)
def test_gpu_batched_against_oracle(K, ora, bmkn):
    import torch
    batch, m, k, n = bmkn
    a = seq_f64(batch * m * k, 0.0625, -1.25).reshape(batch, m, k)
    b = seq_f64(batch * k * n, -0.03125, 2.5).reshape(batch, k, n)
    c = K.matmul(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()).cpu().numpy()
    want = ora.matmul(a, b)
    assert c.shape == want.shape
    assert _close(c, want, 1e-9)
    assert _dd_err(ora, c, a, b) <= 1e-14


@pytest.mark.gpu
def test_gpu_4d_bit_identical_to_3d_and_broadcast(K, ora):
    import torch
    b0, b1, m, k, n = 2, 3, 6, 5, 4
    ad = seq_f64(6 * m * k, 0.1, -0.5)
    bd = seq_f64(6 * k * n, -0.2, 1.0)
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()  # noqa: E731
    c4 = K.matmul(dev(ad.reshape(b0, b1, m, k)), dev(bd.reshape(b0, b1, k, n))).cpu().numpy()
    c3 = K.matmul(dev(ad.reshape(6, m, k)), dev(bd.reshape(6, k, n))).cpu().numpy()
    assert c4.shape == (b0, b1, m, n)
    np.testing.assert_array_equal(c4.reshape(6, m, n), c3)
    for (a, b) in ((seq_f64(2 * 4 * 3, 0.25, -1.0).reshape(2, 1, 4, 3), seq_f64(3 * 3 * 5, -0.5, 2.0).reshape(1, 3, 3, 5)),
                   (seq_f64(3 * 3 * 4, 0.5, -2.0).reshape(3, 3, 4), seq_f64(6 * 4 * 2, -0.25, 1.0).reshape(2, 3, 4, 2))):
        c = K.matmul(dev(a), dev(b)).cpu().numpy()
        want = ora.matmul(a, b)
        assert c.shape == want.shape == (2, 3, a.shape[-2], b.shape[-1])
        assert _close(c, want, 1e-9)
        assert _dd_err(ora, c, a, b) <= 1e-14


@pytest.mark.gpu
def test_gpu_batched_integer_exact_and_f32(K, ora):
    import torch
    batch, m, k, n = 4, 5, 3, 6
    a = seq_i32(batch * m * k, 7, -3).reshape(batch, m, k)
    b = seq_i32(batch * k * n, 5, -2).reshape(batch, k, n)
    c = K.matmul(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()).cpu().numpy()
    np.testing.assert_array_equal(c, ora.matmul(a, b))
    a32 = seq_f64(3 * 20 * 30, 0.01, -4.0).reshape(3, 1, 20, 30).astype(np.float32)
    b32 = seq_f64(4 * 30 * 10, -0.02, 6.0).reshape(4, 30, 10).astype(np.float32)
    c = K.matmul(torch.from_numpy(a32).cuda(), torch.from_numpy(b32).cuda()).cpu().numpy()
    want = ora.matmul(a32, b32)
    assert c.shape == want.shape == (3, 4, 20, 10)
    # f32: the same normalisation at 1e-5 against the double-double product
    assert _dd_err(ora, c, a32, b32) <= 1e-5


@pytest.mark.gpu
def test_gpu_promotion_identity_associativity_errors(K, ora):
    import torch
    import numrs_gb300 as N
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()  # noqa: E731
    a = seq_f64(12, 1.0, 0.0).reshape(3, 4)
    v = seq_f64(4, 0.5, -1.0)
    for x, y in ((v, a.T), (a, v), (v, v), (np.stack([a, a]), v), (v, np.stack([a.T, a.T]))):
        c = K.matmul(dev(x), dev(y)).cpu().numpy()
        want = ora.matmul(x, y)
        assert c.shape == want.shape, (x.shape, y.shape, c.shape, want.shape)
        assert _close(c, want, 1e-12)
    n = 65
    eye = np.eye(n)
    A = seq_f64(n * n, 0.01, -0.5).reshape(n, n)
    B = seq_f64(n * n, -0.02, 0.25).reshape(n, n)
    ai = K.matmul(dev(A), dev(eye)).cpu().numpy()
    ia = K.matmul(dev(eye), dev(A)).cpu().numpy()
    assert _close(ai, A, 1e-12) and _close(ia, A, 1e-12)
    left = K.matmul(K.matmul(dev(A), dev(B)), dev(eye)).cpu().numpy()
    right = K.matmul(dev(A), K.matmul(dev(B), dev(eye))).cpu().numpy()
    assert _close(left, right, 1e-9)
    with pytest.raises(N.ShapeMismatch):
        K.matmul(dev(seq_f64(6, 1, 0).reshape(2, 3)), dev(seq_f64(8, 1, 0).reshape(4, 2)))
    with pytest.raises(N.ShapeMismatch):
        K.matmul(dev(seq_f64(12, 1, 0).reshape(2, 2, 3)), dev(seq_f64(16, 1, 0).reshape(2, 4, 2)))
    with pytest.raises(N.ShapeMismatch):
        K.matmul(dev(np.zeros((2, 3, 4))), dev(np.zeros((3, 4, 5))))
    with pytest.raises(N.DimensionMismatch):
        K.matmul(torch.tensor(2.0, dtype=torch.float64, device="cuda"), dev(a))
