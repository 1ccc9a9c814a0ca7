"""Ufunc reduce / accumulate, cumsum / cumprod on the GPU vs the CPU oracle.

Along an axis every lane is the reference's left-to-right chain, so results
are bit-identical (NaN payloads aside: IEEE leaves them open and the GPU
returns one canonical NaN from arithmetic). Over the flattened array,
maximum / minimum and integer add / multiply are exact; f32/f64 add /
multiply of 64+ elements are reassociated and compared within a tolerance
scaled by the running sum of |x| (subtract / divide stay serial and exact).
"""
import numpy as np
import pytest
import torch

import numrs_gb300 as N
from tests.conftest import bits, to_np
from tests.test_oracle_golden import UFUNC_KAT_ERRORS, UFUNC_KATS

pytestmark = pytest.mark.gpu

OPS = {"add": 2, "subtract": 3, "multiply": 4, "divide": 5, "maximum": 11, "minimum": 12}
NAME = {v: k for k, v in OPS.items()}


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _same(got, ref):
    """Bit-identical, except that two NaNs match whatever their payloads."""
    got, ref = np.ascontiguousarray(got), np.ascontiguousarray(ref)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    if got.dtype.kind == "f":
        nan = np.isnan(ref)
        np.testing.assert_array_equal(np.isnan(got), nan)
        np.testing.assert_array_equal(bits(got[~nan]), bits(ref[~nan]))
    else:
        np.testing.assert_array_equal(got, ref)


def _data(r, shape, dtype, op):
    if np.dtype(dtype).kind == "i":
        lo, hi = (-3, 4) if op == "multiply" else (-1000, 1000)
        return r.integers(lo, hi, shape).astype(dtype)
    if op in ("multiply", "divide"):  # keep running products in range
        return (r.uniform(0.5, 1.5, shape) * r.choice([-1.0, 1.0], shape)).astype(dtype)
    return r.standard_normal(shape).astype(dtype)


@pytest.mark.parametrize("case", UFUNC_KATS, ids=[c[0] for c in UFUNC_KATS])
def test_known_answers(K, case):
    _, kind, op, data, shape, axis, initial, want = case
    x = _dev(np.array(data, dtype=np.float64).reshape(shape))
    if kind == "reduce":
        got = K.ufunc_reduce(NAME[op], x, axis, initial=initial)
    else:
        got = K.ufunc_accumulate(NAME[op], x, axis)
    np.testing.assert_allclose(to_np(got).ravel(), want, rtol=1e-15, atol=0)


@pytest.mark.parametrize("case", UFUNC_KAT_ERRORS, ids=[c[0] for c in UFUNC_KAT_ERRORS])
def test_known_errors(K, case):
    _, op, shape, axis = case
    with pytest.raises(N.NumRs2Error):
        K.ufunc_reduce(NAME[op], torch.zeros(shape, dtype=torch.float64, device="cuda"), axis)


def test_shapes_and_axis_errors(K):
    x = torch.zeros((3, 0), dtype=torch.float64, device="cuda")
    assert tuple(K.ufunc_reduce("add", x, 0).shape) == (0,)
    assert tuple(K.ufunc_reduce("add", x, 1, keepdims=True).shape) == (3, 1)
    y = torch.ones((2, 3), dtype=torch.float32, device="cuda")
    for ax in (2, -3):
        with pytest.raises(N.DimensionMismatch):
            K.ufunc_reduce("add", y, ax)
        with pytest.raises(N.DimensionMismatch):
            K.ufunc_accumulate("maximum", y, ax)
    with pytest.raises(N.NumRs2Error):
        K.ufunc_accumulate("divide", torch.ones(4, dtype=torch.int64, device="cuda"))
    assert tuple(K.ufunc_reduce("add", y, None, keepdims=True).shape) == (1, 1)
    assert tuple(K.cumsum(y).shape) == (6,)


# (shape, axis, view): each exercises one kernel path. "t" = transposed view
# of a buffer of the reversed shape, "s" = every other column (no TMA).
LANE_CASES = [
    ((300, 200), 0, None),     # lanes adjacent: column pipeline, partial lane block
    ((200, 300), 1, None),     # lanes along rows: row pipeline, partial tiles
    ((300, 200), 0, "t"),      # transposed view: row pipeline
    ((200, 300), 1, "t"),      # transposed view: column pipeline
    ((3, 260, 136), 1, None),  # batched columns
    ((3, 40, 300), 2, None),   # collapsed batch rows
    ((1000, 260), 1, None),    # many rows: rows per CTA chosen at launch, partial last CTA
    ((3, 40, 300), 0, None),   # short axis: generic
    ((50, 400), 1, "s"),       # strided columns: generic
    ((1000,), 0, None),        # one lane
]


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
@pytest.mark.parametrize("op", list(OPS))
@pytest.mark.parametrize("case", range(len(LANE_CASES)))
def test_axis_reduce_and_accumulate_bit_exact(K, ora, dtype, op, case):
    if op == "divide" and dtype == np.int64:
        pytest.skip("integer divide is not a ufunc reduce/accumulate")
    shape, axis, view = LANE_CASES[case]
    r = np.random.default_rng(1000 + case)
    if view == "t":
        base = _data(r, shape[::-1], dtype, op)
        x_np, x = base.T, _dev(base).t()
    elif view == "s":
        base = _data(r, (shape[0], shape[1] * 2), dtype, op)
        x_np, x = base[:, ::2], _dev(base)[:, ::2]
    else:
        x_np = _data(r, shape, dtype, op)
        x = _dev(x_np)
    _same(to_np(K.ufunc_accumulate(op, x, axis)), ora.accumulate(OPS[op], x_np, axis))
    got = to_np(K.ufunc_reduce(op, x, axis)).ravel()
    _same(got, ora.ufunc_reduce(OPS[op], x_np, axis))
    init = 3 if dtype == np.int64 else 0.75
    got = to_np(K.ufunc_reduce(op, x, axis, initial=init)).ravel()
    _same(got, ora.ufunc_reduce(OPS[op], x_np, axis, init))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_axis_nan_and_signed_zero(K, ora, dtype):
    """NaN propagation and the tie rule of maximum / minimum (the later of
    two equal values wins: -0.0 vs +0.0) along both pipelines."""
    r = np.random.default_rng(5)
    x = r.choice(np.array([-0.0, 0.0, 1.0, -1.0], dtype=dtype), (300, 260))
    x[r.random(x.shape) < 0.002] = np.nan
    for axis in (0, 1):
        for op in ("maximum", "minimum", "add", "subtract"):
            _same(to_np(K.ufunc_accumulate(op, _dev(x), axis)), ora.accumulate(OPS[op], x, axis))
            _same(to_np(K.ufunc_reduce(op, _dev(x), axis)).ravel(), ora.ufunc_reduce(OPS[op], x, axis))


@pytest.mark.parametrize("offset", [0, 1])  # 1: a view one element in (not 16-byte aligned)
@pytest.mark.parametrize("n", [1, 5, 63, 64, 4095, 4096, 4097, 8191, 8192, 8193, 100003, (1 << 22) + 5])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
def test_flat_accumulate(K, ora, n, dtype, offset):
    r = np.random.default_rng(n)
    for op in OPS:
        if op == "divide" and dtype == np.int64:
            continue
        if op in ("subtract", "divide") and n > 100003:
            continue  # serial chains: the long case is the parallel ops'
        x = _data(r, (n,), dtype, op)
        if np.dtype(dtype).kind == "f" and op in ("maximum", "minimum"):
            x[r.random(n) < 1e-3] = np.nan
            x[r.random(n) < 1e-3] = -0.0
            x[r.random(n) < 1e-3] = 0.0
        xd = _dev(np.concatenate([np.zeros(offset, dtype), x]))[offset:]
        got = to_np(K.ufunc_accumulate(op, xd))
        ref = ora.accumulate(OPS[op], x)
        reassoc = np.dtype(dtype).kind == "f" and op in ("add", "multiply") and n >= 64
        if not reassoc:
            _same(got, ref)
        elif op == "add":
            tol = (4e-6 if dtype == np.float32 else 1e-14) * np.cumsum(np.abs(x.astype(np.float64)))
            assert np.all(np.abs(got.astype(np.float64) - np.cumsum(x.astype(np.float64))) <= tol + 1e-30)
        else:
            # relative error grows with the number of roundings; products
            # that reach the subnormal range keep an absolute floor
            exact = np.cumprod(x.astype(np.float64))
            tol = (4e-6 if dtype == np.float32 else 1e-14) * np.arange(1, n + 1) * np.abs(exact)
            assert np.all(np.abs(got.astype(np.float64) - exact) <= tol + np.finfo(dtype).tiny)


@pytest.mark.parametrize("offset", [0, 1])
@pytest.mark.parametrize("n", [1, 7, 5000, 65537, (1 << 22) + 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
def test_flat_reduce(K, ora, n, dtype, offset):
    r = np.random.default_rng(7 + n)
    for op in OPS:
        if op == "divide" and dtype == np.int64:
            continue
        if op in ("subtract", "divide") and n > 65537:
            continue
        x = _data(r, (n,), dtype, op)
        if np.dtype(dtype).kind == "f" and op in ("maximum", "minimum") and n > 1:
            x[r.integers(0, n, 3)] = -0.0
            x[r.integers(0, n, 3)] = 0.0
        for init in (None, 2 if dtype == np.int64 else 0.5):
            xd = _dev(np.concatenate([np.zeros(offset, dtype), x]))[offset:]
            got = to_np(K.ufunc_reduce(op, xd, None, initial=init))
            ref = ora.ufunc_reduce(OPS[op], x, None, init)
            if np.dtype(dtype).kind == "f" and op in ("add", "multiply"):
                # seed (op) the tiered flat sum / product: within the flat
                # kernels' own tolerance of the restated reference; products
                # that underflow end at the subnormal floor in any order.
                np.testing.assert_allclose(got, ref, rtol=5e-5 if dtype == np.float32 else 1e-12,
                                           atol=1e-5 * float(np.abs(x).sum()) if op == "add"
                                           else float(np.finfo(dtype).tiny))
            else:
                _same(got, ref)
    # a NaN anywhere: maximum / minimum give the canonical NaN
    if np.dtype(dtype).kind == "f" and n > 1:
        x = r.standard_normal(n).astype(dtype)
        x[n // 2] = np.nan
        for op in ("maximum", "minimum"):
            assert np.isnan(to_np(K.ufunc_reduce(op, _dev(x)))[0])


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
def test_flat_accumulate_long(K, ora, dtype):
    """Flattened scans of ~100 MB (more than the L2 holds, 300+ segments of
    many tiles each) with a ragged tail: every order-free op exact against the
    oracle (maximum / minimum with NaNs and signed zeros at segment-scale
    offsets), float add within the reassociation tolerance, and two runs bit
    for bit the same."""
    step = 304 * 3 * (32768 // np.dtype(dtype).itemsize)
    n = int(step * 3.4) + 3
    r = np.random.default_rng(77)
    for op in ("add", "maximum", "minimum", "multiply"):
        x = _data(r, (n,), dtype, op)
        if np.dtype(dtype).kind == "f" and op in ("maximum", "minimum"):
            for e in (step - 1, step, 2 * step + 5):
                x[e] = -0.0 if e % 2 else 0.0
            x[int(step * 2.7)] = np.nan
        xd = _dev(x)
        got = to_np(K.ufunc_accumulate(op, xd))
        again = to_np(K.ufunc_accumulate(op, xd))
        np.testing.assert_array_equal(got.view(np.uint8), again.view(np.uint8))
        if np.dtype(dtype).kind == "f" and op in ("add", "multiply"):
            if op == "add":
                ref = np.cumsum(x.astype(np.float64))
                tol = (4e-6 if dtype == np.float32 else 1e-14) * np.cumsum(np.abs(x.astype(np.float64)))
                assert np.all(np.abs(got.astype(np.float64) - ref) <= tol + 1e-30)
            continue  # long float products reach the subnormal floor: covered above
        _same(got, ora.accumulate(OPS[op], x))
        del xd
    torch.cuda.empty_cache()


def test_full_size_properties(K):
    """16384 x 16384 f32 (the reduction benchmark's array): the last row of
    cumsum(axis=0) is sum(axis=0) bit for bit (both are the zero-seeded
    left-to-right lane sum), the same for axis 1 and for the transposed
    view, and the running maximum ends at max(axis)."""
    n = 16384
    x = torch.empty((n, n), device="cuda")
    K.fill_random(x, N._lib.RNG_NORMAL, 3, 0.0, 1.0)
    c0 = K.cumsum(x, 0)
    assert torch.equal(c0[-1].view(torch.int32), K.sum(x, 0).view(torch.int32))
    del c0
    c1 = K.cumsum(x, 1)
    assert torch.equal(c1[:, -1].contiguous().view(torch.int32), K.sum(x, 1).view(torch.int32))
    del c1
    xt = x.t()
    ct = K.cumsum(xt, 0)
    assert torch.equal(ct[-1].contiguous().view(torch.int32), K.sum(xt, 0).view(torch.int32))
    del ct
    m = K.ufunc_accumulate("maximum", x, 1)
    assert torch.equal(m[:, -1].contiguous(), K.max(x, 1))
    del m
    torch.cuda.empty_cache()
