"""Reductions on the GPU vs the CPU oracle (numrs2 restatement).

Axis folds are sequential per lane on both sides, so float results are
compared BIT FOR BIT (the reference's own fold order), as are integer sums and
all extrema. Flat float sums use a tree inside each 8192-element chunk and
are compared within |s - s_ref| <= 1e-5 * sum|x| (f32) / 1e-14 (f64), plus
the reference's pinned bit patterns.
"""
import json
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.conftest import bits, to_np

pytestmark = pytest.mark.gpu

OPS = {"sum": O.SUM, "mean": O.MEAN, "max": O.MAX, "min": O.MIN, "prod": O.PROD}


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _data(dtype, shape, seed):
    n = int(np.prod(shape))
    if dtype == np.int64:
        from numrs_gb300 import rng
        return rng.int_range(seed, n).reshape(shape)
    r = np.random.default_rng(seed)
    return r.standard_normal(n).astype(dtype).reshape(shape)


def _check_axis(K, ora, x_np, op, axis, transposed=False):
    xd = _dev(x_np)
    if transposed:
        xd = xd.t()
        x_view = x_np.T
    else:
        x_view = x_np
    got = to_np(getattr(K, op)(xd, axis=axis))
    ref = ora.axis(OPS[op], x_view, axis)
    assert got.shape == ref.shape
    if x_np.dtype == np.int64 and op == "mean":
        np.testing.assert_array_equal(got, ref)
    elif op in ("sum", "mean", "prod") and x_np.dtype != np.int64:
        # A NaN produced by arithmetic carries no payload guarantee (the
        # reference's own contract, src/expr/fused_eval.rs:23-56; the GPU
        # writes the canonical NaN): NaN where the reference has NaN, every
        # other lane bit for bit. Max/min return an element, so they keep it.
        nan = np.isnan(ref)
        assert np.array_equal(np.isnan(got), nan)
        np.testing.assert_array_equal(bits(got[~nan]), bits(ref[~nan]))
    else:
        np.testing.assert_array_equal(bits(got), bits(ref))


SHAPES = [(1, 1), (3, 5), (31, 33), (64, 300), (257, 129), (1000, 333), (512, 2048), (2048, 96),
          (300, 4100)]


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("op", ["sum", "mean", "max", "min"])
def test_axis_folds_bit_exact(K, ora, dtype, shape, op):
    x = _data(dtype, shape, 11)
    for axis in (0, 1, -1):
        _check_axis(K, ora, x, op, axis)
        _check_axis(K, ora, x, op, axis, transposed=True)


@pytest.mark.parametrize("dtype", [np.float32, np.int64])
def test_axis_prod(K, ora, dtype):
    x = np.random.default_rng(3).uniform(0.9, 1.1, (40, 700)).astype(np.float32)
    if dtype == np.int64:
        x = np.random.default_rng(3).integers(-3, 4, (40, 700)).astype(np.int64)
    for axis in (0, 1):
        _check_axis(K, ora, x, "prod", axis)


def test_axis_nan_short_circuit(K, ora):
    x = _data(np.float32, (300, 520), 5)
    # distinct NaN payloads: the first NaN of each lane must be returned
    nan1 = np.array([0x7FC00001], np.uint32).view(np.float32)[0]
    nan2 = np.array([0xFFC00002], np.uint32).view(np.float32)[0]
    x[10, 7] = nan1
    x[200, 7] = nan2
    x[250, 9] = nan2
    x[0, 100] = nan1
    x[299, 519] = nan2
    for op in ("max", "min", "sum"):
        for axis in (0, 1):
            _check_axis(K, ora, x, op, axis)
            _check_axis(K, ora, x, op, axis, transposed=True)


def test_axis_3d_views(K, ora):
    x = _data(np.float32, (6, 70, 300), 9)
    for axis in (0, 1, 2):
        _check_axis(K, ora, x, "sum", axis)
    xd = _dev(x).permute(2, 0, 1)
    xv = x.transpose(2, 0, 1)
    for axis in (0, 1, 2):
        got = to_np(K.sum(xd, axis=axis))
        np.testing.assert_array_equal(bits(got), bits(ora.axis(O.SUM, xv, axis)))
    # kept dims that do not collapse: a batch of column folds / row folds
    y = _data(np.float32, (4, 300, 256), 10)
    for op in ("sum", "max", "mean"):
        for axis in (0, 1, 2):
            _check_axis(K, ora, y, op, axis)
    yd = _dev(y).permute(0, 2, 1)
    yv = y.transpose(0, 2, 1)
    for axis in (1, 2):
        got = to_np(K.sum(yd, axis=axis))
        np.testing.assert_array_equal(bits(got), bits(ora.axis(O.SUM, yv, axis)))


def test_axis_keepdims_and_shapes(K):
    x = torch.ones((4, 5), device="cuda")
    assert tuple(K.sum(x, axis=0, keepdims=True).shape) == (1, 5)
    assert tuple(K.sum(x, axis=1).shape) == (4,)
    assert tuple(K.sum(torch.ones(7, device="cuda"), axis=0).shape) == (1,)
    assert tuple(K.sum(x).shape) == (1,)
    assert tuple(K.sum_axis(x.long(), 1).shape) == (4,)


def test_axis_errors(K):
    import numrs_gb300 as N
    x = torch.ones((4, 5), device="cuda")
    with pytest.raises(N.DimensionMismatch):
        K.sum(x, axis=2)
    with pytest.raises(N.DimensionMismatch):
        K.max(x, axis=-3)
    e = torch.ones((0, 5), device="cuda")
    with pytest.raises(N.InvalidOperation):
        K.max(e, axis=1)
    z = K.sum(e, axis=0)
    assert torch.all(z == 0) and tuple(z.shape) == (5,)


GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


@pytest.mark.parametrize("name", sorted(GOLD["determinism"]["pins"]))
def test_flat_pins_on_gpu(K, name):
    pin = GOLD["determinism"]["pins"][name]
    n = GOLD["determinism"]["n"]
    dt = torch.float32 if name.endswith("f32") else torch.float64
    x = torch.arange(n, dtype=dt, device="cuda") * 0.5 - 12345.0
    if name.startswith("sum"):
        got = K.sum(x)
    elif name.startswith("mean"):
        got = K.mean(x)
    elif name.startswith("var"):
        got = K.var(x, ddof=0)
    else:
        got = K.std(x, ddof=0)
    assert int(bits(to_np(got))[0]) == pin["bits"]


@pytest.mark.parametrize("n", [0, 1, 7, 63, 64, 9999, 10000, 10001, 8192 * 3 + 17, 80000 + 8192 + 17,
                               1 << 22])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_flat_reductions(K, ora, n, dtype):
    x = _data(dtype, (n,), 13)
    xd = _dev(x)
    tol = 1e-5 if dtype == np.float32 else 1e-14
    scale = float(np.sum(np.abs(x.astype(np.float64)))) + 1e-30
    for op in ("sum", "mean"):
        got = float(to_np(getattr(K, op)(xd))[0])
        ref = float(ora.flat(op, x))
        div = 1.0 if op == "sum" else max(n, 1)
        assert abs(got - ref) <= tol * scale / div + 1e-30
    for op in ("max", "min"):
        got = to_np(getattr(K, op)(xd))
        np.testing.assert_array_equal(bits(got), bits(np.array([ora.flat(op, x)], dtype)))
    if n > 1:
        for ddof in (0, 1):
            got = float(to_np(K.var(xd, ddof=ddof))[0])
            ref = float(ora.flat("var", x, ddof))
            assert abs(got - ref) <= tol * 10 * abs(ref) + 1e-30


def test_flat_nan_and_empty(K, ora):
    n = 80000 + 8192 + 17
    base = np.arange(n, dtype=np.float64) * 0.5 - 3.0
    for pos in (0, 8192 + 5, 2 * 8192, n - 1):
        d = base.copy()
        d[pos] = np.nan
        assert np.isnan(to_np(K.max(_dev(d)))[0]) and np.isnan(to_np(K.min(_dev(d)))[0])
    e = torch.zeros(0, dtype=torch.float64, device="cuda")
    assert to_np(K.sum(e))[0] == 0 and to_np(K.prod(e))[0] == 1 and to_np(K.max(e))[0] == 0


def test_flat_i64_exact(K, ora):
    x = _data(np.int64, (3_000_001,), 4)
    xd = _dev(x)
    assert int(to_np(K.sum(xd))[0]) == int(ora.flat("sum", x))
    assert int(to_np(K.max(xd))[0]) == int(ora.flat("max", x))
    assert int(to_np(K.min(xd))[0]) == int(ora.flat("min", x))


def test_flat_noncontiguous_view(K, ora):
    x = _data(np.float32, (300, 700), 21)
    xd = _dev(x).t()
    got = float(to_np(K.sum(xd))[0])
    ref = float(ora.flat("sum", np.ascontiguousarray(x.T)))
    assert abs(got - ref) <= 1e-5 * float(np.abs(x).sum())


def test_generator_matches_host_twin(K):
    from numrs_gb300 import _lib as L
    from numrs_gb300 import rng
    t = torch.empty(100000, dtype=torch.int64, device="cuda")
    K.fill_random(t, L.RNG_INT, 4, -(1 << 20), float(1 << 21))
    np.testing.assert_array_equal(to_np(t), rng.int_range(4, 100000))
    u = torch.empty(100000, dtype=torch.float64, device="cuda")
    K.fill_random(u, L.RNG_UNIFORM, 1, -1.0, 1.0)
    np.testing.assert_array_equal(to_np(u), rng.uniform_pm1(1, 100000))


def test_large_c2_shape_properties(K):
    """16384 x 16384 f32 (the bench workload): axis sums agree with a
    float64 torch reduction within 1e-5 * sum|x|, bitwise between row-major
    and transposed views, and determinism run to run."""
    from numrs_gb300 import _lib as L
    x = torch.empty((16384, 16384), dtype=torch.float32, device="cuda")
    K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
    s0 = K.sum(x, axis=0)
    s0b = K.sum(x, axis=0)
    assert torch.equal(s0.view(torch.int32), s0b.view(torch.int32))
    st1 = K.sum(x.t(), axis=1)  # same lanes as axis 0 of x, same fold order
    assert torch.equal(s0.view(torch.int32), st1.view(torch.int32))
    ref = x.double().sum(0)
    scale = x.double().abs().sum(0)
    assert torch.all((s0.double() - ref).abs() <= 1e-5 * scale)
    m1 = K.max(x, axis=1)
    assert torch.equal(m1, x.max(1).values)
    del x


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", ["negatives", "zeros", "nans", "extremes"])
def test_extrema_bit_exact(K, ora, case, dtype):
    """Max / min: f64 on int64 keys (integer pipe), f32 on NaN-propagating
    chains, blocks with a NaN or a zero on the ordered fold; at 700 x 520
    both lane pipelines split the axis into parts combined in order. Both
    pipelines, the flattened partials and the ufunc reduce against the
    oracle bit for bit, on all-negative data (the extreme near zero), signed
    zeros, NaNs, and infinities / subnormals / the largest finite values."""
    r = np.random.default_rng({"negatives": 1, "zeros": 2, "nans": 3, "extremes": 4}[case])
    x = -np.abs(r.standard_normal((700, 520)))
    if case == "zeros":
        x[r.random(x.shape) < 0.004] = -0.0
        x[r.random(x.shape) < 0.004] = 0.0
    elif case == "nans":
        x[r.random(x.shape) < 0.001] = np.nan
    elif case == "extremes":
        tiny, big = (5e-324, 1.7976931348623157e308) if dtype == np.float64 else (1e-45, 3.4028235e38)
        for v in (-np.inf, np.inf, tiny, -tiny, big, -big):
            x[r.random(x.shape) < 0.002] = v
    x = x.astype(dtype)
    xd = _dev(x)
    for op in ("max", "min"):
        for axis in (0, 1):
            _check_axis(K, ora, x, op, axis)
            _check_axis(K, ora, x, op, axis, transposed=True)
        got = to_np(getattr(K, op)(xd))
        want = np.array([ora.flat(op, x)], dtype)
        assert np.isnan(got[0]) == np.isnan(want[0])
        if not np.isnan(want[0]):
            np.testing.assert_array_equal(bits(got), bits(want))
        ufn = "maximum" if op == "max" else "minimum"
        code = 11 if op == "max" else 12
        for axis in (0, 1):
            g = to_np(K.ufunc_reduce(ufn, xd, axis)).ravel()
            w = ora.ufunc_reduce(code, x, axis)
            nan = np.isnan(w)
            np.testing.assert_array_equal(np.isnan(g), nan)
            np.testing.assert_array_equal(bits(g[~nan]), bits(w[~nan]))
    for want_max, fn in ((True, K.argmax), (False, K.argmin)):
        for axis in (0, 1):
            np.testing.assert_array_equal(to_np(fn(xd, axis=axis)), ora.axis_arg(x, axis, want_max))
