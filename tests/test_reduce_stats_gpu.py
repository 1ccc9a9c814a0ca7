"""Axis var/std(ddof) and argmax/argmin on the GPU vs the CPU oracle.

var/std follow math::statistics::var(axis) (per-lane mean, then the
left-to-right sum of (x - mean)^2): the GPU folds each lane in the same
order with each op rounded once, so results are compared bit for bit.
argmax/argmin are integer indices: exact.
"""
import numpy as np
import pytest
import torch

from numrs_gb300 import _lib as L
from tests.conftest import bits, to_np

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(3, 5), (64, 300), (1000, 333), (512, 2048), (300, 4100)])
@pytest.mark.parametrize("ddof", [0, 1])
def test_axis_var_std_bit_exact(K, ora, dtype, shape, ddof):
    x = np.random.default_rng(31).standard_normal(shape).astype(dtype) * 3 + 1
    xd = _dev(x)
    for axis in (0, 1):
        for view, xv in ((xd, x), (xd.t(), x.T)):
            got = to_np(K.var(view, axis=axis, ddof=ddof))
            ref = ora.axis_var(xv, axis, ddof=ddof)
            np.testing.assert_array_equal(bits(got), bits(ref))
            got = to_np(K.std(view, axis=axis, ddof=ddof))
            ref = ora.axis_var(xv, axis, ddof=ddof, std=True)
            np.testing.assert_array_equal(bits(got), bits(ref))


def test_axis_var_errors(K):
    import numrs_gb300 as N
    x = torch.ones((1, 5), device="cuda")
    with pytest.raises(N.InvalidOperation):
        K.var(x, axis=0, ddof=1)  # "Degrees of freedom 1 >= axis size 1"
    xi = torch.ones((3, 5), dtype=torch.int64, device="cuda")
    with pytest.raises(N.NumRs2Error):
        K.var(xi, axis=0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
@pytest.mark.parametrize("shape", [(2, 3), (64, 300), (1000, 333), (300, 4100)])
def test_argmax_argmin(K, ora, dtype, shape):
    r = np.random.default_rng(5)
    if dtype == np.int64:
        x = r.integers(-50, 50, shape).astype(np.int64)  # many ties: first index wins
    else:
        x = np.round(r.standard_normal(shape), 1).astype(dtype)
    xd = _dev(x)
    for want_max, fn in ((True, K.argmax), (False, K.argmin)):
        for axis in (0, 1, None):
            np.testing.assert_array_equal(to_np(fn(xd, axis=axis)), ora.axis_arg(x, axis, want_max))
            if axis is not None:
                np.testing.assert_array_equal(to_np(fn(xd.t(), axis=axis)), ora.axis_arg(x.T, axis, want_max))


def test_argmax_reference_examples_and_nan(K, ora):
    a = _dev(np.array([1.0, 3.0, 2.0, 4.0, 5.0, 1.0]).reshape(2, 3))
    assert to_np(K.argmax(a, axis=1)).tolist() == [1, 1]
    assert to_np(K.argmax(a)).tolist() == [4]
    x = np.random.default_rng(2).standard_normal(50_000)
    x[17] = np.nan
    x[40_000] = 99.0
    assert int(to_np(K.argmax(_dev(x)))[0]) == 40_000  # a NaN is never chosen ...
    x[0] = np.nan
    assert int(to_np(K.argmax(_dev(x)))[0]) == 0  # ... unless it is element 0
    assert int(to_np(K.argmin(_dev(x)))[0]) == ora.axis_arg(x, None, False)[0]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_argmax_axis_nan_and_zero_ties(K, ora, dtype):
    """Lane pipelines (axis length >= 256, >= 64 lanes): NaNs are skipped
    unless a lane starts with one, an all-NaN lane gives 0, and among equal
    extremes (+0.0 / -0.0 included) the first index wins."""
    r = np.random.default_rng(11)
    x = r.choice(np.array([-0.0, 0.0, -1.0, -2.0], dtype=dtype), (300, 4100))
    x[r.random(x.shape) < 0.01] = np.nan
    x[5, 0] = np.nan            # lane 5 along axis 1 starts with NaN
    x[:, 7] = np.nan            # column 7: an all-NaN lane along axis 0
    x[9, :] = np.nan            # row 9: an all-NaN lane along axis 1
    x[0, 3] = np.nan            # column 3 starts with NaN along axis 0
    xd = _dev(x)
    for want_max, fn in ((True, K.argmax), (False, K.argmin)):
        for axis in (0, 1):
            np.testing.assert_array_equal(to_np(fn(xd, axis=axis)), ora.axis_arg(x, axis, want_max))
            np.testing.assert_array_equal(to_np(fn(xd.t(), axis=axis)), ora.axis_arg(x.T, axis, want_max))


def test_argmax_large_flat(K, ora):
    x = np.random.default_rng(9).integers(-1000, 1000, 5_000_001).astype(np.int64)
    xd = _dev(x)
    assert int(to_np(K.argmax(xd))[0]) == ora.axis_arg(x, None, True)[0]
    assert int(to_np(K.argmin(xd))[0]) == ora.axis_arg(x, None, False)[0]
    _ = L.ARGMAX
