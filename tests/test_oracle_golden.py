"""Pins the CPU oracle to the reference's own known answers (CPU only).

* Bit patterns pinned by tests/test_reduction_determinism.rs:126-197.
* NumPy goldens of tests/py/array_operations_reference_data.json (read by
  tests/test_array_operations_reference.rs, tolerance 1e-15).
* NaN-placement and empty-input conventions of src/kernels/reduce.rs:843-925,
  :578-589.
* GEMM against a double-double oracle on the size grid of
  src/kernels/gemm.rs:499-513.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def _x(dtype):
    n = GOLD["determinism"]["n"]
    return (np.arange(n, dtype=dtype) * dtype(0.5) - dtype(12345)).astype(dtype)


@pytest.mark.parametrize("name", sorted(GOLD["determinism"]["pins"]))
def test_determinism_pins(ora, name):
    pin = GOLD["determinism"]["pins"][name]
    if name == "sum_f32":
        got = np.float32(ora.flat("sum", _x(np.float32)))
    elif name == "sum_f64":
        got = np.float64(ora.flat("sum", _x(np.float64)))
    elif name == "mean_f64":
        got = np.float64(ora.flat("mean", _x(np.float64)))
    elif name == "var_f64_ddof0":
        got = np.float64(ora.flat("var", _x(np.float64), 0))
    else:
        got = np.sqrt(np.float64(ora.flat("var", _x(np.float64), 0)))
    width = {32: np.uint32, 64: np.uint64}[pin["width"]]
    assert int(np.array(got).view(width)) == pin["bits"]


def _arr(d):
    return np.array(d["data"], dtype=np.float64).reshape(d["shape"])


@pytest.mark.parametrize("key", sorted(GOLD["statistical_operations"]))
def test_numpy_stat_goldens(ora, key):
    case = GOLD["statistical_operations"][key]
    x = _arr(case["input"])
    op = case["operation"]
    axis = case["axis"]
    if axis is None:
        if op in ("var", "std"):
            got = ora.flat("var", x.ravel(), 0)
            if op == "std":
                got = np.sqrt(got)
        else:
            got = ora.flat(op, x.ravel())
        np.testing.assert_allclose(got, case["result"], rtol=1e-15, atol=1e-15)
    else:
        code = {"sum": O.SUM, "mean": O.MEAN, "max": O.MAX, "min": O.MIN}.get(op)
        if code is None:  # var/std(axis, ddof=0): math::statistics::var restated
            got = ora.axis_var(x, axis, ddof=0, std=(op == "std"))
        else:
            got = ora.axis(code, x, axis)
        np.testing.assert_allclose(got, _arr(case["result"]).ravel(), rtol=1e-15, atol=1e-15)


@pytest.mark.parametrize("key", sorted(GOLD["mathematical_functions"]))
def test_numpy_exp_goldens(ora, key):
    case = GOLD["mathematical_functions"][key]
    x = _arr(case["input"])
    got = ora.exp_affine(x.ravel(), 1.0, 0.0)
    np.testing.assert_allclose(got, _arr(case["result"]).ravel(), rtol=1e-15)


@pytest.mark.parametrize("key", sorted(GOLD["arithmetic_operations"]))
def test_numpy_arith_goldens(ora, key):
    case = GOLD["arithmetic_operations"][key]
    op = case["operation"].replace("scalar_", "")
    code = {"add": O.ADD, "subtract": O.SUB, "multiply": O.MUL, "divide": O.DIV}[op]
    a = _arr(case["input1"] if "input1" in case else case["input"])
    b = _arr(case["input2"]) if "input2" in case else np.array(case["scalar"], dtype=np.float64)
    got = ora.binary(code, a, b)
    np.testing.assert_allclose(got.ravel(), _arr(case["result"]).ravel(), rtol=1e-15)


def test_nan_placement(ora):
    for f in (np.float64, np.float32):
        assert np.isnan(ora.flat("min", np.array([1, np.nan, 3, -2, np.nan], f)))
        assert np.isnan(ora.flat("max", np.array([np.nan, 1, 2], f)))
        assert np.isnan(ora.flat("max", np.array([1, 2, np.nan], f)))
        assert ora.flat("min", np.array([np.inf, 1.0], f)) == 1.0
        assert ora.flat("max", np.array([-np.inf, 1.0], f)) == 1.0
        d = np.ones(64, f)
        d[0] = 5
        for pos in (0, 8, 10, 32, 63):
            e = d.copy()
            e[pos] = np.nan
            assert np.isnan(ora.flat("max", e)) and np.isnan(ora.flat("min", e))


def test_zero_ties_keep_the_first(ora):
    """The reference's min / max fold chunks with a strict compare and
    combines the chunk results in order (src/kernels/reduce.rs:335-364), so
    an extreme of zero keeps the sign of the first zero: the oracle must do
    the same, within one chunk and across the 8192-element chunk edge, for
    the flat and the axis folds."""
    for f in (np.float64, np.float32):
        for first, later in ((-0.0, 0.0), (0.0, -0.0)):
            for n, p0, p1 in ((10, 3, 7), (20000, 8190, 8195), (20000, 100, 16384)):
                x = -np.abs(np.random.default_rng(n).standard_normal(n)).astype(f) - 1
                x[p0], x[p1] = first, later
                assert np.signbit(ora.flat("max", x)) == np.signbit(f(first))
                assert np.signbit(ora.axis(O.MAX, x.reshape(-1, 1), 0)[0]) == np.signbit(f(first))
                y = -x
                y[p0], y[p1] = first, later
                assert np.signbit(ora.flat("min", y)) == np.signbit(f(first))
                assert np.signbit(ora.axis(O.MIN, y.reshape(-1, 1), 0)[0]) == np.signbit(f(first))


def test_empty_conventions(ora):
    e = np.zeros(0, np.float64)
    assert ora.flat("sum", e) == 0 and ora.flat("mean", e) == 0 and ora.flat("max", e) == 0
    assert ora.flat("prod", e) == 1 and ora.flat("var", e, 0) == 0


def test_ddof(ora):
    a = np.array([1, 2, 3, 4, 5], np.float64)
    assert abs(ora.flat("var", a, 0) - 2.0) < 1e-12
    assert abs(ora.flat("var", a, 1) - 2.5) < 1e-12


def test_axis_fold_is_left_to_right(ora):
    # f32 lane of values whose sum depends on order: the oracle must fold
    # left to right from 0 (src/math/aggregation.rs:555-561).
    x = np.array([[1e8], [1.0], [-1e8], [1.0]], np.float32)
    s = np.float32(0)
    for v in x[:, 0]:
        s = np.float32(s + v)
    assert ora.axis(O.SUM, x, 0)[0] == s


SIZE_GRID = [(1, 1, 1), (2, 2, 2), (31, 31, 31), (32, 32, 32), (33, 33, 33), (63, 63, 63),
             (64, 64, 64), (65, 65, 65), (127, 127, 127), (128, 128, 128), (0, 5, 4), (5, 0, 4),
             (5, 4, 0)]


@pytest.mark.parametrize("mkn", SIZE_GRID)
def test_gemm_oracle_vs_double_double(ora, mkn):
    m, k, n = mkn
    A = ora.gen_uniform_pm1(1, m * k).reshape(m, k)
    B = ora.gen_uniform_pm1(2, k * n).reshape(k, n)
    C = ora.gemm(A, B)
    Cdd, ab = ora.gemm_dd(A, B)
    if m * n:
        err = np.abs(C - Cdd) / np.maximum(ab, np.finfo(float).tiny)
        assert np.all(np.where(ab > 0, err, 0) <= 1e-14)
        if k == 0:
            assert np.all(C == 0)


def test_generator_twins(ora):
    # The numpy twin of SplitMix64 used by the host code matches the oracle.
    from numrs_gb300 import rng
    for seed in (1, 2, 3, 12825631960650228096):
        ref = np.array([ora.splitmix64_at(seed, i) for i in range(16)], dtype=np.uint64)
        assert np.array_equal(rng.splitmix64(seed, 16), ref)
    assert np.array_equal(rng.uniform_pm1(7, 1000), ora.gen_uniform_pm1(7, 1000))
    assert np.array_equal(rng.int_range(4, 1000), ora.gen_i64(4, 1000))


def test_argmax_argmin_reference_examples(ora):
    # The reference's own doc examples (src/math/statistics/mod.rs:64-77, :203-216).
    a = np.array([1.0, 3.0, 2.0, 4.0, 5.0, 1.0]).reshape(2, 3)
    assert list(ora.axis_arg(a, 1, True)) == [1, 1]
    assert list(ora.axis_arg(a, -1, True)) == [1, 1]
    assert list(ora.axis_arg(a, None, True)) == [4]
    b = np.array([5.0, 3.0, 2.0, 4.0, 1.0, 6.0]).reshape(2, 3)
    assert list(ora.axis_arg(b, 1, False)) == [2, 1]
    assert list(ora.axis_arg(b, None, False)) == [4]


def test_axis_var_ddof(ora):
    x = np.arange(12, dtype=np.float64).reshape(3, 4)
    np.testing.assert_allclose(ora.axis_var(x, 0, ddof=1), np.var(x, axis=0, ddof=1), rtol=1e-15)
    np.testing.assert_allclose(ora.axis_var(x, 1, ddof=0, std=True), np.std(x, axis=1), rtol=1e-15)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
def test_program_evaluator_matches_binary(ora, dtype):
    """The oracle's postfix-program evaluator agrees with its C binary ops
    (broadcast row, negative integers, zero divisors)."""
    r = np.random.default_rng(11)
    if dtype == np.int64:
        a = r.integers(-1000, 1000, (40, 30)).astype(dtype)
        b = r.integers(-7, 8, (30,)).astype(dtype)
    else:
        a = r.standard_normal((40, 30)).astype(dtype)
        b = r.standard_normal((30,)).astype(dtype)
    for code, op in ((2, O.ADD), (3, O.SUB), (4, O.MUL), (5, O.DIV)):
        p = ora.program([(0, 0, 0.0), (0, 1, 0.0), (code, 0, 0.0)], [a, b])
        c = ora.binary(op, a, b)
        np.testing.assert_array_equal(p.view(np.uint8), c.view(np.uint8))


# Known answers from the reference's own tests of ufunc reduce / accumulate
# (src/ufunc_ops.rs, test module from :932) and cumsum / cumprod
# (tests/test_stats_api_honesty.rs:90-150). Each row: (name, op code, input,
# shape, axis, initial, expected values in row-major order).
A23 = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
UFUNC_KATS = [
    ("reduce_add_axis_none", "reduce", 2, A23, (2, 3), None, None, [21.0]),
    ("reduce_add_axis0", "reduce", 2, A23, (2, 3), 0, None, [5.0, 7.0, 9.0]),
    ("reduce_add_axis1", "reduce", 2, A23, (2, 3), 1, None, [6.0, 15.0]),
    ("reduce_add_axis_neg1", "reduce", 2, A23, (2, 3), -1, None, [6.0, 15.0]),
    ("reduce_multiply_axis1", "reduce", 4, A23, (2, 3), 1, None, [6.0, 120.0]),
    ("reduce_maximum_axis0", "reduce", 11, A23, (2, 3), 0, None, [4.0, 5.0, 6.0]),
    ("reduce_minimum_axis1", "reduce", 12, A23, (2, 3), 1, None, [1.0, 4.0]),
    ("reduce_add_initial", "reduce", 2, A23, (2, 3), 1, 100.0, [106.0, 115.0]),
    ("reduce_multiply_initial", "reduce", 4, A23, (2, 3), 1, 2.0, [12.0, 240.0]),
    ("reduce_maximum_initial0", "reduce", 11, A23, (2, 3), 1, 0.0, [3.0, 6.0]),
    ("reduce_maximum_initial100", "reduce", 11, A23, (2, 3), 1, 100.0, [100.0, 100.0]),
    ("reduce_add_empty", "reduce", 2, [], (0,), None, None, [0.0]),
    ("reduce_multiply_empty", "reduce", 4, [], (0,), None, None, [1.0]),
    ("reduce_add_empty_initial", "reduce", 2, [], (0,), None, 5.0, [5.0]),
    ("reduce_maximum_empty_initial", "reduce", 11, [], (0,), None, 5.0, [5.0]),
    ("reduce_add_empty_lanes", "reduce", 2, [], (3, 0), 1, None, [0.0, 0.0, 0.0]),
    ("reduce_add_empty_lanes_initial", "reduce", 2, [], (3, 0), 1, 7.0, [7.0, 7.0, 7.0]),
    ("reduce_maximum_empty_lanes_initial", "reduce", 11, [], (3, 0), 1, 7.0, [7.0, 7.0, 7.0]),
    ("reduce_add_3d_axis_neg2", "reduce", 2, [float(i) for i in range(24)], (2, 3, 4), -2, None,
     [12.0, 15.0, 18.0, 21.0, 48.0, 51.0, 54.0, 57.0]),
    ("reduce_maximum_3d_axis_neg1", "reduce", 11, [float(i) for i in range(24)], (2, 3, 4), -1, None,
     [3.0, 7.0, 11.0, 15.0, 19.0, 23.0]),
    ("reduce_subtract_doc", "reduce", 3, [1.0, 2.0, 3.0], (3,), None, None, [-4.0]),
    ("accumulate_add", "accumulate", 2, [1.0, 2.0, 3.0, 4.0], (4,), None, None, [1.0, 3.0, 6.0, 10.0]),
    ("accumulate_multiply", "accumulate", 4, [1.0, 2.0, 3.0, 4.0], (4,), None, None, [1.0, 2.0, 6.0, 24.0]),
    ("accumulate_maximum", "accumulate", 11, [1.0, 3.0, 2.0, 5.0, 4.0], (5,), None, None,
     [1.0, 3.0, 3.0, 5.0, 5.0]),
    ("accumulate_minimum", "accumulate", 12, [5.0, 3.0, 4.0, 1.0, 2.0], (5,), None, None,
     [5.0, 3.0, 3.0, 1.0, 1.0]),
    ("accumulate_subtract", "accumulate", 3, [10.0, 1.0, 2.0, 3.0], (4,), None, None, [10.0, 9.0, 7.0, 4.0]),
    ("accumulate_divide", "accumulate", 5, [10.0, 1.0, 2.0, 3.0], (4,), None, None,
     [10.0, 10.0, 5.0, 5.0 / 3.0]),
    ("accumulate_maximum_axis1", "accumulate", 11, [1.0, 5.0, 2.0, 8.0, 1.0, 9.0], (2, 3), 1, None,
     [1.0, 5.0, 5.0, 8.0, 8.0, 9.0]),
    ("accumulate_minimum_axis0", "accumulate", 12, [1.0, 5.0, 2.0, 8.0, 1.0, 9.0], (2, 3), 0, None,
     [1.0, 5.0, 2.0, 1.0, 1.0, 2.0]),
    ("cumsum_axis1", "accumulate", 2, A23, (2, 3), 1, None, [1.0, 3.0, 6.0, 4.0, 9.0, 15.0]),
]
UFUNC_KAT_ERRORS = [  # reduce with no identity and no initial on an empty input
    ("reduce_maximum_empty", 11, (0,), None),
    ("reduce_minimum_empty", 12, (0,), None),
    ("reduce_maximum_empty_lanes", 11, (3, 0), 1),
]


@pytest.mark.parametrize("case", UFUNC_KATS, ids=[c[0] for c in UFUNC_KATS])
def test_ufunc_scan_known_answers_oracle(ora, case):
    _, kind, op, data, shape, axis, initial, want = case
    x = np.array(data, dtype=np.float64).reshape(shape)
    if kind == "reduce":
        got = ora.ufunc_reduce(op, x, axis, initial)
    else:
        got = ora.accumulate(op, x, axis)
    np.testing.assert_allclose(got.ravel(), want, rtol=1e-15, atol=0)


@pytest.mark.parametrize("case", UFUNC_KAT_ERRORS, ids=[c[0] for c in UFUNC_KAT_ERRORS])
def test_ufunc_scan_known_errors_oracle(ora, case):
    _, op, shape, axis = case
    with pytest.raises(ValueError):
        ora.ufunc_reduce(op, np.zeros(shape), axis, None)
