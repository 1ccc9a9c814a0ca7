"""Elementwise ufuncs on the GPU vs the CPU oracle.

Add/sub/mul/div with broadcasting are bit-exact (one IEEE rounding each).
exp uses CUDA's exp/expf and the oracle the host libm, so exp results are
compared within 2 ulp (f32) / 1e-15 relative (f64); the affine part before
the exp is two roundings on both sides (never an FMA).
"""
import json
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.conftest import bits, to_np

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _ulp_diff_f32(a, b):
    ai = a.view(np.int32).astype(np.int64)
    bi = b.view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7FFFFFFF), ai)
    bi = np.where(bi < 0, -(bi & 0x7FFFFFFF), bi)
    return np.abs(ai - bi)


@pytest.mark.parametrize("n", [1, 3, 4, 5, 1000, 4097, 1 << 20, (1 << 22) + 3])
def test_exp_affine_f32(K, ora, n):
    x = np.random.default_rng(n).standard_normal(n).astype(np.float32)
    got = to_np(K.exp_affine(_dev(x), 0.5, -0.25))
    ref = ora.exp_affine(x, 0.5, -0.25)
    assert _ulp_diff_f32(got, ref).max() <= 2
    # the argument of exp is bit-identical (two roundings, no FMA)
    t = (x * np.float32(0.5)).astype(np.float32) + np.float32(-0.25)
    np.testing.assert_allclose(got, np.exp(t.astype(np.float64)), rtol=3e-7)


def test_exp_affine_f64_and_eager_equivalence(K, ora):
    x = np.random.default_rng(1).standard_normal(100003)
    got = to_np(K.exp_affine(_dev(x), 0.5, -0.25))
    np.testing.assert_allclose(got, ora.exp_affine(x, 0.5, -0.25), rtol=1e-15)
    # fused program == eager three-pass spelling
    xf = _dev(x.astype(np.float32))
    eager = K.exp(K.add(K.multiply(xf, torch.tensor(0.5, device="cuda")),
                        torch.tensor(-0.25, device="cuda")))
    fused = (K.Expr.leaf(xf) * 0.5 + (-0.25)).exp().eval()
    assert torch.equal(eager.view(torch.int32), fused.view(torch.int32))


def test_exp_affine_unaligned_and_strided(K, ora):
    x = np.random.default_rng(2).standard_normal(5001).astype(np.float32)
    xd = _dev(x)
    got = to_np(K.exp_affine(xd[1:], 0.5, -0.25))  # 4-byte aligned only
    assert _ulp_diff_f32(got, ora.exp_affine(x[1:], 0.5, -0.25)).max() <= 2
    x2 = np.random.default_rng(3).standard_normal((70, 90)).astype(np.float32)
    got = to_np(K.exp_affine(_dev(x2).t(), 0.5, -0.25))
    assert _ulp_diff_f32(got.ravel(), ora.exp_affine(np.ascontiguousarray(x2.T), 0.5, -0.25).ravel()).max() <= 2


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
@pytest.mark.parametrize("shapes", [((5,), (5,)), ((3, 4), (4,)), ((3, 1), (1, 4)), ((2, 3, 4), (3, 1)),
                                    ((1000, 257), (257,))])
@pytest.mark.parametrize("op", ["add", "subtract", "multiply", "divide"])
def test_broadcast_binary_bit_exact(K, ora, dtype, shapes, op):
    r = np.random.default_rng(7)
    if dtype == np.int64:
        a = r.integers(-1000, 1000, shapes[0]).astype(np.int64)
        b = r.integers(1, 50, shapes[1]).astype(np.int64)
    else:
        a = r.standard_normal(shapes[0]).astype(dtype)
        b = r.standard_normal(shapes[1]).astype(dtype)
    got = to_np(getattr(K, op)(_dev(a), _dev(b)))
    code = {"add": O.ADD, "subtract": O.SUB, "multiply": O.MUL, "divide": O.DIV}[op]
    ref = ora.binary(code, a, b)
    np.testing.assert_array_equal(bits(got.ravel()), bits(ref.ravel()))


def test_expr_trees(K):
    r = np.random.default_rng(9)
    a, b, c = (r.standard_normal((64, 33)).astype(np.float32) for _ in range(3))
    A, B, Cc = _dev(a), _dev(b), _dev(c)
    E = K.Expr.leaf
    got = to_np(((E(A) * E(B)) + E(Cc)).eval())
    ref = (a * b).astype(np.float32) + c  # two roundings
    np.testing.assert_array_equal(bits(got), bits(ref.astype(np.float32)))
    got = to_np((2.0 - E(A) / 3.0).abs().sqrt().eval())
    ref = np.sqrt(np.abs(np.float32(2.0) - (a / np.float32(3.0)).astype(np.float32)))
    np.testing.assert_allclose(got, ref, rtol=1e-6)


def test_program_validation(K):
    import numrs_gb300 as N
    from numrs_gb300 import _lib as L
    x = torch.ones(4, device="cuda")
    with pytest.raises(N.NumRs2Error):
        K.run_program([(L.OP_ADD, 0, 0.0)], [x])  # stack underflow
    with pytest.raises(N.NumRs2Error):
        K.run_program([(L.OP_INPUT, 3, 0.0)], [x])  # missing input
    xi = torch.ones(4, dtype=torch.int64, device="cuda")
    with pytest.raises(N.NumRs2Error):
        K.exp(xi)


GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


@pytest.mark.parametrize("key", sorted(GOLD["mathematical_functions"]))
def test_exp_goldens(K, key):
    case = GOLD["mathematical_functions"][key]
    x = np.array(case["input"]["data"], np.float64)
    got = to_np(K.exp(_dev(x)))
    np.testing.assert_allclose(got, case["result"]["data"], rtol=1e-15)


@pytest.mark.parametrize("key", sorted(GOLD["arithmetic_operations"]))
def test_arith_goldens(K, key):
    case = GOLD["arithmetic_operations"][key]
    op = case["operation"].replace("scalar_", "")
    a = np.array(case["input1" if "input1" in case else "input"]["data"], np.float64)
    a = a.reshape(case["input1" if "input1" in case else "input"]["shape"])
    if "input2" in case:
        b = np.array(case["input2"]["data"], np.float64).reshape(case["input2"]["shape"])
    else:
        b = np.array(case["scalar"], np.float64)
    got = to_np(getattr(K, op)(_dev(a), _dev(b)))
    np.testing.assert_allclose(got.ravel(), case["result"]["data"], rtol=1e-15)


def _random_program(r, n_inputs, n_leaves, dt_kind):
    """A random expression tree in postfix form. Trees lean right half the
    time so the stack reaches the number of leaves (up to 8)."""
    ops = [2, 3, 4, 5, 11, 12]

    def leaf():
        if r.random() < 0.2:
            s = float(r.integers(-5, 6)) if dt_kind != "f" else float(r.standard_normal())
            return [(1, 0, s)]
        return [(0, int(r.integers(0, n_inputs)), 0.0)]

    def tree(nl, right_deep):
        if nl == 1:
            t = leaf()
        else:
            k = 1 if right_deep else int(r.integers(1, nl))
            t = tree(k, right_deep) + tree(nl - k, right_deep) + [(int(r.choice(ops)), 0, 0.0)]
        if r.random() < 0.15:
            t = t + [(int(r.choice([6, 7])), 0, 0.0)]
        return t

    return tree(n_leaves, bool(r.random() < 0.5))


def _depth(prog):
    d = m = 0
    for code, _, _ in prog:
        d += 1 if code in (0, 1) else (0 if code in (6, 7, 8, 9, 10) else -1)
        m = max(m, d)
    return m


def _same_or_both_nan(got, ref):
    got, ref = np.ascontiguousarray(got), np.ascontiguousarray(ref)
    if got.dtype.kind == "f":
        nan = np.isnan(ref)
        np.testing.assert_array_equal(np.isnan(got), nan)
        np.testing.assert_array_equal(bits(got[~nan]), bits(ref[~nan]))
    else:
        np.testing.assert_array_equal(got, ref)


# (input shapes, view): same-shape contiguous -> flat vectors; an aligned
# broadcast row / column -> vector rows; odd widths and transposed views ->
# scalar rows or the full decode.
PROGRAM_CASES = [
    ([(300, 256)] * 4, None),
    ([(300, 256), (256,), (300, 1), (1, 256)], None),
    ([(64, 8, 128), (8, 1), (64, 1, 128), (128,)], None),
    ([(37, 65), (65,), (37, 1), (37, 65)], None),
    ([(33, 70)] * 4, "t"),
    ([(5000,)] * 4, None),
]


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
@pytest.mark.parametrize("case", range(len(PROGRAM_CASES)))
def test_random_programs_bit_exact(K, ora, dtype, case):
    """Random postfix programs of stack depth 1..8 over 1..4 broadcast inputs
    through every access path, bit-exact against the oracle's evaluation."""
    shapes, view = PROGRAM_CASES[case]
    r = np.random.default_rng(100 + case)
    kind = np.dtype(dtype).kind
    if kind == "f":
        arrs = [r.standard_normal(s).astype(dtype) for s in shapes]
    else:
        arrs = [r.integers(-1000, 1000, s).astype(dtype) for s in shapes]
    devs = [_dev(a) for a in arrs]
    if view == "t":  # transposed views of (70, 33) buffers
        arrs = [np.ascontiguousarray(a.T).T for a in arrs]
        devs = [_dev(np.ascontiguousarray(a.T)).t() for a in arrs]
    seen = set()
    for trial in range(24):
        n_in = int(r.integers(1, 5))
        prog = _random_program(r, n_in, int(r.integers(1, 9)), kind)
        if _depth(prog) > 8:
            continue
        seen.add(_depth(prog))
        got = to_np(K.run_program(prog, devs[:n_in]))
        ref = ora.program(prog, arrs[:n_in])
        _same_or_both_nan(got, ref)
    assert max(seen) >= 5 and min(seen) <= 2  # shallow and deep stacks both ran
