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


# ---------------------------------------------------------------------------
# Automatic slice count (slices = 0): the measured spread decides
# ---------------------------------------------------------------------------
def _ozaki_operands(K, m, k, n, phi, seeds=(5, 6)):
    A = torch.empty((m, k), dtype=torch.float64, device="cuda")
    B = torch.empty((k, n), dtype=torch.float64, device="cuda")
    K.fill_random(A, L.RNG_OZAKI, seeds[0], phi, 0.0)
    K.fill_random(B, L.RNG_OZAKI, seeds[1], phi, 0.0)
    return A, B


@pytest.mark.parametrize("phi", [0.0, 1.0, 4.0])
def test_ozaki_auto_count_full_oracle(K, ora, phi):
    """1024^3, entries U(-0.5,0.5)*exp(phi*N(0,1)): with the automatic count
    the componentwise error against the double-double product is at most
    1e-14 and no worse than the native FP64 GEMM's own."""
    A, B = _ozaki_operands(K, 1024, 1024, 1024, phi)
    C, info = K.gemm_ozaki(A, B)
    assert info["slices"] > 0, info
    Cdd, ab = ora.gemm_dd(to_np(A), to_np(B))
    e_oz = _err(to_np(C), Cdd, ab)
    e_dmma = _err(to_np(K.matmul(A, B, variant=L.GEMM_DMMA)), Cdd, ab)
    assert e_oz <= 1e-14, (phi, e_oz, e_dmma, info)
    assert e_oz <= max(e_dmma, 1e-15), (phi, e_oz, e_dmma, info)
    assert e_oz <= 4 * info["est_rel_error"], (e_oz, info)
    if phi == 0.0:
        assert info["slices"] == 7 and info["slice_bits"] == 8, info  # the fast case stays fast
    if phi == 4.0:
        assert info["slices"] >= 10, info


def test_ozaki_auto_count_sampled_4096(K, ora):
    """phi = 4 at 4096^3: 4096 random entries against double-double dots."""
    n = 4096
    A, B = _ozaki_operands(K, n, n, n, 4.0, seeds=(15, 16))
    C, info = K.gemm_ozaki(A, B)
    Cd = K.matmul(A, B, variant=L.GEMM_DMMA)
    r = np.random.default_rng(9)
    rows, cols = r.integers(0, n, 4096), r.integers(0, n, 4096)
    ref, ab = ora.gemm_dd_sampled(to_np(A), to_np(B), rows, cols)
    e_oz = float(np.max(np.abs(to_np(C)[rows, cols] - ref) / ab))
    e_dmma = float(np.max(np.abs(to_np(Cd)[rows, cols] - ref) / ab))
    assert e_oz <= 1e-14 and e_oz <= max(e_dmma, 1e-15), (e_oz, e_dmma, info)


def test_ozaki_auto_identity_second_pass(K):
    """I * I: every off-diagonal |A'||B'| is 0 while the row sums are not,
    so the second pass (counting only k with a nonzero partner) sets the
    count; the product is exact and the tensor cores still run it."""
    n = 300
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    C, info = K.gemm_ozaki(eye, eye)
    assert info["slices"] > 0, info
    assert torch.equal(C, eye)
    # block-diagonal operands: the same structure with random blocks
    A = torch.zeros((256, 256), dtype=torch.float64, device="cuda")
    B = torch.zeros_like(A)
    a = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, (128, 128))).cuda()
    b = torch.from_numpy(np.random.default_rng(4).uniform(-1, 1, (128, 128))).cuda()
    A[:128, :128] = a
    A[128:, 128:] = a
    B[:128, :128] = b
    B[128:, 128:] = b
    C, info = K.gemm_ozaki(A, B)
    assert info["slices"] > 0, info
    assert torch.all(C[:128, 128:] == 0) and torch.all(C[128:, :128] == 0)


def test_ozaki_auto_falls_back_to_fp64(K):
    """Operands whose magnitudes that meet in a dot product are ~2^660 apart,
    or that hold Inf / NaN, run the native FP64 GEMM (slices = 0 reported),
    bit for bit the DMMA result."""
    A = torch.tensor([[1.0, 1e-200], [2.0, 3.0]], dtype=torch.float64, device="cuda")
    B = torch.tensor([[1e-200, 0.5], [1.0, 0.25]], dtype=torch.float64, device="cuda")
    C, info = K.gemm_ozaki(A, B)
    assert info["slices"] == 0, info
    assert torch.equal(C, K.matmul(A, B, variant=L.GEMM_DMMA))
    A2 = torch.ones((64, 64), dtype=torch.float64, device="cuda")
    A2[3, 5] = float("inf")
    A2[7, 1] = float("nan")
    C, info = K.gemm_ozaki(A2, A2)
    assert info["slices"] == 0
    Cd = K.matmul(A2, A2, variant=L.GEMM_DMMA)
    assert torch.equal(torch.isnan(C), torch.isnan(Cd)) and torch.equal(C[~torch.isnan(C)], Cd[~torch.isnan(Cd)])


def test_ozaki_transposed_views_and_accumulate(K, ora):
    """Transposed operand views go through the column slicers without a
    copy; NRS_GEMM_ACCUMULATE adds the rounded product to C."""
    m, k, n = 200, 333, 150
    At = torch.from_numpy(ora.gen_uniform_pm1(21, m * k).reshape(k, m)).cuda()  # A = At.T
    Bt = torch.from_numpy(ora.gen_uniform_pm1(22, k * n).reshape(n, k)).cuda()  # B = Bt.T
    A, B = At.t(), Bt.t()
    Cdd, ab = ora.gemm_dd(to_np(A), to_np(B))
    for a, b in ((A, B), (A.contiguous(), B), (A, B.contiguous())):
        C, info = K.gemm_ozaki(a, b)
        assert _err(to_np(C), Cdd, ab) <= 1e-15, info
    C0 = torch.full((m, n), 1.0, dtype=torch.float64, device="cuda")
    C, _ = K.gemm_ozaki(A, B, out=C0, accumulate=True)
    assert C is C0
    want = 1.0 + to_np(K.gemm_ozaki(A, B)[0])
    np.testing.assert_array_equal(to_np(C0), want)


# ---------------------------------------------------------------------------
# Grouped tensor-core f64 GEMMs (nrs_gemm_ozaki_grouped, plan f64 mode OZAKI)
# ---------------------------------------------------------------------------
def _group_problems(seed, count, hi=512):
    r = np.random.default_rng(seed)
    lu = lambda lo, hi_, n: np.exp(r.uniform(np.log(lo), np.log(hi_), n)).astype(np.int64)  # noqa: E731
    M, N, Kk = lu(1, hi, count), lu(1, hi, count), lu(1, hi, count)
    probs = []
    for i in range(count):
        a = torch.from_numpy(r.uniform(-1, 1, (M[i], Kk[i]))).cuda()
        b = torch.from_numpy(r.uniform(-1, 1, (Kk[i], N[i])) * np.exp(r.normal(0, 1, (Kk[i], N[i])))).cuda()
        c = torch.full((M[i], N[i]), float("nan"), dtype=torch.float64, device="cuda")
        probs.append((a, b, c, False))
    return probs


def _check_against_dd(ora, K, probs, bar=1e-14):
    for a, b, c, _ in probs:
        Cdd, ab = ora.gemm_dd(to_np(a), to_np(b))
        e = _err(to_np(c), Cdd, ab)
        ed = _err(to_np(K.matmul(a, b, variant=L.GEMM_DMMA)), Cdd, ab)
        assert e <= bar and e <= max(ed, 1e-15), (a.shape, b.shape, e, ed)


def test_ozaki_grouped_against_double_double(K, ora):
    probs = _group_problems(41, 60)
    # a transposed A, a long K and a NaN: the first and last go to DMMA
    at = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, (70, 50))).cuda()
    probs.append((at.t(), torch.rand((70, 33), dtype=torch.float64, device="cuda"),
                  torch.empty((50, 33), dtype=torch.float64, device="cuda"), False))
    probs.append((torch.rand((40, 3000), dtype=torch.float64, device="cuda") - 0.5,
                  torch.rand((3000, 90), dtype=torch.float64, device="cuda") - 0.5,
                  torch.empty((40, 90), dtype=torch.float64, device="cuda"), False))
    bad = torch.rand((16, 16), dtype=torch.float64, device="cuda")
    bad[3, 4] = float("nan")
    probs.append((bad, bad.clone(), torch.empty((16, 16), dtype=torch.float64, device="cuda"), False))
    on_tc, info = K.gemm_ozaki_grouped(probs)
    assert info["slices"] >= 7 and all(on_tc[:60]) and on_tc[61] and not on_tc[60] and not on_tc[62]
    _check_against_dd(ora, K, probs[:62])
    d = K.matmul(bad, bad.clone(), variant=L.GEMM_DMMA)
    assert torch.equal(torch.isnan(probs[62][2]), torch.isnan(d))


def test_plan_f64_on_tensor_cores_replays_and_accumulates(K, ora):
    probs = _group_problems(43, 40, hi=300)
    x = [torch.randn(int(n), device="cuda") for n in (100, 5000, 70000)]
    reds = [(v, L.SUM, torch.empty(1, device="cuda")) for v in x]
    f32 = [(torch.rand((50, 60), device="cuda"), torch.rand((60, 70), device="cuda"),
            torch.empty((50, 70), device="cuda"), False)]
    plan = K.Plan(probs + f32, reds, f64_mode=L.PLAN_F64_OZAKI)
    n_tc, S, bits = plan.f64_info()
    assert n_tc == 40 and S >= 7 and bits in (6, 7, 8)
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    _check_against_dd(ora, K, probs)
    for v, _, o in reds:
        assert torch.equal(o.reshape(()), K.sum(v).reshape(()))
    # new values of the same range: the replayed graph picks them up
    for a, b, c, _ in probs:
        a.mul_(-0.5)
        c.fill_(float("nan"))
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    _check_against_dd(ora, K, probs)
    plan.close()
    # C += A B through the grouped path
    accp = [(a, b, torch.ones_like(c), True) for a, b, c, _ in probs[:8]]
    plan = K.Plan(accp, f64_mode=L.PLAN_F64_OZAKI, f64_slices=8)
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    for a, b, c, _ in accp:
        Cdd, ab = ora.gemm_dd(to_np(a), to_np(b))
        assert np.max(np.abs(to_np(c) - (Cdd + 1.0)) / (ab + 1.0)) <= 1e-14
    plan.close()


@pytest.mark.parametrize("bits,slices", [(8, 1), (8, 3), (7, 3), (6, 5)])
def test_ozaki_grouped_integer_known_answer(K, bits, slices):
    """Grouped launches carry the diagonal sums through int32 R with one
    retired digit per diagonal. Integers |x| <= 4096 need two 8- or 7-bit
    digits (three 6-bit ones), so every nonzero slice product is among the
    computed pairs and C must equal the exact integer product bit for bit;
    random signs exercise negative carries. slices = 1 uses |x| <= 3."""
    r = np.random.default_rng(11 + bits + slices)
    lim = 3 if slices == 1 else 4096
    shapes = [(1, 7, 1), (129, 65, 257), (40, 1000, 300), (300, 33, 17), (128, 128, 128), (17, 700, 130)]
    probs, exact = [], []
    for m, k, n in shapes:
        A = r.integers(-lim, lim + 1, (m, k))
        B = r.integers(-lim, lim + 1, (k, n))
        exact.append((A @ B).astype(np.float64))
        probs.append((_dev(A.astype(np.float64)), _dev(B.astype(np.float64)),
                      torch.full((m, n), float("nan"), dtype=torch.float64, device="cuda"), False))
    plan = K.Plan(probs, f64_mode=L.PLAN_F64_OZAKI, f64_slices=slices, f64_digit_bits=bits)
    assert plan.f64_info() == (len(shapes), slices, bits)
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    for (_, _, c, _), e in zip(probs, exact):
        np.testing.assert_array_equal(to_np(c), e)
    plan.close()


@pytest.mark.parametrize("bits,slices", [(8, 12), (7, 10), (6, 14), (7, 9)])
def test_ozaki_grouped_digit_widths(K, ora, bits, slices):
    """Every digit width, 8-byte (S <= 9) and 16-byte digit records, and a
    K of 3000 (three exact K chunks at b = 8), against double-double. Each
    count carries at least 63 bits: these operands' spread needs more than
    the 53 of a spread-free product."""
    probs = _group_problems(53, 24)
    probs.append((torch.rand((40, 3000), dtype=torch.float64, device="cuda") - 0.5,
                  torch.rand((3000, 90), dtype=torch.float64, device="cuda") - 0.5,
                  torch.empty((40, 90), dtype=torch.float64, device="cuda"), False))
    plan = K.Plan(probs, f64_mode=L.PLAN_F64_OZAKI, f64_slices=slices, f64_digit_bits=bits)
    assert plan.f64_info() == (len(probs), slices, bits)
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    _check_against_dd(ora, K, probs)
    plan.close()


# ---------------------------------------------------------------------------
# f32 GEMMs on the tensor cores (plan option f32_mode = PLAN_F32_OZAKI)
# ---------------------------------------------------------------------------
def _f32_problems(seed, count, hi=512, phi=0.0):
    r = np.random.default_rng(seed)
    lu = lambda lo, hi_, n: np.exp(r.uniform(np.log(lo), np.log(hi_), n)).astype(np.int64)  # noqa: E731
    M, N, Kk = lu(1, hi, count), lu(1, hi, count), lu(1, hi, count)
    probs = []
    for i in range(count):
        a = r.uniform(-1, 1, (M[i], Kk[i])) * np.exp(phi * r.normal(0, 1, (M[i], Kk[i])))
        b = r.uniform(-1, 1, (Kk[i], N[i])) * np.exp(phi * r.normal(0, 1, (Kk[i], N[i])))
        probs.append((_dev(a.astype(np.float32)), _dev(b.astype(np.float32)),
                      torch.full((M[i], N[i]), float("nan"), dtype=torch.float32, device="cuda"), False))
    return probs


def test_plan_f32_on_tensor_cores_integer_known_answer(K):
    """Integers |x| <= 64 with K <= 1000: every product sum is an integer
    below 2^24, exact in f32, so C must equal it bit for bit."""
    r = np.random.default_rng(21)
    shapes = [(1, 7, 1), (129, 65, 257), (40, 1000, 300), (300, 33, 17), (128, 128, 128)]
    probs, exact = [], []
    for m, k, n in shapes:
        A = r.integers(-64, 65, (m, k))
        B = r.integers(-64, 65, (k, n))
        exact.append((A @ B).astype(np.float32))
        probs.append((_dev(A.astype(np.float32)), _dev(B.astype(np.float32)),
                      torch.full((m, n), float("nan"), dtype=torch.float32, device="cuda"), False))
    plan = K.Plan(probs, f32_mode=L.PLAN_F32_OZAKI)
    n_tc, S, bits = plan.f32_info()
    assert n_tc == len(shapes) and S >= 3 and bits in (6, 7, 8)
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    for (_, _, c, _), e in zip(probs, exact):
        np.testing.assert_array_equal(to_np(c), e)
    plan.close()


@pytest.mark.parametrize("phi", [0.0, 2.0])
def test_plan_f32_on_tensor_cores_accuracy(K, ora, phi):
    """Against the double-double product of the f32 operands: the error stays
    at f32 rounding (componentwise <= 2^-23 of (|A||B|)_ij), at most the
    FMA tiles' own error, with magnitudes spread by exp(phi N(0,1))."""
    probs = _f32_problems(31, 40, phi=phi)
    probs.append((_dev(np.random.default_rng(2).uniform(-1, 1, (40, 3000)).astype(np.float32)),
                  _dev(np.random.default_rng(3).uniform(-1, 1, (3000, 90)).astype(np.float32)),
                  torch.empty((40, 90), dtype=torch.float32, device="cuda"), False))
    fma = [(a, b, torch.empty_like(c), acc) for a, b, c, acc in probs]
    plan = K.Plan(probs, f32_mode=L.PLAN_F32_OZAKI)
    assert plan.f32_info()[0] == len(probs)
    plan.run(use_graph=True)
    ref = K.Plan(fma)
    ref.run(use_graph=False)
    torch.cuda.synchronize()
    for (a, b, c, _), (_, _, cf, _) in zip(probs, fma):
        A64, B64 = to_np(a).astype(np.float64), to_np(b).astype(np.float64)
        Cdd, ab = ora.gemm_dd(A64, B64)
        e = _err(to_np(c).astype(np.float64), Cdd, ab)
        ef = _err(to_np(cf).astype(np.float64), Cdd, ab)
        assert e <= 2.0 ** -23 and e <= max(ef, 2.0 ** -24), (a.shape, b.shape, e, ef)
    plan.close()
    ref.close()


def test_plan_f32_and_f64_on_tensor_cores_together(K, ora):
    """Both groups in one plan with reductions, a NaN-holding f32 problem on
    the FMA tiles, replayed from the graph after the inputs change."""
    p64 = _group_problems(61, 12, hi=300)
    p32 = _f32_problems(62, 12, hi=300)
    bad = torch.rand((16, 16), device="cuda")
    bad[2, 3] = float("nan")
    p32.append((bad, bad.clone(), torch.empty((16, 16), device="cuda"), False))
    x = [torch.randn(int(n), device="cuda") for n in (100, 70000)]
    reds = [(v, L.SUM, torch.empty(1, device="cuda")) for v in x]
    plan = K.Plan(p64 + p32, reds, f64_mode=L.PLAN_F64_OZAKI, f32_mode=L.PLAN_F32_OZAKI)
    assert plan.f64_info()[0] == 12 and plan.f32_info()[0] == 12
    for step in range(2):
        if step:
            for a, b, c, _ in p64 + p32[:12]:
                a.mul_(-0.5)
                c.fill_(float("nan"))
        plan.run(use_graph=True)
        torch.cuda.synchronize()
        _check_against_dd(ora, K, p64)
        for a, b, c, _ in p32[:12]:
            Cdd, ab = ora.gemm_dd(to_np(a).astype(np.float64), to_np(b).astype(np.float64))
            assert _err(to_np(c).astype(np.float64), Cdd, ab) <= 2.0 ** -23
        assert torch.isnan(p32[12][2]).any()
        for v, _, o in reds:
            assert torch.equal(o.reshape(()), K.sum(v).reshape(()))
    plan.close()


def test_autotune_considers_tensor_core_f64(K, ora):
    probs = _group_problems(47, 80)
    f32 = []
    for i in range(40):
        m, k, n = 32 + i, 64, 48 + i
        f32.append((torch.rand((m, k), device="cuda"), torch.rand((k, n), device="cuda"),
                    torch.empty((m, n), device="cuda"), False))
    K.tuner_clear()
    rep = K.autotune_plan(probs + f32, (), max_trials=8, reps=3, f64_ozaki=True, f32_ozaki=True)
    assert rep["final_ms"] <= rep["untuned_ms"]
    assert rep["ozaki_ms"] > 0 and rep["ozaki_f32_ms"] > 0
    assert set(rep["plan_kwargs"]) == {"f64_mode", "f64_slices", "f64_digit_bits", "f32_mode"}
    for a, b, c, _ in probs + f32:
        c.fill_(float("nan"))
    plan = K.Plan(probs + f32, (), **rep["plan_kwargs"])
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    _check_against_dd(ora, K, probs[:20])
    for a, b, c, _ in f32[:10]:
        Cdd, ab = ora.gemm_dd(to_np(a).astype(np.float64), to_np(b).astype(np.float64))
        assert _err(to_np(c).astype(np.float64), Cdd, ab) <= 1e-5
    plan.close()
    K.tuner_clear()
