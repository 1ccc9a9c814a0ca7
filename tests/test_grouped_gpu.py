"""Grouped persistent launch, autotuner and learned selector on the GPU.

* Grouped GEMM tiles run the standalone kernels' tile bodies, so unsplit
  results equal nrs_gemm's bit for bit; split-K results are checked against
  the double-double oracle. Grouped row reductions equal nrs_reduce's flat
  reductions bit for bit.
* CUDA-graph replays pick up new input values.
* The MLP selector's GPU gradients match the CPU oracle's restatement.
"""
import numpy as np
import pytest
import torch

from numrs_gb300 import _lib as L
from tests.conftest import bits, to_np

pytestmark = pytest.mark.gpu


def _logu(r, lo, hi, n):
    return np.exp(r.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)


def _problems(seed, n_gemm, n_red, hi=256):
    r = np.random.default_rng(seed)
    gemms, reds = [], []
    M, N, Kk = _logu(r, 16, hi, n_gemm), _logu(r, 16, hi, n_gemm), _logu(r, 16, hi, n_gemm)
    for i in range(n_gemm):
        dt = torch.float32 if i % 2 == 0 else torch.float64
        a = torch.empty((M[i], Kk[i]), dtype=dt, device="cuda").uniform_(-1, 1)
        b = torch.empty((Kk[i], N[i]), dtype=dt, device="cuda").uniform_(-1, 1)
        c = torch.full((M[i], N[i]), float("nan"), dtype=dt, device="cuda")
        gemms.append((a, b, c, False))
    lens = _logu(r, 64, 65536, n_red)
    for i in range(n_red):
        dt = [torch.float32, torch.float64, torch.int64][i % 3]
        if dt == torch.int64:
            x = torch.randint(-1 << 20, 1 << 20, (int(lens[i]),), device="cuda")
        else:
            x = torch.randn(int(lens[i]), dtype=dt, device="cuda")
        op = [L.SUM, L.MEAN, L.MAX, L.MIN][i % 4]
        out_dt = torch.float64 if (dt == torch.int64 and op == L.MEAN) else dt
        reds.append((x, op, torch.empty(1, dtype=out_dt, device="cuda")))
    return gemms, reds


def test_grouped_matches_individual_and_oracle(K, ora):
    gemms, reds = _problems(7, 120, 90)
    plan = K.Plan(gemms, reds)
    st = plan.stats()
    assert st["work_items"] >= 120 + 90
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    for a, b, c, _ in gemms:
        m, k = a.shape
        n = b.shape[1]
        variant = L.GEMM_DMMA if a.dtype == torch.float64 else L.GEMM_SIMT
        ref = K.matmul(a, b, variant=variant)
        got = c
        if a.dtype == torch.float64:
            Cdd, ab = ora.gemm_dd(to_np(a), to_np(b))
            err = np.max(np.abs(to_np(got) - Cdd) / ab)
            assert err <= 1e-14
        else:
            Cdd, ab = ora.gemm_dd(to_np(a).astype(np.float64), to_np(b).astype(np.float64))
            err = np.max(np.abs(to_np(got).astype(np.float64) - Cdd) / ab)
            assert err <= 1e-5
        # Unsplit f32 tiles: identical arithmetic to the plain SIMT GEMM. (The
        # plain f64 DMMA GEMM may split k to fill the GPU, so f64 is held to
        # the double-double bound above.)
        if a.dtype == torch.float32 and k < 8 * max(m, n):
            assert torch.equal(got.view(torch.int64 if a.dtype == torch.float64 else torch.int32),
                               ref.view(torch.int64 if a.dtype == torch.float64 else torch.int32))
    for x, op, out in reds:
        ref = K.reduce(x, op)
        np.testing.assert_array_equal(bits(to_np(out)), bits(to_np(ref)))


def test_grouped_graph_replay_sees_new_inputs(K):
    gemms, reds = _problems(9, 40, 30, hi=128)
    plan = K.Plan(gemms, reds)
    plan.run(use_graph=True)
    first = [c.clone() for _, _, c, _ in gemms]
    for a, _, _, _ in gemms:
        a.mul_(2.0)
    for x, _, _ in reds:
        x.copy_(x * 2) if x.dtype != torch.int64 else x.mul_(2)
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    for (a, b, c, _), c0 in zip(gemms, first):
        assert torch.allclose(c, 2 * c0, rtol=1e-5 if c.dtype == torch.float32 else 1e-12, atol=1e-4)
    for x, op, out in reds:
        assert torch.equal(to_np_t(out), to_np_t(K.reduce(x, op)))
    plan.close()


def to_np_t(t):
    return t.view(torch.int64) if t.element_size() == 8 else t.view(torch.int32)


def test_split_k_and_accumulate(K, ora):
    a = torch.empty((40, 3000), dtype=torch.float64, device="cuda").uniform_(-1, 1)
    b = torch.empty((3000, 24), dtype=torch.float64, device="cuda").uniform_(-1, 1)
    c = torch.ones((40, 24), dtype=torch.float64, device="cuda")
    K.tuner_set(L.F64, 40, 3000, 24, 5)  # force the split-K variant for this bucket
    plan = K.Plan([(a, b, c, True)])
    for _ in range(3):  # counters reset correctly between replays
        c.fill_(1.0)
        plan.run(use_graph=True)
        torch.cuda.synchronize()
        Cdd, ab = ora.gemm_dd(to_np(a), to_np(b))
        assert np.max(np.abs(to_np(c) - 1.0 - Cdd) / ab) <= 1e-14
    K.tuner_clear()
    plan.close()


def test_transposed_grouped(K):
    a = torch.randn(70, 50, dtype=torch.float64, device="cuda")
    b = torch.randn(90, 70, dtype=torch.float64, device="cuda")
    c = torch.empty((50, 90), dtype=torch.float64, device="cuda")
    plan = K.Plan([(a.t(), b.t(), c, False)])
    plan.run(use_graph=False)
    assert torch.allclose(c, a.t() @ b.t(), rtol=1e-12, atol=1e-12)
    plan.close()


def test_tuner_times_every_variant(K):
    times, best = K.tune_gemm(L.F32, 96, 200, 80, reps=2)
    vs = K.tile_variants()
    for v, t in enumerate(times):
        assert (t > 0) == (vs[v]["dtype"] == L.F32)
    assert vs[best]["dtype"] == L.F32
    times, best = K.tune_gemm(L.F64, 64, 64, 64, flags=L.GEMM_TRANS_A, batch=8, reps=2)
    assert vs[best]["dtype"] == L.F64


def _bf16_round(a):
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def test_selector_gradcheck_vs_oracle(K, ora):
    sel = K.Selector(7, 64, L.TILE_VARIANTS, seed=3)
    p = sel.get_params()
    F, H, V = 7, 64, L.TILE_VARIANTS
    r = np.random.default_rng(4)
    B = 48
    x = r.uniform(0, 1, (B, F)).astype(np.float32)
    t = r.normal(0, 1, (B, V)).astype(np.float32)
    mask = (r.uniform(0, 1, (B, V)) > 0.3).astype(np.float32)
    y, g, loss = sel.forward_backward(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda(),
                                      torch.from_numpy(mask).cuda())
    pb = _bf16_round(p)
    o = 0
    parts = []
    for shape in ((H, F), (H,), (H, H), (H,), (V, H), (V,)):
        cnt = int(np.prod(shape))
        parts.append(pb[o:o + cnt].reshape(shape))
        o += cnt
    lo, yo, go = ora.mlp_forward_backward(x, t, mask, *parts)
    np.testing.assert_allclose(to_np(y), yo, rtol=1e-4, atol=1e-5)
    assert abs(loss - lo) <= 1e-4 * max(1.0, abs(lo))
    gflat = np.concatenate([gg.ravel() for gg in go])
    gg = to_np(g)
    scale = np.abs(gflat).max()
    assert np.max(np.abs(gg - gflat)) <= 1e-4 * scale
    sel.close()


def test_selector_training_reduces_loss(K):
    sel = K.Selector(7, 64, L.TILE_VARIANTS, seed=5)
    r = np.random.default_rng(6)
    n = 2000
    x = r.uniform(0, 1, (n, 7)).astype(np.float32)
    # a smooth synthetic target: per-variant linear forms of the features
    W = r.normal(0, 1, (7, L.TILE_VARIANTS)).astype(np.float32)
    t = (x @ W + 0.5 * np.sin(3 * x[:, :1])).astype(np.float32)
    mask = np.ones_like(t)
    xd, td, md = (torch.from_numpy(v).cuda() for v in (x, t, mask))
    l0 = sel.train(xd, td, md, epochs=1, batch=128, lr=3e-3)
    l1 = sel.train(xd, td, md, epochs=40, batch=128, lr=3e-3)
    assert l1 < 0.2 * l0
    y = sel.predict(xd)
    assert float(((y - td) ** 2).mean()) < 0.2 * float(((td - td.mean(0)) ** 2).mean())
    sel.close()


def test_learned_selector_vs_heuristic_on_held_out_shapes(K):
    """The selector trains on the GPU on the committed autotuner timings of
    this GPU model (tests/golden/selector_timings_gb300.npz, made by
    tune_selector.py --save-timings), then picks tiles for 200 held-out
    shapes drawn now from another stream of the same distribution and timed
    exhaustively: its picks reach at least 0.95 of the exhaustively tuned
    throughput and beat the size heuristic's mean regret."""
    import os
    import tune_selector as TS
    path = os.path.join(os.path.dirname(__file__), "golden", "selector_timings_gb300.npz")
    if not os.path.exists(path):
        pytest.skip("no committed selector timings")
    res, sel = TS.run_from_timings(path, 200, seed=2024, reps=1)
    print("selector", res["selector"], "heuristic", res["heuristic"])
    assert res["selector"]["throughput_vs_exhaustive"] >= 0.95, res
    assert res["selector"]["mean_regret"] < res["heuristic"]["mean_regret"], res
    assert res["tuning_time_saved_x"] > 10
    sel.close()


def test_learned_selector_small_collection(K):
    """Collect, train and evaluate end to end on a small live collection."""
    import tune_selector as TS
    res, sel, rows, _ = TS.run(360, 120, seed=11, reps=1, epochs=200, hi=1024,
                               f64_max_flops=2e10, f32_max_flops=2e11)
    assert res["selector"]["throughput_vs_exhaustive"] >= 0.85
    assert res["tuning_time_saved_x"] > 10
    sel.close()


def test_plan_autotune_never_slower_than_untuned_and_exact(K, ora):
    """nrs_plan_autotune judges assignments by timing the whole group; its
    final choice is at least as fast as the untuned plan (as measured in the
    same call), and the tuned plan still gives the parity results."""
    gemms, reds = _problems(17, 200, 60)
    K.tuner_clear()
    rep = K.autotune_plan(gemms, reds, max_trials=12, reps=3)
    assert rep["buckets"] > 0 and rep["trials"] <= 12
    assert rep["final_ms"] <= rep["untuned_ms"]
    assert rep["final_ms"] <= rep["isolated_ms"]
    for a, b, c, _ in gemms:
        c.fill_(float("nan"))
    plan = K.Plan(gemms, reds, **rep["plan_kwargs"])
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    for a, b, c, _ in gemms[1::2][:40]:  # f64 problems against double-double
        Cdd, ab = ora.gemm_dd(to_np(a), to_np(b))
        err = np.max(np.abs(to_np(c) - Cdd) / np.where(ab > 0, ab, 1))
        assert err <= 1e-14
    for x, op, out in reds:
        want = K.reduce(x, op).reshape(1)
        assert torch.equal(out.view(torch.int64 if out.element_size() == 8 else torch.int32),
                           want.view(torch.int64 if want.element_size() == 8 else torch.int32))
    plan.close()
    K.tuner_clear()


def test_tuner_and_selector_files_are_keyed(K, tmp_path):
    import numrs_gb300 as N
    K.tuner_clear()
    K.tuner_set(L.F64, 100, 200, 300, 4)
    K.tuner_set(L.F32, 32, 32, 32, 1)
    path = str(tmp_path / "tuner.txt")
    K.tuner_save(path)
    K.tuner_clear()
    assert K.tuner_get(L.F64, 100, 200, 300) == -1
    K.tuner_load(path)
    assert K.tuner_get(L.F64, 100, 200, 300) == 4 and K.tuner_get(L.F32, 32, 32, 32) == 1
    # a file made for another GPU / driver / build is refused and changes nothing
    text = open(path).read().splitlines()
    for i, line in ((1, "gpu other"), (2, "driver 1"), (3, "source other")):
        bad = list(text)
        bad[i] = line
        open(path + ".bad", "w").write("\n".join(bad) + "\n")
        K.tuner_clear()
        with pytest.raises(N.NumRs2Error):
            K.tuner_load(path + ".bad")
        assert K.tuner_get(L.F64, 100, 200, 300) == -1
    K.tuner_clear()
    # selector weights round-trip bit for bit; another network shape is refused
    s1 = K.Selector(7, 64, L.TILE_VARIANTS, seed=3)
    s2 = K.Selector(7, 64, L.TILE_VARIANTS, seed=4)
    wpath = str(tmp_path / "sel.bin")
    s1.save(wpath)
    assert not np.array_equal(s1.get_params(), s2.get_params())
    s2.load(wpath)
    np.testing.assert_array_equal(s1.get_params(), s2.get_params())
    s3 = K.Selector(7, 32, L.TILE_VARIANTS, seed=4)
    with pytest.raises(N.ShapeMismatch):
        s3.load(wpath)
    for sel in (s1, s2, s3):
        sel.close()


def test_grouped_row_extrema_first_zero(K, ora):
    """Max / min rows whose extreme is a zero of both signs: the grouped row
    reductions and nrs_reduce both keep the first zero, as the left-to-right
    fold does (one chunk, chunk edges, several chunks)."""
    r = np.random.default_rng(3)
    a = torch.empty((32, 32), dtype=torch.float64, device="cuda").uniform_(-1, 1)
    gemms = [(a, a.clone(), torch.empty_like(a), False)]
    reds, hosts = [], []
    for n in (100, 8192, 8193, 30000, 70001):
        for dt in (np.float32, np.float64):
            for op, sign in ((L.MAX, -1.0), (L.MIN, 1.0)):
                x = (sign * np.abs(r.standard_normal(n))).astype(dt)
                z = r.choice(n, 6, replace=False)
                first = np.sort(z)
                x[z] = 0.0
                x[first[0]] = -0.0 if r.random() < 0.5 else 0.0
                x[first[1:]] = np.where(np.signbit(x[first[0]]), 0.0, -0.0)  # later zeros: the other sign
                xd = torch.from_numpy(x).cuda()
                reds.append((xd, op, torch.empty(1, dtype=xd.dtype, device="cuda")))
                hosts.append(x)
    plan = K.Plan(gemms, reds)
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    for (xd, op, out), x in zip(reds, hosts):
        want = np.array([ora.flat("max" if op == L.MAX else "min", x)], x.dtype)
        np.testing.assert_array_equal(bits(to_np(out)), bits(want))
        np.testing.assert_array_equal(bits(to_np(K.reduce(xd, op))), bits(want))
