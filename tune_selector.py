"""Learned tile selection: collect autotuner timings, train the MLP selector
on the GPU, evaluate it against exhaustive tuning.

    python tune_selector.py --shapes 6700 --holdout 2000 \
        --out selector_run.json [--save-timings timings.npz] [--sweep]
    python tune_selector.py --train-from tests/golden/selector_timings_gb300.npz \
        --holdout 500 --out selector_eval.json

Shapes are log-uniform in [1, 16384]^3 (dtype f32 or f64 with equal
probability, transpose flags and a batch count of 1..64 drawn per shape);
every tile variant of the shape's dtype is timed by nrs_tune_gemm (one
warm-up, `reps` timed launches of `batch` copies), giving one timing per
(shape, variant). A budget cap skips f64 shapes above `--f64-max-flops`
and f32 shapes above `--f32-max-flops` per problem (redrawn), so one
collection fits in minutes; the cap is reported.

The selector (7 features -> 64 -> 64 -> one log2-time per variant) trains on
the GPU with the library's own kernels (nrs_selector_train). On held-out
shapes it picks the variant with the smallest predicted time; regret is
1 - t_best / t_chosen with t measured, against the exhaustive choice (the
judge and the fallback) and against the size heuristic the library uses
without a selector. The selector only picks among variants that all pass
the same parity tests, so it never changes numerics.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np
import torch

from numrs_gb300 import _lib as L
from numrs_gb300 import kernels as K


def heuristic(dtype: int, m: int, k: int, n: int) -> int:
    """The plan builder's size rule (grouped.cu heuristic_variant)."""
    mx = max(m, n)
    if dtype == L.F32:
        if m * n >= 128 * 128:
            return 0
        return 2 if (k >= 8 * mx and m * n <= 64 * 64) else 1
    if m * n >= 256 * 256:
        return 3
    return 5 if (k >= 8 * mx and m * n <= 64 * 64) else 4


def features(m, n, k, dtype, ta, tb, batch):
    lg = lambda v: math.log2(max(v, 1)) / 14.0  # noqa: E731
    return [lg(m), lg(n), lg(k), 1.0 if dtype == L.F64 else 0.0, float(ta), float(tb), lg(batch)]


def collect(n_shapes: int, seed: int, reps: int, lo: int = 1, hi: int = 16384,
            f64_max_flops: float = 1e11, f32_max_flops: float = 4e12, max_batch: int = 64,
            log_every: int = 0):
    r = np.random.default_rng(seed)
    rows = []
    skipped = 0
    t0 = time.perf_counter()
    while len(rows) < n_shapes:
        m, n, k = (int(round(math.exp(r.uniform(math.log(lo), math.log(hi))))) for _ in range(3))
        dtype = L.F64 if r.uniform() < 0.5 else L.F32
        ta, tb = int(r.uniform() < 0.25), int(r.uniform() < 0.25)
        batch = int(round(math.exp(r.uniform(0, math.log(max_batch)))))
        flops = 2.0 * m * n * k * batch
        if flops > (f64_max_flops if dtype == L.F64 else f32_max_flops):
            skipped += 1
            continue
        flags = (L.GEMM_TRANS_A if ta else 0) | (L.GEMM_TRANS_B if tb else 0)
        ts = time.perf_counter()
        times, best = K.tune_gemm(dtype, m, k, n, flags=flags, batch=batch, reps=reps)
        tune_s = time.perf_counter() - ts
        rows.append({"m": m, "n": n, "k": k, "dtype": dtype, "ta": ta, "tb": tb, "batch": batch,
                     "times_us": [float(t) for t in times], "best": best, "tune_s": tune_s})
        if log_every and len(rows) % log_every == 0:
            print(f"[collect] {len(rows)}/{n_shapes} shapes, {time.perf_counter() - t0:.1f}s", flush=True)
    return rows, skipped


def to_arrays(rows):
    X = np.array([features(r["m"], r["n"], r["k"], r["dtype"], r["ta"], r["tb"], r["batch"]) for r in rows],
                 np.float32)
    T = np.zeros((len(rows), L.TILE_VARIANTS), np.float32)
    M = np.zeros_like(T)
    for i, r in enumerate(rows):
        for v, t in enumerate(r["times_us"]):
            if t > 0:
                T[i, v] = math.log2(t)
                M[i, v] = 1.0
    return X, T, M


def choose(sel, X, rows):
    y = sel.predict(torch.from_numpy(X).cuda()).cpu().numpy()
    out = []
    for i, r in enumerate(rows):
        cand = [v for v in range(L.TILE_VARIANTS) if r["times_us"][v] > 0]
        out.append(min(cand, key=lambda v: y[i, v]))
    return out


def regret_of(rows, picks):
    best = np.array([min(t for t in r["times_us"] if t > 0) for r in rows])
    chosen = np.array([r["times_us"][p] for r, p in zip(rows, picks)])
    per = 1.0 - best / chosen
    return {"mean_regret": float(per.mean()), "p90_regret": float(np.quantile(per, 0.9)),
            "throughput_vs_exhaustive": float(best.sum() / chosen.sum()),
            "mean_throughput_ratio": float((best / chosen).mean()),
            "exact_pick_rate": float((per <= 1e-9).mean())}


def train(train_rows, seed: int = 8, epochs: int = 300, batch: int = 256, lr: float = 3e-3):
    """Trains the selector on the GPU (nrs_selector_train) on one timing per
    (shape, variant); returns (selector, final loss, seconds)."""
    X, T, M = to_arrays(train_rows)
    # Targets relative to each shape's mean log-time over its variants: the
    # choice only depends on differences between variants, and removing the
    # shape's overall cost (which spans ~30 octaves) keeps the loss on them.
    rowmean = (T * M).sum(1, keepdims=True) / np.maximum(M.sum(1, keepdims=True), 1)
    T = (T - rowmean) * M
    sd = np.sqrt(((T * M) ** 2).sum(0) / np.maximum(M.sum(0), 1)) + 1e-6
    Tn = (T / sd * M).astype(np.float32)
    sel = K.Selector(7, 64, L.TILE_VARIANTS, seed=seed)
    t0 = time.perf_counter()
    loss = sel.train(torch.from_numpy(X).cuda(), torch.from_numpy(Tn).cuda(), torch.from_numpy(M).cuda(),
                     epochs=epochs, batch=batch, lr=lr, seed=seed)
    torch.cuda.synchronize()
    return sel, loss, time.perf_counter() - t0


def evaluate(sel, test_rows):
    """Regret of the selector's and the size heuristic's picks against the
    exhaustive choice on measured held-out timings."""
    Xt, _, _ = to_arrays(test_rows)
    t0 = time.perf_counter()
    picks = choose(sel, Xt, test_rows)
    infer_s = time.perf_counter() - t0
    heur = [heuristic(r["dtype"], r["m"], r["k"], r["n"]) for r in test_rows]
    tune_s = sum(r["tune_s"] for r in test_rows)
    return {"shapes_holdout": len(test_rows), "selector": regret_of(test_rows, picks),
            "heuristic": regret_of(test_rows, heur), "exhaustive_tuning_seconds_holdout": tune_s,
            "selector_inference_seconds_holdout": infer_s, "tuning_time_saved_x": tune_s / max(infer_s, 1e-9)}


def run(n_shapes: int, holdout: int, seed: int = 8, reps: int = 1, epochs: int = 300,
        batch: int = 256, lr: float = 3e-3, **collect_kw):
    """Collects n_shapes + holdout shapes, trains on the first n_shapes and
    evaluates on the rest."""
    rows, skipped = collect(n_shapes + holdout, seed, reps, **collect_kw)
    train_rows, test_rows = rows[:n_shapes], rows[n_shapes:]
    sel, loss, train_s = train(train_rows, seed=seed, epochs=epochs, batch=batch, lr=lr)
    n_timings = sum(sum(1 for t in r["times_us"] if t > 0) for r in rows)
    res = {"shapes_train": len(train_rows), "timings": n_timings, "skipped_by_budget_cap": skipped,
           "final_train_loss": loss, "train_seconds": train_s}
    res.update(evaluate(sel, test_rows))
    return res, sel, rows, None


_COLS = ("m", "n", "k", "dtype", "ta", "tb", "batch")


def save_timings(path: str, rows) -> None:
    """The training timings as a compressed .npz (shape columns + microseconds
    per problem for every variant, -1 where a variant does not apply)."""
    np.savez_compressed(path, **{c: np.array([r[c] for r in rows], np.int64) for c in _COLS},
                        times_us=np.array([r["times_us"] for r in rows], np.float32))


def load_timings(path: str):
    z = np.load(path)
    out = []
    for i in range(len(z["m"])):
        r = {c: int(z[c][i]) for c in _COLS}
        r["times_us"] = [float(t) for t in z["times_us"][i]]
        r["best"] = int(np.argmin(np.where(z["times_us"][i] > 0, z["times_us"][i], np.inf)))
        r["tune_s"] = 0.0
        out.append(r)
    return out


def run_from_timings(path: str, holdout: int, seed: int = 1008, reps: int = 1, epochs: int = 300,
                     batch: int = 256, lr: float = 3e-3, **collect_kw):
    """Trains on saved timings (load_timings) and evaluates on `holdout`
    shapes collected now from another stream of the same distribution."""
    train_rows = load_timings(path)
    test_rows, skipped = collect(holdout, seed, reps, **collect_kw)
    sel, loss, train_s = train(train_rows, seed=seed, epochs=epochs, batch=batch, lr=lr)
    res = {"shapes_train": len(train_rows), "train_timings_file": os.path.basename(path),
           "timings": sum(sum(1 for t in r["times_us"] if t > 0) for r in train_rows),
           "skipped_by_budget_cap_holdout": skipped, "final_train_loss": loss, "train_seconds": train_s}
    res.update(evaluate(sel, test_rows))
    return res, sel


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shapes", type=int, default=6700)
    ap.add_argument("--holdout", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--seed", type=int, default=8)
    ap.add_argument("--reps", type=int, default=1)
    ap.add_argument("--hi", type=int, default=16384)
    ap.add_argument("--f64-max-flops", type=float, default=1e11)
    ap.add_argument("--f32-max-flops", type=float, default=4e12)
    ap.add_argument("--out", default="selector_run.json")
    ap.add_argument("--save-timings", default=None, help="write the training rows as .npz")
    ap.add_argument("--train-from", default=None, help="train on a saved .npz instead of collecting")
    ap.add_argument("--sweep", action="store_true", help="also evaluate training recipes on a validation split")
    a = ap.parse_args()
    kw = dict(hi=a.hi, f64_max_flops=a.f64_max_flops, f32_max_flops=a.f32_max_flops)
    if a.train_from:
        res, sel = run_from_timings(a.train_from, a.holdout, seed=a.seed + 1000, reps=a.reps, epochs=a.epochs,
                                    batch=a.batch, lr=a.lr, log_every=500, **kw)
        json.dump(res, open(a.out, "w"), indent=1)
        print(json.dumps(res))
        return
    rows, skipped = collect(a.shapes + a.holdout, a.seed, a.reps, log_every=500, **kw)
    train_rows, test_rows = rows[:a.shapes], rows[a.shapes:]
    if a.save_timings:
        save_timings(a.save_timings, train_rows)
    sel, loss, train_s = train(train_rows, seed=a.seed, epochs=a.epochs, batch=a.batch, lr=a.lr)
    res = {"shapes_train": len(train_rows), "skipped_by_budget_cap": skipped,
           "timings": sum(sum(1 for t in r["times_us"] if t > 0) for r in rows),
           "final_train_loss": loss, "train_seconds": train_s}
    res.update(evaluate(sel, test_rows))
    if a.sweep:
        # training recipes judged on a validation split of the TRAINING rows
        # (the held-out shapes stay unseen by the choice)
        cut = int(len(train_rows) * 0.8)
        fit_rows, val_rows = train_rows[:cut], train_rows[cut:]
        res["sweep"] = []
        for ep in (300, 600, 1200):
            for lr in (1e-3, 3e-3, 1e-2):
                for bs in (128, 256):
                    s2, l2, t2 = train(fit_rows, seed=a.seed, epochs=ep, batch=bs, lr=lr)
                    ev = evaluate(s2, val_rows)
                    res["sweep"].append({"epochs": ep, "lr": lr, "batch": bs, "loss": l2, "train_s": t2,
                                         "throughput_vs_exhaustive": ev["selector"]["throughput_vs_exhaustive"],
                                         "mean_regret": ev["selector"]["mean_regret"]})
                    s2.close()
    json.dump(res, open(a.out, "w"), indent=1)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
