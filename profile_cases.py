"""Small, self-contained launch cases for profiling one kernel at a time.

    python profile_cases.py --case fold_cols_f32_max [--n 8192] [--launches 3]

Each case allocates inputs larger than the 129 MB L2 but only a few GB in
total, runs one warm-up launch and then `--launches` launches of the kernel
under study, so a profiler can capture them with -k/-c.
"""
from __future__ import annotations

import argparse

import torch

from numrs_gb300 import _lib as L
from numrs_gb300 import kernels as K

CASES = {
    "fold_cols_f32_sum": ("f32", L.SUM, 0),
    "fold_cols_f32_max": ("f32", L.MAX, 0),
    "fold_rows_f32_sum": ("f32", L.SUM, 1),
    "fold_rows_f32_max": ("f32", L.MAX, 1),
    "fold_cols_i64_sum": ("i64", L.SUM, 0),
    "fold_cols_i64_max": ("i64", L.MAX, 0),
    "fold_rows_i64_sum": ("i64", L.SUM, 1),
    "flat_sum_f32": ("f32", L.SUM, None),
    "flat_max_f32": ("f32", L.MAX, None),
    "flat_argmax_f32": ("f32", L.ARGMAX, None),
    "fold_cols_f64_max": ("f64", L.MAX, 0),
    "fold_rows_f64_max": ("f64", L.MAX, 1),
    "flat_max_f64": ("f64", L.MAX, None),
    "exp_affine_f32": ("f32", None, None),
    "ozaki_f64": ("f64", None, None),
    "dmma_f64": ("f64", None, None),
    "grouped": (None, None, None),
    "cumsum_cols_f32": ("f32", "add", 0),
    "cumsum_rows_f32": ("f32", "add", 1),
    "cumsum_flat_f32": ("f32", "add", None),
    "expr_abc_f32": ("f32", None, None),
    "add_row_f32": ("f32", None, None),
    "dmma_splitk_f64": ("f64", None, None),
    "simt_f32": ("f32", None, None),
    "argmax_rows_f32": ("f32", L.ARGMAX, 1),
    "argmax_cols_f32": ("f32", L.ARGMAX, 0),
    "maximum_reduce_cols_f32": ("f32", "maximum", 0),
    "maximum_reduce_rows_f32": ("f32", "maximum", 1),
    "add_decode_f32": ("f32", None, None),
    "selector_train": (None, None, None),
    "grouped_ozaki": (None, None, None),
    "c4_f64_ozaki": (None, None, None),
    "c4_f32_ozaki": (None, None, None),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", required=True, choices=sorted(CASES))
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--slices", type=int, default=0)  # 0: the library's default
    a = ap.parse_args()
    dt, op, axis = CASES[a.case]
    n = a.n
    if a.case.startswith("fold") or a.case.startswith("flat"):
        if dt in ("f32", "f64"):
            x = torch.empty((n, n), dtype=torch.float32 if dt == "f32" else torch.float64, device="cuda")
            K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
        else:
            x = torch.empty((n, n), dtype=torch.int64, device="cuda")
            K.fill_random(x, L.RNG_INT, 4, -(1 << 20), float(1 << 21))
        fn = lambda: K.reduce(x, op, axis)  # noqa: E731
    elif a.case.startswith("cumsum"):
        x = torch.empty((n, n), dtype=torch.float32, device="cuda")
        K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
        fn = lambda: K.ufunc_accumulate(op, x, axis)  # noqa: E731
    elif a.case in ("expr_abc_f32", "add_row_f32"):
        x = torch.empty((n, n), dtype=torch.float32, device="cuda")
        K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
        if a.case == "expr_abc_f32":
            b, c = torch.empty_like(x), torch.empty_like(x)
            K.fill_random(b, L.RNG_NORMAL, 4, 0.0, 1.0)
            K.fill_random(c, L.RNG_NORMAL, 5, 0.0, 1.0)
            E = K.Expr.leaf
            fn = lambda: ((E(x) * E(b)) + E(c)).eval()  # noqa: E731
        else:
            row = x[0].clone()
            fn = lambda: K.add(x, row)  # noqa: E731
    elif a.case == "exp_affine_f32":
        x = torch.empty((n, n), dtype=torch.float32, device="cuda")
        K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
        y = torch.empty_like(x)
        fn = lambda: K.exp_affine(x, 0.5, -0.25, out=y)  # noqa: E731
    elif a.case in ("ozaki_f64", "dmma_f64"):
        A = torch.empty((n, n), dtype=torch.float64, device="cuda")
        B = torch.empty_like(A)
        C = torch.empty_like(A)
        K.fill_random(A, L.RNG_UNIFORM, 5, -0.5, 0.5)
        K.fill_random(B, L.RNG_UNIFORM, 6, -0.5, 0.5)
        if a.case == "ozaki_f64":
            fn = lambda: K.gemm_ozaki(A, B, slices=a.slices, out=C)  # noqa: E731
        else:
            fn = lambda: K.gemm_2d(n, n, n, A, B, C, variant=L.GEMM_DMMA)  # noqa: E731
    elif a.case == "dmma_splitk_f64":
        # 512^3: 32x32 tiles in 4 k chunks, then splitk_finish adds the slabs
        n = 512
        A = torch.empty((n, n), dtype=torch.float64, device="cuda")
        B, C = torch.empty_like(A), torch.empty_like(A)
        K.fill_random(A, L.RNG_UNIFORM, 1, -1.0, 1.0)
        K.fill_random(B, L.RNG_UNIFORM, 2, -1.0, 1.0)
        fn = lambda: K.gemm_2d(n, n, n, A, B, C, variant=L.GEMM_DMMA)  # noqa: E731
    elif a.case == "simt_f32":
        A = torch.empty((n, n), dtype=torch.float32, device="cuda")
        B, C = torch.empty_like(A), torch.empty_like(A)
        K.fill_random(A, L.RNG_UNIFORM, 1, -1.0, 1.0)
        K.fill_random(B, L.RNG_UNIFORM, 2, -1.0, 1.0)
        fn = lambda: K.gemm_2d(n, n, n, A, B, C, variant=L.GEMM_SIMT)  # noqa: E731
    elif a.case.startswith("argmax") or a.case.startswith("maximum_reduce"):
        x = torch.empty((n, n), dtype=torch.float32, device="cuda")
        K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
        if a.case.startswith("argmax"):
            fn = lambda: K.reduce(x, op, axis)  # noqa: E731
        else:
            fn = lambda: K.ufunc_reduce(op, x, axis)  # noqa: E731
    elif a.case == "add_decode_f32":
        # (n, 128, n/128) views with a strided short last axis: every element
        # index is decoded (ufunc_decode)
        x = torch.empty((n, n), dtype=torch.float32, device="cuda")
        K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
        v = x.view(n, n // 128, 128).transpose(1, 2)
        fn = lambda: K.add(v, v)  # noqa: E731
    elif a.case == "selector_train":
        # the learned selector's training loop: mlp_forward, mlp_backward,
        # mlp_grad and adam_step per minibatch (20000 samples, batch 256)
        g = torch.Generator(device="cuda").manual_seed(1)
        xs = torch.rand((20000, 7), device="cuda", generator=g)
        ts = torch.randn((20000, L.TILE_VARIANTS), device="cuda", generator=g)
        ms = torch.ones_like(ts)
        sel = K.Selector()
        fn = lambda: sel.train(xs, ts, ms, epochs=1)  # noqa: E731
    elif a.case in ("c4_f64_ozaki", "c4_f32_ozaki"):
        # bench.py's C4 group (seed 7: 4096 GEMMs, M, N, K log-uniform in
        # [16, 512], even indices f32, odd f64), only its f64 (or f32) GEMMs,
        # as one plan with them on the tensor cores, replayed from its graph
        import numpy as np
        r = np.random.default_rng(7)
        lu = lambda lo, hi, k: np.exp(r.uniform(np.log(lo), np.log(hi), k)).astype(np.int64)  # noqa: E731
        M, N, Kd = lu(16, 512, 4096), lu(16, 512, 4096), lu(16, 512, 4096)
        f64 = a.case == "c4_f64_ozaki"
        t = torch.float64 if f64 else torch.float32
        gemms = []
        for i in range(1 if f64 else 0, 4096, 2):
            gemms.append((torch.empty((int(M[i]), int(Kd[i])), dtype=t, device="cuda").uniform_(-1, 1),
                          torch.empty((int(Kd[i]), int(N[i])), dtype=t, device="cuda").uniform_(-1, 1),
                          torch.empty((int(M[i]), int(N[i])), dtype=t, device="cuda"), False))
        plan = K.Plan(gemms, f64_mode=L.PLAN_F64_OZAKI) if f64 else K.Plan(gemms, f32_mode=L.PLAN_F32_OZAKI)
        fn = lambda: plan.run(use_graph=True)  # noqa: E731
    else:
        import numpy as np
        r = np.random.default_rng(7)
        lu = lambda lo, hi, k: np.exp(r.uniform(np.log(lo), np.log(hi), k)).astype(np.int64)  # noqa: E731
        M, N, Kd = lu(16, 512, 512), lu(16, 512, 512), lu(16, 512, 512)
        gemms = []
        for i in range(512):
            t = torch.float32 if i % 2 == 0 else torch.float64
            gemms.append((torch.randn(int(M[i]), int(Kd[i]), dtype=t, device="cuda"),
                          torch.randn(int(Kd[i]), int(N[i]), dtype=t, device="cuda"),
                          torch.empty(int(M[i]), int(N[i]), dtype=t, device="cuda"), False))
        if a.case == "grouped_ozaki":
            # the same mix with its f64 GEMMs on the tensor cores
            plan = K.Plan(gemms, f64_mode=L.PLAN_F64_OZAKI)
        else:
            plan = K.Plan(gemms)
        fn = lambda: plan.run(use_graph=False)  # noqa: E731
    fn()
    torch.cuda.synchronize()
    for _ in range(a.launches):
        fn()
    torch.cuda.synchronize()
    print("ok", a.case)


if __name__ == "__main__":
    main()
