"""Benchmark of the reduction / fused-ufunc hot path (HBM GB/s).

Workload (one "step"): over a 16384 x 16384 f32 array of N(0,1) values
(SplitMix64 seed 3) and a 16384 x 16384 i64 array uniform in [-2^20, 2^20)
(seed 4), in the row-major layout and as the transposed-stride view
(shape swapped, strides (1, 16384)):
  f32 sum / mean / max  x axis 0, 1 x 2 views   (12 reductions)
  i64 sum / max         x axis 0, 1 x 2 views   ( 8 reductions)
  fused y = exp(0.5 * x - 0.25) over the f32 array (1 ufunc pass)
Each is one kernel launch. Algorithmic bytes = every input element read once
plus every output written once. Inputs are 1 GiB and 2 GiB (far larger than
the 129 MB L2), so no L2 flush is needed between steps.

Printed JSON (one line, rank 0): value = device-resident GB/s of the whole
step; e2e = the same bytes through the C ABI with pinned HOST buffers (host
-> device copies of both arrays and device -> host copies of every result
inside the timed region), with e2e.link = the pinned copy rates measured in
the same run and the step's floor at that H2D rate (frac = floor / step);
roofline = the dominant kernel class against the
measured HBM peak; cpu_baseline = the CPU oracle (numrs2 restatement) on a
bounded row slab of the same workload, all host threads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

R = C_ = 16384
F32_SEED, I64_SEED = 3, 4
A_SCALE, B_SHIFT = 0.5, -0.25


E2E_BLOCKS = 8  # row blocks of the i64 upload in the end-to-end step
CONFIG = {"workload": "16384x16384 f32 N(0,1) + i64 U[-2^20,2^20): axis-0/1 sum/mean/max (f32), "
                      "sum/max (i64), row-major and transposed-stride views, + fused exp(0.5x-0.25); "
                      "one step = 21 launches",
          "l2": "no flush: inputs (1 GiB, 2 GiB) > 129 MB L2"}


def max_over_ranks(value: float, dist, device) -> float:
    """The slowest rank's time (replicas: the job ends with the last one)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gbs(step_bytes: int, world: int, ms_per_step: float) -> float:
    """Whole-job throughput: every rank processes its own replica of the step."""
    return step_bytes * world / (ms_per_step / 1e3) / 1e9


def profiled_traffic(kernel_class: str):
    """DRAM bytes per full-size launch of `kernel_class` from the ncu capture
    recorded in profiles/traffic_per_launch.json (None if not recorded)."""
    p = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    if not os.path.exists(p):
        return None
    return json.load(open(p))["traffic_per_launch_bytes"].get(kernel_class)


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _bf16_peak():
    """Dense BF16 burst rate (TFLOP/s) of MEASURED_PEAKS.json, else the
    fallback figure."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["bf16_tflops"])
    return 1900.0


class Clocks:
    """nvidia-smi sampler over the timed region."""

    def __init__(self, gpu: int):
        # raw samples beside the run's other outputs (NRS_BENCH_OUT), else a temp dir
        out_dir = os.environ.get("NRS_BENCH_OUT") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_bench_{os.getpid()}.csv")
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_ops(K, x32, x64):
    """The step's launches as (class, bytes, callable)."""
    from numrs_gb300 import _lib as L
    ops = []
    n = R * C_
    views32 = [("rm", x32), ("tr", x32.t())]
    views64 = [("rm", x64), ("tr", x64.t())]
    for vname, v in views32:
        for op, code in (("sum", L.SUM), ("mean", L.MEAN), ("max", L.MAX)):
            for axis in (0, 1):
                # which kernel serves it: lanes contiguous -> rows kernel
                lanes_contig = (axis == 1) == (vname == "rm")
                cls = "fold_rows_tma" if lanes_contig else "fold_cols_tma"
                ops.append((f"{cls}/f32", n * 4 + 16384 * 4,
                            (lambda v=v, code=code, axis=axis: K.reduce(v, code, axis))))
    for vname, v in views64:
        for op, code in (("sum", L.SUM), ("max", L.MAX)):
            for axis in (0, 1):
                lanes_contig = (axis == 1) == (vname == "rm")
                cls = "fold_rows_tma" if lanes_contig else "fold_cols_tma"
                ops.append((f"{cls}/i64", n * 8 + 16384 * 8,
                            (lambda v=v, code=code, axis=axis: K.reduce(v, code, axis))))
    y = x32.new_empty(x32.shape)
    ops.append(("exp_affine_vec/f32", n * 8, (lambda: K.exp_affine(x32, A_SCALE, B_SHIFT, out=y))))
    return ops, y


def cpu_sample(steps: int | None, min_seconds: float, x32_np, x64_np):
    """Times the oracle (numrs2's CPU kernels restated) on the row slab."""
    from oracle import Oracle
    from oracle import oracle as O
    ora = Oracle()
    rows = x32_np.shape[0]
    nbytes = 0
    calls = []
    for v in (x32_np, x32_np.T):
        for code in (O.SUM, O.MEAN, O.MAX):
            for axis in (0, 1):
                calls.append((v, code, axis))
                nbytes += v.size * 4 + (v.shape[1 - axis]) * 4
    for v in (x64_np, x64_np.T):
        for code in (O.SUM, O.MAX):
            for axis in (0, 1):
                calls.append((v, code, axis))
                nbytes += v.size * 8 + (v.shape[1 - axis]) * 8
    nbytes += x32_np.size * 8

    def one_pass():
        for v, code, axis in calls:
            ora.axis(code, v, axis)
        ora.exp_affine(x32_np, A_SCALE, B_SHIFT)

    times = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        one_pass()
        times.append(time.perf_counter() - t0)
        if steps is not None and len(times) >= steps:
            break
        if steps is None and time.perf_counter() - t_start >= min_seconds:
            break
    shape = f"{rows}x{x32_np.shape[1]}"
    what = "the full arrays" if rows == R else f"a {shape} row slab of both arrays"
    return nbytes, times, ora.num_threads(), f"{what}, all 21 ops, numrs2 kernels restated in C (OpenMP)"


def reference_inputs():
    """The step's two arrays on the host, from the same SplitMix64 streams as
    the device generator (seed 3: f32 N(0,1); seed 4: i64 U[-2^20, 2^20))."""
    from oracle import Oracle
    ora = Oracle()
    x32 = ora.gen_normal_f32(F32_SEED, R * C_).reshape(R, C_)
    x64 = ora.gen_i64(I64_SEED, R * C_).reshape(R, C_)
    return x32, x64


def run_reference(args):
    """`--impl reference`: the CPU restatement of numrs2's kernels (the
    reference is Rust and cannot be built here) on the full step, all host
    threads, the same config as the GPU arm."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    x32, x64 = reference_inputs()
    nbytes, times, cores, sample = cpu_sample(args.warmup + args.steps, 0, x32, x64)
    t = sum(times[args.warmup:])
    val = nbytes * args.steps / t / 1e9
    line = {"impl": "reference", "metric": "reduce GB/s", "value": round(val, 2), "unit": "GB/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic (SplitMix64, seeds 3/4)",
            "config": dict(CONFIG, bytes_per_step=nbytes, parallelism=f"replicas x{args.gpus}"),
            "cpu_baseline": {"value": round(val, 2), "unit": "GB/s", "cores": cores, "kind": "port",
                             "sample": sample + f"; each of the {args.steps} timed steps is the whole step"},
            "e2e": {"value": round(val, 2), "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _time_ms(fn, reps, stream):
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _flush_l2(buf):
    """Overwrite a buffer larger than the 129 MB L2 between timed launches."""
    buf.add_(1)


def _event_median_ms(fn, reps, stream, flush=None):
    """Median of individually event-timed calls (L2 flushed before each)."""
    import torch
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        if flush is not None:
            flush()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def _gemm_peaks(K, L):
    """FP64 DMMA and FP32 FMA pipe rates measured on this GPU now."""
    return {"fp64_dmma_tflops": round(K.probe_peak(L.PEAK_FP64_DMMA), 4),
            "fp32_fma_tflops": round(K.probe_peak(L.PEAK_FP32_FMA), 3),
            "kind": "measured (nrs_probe_peak: register-resident mma.sync f64 / fp32 FMA chains on every SM)"}


def _cpu_gemm_tflops(n: int, seconds: float):
    """The oracle's restated gemm_2d (f64, all host threads) at n^3."""
    from oracle import Oracle
    ora = Oracle()
    A = ora.gen_uniform_pm1(1, n * n).reshape(n, n)
    B = ora.gen_uniform_pm1(2, n * n).reshape(n, n)
    times = []
    t_end = time.perf_counter() + seconds
    while not times or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        ora.gemm(A, B)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return {"value": round(2.0 * n ** 3 / t / 1e12, 5), "unit": "TFLOP/s", "cores": ora.num_threads(),
            "kind": "port", "sample": f"f64 {n}^3 gemm_2d restatement (i-k-j, KC=256, row split), "
                                     f"median of {len(times)} runs"}


def gemm_section(K, L, quick: bool, cpu: bool = True):
    """C1: plain f64 GEMM 512^3 (DMMA), against the FP64 pipe rate and the
    CPU restatement. C3: the 8192^3 split-precision GEMM with the automatic
    slice count beside the native FP64 DMMA GEMM for phi in {0, 1, 4};
    errors of both against 4096 double-double entries (i, j uniform) as
    max |C - C_dd| / (|A||B|)_ij."""
    import numpy as np
    import torch
    from oracle import Oracle
    ora = Oracle()
    stream = torch.cuda.current_stream()
    out = {"peaks": _gemm_peaks(K, L)}
    fp64_peak = out["peaks"]["fp64_dmma_tflops"]
    flush_buf = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    n1 = 512
    A = torch.empty((n1, n1), dtype=torch.float64, device="cuda")
    B = torch.empty_like(A)
    K.fill_random(A, L.RNG_UNIFORM, 1, -1.0, 1.0)
    K.fill_random(B, L.RNG_UNIFORM, 2, -1.0, 1.0)
    C = torch.empty_like(A)
    ms = _event_median_ms(lambda: K.gemm_2d(n1, n1, n1, A, B, C, variant=L.GEMM_DMMA), 20, stream,
                          flush=lambda: _flush_l2(flush_buf))
    tf = 2 * n1 ** 3 / ms / 1e9
    Cdd, ab = ora.gemm_dd(A.cpu().numpy(), B.cpu().numpy())
    c1 = {"workload": "f64 C=A*B 512^3, U(-1,1) SplitMix64 seeds 1/2, row-major", "ms": round(ms, 4),
          "tflops": round(tf, 4), "l2": "flushed before each timed call",
          "max_err_vs_dd": float(np.max(np.abs(C.cpu().numpy() - Cdd) / ab)),
          "roofline": {"bound": "fp64 dmma", "kernel": "dmma_gemm", "achieved": round(tf, 4),
                       "peak": fp64_peak, "unit": "TFLOP/s", "frac": round(tf / fp64_peak, 4)}}
    if cpu:
        c1["cpu_baseline"] = _cpu_gemm_tflops(n1, 3.0)
    out["c1_f64_512_dmma"] = c1
    del A, B, C
    n = 2048 if quick else 8192
    A = torch.empty((n, n), dtype=torch.float64, device="cuda")
    B = torch.empty_like(A)
    Cd = torch.empty_like(A)
    Co = torch.empty_like(A)
    flops = 2.0 * n ** 3
    r = np.random.default_rng(11)
    rows, cols = r.integers(0, n, 4096), r.integers(0, n, 4096)
    res = {}
    bf16_peak = _bf16_peak()
    for phi in (0.0, 1.0, 4.0):
        K.fill_random(A, L.RNG_OZAKI, 5, phi, 0.0)
        K.fill_random(B, L.RNG_OZAKI, 6, phi, 0.0)
        ms_d = _event_median_ms(lambda: K.gemm_2d(n, n, n, A, B, Cd, variant=L.GEMM_DMMA), 1, stream)
        # automatic slice count: spread estimate (one host read-back) + slices
        # + tensor-core products, timed as the whole call
        ms_o = _event_median_ms(lambda: K.gemm_ozaki(A, B, out=Co), 3, stream)
        info = K.gemm_ozaki(A, B, out=Co)[1]
        ref, ab = ora.gemm_dd_sampled(A.cpu().numpy(), B.cpu().numpy(), rows, cols)
        e_d = float(np.max(np.abs(Cd.cpu().numpy()[rows, cols] - ref) / ab))
        e_o = float(np.max(np.abs(Co.cpu().numpy()[rows, cols] - ref) / ab))
        entry = {"dmma_ms": round(ms_d, 2), "dmma_tflops": round(flops / ms_d / 1e9, 4),
                 "dmma_frac_of_fp64_peak": round(flops / ms_d / 1e9 / fp64_peak, 4),
                 "dmma_max_err_vs_dd": e_d,
                 "ozaki_auto": {"ms": round(ms_o, 2), "tflops_f64_equiv": round(flops / ms_o / 1e9, 2),
                                "slices": info["slices"], "slice_bits": info["slice_bits"],
                                "products": info["products"], "spread": info["spread"],
                                "est_rel_error": info["est_rel_error"], "max_err_vs_dd": e_o,
                                "speedup_vs_dmma": round(ms_d / ms_o, 2),
                                "error_within_dmma_or_1e-14": e_o <= max(e_d, 1e-14)}}
        if info["slices"] > 0:
            # the same slices without the estimate: the tensor-core kernel's
            # BF16 rate (slice-pair flops; slicing's ~3% of the time included)
            S = info["slices"]
            ms_x = _event_median_ms(lambda: K.gemm_ozaki(A, B, slices=S, out=Co), 3, stream)
            bf = 2.0 * n ** 3 * S * (S + 1) / 2
            entry["ozaki_auto"]["explicit_count_ms"] = round(ms_x, 2)
            entry["ozaki_auto"]["estimate_ms"] = round(ms_o - ms_x, 2)
            entry["ozaki_auto"]["roofline"] = {
                "bound": "tensor (bf16)", "kernel": "ozaki_tc_kernel + slicing",
                "achieved": round(bf / ms_x / 1e9, 1), "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": round(bf / ms_x / 1e9 / bf16_peak, 4)}
        res[f"phi={phi:g}"] = entry
    out[f"c3_f64_{n}_split_vs_dmma"] = res
    if cpu:
        out[f"c3_cpu_baseline"] = dict(_cpu_gemm_tflops(2048, 2.0),
                                       note="C3's 8192^3 is ~1 min on the host; the 2048^3 rate stands for it")
    del A, B, Cd, Co, flush_buf
    torch.cuda.empty_cache()
    return out


def elementwise_section(K, L):
    """Operators on 16384x16384 f32 (binary_serial / *_broadcast): same-shape
    add (12 B/elem), add of a broadcast row (8 B/elem), and an ExprNode tree
    (a*b + c, 16 B/elem), each one launch."""
    import torch
    n = R * C_
    stream = torch.cuda.current_stream()
    a = torch.empty((R, C_), device="cuda")
    b = torch.empty_like(a)
    c = torch.empty_like(a)
    K.fill_random(a, L.RNG_NORMAL, 11, 0.0, 1.0)
    K.fill_random(b, L.RNG_NORMAL, 12, 0.0, 1.0)
    K.fill_random(c, L.RNG_NORMAL, 13, 0.0, 1.0)
    row = b[0].clone()
    E = K.Expr.leaf
    cases = {"add_same_shape": (lambda: K.add(a, b), 12 * n),
             "add_broadcast_row": (lambda: K.add(a, row), 8 * n + 4 * C_),
             "expr_a_mul_b_add_c": (lambda: ((E(a) * E(b)) + E(c)).eval(), 16 * n)}
    out = {}
    for name, (fn, nbytes) in cases.items():
        ms = _time_ms(fn, 5, stream)
        out[name] = {"ms": round(ms, 4), "gbs": round(nbytes / ms / 1e6, 1)}
    del a, b, c
    torch.cuda.empty_cache()
    return out


def reductions_extra_section(K, L):
    """The reductions outside the C2 step, on the same 16384x16384 f32
    N(0,1) array (1 GiB, seed 3): flat sum / mean / max / var (the
    reference's 8192-chunk tiering; var reads the array twice), axis var
    (two passes: lane means, then squared deviations) and axis argmax.
    GB/s = algorithmic bytes (every pass's read) / time."""
    import torch
    n = R * C_
    stream = torch.cuda.current_stream()
    x = torch.empty((R, C_), device="cuda")
    K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
    cases = {"flat_sum": (lambda: K.sum(x), 4 * n),
             "flat_mean": (lambda: K.mean(x), 4 * n),
             "flat_max": (lambda: K.max(x), 4 * n),
             "flat_var": (lambda: K.var(x), 8 * n),
             "var_axis0": (lambda: K.var(x, 0), 8 * n),
             "var_axis1": (lambda: K.var(x, 1), 8 * n),
             "argmax_axis1": (lambda: K.argmax(x, 1), 4 * n),
             "argmax_flat": (lambda: K.argmax(x), 4 * n)}
    out = {}
    for name, (fn, nbytes) in cases.items():
        ms = _time_ms(fn, 5, stream)
        out[name] = {"ms": round(ms, 4), "gbs": round(nbytes / ms / 1e6, 1)}
    del x
    torch.cuda.empty_cache()
    return out


def scan_section(K, L):
    """Running folds on 16384x16384 f32 N(0,1) (seed 3): cumsum and
    maximum.accumulate along axis 0 (column pipeline), axis 1 (row pipeline)
    and over the flattened array (segmented parallel scan), each one call;
    algorithmic bytes = read + write of the array (8 B/elem)."""
    import torch
    n = R * C_
    stream = torch.cuda.current_stream()
    x = torch.empty((R, C_), device="cuda")
    K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
    cases = {"cumsum_axis0": lambda: K.cumsum(x, 0),
             "cumsum_axis1": lambda: K.cumsum(x, 1),
             "cumsum_flat": lambda: K.cumsum(x),
             "maximum_accumulate_axis1": lambda: K.ufunc_accumulate("maximum", x, 1),
             "maximum_accumulate_axis0": lambda: K.ufunc_accumulate("maximum", x, 0),
             "maximum_accumulate_flat": lambda: K.ufunc_accumulate("maximum", x, None)}
    out = {}
    for name, fn in cases.items():
        ms = _time_ms(fn, 5, stream)
        out[name] = {"ms": round(ms, 4), "gbs": round(8 * n / ms / 1e6, 1)}
    del x
    torch.cuda.empty_cache()
    return out


def io_section(K, L):
    """NPY straight to / from device memory (io::npy_npz): a 16384x16384 f32
    array (1 GiB) saved with save_npy and loaded with load_npy through the
    page cache of a temporary directory, beside a single-threaded host read
    of the same file into a host array (the shape of the reference's
    read_exact + decode)."""
    import tempfile
    import numpy as np
    import torch
    x = torch.empty((R, C_), device="cuda")
    K.fill_random(x, L.RNG_NORMAL, 3, 0.0, 1.0)
    nbytes = x.numel() * 4
    out = {}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "x.npy")
        K.save_npy(path, x)  # warm the page cache
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        K.save_npy(path, x)
        torch.cuda.synchronize()
        out["save_npy_gbs"] = round(nbytes / (time.perf_counter() - t0) / 1e9, 2)
        K.load_npy(path)
        torch.cuda.synchronize()
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            y = K.load_npy(path)
        torch.cuda.synchronize()
        out["load_npy_gbs"] = round(reps * nbytes / (time.perf_counter() - t0) / 1e9, 2)
        out["load_bit_exact"] = bool(torch.equal(x.view(torch.int32), y.view(torch.int32)))
        t0 = time.perf_counter()
        with open(path, "rb") as f:
            f.seek(K.npy_info(path)["data_offset"])
            host = np.fromfile(f, dtype=np.float32, count=R * C_)
        out["host_read_gbs"] = round(nbytes / (time.perf_counter() - t0) / 1e9, 2)
        del host, y
    del x
    torch.cuda.empty_cache()
    out["bytes"] = nbytes
    return out


def grouped_section(K, L, seed: int = 7, cpu: bool = True, peaks=None):
    """C4: 4096 GEMMs (M, N, K log-uniform in [16, 512], half f32 / half f64)
    and 4096 row reductions (length log-uniform in [64, 65536]) in one
    persistent launch replayed from a CUDA graph: untuned, with the f64
    GEMMs on the tensor cores, as chosen by the plan-level autotuner
    (nrs_plan_autotune, which also tries the f32 GEMMs on the tensor cores),
    and launched one by one. Roofline: the time the group needs at the
    measured rates (f64 and f32 flops at the DMMA / FMA rates, or as BF16
    slice products at the BF16 rate for the GEMMs the plan puts on the
    tensor cores; reduction bytes at the HBM copy rate) over the measured
    time."""
    import numpy as np
    import torch
    r = np.random.default_rng(seed)
    lu = lambda lo, hi, n: np.exp(r.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)  # noqa: E731
    M, N, Kd = lu(16, 512, 4096), lu(16, 512, 4096), lu(16, 512, 4096)
    gemms = []
    f32_flops = f64_flops = 0.0
    for i in range(4096):
        dt = torch.float32 if i % 2 == 0 else torch.float64
        a = torch.empty((int(M[i]), int(Kd[i])), dtype=dt, device="cuda").uniform_(-1, 1)
        b = torch.empty((int(Kd[i]), int(N[i])), dtype=dt, device="cuda").uniform_(-1, 1)
        c = torch.empty((int(M[i]), int(N[i])), dtype=dt, device="cuda")
        gemms.append((a, b, c, False))
        if dt == torch.float32:
            f32_flops += 2.0 * M[i] * N[i] * Kd[i]
        else:
            f64_flops += 2.0 * M[i] * N[i] * Kd[i]
    flops = f32_flops + f64_flops
    lens = lu(64, 65536, 4096)
    reds = []
    rbytes = 0
    for i in range(4096):
        x = torch.randn(int(lens[i]), device="cuda")
        reds.append((x, L.SUM, torch.empty(1, device="cuda")))
        rbytes += int(lens[i]) * 4
    stream = torch.cuda.current_stream()
    K.tuner_clear()
    plan_h = K.Plan(gemms, reds)
    ms_h = _event_median_ms(lambda: plan_h.run(use_graph=True), 5, stream)
    plan_h.close()
    # f64 GEMMs on the tensor cores, slice count from each problem's spread
    plan_o = K.Plan(gemms, reds, f64_mode=L.PLAN_F64_OZAKI)
    n_tc, oz_s, _ = plan_o.f64_info()
    ms_o = _event_median_ms(lambda: plan_o.run(use_graph=True), 5, stream)
    plan_o.close()
    t_tune = time.perf_counter()
    rep = K.autotune_plan(gemms, reds, max_trials=48, reps=3, f64_ozaki=True, f32_ozaki=True)
    tune_s = time.perf_counter() - t_tune
    plan = K.Plan(gemms, reds, **rep["plan_kwargs"])
    st = plan.stats()
    n_tc_final, s_final, b_final = plan.f64_info()
    n32_final, s32_final, _ = plan.f32_info()
    ms_g = _event_median_ms(lambda: plan.run(use_graph=True), 5, stream)
    K.tuner_clear()

    def one_by_one():
        for a, b, c, _ in gemms:
            K.gemm_2d(a.shape[0], a.shape[1], b.shape[1], a, b, c)
        for x, op, o in reds:
            K.reduce(x, op)
    ms_1 = _time_ms(one_by_one, 1, stream)
    plan.close()
    out = {"gemms": 4096, "row_reductions": 4096, "work_items": st["work_items"],
           "grouped_graph_ms": round(ms_g, 3), "untuned_graph_ms": round(ms_h, 3),
           "f64_on_tensor_cores_untuned_ms": round(ms_o, 3),
           "f64_tensor_core_gemms": n_tc_final, "f64_slices": s_final, "f64_digit_bits": b_final,
           "f32_tensor_core_gemms": n32_final, "f32_slices": s32_final,
           "f64_tensor_core_gemms_auto": n_tc, "f64_slices_auto": oz_s,
           "one_by_one_ms": round(ms_1, 3), "speedup_vs_one_by_one": round(ms_1 / ms_g, 2),
           "gflops": round(flops / ms_g / 1e6, 1), "f64_share_of_flops": round(f64_flops / flops, 3),
           "reduce_bytes": rbytes,
           "autotune": {"seconds": round(tune_s, 2), "buckets": rep["buckets"], "trials": rep["trials"],
                        "untuned_ms": round(rep["untuned_ms"], 3), "isolated_buckets_ms": round(rep["isolated_ms"], 3),
                        "ozaki_mode_ms": round(rep["ozaki_ms"], 3),
                        "ozaki_f32_mode_ms": round(rep["ozaki_f32_ms"], 3), "final_ms": round(rep["final_ms"], 3),
                        "chosen": rep["plan_kwargs"]}}
    if peaks:
        # each part at its measured rate: f64 on DMMA or as BF16 slice
        # products, f32 on FMA or as BF16 slice products, reductions at HBM
        if n32_final:
            f32_t = f32_flops * s32_final * (s32_final + 1) / 2 / (_bf16_peak() * 1e12)
            f32_part = "f32 as BF16 slice products"
        else:
            f32_t = f32_flops / (peaks["fp32_fma_tflops"] * 1e12)
            f32_part = "f32 FMA"
        red_t = rbytes / (_peaks()[0] * 1e9)
        dmma_t = f64_flops / (peaks["fp64_dmma_tflops"] * 1e12)
        if n_tc_final:
            bf16_t = f64_flops * s_final * (s_final + 1) / 2 / (_bf16_peak() * 1e12)
            t_lb, bound = (bf16_t + f32_t + red_t) * 1e3, f"mixed: f64 as BF16 slice products + {f32_part} + HBM"
        else:
            t_lb, bound = (dmma_t + f32_t + red_t) * 1e3, f"mixed: f64 DMMA + {f32_part} + HBM"
        out["roofline"] = {"bound": bound, "kernel": "ozaki_tc_kernel (grouped) + grouped_kernel",
                           "lower_bound_ms": round(t_lb, 3), "achieved_ms": round(ms_g, 3),
                           "frac": round(t_lb / ms_g, 4), "unit": "ms",
                           "f64_dmma_floor_ms": round(dmma_t * 1e3, 3)}
    if cpu:
        # the oracle's gemm_2d / reduce::sum restatements over the first 256
        # GEMMs and 256 reductions of the same group, scaled to the 4096 + 4096
        from oracle import Oracle
        ora = Oracle()
        sample = 256
        ga = [(a.cpu().numpy(), b.cpu().numpy()) for a, b, _, _ in gemms[:sample]]
        ra = [x.cpu().numpy() for x, _, _ in reds[:sample]]
        t0 = time.perf_counter()
        for a, b in ga:
            ora.gemm(a, b)
        for x in ra:
            ora.flat("sum", x)
        t_s = time.perf_counter() - t0
        s_flops = sum(2.0 * a.shape[0] * a.shape[1] * b.shape[1] for a, b in ga)
        s_work = s_flops + sum(x.nbytes for x in ra)
        out["cpu_baseline"] = {"value": round(t_s * (flops + rbytes) / s_work * 1e3, 1),
                               "unit": "ms (whole group, scaled by work)", "cores": ora.num_threads(), "kind": "port",
                               "sample": f"first {sample} GEMMs + {sample} reductions of the group, {t_s:.2f} s",
                               "gflops": round(s_flops / t_s / 1e9, 2)}
    return out


def selector_section(holdout: int = 300):
    """C5: the MLP selector trained on the GPU on the committed autotuner
    timings of this GPU model, evaluated on `holdout` shapes drawn now
    (another seed of the same distribution) and tuned exhaustively: regret
    against exhaustive tuning, beside the size heuristic's, and the tuning
    time the selector saves."""
    import tune_selector as TS
    path = os.path.join(ROOT, "tests", "golden", "selector_timings_gb300.npz")
    if not os.path.exists(path):
        return {"unavailable": "no committed selector timings"}
    t0 = time.perf_counter()
    res, sel = TS.run_from_timings(path, holdout, seed=4242, reps=1)
    sel.close()
    res["seconds"] = round(time.perf_counter() - t0, 2)
    res["target"] = "selector throughput within 5% of exhaustive tuning (>= 0.95)"
    res["meets_target"] = res["selector"]["throughput_vs_exhaustive"] >= 0.95
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=R, help="rows of the CPU baseline's sample (default: all)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-gemm", action="store_true")
    ap.add_argument("--quick-gemm", action="store_true", help="2048^3 instead of 8192^3")
    ap.add_argument("--no-grouped", action="store_true")
    ap.add_argument("--no-selector", action="store_true")
    ap.add_argument("--no-elementwise", action="store_true")
    ap.add_argument("--no-scan", action="store_true")
    ap.add_argument("--no-io", action="store_true")
    ap.add_argument("--no-extra", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from numrs_gb300 import _lib as L
    from numrs_gb300 import kernels as K
    lib = L.load()

    x32 = torch.empty((R, C_), dtype=torch.float32, device="cuda")
    x64 = torch.empty((R, C_), dtype=torch.int64, device="cuda")
    K.fill_random(x32, L.RNG_NORMAL, F32_SEED, 0.0, 1.0)
    K.fill_random(x64, L.RNG_INT, I64_SEED, -(1 << 20), float(1 << 21))
    ops, y = build_ops(K, x32, x64)
    step_bytes = sum(b for _, b, _ in ops)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        for _, _, fn in ops:
            fn()
    barrier()
    stream = torch.cuda.current_stream()
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in ops]
          for _ in range(args.steps)]
    clocks = Clocks(local)
    time.sleep(0.3)
    barrier()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    launches = 0
    for s_i in range(args.steps):
        for i, (cls, _, fn) in enumerate(ops):
            ev[s_i][i][0].record(stream)
            fn()
            ev[s_i][i][1].record(stream)
            launches += 1
    t_end.record(stream)
    barrier()
    per_class: dict[str, list[float]] = {}
    for s_i in range(args.steps):
        for i, (cls, _, _) in enumerate(ops):
            per_class.setdefault(cls, []).append(ev[s_i][i][0].elapsed_time(ev[s_i][i][1]))
    clk = clocks.stop()
    ms_total = max_over_ranks(t_start.elapsed_time(t_end), dist, "cuda")
    ms_per_step = ms_total / args.steps
    value = whole_job_gbs(step_bytes, world, ms_per_step)

    peak, peak_kind = _peaks()
    # per kernel class: algorithmic bytes per launch / mean launch time
    bytes_of = {}
    for cls, b, _ in ops:
        bytes_of.setdefault(cls, []).append(b)
    kernels = {}
    for cls, ts in per_class.items():
        avg_ms = sum(ts) / len(ts)
        avg_b = sum(bytes_of[cls]) / len(bytes_of[cls])
        gbs = avg_b / (avg_ms / 1e3) / 1e9
        kernels[cls] = {"launches_per_step": len(bytes_of[cls]), "avg_ms": round(avg_ms, 4),
                        "median_ms": round(statistics.median(ts), 4), "timed_launches": len(ts),
                        "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4),
                        "share": round(sum(ts) / sum(sum(v) for v in per_class.values()), 4)}
    dom = max(kernels, key=lambda c: kernels[c]["share"])
    traffic = profiled_traffic(dom)

    out = {"metric": "reduce GB/s", "value": round(value, 1), "unit": "GB/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64",
           "data": "synthetic (SplitMix64, seeds 3/4)",
           "config": dict(CONFIG, bytes_per_step=step_bytes, parallelism=f"replicas x{world}"),
           "gpu_launches": launches,
           "roofline": {"bound": "hbm", "kernel": dom, "achieved": kernels[dom]["achieved_gbs"],
                        "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                        "frac": kernels[dom]["frac"], "traffic": traffic},
           "kernels": kernels, "clocks": clk}

    # ---- end to end through the C ABI with pinned host buffers --------------
    if not args.no_e2e:
        h = K.handle()
        nb32, nb64 = R * C_ * 4, R * C_ * 8
        hp32, hp64, hy = C.c_void_p(), C.c_void_p(), C.c_void_p()
        L.check(lib.nrs_host_alloc(h, nb32, C.byref(hp32)), h)
        L.check(lib.nrs_host_alloc(h, nb64, C.byref(hp64)), h)
        L.check(lib.nrs_host_alloc(h, nb32, C.byref(hy)), h)
        L.check(lib.nrs_memcpy_d2h(h, hp32, C.c_void_p(x32.data_ptr()), nb32), h)
        L.check(lib.nrs_memcpy_d2h(h, hp64, C.c_void_p(x64.data_ptr()), nb64), h)
        L.check(lib.nrs_synchronize(h), h)
        # Two extra handles on their own non-blocking streams carry the bulk
        # copies (H2D and D2H use separate copy engines); CUDA events order
        # them against the compute on the current stream, so the i64 upload
        # and the ufunc download overlap the f32 reductions. The i64 array
        # lands in E2E_BLOCKS row blocks and each block is reduced as soon as
        # it is in: reductions whose lanes are rows write their block's slice
        # of the result, the others a per-block partial that one more
        # nrs_reduce folds over the blocks (integer sum and max: exact in any
        # grouping), so only the last block's reductions trail the link.
        h_in, h_out = C.c_void_p(), C.c_void_p()
        L.check(lib.nrs_create(local, C.byref(h_in)))
        L.check(lib.nrs_create(local, C.byref(h_out)))
        s_in = torch.cuda.ExternalStream(lib.nrs_get_stream(h_in))
        s_out = torch.cuda.ExternalStream(lib.nrs_get_stream(h_out))
        ev32, evy = torch.cuda.Event(), torch.cuda.Event()
        ev64 = [torch.cuda.Event() for _ in range(E2E_BLOCKS)]
        cur = torch.cuda.current_stream()
        f32_ops = [fn for cls, _, fn in ops if cls.endswith("/f32") and not cls.startswith("exp")]
        rb = R // E2E_BLOCKS
        blk = rb * C_ * 8
        # (view, op, axis, lanes are x64 rows) for the eight i64 reductions
        i64_red = [(vn, code, axis, axis == (1 if vn == "rm" else 0))
                   for vn in ("rm", "tr") for code in (L.SUM, L.MAX) for axis in (0, 1)]
        i64_res = [torch.empty(C_, dtype=torch.int64, device=x64.device) for _ in i64_red]
        i64_part = [None if rows else torch.empty((E2E_BLOCKS, C_), dtype=torch.int64, device=x64.device)
                    for (_, _, _, rows) in i64_red]

        # Three more handles on their own streams: a block's eight reductions
        # run on four streams at once (the lanes-along-rows ones use few CTAs
        # on a block's rows, so alone they would not fill the GPU).
        hx = [h]
        for _ in range(3):
            hh = C.c_void_p()
            L.check(lib.nrs_create(local, C.byref(hh)))
            hx.append(hh)
        sx = [cur] + [torch.cuda.ExternalStream(lib.nrs_get_stream(hh)) for hh in hx[1:]]
        evx = [torch.cuda.Event() for _ in sx]
        ev_done = torch.cuda.Event()

        def reduce_into(hh, view, code, axis, out):
            L.check(lib.nrs_reduce(hh, L.I64, code, view.dim(), L.i64_array(view.shape),
                                   L.i64_array(view.stride()), axis, 0, C.c_void_p(view.data_ptr()),
                                   C.c_void_p(out.data_ptr())), hh)

        def i64_block(b):
            xb = x64[b * rb:(b + 1) * rb]
            for k in range(len(sx)):
                sx[k].wait_event(ev64[b])
            for j, (vn, code, axis, rows) in enumerate(i64_red):
                v = xb if vn == "rm" else xb.t()
                reduce_into(hx[j % len(hx)], v, code, axis,
                            i64_res[j][b * rb:(b + 1) * rb] if rows else i64_part[j][b])

        res_host = {}

        def d2h_small(r, key):
            # result reads go on the download stream, after ev_done
            nbytes = r.numel() * r.element_size()
            if key not in res_host:
                res_host[key] = torch.empty(r.shape, dtype=r.dtype, pin_memory=True)
            L.check(lib.nrs_memcpy_d2h(h_out, C.c_void_p(res_host[key].data_ptr()), C.c_void_p(r.data_ptr()),
                                       nbytes), h_out)
            return nbytes

        def e2e_step():
            L.check(lib.nrs_memcpy_h2d(h_in, C.c_void_p(x32.data_ptr()), hp32, nb32), h_in)
            ev32.record(s_in)
            for b in range(E2E_BLOCKS):
                L.check(lib.nrs_memcpy_h2d(h_in, C.c_void_p(x64.data_ptr() + b * blk),
                                           C.c_void_p(hp64.value + b * blk), blk), h_in)
                ev64[b].record(s_in)
            cur.wait_event(ev32)
            K.exp_affine(x32, A_SCALE, B_SHIFT, out=y)
            evy.record(cur)
            s_out.wait_event(evy)
            L.check(lib.nrs_memcpy_d2h(h_out, hy, C.c_void_p(y.data_ptr()), nb32), h_out)
            d2h = nb32
            f32_res = [fn() for fn in f32_ops]
            for b in range(E2E_BLOCKS):
                i64_block(b)
            for k in range(1, len(sx)):
                evx[k].record(sx[k])
                cur.wait_event(evx[k])
            for j, (_, code, _, rows) in enumerate(i64_red):
                if not rows:
                    reduce_into(h, i64_part[j], code, 0, i64_res[j])
            ev_done.record(cur)
            s_out.wait_event(ev_done)
            for i, r in enumerate(f32_res):
                d2h += d2h_small(r, ("f32", i))
            for j, r in enumerate(i64_res):
                d2h += d2h_small(r, ("i64", j))
            for hh in (h_in, h_out, *hx):
                L.check(lib.nrs_synchronize(hh), hh)
            return d2h

        # The host link alone: the best of three 1 GiB pinned copies each way
        # (H2D and D2H), on the copy streams the step uses; the step cannot
        # beat its H2D bytes at the H2D rate.
        def link_gbs(fn, nbytes):
            best = float("inf")
            for _ in range(3):
                t0 = time.perf_counter()
                fn()
                best = min(best, time.perf_counter() - t0)
            return nbytes / best / 1e9
        h2d_gbs = link_gbs(lambda: (L.check(lib.nrs_memcpy_h2d(h_in, C.c_void_p(x32.data_ptr()), hp32, nb32), h_in),
                                    L.check(lib.nrs_synchronize(h_in), h_in)), nb32)
        d2h_gbs = link_gbs(lambda: (L.check(lib.nrs_memcpy_d2h(h_out, hy, C.c_void_p(x32.data_ptr()), nb32), h_out),
                                    L.check(lib.nrs_synchronize(h_out), h_out)), nb32)
        e2e_step()
        # the blocked i64 reductions give the whole-array results bit for bit
        for j, (vn, code, axis, _) in enumerate(i64_red):
            want = K.reduce(x64 if vn == "rm" else x64.t(), code, axis)
            if not torch.equal(want, i64_res[j]):
                raise RuntimeError(f"blocked i64 reduction {j} differs from the whole-array one")
        e2e_step()
        barrier()
        # Each step is timed on its own (host clock around the step, which
        # ends synchronised). The host link is shared with the machine's other
        # GPUs: single steps intermittently ran 1.5-3x long with both copy
        # directions slowed, so the value is the median step, with the mean
        # and the slowest step beside it.
        e_steps = max(5, min(args.steps, 9))
        times = []
        for _ in range(e_steps):
            t0 = time.perf_counter()
            d2h = e2e_step()
            times.append(time.perf_counter() - t0)
        barrier()
        dt = max_over_ranks(statistics.median(times), dist, "cuda")
        out["e2e"] = {"value": round(whole_job_gbs(step_bytes, world, dt * 1e3), 1), "unit": "GB/s",
                      "h2d_bytes_per_step": nb32 + nb64, "d2h_bytes_per_step": d2h,
                      "ms_per_step": round(dt * 1e3, 3), "steps": e_steps, "stat": "median",
                      "ms_per_step_mean": round(sum(times) / len(times) * 1e3, 3),
                      "ms_per_step_max": round(max(times) * 1e3, 3),
                      "link": {"h2d_gbs": round(h2d_gbs, 1), "d2h_gbs": round(d2h_gbs, 1),
                               "h2d_bound_ms": round((nb32 + nb64) / h2d_gbs / 1e6, 3),
                               "frac": round((nb32 + nb64) / h2d_gbs / 1e6 / (dt * 1e3), 3)}}
        for p in (hp32, hp64, hy):
            lib.nrs_host_free(h, p)
        for hh in (h_in, h_out, *hx[1:]):
            lib.nrs_destroy(hh)

    # ---- CPU baseline (rank 0, N = 1 only) ------------------------------------
    if rank == 0 and world == 1 and not args.no_cpu:
        # the device arrays themselves, copied to the host: the same inputs
        rows = args.cpu_rows
        x32n = x32[:rows].cpu().numpy()
        x64n = x64[:rows].cpu().numpy()
        nbytes, times, cores, sample = cpu_sample(None, args.cpu_seconds, x32n, x64n)
        del x32n, x64n
        t = sum(times)
        out["cpu_baseline"] = {"value": round(nbytes * len(times) / t / 1e9, 2), "unit": "GB/s",
                               "cores": cores, "kind": "port", "sample": sample,
                               "passes": len(times), "seconds": round(t, 2)}
    if rank == 0 and not args.no_gemm:
        del x32, x64, y
        ops = None
        torch.cuda.empty_cache()
        out["gemm"] = gemm_section(K, L, quick=args.quick_gemm, cpu=not args.no_cpu)
    if rank == 0 and not args.no_elementwise:
        out["elementwise"] = elementwise_section(K, L)
    if rank == 0 and not args.no_extra:
        out["reductions_extra"] = reductions_extra_section(K, L)
    if rank == 0 and not args.no_scan:
        out["scan"] = scan_section(K, L)
    if rank == 0 and not args.no_io:
        out["io"] = io_section(K, L)
    if rank == 0 and not args.no_grouped:
        out["grouped"] = grouped_section(K, L, cpu=not args.no_cpu,
                                         peaks=(out.get("gemm") or {}).get("peaks") or _gemm_peaks(K, L))
    if rank == 0 and not args.no_selector:
        out["selector"] = selector_section()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
