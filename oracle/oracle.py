"""ctypes front end of the CPU oracle (test infrastructure; see ``oracle.c``).

``build()`` compiles ``oracle.c`` with gcc into ``oracle/_build/liboracle.so``
(OpenMP on, FP contraction off, no host-specific ``-march``), so the same
recipe works on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "oracle.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB = os.path.join(_OUT_DIR, "liboracle.so")
_lock = threading.Lock()
_lib = None

SUM, MEAN, MAX, MIN, PROD = 0, 1, 2, 3, 4
ADD, SUB, MUL, DIV = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile the oracle shared library (idempotent unless ``force``)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC):
        return _LIB
    tmp = _LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", _SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


def load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = C.CDLL(_LIB)
            _declare(_lib)
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _declare(L):
    vp, i64, u64, f32, f64, i32 = C.c_void_p, C.c_int64, C.c_uint64, C.c_float, C.c_double, C.c_int
    for suf, T in (("f32", f32), ("f64", f64)):
        for name in ("sum", "mean", "min", "max", "prod"):
            fn = getattr(L, f"orc_{name}_{suf}")
            fn.argtypes, fn.restype = [vp, i64], T
        fn = getattr(L, f"orc_var_{suf}")
        fn.argtypes, fn.restype = [vp, i64, i64], T
        fn = getattr(L, f"orc_sum_sq_dev_{suf}")
        fn.argtypes, fn.restype = [vp, i64, T], T
        fn = getattr(L, f"orc_axis_{suf}")
        fn.argtypes, fn.restype = [i32, i32, vp, vp, i32, vp, vp], None
        fn = getattr(L, f"orc_binary_{suf}")
        fn.argtypes, fn.restype = [i32, i32, vp, vp, vp, vp, vp, vp], None
        fn = getattr(L, f"orc_gemm_{suf}")
        fn.argtypes, fn.restype = [i64, i64, i64, vp, i64, vp, i64, vp, i64], None
        fn = getattr(L, f"orc_exp_affine_{suf}")
        fn.argtypes, fn.restype = [vp, i64, T, T, vp], None
    for name in ("sum", "max", "min", "prod"):
        fn = getattr(L, f"orc_{name}_i64")
        fn.argtypes, fn.restype = [vp, i64], i64
    L.orc_axis_i64.argtypes, L.orc_axis_i64.restype = [i32, i32, vp, vp, i32, vp, vp], None
    L.orc_binary_i64.argtypes, L.orc_binary_i64.restype = [i32, i32, vp, vp, vp, vp, vp, vp], None
    L.orc_gemm_i64.argtypes, L.orc_gemm_i64.restype = [i64, i64, i64, vp, i64, vp, i64, vp, i64], None
    L.orc_exp_affine_eager_f32.argtypes = [vp, i64, f32, f32, vp, vp]
    L.orc_exp_affine_eager_f32.restype = None
    L.orc_gemm_dd.argtypes, L.orc_gemm_dd.restype = [i64, i64, i64, vp, i64, vp, i64, vp, vp], None
    L.orc_gemm_dd_sampled.argtypes = [i64, vp, i64, vp, i64, i64, vp, vp, vp, vp]
    L.orc_gemm_dd_sampled.restype = None
    L.orc_splitmix64_at.argtypes, L.orc_splitmix64_at.restype = [u64, u64], u64
    L.orc_gen_uniform_pm1_f64.argtypes, L.orc_gen_uniform_pm1_f64.restype = [u64, i64, vp], None
    L.orc_gen_uniform_pm1_f32.argtypes, L.orc_gen_uniform_pm1_f32.restype = [u64, i64, vp], None
    L.orc_gen_i64.argtypes, L.orc_gen_i64.restype = [u64, i64, vp], None
    L.orc_gen_normal_f32.argtypes, L.orc_gen_normal_f32.restype = [u64, i64, f64, f64, vp], None
    L.orc_num_threads.argtypes, L.orc_num_threads.restype = [], i32
    L.orc_set_threads.argtypes, L.orc_set_threads.restype = [i32], None
    L.orc_mlp_forward_backward.argtypes = [i64, i64, i64, i64] + [vp] * 16
    L.orc_mlp_forward_backward.restype = f32
    for suf in ("f32", "f64"):
        fn = getattr(L, f"orc_axis_var_{suf}")
        fn.argtypes, fn.restype = [i32, vp, vp, i32, i64, i32, vp, vp], None
    for suf in ("f32", "f64", "i64"):
        fn = getattr(L, f"orc_axis_arg_{suf}")
        fn.argtypes, fn.restype = [i32, i32, vp, vp, i32, vp, vp], None
        fn = getattr(L, f"orc_flat_arg_{suf}")
        fn.argtypes, fn.restype = [i32, vp, i64], i64
    for suf, T in (("f32", f32), ("f64", f64), ("i64", i64)):
        fn = getattr(L, f"orc_ufunc_reduce_{suf}")
        fn.argtypes, fn.restype = [i32, i32, vp, vp, i32, i32, T, vp, vp], i32
        fn = getattr(L, f"orc_accumulate_{suf}")
        fn.argtypes, fn.restype = [i32, i32, vp, vp, i32, vp, vp], None


_SUF = {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64", np.dtype(np.int64): "i64"}


class Oracle:
    """Thin numpy-facing wrapper around the restated reference kernels."""

    def __init__(self):
        self.L = load()

    # -- threads -----------------------------------------------------------
    def num_threads(self) -> int:
        return self.L.orc_num_threads()

    def set_threads(self, n: int) -> None:
        self.L.orc_set_threads(int(n))

    # -- flat reductions (kernels::reduce) ----------------------------------
    def flat(self, op: str, a: np.ndarray, ddof: int = 0):
        a = np.ascontiguousarray(a)
        suf = _SUF[a.dtype]
        if op == "var":
            return getattr(self.L, f"orc_var_{suf}")(_p(a), a.size, ddof)
        return getattr(self.L, f"orc_{op}_{suf}")(_p(a), a.size)

    def sum_sq_dev(self, a: np.ndarray, mean: float):
        a = np.ascontiguousarray(a)
        return getattr(self.L, f"orc_sum_sq_dev_{_SUF[a.dtype]}")(_p(a), a.size, mean)

    # -- axis folds (math::sum/mean/max/min, Array::sum_axis) ----------------
    def axis(self, op: int, x: np.ndarray, axis: int, base: np.ndarray | None = None) -> np.ndarray:
        """Fold ``x`` (any strided numpy view) along ``axis``.

        The element strides are taken from the view; ``base`` is the buffer
        the view points into (defaults to the view's own base array)."""
        if axis < 0:
            axis += x.ndim
        suf = _SUF[x.dtype]
        item = x.dtype.itemsize
        shape = np.array(x.shape, dtype=np.int64)
        strides = np.array([s // item for s in x.strides], dtype=np.int64)
        out_shape = [d for i, d in enumerate(x.shape) if i != axis]
        out_dtype = np.float64 if (suf == "i64" and op == MEAN) else x.dtype
        out = np.empty(out_shape if out_shape else [1], dtype=out_dtype)
        # pointer to x's first element; strides may be negative-free views only
        ptr = C.c_void_p(x.__array_interface__["data"][0])
        fn = getattr(self.L, f"orc_axis_{suf}")
        fn(op, x.ndim, _p(shape), _p(strides), axis, ptr, _p(out))
        return out

    def _view_args(self, x, axis):
        if axis < 0:
            axis += x.ndim
        item = x.dtype.itemsize
        shape = np.array(x.shape, dtype=np.int64)
        strides = np.array([s // item for s in x.strides], dtype=np.int64)
        out_shape = [d for i, d in enumerate(x.shape) if i != axis]
        return axis, shape, strides, (out_shape if out_shape else [1])

    def axis_var(self, x: np.ndarray, axis: int, ddof: int = 0, std: bool = False) -> np.ndarray:
        """math::statistics::var/std(axis, ddof) restated (two passes per lane)."""
        axis, shape, strides, out_shape = self._view_args(x, axis)
        out = np.empty(out_shape, dtype=x.dtype)
        getattr(self.L, f"orc_axis_var_{_SUF[x.dtype]}")(
            x.ndim, _p(shape), _p(strides), axis, ddof, int(std),
            C.c_void_p(x.__array_interface__["data"][0]), _p(out))
        return out

    def axis_arg(self, x: np.ndarray, axis, want_max: bool) -> np.ndarray:
        """math::statistics::argmax/argmin restated (axis=None: flattened)."""
        if axis is None:
            flat = np.ascontiguousarray(x).ravel()
            return np.array([getattr(self.L, f"orc_flat_arg_{_SUF[x.dtype]}")(int(want_max), _p(flat), flat.size)],
                            dtype=np.int64)
        axis, shape, strides, out_shape = self._view_args(x, axis)
        out = np.empty(out_shape, dtype=np.int64)
        getattr(self.L, f"orc_axis_arg_{_SUF[x.dtype]}")(
            int(want_max), x.ndim, _p(shape), _p(strides), axis,
            C.c_void_p(x.__array_interface__["data"][0]), _p(out))
        return out

    # -- ufunc reduce / accumulate ----------------------------------------
    def ufunc_reduce(self, op: int, x: np.ndarray, axis=None, initial=None) -> np.ndarray:
        """ufunc_ops::ufunc_reduce restated (op codes of nrs_ufunc). Returns
        the values in row-major order over the kept dims (one value when
        axis is None); raises ValueError where the reference errors."""
        item = x.dtype.itemsize
        shape = np.array(x.shape if x.ndim else [1], dtype=np.int64)
        strides = np.array([s // item for s in x.strides] if x.ndim else [1], dtype=np.int64)
        nd = max(x.ndim, 1)
        if axis is None:
            ax, n_out = -1, 1
        else:
            ax = axis + x.ndim if axis < 0 else axis
            n_out = int(np.prod([d for i, d in enumerate(x.shape) if i != ax]))
        out = np.empty(max(n_out, 1), dtype=x.dtype)
        rc = getattr(self.L, f"orc_ufunc_reduce_{_SUF[x.dtype]}")(
            op, nd, _p(shape), _p(strides), ax, int(initial is not None),
            0 if initial is None else initial, C.c_void_p(x.__array_interface__["data"][0]), _p(out))
        if rc != 0:
            raise ValueError("zero-size array to reduction operation which has no identity")
        return out[:n_out]

    def accumulate(self, op: int, x: np.ndarray, axis=None) -> np.ndarray:
        """ufunc_accumulate / cumsum / cumprod restated: the full shape in
        row-major order for an axis, the flattened n values for None."""
        item = x.dtype.itemsize
        shape = np.array(x.shape if x.ndim else [1], dtype=np.int64)
        strides = np.array([s // item for s in x.strides] if x.ndim else [1], dtype=np.int64)
        nd = max(x.ndim, 1)
        ax = -1 if axis is None else (axis + x.ndim if axis < 0 else axis)
        out = np.empty(x.shape if axis is not None else (x.size,), dtype=x.dtype)
        getattr(self.L, f"orc_accumulate_{_SUF[x.dtype]}")(
            op, nd, _p(shape), _p(strides), ax, C.c_void_p(x.__array_interface__["data"][0]), _p(out))
        return out

    # -- elementwise ------------------------------------------------------
    def exp_affine(self, x: np.ndarray, a: float, b: float) -> np.ndarray:
        x = np.ascontiguousarray(x)
        y = np.empty_like(x)
        getattr(self.L, f"orc_exp_affine_{_SUF[x.dtype]}")(_p(x), x.size, a, b, _p(y))
        return y

    def exp_affine_eager(self, x: np.ndarray, a: float, b: float) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty_like(x)
        tmp = np.empty_like(x)
        self.L.orc_exp_affine_eager_f32(_p(x), x.size, a, b, _p(tmp), _p(y))
        return y

    def program(self, prog, inputs):
        """Postfix ufunc program over broadcast numpy inputs, one IEEE
        rounding per op (numpy's elementwise float ops never contract), as
        ExprNode's eager evaluation does (src/expr/owned.rs:557; two
        roundings for a*b+c, src/expr/fused_eval.rs:17-21). Codes follow
        nrs_ufunc: INPUT 0, SCALAR 1, ADD 2, SUB 3, MUL 4, DIV 5, NEG 6,
        ABS 7, SQRT 8, EXP 9, LN 10, MAX 11, MIN 12. MAX/MIN keep the left
        operand if it is NaN or strictly greater (smaller). Integer division
        truncates toward zero and gives 0 for a zero divisor or MIN / -1."""
        dt = inputs[0].dtype
        shape = np.broadcast_shapes(*[x.shape for x in inputs])
        ins = [np.broadcast_to(x, shape) for x in inputs]
        st = []
        with np.errstate(all="ignore"):
            for code, arg, scal in prog:
                if code == 0:
                    st.append(np.array(ins[arg], dtype=dt))
                elif code == 1:
                    st.append(np.full(shape, scal, dtype=dt))
                elif code in (6, 7, 8, 9, 10):
                    v = st.pop()
                    f = {6: np.negative, 7: np.abs, 8: np.sqrt, 9: np.exp, 10: np.log}[code]
                    st.append(f(v).astype(dt))
                else:
                    b = st.pop()
                    a = st.pop()
                    if code == 2:
                        r = a + b
                    elif code == 3:
                        r = a - b
                    elif code == 4:
                        r = a * b
                    elif code == 5 and dt.kind == "f":
                        r = a / b
                    elif code == 5:
                        bad = (b == 0) | ((b == -1) & (a == np.iinfo(dt).min))
                        bs = np.where(bad, 1, b)
                        # C division: the remainder takes the dividend's sign,
                        # so (a - rem) / b is exact and truncates toward zero.
                        r = np.where(bad, 0, (a - np.fmod(a, bs)) // bs)
                    elif code == 11:
                        r = np.where((a != a) | (a > b), a, b)
                    else:
                        r = np.where((a != a) | (a < b), a, b)
                    st.append(np.asarray(r).astype(dt))
        assert len(st) == 1
        return st[0]

    def binary(self, op: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        shape = np.broadcast_shapes(a.shape, b.shape)
        ab = np.broadcast_to(a, shape)
        bb = np.broadcast_to(b, shape)
        item = a.dtype.itemsize
        out = np.empty(shape, dtype=a.dtype)
        sh = np.array(shape, dtype=np.int64)
        sa = np.array([s // item for s in ab.strides], dtype=np.int64)
        sb = np.array([s // item for s in bb.strides], dtype=np.int64)
        fn = getattr(self.L, f"orc_binary_{_SUF[a.dtype]}")
        fn(op, len(shape), _p(sh), _p(sa), _p(sb), C.c_void_p(ab.__array_interface__["data"][0]),
           C.c_void_p(bb.__array_interface__["data"][0]), _p(out))
        return out

    # -- GEMM -------------------------------------------------------------
    def gemm(self, A: np.ndarray, B: np.ndarray) -> np.ndarray:
        A = np.ascontiguousarray(A)
        B = np.ascontiguousarray(B)
        m, k = A.shape
        k2, n = B.shape
        assert k == k2
        Cm = np.full((m, n), np.nan if A.dtype.kind == "f" else 0, dtype=A.dtype)
        getattr(self.L, f"orc_gemm_{_SUF[A.dtype]}")(m, k, n, _p(A), k, _p(B), n, _p(Cm), n)
        return Cm

    def matmul(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        """Array::matmul (src/array/linalg.rs:153-266) over batched_gemm
        (:56-136): two 2-D operands go straight to gemm_2d; otherwise a 1-D
        operand is promoted to [1, k] (left) or [k, 1] (right) and KEPT in
        the output shape, the batch axes (all but the last two) broadcast by
        NumPy's rules (Array::broadcast_shape, src/array/manipulation.rs:16),
        and every panel of the row-major broadcast operands is one gemm_2d.
        Errors: ValueError("dimension") for a 0-D operand (DimensionMismatch),
        ValueError("shape") for mismatched inner or batch dimensions
        (ShapeMismatch)."""
        a = np.asarray(a)
        b = np.asarray(b)
        if a.ndim == 2 and b.ndim == 2:
            if a.shape[1] != b.shape[0]:
                raise ValueError("shape")
            return self.gemm(a, b)
        if a.ndim == 1:
            a = a.reshape(1, a.shape[0])
        if b.ndim == 1:
            b = b.reshape(b.shape[0], 1)
        if a.ndim < 2 or b.ndim < 2:
            raise ValueError("dimension")
        m, k = a.shape[-2:]
        k2, n = b.shape[-2:]
        if k != k2:
            raise ValueError("shape")
        ba, bb = a.shape[:-2], b.shape[:-2]
        nd = max(len(ba), len(bb))
        pa, pb = (1,) * (nd - len(ba)) + ba, (1,) * (nd - len(bb)) + bb
        batch = []
        for x, y in zip(pa, pb):
            if x == y or y == 1:
                batch.append(x)
            elif x == 1:
                batch.append(y)
            else:
                raise ValueError("shape")
        batch = tuple(batch)
        af = np.ascontiguousarray(np.broadcast_to(a, batch + (m, k))).reshape(-1, m, k)
        bf = np.ascontiguousarray(np.broadcast_to(b, batch + (k, n))).reshape(-1, k, n)
        out = np.zeros((af.shape[0], m, n), dtype=a.dtype)
        for t in range(af.shape[0]):
            if m and n:
                out[t] = self.gemm(af[t], bf[t]) if k else 0
        return out.reshape(batch + (m, n))

    def gemm_dd(self, A: np.ndarray, B: np.ndarray):
        """Double-double product rounded to f64, and (|A||B|)_ij."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        m, k = A.shape
        n = B.shape[1]
        Cm = np.empty((m, n))
        ab = np.empty((m, n))
        self.L.orc_gemm_dd(m, k, n, _p(A), k, _p(B), n, _p(Cm), _p(ab))
        return Cm, ab

    def gemm_dd_sampled(self, A: np.ndarray, B: np.ndarray, rows: np.ndarray, cols: np.ndarray):
        A = np.ascontiguousarray(A, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        k = A.shape[1]
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        cols = np.ascontiguousarray(cols, dtype=np.int64)
        Cv = np.empty(rows.size)
        ab = np.empty(rows.size)
        self.L.orc_gemm_dd_sampled(k, _p(A), A.shape[1], _p(B), B.shape[1], rows.size, _p(rows),
                                   _p(cols), _p(Cv), _p(ab))
        return Cv, ab

    # -- generator twins ---------------------------------------------------
    def splitmix64_at(self, seed: int, i: int) -> int:
        return self.L.orc_splitmix64_at(seed, i)

    def gen_uniform_pm1(self, seed: int, n: int, dtype=np.float64) -> np.ndarray:
        out = np.empty(n, dtype=dtype)
        fn = self.L.orc_gen_uniform_pm1_f64 if dtype == np.float64 else self.L.orc_gen_uniform_pm1_f32
        fn(seed, n, _p(out))
        return out

    def gen_i64(self, seed: int, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.int64)
        self.L.orc_gen_i64(seed, n, _p(out))
        return out

    def gen_normal_f32(self, seed: int, n: int, mu: float = 0.0, sigma: float = 1.0) -> np.ndarray:
        out = np.empty(n, dtype=np.float32)
        self.L.orc_gen_normal_f32(seed, n, mu, sigma, _p(out))
        return out

    # -- MLP selector -------------------------------------------------------
    def mlp_forward_backward(self, x, t, mask, W1, b1, W2, b2, W3, b3):
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, t, mask, W1, b1, W2, b2, W3, b3)]
        x, t, mask, W1, b1, W2, b2, W3, b3 = arrs
        B, F = x.shape
        H = W1.shape[0]
        V = W3.shape[0]
        y = np.empty((B, V), np.float32)
        grads = [np.empty_like(w) for w in (W1, b1, W2, b2, W3, b3)]
        loss = self.L.orc_mlp_forward_backward(B, F, H, V, *[_p(a) for a in arrs], _p(y),
                                               *[_p(g) for g in grads])
        return loss, y, grads
