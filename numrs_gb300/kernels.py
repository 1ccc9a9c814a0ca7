"""Host-side mirror of NumRS2's `kernels` dispatch layer and its Array-level
callers, running on the GB300 through the C ABI.

Arrays are torch CUDA tensors of any strides (torch provides device memory
and streams only; every computation is one of this library's kernels). Work
is enqueued on torch's current stream.

Reference names (numrs2 0.4.1):
  sum / mean / max / min / prod / var / std  -> math::{sum,max,min}
      (src/math/aggregation.rs:416,:160,:289), math::statistics::{mean,var}
      (src/math/statistics/mod.rs:971,:1334), kernels::reduce::*
  sum_axis                                   -> Array::sum_axis (src/array/operations.rs:75)
  gemm_2d                                    -> kernels::gemm::gemm_2d (src/kernels/gemm.rs:246)
  matmul / matmul_to                         -> Array::matmul (src/array/linalg.rs:153),
                                                Array::matmul_to (src/array/operations_optimized.rs:385)
  add / subtract / multiply / divide         -> Add/Sub/Mul/Div for &Array (src/array/arithmetic.rs)
  exp                                        -> ElementWiseMath::exp (src/math/elementwise.rs:145)
  Expr(...).eval()                           -> expr::ExprNode::eval (src/expr/owned.rs:557)
"""
from __future__ import annotations

import builtins as _bi
import ctypes as C
import threading

import torch

from . import _lib as L

_DT = {torch.float32: L.F32, torch.float64: L.F64, torch.int32: L.I32, torch.int64: L.I64}
_handles: dict[int, C.c_void_p] = {}
_hlock = threading.Lock()


def handle(device: int | None = None) -> C.c_void_p:
    """The library handle for `device`, bound to torch's current stream."""
    lib = L.load()
    if device is None:
        device = torch.cuda.current_device()
    with _hlock:
        h = _handles.get(device)
        if h is None:
            h = C.c_void_p()
            L.check(lib.nrs_create(device, C.byref(h)))
            _handles[device] = h
    L.check(lib.nrs_set_stream(h, C.c_void_p(torch.cuda.current_stream(device).cuda_stream)), h)
    return h


def dtype_code(t: torch.Tensor) -> int:
    try:
        return _DT[t.dtype]
    except KeyError:
        raise L.NumRs2Error(L.ERR_DTYPE, f"unsupported dtype {t.dtype}") from None


def _ptr(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _need_cuda(*ts: torch.Tensor) -> None:
    for t in ts:
        if not t.is_cuda:
            raise L.NumRs2Error(L.ERR_INVALID, "arrays must be CUDA tensors (no CPU fallback)")


def synchronize() -> None:
    h = handle()
    L.check(L.load().nrs_synchronize(h), h)


# ---------------------------------------------------------------------------
# Reductions
# ---------------------------------------------------------------------------
def reduce(a: torch.Tensor, op: int, axis: int | None = None, keepdims: bool = False,
           ddof: int = 0) -> torch.Tensor:
    """One reduction through nrs_reduce. Output shape follows the reference:
    the reduced axis removed (or kept as 1 with keepdims); `[1]` when nothing
    is left; a full reduction gives `[1]` (or all-ones dims with keepdims)."""
    _need_cuda(a)
    lib = L.load()
    h = handle(a.device.index)
    code = dtype_code(a)
    nd = a.dim()
    if axis is None:
        out_shape = [1] * nd if keepdims else [1]
        ax = L.AXIS_NONE
    else:
        ax = axis
        norm = axis + nd if axis < 0 else axis
        if 0 <= norm < nd:
            out_shape = list(a.shape)
            if keepdims:
                out_shape[norm] = 1
            else:
                out_shape.pop(norm)
            if not out_shape:
                out_shape = [1]
        else:
            out_shape = [1]
    if op in (L.ARGMAX, L.ARGMIN):
        out_dtype = torch.int64
    else:
        out_dtype = torch.float64 if (op == L.MEAN and code in (L.I32, L.I64)) else a.dtype
    out = torch.empty(out_shape, dtype=out_dtype, device=a.device)
    shape = L.i64_array(a.shape)
    strides = L.i64_array(a.stride())
    st = lib.nrs_reduce(h, code, op, nd, shape, strides, ax, ddof, _ptr(a), _ptr(out))
    L.check(st, h)
    return out


def sum(a, axis=None, keepdims=False):  # noqa: A001 - reference name
    return reduce(a, L.SUM, axis, keepdims)


def mean(a, axis=None, keepdims=False):
    return reduce(a, L.MEAN, axis, keepdims)


def max(a, axis=None, keepdims=False):  # noqa: A001
    return reduce(a, L.MAX, axis, keepdims)


def min(a, axis=None, keepdims=False):  # noqa: A001
    return reduce(a, L.MIN, axis, keepdims)


def prod(a, axis=None, keepdims=False):
    return reduce(a, L.PROD, axis, keepdims)


def var(a, axis=None, ddof=0, keepdims=False):
    return reduce(a, L.VAR, axis, keepdims, ddof)


def std(a, axis=None, ddof=0, keepdims=False):
    return reduce(a, L.STD, axis, keepdims, ddof)


def argmax(a, axis=None, keepdims=False):
    """math::statistics::argmax: int64 indices (first index of the maximum)."""
    return reduce(a, L.ARGMAX, axis, keepdims)


def argmin(a, axis=None, keepdims=False):
    return reduce(a, L.ARGMIN, axis, keepdims)


def sum_axis(a, axis: int):
    """Array::sum_axis: the axis removed, no keepdims, no `[1]` padding."""
    out = reduce(a, L.SUM, axis, False)
    return out.reshape([d for i, d in enumerate(a.shape) if i != axis])


# ---------------------------------------------------------------------------
# Ufunc reduce / accumulate (src/ufunc_ops.rs)
# ---------------------------------------------------------------------------
UFUNC_OPS = {"add": L.OP_ADD, "subtract": L.OP_SUB, "multiply": L.OP_MUL, "divide": L.OP_DIV,
             "maximum": L.OP_MAX, "minimum": L.OP_MIN}
_CSCALAR = {L.F32: C.c_float, L.F64: C.c_double, L.I64: C.c_int64, L.I32: C.c_int32}


def _ufunc_code(op) -> int:
    if isinstance(op, str):
        try:
            return UFUNC_OPS[op]
        except KeyError:
            raise L.NumRs2Error(L.ERR_INVALID, f"unknown ufunc {op!r}") from None
    return int(op)


def ufunc_reduce(op, a: torch.Tensor, axis: int | None = None, keepdims: bool = False,
                 initial=None) -> torch.Tensor:
    """ufunc_ops::ufunc_reduce (src/ufunc_ops.rs:417): `op` is a UfuncOp name
    ("add", "subtract", "multiply", "divide", "maximum", "minimum"). Output
    shape as ufunc_reduce: the axis removed (kept as 1 with keepdims), `[1]`
    for a full reduction (all-ones dims with keepdims)."""
    _need_cuda(a)
    lib = L.load()
    h = handle(a.device.index)
    code = dtype_code(a)
    nd = a.dim()
    if axis is None:
        out_shape = [1] * nd if keepdims else [1]
        ax = L.AXIS_NONE
    else:
        ax = axis
        norm = axis + nd if axis < 0 else axis
        out_shape = [1]
        if 0 <= norm < nd:
            out_shape = list(a.shape)
            if keepdims:
                out_shape[norm] = 1
            else:
                out_shape.pop(norm)
            if not out_shape:
                out_shape = [1]
    out = torch.empty(out_shape, dtype=a.dtype, device=a.device)
    seed = None if initial is None else _CSCALAR[code](initial)
    init = None if seed is None else C.cast(C.pointer(seed), C.c_void_p)
    st = lib.nrs_ufunc_reduce(h, code, _ufunc_code(op), nd, L.i64_array(a.shape),
                              L.i64_array(a.stride()), ax, init, _ptr(a), _ptr(out))
    L.check(st, h)
    return out


def ufunc_accumulate(op, a: torch.Tensor, axis: int | None = None) -> torch.Tensor:
    """ufunc_ops::ufunc_accumulate (src/ufunc_ops.rs:523): the running fold
    along `axis` (same shape as `a`, allocated with `a`'s memory layout when
    that is dense, so a transposed view streams the same way in and out), or
    over the flattened array for axis=None (1-D, `a.numel()` values)."""
    _need_cuda(a)
    lib = L.load()
    h = handle(a.device.index)
    code = dtype_code(a)
    if axis is None:
        out = torch.empty(a.numel(), dtype=a.dtype, device=a.device)
        ax, ostr = L.AXIS_NONE, None
    else:
        out = torch.empty_like(a)
        ax, ostr = axis, L.i64_array(out.stride())
    st = lib.nrs_accumulate(h, code, _ufunc_code(op), a.dim(), L.i64_array(a.shape),
                            L.i64_array(a.stride()), ax, _ptr(a), _ptr(out), ostr)
    L.check(st, h)
    return out


def cumsum(a, axis=None):
    """math::cumsum (src/math/statistics/mod.rs:584): running sum from 0."""
    return ufunc_accumulate("add", a, axis)


def cumprod(a, axis=None):
    """math::cumprod (src/math/statistics/mod.rs:795): running product from 1."""
    return ufunc_accumulate("multiply", a, axis)


# ---------------------------------------------------------------------------
# NPY / NPZ (src/io/npy_npz.rs)
# ---------------------------------------------------------------------------
_NPY_TORCH = {L.F32: torch.float32, L.F64: torch.float64, L.I32: torch.int32, L.I64: torch.int64}


def npy_info(path: str, offset: int = 0) -> dict:
    """Header of the NPY file at `offset` (parse_npy_header's rules); touches
    no GPU."""
    lib = L.load()
    info = L.NpyInfo()
    L.check(lib.nrs_npy_inspect(None, str(path).encode(), int(offset), C.byref(info)))
    return {"descr": info.descr.decode(), "dtype": info.dtype, "itemsize": info.itemsize,
            "fortran_order": bool(info.fortran_order), "shape": tuple(info.shape[:info.ndim]),
            "data_offset": info.data_offset, "nbytes": info.nbytes}


def _load_at(path: str, offset: int, device) -> torch.Tensor:
    lib = L.load()
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    h = handle(dev.index)
    info = L.NpyInfo()
    L.check(lib.nrs_npy_inspect(h, str(path).encode(), int(offset), C.byref(info)), h)
    if info.dtype not in _NPY_TORCH:
        raise L.NumRs2Error(L.ERR_DTYPE, f"NPY descr {info.descr.decode()!r} is not f32/f64/i32/i64")
    out = torch.empty(tuple(info.shape[:info.ndim]), dtype=_NPY_TORCH[info.dtype], device=dev)
    L.check(lib.nrs_npy_read(h, str(path).encode(), C.byref(info), _ptr(out), info.nbytes), h)
    return out


def load_npy(path: str, device=None) -> torch.Tensor:
    """io::npy_npz read_npy_generic (src/io/npy_npz.rs:390): the file's array
    straight into device memory."""
    return _load_at(path, 0, device)


def load_npz(path: str, name: str | None = None, device=None) -> torch.Tensor:
    """load_npz_array (src/io/npy_npz.rs:541): member `name`.npy (or, with no
    name, the first .npy member as read_npz_generic does); stored members
    only."""
    lib = L.load()
    off = C.c_int64()
    L.check(lib.nrs_npz_locate(None, str(path).encode(), None if name is None else name.encode(),
                               C.byref(off), None))
    return _load_at(path, off.value, device)


def save_npy(path: str, t: torch.Tensor) -> None:
    """serialize_to_file(..., Npy) (src/io/npy_npz.rs:342): construct_npy_header
    then the row-major payload, written from device memory."""
    _need_cuda(t)
    if not t.is_contiguous():
        raise L.NumRs2Error(L.ERR_STRIDE, "save_npy needs a contiguous array")
    lib = L.load()
    h = handle(t.device.index)
    L.check(lib.nrs_npy_write(h, str(path).encode(), dtype_code(t), t.dim(), L.i64_array(t.shape),
                              _ptr(t)), h)


# ---------------------------------------------------------------------------
# GEMM
# ---------------------------------------------------------------------------
def _mat_strides(t: torch.Tensor):
    """(leading dim, transposed?) for a 2-D operand, or None if neither
    row- nor column-contiguous."""
    r, c = t.stride()
    rows, cols = t.shape
    if c == 1 or cols <= 1:
        return (r if rows > 1 else _bi.max(cols, 1)), False
    if r == 1 or rows <= 1:
        return (c if cols > 1 else _bi.max(rows, 1)), True
    return None


def gemm_2d(m: int, k: int, n: int, a: torch.Tensor, b: torch.Tensor, c: torch.Tensor,
            accumulate: bool = False, variant: int = L.GEMM_AUTO) -> None:
    """kernels::gemm::gemm_2d on flat row-major buffers (overwrites c)."""
    _need_cuda(a, b, c)
    if a.numel() != m * k or b.numel() != k * n or c.numel() != m * n:
        raise L.ShapeMismatch(L.ERR_SHAPE, "gemm_2d length mismatch")
    lib = L.load()
    h = handle(c.device.index)
    flags = L.GEMM_ACCUMULATE if accumulate else 0
    st = lib.nrs_gemm(h, dtype_code(c), m, k, n, _ptr(a), _bi.max(k, 1), _ptr(b), _bi.max(n, 1),
                      _ptr(c), _bi.max(n, 1), flags, variant)
    L.check(st, h)


def _logical_copy(t: torch.Tensor) -> torch.Tensor:
    """A row-major copy of a view in logical order, made by the library's
    ufunc kernel (kernels::borrow::operand copies non-contiguous operands the
    same way, src/kernels/borrow.rs:59)."""
    return run_program([(L.OP_INPUT, 0, 0.0)], [t])


def _gemm_operands(a, b):
    """(a, (ld, transposed)) and (b, ...) for the GEMM entry points: row- or
    column-contiguous views go as they are, any other view is copied."""
    sa, sb = _mat_strides(a), _mat_strides(b)
    if sa is None:
        a = _logical_copy(a)
        sa = _mat_strides(a)
    if sb is None:
        b = _logical_copy(b)
        sb = _mat_strides(b)
    return a, sa, b, sb


def _gemm_views(a, b, c, accumulate, variant):
    lib = L.load()
    h = handle(c.device.index)
    m, k = a.shape
    n = b.shape[1]
    a, sa, b, sb = _gemm_operands(a, b)
    flags = (L.GEMM_ACCUMULATE if accumulate else 0) | (L.GEMM_TRANS_A if sa[1] else 0) | (
        L.GEMM_TRANS_B if sb[1] else 0)
    ldc = c.stride(0) if m > 1 else _bi.max(n, 1)
    st = lib.nrs_gemm(h, dtype_code(c), m, k, n, _ptr(a), sa[0], _ptr(b), sb[0], _ptr(c), ldc,
                      flags, variant)
    L.check(st, h)


def matmul(a: torch.Tensor, b: torch.Tensor, variant: int = L.GEMM_AUTO) -> torch.Tensor:
    """Array::matmul (src/array/linalg.rs:153-266): two 2-D operands are one
    GEMM; otherwise a 1-D operand becomes [1, k] (left) or [k, 1] (right) and
    stays so in the result (the reference does not squeeze it), the batch
    axes broadcast by NumPy's rules, and every panel is one GEMM of the batch
    (batched_gemm, :56-136; f32/f64 panels run as one grouped launch).
    0-D operands raise DimensionMismatch; mismatched inner or batch
    dimensions raise ShapeMismatch."""
    _need_cuda(a, b)
    if a.dtype != b.dtype:
        raise L.NumRs2Error(L.ERR_DTYPE, "matmul operands must share a dtype")
    if a.dim() == 2 and b.dim() == 2:
        if a.shape[1] != b.shape[0]:
            raise L.ShapeMismatch(L.ERR_SHAPE, f"matmul: {tuple(a.shape)} @ {tuple(b.shape)}")
        out = torch.empty((a.shape[0], b.shape[1]), dtype=a.dtype, device=a.device)
        _gemm_views(a, b, out, False, variant)
        return out
    if a.dim() == 1:
        a = a.unsqueeze(0)
    if b.dim() == 1:
        b = b.unsqueeze(1)
    if a.dim() < 2 or b.dim() < 2:
        raise L.DimensionMismatch(L.ERR_AXIS, "matmul requires operands with at least 1 dimension")
    if a.shape[-1] != b.shape[-2]:
        raise L.ShapeMismatch(L.ERR_SHAPE, f"matmul: {tuple(a.shape)} @ {tuple(b.shape)}")
    m, k, n = a.shape[-2], a.shape[-1], b.shape[-1]
    try:
        batch = torch.broadcast_shapes(a.shape[:-2], b.shape[:-2])
    except RuntimeError:
        raise L.ShapeMismatch(L.ERR_SHAPE, f"matmul batch axes: {tuple(a.shape)} @ {tuple(b.shape)}") from None
    out = torch.empty((*batch, m, n), dtype=a.dtype, device=a.device)
    if len(batch) == 0:
        _gemm_views(a, b, out, False, variant)
        return out
    # Broadcast operands are stride-0 views, not copies: each panel is a
    # view of the original operand (the reference materialises them,
    # Array::broadcast_to, before borrowing the flat panels).
    ab = a.expand(*batch, m, k)
    bb = b.expand(*batch, k, n)
    panels = []
    for idx in range(out[..., 0, 0].numel()):
        bi = torch.unravel_index(torch.tensor(idx), batch)
        bi = tuple(int(x) for x in bi)
        panels.append((ab[bi], bb[bi], out[bi]))
    grouped_ok = a.dtype in (torch.float32, torch.float64) and variant == L.GEMM_AUTO and all(
        _mat_strides(p[0]) is not None and _mat_strides(p[1]) is not None for p in panels)
    if grouped_ok and m > 0 and n > 0:
        plan = Plan([(pa, pb, pc, False) for pa, pb, pc in panels])
        plan.run(use_graph=False)
        plan.close()
    else:
        for pa, pb, pc in panels:
            _gemm_views(pa, pb, pc, False, variant)
    return out


def matmul_to(a: torch.Tensor, b: torch.Tensor, out: torch.Tensor) -> None:
    """Array::matmul_to: out += a @ b (2-D)."""
    _need_cuda(a, b, out)
    if a.dim() != 2 or b.dim() != 2 or out.shape != (a.shape[0], b.shape[1]) or a.shape[1] != b.shape[0]:
        raise L.ShapeMismatch(L.ERR_SHAPE, "matmul_to shape mismatch")
    if out.stride(1) != 1:
        raise L.NumRs2Error(L.ERR_STRIDE, "matmul_to needs a row-contiguous output")
    _gemm_views(a, b, out, True, L.GEMM_AUTO)


# ---------------------------------------------------------------------------
# Elementwise
# ---------------------------------------------------------------------------
def run_program(prog: list[tuple[int, int, float]], inputs: list[torch.Tensor],
                dtype: torch.dtype | None = None) -> torch.Tensor:
    """Evaluate a postfix ufunc program over broadcast inputs into a new
    contiguous array."""
    _need_cuda(*inputs)
    lib = L.load()
    dev = inputs[0].device
    dt = dtype or inputs[0].dtype
    for t in inputs:
        if t.dtype != dt:
            raise L.NumRs2Error(L.ERR_DTYPE, "ufunc inputs must share a dtype")
    shape = torch.broadcast_shapes(*[t.shape for t in inputs])
    h = handle(dev.index)
    nd = len(shape)
    strides = []
    for t in inputs:
        e = t.expand(shape)
        strides.extend(e.stride())
    out = torch.empty(shape, dtype=dt, device=dev)
    ops = (L.UfuncOp * len(prog))(*[L.UfuncOp(c, a, s) for c, a, s in prog])
    ptrs = (C.c_void_p * len(inputs))(*[t.data_ptr() for t in inputs])
    st = lib.nrs_ufunc(h, _DT[dt], ops, len(prog), nd, L.i64_array(shape), len(inputs), ptrs,
                       L.i64_array(strides), _ptr(out), None)
    L.check(st, h)
    return out


def _binary(code, a, b):
    return run_program([(L.OP_INPUT, 0, 0.0), (L.OP_INPUT, 1, 0.0), (code, 0, 0.0)], [a, b])


def add(a, b):
    return _binary(L.OP_ADD, a, b)


def subtract(a, b):
    return _binary(L.OP_SUB, a, b)


def multiply(a, b):
    return _binary(L.OP_MUL, a, b)


def divide(a, b):
    return _binary(L.OP_DIV, a, b)


def exp(x):
    return run_program([(L.OP_INPUT, 0, 0.0), (L.OP_EXP, 0, 0.0)], [x])


def exp_affine(x: torch.Tensor, a: float, b: float, out: torch.Tensor | None = None) -> torch.Tensor:
    """y = exp(a*x + b) in one fused pass (two roundings before the exp)."""
    _need_cuda(x)
    if not x.is_contiguous():
        return Expr.leaf(x).mul_scalar(a).add_scalar(b).exp().eval()
    lib = L.load()
    h = handle(x.device.index)
    y = torch.empty_like(x) if out is None else out
    L.check(lib.nrs_exp_affine(h, dtype_code(x), x.numel(), _ptr(x), float(a), float(b), _ptr(y)), h)
    return y


class Expr:
    """ExprNode-like builder (src/expr/owned.rs:204): Leaf, Binary,
    ScalarRhs/ScalarLhs and Unary nodes compiled into one fused program."""

    def __init__(self, prog, inputs):
        self.prog = prog
        self.inputs = inputs

    @staticmethod
    def leaf(t: torch.Tensor) -> "Expr":
        return Expr([("in", t)], [t])

    def _merge(self, other: "Expr", code: int) -> "Expr":
        return Expr(self.prog + other.prog + [("op", code)], self.inputs + other.inputs)

    def _scalar(self, code: int, s: float, lhs: bool = False) -> "Expr":
        sc = [("sc", float(s))]
        body = (sc + self.prog) if lhs else (self.prog + sc)
        return Expr(body + [("op", code)], self.inputs)

    def __add__(self, o):
        return self._merge(o, L.OP_ADD) if isinstance(o, Expr) else self._scalar(L.OP_ADD, o)

    def __sub__(self, o):
        return self._merge(o, L.OP_SUB) if isinstance(o, Expr) else self._scalar(L.OP_SUB, o)

    def __mul__(self, o):
        return self._merge(o, L.OP_MUL) if isinstance(o, Expr) else self._scalar(L.OP_MUL, o)

    def __truediv__(self, o):
        return self._merge(o, L.OP_DIV) if isinstance(o, Expr) else self._scalar(L.OP_DIV, o)

    def __radd__(self, s):
        return self._scalar(L.OP_ADD, s, lhs=True)

    def __rsub__(self, s):
        return self._scalar(L.OP_SUB, s, lhs=True)

    def __rmul__(self, s):
        return self._scalar(L.OP_MUL, s, lhs=True)

    def __rtruediv__(self, s):
        return self._scalar(L.OP_DIV, s, lhs=True)

    def mul_scalar(self, s):
        return self._scalar(L.OP_MUL, s)

    def add_scalar(self, s):
        return self._scalar(L.OP_ADD, s)

    def _unary(self, code):
        return Expr(self.prog + [("op", code)], self.inputs)

    def exp(self):
        return self._unary(L.OP_EXP)

    def ln(self):
        return self._unary(L.OP_LN)

    def sqrt(self):
        return self._unary(L.OP_SQRT)

    def abs(self):
        return self._unary(L.OP_ABS)

    def __neg__(self):
        return self._unary(L.OP_NEG)

    def eval(self) -> torch.Tensor:
        # Deduplicate inputs by identity.
        uniq: list[torch.Tensor] = []
        prog = []
        for kind, v in self.prog:
            if kind == "in":
                idx = next((i for i, u in enumerate(uniq) if u is v), None)
                if idx is None:
                    uniq.append(v)
                    idx = len(uniq) - 1
                prog.append((L.OP_INPUT, idx, 0.0))
            elif kind == "sc":
                prog.append((L.OP_SCALAR, 0, v))
            else:
                prog.append((v, 0, 0.0))
        return run_program(prog, uniq)


def gemm_ozaki(a: torch.Tensor, b: torch.Tensor, slices: int = 0, out: torch.Tensor | None = None,
               accumulate: bool = False):
    """f64 C = a @ b (or out += a @ b with accumulate) from BF16 slice products
    on the tensor cores (Ozaki scheme); returns (C, info dict). slices = 0
    picks the count from the operands' measured spread (info["slices"] == 0:
    the call ran the native FP64 GEMM). Row- or column-contiguous operands
    go as they are (transposed views included); other views are copied."""
    _need_cuda(a, b)
    if a.dtype != torch.float64 or b.dtype != torch.float64:
        raise L.NumRs2Error(L.ERR_DTYPE, "gemm_ozaki takes f64 operands")
    if a.dim() != 2 or b.dim() != 2 or a.shape[1] != b.shape[0]:
        raise L.ShapeMismatch(L.ERR_SHAPE, "gemm_ozaki shape mismatch")
    m, k = a.shape
    n = b.shape[1]
    if out is None:
        if accumulate:
            raise L.NumRs2Error(L.ERR_INVALID, "accumulate needs out")
        c = torch.empty((m, n), dtype=torch.float64, device=a.device)
    else:
        c = out
        if c.shape != (m, n) or c.dtype != torch.float64 or (c.stride(1) != 1 and n > 1):
            raise L.ShapeMismatch(L.ERR_SHAPE, "gemm_ozaki output must be a row-contiguous m x n f64 array")
    a, sa, b, sb = _gemm_operands(a, b)
    lib = L.load()
    h = handle(a.device.index)
    info = L.OzakiInfo()
    flags = (L.GEMM_ACCUMULATE if accumulate else 0) | (L.GEMM_TRANS_A if sa[1] else 0) | (
        L.GEMM_TRANS_B if sb[1] else 0)
    ldc = c.stride(0) if m > 1 else _bi.max(n, 1)
    st = lib.nrs_gemm_ozaki(h, m, k, n, _ptr(a), sa[0], _ptr(b), sb[0], _ptr(c), ldc, flags, slices,
                            C.byref(info))
    L.check(st, h)
    return c, {"slices": info.slices, "products": info.products, "slice_bits": info.slice_bits,
               "k_chunk": info.k_chunk, "est_rel_error": info.est_rel_error, "spread": info.spread}


class sm_budget:
    """Context manager: size the device handle's grids for at most `sms` SMs
    (nrs_set_sm_budget); results do not change."""

    def __init__(self, sms: int, device: int | None = None):
        self.sms, self.h = sms, handle(device)

    def __enter__(self):
        L.check(L.load().nrs_set_sm_budget(self.h, self.sms), self.h)
        return self

    def __exit__(self, *exc):
        L.load().nrs_set_sm_budget(self.h, 0)


def probe_peak(kind: int, device: int | None = None) -> float:
    """TFLOP/s of a compute pipe on this device (nrs_probe_peak):
    L.PEAK_FP64_DMMA or L.PEAK_FP32_FMA."""
    lib = L.load()
    h = handle(device)
    v = C.c_double()
    L.check(lib.nrs_probe_peak(h, kind, C.byref(v)), h)
    return v.value


# ---------------------------------------------------------------------------
# Grouped persistent launch, autotuner, learned selector
# ---------------------------------------------------------------------------
class Plan:
    """A grouped launch of GEMMs and row reductions (nrs_plan_*).

    gemms: list of (A, B, C, accumulate) 2-D CUDA tensors (f32 or f64; A and
    B may be transposed views); reds: list of (x, op, out) with x a
    contiguous 1-D tensor and out a 1-element tensor. f64_mode / f32_mode:
    nrs_plan_options (PLAN_F64_OZAKI / PLAN_F32_OZAKI put the row-major
    GEMMs of that type on the tensor cores)."""

    def __init__(self, gemms=(), reds=(), f64_mode: int = L.PLAN_F64_DMMA, f64_slices: int = 0,
                 f64_digit_bits: int = 0, f32_mode: int = L.PLAN_F32_FMA):
        lib = L.load()
        self.h = handle()
        gd, rd, self._keep = _group_descs(gemms, reds)
        self.p = C.c_void_p()
        opt = L.PlanOptions(f64_mode, f64_slices, f64_digit_bits, f32_mode)
        L.check(lib.nrs_plan_create_ex(self.h, len(gemms), gd, len(reds), rd, C.byref(opt), C.byref(self.p)),
                self.h)

    def run(self, use_graph: bool = True) -> None:
        h = handle()
        L.check(L.load().nrs_plan_run(h, self.p, 1 if use_graph else 0), h)

    def stats(self):
        wi, gt = C.c_int64(), C.c_int64()
        L.check(L.load().nrs_plan_stats(self.p, C.byref(wi), C.byref(gt)))
        return {"work_items": wi.value, "gemm_tiles": gt.value}

    def f64_info(self):
        """(f64 GEMMs on the tensor cores, slice count, digit bits)."""
        n, sl, b = C.c_int64(), C.c_int(), C.c_int()
        L.check(L.load().nrs_plan_f64_info(self.p, C.byref(n), C.byref(sl), C.byref(b)))
        return n.value, sl.value, b.value

    def f32_info(self):
        """(f32 GEMMs on the tensor cores, slice count, digit bits)."""
        n, sl, b = C.c_int64(), C.c_int(), C.c_int()
        L.check(L.load().nrs_plan_f32_info(self.p, C.byref(n), C.byref(sl), C.byref(b)))
        return n.value, sl.value, b.value

    def close(self) -> None:
        if self.p:
            L.load().nrs_plan_destroy(self.p)
            self.p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _group_descs(gemms, reds):
    """Descriptor arrays of a group (and the tensors they point into)."""
    keep = []
    gd = (L.GemmDesc * _bi.max(1, len(gemms)))()
    for i, (a, b, c, acc) in enumerate(gemms):
        _need_cuda(a, b, c)
        sa, sb = _mat_strides(a), _mat_strides(b)
        if sa is None or sb is None or c.stride(1) != 1:
            raise L.NumRs2Error(L.ERR_STRIDE, "grouped GEMM operands must be row- or column-contiguous")
        flags = (L.GEMM_ACCUMULATE if acc else 0) | (L.GEMM_TRANS_A if sa[1] else 0) | (
            L.GEMM_TRANS_B if sb[1] else 0)
        m, k = a.shape
        n = b.shape[1]
        gd[i] = L.GemmDesc(dtype_code(c), flags, m, k, n, a.data_ptr(), sa[0], b.data_ptr(), sb[0],
                           c.data_ptr(), c.stride(0) if m > 1 else _bi.max(n, 1))
        keep += [a, b, c]
    rd = (L.RowReduceDesc * _bi.max(1, len(reds)))()
    for i, (x, op, out) in enumerate(reds):
        _need_cuda(x, out)
        if not x.is_contiguous():
            raise L.NumRs2Error(L.ERR_STRIDE, "row reductions need contiguous rows")
        rd[i] = L.RowReduceDesc(dtype_code(x), op, x.numel(), x.data_ptr(), out.data_ptr())
        keep += [x, out]
    return gd, rd, keep


def autotune_plan(gemms=(), reds=(), max_trials: int = 48, reps: int = 3, f64_ozaki: bool = False,
                  f32_ozaki: bool = False) -> dict:
    """nrs_plan_autotune: tile variants (and, with f64_ozaki / f32_ozaki, the
    tensor-core f64 mode and its digit width / the tensor-core f32 mode)
    chosen by timing the whole group; fills the tuner table that the next
    Plan uses and returns the Plan keyword arguments in "plan_kwargs".
    Outputs' contents are undefined afterwards."""
    lib = L.load()
    h = handle()
    gd, rd, keep = _group_descs(gemms, reds)
    rep = L.AutotuneReport()
    opt = L.PlanOptions(L.PLAN_F64_OZAKI if f64_ozaki else L.PLAN_F64_DMMA, 0, 0,
                        L.PLAN_F32_OZAKI if f32_ozaki else L.PLAN_F32_FMA)
    L.check(lib.nrs_plan_autotune(h, len(gemms), gd, len(reds), rd, C.byref(opt), max_trials, reps,
                                  C.byref(rep)), h)
    del keep
    o = rep.options
    return {"untuned_ms": rep.untuned_ms, "isolated_ms": rep.isolated_ms, "final_ms": rep.final_ms,
            "ozaki_ms": rep.ozaki_ms, "ozaki_f32_ms": rep.ozaki_f32_ms, "buckets": rep.buckets,
            "trials": rep.trials,
            "plan_kwargs": {"f64_mode": o.f64_mode, "f64_slices": o.f64_slices, "f64_digit_bits": o.f64_digit_bits,
                            "f32_mode": o.f32_mode}}


def gemm_ozaki_grouped(problems, slices: int = 0):
    """nrs_gemm_ozaki_grouped over (A, B, C, accumulate) f64 problems; returns
    (list of on-tensor-cores flags, info dict)."""
    lib = L.load()
    h = handle()
    gd, _, keep = _group_descs(problems, ())
    flags = (C.c_int * _bi.max(1, len(problems)))()
    info = L.OzakiInfo()
    L.check(lib.nrs_gemm_ozaki_grouped(h, len(problems), gd, slices, flags, C.byref(info)), h)
    del keep
    return [bool(flags[i]) for i in range(len(problems))], {"slices": info.slices, "slice_bits": info.slice_bits}


def tile_variants():
    lib = L.load()
    out = []
    for v in range(L.TILE_VARIANTS):
        tm, tn, sk, dt = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.check(lib.nrs_tile_variant_info(v, C.byref(tm), C.byref(tn), C.byref(sk), C.byref(dt)))
        out.append({"tile_m": tm.value, "tile_n": tn.value, "split_k": sk.value, "dtype": dt.value})
    return out


def tune_gemm(dtype: int, m: int, k: int, n: int, flags: int = 0, batch: int = 1, reps: int = 3):
    """Exhaustive timing of every tile variant (microseconds per problem)."""
    lib = L.load()
    h = handle()
    times = (C.c_float * L.TILE_VARIANTS)()
    best = C.c_int()
    L.check(lib.nrs_tune_gemm(h, dtype, m, k, n, flags, batch, reps, times, C.byref(best)), h)
    return list(times), best.value


def tuner_set(dtype, m, k, n, variant):
    L.check(L.load().nrs_tuner_set(handle(), dtype, m, k, n, variant))


def tuner_get(dtype, m, k, n) -> int:
    return L.load().nrs_tuner_get(handle(), dtype, m, k, n)


def tuner_save(path: str) -> None:
    h = handle()
    L.check(L.load().nrs_tuner_save(h, path.encode()), h)


def tuner_load(path: str) -> None:
    h = handle()
    L.check(L.load().nrs_tuner_load(h, path.encode()), h)


def tuner_clear():
    L.check(L.load().nrs_tuner_clear(handle()))


class Selector:
    """The MLP cost model (nrs_selector_*): 7 features -> 2 x hidden ReLU ->
    one predicted log2(us) per tile variant."""

    def __init__(self, n_features: int = 7, hidden: int = 64, n_out: int = L.TILE_VARIANTS,
                 seed: int = 8):
        self.lib = L.load()
        self.h = handle()
        self.s = C.c_void_p()
        L.check(self.lib.nrs_selector_create(self.h, n_features, hidden, n_out, seed, C.byref(self.s)), self.h)
        self.F, self.H, self.V = n_features, hidden, n_out

    @property
    def n_params(self) -> int:
        return self.lib.nrs_selector_num_params(self.s)

    def get_params(self):
        import numpy as np
        out = np.empty(self.n_params, np.float32)
        L.check(self.lib.nrs_selector_get_params(handle(), self.s, out.ctypes.data_as(C.c_void_p)), self.h)
        return out

    def set_params(self, p):
        import numpy as np
        p = np.ascontiguousarray(p, dtype=np.float32)
        L.check(self.lib.nrs_selector_set_params(handle(), self.s, p.ctypes.data_as(C.c_void_p)), self.h)

    def forward_backward(self, x, t, mask):
        B = x.shape[0]
        y = torch.empty((B, self.V), device=x.device)
        g = torch.empty(self.n_params, device=x.device)
        loss = C.c_float()
        L.check(self.lib.nrs_selector_forward_backward(handle(), self.s, B, _ptr(x), _ptr(t), _ptr(mask),
                                                       _ptr(y), _ptr(g), C.byref(loss)), self.h)
        return y, g, loss.value

    def train(self, x, t, mask, epochs: int, batch: int = 256, lr: float = 3e-3, seed: int = 8) -> float:
        loss = C.c_float()
        L.check(self.lib.nrs_selector_train(handle(), self.s, x.shape[0], _ptr(x), _ptr(t), _ptr(mask),
                                            epochs, batch, lr, seed, C.byref(loss)), self.h)
        return loss.value

    def predict(self, x):
        y = torch.empty((x.shape[0], self.V), device=x.device)
        L.check(self.lib.nrs_selector_predict(handle(), self.s, x.shape[0], _ptr(x), _ptr(y)), self.h)
        return y

    def save(self, path: str) -> None:
        L.check(self.lib.nrs_selector_save(handle(), self.s, path.encode()), self.h)

    def load(self, path: str) -> None:
        L.check(self.lib.nrs_selector_load(handle(), self.s, path.encode()), self.h)

    def install(self, on: bool = True) -> None:
        L.check(self.lib.nrs_tuner_set_selector(handle(), self.s if on else None), self.h)

    def close(self) -> None:
        if self.s:
            self.lib.nrs_tuner_set_selector(handle(), None)
            self.lib.nrs_selector_destroy(self.s)
            self.s = C.c_void_p()


def fill_random(out: torch.Tensor, dist: int, seed: int, p0: float, p1: float) -> torch.Tensor:
    """Seeded SplitMix64 generator on the device (nrs_fill_random)."""
    _need_cuda(out)
    if not out.is_contiguous():
        raise L.NumRs2Error(L.ERR_STRIDE, "fill_random needs a contiguous array")
    lib = L.load()
    h = handle(out.device.index)
    L.check(lib.nrs_fill_random(h, dtype_code(out), dist, seed, out.numel(), p0, p1, _ptr(out)), h)
    return out
