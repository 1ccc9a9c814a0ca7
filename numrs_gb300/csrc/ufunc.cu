// Elementwise ufunc programs and the fused y = exp(a*x + b) kernel.
//
// The reference's elementwise kernels take closures
// (kernels::elementwise::binary_serial, src/kernels/elementwise.rs:51) and
// ExprNode trees (src/expr/owned.rs:204). Across a C ABI they become postfix
// programs over a value stack. Every op rounds once (MUL then ADD is two
// roundings, never contracted into an FMA: the reference documents this at
// src/expr/fused_eval.rs:17-21), so results match a scalar evaluation of the
// same closure element for element; exp/ln/sqrt are CUDA's.
#include <type_traits>

#include "nrs_internal.cuh"

namespace {

struct Prog {
  int len;
  int32_t code[NRS_UFUNC_MAX_OPS];
  int32_t arg[NRS_UFUNC_MAX_OPS];
  double scalar[NRS_UFUNC_MAX_OPS];
};

struct Geometry {
  int ndim;
  int n_inputs;
  int64_t shape[NRS_UFUNC_MAX_DIMS];
  int64_t in_stride[NRS_UFUNC_MAX_INPUTS][NRS_UFUNC_MAX_DIMS];
  int64_t out_stride[NRS_UFUNC_MAX_DIMS];
  const void* in[NRS_UFUNC_MAX_INPUTS];
};

constexpr int kStack = 8;

// Non-contracting arithmetic.
template <typename T> __device__ __forceinline__ T radd(T a, T b);
template <typename T> __device__ __forceinline__ T rsub(T a, T b);
template <typename T> __device__ __forceinline__ T rmul(T a, T b);
template <typename T> __device__ __forceinline__ T rdiv(T a, T b);
template <> __device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
template <> __device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }
#define NRS_INT_OPS(T, U)                                                                      \
  template <> __device__ __forceinline__ T radd(T a, T b) { return (T)((U)a + (U)b); }         \
  template <> __device__ __forceinline__ T rsub(T a, T b) { return (T)((U)a - (U)b); }         \
  template <> __device__ __forceinline__ T rmul(T a, T b) { return (T)((U)a * (U)b); }         \
  template <> __device__ __forceinline__ T rdiv(T a, T b) {                                    \
    return (b == 0 || (b == (T)-1 && a == (T)((U)1 << (sizeof(T) * 8 - 1)))) ? (T)0 : a / b;   \
  }
NRS_INT_OPS(int64_t, unsigned long long)
NRS_INT_OPS(int32_t, unsigned)

template <typename T>
__device__ __forceinline__ T unary(int code, T v) {
  if constexpr (std::is_floating_point<T>::value) {
    switch (code) {
      case NRS_OP_NEG: return -v;
      case NRS_OP_ABS: return fabs(v);
      case NRS_OP_SQRT: return sqrt(v);
      case NRS_OP_EXP: return exp(v);
      default: return log(v);
    }
  } else {
    switch (code) {
      case NRS_OP_NEG: return rsub<T>(T(0), v);
      default: return v < 0 ? rsub<T>(T(0), v) : v;
    }
  }
}

template <typename T>
__device__ __forceinline__ T binop(int code, T a, T b) {
  switch (code) {
    case NRS_OP_ADD: return radd(a, b);
    case NRS_OP_SUB: return rsub(a, b);
    case NRS_OP_MUL: return rmul(a, b);
    case NRS_OP_DIV: return rdiv(a, b);
    case NRS_OP_MAX:
      if constexpr (std::is_floating_point<T>::value) return (a != a || a > b) ? a : b;
      else return a > b ? a : b;
    default:
      if constexpr (std::is_floating_point<T>::value) return (a != a || a < b) ? a : b;
      else return a < b ? a : b;
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    ufunc_generic(Prog prog, Geometry g, int64_t n, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t off[NRS_UFUNC_MAX_INPUTS];
    int64_t ooff = 0;
#pragma unroll
    for (int k = 0; k < NRS_UFUNC_MAX_INPUTS; ++k) off[k] = 0;
    int64_t rem = i;
    for (int d = g.ndim - 1; d >= 0; --d) {
      int64_t c = rem % g.shape[d];
      rem /= g.shape[d];
      ooff += c * g.out_stride[d];
      for (int k = 0; k < g.n_inputs; ++k) off[k] += c * g.in_stride[k][d];
    }
    T st[kStack];
    int sp = 0;
    for (int pc = 0; pc < prog.len; ++pc) {
      const int code = prog.code[pc];
      if (code == NRS_OP_INPUT) {
        st[sp++] = static_cast<const T*>(g.in[prog.arg[pc]])[off[prog.arg[pc]]];
      } else if (code == NRS_OP_SCALAR) {
        st[sp++] = (T)prog.scalar[pc];
      } else if (code >= NRS_OP_NEG && code <= NRS_OP_LN) {
        st[sp - 1] = unary<T>(code, st[sp - 1]);
      } else {
        T b = st[--sp];
        st[sp - 1] = binop<T>(code, st[sp - 1], b);
      }
    }
    out[ooff] = st[0];
  }
}

// y = exp((a*x) + b), contiguous, 16-byte vectors, streaming loads/stores
// (every byte is touched once, so keep it from displacing L2 contents).
__device__ __forceinline__ float ea(float x, float a, float b) {
  return expf(__fadd_rn(__fmul_rn(a, x), b));
}
__device__ __forceinline__ double ea(double x, double a, double b) {
  return exp(__dadd_rn(__dmul_rn(a, x), b));
}

template <typename T>
__global__ void __launch_bounds__(256)
    exp_affine_vec(const T* __restrict__ x, int64_t n, T a, T b, T* __restrict__ y) {
  using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  constexpr int PER = 16 / sizeof(T);
  constexpr int UNROLL = 4;
  const int64_t nv = n / PER;
  const V* xv = reinterpret_cast<const V*>(x);
  V* yv = reinterpret_cast<V*>(y);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + (UNROLL - 1) * stride < nv; i += UNROLL * stride) {
    V v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) v[u] = __ldcs(xv + i + u * stride);
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      T* e = reinterpret_cast<T*>(&v[u]);
#pragma unroll
      for (int k = 0; k < PER; ++k) e[k] = ea(e[k], a, b);
      __stcs(yv + i + u * stride, v[u]);
    }
  }
  for (; i < nv; i += stride) {
    V v = __ldcs(xv + i);
    T* e = reinterpret_cast<T*>(&v);
#pragma unroll
    for (int k = 0; k < PER; ++k) e[k] = ea(e[k], a, b);
    __stcs(yv + i, v);
  }
  // scalar tail
  const int64_t t = nv * PER + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n) y[t] = ea(x[t], a, b);
}

template <typename T>
__global__ void exp_affine_scalar(const T* __restrict__ x, int64_t n, T a, T b, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = ea(x[i], a, b);
}

template <typename T>
int launch_exp_affine(nrs_handle* h, int64_t n, const T* x, T a, T b, T* y) {
  if (n == 0) return NRS_OK;
  const bool aligned = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0;
  int grid = h->num_sms * 8;
  if (aligned) {
    int64_t nv = n / (16 / (int64_t)sizeof(T));
    int64_t need = (nv + 255) / 256;
    if (need < grid) grid = (int)(need > 0 ? need : 1);
    exp_affine_vec<T><<<grid, 256, 0, h->stream>>>(x, n, a, b, y);
  } else {
    exp_affine_scalar<T><<<grid, 256, 0, h->stream>>>(x, n, a, b, y);
  }
  return nrs_after_launch(h, "exp_affine");
}

template <typename T>
int launch_generic(nrs_handle* h, const Prog& p, const Geometry& g, int64_t n, void* out) {
  if (n == 0) return NRS_OK;
  int64_t need = (n + 255) / 256;
  int grid = (int)(need < (int64_t)h->num_sms * 16 ? need : (int64_t)h->num_sms * 16);
  ufunc_generic<T><<<grid, 256, 0, h->stream>>>(p, g, n, (T*)out);
  return nrs_after_launch(h, "ufunc_generic");
}

}  // namespace

extern "C" int nrs_exp_affine(nrs_handle* h, int dtype, int64_t n, const void* x, double a,
                              double b, void* y) {
  if (!h || n < 0 || (n && (!x || !y))) return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  if (dtype == NRS_F32)
    return launch_exp_affine<float>(h, n, (const float*)x, (float)a, (float)b, (float*)y);
  if (dtype == NRS_F64)
    return launch_exp_affine<double>(h, n, (const double*)x, a, b, (double*)y);
  return nrs_fail(h, NRS_ERR_DTYPE, "exp needs f32 or f64");
}

extern "C" int nrs_ufunc(nrs_handle* h, int dtype, const nrs_ufunc_op* prog, int prog_len,
                         int ndim, const int64_t* shape, int n_inputs, const void* const* inputs,
                         const int64_t* in_strides, void* out, const int64_t* out_strides) {
  if (!h) return NRS_ERR_INVALID;
  h->last_error.clear();
  if (!prog || prog_len < 1 || prog_len > NRS_UFUNC_MAX_OPS)
    return nrs_fail(h, NRS_ERR_INVALID, "program length must be 1..32");
  if (ndim < 0 || ndim > NRS_UFUNC_MAX_DIMS || (ndim && !shape))
    return nrs_fail(h, NRS_ERR_INVALID, "bad ndim/shape");
  if (n_inputs < 0 || n_inputs > NRS_UFUNC_MAX_INPUTS || (n_inputs && (!inputs || (ndim && !in_strides))))
    return nrs_fail(h, NRS_ERR_INVALID, "bad inputs");
  const size_t es = nrs_dtype_size(dtype);
  if (!es) return nrs_fail(h, NRS_ERR_DTYPE, "unknown dtype");
  const bool is_int = (dtype == NRS_I32 || dtype == NRS_I64);
  // Validate the program: stack discipline, input indices, dtype support.
  Prog p{};
  p.len = prog_len;
  int depth = 0;
  for (int i = 0; i < prog_len; ++i) {
    const int c = prog[i].code;
    p.code[i] = c;
    p.arg[i] = prog[i].arg;
    p.scalar[i] = prog[i].scalar;
    if (c == NRS_OP_INPUT) {
      if (prog[i].arg < 0 || prog[i].arg >= n_inputs)
        return nrs_fail(h, NRS_ERR_INVALID, "program reads a missing input");
      ++depth;
    } else if (c == NRS_OP_SCALAR) {
      ++depth;
    } else if (c >= NRS_OP_NEG && c <= NRS_OP_LN) {
      if (depth < 1) return nrs_fail(h, NRS_ERR_INVALID, "stack underflow");
      if (is_int && c >= NRS_OP_SQRT) return nrs_fail(h, NRS_ERR_DTYPE, "sqrt/exp/ln need f32/f64");
    } else if ((c >= NRS_OP_ADD && c <= NRS_OP_DIV) || c == NRS_OP_MAX || c == NRS_OP_MIN) {
      if (depth < 2) return nrs_fail(h, NRS_ERR_INVALID, "stack underflow");
      --depth;
    } else {
      return nrs_fail(h, NRS_ERR_INVALID, "unknown op code");
    }
    if (depth > kStack) return nrs_fail(h, NRS_ERR_INVALID, "stack deeper than 8");
  }
  if (depth != 1) return nrs_fail(h, NRS_ERR_INVALID, "program must leave exactly one value");
  int64_t n = 1;
  for (int d = 0; d < ndim; ++d) {
    if (shape[d] < 0) return nrs_fail(h, NRS_ERR_SHAPE, "negative dimension");
    n *= shape[d];
  }
  if (n == 0) return NRS_OK;
  if (!out) return nrs_fail(h, NRS_ERR_INVALID, "null output");
  Geometry g{};
  g.ndim = ndim;
  g.n_inputs = n_inputs;
  int64_t contig = 1;
  for (int d = ndim - 1; d >= 0; --d) {
    g.shape[d] = shape[d];
    g.out_stride[d] = out_strides ? out_strides[d] : contig;
    if (g.out_stride[d] < 0) return nrs_fail(h, NRS_ERR_STRIDE, "negative stride");
    contig *= shape[d];
  }
  bool all_contig = (out_strides == nullptr);
  for (int k = 0; k < n_inputs; ++k) {
    if (!inputs[k]) return nrs_fail(h, NRS_ERR_INVALID, "null input");
    g.in[k] = inputs[k];
    int64_t c = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      int64_t s = in_strides[(size_t)k * ndim + d];
      if (s < 0) return nrs_fail(h, NRS_ERR_STRIDE, "negative stride");
      g.in_stride[k][d] = s;
      if (shape[d] != 1 && s != c) all_contig = false;
      c *= shape[d];
    }
  }
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  // The fused affine-exp program on contiguous data takes the vectorised path.
  if (all_contig && n_inputs == 1 && prog_len == 6 && prog[0].code == NRS_OP_INPUT &&
      prog[1].code == NRS_OP_SCALAR && prog[2].code == NRS_OP_MUL &&
      prog[3].code == NRS_OP_SCALAR && prog[4].code == NRS_OP_ADD && prog[5].code == NRS_OP_EXP &&
      (dtype == NRS_F32 || dtype == NRS_F64)) {
    // (x * a) rounds the same as (a * x): IEEE multiplication is commutative.
    return nrs_exp_affine(h, dtype, n, inputs[0], prog[1].scalar, prog[3].scalar, out);
  }
  switch (dtype) {
    case NRS_F32: return launch_generic<float>(h, p, g, n, out);
    case NRS_F64: return launch_generic<double>(h, p, g, n, out);
    case NRS_I64: return launch_generic<int64_t>(h, p, g, n, out);
    default: return launch_generic<int32_t>(h, p, g, n, out);
  }
}
