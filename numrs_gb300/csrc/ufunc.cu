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

// ---------------------------------------------------------------------------
// Evaluators. An evaluator maps W elements of every input to W results:
// run<W>(in[kMaxIn][W], res[W]). Everything stays in registers. The program
// is the same for every thread, so its op codes, input numbers and stack
// depth are warp-uniform: each step is decoded once per W elements and
// dispatched with a uniform switch whose cases touch the register arrays at
// compile-time indices only (a dynamic index would move them to local
// memory, a per-element select chain would cost ~8 instructions per slot).
// The top of the stack lives in `acc`; slots below it in `st`.
// ---------------------------------------------------------------------------
constexpr int kMaxIn = 4;  // inputs the register evaluators handle

#define NRS_SLOT_CASES(X) X(0) X(1) X(2) X(3) X(4) X(5) X(6)
static_assert(kStack - 1 == 7, "NRS_SLOT_CASES lists the kStack - 1 slots below the top");

// st has SL slots (the program's depth - 1, rounded up to 1, 3 or 7).
template <typename T, int SL, int W>
__device__ __forceinline__ void slot_store(T (&st)[SL][W], int slot, const T (&v)[W]) {
  switch (slot) {
#define NRS_STORE(S)                                                            \
  case S:                                                                       \
    if constexpr (S < SL) {                                                     \
      _Pragma("unroll") for (int e = 0; e < W; ++e) st[S < SL ? S : 0][e] = v[e]; \
    }                                                                           \
    break;
    NRS_SLOT_CASES(NRS_STORE)
#undef NRS_STORE
  }
}
template <typename T, int SL, int W>
__device__ __forceinline__ void slot_load(const T (&st)[SL][W], int slot, T (&v)[W]) {
  switch (slot) {
#define NRS_LOAD(S)                                                             \
  case S:                                                                       \
    if constexpr (S < SL) {                                                     \
      _Pragma("unroll") for (int e = 0; e < W; ++e) v[e] = st[S < SL ? S : 0][e]; \
    }                                                                           \
    break;
    NRS_SLOT_CASES(NRS_LOAD)
#undef NRS_LOAD
  }
}
template <typename T, int W>
__device__ __forceinline__ void input_load(const T (&in)[kMaxIn][W], int k, T (&v)[W]) {
  switch (k) {
#define NRS_IN(S) \
  case S:         \
    _Pragma("unroll") for (int e = 0; e < W; ++e) v[e] = in[S][e]; break;
    NRS_IN(0) NRS_IN(1) NRS_IN(2) NRS_IN(3)
#undef NRS_IN
  }
}
template <typename T, int W>
__device__ __forceinline__ void unary_vec(int code, T (&acc)[W]) {
  switch (code) {
#define NRS_UN(C) \
  case C:         \
    _Pragma("unroll") for (int e = 0; e < W; ++e) acc[e] = unary<T>(C, acc[e]); break;
    NRS_UN(NRS_OP_NEG) NRS_UN(NRS_OP_ABS) NRS_UN(NRS_OP_SQRT) NRS_UN(NRS_OP_EXP) NRS_UN(NRS_OP_LN)
#undef NRS_UN
  }
}
// acc = lhs (op) acc
template <typename T, int W>
__device__ __forceinline__ void binary_vec(int code, const T (&lhs)[W], T (&acc)[W]) {
  switch (code) {
#define NRS_BIN(C) \
  case C:          \
    _Pragma("unroll") for (int e = 0; e < W; ++e) acc[e] = binop<T>(C, lhs[e], acc[e]); break;
    NRS_BIN(NRS_OP_ADD) NRS_BIN(NRS_OP_SUB) NRS_BIN(NRS_OP_MUL) NRS_BIN(NRS_OP_DIV)
    NRS_BIN(NRS_OP_MAX) NRS_BIN(NRS_OP_MIN)
#undef NRS_BIN
  }
}

// The general program (validated on the host: depth 1..D, inputs
// < n_inputs, ends with one value). D (2, 4 or 8) bounds the stack the
// program reaches, so a shallow program holds only D - 1 slots in registers.
template <typename T, int D>
struct ProgEval {
  // 16-byte vectors per thread step in the vector kernels (register budget).
  static constexpr int kUnroll = D <= 4 ? 2 : 1;
  Prog prog;
  template <int W>
  __device__ __forceinline__ void run(const T (&in)[kMaxIn][W], T (&res)[W]) const {
    T acc[W], lhs[W], st[D - 1][W];
    int depth = 0;  // values on the stack, acc included
    for (int pc = 0; pc < prog.len; ++pc) {
      const int code = prog.code[pc];
      if (code == NRS_OP_INPUT || code == NRS_OP_SCALAR) {
        if (depth > 0) slot_store(st, depth - 1, acc);
        ++depth;
        if (code == NRS_OP_INPUT) {
          input_load(in, prog.arg[pc], acc);
        } else {
          const T s = (T)prog.scalar[pc];
#pragma unroll
          for (int e = 0; e < W; ++e) acc[e] = s;
        }
      } else if (code >= NRS_OP_NEG && code <= NRS_OP_LN) {
        unary_vec(code, acc);
      } else {
        --depth;
        slot_load(st, depth - 1, lhs);
        binary_vec(code, lhs, acc);
      }
    }
#pragma unroll
    for (int e = 0; e < W; ++e) res[e] = acc[e];
  }
};

// `inputs[0] op inputs[1]`: the operators and binary closures.
template <typename T, int OP>
struct BinEval {
  static constexpr int kUnroll = 4;
  template <int W>
  __device__ __forceinline__ void run(const T (&in)[kMaxIn][W], T (&res)[W]) const {
#pragma unroll
    for (int e = 0; e < W; ++e) res[e] = binop<T>(OP, in[0][e], in[1][e]);
  }
};

// Any strides, one element per thread, full index decode (small inner dims).
template <typename T, typename Eval>
__global__ void __launch_bounds__(256)
    ufunc_decode(Eval ev, Geometry g, int64_t n, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t off[kMaxIn] = {0, 0, 0, 0};
    int64_t ooff = 0;
    int64_t rem = i;
    for (int d = g.ndim - 1; d >= 0; --d) {
      const int64_t c = rem % g.shape[d];
      rem /= g.shape[d];
      ooff += c * g.out_stride[d];
#pragma unroll
      for (int k = 0; k < kMaxIn; ++k) off[k] += c * g.in_stride[k][d];
    }
    T v[kMaxIn][1], r[1];
#pragma unroll
    for (int k = 0; k < kMaxIn; ++k)
      v[k][0] = k < g.n_inputs ? static_cast<const T*>(g.in[k])[off[k]] : T(0);
    ev.template run<1>(v, r);
    out[ooff] = r[0];
  }
}

// Broadcast / strided views with a long last dimension: a CTA takes one
// row (all dims but the last) at a time, decodes its offsets once and walks
// the row with plain strided increments.
template <typename T, typename Eval>
__global__ void __launch_bounds__(256)
    ufunc_rows(Eval ev, Geometry g, int64_t rows, T* __restrict__ out) {
  const int last = g.ndim - 1;
  const int64_t inner = g.shape[last];
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t off[kMaxIn] = {0, 0, 0, 0};
    int64_t ooff = 0;
    int64_t rem = r;
    for (int d = last - 1; d >= 0; --d) {
      const int64_t c = rem % g.shape[d];
      rem /= g.shape[d];
      ooff += c * g.out_stride[d];
#pragma unroll
      for (int k = 0; k < kMaxIn; ++k) off[k] += c * g.in_stride[k][d];
    }
    for (int64_t j = threadIdx.x; j < inner; j += blockDim.x) {
      T v[kMaxIn][1], res[1];
#pragma unroll
      for (int k = 0; k < kMaxIn; ++k)
        v[k][0] = k < g.n_inputs ? static_cast<const T*>(g.in[k])[off[k] + j * g.in_stride[k][last]] : T(0);
      ev.template run<1>(v, res);
      out[ooff + j * g.out_stride[last]] = res[0];
    }
  }
}

// Broadcast rows with 16-byte vectors: the last dimension has stride 1 in
// the output and stride 1 or 0 in every input (a broadcast row or column),
// every row starts 16-byte aligned and the row length is a multiple of the
// vector width (the host checks all three). A stride-0 input is one value
// per row, loaded once.
template <typename T, typename Eval>
__global__ void __launch_bounds__(256)
    ufunc_rows_vec(Eval ev, Geometry g, int64_t rows, T* __restrict__ out) {
  using V = typename std::conditional<sizeof(T) == 4, int4, longlong2>::type;
  constexpr int PER = 16 / sizeof(T);
  const int last = g.ndim - 1;
  const int64_t nv = g.shape[last] / PER;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t off[kMaxIn] = {0, 0, 0, 0};
    int64_t ooff = 0;
    int64_t rem = r;
    for (int d = last - 1; d >= 0; --d) {
      const int64_t c = rem % g.shape[d];
      rem /= g.shape[d];
      ooff += c * g.out_stride[d];
#pragma unroll
      for (int k = 0; k < kMaxIn; ++k) off[k] += c * g.in_stride[k][d];
    }
    T bcast[kMaxIn];
#pragma unroll
    for (int k = 0; k < kMaxIn; ++k)
      bcast[k] = (k < g.n_inputs && g.in_stride[k][last] == 0) ? static_cast<const T*>(g.in[k])[off[k]] : T(0);
    // U vectors per thread step, all loads issued before any compute.
    constexpr int U = Eval::kUnroll;
    for (int64_t j = threadIdx.x; j < nv; j += (int64_t)blockDim.x * U) {
      T x[U][kMaxIn][PER];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t jj = j + (int64_t)u * blockDim.x;
#pragma unroll
        for (int k = 0; k < kMaxIn; ++k) {
          if (jj < nv && k < g.n_inputs && g.in_stride[k][last] != 0) {
            const V q = __ldcs(reinterpret_cast<const V*>(static_cast<const T*>(g.in[k]) + off[k]) + jj);
            memcpy(x[u][k], &q, 16);
          } else {
#pragma unroll
            for (int e = 0; e < PER; ++e) x[u][k][e] = bcast[k];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t jj = j + (int64_t)u * blockDim.x;
        if (jj >= nv) break;
        T res[PER];
        ev.template run<PER>(x[u], res);
        V q;
        memcpy(&q, res, 16);
        __stcs(reinterpret_cast<V*>(out + ooff) + jj, q);
      }
    }
  }
}

// Same-shape contiguous, 16-byte aligned inputs and output (the common
// `&a + &b` of binary_serial): 16 bytes of every input per thread step.
template <typename T, typename Eval>
__global__ void __launch_bounds__(256)
    ufunc_flat_vec(Eval ev, Geometry g, int64_t n, T* __restrict__ out) {
  using V = typename std::conditional<sizeof(T) == 4, int4, longlong2>::type;
  constexpr int PER = 16 / sizeof(T);
  const int64_t nv = n / PER;
  // A block covers U * blockDim consecutive vectors per step (coalesced for
  // each u); all loads are issued before any compute.
  constexpr int U = Eval::kUnroll;
  const int64_t step = (int64_t)gridDim.x * blockDim.x * U;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x * U + threadIdx.x; i < nv; i += step) {
    T x[U][kMaxIn][PER];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t ii = i + (int64_t)u * blockDim.x;
#pragma unroll
      for (int k = 0; k < kMaxIn; ++k) {
        if (ii < nv && k < g.n_inputs) {
          const V q = __ldcs(reinterpret_cast<const V*>(g.in[k]) + ii);
          memcpy(x[u][k], &q, 16);
        } else {
#pragma unroll
          for (int e = 0; e < PER; ++e) x[u][k][e] = T(0);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t ii = i + (int64_t)u * blockDim.x;
      if (ii >= nv) break;
      T res[PER];
      ev.template run<PER>(x[u], res);
      V q;
      memcpy(&q, res, 16);
      __stcs(reinterpret_cast<V*>(out) + ii, q);
    }
  }
  // scalar tail (< PER elements)
  const int64_t t = nv * PER + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n) {
    T v[kMaxIn][1], r[1];
#pragma unroll
    for (int k = 0; k < kMaxIn; ++k) v[k][0] = k < g.n_inputs ? static_cast<const T*>(g.in[k])[t] : T(0);
    ev.template run<1>(v, r);
    out[t] = r[0];
  }
}

// Programs with more than kMaxIn inputs: the stack interpreter over up to 8
// inputs with a full index decode per element.
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

enum class Access { kFlat, kRowsVec, kStrided };

// Picks the access pattern: flat vectors, vector row walks, scalar row walks,
// or a full decode.
template <typename T, typename Eval>
int launch_eval(nrs_handle* h, const Eval& ev, const Geometry& g, int64_t n, Access acc, void* out) {
  if (n == 0) return NRS_OK;
  const int cap = h->num_sms * 8;
  if (acc == Access::kFlat) {
    const int64_t per_block = 256 * (int64_t)Eval::kUnroll;
    const int64_t need = (n / (16 / (int64_t)sizeof(T)) + per_block - 1) / per_block + 1;
    const int grid = (int)(need < cap ? need : cap);
    ufunc_flat_vec<T, Eval><<<grid, 256, 0, h->stream>>>(ev, g, n, (T*)out);
    return nrs_after_launch(h, "ufunc_flat_vec");
  }
  if (acc == Access::kRowsVec) {
    const int64_t rows = n / g.shape[g.ndim - 1];
    const int grid = (int)(rows < (int64_t)h->num_sms * 16 ? rows : (int64_t)h->num_sms * 16);
    ufunc_rows_vec<T, Eval><<<grid, 256, 0, h->stream>>>(ev, g, rows, (T*)out);
    return nrs_after_launch(h, "ufunc_rows_vec");
  }
  if (g.ndim >= 1 && g.shape[g.ndim - 1] >= 256) {
    const int64_t rows = n / g.shape[g.ndim - 1];
    const int grid = (int)(rows < (int64_t)h->num_sms * 16 ? rows : (int64_t)h->num_sms * 16);
    ufunc_rows<T, Eval><<<grid, 256, 0, h->stream>>>(ev, g, rows, (T*)out);
    return nrs_after_launch(h, "ufunc_rows");
  }
  const int64_t need = (n + 255) / 256;
  const int grid = (int)(need < (int64_t)h->num_sms * 16 ? need : (int64_t)h->num_sms * 16);
  ufunc_decode<T, Eval><<<grid, 256, 0, h->stream>>>(ev, g, n, (T*)out);
  return nrs_after_launch(h, "ufunc_decode");
}

// Dispatch on the program's shape: a lone binary op gets its own functor.
template <typename T>
int launch_program(nrs_handle* h, const Prog& p, int depth, const Geometry& g, int64_t n, Access flat,
                   void* out) {
  if (g.n_inputs > kMaxIn) {
    const int64_t need = (n + 255) / 256;
    const int grid = (int)(need < (int64_t)h->num_sms * 16 ? need : (int64_t)h->num_sms * 16);
    ufunc_generic<T><<<grid, 256, 0, h->stream>>>(p, g, n, (T*)out);
    return nrs_after_launch(h, "ufunc_generic");
  }
  if (p.len == 3 && p.code[0] == NRS_OP_INPUT && p.arg[0] == 0 && p.code[1] == NRS_OP_INPUT &&
      p.arg[1] == 1) {
    switch (p.code[2]) {
      case NRS_OP_ADD: return launch_eval<T>(h, BinEval<T, NRS_OP_ADD>{}, g, n, flat, out);
      case NRS_OP_SUB: return launch_eval<T>(h, BinEval<T, NRS_OP_SUB>{}, g, n, flat, out);
      case NRS_OP_MUL: return launch_eval<T>(h, BinEval<T, NRS_OP_MUL>{}, g, n, flat, out);
      case NRS_OP_DIV: return launch_eval<T>(h, BinEval<T, NRS_OP_DIV>{}, g, n, flat, out);
      default: break;
    }
  }
  if (depth <= 2) return launch_eval<T>(h, ProgEval<T, 2>{p}, g, n, flat, out);
  if (depth <= 4) return launch_eval<T>(h, ProgEval<T, 4>{p}, g, n, flat, out);
  return launch_eval<T>(h, ProgEval<T, kStack>{p}, g, n, flat, out);
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
  int depth = 0, max_depth = 0;
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
    if (depth > max_depth) max_depth = depth;
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
  // Same-shape contiguous operands, all 16-byte aligned: flat vector path.
  // Otherwise rows of 16-byte vectors when the last dimension is unit-stride
  // (or broadcast) everywhere and every row starts 16-byte aligned.
  Access flat = Access::kStrided;
  uintptr_t align = reinterpret_cast<uintptr_t>(out);
  for (int k = 0; k < n_inputs; ++k) align |= reinterpret_cast<uintptr_t>(inputs[k]);
  if (all_contig && (align & 15) == 0) {
    flat = Access::kFlat;
  } else if (ndim >= 1 && (align & 15) == 0 && g.shape[ndim - 1] >= 64 &&
             (g.shape[ndim - 1] * (int64_t)es) % 16 == 0 && g.out_stride[ndim - 1] == 1) {
    bool ok = true;
    for (int d = 0; d < ndim - 1; ++d)
      if (g.shape[d] > 1 && (g.out_stride[d] * (int64_t)es) % 16 != 0) ok = false;
    for (int k = 0; k < n_inputs && ok; ++k) {
      const int64_t ls = g.in_stride[k][ndim - 1];
      if (ls > 1) ok = false;
      for (int d = 0; d < ndim - 1 && ok; ++d)
        if (ls == 1 && g.shape[d] > 1 && (g.in_stride[k][d] * (int64_t)es) % 16 != 0) ok = false;
    }
    if (ok) flat = Access::kRowsVec;
  }
  switch (dtype) {
    case NRS_F32: return launch_program<float>(h, p, max_depth, g, n, flat, out);
    case NRS_F64: return launch_program<double>(h, p, max_depth, g, n, flat, out);
    case NRS_I64: return launch_program<int64_t>(h, p, max_depth, g, n, flat, out);
    default: return launch_program<int32_t>(h, p, max_depth, g, n, flat, out);
  }
}
