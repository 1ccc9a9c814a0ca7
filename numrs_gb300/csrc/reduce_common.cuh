// Fold operators and block-level combine shared by the reduction kernels
// (reduce.cu) and the persistent grouped kernel (grouped.cu), so a row
// reduced inside a grouped launch is bit-identical to the same row reduced
// by nrs_reduce.
#pragma once

#include <climits>
#include <cmath>
#include <type_traits>

#include "f64_round.cuh"
#include "nrs_internal.cuh"

namespace nrs_red {

// ---------------------------------------------------------------------------
// Fold operators
// ---------------------------------------------------------------------------
template <typename T> struct Lim;
template <> struct Lim<float> {
  static __device__ __forceinline__ float lowest() { return -INFINITY; }
  static __device__ __forceinline__ float highest() { return INFINITY; }
};
template <> struct Lim<double> {
  static __device__ __forceinline__ double lowest() { return -INFINITY; }
  static __device__ __forceinline__ double highest() { return INFINITY; }
};
template <> struct Lim<int64_t> {
  static __device__ __forceinline__ int64_t lowest() { return LLONG_MIN; }
  static __device__ __forceinline__ int64_t highest() { return LLONG_MAX; }
};
template <> struct Lim<int32_t> {
  static __device__ __forceinline__ int32_t lowest() { return INT_MIN; }
  static __device__ __forceinline__ int32_t highest() { return INT_MAX; }
};

template <typename T> __device__ __forceinline__ bool is_nan(T v) { return v != v; }

// Lane fold step. MAX/MIN: the accumulator starts at -inf/+inf, so the first
// element always replaces it (or keeps it, bitwise equal, when it is the same
// infinity); a NaN accumulator is sticky, so the first NaN of the lane is the
// result -- the reference's short-circuit on `is_unordered(&val)`.
template <typename T, int OP>
struct Fold {
  static __device__ __forceinline__ T init() {
    if (OP == NRS_MAX) return Lim<T>::lowest();
    if (OP == NRS_MIN) return Lim<T>::highest();
    if (OP == NRS_PROD) return T(1);
    return T(0);
  }
  static __device__ __forceinline__ T step(T acc, T v) {
    if (OP == NRS_MAX) return (!is_nan(acc) && (is_nan(v) || v > acc)) ? v : acc;
    if (OP == NRS_MIN) return (!is_nan(acc) && (is_nan(v) || v < acc)) ? v : acc;
    if (OP == NRS_PROD) return mul(acc, v);
    return add(acc, v);
  }
  // Integer sums/products wrap (two's complement), float ones round once.
  static __device__ __forceinline__ T add(T a, T b) {
    if constexpr (sizeof(T) == 8 && !std::is_floating_point<T>::value)
      return (T)((unsigned long long)a + (unsigned long long)b);
    else if constexpr (sizeof(T) == 4 && !std::is_floating_point<T>::value)
      return (T)((unsigned)a + (unsigned)b);
    else
      return a + b;
  }
  static __device__ __forceinline__ T mul(T a, T b) {
    if constexpr (sizeof(T) == 8 && !std::is_floating_point<T>::value)
      return (T)((unsigned long long)a * (unsigned long long)b);
    else if constexpr (sizeof(T) == 4 && !std::is_floating_point<T>::value)
      return (T)((unsigned)a * (unsigned)b);
    else
      return a * b;
  }
};

// Output of a lane: MEAN divides by the axis length in T (f64 for integers).
template <typename T, int OP> struct OutOf { using type = T; };
template <> struct OutOf<int64_t, NRS_MEAN> { using type = double; };
template <> struct OutOf<int32_t, NRS_MEAN> { using type = double; };

// `div` is the variance divisor (axis length - ddof) for VAR/STD.
template <typename T, int OP>
__device__ __forceinline__ typename OutOf<T, OP>::type finish(T acc, int64_t n, T div = T(1)) {
  if constexpr (OP == NRS_MEAN) {
    if constexpr (std::is_floating_point<T>::value)
      return acc / (T)n;
    else
      return (double)acc / (double)n;
  } else if constexpr (OP == NRS_VAR || OP == NRS_STD) {
    if constexpr (std::is_floating_point<T>::value) {
      const T v = acc / div;
      return OP == NRS_STD ? sqrt(v) : v;
    } else {
      return acc;
    }
  } else {
    return acc;
  }
}

// Per-element transform of a lane fold: VAR/STD fold (x - mean)^2 of the
// lane (math::statistics::var(axis), src/math/statistics/mod.rs:1483-1488:
// `diff = val - mean; sum_sq + diff * diff`, each op rounded once).
template <typename T, int OP>
__device__ __forceinline__ T lane_xform(T v, T m) {
  if constexpr ((OP == NRS_VAR || OP == NRS_STD) && std::is_same<T, float>::value) {
    const float d = __fsub_rn(v, m);
    return __fmul_rn(d, d);
  } else if constexpr ((OP == NRS_VAR || OP == NRS_STD) && std::is_same<T, double>::value) {
    const double d = __dsub_rn(v, m);
    return __dmul_rn(d, d);
  } else {
    return v;
  }
}

// Partial of one chunk: value plus a NaN flag (min/max only).
template <typename T>
struct Partial {
  T v;
  int nan;
};

// Block-wide tree combine of per-thread values (fixed shape: warp butterfly,
// then the 8 warp results in order), result valid in thread 0.
template <typename T, int OP>
__device__ __forceinline__ T block_combine(T v, T* sh) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    T o = __shfl_xor_sync(0xffffffffu, v, off);
    v = Fold<T, OP>::step(v, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  T r = v;
  if (threadIdx.x == 0) {
    r = sh[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = Fold<T, OP>::step(r, sh[i]);
  }
  __syncthreads();
  return r;
}

// Folds a run of N values into a lane accumulator with exactly the result of
// N sequential Fold<T, OP>::step calls, using four independent chains where
// the order cannot matter:
//  * integer folds (wrapping sums/products, max, min) are exact in any order;
//  * float max/min are order-free as long as the run holds no NaN (the first
//    NaN of a lane is its result) and no zero (a lane keeps the FIRST of -0.0
//    and +0.0); such runs are detected off the dependency chain and refolded
//    sequentially from the incoming accumulator;
//  * float sums/products stay one sequential chain: their rounding depends on
//    the order, and the reference's order is left to right.
template <typename T, int OP>
struct RunFold {
  static constexpr bool kFloat = std::is_floating_point<T>::value;
  static constexpr bool kMinMax = (OP == NRS_MAX || OP == NRS_MIN);
  static constexpr bool kChains = !kFloat || kMinMax;

  static __device__ __forceinline__ T pick(T a, T v) {
    if constexpr (OP == NRS_MAX) return v > a ? v : a;
    else return v < a ? v : a;
  }
  // pick for operands that are neither NaN nor zero: one max / min
  // instruction (equal operands then have equal bits).
  static __device__ __forceinline__ T pick_plain(T a, T v) {
    if constexpr (OP == NRS_MAX) return fmax(a, v);
    else return fmin(a, v);
  }

  // max / min that return NaN when either operand is NaN (f32 only: the
  // instruction has no f64 form).
  static __device__ __forceinline__ float pick_nan(float a, float v) {
    float d;
    if constexpr (OP == NRS_MAX) asm("max.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(v));
    else asm("min.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(v));
    return d;
  }

  // f64 order on the integer pipe (f64_round.cuh)
  static __device__ __forceinline__ int64_t key64(uint64_t u) { return nrs_f64_key(u); }
  static __device__ __forceinline__ bool nan_or_zero64(uint64_t u) { return nrs_f64_nan_or_zero(u); }

  template <int N, typename Get>
  static __device__ __forceinline__ T run(T acc, Get get) {
    if constexpr (!kChains) {
#pragma unroll
      for (int i = 0; i < N; ++i) acc = Fold<T, OP>::step(acc, get(i));
      return acc;
    } else if constexpr (!kFloat) {
      T a[4] = {acc, Fold<T, OP>::init(), Fold<T, OP>::init(), Fold<T, OP>::init()};
#pragma unroll
      for (int i = 0; i < N; ++i) a[i & 3] = Fold<T, OP>::step(a[i & 3], get(i));
      return Fold<T, OP>::step(Fold<T, OP>::step(a[0], a[1]), Fold<T, OP>::step(a[2], a[3]));
    } else if constexpr (std::is_same<T, float>::value) {
      // Four NaN-propagating chains, one instruction per element. A result
      // that is neither NaN nor zero is the ordered fold's bit for bit (equal
      // nonzero values have equal bits); a NaN (whose first payload the
      // ordered fold keeps) or a zero (where -0 and +0 tie) re-folds the
      // block in order.
      static_assert(N % 4 == 0, "blocks of four");
      if (acc != acc) return acc;  // the lane already holds its first NaN
      float v[N];
#pragma unroll
      for (int i = 0; i < N; ++i) v[i] = get(i);
      float a[4] = {pick_nan(acc, v[0]), v[1], v[2], v[3]};
#pragma unroll
      for (int i = 4; i < N; ++i) a[i & 3] = pick_nan(a[i & 3], v[i]);
      const float r = pick_nan(pick_nan(a[0], a[1]), pick_nan(a[2], a[3]));
      if (r == r && r != 0.0f) return r;
#pragma unroll
      for (int i = 0; i < N; ++i) acc = Fold<T, OP>::step(acc, v[i]);
      return acc;
    } else if constexpr (std::is_same<T, double>::value) {
      // Four chains of int64 keys (no FP64 instruction per element): exact
      // when the block and the accumulator hold no NaN and no zero; else the
      // block re-folds in order.
      static_assert(N % 4 == 0, "blocks of four");
      const uint64_t ua = (uint64_t)__double_as_longlong(acc);
      if (nrs_f64_is_nan(ua)) return acc;  // the lane already holds its first NaN
      double v[N];
#pragma unroll
      for (int i = 0; i < N; ++i) v[i] = get(i);
      bool special = nan_or_zero64(ua);
      const int64_t k0 = key64((uint64_t)__double_as_longlong(Fold<T, OP>::init()));
      int64_t a[4] = {key64(ua), k0, k0, k0};
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const uint64_t u = (uint64_t)__double_as_longlong(v[i]);
        special |= nan_or_zero64(u);
        const int64_t k = key64(u);
        a[i & 3] = (OP == NRS_MAX ? (k > a[i & 3]) : (k < a[i & 3])) ? k : a[i & 3];
      }
      if (!special) {
        const int64_t b0 = (OP == NRS_MAX ? (a[1] > a[0]) : (a[1] < a[0])) ? a[1] : a[0];
        const int64_t b1 = (OP == NRS_MAX ? (a[3] > a[2]) : (a[3] < a[2])) ? a[3] : a[2];
        const int64_t b = (OP == NRS_MAX ? (b1 > b0) : (b1 < b0)) ? b1 : b0;
        return __longlong_as_double((long long)key64((uint64_t)b));
      }
#pragma unroll
      for (int i = 0; i < N; ++i) acc = Fold<T, OP>::step(acc, v[i]);
      return acc;
    } else {
      if (acc != acc) return acc;  // the lane already holds its first NaN
      T a[4] = {acc, Fold<T, OP>::init(), Fold<T, OP>::init(), Fold<T, OP>::init()};
      bool special = false;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const T v = get(i);
        special |= !(fabs(v) > T(0));  // NaN or a zero
        a[i & 3] = pick_plain(a[i & 3], v);
      }
      if (!special) return pick(pick(a[0], a[1]), pick(a[2], a[3]));
#pragma unroll
      for (int i = 0; i < N; ++i) acc = Fold<T, OP>::step(acc, get(i));
      return acc;
    }
  }
};

}  // namespace nrs_red
