/*
 * oracle.c -- CPU restatement of NumRS2's `kernels` hot path (reductions,
 * axis folds, elementwise/fused ufuncs, GEMM) plus double-double reference
 * kernels and the MLP selector's forward/backward pass.
 *
 * THIS IS TEST INFRASTRUCTURE. It is the checker, never the product: only the
 * test suite, the smoke check and the CPU-baseline leg of the benchmark load
 * it. The CUDA library never links or calls it.
 *
 * Every function names the reference routine it restates (paths relative to
 * the numrs2 0.4.1 source tree). Pinning: the reductions reproduce the
 * reference's own known-answer bit patterns (tests/test_reduction_determinism.rs
 * :126-197) and the NumPy goldens of tests/py/array_operations_reference_data.json;
 * see tests/test_oracle_golden.py.
 *
 * Two pieces of the reference live in un-vendored crates and are restated
 * from their published algorithm rather than their source:
 *   - scirs2-core 0.6.5 `SimdUnifiedOps::simd_sum` (called at
 *     src/kernels/reduce.rs:212,219): restated as an 8-lane striped sum whose
 *     lanes are combined pairwise (the AVX2 f32x8 / 2x f64x4 shape). Only the
 *     float rounding of intra-chunk sums depends on this; parity there is
 *     tolerance-based.
 *   - matrixmultiply (reached through ndarray's general_mat_mul,
 *     src/kernels/gemm.rs:339; version unpinned): restated as a K-blocked
 *     (KC=256) i-k-j loop; GEMM parity is tolerance-based.
 *
 * Compile with -ffp-contract=off: the reference never contracts a*b+c into
 * an FMA (src/expr/fused_eval.rs:17-21), and neither may its restatement.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Tiering constants: src/kernels/mod.rs:63,74,92,106 and                    */
/* src/kernels/reduce.rs:200,202.                                            */
/* ------------------------------------------------------------------------ */
#define PARALLEL_MIN_LEN 10000
#define PARALLEL_CHUNK 8192
#define MINMAX_PARALLEL_MIN_LEN (8 * PARALLEL_MIN_LEN)
#define VAR_PARALLEL_MIN_LEN (4 * PARALLEL_MIN_LEN)

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* SplitMix64 input generator (Vigna). Same step and mix constants as the    */
/* reference's test generator, tests/test_expr_fused_equivalence.rs:96-112:  */
/* state starts at seed ^ GAMMA, each draw adds GAMMA then mixes. Draw i     */
/* (0-based) is therefore mix((seed ^ GAMMA) + (i + 1) * GAMMA), which lets  */
/* every element be generated independently.                                 */
/* ------------------------------------------------------------------------ */
#define SM64_GAMMA 0x9E3779B97F4A7C15ULL

static inline uint64_t sm64_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

uint64_t orc_splitmix64_at(uint64_t seed, uint64_t i) {
  return sm64_mix((seed ^ SM64_GAMMA) + (i + 1) * SM64_GAMMA);
}

static inline double sm64_u01(uint64_t seed, uint64_t i) {
  return (double)(orc_splitmix64_at(seed, i) >> 11) * (1.0 / 9007199254740992.0);
}

/* U(-1,1): 2u-1. */
void orc_gen_uniform_pm1_f64(uint64_t seed, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = 2.0 * sm64_u01(seed, (uint64_t)i) - 1.0;
}
void orc_gen_uniform_pm1_f32(uint64_t seed, int64_t n, float* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = (float)(2.0 * sm64_u01(seed, (uint64_t)i) - 1.0);
}

/* i64 uniform in [-2^20, 2^20): the top 21 bits minus 2^20, (x >> 43) - 2^20. */
void orc_gen_i64(uint64_t seed, int64_t n, int64_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    out[i] = (int64_t)(orc_splitmix64_at(seed, (uint64_t)i) >> 43) - (int64_t)(1 << 20);
}

/* N(mu, sigma) as f32: the device generator's formula (Box-Muller, cosine
 * branch, on draws 2i and 2i+1, in double, then rounded to float). Host libm's
 * log/cos may differ from the device's in the last bits of the double, so in
 * rare cases a float element differs by one ulp from the device array. */
void orc_gen_normal_f32(uint64_t seed, int64_t n, double mu, double sigma, float* out) {
  const double two_pi = 6.283185307179586476925286766559;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const double u1 = 1.0 - sm64_u01(seed, 2 * (uint64_t)i);
    const double u2 = sm64_u01(seed, 2 * (uint64_t)i + 1);
    const double z = sqrt(-2.0 * log(u1)) * cos(two_pi * u2);
    out[i] = (float)(mu + sigma * z);
  }
}

/* ------------------------------------------------------------------------ */
/* simd_sum restatement (scirs2-core 0.6.5, un-vendored; see header).        */
/* ------------------------------------------------------------------------ */
#define SIMD_LANES 8
#define DEFINE_SIMD_SUM(T, NAME)                                              \
  static T NAME(const T* a, int64_t n) {                                      \
    T acc[SIMD_LANES];                                                        \
    for (int l = 0; l < SIMD_LANES; ++l) acc[l] = (T)0;                       \
    int64_t i = 0;                                                            \
    for (; i + SIMD_LANES <= n; i += SIMD_LANES)                              \
      for (int l = 0; l < SIMD_LANES; ++l) acc[l] = acc[l] + a[i + l];        \
    T s = ((acc[0] + acc[1]) + (acc[2] + acc[3])) +                           \
          ((acc[4] + acc[5]) + (acc[6] + acc[7]));                            \
    for (; i < n; ++i) s = s + a[i];                                          \
    return s;                                                                 \
  }
DEFINE_SIMD_SUM(float, simd_sum_f32)
DEFINE_SIMD_SUM(double, simd_sum_f64)

/* ------------------------------------------------------------------------ */
/* Flat reductions: src/kernels/reduce.rs:204-444 (macro define_reduce_     */
/* kernels). Empty conventions: 0 for sum/mean/var/min/max, 1 for prod.      */
/* ------------------------------------------------------------------------ */
#define DEFINE_FLAT(T, SUF, NANV, INFV)                                         \
  /* reduce.rs:207-224: simd_sum below 10k, else 8192-chunk partials folded  \
     sequentially in chunk order. */                                          \
  T orc_sum_##SUF(const T* a, int64_t n) {                                    \
    if (n == 0) return (T)0;                                                  \
    if (n < PARALLEL_MIN_LEN) return simd_sum_##SUF(a, n);                    \
    int64_t nc = (n + PARALLEL_CHUNK - 1) / PARALLEL_CHUNK;                   \
    T* part = (T*)malloc(sizeof(T) * (size_t)nc);                             \
    _Pragma("omp parallel for schedule(static)")                              \
    for (int64_t c = 0; c < nc; ++c) {                                        \
      int64_t lo = c * PARALLEL_CHUNK;                                        \
      int64_t len = (n - lo < PARALLEL_CHUNK) ? n - lo : PARALLEL_CHUNK;      \
      part[c] = simd_sum_##SUF(a + lo, len);                                  \
    }                                                                         \
    T s = (T)0;                                                               \
    for (int64_t c = 0; c < nc; ++c) s = s + part[c];                         \
    free(part);                                                               \
    return s;                                                                 \
  }                                                                           \
  /* reduce.rs:227: mean = sum / n. */                                        \
  T orc_mean_##SUF(const T* a, int64_t n) {                                   \
    if (n == 0) return (T)0;                                                  \
    return orc_sum_##SUF(a, n) / (T)n;                                        \
  }                                                                           \
  static T ssd_chunk_##SUF(const T* a, int64_t n, T mean) {                   \
    T s = (T)0;                                                               \
    for (int64_t i = 0; i < n; ++i) s = s + (a[i] - mean) * (a[i] - mean);    \
    return s;                                                                 \
  }                                                                           \
  /* reduce.rs:239-262: second pass of the two-pass variance. */              \
  T orc_sum_sq_dev_##SUF(const T* a, int64_t n, T mean) {                     \
    if (n < PARALLEL_MIN_LEN) return ssd_chunk_##SUF(a, n, mean);             \
    int64_t nc = (n + PARALLEL_CHUNK - 1) / PARALLEL_CHUNK;                   \
    T s = (T)0;                                                               \
    for (int64_t c = 0; c < nc; ++c) {                                        \
      int64_t lo = c * PARALLEL_CHUNK;                                        \
      int64_t len = (n - lo < PARALLEL_CHUNK) ? n - lo : PARALLEL_CHUNK;      \
      s = s + ssd_chunk_##SUF(a + lo, len, mean);                             \
    }                                                                         \
    return s;                                                                 \
  }                                                                           \
  /* reduce.rs:284-314: fused var(ddof), one tier decision at 40k. */         \
  T orc_var_##SUF(const T* a, int64_t n, int64_t ddof) {                      \
    if (n == 0) return (T)0;                                                  \
    T divisor = (T)n - (T)ddof;                                               \
    T mean;                                                                   \
    T ssd = (T)0;                                                             \
    if (n < VAR_PARALLEL_MIN_LEN) {                                           \
      mean = simd_sum_##SUF(a, n) / (T)n;                                     \
      ssd = ssd_chunk_##SUF(a, n, mean);                                      \
    } else {                                                                  \
      int64_t nc = (n + PARALLEL_CHUNK - 1) / PARALLEL_CHUNK;                 \
      T s = (T)0;                                                             \
      for (int64_t c = 0; c < nc; ++c) {                                      \
        int64_t lo = c * PARALLEL_CHUNK;                                      \
        int64_t len = (n - lo < PARALLEL_CHUNK) ? n - lo : PARALLEL_CHUNK;    \
        s = s + simd_sum_##SUF(a + lo, len);                                  \
      }                                                                       \
      mean = s / (T)n;                                                        \
      for (int64_t c = 0; c < nc; ++c) {                                      \
        int64_t lo = c * PARALLEL_CHUNK;                                      \
        int64_t len = (n - lo < PARALLEL_CHUNK) ? n - lo : PARALLEL_CHUNK;    \
        ssd = ssd + ssd_chunk_##SUF(a + lo, len, mean);                       \
      }                                                                       \
    }                                                                         \
    return ssd / divisor;                                                     \
  }                                                                           \
  /* reduce.rs:323-412: comparison fold with a saw_nan flag; any NaN gives   \
     the canonical NaN, 0 for empty. Chunking does not change the result. */  \
  T orc_min_##SUF(const T* a, int64_t n) {                                    \
    if (n == 0) return (T)0;                                                  \
    T acc = INFV;                                                             \
    int saw_nan = 0;                                                          \
    for (int64_t i = 0; i < n; ++i) {                                         \
      saw_nan |= (a[i] != a[i]);                                              \
      if (a[i] < acc) acc = a[i];                                             \
    }                                                                         \
    return saw_nan ? NANV : acc;                                              \
  }                                                                           \
  T orc_max_##SUF(const T* a, int64_t n) {                                    \
    if (n == 0) return (T)0;                                                  \
    T acc = -INFV;                                                            \
    int saw_nan = 0;                                                          \
    for (int64_t i = 0; i < n; ++i) {                                         \
      saw_nan |= (a[i] != a[i]);                                              \
      if (a[i] > acc) acc = a[i];                                             \
    }                                                                         \
    return saw_nan ? NANV : acc;                                              \
  }                                                                           \
  /* reduce.rs:419: strict left-to-right product, 1 for empty. */             \
  T orc_prod_##SUF(const T* a, int64_t n) {                                   \
    T acc = (T)1;                                                             \
    for (int64_t i = 0; i < n; ++i) acc = acc * a[i];                         \
    return acc;                                                               \
  }
DEFINE_FLAT(float, f32, NAN, INFINITY)
DEFINE_FLAT(double, f64, (double)NAN, (double)INFINITY)

/* Integer full reductions: Array::sum generic fold (src/array/operations.rs
 * :303-320) and math::max/min(None) -> flat_max/flat_min
 * (src/math/aggregation.rs:173-181). Wrapping two's-complement addition. */
int64_t orc_sum_i64(const int64_t* a, int64_t n) {
  uint64_t s = 0;
  for (int64_t i = 0; i < n; ++i) s += (uint64_t)a[i];
  return (int64_t)s;
}
int64_t orc_max_i64(const int64_t* a, int64_t n) {
  if (n == 0) return 0;
  int64_t m = a[0];
  for (int64_t i = 1; i < n; ++i) if (a[i] > m) m = a[i];
  return m;
}
int64_t orc_min_i64(const int64_t* a, int64_t n) {
  if (n == 0) return 0;
  int64_t m = a[0];
  for (int64_t i = 1; i < n; ++i) if (a[i] < m) m = a[i];
  return m;
}
int64_t orc_prod_i64(const int64_t* a, int64_t n) {
  uint64_t p = 1;
  for (int64_t i = 0; i < n; ++i) p *= (uint64_t)a[i];
  return (int64_t)p;
}

/* ------------------------------------------------------------------------ */
/* Axis folds over an N-D strided view.                                      */
/*                                                                           */
/*  SUM  : math::sum(axis)  src/math/aggregation.rs:460-566 -- per lane a     */
/*         zero-seeded left-to-right fold `sum = sum + x` (fold :555-561);    */
/*         for integers Array::sum_axis src/array/operations.rs:75-156.       */
/*  MEAN : math::statistics::mean(axis) src/math/statistics/mod.rs:1021-1073 */
/*         -- the same fold, then `/ axis_len`.                               */
/*  MAX/MIN : math::max/min(axis) src/math/aggregation.rs:160-266, :289 --    */
/*         the first unordered element (NaN) short-circuits the lane and is   */
/*         its result, bit for bit; otherwise `val > acc` keeps the first max.*/
/*  PROD : ufunc multiply.reduce along an axis (src/ufunc_ops.rs:317),        */
/*         one-seeded left-to-right.                                          */
/*                                                                           */
/* The view is walked in logical order, which is what kernels::borrow::      */
/* operand (src/kernels/borrow.rs:59) materialises for non-contiguous views. */
/* Output order: NumPy row-major over the kept dimensions (the order         */
/* Array::sum_axis uses). Strides are in elements.                           */
/* ------------------------------------------------------------------------ */
enum { ORC_SUM = 0, ORC_MEAN = 1, ORC_MAX = 2, ORC_MIN = 3, ORC_PROD = 4 };

static void lane_bases(int ndim, const int64_t* shape, const int64_t* strides, int axis,
                       int64_t out_idx, int64_t* base) {
  int64_t off = 0, rem = out_idx;
  for (int d = ndim - 1; d >= 0; --d) {
    if (d == axis) continue;
    int64_t i = rem % shape[d];
    rem /= shape[d];
    off += i * strides[d];
  }
  *base = off;
}

#define DEFINE_AXIS_FLOAT(T, SUF)                                                         \
  void orc_axis_##SUF(int op, int ndim, const int64_t* shape, const int64_t* strides,     \
                      int axis, const T* x, T* out) {                                     \
    int64_t n_out = 1;                                                                    \
    for (int d = 0; d < ndim; ++d) if (d != axis) n_out *= shape[d];                      \
    const int64_t alen = shape[axis], ast = strides[axis];                                \
    _Pragma("omp parallel for schedule(static)")                                          \
    for (int64_t o = 0; o < n_out; ++o) {                                                 \
      int64_t b;                                                                          \
      lane_bases(ndim, shape, strides, axis, o, &b);                                      \
      const T* p = x + b;                                                                 \
      T acc;                                                                              \
      if (op == ORC_SUM || op == ORC_MEAN) {                                              \
        acc = (T)0;                                                                       \
        for (int64_t j = 0; j < alen; ++j) acc = acc + p[j * ast];                        \
        if (op == ORC_MEAN) acc = acc / (T)alen;                                          \
      } else if (op == ORC_PROD) {                                                        \
        acc = (T)1;                                                                       \
        for (int64_t j = 0; j < alen; ++j) acc = acc * p[j * ast];                        \
      } else {                                                                            \
        acc = p[0];                                                                       \
        if (acc == acc) {                                                                 \
          for (int64_t j = 1; j < alen; ++j) {                                            \
            T v = p[j * ast];                                                             \
            if (v != v) { acc = v; break; }                                               \
            if (op == ORC_MAX ? (v > acc) : (v < acc)) acc = v;                           \
          }                                                                               \
        }                                                                                 \
      }                                                                                   \
      out[o] = acc;                                                                       \
    }                                                                                     \
  }
DEFINE_AXIS_FLOAT(float, f32)
DEFINE_AXIS_FLOAT(double, f64)

/* math::statistics::var(axis, ddof) (src/math/statistics/mod.rs:1404-1500):
 * the lane mean from mean(axis) (zero-seeded left-to-right sum / n), then a
 * zero-seeded left-to-right sum of diff*diff (diff = val - mean), divided by
 * (axis_size - ddof); std = sqrt(var) (:1308). */
#define DEFINE_AXIS_VAR(T, SUF, SQRT)                                                      \
  void orc_axis_var_##SUF(int ndim, const int64_t* shape, const int64_t* strides,          \
                          int axis, int64_t ddof, int want_std, const T* x, T* out) {      \
    int64_t n_out = 1;                                                                     \
    for (int d = 0; d < ndim; ++d) if (d != axis) n_out *= shape[d];                       \
    const int64_t alen = shape[axis], ast = strides[axis];                                 \
    const T divisor = (T)(alen - ddof);                                                    \
    _Pragma("omp parallel for schedule(static)")                                           \
    for (int64_t o = 0; o < n_out; ++o) {                                                  \
      int64_t b;                                                                           \
      lane_bases(ndim, shape, strides, axis, o, &b);                                       \
      const T* p = x + b;                                                                  \
      T s = (T)0;                                                                          \
      for (int64_t j = 0; j < alen; ++j) s = s + p[j * ast];                               \
      const T mean = s / (T)alen;                                                          \
      T sq = (T)0;                                                                         \
      for (int64_t j = 0; j < alen; ++j) {                                                 \
        T diff = p[j * ast] - mean;                                                        \
        sq = sq + diff * diff;                                                             \
      }                                                                                    \
      T v = sq / divisor;                                                                  \
      out[o] = want_std ? SQRT(v) : v;                                                     \
    }                                                                                      \
  }
DEFINE_AXIS_VAR(float, f32, sqrtf)
DEFINE_AXIS_VAR(double, f64, sqrt)

/* math::statistics::argmax/argmin (src/math/statistics/mod.rs:79-198,
 * :218-330): axis = Some -> per lane, the first element starts, a later one
 * wins only if strictly greater (smaller); axis = None -> the same scan over
 * the flattened array. Written for any dtype through a comparison macro. */
#define DEFINE_ARG(T, SUF)                                                                 \
  void orc_axis_arg_##SUF(int want_max, int ndim, const int64_t* shape,                    \
                          const int64_t* strides, int axis, const T* x, int64_t* out) {    \
    int64_t n_out = 1;                                                                     \
    for (int d = 0; d < ndim; ++d) if (d != axis) n_out *= shape[d];                       \
    const int64_t alen = shape[axis], ast = strides[axis];                                 \
    for (int64_t o = 0; o < n_out; ++o) {                                                  \
      int64_t b;                                                                           \
      lane_bases(ndim, shape, strides, axis, o, &b);                                       \
      const T* p = x + b;                                                                  \
      T best = p[0];                                                                       \
      int64_t bi = 0;                                                                      \
      for (int64_t j = 1; j < alen; ++j) {                                                 \
        T v = p[j * ast];                                                                  \
        if (want_max ? (v > best) : (v < best)) { best = v; bi = j; }                      \
      }                                                                                    \
      out[o] = bi;                                                                         \
    }                                                                                      \
  }                                                                                        \
  int64_t orc_flat_arg_##SUF(int want_max, const T* x, int64_t n) {                        \
    T best = x[0];                                                                         \
    int64_t bi = 0;                                                                        \
    for (int64_t i = 1; i < n; ++i)                                                        \
      if (want_max ? (x[i] > best) : (x[i] < best)) { best = x[i]; bi = i; }               \
    return bi;                                                                             \
  }
DEFINE_ARG(float, f32)
DEFINE_ARG(double, f64)
DEFINE_ARG(int64_t, i64)

/* Integer axis folds: Array::sum_axis (src/array/operations.rs:75-156),
 * math::max/min(axis) for T: PartialOrd. There is no integer mean in the
 * reference (math::mean needs T: Float); MEAN here is the f64 lane sum / n
 * and has no reference counterpart. */
void orc_axis_i64(int op, int ndim, const int64_t* shape, const int64_t* strides, int axis,
                  const int64_t* x, void* out) {
  int64_t n_out = 1;
  for (int d = 0; d < ndim; ++d) if (d != axis) n_out *= shape[d];
  const int64_t alen = shape[axis], ast = strides[axis];
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < n_out; ++o) {
    int64_t b;
    lane_bases(ndim, shape, strides, axis, o, &b);
    const int64_t* p = x + b;
    if (op == ORC_SUM || op == ORC_MEAN) {
      uint64_t s = 0;
      for (int64_t j = 0; j < alen; ++j) s += (uint64_t)p[j * ast];
      if (op == ORC_MEAN)
        ((double*)out)[o] = (double)(int64_t)s / (double)alen;
      else
        ((int64_t*)out)[o] = (int64_t)s;
    } else if (op == ORC_PROD) {
      uint64_t s = 1;
      for (int64_t j = 0; j < alen; ++j) s *= (uint64_t)p[j * ast];
      ((int64_t*)out)[o] = (int64_t)s;
    } else {
      int64_t m = p[0];
      for (int64_t j = 1; j < alen; ++j) {
        int64_t v = p[j * ast];
        if (op == ORC_MAX ? (v > m) : (v < m)) m = v;
      }
      ((int64_t*)out)[o] = m;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Ufunc reduce / accumulate (src/ufunc_ops.rs) and cumsum / cumprod          */
/* (src/math/statistics/mod.rs:584-900).                                      */
/*                                                                           */
/* UfuncOp::apply (src/ufunc_ops.rs:153-181): add/sub/mul/div round once;    */
/* maximum/minimum give NaN (Rust's quiet-NaN bits) if either side is NaN,   */
/* else the left operand only if strictly greater (smaller).                 */
/* reduce_lane (:230-255): seeded by `initial` and folding every element, or */
/* by the lane's first element; an empty lane gives `initial`, the op's      */
/* identity (add 0, multiply 1) or an error.                                 */
/* reduce_full (:265-297): add / multiply on f32/f64 are seed + sum and      */
/* seed * prod through the tiered flat kernels; every other case is          */
/* reduce_lane over the flattened array.                                     */
/* accumulate (:523): add -> cumsum, a zero-seeded running sum per lane or   */
/* over the flattened array (:596-735); multiply -> cumprod, one-seeded      */
/* (:807-900); the rest seeded by the first element (accumulate_flat :452,   */
/* accumulate_along_axis :470). The f32/f64 flat cumsum of 64 or more        */
/* elements goes through scirs2-core's simd_cumsum, which is outside the     */
/* repository; it is restated as the same running sum (parity there is      */
/* tolerance-based).                                                          */
/* Op codes are nrs_ufunc's: ADD 2, SUB 3, MUL 4, DIV 5, MAX 11, MIN 12.     */
/* Integer arithmetic wraps (two's complement); integer DIV is not defined.  */
/* Outputs: reduce -> the kept dims row-major; accumulate -> the full shape  */
/* row-major (the flat case: n elements).                                    */
/* ------------------------------------------------------------------------ */
enum { U_ADD = 2, U_SUB = 3, U_MUL = 4, U_DIV = 5, U_MAX = 11, U_MIN = 12 };

static inline float qnan_f32(void) {
  uint32_t b = 0x7fc00000u;
  float f;
  memcpy(&f, &b, 4);
  return f;
}
static inline double qnan_f64(void) {
  uint64_t b = 0x7ff8000000000000ull;
  double f;
  memcpy(&f, &b, 8);
  return f;
}
static inline float uapply_f32(int op, float a, float b) {
  switch (op) {
    case U_ADD: return a + b;
    case U_SUB: return a - b;
    case U_MUL: return a * b;
    case U_DIV: return a / b;
    case U_MAX: return (a != a || b != b) ? qnan_f32() : (a > b ? a : b);
    default: return (a != a || b != b) ? qnan_f32() : (a < b ? a : b);
  }
}
static inline double uapply_f64(int op, double a, double b) {
  switch (op) {
    case U_ADD: return a + b;
    case U_SUB: return a - b;
    case U_MUL: return a * b;
    case U_DIV: return a / b;
    case U_MAX: return (a != a || b != b) ? qnan_f64() : (a > b ? a : b);
    default: return (a != a || b != b) ? qnan_f64() : (a < b ? a : b);
  }
}
static inline int64_t uapply_i64(int op, int64_t a, int64_t b) {
  switch (op) {
    case U_ADD: return (int64_t)((uint64_t)a + (uint64_t)b);
    case U_SUB: return (int64_t)((uint64_t)a - (uint64_t)b);
    case U_MUL: return (int64_t)((uint64_t)a * (uint64_t)b);
    case U_MAX: return a > b ? a : b;
    default: return a < b ? a : b;
  }
}
static inline float useq_sum_f32(const float* a, int64_t n) { return orc_sum_f32(a, n); }
static inline double useq_sum_f64(const double* a, int64_t n) { return orc_sum_f64(a, n); }
static inline int64_t useq_sum_i64(const int64_t* a, int64_t n) { return orc_sum_i64(a, n); }
static inline float useq_prod_f32(const float* a, int64_t n) { return orc_prod_f32(a, n); }
static inline double useq_prod_f64(const double* a, int64_t n) { return orc_prod_f64(a, n); }
static inline int64_t useq_prod_i64(const int64_t* a, int64_t n) { return orc_prod_i64(a, n); }

/* Offset of logical (row-major) element i of a strided view. */
static int64_t logical_offset(int ndim, const int64_t* shape, const int64_t* strides, int64_t i) {
  int64_t off = 0;
  for (int d = ndim - 1; d >= 0; --d) {
    off += (i % shape[d]) * strides[d];
    i /= shape[d];
  }
  return off;
}

#define DEFINE_UFUNC_SCAN(T, SUF)                                                           \
  /* Returns 0, or -1 for an empty lane with no initial and no identity. */                 \
  int orc_ufunc_reduce_##SUF(int op, int ndim, const int64_t* shape, const int64_t* strides, \
                             int axis, int has_init, T init, const T* x, T* out) {          \
    int64_t n = 1;                                                                          \
    for (int d = 0; d < ndim; ++d) n *= shape[d];                                           \
    if (axis < 0) {                                                                         \
      T* flat = (T*)malloc((size_t)(n > 0 ? n : 1) * sizeof(T));                            \
      for (int64_t i = 0; i < n; ++i) flat[i] = x[logical_offset(ndim, shape, strides, i)]; \
      int rc = 0;                                                                           \
      if (op == U_ADD) {                                                                    \
        out[0] = uapply_##SUF(U_ADD, has_init ? init : (T)0, useq_sum_##SUF(flat, n));      \
      } else if (op == U_MUL) {                                                             \
        out[0] = uapply_##SUF(U_MUL, has_init ? init : (T)1, useq_prod_##SUF(flat, n));     \
      } else if (n == 0) {                                                                  \
        if (has_init) out[0] = init; else rc = -1;                                          \
      } else {                                                                              \
        T acc = has_init ? uapply_##SUF(op, init, flat[0]) : flat[0];                       \
        for (int64_t i = 1; i < n; ++i) acc = uapply_##SUF(op, acc, flat[i]);               \
        out[0] = acc;                                                                       \
      }                                                                                     \
      free(flat);                                                                           \
      return rc;                                                                            \
    }                                                                                       \
    int64_t n_out = 1;                                                                      \
    for (int d = 0; d < ndim; ++d) if (d != axis) n_out *= shape[d];                        \
    const int64_t alen = shape[axis], ast = strides[axis];                                  \
    if (alen == 0 && n_out > 0 && !has_init && op != U_ADD && op != U_MUL) return -1;       \
    for (int64_t o = 0; o < n_out; ++o) {                                                   \
      int64_t b;                                                                            \
      lane_bases(ndim, shape, strides, axis, o, &b);                                        \
      const T* p = x + b;                                                                   \
      T acc;                                                                                \
      int64_t j0;                                                                           \
      if (has_init) { acc = init; j0 = 0; }                                                 \
      else if (alen == 0) { acc = (op == U_MUL) ? (T)1 : (T)0; j0 = 0; }                    \
      else { acc = p[0]; j0 = 1; }                                                          \
      for (int64_t j = j0; j < alen; ++j) acc = uapply_##SUF(op, acc, p[j * ast]);          \
      out[o] = acc;                                                                         \
    }                                                                                       \
    return 0;                                                                               \
  }                                                                                         \
  void orc_accumulate_##SUF(int op, int ndim, const int64_t* shape, const int64_t* strides, \
                            int axis, const T* x, T* out) {                                 \
    int64_t n = 1;                                                                          \
    for (int d = 0; d < ndim; ++d) n *= shape[d];                                           \
    if (n == 0) return;                                                                     \
    if (axis < 0) {                                                                         \
      T acc = (op == U_MUL) ? (T)1 : (T)0;                                                  \
      for (int64_t i = 0; i < n; ++i) {                                                     \
        T v = x[logical_offset(ndim, shape, strides, i)];                                   \
        if (i == 0 && op != U_ADD && op != U_MUL) acc = v;                                  \
        else acc = uapply_##SUF(op, acc, v);                                                \
        out[i] = acc;                                                                       \
      }                                                                                     \
      return;                                                                               \
    }                                                                                       \
    int64_t cstr[16];                                                                       \
    cstr[ndim - 1] = 1;                                                                     \
    for (int d = ndim - 2; d >= 0; --d) cstr[d] = cstr[d + 1] * shape[d + 1];               \
    int64_t n_out = n / shape[axis];                                                        \
    const int64_t alen = shape[axis], ast = strides[axis], ost = cstr[axis];                \
    _Pragma("omp parallel for schedule(static)")                                            \
    for (int64_t o = 0; o < n_out; ++o) {                                                   \
      int64_t b, ob;                                                                        \
      lane_bases(ndim, shape, strides, axis, o, &b);                                        \
      lane_bases(ndim, shape, cstr, axis, o, &ob);                                          \
      T acc = (op == U_MUL) ? (T)1 : (T)0;                                                  \
      for (int64_t j = 0; j < alen; ++j) {                                                  \
        T v = x[b + j * ast];                                                               \
        if (j == 0 && op != U_ADD && op != U_MUL) acc = v;                                  \
        else acc = uapply_##SUF(op, acc, v);                                                \
        out[ob + j * ost] = acc;                                                            \
      }                                                                                     \
    }                                                                                       \
  }
DEFINE_UFUNC_SCAN(float, f32)
DEFINE_UFUNC_SCAN(double, f64)
DEFINE_UFUNC_SCAN(int64_t, i64)

/* ------------------------------------------------------------------------ */
/* Elementwise.                                                              */
/*                                                                           */
/* y = exp(a*x + b): the eager spelling is three passes, `x * a` and `+ b`   */
/* through Array::map (src/array/operations.rs:182,450,464) and exp through   */
/* ElementWiseMath::exp (src/math/elementwise.rs:145); the fused spelling is */
/* ExprNode Unary(Exp, ScalarRhs(Add, ScalarRhs(Mul, Leaf, a), b)) evaluated */
/* in one zip (src/expr/owned.rs:557, src/expr/fused_eval.rs). Both round    */
/* after the multiply and after the add (never an FMA), so they agree bit    */
/* for bit; the exp itself is the platform's (simd_exp is un-vendored).      */
/* ------------------------------------------------------------------------ */
void orc_exp_affine_f32(const float* x, int64_t n, float a, float b, float* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    float t = x[i] * a;
    float u = t + b;
    y[i] = expf(u);
  }
}
void orc_exp_affine_f64(const double* x, int64_t n, double a, double b, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double t = x[i] * a;
    double u = t + b;
    y[i] = exp(u);
  }
}
/* Eager three-pass spelling (each pass materialises an array). */
void orc_exp_affine_eager_f32(const float* x, int64_t n, float a, float b, float* tmp, float* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) tmp[i] = x[i] * a;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) tmp[i] = tmp[i] + b;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] = expf(tmp[i]);
}

/* Binary ops with NumPy broadcasting: operators + - * / on Array
 * (src/array/arithmetic.rs:35-258) -> *_broadcast (src/array/operations.rs
 * :370-446) -> binary_serial (src/kernels/elementwise.rs:51). The output has
 * the broadcast shape; strides of broadcast dimensions are 0. */
enum { ORC_ADD = 0, ORC_SUB = 1, ORC_MUL = 2, ORC_DIV = 3 };
#define DEFINE_BINARY(T, SUF)                                                              \
  void orc_binary_##SUF(int op, int ndim, const int64_t* shape, const int64_t* sa,         \
                        const int64_t* sb, const T* a, const T* b, T* out) {               \
    int64_t n = 1;                                                                         \
    for (int d = 0; d < ndim; ++d) n *= shape[d];                                          \
    _Pragma("omp parallel for schedule(static)")                                           \
    for (int64_t i = 0; i < n; ++i) {                                                      \
      int64_t rem = i, oa = 0, ob = 0;                                                     \
      for (int d = ndim - 1; d >= 0; --d) {                                                \
        int64_t c = rem % shape[d];                                                        \
        rem /= shape[d];                                                                   \
        oa += c * sa[d];                                                                   \
        ob += c * sb[d];                                                                   \
      }                                                                                    \
      T x = a[oa], y = b[ob], r;                                                           \
      switch (op) {                                                                        \
        case ORC_ADD: r = x + y; break;                                                    \
        case ORC_SUB: r = x - y; break;                                                    \
        case ORC_MUL: r = x * y; break;                                                    \
        default: r = x / y; break;                                                         \
      }                                                                                    \
      out[i] = r;                                                                          \
    }                                                                                      \
  }
DEFINE_BINARY(float, f32)
DEFINE_BINARY(double, f64)

void orc_binary_i64(int op, int ndim, const int64_t* shape, const int64_t* sa, const int64_t* sb,
                    const int64_t* a, const int64_t* b, int64_t* out) {
  int64_t n = 1;
  for (int d = 0; d < ndim; ++d) n *= shape[d];
  for (int64_t i = 0; i < n; ++i) {
    int64_t rem = i, oa = 0, ob = 0;
    for (int d = ndim - 1; d >= 0; --d) {
      int64_t c = rem % shape[d];
      rem /= shape[d];
      oa += c * sa[d];
      ob += c * sb[d];
    }
    uint64_t x = (uint64_t)a[oa], y = (uint64_t)b[ob];
    int64_t r;
    switch (op) {
      case ORC_ADD: r = (int64_t)(x + y); break;
      case ORC_SUB: r = (int64_t)(x - y); break;
      case ORC_MUL: r = (int64_t)(x * y); break;
      default: r = (b[ob] == 0) ? 0 : a[oa] / b[ob]; break;
    }
    out[i] = r;
  }
}

/* ------------------------------------------------------------------------ */
/* GEMM: kernels::gemm::gemm_2d (src/kernels/gemm.rs:246-445).               */
/*  - overwrite semantics (beta = 0); m == 0 || n == 0 -> no-op; k == 0 ->    */
/*    zero-fill (gemm_float_tier :290-302);                                   */
/*  - f64/f32: packed matrixmultiply call under an M-only row split           */
/*    (:329-381), restated as a KC=256 K-blocked i-k-j loop per row chunk;    */
/*  - any other T: gemm_generic (:408-445), 64-blocked i-k-j after zeroing C. */
/* Row-major, leading dimensions lda/ldb/ldc in elements.                    */
/* ------------------------------------------------------------------------ */
#define GEMM_KC 256
#define DEFINE_GEMM_FLOAT(T, SUF)                                                          \
  void orc_gemm_##SUF(int64_t m, int64_t k, int64_t n, const T* A, int64_t lda,            \
                      const T* B, int64_t ldb, T* C, int64_t ldc) {                        \
    if (m == 0 || n == 0) return;                                                          \
    _Pragma("omp parallel for schedule(static)")                                           \
    for (int64_t i = 0; i < m; ++i) {                                                      \
      T* c = C + i * ldc;                                                                  \
      for (int64_t j = 0; j < n; ++j) c[j] = (T)0;                                         \
      for (int64_t kb = 0; kb < k; kb += GEMM_KC) {                                        \
        int64_t ke = kb + GEMM_KC < k ? kb + GEMM_KC : k;                                  \
        for (int64_t p = kb; p < ke; ++p) {                                                \
          T aik = A[i * lda + p];                                                          \
          const T* b = B + p * ldb;                                                        \
          for (int64_t j = 0; j < n; ++j) c[j] = c[j] + aik * b[j];                        \
        }                                                                                  \
      }                                                                                    \
    }                                                                                      \
  }
DEFINE_GEMM_FLOAT(float, f32)
DEFINE_GEMM_FLOAT(double, f64)

void orc_gemm_i64(int64_t m, int64_t k, int64_t n, const int64_t* A, int64_t lda,
                  const int64_t* B, int64_t ldb, int64_t* C, int64_t ldc) {
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j) C[i * ldc + j] = 0;
  const int64_t BS = 64;
  for (int64_t ib = 0; ib < m; ib += BS)
    for (int64_t kb = 0; kb < k; kb += BS)
      for (int64_t jb = 0; jb < n; jb += BS)
        for (int64_t i = ib; i < (ib + BS < m ? ib + BS : m); ++i)
          for (int64_t p = kb; p < (kb + BS < k ? kb + BS : k); ++p) {
            uint64_t aik = (uint64_t)A[i * lda + p];
            for (int64_t j = jb; j < (jb + BS < n ? jb + BS : n); ++j)
              C[i * ldc + j] = (int64_t)((uint64_t)C[i * ldc + j] + aik * (uint64_t)B[p * ldb + j]);
          }
}

/* ------------------------------------------------------------------------ */
/* Double-double reference (Dekker/Knuth error-free transforms, written out  */
/* with explicit two-product splitting so no FMA is needed). Used as the     */
/* "exact" oracle for GEMM error bounds: |C - C_dd| / (|A||B|)_ij.           */
/* ------------------------------------------------------------------------ */
static inline void two_sum(double a, double b, double* s, double* e) {
  double x = a + b;
  double bb = x - a;
  *e = (a - (x - bb)) + (b - bb);
  *s = x;
}
static inline void split_d(double a, double* hi, double* lo) {
  double t = 134217729.0 * a; /* 2^27 + 1 */
  double h = t - (t - a);
  *hi = h;
  *lo = a - h;
}
static inline void two_prod(double a, double b, double* p, double* e) {
  double x = a * b, ah, al, bh, bl;
  split_d(a, &ah, &al);
  split_d(b, &bh, &bl);
  *e = ((ah * bh - x) + ah * bl + al * bh) + al * bl;
  *p = x;
}

static void dd_dot(const double* a, int64_t sa, const double* b, int64_t sb, int64_t k,
                   double* hi_out, double* abs_out) {
  double hi = 0.0, lo = 0.0, ab = 0.0;
  for (int64_t p = 0; p < k; ++p) {
    double x = a[p * sa], y = b[p * sb], ph, pl, s, e;
    two_prod(x, y, &ph, &pl);
    two_sum(hi, ph, &s, &e);
    e += lo + pl;
    two_sum(s, e, &hi, &lo);
    ab += fabs(x) * fabs(y);
  }
  *hi_out = hi + lo;
  *abs_out = ab;
}

/* Full double-double GEMM (small sizes): C_dd rounded to double, and the
 * componentwise scale (|A||B|)_ij. */
void orc_gemm_dd(int64_t m, int64_t k, int64_t n, const double* A, int64_t lda,
                 const double* B, int64_t ldb, double* C, double* absAB) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j)
      dd_dot(A + i * lda, 1, B + j, ldb, k, &C[i * n + j], &absAB[i * n + j]);
}

/* Sampled double-double entries for large GEMMs (the 8192^3 error check). */
void orc_gemm_dd_sampled(int64_t k, const double* A, int64_t lda, const double* B,
                         int64_t ldb, int64_t count, const int64_t* rows, const int64_t* cols,
                         double* C, double* absAB) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t s = 0; s < count; ++s)
    dd_dot(A + rows[s] * lda, 1, B + cols[s], ldb, k, &C[s], &absAB[s]);
}

/* ------------------------------------------------------------------------ */
/* MLP tile selector (no reference counterpart). Restates the GPU network:   */
/* x[B,F] -> h1 = relu(x W1^T + b1) -> h2 = relu(h1 W2^T + b2) -> y = h2 W3^T */
/* + b3, weights stored as bf16 (given here already widened to float), fp32  */
/* accumulation. Loss = mean over the batch and outputs of mask*(y-t)^2.     */
/* Backward returns fp32 gradients of the loss w.r.t. every weight and bias. */
/* ------------------------------------------------------------------------ */
static void dense_fwd(const float* x, int64_t B, int64_t I, const float* W, const float* b,
                      int64_t O, int relu, float* y) {
  for (int64_t r = 0; r < B; ++r)
    for (int64_t o = 0; o < O; ++o) {
      float acc = 0.0f;
      for (int64_t i = 0; i < I; ++i) acc += x[r * I + i] * W[o * I + i];
      acc += b[o];
      y[r * O + o] = (relu && acc < 0.0f) ? 0.0f : acc;
    }
}

float orc_mlp_forward_backward(int64_t B, int64_t F, int64_t H, int64_t V, const float* x,
                               const float* t, const float* mask, const float* W1,
                               const float* b1, const float* W2, const float* b2,
                               const float* W3, const float* b3, float* y, float* gW1,
                               float* gb1, float* gW2, float* gb2, float* gW3, float* gb3) {
  float* h1 = (float*)calloc((size_t)(B * H), sizeof(float));
  float* h2 = (float*)calloc((size_t)(B * H), sizeof(float));
  float* d3 = (float*)calloc((size_t)(B * V), sizeof(float));
  float* d2 = (float*)calloc((size_t)(B * H), sizeof(float));
  float* d1 = (float*)calloc((size_t)(B * H), sizeof(float));
  dense_fwd(x, B, F, W1, b1, H, 1, h1);
  dense_fwd(h1, B, H, W2, b2, H, 1, h2);
  dense_fwd(h2, B, H, W3, b3, V, 0, y);
  double loss = 0.0;
  float denom = 0.0f;
  for (int64_t i = 0; i < B * V; ++i) denom += mask[i];
  if (denom <= 0.0f) denom = 1.0f;
  for (int64_t i = 0; i < B * V; ++i) {
    float diff = y[i] - t[i];
    loss += (double)(mask[i] * diff * diff);
    d3[i] = 2.0f * mask[i] * diff / denom;
  }
  /* layer 3 */
  memset(gW3, 0, sizeof(float) * (size_t)(V * H));
  memset(gb3, 0, sizeof(float) * (size_t)V);
  for (int64_t r = 0; r < B; ++r)
    for (int64_t o = 0; o < V; ++o) {
      gb3[o] += d3[r * V + o];
      for (int64_t i = 0; i < H; ++i) gW3[o * H + i] += d3[r * V + o] * h2[r * H + i];
    }
  for (int64_t r = 0; r < B; ++r)
    for (int64_t i = 0; i < H; ++i) {
      float acc = 0.0f;
      for (int64_t o = 0; o < V; ++o) acc += d3[r * V + o] * W3[o * H + i];
      d2[r * H + i] = h2[r * H + i] > 0.0f ? acc : 0.0f;
    }
  /* layer 2 */
  memset(gW2, 0, sizeof(float) * (size_t)(H * H));
  memset(gb2, 0, sizeof(float) * (size_t)H);
  for (int64_t r = 0; r < B; ++r)
    for (int64_t o = 0; o < H; ++o) {
      gb2[o] += d2[r * H + o];
      for (int64_t i = 0; i < H; ++i) gW2[o * H + i] += d2[r * H + o] * h1[r * H + i];
    }
  for (int64_t r = 0; r < B; ++r)
    for (int64_t i = 0; i < H; ++i) {
      float acc = 0.0f;
      for (int64_t o = 0; o < H; ++o) acc += d2[r * H + o] * W2[o * H + i];
      d1[r * H + i] = h1[r * H + i] > 0.0f ? acc : 0.0f;
    }
  /* layer 1 */
  memset(gW1, 0, sizeof(float) * (size_t)(H * F));
  memset(gb1, 0, sizeof(float) * (size_t)H);
  for (int64_t r = 0; r < B; ++r)
    for (int64_t o = 0; o < H; ++o) {
      gb1[o] += d1[r * H + o];
      for (int64_t i = 0; i < F; ++i) gW1[o * F + i] += d1[r * H + o] * x[r * F + i];
    }
  free(h1);
  free(h2);
  free(d3);
  free(d2);
  free(d1);
  return (float)(loss / (double)denom);
}
