/*
 * numrs_gpu.h -- C ABI of the GB300 (sm_103a) implementation of NumRS2's
 * crate-private `kernels` dispatch layer: GEMM, axis/flat reductions and
 * elementwise/fused ufuncs behind `Array<T>`.
 *
 * Every entry point names the reference interface it replaces
 * (numrs2 0.4.1, paths relative to the crate root). The reference passes Rust
 * slices (`&[T]`, `&mut [T]`) and closures; this ABI passes plain pointers,
 * sizes and element strides, and op-code programs instead of closures.
 *
 * Conventions
 *  - All data pointers given to compute entry points are DEVICE pointers
 *    (cudaMalloc / nrs_malloc / any allocator of the same context); the caller
 *    owns them. Host data is moved with nrs_memcpy_h2d / nrs_memcpy_d2h.
 *  - Strides are in ELEMENTS (not bytes), may be 0 for broadcast dimensions,
 *    and must be non-negative.
 *  - Work is enqueued on the handle's stream (nrs_set_stream); calls return
 *    once the work is enqueued. Results are visible after nrs_synchronize or
 *    any later work on the same stream.
 *  - Status codes: NRS_OK (0) or a negative nrs_status. Shape/axis/dtype
 *    errors are reported before anything is launched (the reference raises
 *    them one layer up as NumRs2Error, src/error/legacy.rs:12-60). A device
 *    fault or a device-side bounded wait that gave up is reported by the call
 *    that observed it (NRS_ERR_CUDA / NRS_ERR_TIMEOUT) and by nrs_synchronize.
 *  - Threading: a handle is used by one host thread at a time; distinct
 *    handles are independent. The library never falls back to the CPU.
 */
#ifndef NUMRS_GPU_H
#define NUMRS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NRS_ABI_VERSION 3

typedef struct nrs_handle nrs_handle;

/* Element types. The reference dispatches on TypeId through kernels::cast
 * (src/kernels/cast.rs:35-140); here the dtype is explicit. */
typedef enum nrs_dtype { NRS_F32 = 0, NRS_F64 = 1, NRS_I32 = 2, NRS_I64 = 3 } nrs_dtype;

typedef enum nrs_status {
  NRS_OK = 0,
  NRS_ERR_INVALID = -1,     /* null pointer, bad enum or negative size     */
  NRS_ERR_SHAPE = -2,       /* ShapeMismatch / DimensionMismatch           */
  NRS_ERR_DTYPE = -3,       /* operation not defined for this dtype        */
  NRS_ERR_AXIS = -4,        /* "Axis {} out of bounds for array of ..."     */
  NRS_ERR_EMPTY = -5,       /* InvalidOperation on an empty array          */
  NRS_ERR_STRIDE = -6,      /* negative or overflowing stride              */
  NRS_ERR_CUDA = -7,        /* CUDA runtime error (message: nrs_last_error) */
  NRS_ERR_TIMEOUT = -8,     /* a device-side bounded wait gave up          */
  NRS_ERR_ALLOC = -9,       /* workspace allocation failed                 */
  NRS_ERR_UNSUPPORTED = -10,
  NRS_ERR_TOO_LARGE = -11,  /* size beyond a documented maximum            */
  NRS_ERR_IO = -12          /* a file could not be opened, read or written */
} nrs_status;

/* ---------------------------------------------------------------------- */
/* Handle, stream and memory                                                */
/* ---------------------------------------------------------------------- */
int nrs_abi_version(void);
const char* nrs_status_string(int status);

/* Creates a handle bound to `device`, with its own non-blocking stream. */
int nrs_create(int device, nrs_handle** out);
int nrs_destroy(nrs_handle* h);
/* Enqueue on a caller-owned cudaStream_t; NULL means CUDA's default stream. */
int nrs_set_stream(nrs_handle* h, void* cuda_stream);
/* Enqueue on the handle's own non-blocking stream (the state after create). */
int nrs_use_own_stream(nrs_handle* h);
void* nrs_get_stream(nrs_handle* h);
/* Sizes the handle's grids for at most `sms` SMs (0 = all of the device's),
 * for sharing the GPU with concurrent work. No reference counterpart. Results
 * do not depend on it: every plan that decides a rounding order (a GEMM's k
 * split, a flattened scan's segments, chunk groupings) is fixed by the
 * problem's sizes alone, as the reference's results are independent of its
 * thread count (src/kernels/gemm.rs:364-381). */
int nrs_set_sm_budget(nrs_handle* h, int sms);
/* Waits for the stream, then reports any device-side error flag. */
int nrs_synchronize(nrs_handle* h);
/* Test support for the bounded-wait path (no reference counterpart): the
 * next axis reduction on this handle served by the column-fold TMA pipeline
 * leaves its first CTA's first tile unloaded, so that CTA waits on a barrier
 * nothing completes; the wait gives up after `probes` probes, the CTA sets
 * the device error word and returns, and the next nrs_synchronize reports
 * NRS_ERR_TIMEOUT. Nothing faults or hangs, and the handle stays usable
 * (that launch's output for the first 64 lanes is not written). */
int nrs_test_expire_next_wait(nrs_handle* h, uint32_t probes);
/* Message of the last failing call on this handle ("" if none). */
const char* nrs_last_error(nrs_handle* h);

int nrs_malloc(nrs_handle* h, size_t bytes, void** dptr);
int nrs_free(nrs_handle* h, void* dptr);
int nrs_host_alloc(nrs_handle* h, size_t bytes, void** hptr); /* pinned */
int nrs_host_free(nrs_handle* h, void* hptr);
int nrs_memcpy_h2d(nrs_handle* h, void* dst, const void* src, size_t bytes);
int nrs_memcpy_d2h(nrs_handle* h, void* dst, const void* src, size_t bytes);

/* Seeded SplitMix64 input generator, element i = f(mix((seed ^ GAMMA) +
 * (i+1) * GAMMA)) with the step/mix constants of the reference's test
 * generator (tests/test_expr_fused_equivalence.rs:96-112).
 *   NRS_RNG_UNIFORM : p0 + (p1 - p0) * u,  u = (x >> 11) * 2^-53   (f32/f64)
 *   NRS_RNG_NORMAL  : p0 + p1 * z, Box-Muller on draws 2i, 2i+1      (f32/f64)
 *   NRS_RNG_INT     : (x >> s) + p0 with s = 64 - log2(p1)           (i64/i32)
 *   NRS_RNG_OZAKI   : U(-0.5,0.5) * exp(p0 * z), z normal            (f64)  */
typedef enum nrs_rng { NRS_RNG_UNIFORM = 0, NRS_RNG_NORMAL = 1, NRS_RNG_INT = 2, NRS_RNG_OZAKI = 3 } nrs_rng;
int nrs_fill_random(nrs_handle* h, int dtype, int dist, uint64_t seed, int64_t n, double p0,
                    double p1, void* out);

/* ---------------------------------------------------------------------- */
/* Reductions                                                               */
/* ---------------------------------------------------------------------- */
typedef enum nrs_reduce_op {
  NRS_SUM = 0, NRS_MEAN = 1, NRS_MAX = 2, NRS_MIN = 3, NRS_PROD = 4, NRS_VAR = 5, NRS_STD = 6,
  NRS_ARGMAX = 7, NRS_ARGMIN = 8 /* output: int64 indices */
} nrs_reduce_op;
#define NRS_AXIS_NONE INT64_MIN

/* Reduce an N-D strided view (ndim <= 8) of `x`.
 *
 * axis == NRS_AXIS_NONE: flat reduction of all elements in logical order,
 *   out = 1 element. Replaces kernels::reduce::{sum,mean,var,min,max,prod}_
 *   {f64,f32} (src/kernels/reduce.rs:204-444; empty -> 0, prod empty -> 1,
 *   min/max: any NaN -> NaN) and, for i64, Array::sum (src/array/
 *   operations.rs:303) and math::max/min(None) (src/math/aggregation.rs:160,
 *   :289). VAR/STD use `ddof` as reduce::var does (divisor n - ddof).
 * axis >= 0 or negative (counted from the end, as the reference does):
 *   per-lane fold along `axis`, out = prod(kept dims) elements in row-major
 *   order of the kept dimensions. Replaces math::sum(axis)
 *   (src/math/aggregation.rs:416, fold :555-561), math::statistics::mean(axis)
 *   (src/math/statistics/mod.rs:971), math::max/min(axis)
 *   (src/math/aggregation.rs:160, :289) and Array::sum_axis
 *   (src/array/operations.rs:75). Each lane is folded left to right from a
 *   zero seed (sum/mean), one seed (prod) or its first element (max/min, the
 *   first NaN short-circuits and is the lane's result bit for bit), so float
 *   lane sums match the reference's fold order exactly.
 *   MAX/MIN/MEAN over an empty axis return NRS_ERR_EMPTY (the reference's
 *   "Cannot find max of empty array"); SUM gives zeros.
 *   VAR/STD along an axis follow math::statistics::var/std(axis, ddof)
 *   (src/math/statistics/mod.rs:1334-1500, :1308): per-lane mean, then the
 *   left-to-right sum of (x - mean)^2, / (axis length - ddof), sqrt for STD;
 *   axis length <= ddof returns NRS_ERR_EMPTY ("Degrees of freedom ...").
 *   ARGMAX/ARGMIN follow math::statistics::argmax/argmin
 *   (src/math/statistics/mod.rs:79, :218): first index of the strictly
 *   greatest (smallest) value, NaN never chosen unless it is element 0 of
 *   its lane; `out` is int64.
 * dtypes: F32, F64, I64 (I32 for SUM/MAX/MIN/PROD/ARG*). For I64, MEAN writes
 *   f64 (no reference counterpart: math::mean requires T: Float). */
int nrs_reduce(nrs_handle* h, int dtype, int op, int ndim, const int64_t* shape,
               const int64_t* strides, int64_t axis, int64_t ddof, const void* x, void* out);

/* Allocation-free flat reduction. This entry point has no counterpart in the
 * reference; it exists for callers that must not let a library allocate
 * device memory: code running under another runtime's memory discipline (a
 * serving stack or framework allocator that owns and budgets all device
 * memory) and latency-critical loops that cannot afford the device-wide
 * synchronisation a cudaMalloc may cause. It computes what
 * nrs_reduce(..., NRS_AXIS_NONE, ...) computes for a contiguous f32/f64
 * buffer of n elements (op NRS_SUM, NRS_MEAN, NRS_MAX or NRS_MIN; same
 * kernels, same chunk order, same result) on `cuda_stream` (NULL = default
 * stream) of the CURRENT device, with no handle and no allocation: the chunk
 * partials live in a 128 KiB (+256 B) file-scope device array that every GPU
 * holds from the moment it loads the library until the process exits.
 *   - Limit: n <= 67,108,864 (8192 chunks of 8192); larger n returns
 *     NRS_ERR_TOO_LARGE before anything is launched.
 *   - The first call on a device looks the array's address up (and the SM
 *     count) with that device current and caches them with the current
 *     context; a call in another context of the device (for instance after
 *     cudaDeviceReset) looks them up again. Make the first call in a context
 *     before any stream capture.
 *   - `cuda_stream` must belong to the current device.
 *   - All calls share the one array and it keeps the last call's contents;
 *     every call rewrites each partial it reads, so nothing has to start at
 *     zero. Calls whose work overlaps on the GPU (different streams, no
 *     ordering between them) race on the array: serialise them.
 *   - Returns NRS_OK, NRS_ERR_INVALID, NRS_ERR_DTYPE, NRS_ERR_TOO_LARGE or
 *     NRS_ERR_CUDA (there is no handle, hence no message string). */
int nrs_reduce_flat_noalloc(void* cuda_stream, int dtype, int op, int64_t n, const void* x,
                            void* out);

/* ---------------------------------------------------------------------- */
/* Elementwise ufunc programs                                               */
/* ---------------------------------------------------------------------- */
/* A closure `|x, y| ...` of kernels::elementwise::{binary,unary}_* or an
 * expr::ExprNode tree (src/expr/owned.rs:204; Leaf/Binary/ScalarRhs/
 * ScalarLhs/Unary) becomes a postfix program over a small value stack.
 * Every op rounds once: MUL followed by ADD is two roundings, never an FMA,
 * as in src/expr/fused_eval.rs:17-21. */
typedef enum nrs_ufunc_code {
  NRS_OP_INPUT = 0,  /* push inputs[arg][i]           */
  NRS_OP_SCALAR = 1, /* push scalar                   */
  NRS_OP_ADD = 2, NRS_OP_SUB = 3, NRS_OP_MUL = 4, NRS_OP_DIV = 5, /* pop b, pop a, push a op b */
  NRS_OP_NEG = 6, NRS_OP_ABS = 7, NRS_OP_SQRT = 8, NRS_OP_EXP = 9, NRS_OP_LN = 10, /* unary */
  NRS_OP_MAX = 11, NRS_OP_MIN = 12
} nrs_ufunc_code;

typedef struct nrs_ufunc_op {
  int32_t code;
  int32_t arg;
  double scalar;
} nrs_ufunc_op;

#define NRS_UFUNC_MAX_OPS 32
#define NRS_UFUNC_MAX_INPUTS 8
#define NRS_UFUNC_MAX_DIMS 8

/* out[i] = program(inputs[0][i], ...) over the broadcast shape `shape`
 * (ndim dims). in_strides is n_inputs x ndim element strides (0 on
 * broadcast dims, i.e. NumPy broadcasting as in *_broadcast,
 * src/array/operations.rs:370-446); out_strides NULL means row-major
 * contiguous. Integer dtypes accept ADD/SUB/MUL/DIV/NEG/ABS/MAX/MIN with
 * wrapping arithmetic (DIV by zero gives 0); EXP/LN/SQRT need F32/F64.
 * Replaces binary_serial/binary_{f64,f32}/binary_dispatch/unary_dispatch
 * (src/kernels/elementwise.rs:51-258), Array::map scalar ops
 * (src/array/operations.rs:182, :450-475), ElementWiseMath::exp
 * (src/math/elementwise.rs:145), ufuncs::exp (src/ufuncs.rs:398) and
 * ExprNode::eval (src/expr/owned.rs:557). */
int nrs_ufunc(nrs_handle* h, int dtype, const nrs_ufunc_op* prog, int prog_len, int ndim,
              const int64_t* shape, int n_inputs, const void* const* inputs,
              const int64_t* in_strides, void* out, const int64_t* out_strides);

/* y[i] = exp((a * x[i]) + b), two roundings before the exp, contiguous f32 or
 * f64: the fused form of `(x * a + b).exp()` (eager: three Array::map/exp
 * passes; fused: ExprNode Unary(Exp, ScalarRhs(Add, ScalarRhs(Mul, Leaf, a),
 * b))). One HBM pass: 8 B/elem for f32. */
int nrs_exp_affine(nrs_handle* h, int dtype, int64_t n, const void* x, double a, double b,
                   void* y);

/* ---------------------------------------------------------------------- */
/* Ufunc reduce / accumulate                                                */
/* ---------------------------------------------------------------------- */
/* `op` is one of the binary op codes of nrs_ufunc_op: NRS_OP_ADD, _SUB,
 * _MUL, _DIV, _MAX, _MIN (UfuncOp::{Add, Subtract, Multiply, Divide,
 * Maximum, Minimum}, src/ufunc_ops.rs:106). The op is UfuncOp::apply
 * (:153-181): one rounding; maximum/minimum give NaN if either side is NaN,
 * else the left operand only if strictly greater (smaller). Integer dtypes
 * wrap; integer DIV returns NRS_ERR_DTYPE. */

/* op.reduce(x, axis, initial): replaces ufunc_ops::ufunc_reduce
 * (src/ufunc_ops.rs:417). `initial` points to one host value of `dtype`, or
 * is NULL for none.
 * axis == NRS_AXIS_NONE (reduce_full, :265): add / multiply are
 *   initial-or-0 + the flat sum and initial-or-1 * the flat product (the
 *   tiered flat kernels of nrs_reduce); maximum / minimum / subtract /
 *   divide fold the flattened array from `initial` or from its first
 *   element. out = 1 element.
 * axis given (reduce_along_axis, :317): every lane folds left to right from
 *   `initial` or from its first element (reduce_lane, :230); out = the kept
 *   dimensions in row-major order. Negative axes count from the end.
 * Empty input or empty lanes without `initial`: add gives 0, multiply 1,
 * the rest NRS_ERR_EMPTY ("zero-size array to reduction operation maximum
 * which has no identity"). */
int nrs_ufunc_reduce(nrs_handle* h, int dtype, int op, int ndim, const int64_t* shape,
                     const int64_t* strides, int64_t axis, const void* initial, const void* x,
                     void* out);

/* op.accumulate(x, axis): replaces ufunc_ops::ufunc_accumulate
 * (src/ufunc_ops.rs:523) and math::cumsum / cumprod
 * (src/math/statistics/mod.rs:584, :795). add is cumsum (every lane, or the
 * flattened array, a running sum from 0), multiply is cumprod (from 1), the
 * other ops start from the first element (accumulate_flat :452,
 * accumulate_along_axis :470).
 * axis given: out has x's shape; out_strides (NULL = row-major contiguous)
 *   are its element strides. Lanes are folded left to right, bit-identical
 *   to the reference's loops.
 * axis == NRS_AXIS_NONE: out is the prod(shape) values of the flattened array
 *   in logical order, contiguous (out_strides ignored). Maximum / minimum and
 *   integer add / multiply are exact; f32/f64 add / multiply of 64 or more
 *   elements reassociate the running sum / product (a chunked parallel
 *   scan), like the reference's f32/f64 cumsum at that size (scirs2-core's
 *   simd_cumsum); subtract / divide (and float add / multiply below 64
 *   elements) run the strict left-to-right chain.
 * Empty input: nothing is written. */
int nrs_accumulate(nrs_handle* h, int dtype, int op, int ndim, const int64_t* shape,
                   const int64_t* strides, int64_t axis, const void* x, void* out,
                   const int64_t* out_strides);

/* ---------------------------------------------------------------------- */
/* NPY / NPZ files straight to and from device memory                       */
/* ---------------------------------------------------------------------- */
/* Replaces io::npy_npz (src/io/npy_npz.rs): the payload moves between the
 * file and device memory through pinned staging slots (parallel pread /
 * pwrite overlapped with cudaMemcpyAsync on the handle's stream); it never
 * lands in a pageable host array. */
#define NRS_NPY_MAX_DIMS 32

typedef struct nrs_npy_info {
  char descr[16];        /* the header's 'descr', e.g. "<f4"                    */
  int dtype;             /* NRS_F32/F64/I32/I64 for <f4 <f8 <i4 <i8, else -1    */
  int itemsize;          /* bytes per element                                   */
  int fortran_order;     /* 1 if the header says True (the payload is moved as
                            stored, as the reference reads it)                 */
  int ndim;
  int64_t shape[NRS_NPY_MAX_DIMS];
  int64_t data_offset;   /* file offset of the first payload byte               */
  int64_t nbytes;        /* payload bytes (prod(shape) * itemsize)               */
} nrs_npy_info;

/* Parses the NPY header that starts at file offset `offset` (0 for an .npy
 * file, nrs_npz_locate's offset for an NPZ member) with parse_npy_header's
 * rules (src/io/npy_npz.rs:263-339): magic, version 1.0 only
 * (NRS_ERR_UNSUPPORTED otherwise), 'descr' and 'shape' by string search.
 * Checks that the file holds the whole payload. `h` may be NULL (no GPU is
 * touched; errors then have no message). */
int nrs_npy_inspect(nrs_handle* h, const char* path, int64_t offset, nrs_npy_info* info);

/* Finds NPZ member "<array_name>.npy" (load_npz_array, :541) or, with
 * array_name NULL, the first ".npy" member (read_npz_generic, :465) through
 * the ZIP central directory (ZIP64 included) and returns the file offset of
 * its embedded NPY file. Compressed members return NRS_ERR_UNSUPPORTED: only
 * stored members (what serialize_to_file writes, :369-375) are read in
 * place. `h` may be NULL. */
int nrs_npz_locate(nrs_handle* h, const char* path, const char* array_name, int64_t* npy_offset,
                   int64_t* npy_bytes);

/* Copies the payload described by `info` (from nrs_npy_inspect) into device
 * memory `dst` (dst_bytes >= info->nbytes), enqueued on the handle's stream;
 * returns once every byte has been copied. */
int nrs_npy_read(nrs_handle* h, const char* path, const nrs_npy_info* info, void* dst,
                 int64_t dst_bytes);

/* Writes device array `src` (row-major contiguous, dtype F32/F64/I32/I64) as
 * an NPY file with construct_npy_header's header, byte for byte
 * (src/io/npy_npz.rs:48-99: version 1.0, no trailing newline). Returns once
 * the file is written. */
int nrs_npy_write(nrs_handle* h, const char* path, int dtype, int ndim, const int64_t* shape,
                  const void* src);

/* ---------------------------------------------------------------------- */
/* GEMM                                                                     */
/* ---------------------------------------------------------------------- */
#define NRS_GEMM_ACCUMULATE 1u /* C += A*B (Array::matmul_to, src/array/operations_optimized.rs:385) */
#define NRS_GEMM_TRANS_A 2u    /* A is stored k x m (lda >= m): a transposed view of A  */
#define NRS_GEMM_TRANS_B 4u    /* B is stored n x k (ldb >= k): a transposed view of B  */

typedef enum nrs_gemm_variant {
  NRS_GEMM_AUTO = 0,     /* autotuner choice (plain kernels only; never Ozaki) */
  NRS_GEMM_DMMA = 1,     /* f64: FP64 tensor-core mma.sync m8n8k4 tiles        */
  NRS_GEMM_SIMT = 2,     /* f32 / f64: register-tiled CUDA-core GEMM           */
  NRS_GEMM_GENERIC = 3,  /* any dtype: one thread per C element (ints, checks) */
  NRS_GEMM_SIMT_SMALL = 4 /* f32: 32x32 tiles for small problems               */
} nrs_gemm_variant;

/* C := A*B (or C += A*B with NRS_GEMM_ACCUMULATE) for row-major m x k A,
 * k x n B, m x n C with leading dimensions lda/ldb/ldc.
 * Replaces kernels::gemm::gemm_2d (src/kernels/gemm.rs:246): m == 0 or
 * n == 0 is a no-op, k == 0 zero-fills C (overwrite contract, :294-302);
 * integer dtypes wrap like gemm_generic (:408). */
int nrs_gemm(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n, const void* A,
             int64_t lda, const void* B, int64_t ldb, void* C, int64_t ldc, unsigned flags,
             int variant);

/* Measures a compute pipe's rate on the handle's device (TFLOP/s, best of
 * three timed launches after a warm-up, CUDA events on the handle's stream;
 * returns after synchronising). No reference counterpart: the denominators
 * of the GEMM rooflines. NRS_PEAK_FP64_DMMA: register-resident chains of
 * mma.sync m8n8k4 f64 (512 flops each) on every SM; NRS_PEAK_FP32_FMA:
 * chains of fp32 FMA (2 flops each). */
typedef enum nrs_peak_kind { NRS_PEAK_FP64_DMMA = 0, NRS_PEAK_FP32_FMA = 1 } nrs_peak_kind;
int nrs_probe_peak(nrs_handle* h, int kind, double* tflops);

/* ---------------------------------------------------------------------- */
/* f64-accurate split GEMM (Ozaki scheme on BF16 tcgen05 tensor cores)      */
/* ---------------------------------------------------------------------- */
typedef struct nrs_ozaki_info {
  int32_t slices;        /* slices per operand used; 0 = the call ran the native
                            FP64 (DMMA) GEMM instead (see below)              */
  int32_t products;      /* slice-pair GEMM work units executed              */
  int32_t slice_bits;    /* bits carried by each slice after the first       */
  int32_t k_chunk;       /* K block inside which fp32 accumulation is exact  */
  double est_rel_error;  /* slices = 0 (auto): estimated max_ij |C - AB|_ij /
                            (|A||B|)_ij; explicit count: a-priori bound on
                            |C - AB| / (rowmax|A| colmax|B| k)               */
  double spread;         /* auto: max_ij R_ij measured (below); else 0       */
} nrs_ozaki_info;

/* C := A*B (or C += A*B with NRS_GEMM_ACCUMULATE) in f64 accuracy from BF16
 * slice products on tcgen05 tensor cores with per-row (A) / per-column (B)
 * power-of-two scaling, exact fp32 accumulation inside K blocks, exact int32
 * sums carried across the slice diagonals (one retired digit per diagonal),
 * one exactly rounded conversion to f64 per element.
 * No reference counterpart: replaces the f64 tier of gemm_2d
 * (src/kernels/gemm.rs:290) for large problems. Operands as in nrs_gemm
 * (row-major, NRS_GEMM_TRANS_A / _TRANS_B for transposed views); operands
 * must be finite unless slices = 0.
 *
 * slices = 0 (automatic) measures how far apart the magnitudes that meet in
 * each dot product are: with A' and B' the operands scaled by their row and
 * column exponents, R_ij = sum_k (|a'_ik| + |b'_kj|) / (|A'||B'|)_ij (a BF16
 * tensor-core product of |A'| and |B'| and the row / column sums; if some
 * (|A'||B'|)_ij is 0, a second pass counts only the k where the other factor
 * is nonzero). Each operand is then carried to 53 + log2(max R) bits, which
 * keeps max_ij |C - AB|_ij / (|A||B|)_ij at about 2^-53. If no count within
 * the limits (16 slices, 126 bits, exact int32 sums for this K, an exact
 * total within 128 bits: b (S - 1) <= 95 for b-bit digits) reaches that, or an operand holds Inf or NaN, the call runs the native FP64 DMMA
 * GEMM and reports slices = 0. The automatic mode reads the measured spread
 * back to the host: one synchronisation of the handle's stream, so it
 * cannot be captured in a CUDA graph; pass the count a previous call
 * reported to capture.
 * slices = 1..16 uses that count as given. `info` may be NULL. */
int nrs_gemm_ozaki(nrs_handle* h, int64_t m, int64_t k, int64_t n, const double* A, int64_t lda,
                   const double* B, int64_t ldb, double* C, int64_t ldc, unsigned flags, int slices,
                   nrs_ozaki_info* info);

/* ---------------------------------------------------------------------- */
/* Grouped persistent launch (no reference counterpart; the reference's     */
/* closest analogue is a caller loop over Array::matmul or batched_gemm,    */
/* src/array/linalg.rs:56-136, and a loop over reduce::sum_*).              */
/* ---------------------------------------------------------------------- */
typedef struct nrs_gemm_desc {
  int32_t dtype; /* NRS_F32 or NRS_F64 */
  uint32_t flags; /* NRS_GEMM_ACCUMULATE only */
  int64_t m, k, n;
  const void* A;
  int64_t lda;
  const void* B;
  int64_t ldb;
  void* C;
  int64_t ldc;
} nrs_gemm_desc;

typedef struct nrs_rowreduce_desc {
  int32_t dtype; /* NRS_F32, NRS_F64 or NRS_I64 */
  int32_t op;    /* NRS_SUM, NRS_MEAN, NRS_MAX, NRS_MIN */
  int64_t len;
  const void* x; /* contiguous */
  void* out;     /* one element */
} nrs_rowreduce_desc;

/* Many f64 GEMMs on the tensor cores in one pass (no reference counterpart;
 * the caller loop over gemm_2d, src/kernels/gemm.rs:246): every row-major
 * problem's slices are made by one launch of each slicing kernel and every
 * tile runs in one persistent tcgen05 launch, with one slice count for the
 * group (0 = measured from each problem's spread, one read-back each; the
 * largest count is used). Problems with transposed operands, Inf / NaN or a
 * spread no count covers run on FP64 DMMA instead; on_tensor_cores[i]
 * (may be NULL) says which. Returns after synchronising the stream. */
int nrs_gemm_ozaki_grouped(nrs_handle* h, int64_t count, const nrs_gemm_desc* descs, int slices,
                           int* on_tensor_cores, nrs_ozaki_info* info);

typedef struct nrs_plan nrs_plan;

/* Plan options (nrs_plan_create_ex). f64_mode NRS_PLAN_F64_DMMA (0): f64
 * GEMMs run as FP64 DMMA tiles of the persistent kernel (nrs_plan_create's
 * behaviour). NRS_PLAN_F64_OZAKI (1): row-major f64 GEMMs run first as one
 * grouped Ozaki launch on the tensor cores (nrs_gemm_ozaki's scheme, one
 * slice count for the group); f64_slices 0 = measured from each problem's
 * spread when the plan is created (the largest count; problems whose spread
 * no count covers, or with Inf / NaN, stay on DMMA tiles), 1..16 = given;
 * f64_digit_bits 0 = the widest digits the group's K allows, or 6..8. The
 * slice count is fixed when the plan is created: replaying it on data whose
 * magnitudes are spread wider than at creation loses accuracy -- create the
 * plan again (or give a count) when the data's range changes.
 * f32_mode NRS_PLAN_F32_FMA (0): f32 GEMMs run as FP32 FMA tiles of the
 * persistent kernel. NRS_PLAN_F32_OZAKI (1): row-major f32 GEMMs run as a
 * second grouped launch of the same scheme, each operand carried to
 * 26 + log2(max R) bits (f32's 24 and two guard bits; the slice count is
 * measured when the plan is created), the exact sums rounded once to f32:
 * max_ij |C - AB|_ij / (|A||B|)_ij stays near 2^-24 for any K, where the
 * FMA tiles' sequential f32 sum grows with K. */
typedef enum nrs_plan_f64_mode { NRS_PLAN_F64_DMMA = 0, NRS_PLAN_F64_OZAKI = 1 } nrs_plan_f64_mode;
typedef enum nrs_plan_f32_mode { NRS_PLAN_F32_FMA = 0, NRS_PLAN_F32_OZAKI = 1 } nrs_plan_f32_mode;
typedef struct nrs_plan_options {
  int32_t f64_mode;
  int32_t f64_slices;
  int32_t f64_digit_bits;
  int32_t f32_mode;
} nrs_plan_options;

/* Builds the tile/work queue for `n_gemm` GEMMs and `n_red` row reductions
 * (tile shapes from the autotuner's table, see nrs_tune_gemm) and uploads
 * it. Descriptors are copied; the data pointers must stay valid while the
 * plan is used. */
int nrs_plan_create(nrs_handle* h, int64_t n_gemm, const nrs_gemm_desc* gemms, int64_t n_red,
                    const nrs_rowreduce_desc* reds, nrs_plan** out);
int nrs_plan_create_ex(nrs_handle* h, int64_t n_gemm, const nrs_gemm_desc* gemms, int64_t n_red,
                       const nrs_rowreduce_desc* reds, const nrs_plan_options* options, nrs_plan** out);
/* f64 GEMMs the plan runs on the tensor cores, with their slice count and
 * digit width (0, 0, 0 for a DMMA-only plan). */
int nrs_plan_f64_info(nrs_plan* plan, int64_t* on_tensor_cores, int* slices, int* digit_bits);
/* The same for the plan's f32 GEMMs (NRS_PLAN_F32_OZAKI). */
int nrs_plan_f32_info(nrs_plan* plan, int64_t* on_tensor_cores, int* slices, int* digit_bits);
/* Runs the whole group as ONE persistent kernel launch (preceded, with
 * NRS_PLAN_F64_OZAKI / NRS_PLAN_F32_OZAKI, by the grouped tensor-core
 * launches of its f64 / f32 GEMMs).
 * With use_graph != 0
 * the launch is captured once into a CUDA graph owned by the plan and
 * replayed on later calls. */
int nrs_plan_run(nrs_handle* h, nrs_plan* plan, int use_graph);
/* Number of work items and tiles in the plan. */
int nrs_plan_stats(nrs_plan* plan, int64_t* work_items, int64_t* gemm_tiles);
int nrs_plan_destroy(nrs_plan* plan);

/* ---------------------------------------------------------------------- */
/* Autotuner and learned selector (no reference counterpart)               */
/* ---------------------------------------------------------------------- */
#define NRS_TILE_VARIANTS 6 /* tile configurations known to the grouped kernel */

/* Describes grouped-kernel tile variant v: tile rows/cols, dtype support. */
int nrs_tile_variant_info(int v, int* tile_m, int* tile_n, int* split_k, int* dtype_mask);

/* Exhaustive autotuning of one (dtype, m, k, n, flags) shape: every tile
 * variant of that dtype is timed as a grouped launch of `batch` copies of
 * the problem (library-owned random operands, CUDA events on the handle's
 * stream, one warm-up then `reps` launches). Writes microseconds per problem
 * to times_us[NRS_TILE_VARIANTS] (-1 where a variant does not apply) and the
 * fastest variant to *best. flags: NRS_GEMM_TRANS_A / NRS_GEMM_TRANS_B. */
int nrs_tune_gemm(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n, unsigned flags,
                  int64_t batch, int reps, float* times_us, int* best);
/* Plan-level autotuning of a group (the problems nrs_plan_create would get):
 * candidates are judged by timing the WHOLE group as one grouped launch, not
 * one shape alone. Times (median of `reps` launches after a warm-up) the
 * untuned plan; with `options` f64_mode OZAKI, the f64 GEMMs on the tensor
 * cores at each digit width (the slice count follows from the width at the
 * same accuracy); with `options` f32_mode OZAKI, the f32 GEMMs on the tensor
 * cores on top of the best of those; then every remaining shape bucket
 * tuned in isolation
 * (nrs_tune_gemm); and then, from the fastest so far, tries every other
 * variant of the buckets with the most estimated work, keeping a change only
 * if the group gets faster, until `max_trials` group timings. The tile
 * choices go into the handle's tuner table (a later nrs_plan_create uses
 * them) and the chosen f64 mode into report->options (pass it to
 * nrs_plan_create_ex); the result is never slower than the untuned plan as
 * measured. The group is run many times on the caller's buffers: C's
 * contents are undefined afterwards (accumulating GEMMs are timed as
 * overwriting ones). */
typedef struct nrs_autotune_report {
  double untuned_ms;   /* selector / size heuristic, f64 on DMMA tiles       */
  double isolated_ms;  /* every bucket tuned alone                           */
  double final_ms;     /* the choice written to the table / options          */
  double ozaki_ms;     /* best tensor-core f64 mode tried (-1 if none)       */
  int32_t buckets;     /* shape buckets tuned                                */
  int32_t trials;      /* whole-group timings in the refinement pass         */
  nrs_plan_options options; /* the f64 / f32 modes and digit width chosen     */
  double ozaki_f32_ms; /* with the f32 GEMMs on the tensor cores (-1: not tried) */
} nrs_autotune_report;
int nrs_plan_autotune(nrs_handle* h, int64_t n_gemm, const nrs_gemm_desc* gemms, int64_t n_red,
                      const nrs_rowreduce_desc* reds, const nrs_plan_options* options, int max_trials,
                      int reps, nrs_autotune_report* report);
/* Records the tuned variant for a shape bucket, used by nrs_plan_create. */
int nrs_tuner_set(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n, int variant);
/* Looks a shape bucket up; -1 if untuned. */
int nrs_tuner_get(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n);
/* Clears the table. */
int nrs_tuner_clear(nrs_handle* h);
/* Saves / loads the table as a text file keyed by the GPU model, the driver
 * version and the library build (a hash of its sources). Loading a file made
 * for another GPU, driver or build returns NRS_ERR_UNSUPPORTED and changes
 * nothing; loaded entries replace the table's entries for the same buckets. */
int nrs_tuner_save(nrs_handle* h, const char* path);
int nrs_tuner_load(nrs_handle* h, const char* path);

/* MLP cost model: features[F] -> 2 x hidden ReLU layers -> one predicted
 * log-time per tile variant. Weights are kept in fp32 (master) and BF16
 * (the copy every forward pass reads); accumulation is fp32. */
typedef struct nrs_selector nrs_selector;
int nrs_selector_create(nrs_handle* h, int n_features, int hidden, int n_out, uint64_t seed,
                        nrs_selector** out);
int nrs_selector_destroy(nrs_selector* s);
/* Parameter count and host copies of the fp32 master weights, layer order
 * W1[H,F], b1[H], W2[H,H], b2[H], W3[V,H], b3[V]. */
int64_t nrs_selector_num_params(nrs_selector* s);
int nrs_selector_get_params(nrs_handle* h, nrs_selector* s, float* host_params);
int nrs_selector_set_params(nrs_handle* h, nrs_selector* s, const float* host_params);
/* One forward + backward pass on device buffers: x[B,F], target[B,V],
 * mask[B,V] (1 where the target is known). Writes y[B,V], the gradient of
 * the masked mean-squared loss in host layout order to grads (device, one
 * float per parameter) and the loss to *loss (host). */
int nrs_selector_forward_backward(nrs_handle* h, nrs_selector* s, int64_t batch, const float* x,
                                  const float* target, const float* mask, float* y, float* grads,
                                  float* loss);
/* Trains with Adam for `epochs` passes over n samples in minibatches of
 * `batch` (device buffers), entirely on the GPU. Writes the final epoch's
 * mean loss to *loss. */
int nrs_selector_train(nrs_handle* h, nrs_selector* s, int64_t n, const float* x,
                       const float* target, const float* mask, int epochs, int64_t batch,
                       float lr, uint64_t seed, float* loss);
/* Saves / loads the fp32 master weights with the same key as the tuner
 * table (refused for another GPU, driver or build; NRS_ERR_SHAPE for another
 * network shape). */
int nrs_selector_save(nrs_handle* h, nrs_selector* s, const char* path);
int nrs_selector_load(nrs_handle* h, nrs_selector* s, const char* path);
/* Predicted per-variant outputs y[n, V] for x[n, F] (device buffers). */
int nrs_selector_predict(nrs_handle* h, nrs_selector* s, int64_t n, const float* x, float* y);
/* Installs `s` (F = 7 features, V = NRS_TILE_VARIANTS outputs) as the choice
 * for GEMM shapes the tuner table lacks when a plan is created; NULL removes
 * it. Features: log2(m)/14, log2(n)/14, log2(k)/14, dtype (1 = f64),
 * trans_a, trans_b, log2(number of GEMMs in the plan)/14. The handle does not
 * own `s`: remove it before nrs_selector_destroy. */
int nrs_tuner_set_selector(nrs_handle* h, nrs_selector* s);

#ifdef __cplusplus
}
#endif
#endif /* NUMRS_GPU_H */
