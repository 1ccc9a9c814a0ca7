// Plain GEMM: C := A*B (or C += A*B), the GPU form of kernels::gemm::gemm_2d
// (src/kernels/gemm.rs:246).
//
//  * dmma_gemm   : f64 on the FP64 tensor path, mma.sync.m8n8k4.f64 fragments
//                  from shared-memory tiles (GB300's FP64 rate is the bound).
//  * simt_gemm   : f32 / f64 register-tiled CUDA-core GEMM.
//  * generic_gemm: one thread per C element, any dtype (integers wrap like
//                  gemm_generic, src/kernels/gemm.rs:408).
//
// Operands are addressed with (row, col) element strides, so transposed views
// need no copy (the reference copies them in kernels::borrow::operand).
// Overwrite contract: C is written, never read, unless ACCUMULATE is set, in
// which case C += (A*B) with the product rounded first (matmul_to computes a
// temporary and adds it, src/array/operations_optimized.rs:385).
#include <cmath>
#include <type_traits>

#include "gemm_tiles.cuh"

using namespace nrs_tiles;

namespace {

// blockIdx.z takes k-values [z*kc, min(k, (z+1)*kc)). With one chunk the
// tile goes to C; with several, chunk z writes its product to the partial
// slab P + z*m*n (row pitch n) and splitk_finish adds the slabs.
template <int BM, int BN, int WM, int WN>
__global__ void __launch_bounds__(WM * WN * 32)
    dmma_gemm(int64_t m, int64_t n, int64_t k, int64_t kc, const double* __restrict__ A, int64_t rsa,
              int64_t csa, const double* __restrict__ B, int64_t rsb, int64_t csb,
              double* __restrict__ C, int64_t ldc, int accumulate, double* __restrict__ P) {
  using Tile = Dmma<BM, BN, WM, WN>;
  __shared__ __align__(16) uint8_t smem[Tile::kSmem];
  Tile t;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const int64_t k0 = (int64_t)blockIdx.z * kc, k1 = (k0 + kc < k) ? k0 + kc : k;
  t.run(A, rsa, csa, B, rsb, csb, m, n, m0, n0, k0, k1, smem);
  if (gridDim.z == 1)
    tile_store<double>(t, C, ldc, m, n, m0, n0, accumulate != 0);
  else
    tile_store<double>(t, P + (int64_t)blockIdx.z * m * n, n, m, n, m0, n0, false);
}

// C := p_0 + p_1 + ... + p_{S-1} (slab order), or C += that sum: the product
// is rounded before it meets C, as without the split.
__global__ void splitk_finish(const double* __restrict__ P, int splits, int64_t m, int64_t n,
                              double* __restrict__ C, int64_t ldc, int accumulate) {
  const int64_t mn = m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mn;
       e += (int64_t)gridDim.x * blockDim.x) {
    double v = P[e];
    for (int z = 1; z < splits; ++z) v += P[z * mn + e];
    double* c = C + (e / n) * ldc + (e % n);
    *c = accumulate ? *c + v : v;
  }
}

// DMMA tiling for an m x n x k product on `sms` SMs: 32x32 or 64x64 tiles and
// the number of k chunks (multiples of 16, at least 64 values each when split)
// that minimise the busiest SM's share of the work, ceil(ctas / sms) x the
// work of one CTA, a split charged 1% (its partial slabs and the finish).
// Measured at 256^3-2048^3: per flop the two tiles run within 4% of each
// other (32x32 ahead), and the CTAs' pipeline fill overlaps across the many
// CTAs an SM holds, so whole-wave balance is what decides.
struct DmmaPlan {
  int tile;
  int splits;
  int64_t kc;
};
DmmaPlan plan_dmma(int64_t m, int64_t n, int64_t k, int sms) {
#if defined(NRS_DMMA_TILE) && defined(NRS_DMMA_SPLITS)  // fixed plan, for measuring the model
  {
    int64_t kc = (k + NRS_DMMA_SPLITS - 1) / NRS_DMMA_SPLITS;
    kc = (kc + 15) / 16 * 16;
    return DmmaPlan{NRS_DMMA_TILE, (int)((k + kc - 1) / kc), kc};
  }
#endif
  DmmaPlan best{32, 1, k};
  double best_cost = 1e300;
  for (int tile : {32, 64}) {
    const double ntiles = (double)((m + tile - 1) / tile) * (double)((n + tile - 1) / tile);
    const double w = tile == 64 ? 4.0 : 1.0;
    for (int s = 1; s <= 16; ++s) {
      int64_t kc = (k + s - 1) / s;
      kc = (kc + 15) / 16 * 16;
      if (s > 1 && kc < 64) break;
      const int splits = (int)((k + kc - 1) / kc);
      if (splits != s) continue;
      if (splits > 1 && (double)splits * (double)m * (double)n * 8.0 > 256.0 * (1 << 20)) break;
      const double cost = std::ceil(ntiles * splits / sms) * w * ((double)kc / (double)k) * (splits > 1 ? 1.01 : 1.0);
      if (cost < best_cost - 1e-12) {
        best_cost = cost;
        best = DmmaPlan{tile, splits, kc};
      }
    }
  }
  return best;
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN), (BM * BN >= 128 * 128 ? 2 : 1))
    simt_gemm(int64_t m, int64_t n, int64_t k, const T* __restrict__ A, int64_t rsa, int64_t csa,
              const T* __restrict__ B, int64_t rsb, int64_t csb, T* __restrict__ C, int64_t ldc,
              int accumulate) {
  using Tile = Simt<T, BM, BN, BK, TM, TN>;
  __shared__ __align__(16) uint8_t smem[Tile::kSmem];
  Tile t;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  t.run(A, rsa, csa, B, rsb, csb, m, n, m0, n0, 0, k, smem);
  tile_store<T>(t, C, ldc, m, n, m0, n0, accumulate != 0);
}

// Generic GEMM: one thread per C element, k ascending, one rounding per op.
template <typename T> __device__ __forceinline__ T gmul(T a, T b) { return a * b; }
template <typename T> __device__ __forceinline__ T gadd(T a, T b) { return a + b; }
template <> __device__ __forceinline__ int64_t gmul(int64_t a, int64_t b) {
  return (int64_t)((unsigned long long)a * (unsigned long long)b);
}
template <> __device__ __forceinline__ int64_t gadd(int64_t a, int64_t b) {
  return (int64_t)((unsigned long long)a + (unsigned long long)b);
}
template <> __device__ __forceinline__ int32_t gmul(int32_t a, int32_t b) {
  return (int32_t)((unsigned)a * (unsigned)b);
}
template <> __device__ __forceinline__ int32_t gadd(int32_t a, int32_t b) {
  return (int32_t)((unsigned)a + (unsigned)b);
}
template <> __device__ __forceinline__ double gmul(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double gadd(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float gmul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ float gadd(float a, float b) { return __fadd_rn(a, b); }

template <typename T>
__global__ void generic_gemm(int64_t m, int64_t n, int64_t k, const T* __restrict__ A, int64_t rsa,
                             int64_t csa, const T* __restrict__ B, int64_t rsb, int64_t csb,
                             T* __restrict__ C, int64_t ldc, int accumulate) {
  const int64_t total = m * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / n, j = idx % n;
    T acc = T(0);
    for (int64_t p = 0; p < k; ++p) acc = gadd(acc, gmul(A[i * rsa + p * csa], B[p * rsb + j * csb]));
    T* c = C + i * ldc + j;
    *c = accumulate ? gadd(*c, acc) : acc;
  }
}

template <typename T>
__global__ void zero_fill_2d(T* C, int64_t m, int64_t n, int64_t ldc) {
  const int64_t total = m * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x)
    C[(idx / n) * ldc + idx % n] = T(0);
}

dim3 tiles(int64_t m, int64_t n, int bm, int bn) {
  return dim3((unsigned)((n + bn - 1) / bn), (unsigned)((m + bm - 1) / bm));
}

}  // namespace

// Launches one plain GEMM. Sizes are validated by the caller.
int nrs_plain_gemm_launch(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n,
                          const void* A, int64_t rsa, int64_t csa, const void* B, int64_t rsb,
                          int64_t csb, void* C, int64_t ldc, bool accumulate, int variant) {
  const int acc = accumulate ? 1 : 0;
  cudaStream_t s = h->stream;
  if ((n + 31) / 32 > 0x7fffffffLL || (m + 31) / 32 > 65535) variant = NRS_GEMM_GENERIC;
  if (variant == NRS_GEMM_AUTO) {
    if (dtype == NRS_F64) variant = NRS_GEMM_DMMA;
    else if (dtype == NRS_F32) variant = (m * n >= 256LL * 256 * 16) ? NRS_GEMM_SIMT : NRS_GEMM_SIMT_SMALL;
    else variant = NRS_GEMM_GENERIC;
  }
  if (variant == NRS_GEMM_DMMA && dtype == NRS_F64) {
    // The k split decides the rounding: plan for a fixed SM count.
    const DmmaPlan pl = plan_dmma(m, n, k, NRS_PLAN_SMS);
    double* P = nullptr;
    if (pl.splits > 1) {
      int st;
      P = (double*)nrs_workspace(h, (size_t)pl.splits * (size_t)(m * n) * sizeof(double), &st);
      if (!P) return st;
    }
    dim3 g = tiles(m, n, pl.tile, pl.tile);
    g.z = (unsigned)pl.splits;
    if (pl.tile == 64)
      dmma_gemm<64, 64, 2, 4><<<g, 256, 0, s>>>(m, n, k, pl.kc, (const double*)A, rsa, csa, (const double*)B,
                                                rsb, csb, (double*)C, ldc, acc, P);
    else
      dmma_gemm<32, 32, 2, 2><<<g, 128, 0, s>>>(m, n, k, pl.kc, (const double*)A, rsa, csa, (const double*)B,
                                                rsb, csb, (double*)C, ldc, acc, P);
    if (pl.splits > 1) {
      const int64_t blocks = (m * n + 255) / 256;
      const int grid = (int)(blocks < (int64_t)h->num_sms * 8 ? blocks : (int64_t)h->num_sms * 8);
      splitk_finish<<<grid, 256, 0, s>>>(P, pl.splits, m, n, (double*)C, ldc, acc);
    }
    return nrs_after_launch(h, "dmma_gemm");
  }
  if (variant == NRS_GEMM_SIMT && dtype == NRS_F32) {
    simt_gemm<float, 128, 128, 8, 8, 8><<<tiles(m, n, 128, 128), 256, 0, s>>>(
        m, n, k, (const float*)A, rsa, csa, (const float*)B, rsb, csb, (float*)C, ldc, acc);
    return nrs_after_launch(h, "simt_gemm<f32,128>");
  }
  if (variant == NRS_GEMM_SIMT_SMALL && dtype == NRS_F32) {
    simt_gemm<float, 32, 32, 16, 2, 2><<<tiles(m, n, 32, 32), 256, 0, s>>>(
        m, n, k, (const float*)A, rsa, csa, (const float*)B, rsb, csb, (float*)C, ldc, acc);
    return nrs_after_launch(h, "simt_gemm<f32,32>");
  }
  if (variant == NRS_GEMM_SIMT && dtype == NRS_F64) {
    simt_gemm<double, 64, 64, 8, 4, 4><<<tiles(m, n, 64, 64), 256, 0, s>>>(
        m, n, k, (const double*)A, rsa, csa, (const double*)B, rsb, csb, (double*)C, ldc, acc);
    return nrs_after_launch(h, "simt_gemm<f64,64>");
  }
  if (variant != NRS_GEMM_GENERIC && variant != NRS_GEMM_DMMA && variant != NRS_GEMM_SIMT &&
      variant != NRS_GEMM_SIMT_SMALL)
    return nrs_fail(h, NRS_ERR_INVALID, "unknown GEMM variant");
  if (variant != NRS_GEMM_GENERIC)
    return nrs_fail(h, NRS_ERR_DTYPE, "variant not available for this dtype");
  int64_t blocks = (m * n + 255) / 256;
  int grid = (int)(blocks < (int64_t)h->num_sms * 16 ? blocks : (int64_t)h->num_sms * 16);
  switch (dtype) {
    case NRS_F32:
      generic_gemm<float><<<grid, 256, 0, s>>>(m, n, k, (const float*)A, rsa, csa, (const float*)B, rsb, csb, (float*)C, ldc, acc);
      break;
    case NRS_F64:
      generic_gemm<double><<<grid, 256, 0, s>>>(m, n, k, (const double*)A, rsa, csa, (const double*)B, rsb, csb, (double*)C, ldc, acc);
      break;
    case NRS_I64:
      generic_gemm<int64_t><<<grid, 256, 0, s>>>(m, n, k, (const int64_t*)A, rsa, csa, (const int64_t*)B, rsb, csb, (int64_t*)C, ldc, acc);
      break;
    default:
      generic_gemm<int32_t><<<grid, 256, 0, s>>>(m, n, k, (const int32_t*)A, rsa, csa, (const int32_t*)B, rsb, csb, (int32_t*)C, ldc, acc);
      break;
  }
  return nrs_after_launch(h, "generic_gemm");
}

extern "C" int nrs_gemm(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n, const void* A,
                        int64_t lda, const void* B, int64_t ldb, void* C, int64_t ldc,
                        unsigned flags, int variant) {
  if (!h) return NRS_ERR_INVALID;
  h->last_error.clear();
  if (m < 0 || k < 0 || n < 0) return nrs_fail(h, NRS_ERR_SHAPE, "negative GEMM dimension");
  if (!nrs_dtype_size(dtype)) return nrs_fail(h, NRS_ERR_DTYPE, "unknown dtype");
  if (flags & ~(NRS_GEMM_ACCUMULATE | NRS_GEMM_TRANS_A | NRS_GEMM_TRANS_B))
    return nrs_fail(h, NRS_ERR_INVALID, "unknown GEMM flag");
  if (variant < NRS_GEMM_AUTO || variant > NRS_GEMM_SIMT_SMALL)
    return nrs_fail(h, NRS_ERR_INVALID, "unknown GEMM variant");
  const bool ta = flags & NRS_GEMM_TRANS_A, tb = flags & NRS_GEMM_TRANS_B;
  // Leading-dimension checks (the reference checks slice lengths, :250).
  if (ldc < (n > 0 ? n : 1)) return nrs_fail(h, NRS_ERR_SHAPE, "ldc < n");
  if (lda < ((ta ? m : k) > 0 ? (ta ? m : k) : 1)) return nrs_fail(h, NRS_ERR_SHAPE, "lda too small");
  if (ldb < ((tb ? k : n) > 0 ? (tb ? k : n) : 1)) return nrs_fail(h, NRS_ERR_SHAPE, "ldb too small");
  if (m == 0 || n == 0) return NRS_OK;  // nothing to overwrite
  if (!C) return nrs_fail(h, NRS_ERR_INVALID, "null C");
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  const bool accumulate = flags & NRS_GEMM_ACCUMULATE;
  if (k == 0) {
    if (accumulate) return NRS_OK;  // C += 0
    int grid = h->num_sms * 4;
    switch (dtype) {
      case NRS_F32: zero_fill_2d<float><<<grid, 256, 0, h->stream>>>((float*)C, m, n, ldc); break;
      case NRS_F64: zero_fill_2d<double><<<grid, 256, 0, h->stream>>>((double*)C, m, n, ldc); break;
      case NRS_I64: zero_fill_2d<int64_t><<<grid, 256, 0, h->stream>>>((int64_t*)C, m, n, ldc); break;
      default: zero_fill_2d<int32_t><<<grid, 256, 0, h->stream>>>((int32_t*)C, m, n, ldc); break;
    }
    return nrs_after_launch(h, "zero_fill_2d");
  }
  if (!A || !B) return nrs_fail(h, NRS_ERR_INVALID, "null A or B");
  const int64_t rsa = ta ? 1 : lda, csa = ta ? lda : 1;
  const int64_t rsb = tb ? 1 : ldb, csb = tb ? ldb : 1;
  return nrs_plain_gemm_launch(h, dtype, m, k, n, A, rsa, csa, B, rsb, csb, C, ldc, accumulate,
                               variant);
}

// ---------------------------------------------------------------------------
// Pipe-rate probes: the denominators for the GEMM rooflines on this device.
// ---------------------------------------------------------------------------
namespace {

// Every warp issues `iters` rounds of 8 independent m8n8k4 DMMA chains
// (8 x 512 flops per round) from registers; the operands change with the
// thread so nothing folds at compile time, and the result is stored only if
// it is NaN (never) so the chains stay live.
__global__ void __launch_bounds__(256) dmma_rate(int64_t iters, double seed, double* sink) {
  double a = seed + threadIdx.x * 1e-3, b = 1.0 - a * 1e-3;
  double d[8][2];
#pragma unroll
  for (int c = 0; c < 8; ++c) d[c][0] = d[c][1] = 0.0;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) dmma_m8n8k4(d[c][0], d[c][1], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += d[c][0] + d[c][1];
  if (s != s) sink[threadIdx.x] = s;
}

// FP32 FMA rate: 8 independent FMA chains per thread.
__global__ void __launch_bounds__(256) ffma_rate(int64_t iters, float seed, float* sink) {
  float x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = seed + (float)(threadIdx.x + c) * 1e-3f;
  const float a = 0.999f, b = 1e-4f;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fmaf(x[c], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  if (s != s) sink[threadIdx.x] = s;
}

}  // namespace

extern "C" int nrs_probe_peak(nrs_handle* h, int kind, double* tflops) {
  if (!h || !tflops) return NRS_ERR_INVALID;
  if (kind != NRS_PEAK_FP64_DMMA && kind != NRS_PEAK_FP32_FMA)
    return nrs_fail(h, NRS_ERR_INVALID, "unknown probe kind");
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  void* sink = nrs_workspace(h, 4096, &st);
  if (!sink) return st;
  // 32 warps per SM; long enough (tens of ms) that launch overhead is noise.
  const int blocks = h->num_sms * 4;
  const int64_t iters = kind == NRS_PEAK_FP64_DMMA ? 4096 : (1 << 20);
  cudaEvent_t e0, e1;
  if ((st = nrs_cuda_check(h, cudaEventCreate(&e0), "cudaEventCreate"))) return st;
  if ((st = nrs_cuda_check(h, cudaEventCreate(&e1), "cudaEventCreate"))) {
    cudaEventDestroy(e0);
    return st;
  }
  float best_ms = 1e30f;
  for (int rep = 0; rep < 4 && st == NRS_OK; ++rep) {  // first launch is a warm-up
    cudaEventRecord(e0, h->stream);
    if (kind == NRS_PEAK_FP64_DMMA)
      dmma_rate<<<blocks, 256, 0, h->stream>>>(iters, 0.5, (double*)sink);
    else
      ffma_rate<<<blocks, 256, 0, h->stream>>>(iters, 0.5f, (float*)sink);
    cudaEventRecord(e1, h->stream);
    st = nrs_cuda_check(h, cudaEventSynchronize(e1), "probe");
    float ms = 0.0f;
    if (st == NRS_OK) st = nrs_cuda_check(h, cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    if (st == NRS_OK && rep > 0 && ms < best_ms) best_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  const double warps = (double)blocks * 8.0;
  const double flops = kind == NRS_PEAK_FP64_DMMA ? warps * (double)iters * 8.0 * 512.0
                                                  : warps * 32.0 * (double)iters * 8.0 * 2.0;
  *tflops = flops / (best_ms * 1e-3) / 1e12;
  return NRS_OK;
}
