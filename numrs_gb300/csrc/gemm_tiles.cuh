// Block-level GEMM tile bodies shared by the standalone GEMM kernels
// (gemm.cu) and the persistent grouped kernel (grouped.cu), so both produce
// bit-identical results for the same tile shape.
//
// A tile computes acc = A[m0:m0+BM, k0:k1] * B[k0:k1, n0:n0+BN] with
// (row, col) element strides, into registers; `tile_store` writes (or adds)
// it to C. Shared memory comes from the caller (a raw byte buffer).
#pragma once

#include "nrs_internal.cuh"

namespace nrs_tiles {

__device__ __forceinline__ void dmma_m8n8k4(double& d0, double& d1, double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
      : "+d"(d0), "+d"(d1)
      : "d"(a), "d"(b));
}

// ---------------------------------------------------------------------------
// FP64 DMMA tile: warp grid WM x WN, warp tile (BM/WM) x (BN/WN) built from
// m8n8k4 fragments; k-major shared tiles with a pitch of BM+8 / BN+8 doubles
// so a fragment load touches each bank pair at most twice (256 B minimum).
// ---------------------------------------------------------------------------
template <int BM, int BN, int WM, int WN>
struct Dmma {
  static constexpr int BK = 16;
  static constexpr int NT = WM * WN * 32;
  static constexpr int TM = BM / WM, TN = BN / WN;
  static constexpr int FM = TM / 8, FN = TN / 8;
  static constexpr int PA = BM + 8, PB = BN + 8;
  static constexpr int LA = BM * BK / NT, LB = BN * BK / NT;
  static constexpr int kSmem = 2 * BK * (PA + PB) * 8;
  double acc[FM][FN][2];

  __device__ __forceinline__ void run(const double* __restrict__ A, int64_t rsa, int64_t csa,
                                      const double* __restrict__ B, int64_t rsb, int64_t csb,
                                      int64_t m, int64_t n, int64_t m0, int64_t n0, int64_t k0,
                                      int64_t k1, uint8_t* smem) {
    double(*As)[BK][PA] = reinterpret_cast<double(*)[BK][PA]>(smem);
    double(*Bs)[BK][PB] = reinterpret_cast<double(*)[BK][PB]>(smem + 2 * BK * PA * 8);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp / WN, wn = warp % WN;
    const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int i = 0; i < FM; ++i)
#pragma unroll
      for (int j = 0; j < FN; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
    double ra[LA], rb[LB];
    auto load = [&](int64_t kt) {
#pragma unroll
      for (int i = 0; i < LA; ++i) {
        int e = tid + i * NT;
        int r = e / BK, kk = e % BK;
        int64_t gi = m0 + r, gk = kt + kk;
        ra[i] = (gi < m && gk < k1) ? A[gi * rsa + gk * csa] : 0.0;
      }
#pragma unroll
      for (int i = 0; i < LB; ++i) {
        int e = tid + i * NT;
        int kk = e / BN, c = e % BN;
        int64_t gk = kt + kk, gj = n0 + c;
        rb[i] = (gk < k1 && gj < n) ? B[gk * rsb + gj * csb] : 0.0;
      }
    };
    auto store = [&](int buf) {
#pragma unroll
      for (int i = 0; i < LA; ++i) {
        int e = tid + i * NT;
        As[buf][e % BK][e / BK] = ra[i];
      }
#pragma unroll
      for (int i = 0; i < LB; ++i) {
        int e = tid + i * NT;
        Bs[buf][e / BN][e % BN] = rb[i];
      }
    };
    const int64_t ktiles = (k1 - k0 + BK - 1) / BK;
    if (ktiles > 0) {
      load(k0);
      store(0);
    }
    __syncthreads();
    for (int64_t kt = 0; kt < ktiles; ++kt) {
      const int buf = (int)(kt & 1);
      if (kt + 1 < ktiles) load(k0 + (kt + 1) * BK);
#pragma unroll
      for (int ks = 0; ks < BK; ks += 4) {
        double af[FM], bf[FN];
#pragma unroll
        for (int i = 0; i < FM; ++i) af[i] = As[buf][ks + t4][wm * TM + i * 8 + g];
#pragma unroll
        for (int j = 0; j < FN; ++j) bf[j] = Bs[buf][ks + t4][wn * TN + j * 8 + g];
#pragma unroll
        for (int i = 0; i < FM; ++i)
#pragma unroll
          for (int j = 0; j < FN; ++j) dmma_m8n8k4(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
      }
      if (kt + 1 < ktiles) store(buf ^ 1);
      __syncthreads();
    }
  }

  // Element (r, c) of the tile held by this thread, e = 0 .. FM*FN*2-1.
  __device__ __forceinline__ void coords(int e, int& r, int& c) const {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wm = warp / WN, wn = warp % WN;
    const int i = e / (FN * 2), j = (e / 2) % FN, h = e & 1;
    r = wm * TM + i * 8 + (lane >> 2);
    c = wn * TN + j * 8 + 2 * (lane & 3) + h;
  }
  __device__ __forceinline__ double value(int e) const {
    const int i = e / (FN * 2), j = (e / 2) % FN, h = e & 1;
    return acc[i][j][h];
  }
  static constexpr int kPerThread = FM * FN * 2;
};

// ---------------------------------------------------------------------------
// SIMT register tile (f32 / f64). f32 tiles with TM, TN multiples of 4: thread
// (tr, tc) owns TM/4 groups of 4 consecutive rows, group g at
// g*(BM/(TM/4)) + 4*tr (columns likewise), so each k step reads its A and B
// fragments as 16-byte shared loads (TM/4 + TN/4 of them per TM*TN FMAs).
// Otherwise thread (tr, tc) owns rows tr + i*(BM/TM), cols tc + j*(BN/TN).
// Either way every C element is the same k-ordered FMA chain, so the mapping
// does not change a bit of the result.
// ---------------------------------------------------------------------------
template <typename T, int BM, int BN, int BK, int TM, int TN>
struct Simt {
  static constexpr int NT = (BM / TM) * (BN / TN);
  static constexpr int LA = BM * BK / NT, LB = BN * BK / NT;
  static constexpr int kSmem = 2 * BK * ((BM + 4) + (BN + 4)) * (int)sizeof(T);
  static constexpr bool kVec = sizeof(T) == 4 && TM % 4 == 0 && TN % 4 == 0;
  T acc[TM][TN];
  // Row (column) of fragment element i (j) for thread row tr (column tc).
  static __device__ __forceinline__ int row_of(int tr, int i) {
    return kVec ? (i / 4) * (BM / (TM / 4)) + 4 * tr + (i % 4) : tr + i * (BM / TM);
  }
  static __device__ __forceinline__ int col_of(int tc, int j) {
    return kVec ? (j / 4) * (BN / (TN / 4)) + 4 * tc + (j % 4) : tc + j * (BN / TN);
  }

  __device__ __forceinline__ void run(const T* __restrict__ A, int64_t rsa, int64_t csa,
                                      const T* __restrict__ B, int64_t rsb, int64_t csb,
                                      int64_t m, int64_t n, int64_t m0, int64_t n0, int64_t k0,
                                      int64_t k1, uint8_t* smem) {
    T(*As)[BK][BM + 4] = reinterpret_cast<T(*)[BK][BM + 4]>(smem);
    T(*Bs)[BK][BN + 4] = reinterpret_cast<T(*)[BK][BN + 4]>(smem + 2 * BK * (BM + 4) * sizeof(T));
    const int tid = threadIdx.x;
    const int tr = tid / (BN / TN), tc = tid % (BN / TN);
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
    T ra[LA], rb[LB];
    auto load = [&](int64_t kt) {
#pragma unroll
      for (int i = 0; i < LA; ++i) {
        int e = tid + i * NT;
        int r = e / BK, kk = e % BK;
        int64_t gi = m0 + r, gk = kt + kk;
        ra[i] = (gi < m && gk < k1) ? A[gi * rsa + gk * csa] : T(0);
      }
#pragma unroll
      for (int i = 0; i < LB; ++i) {
        int e = tid + i * NT;
        int kk = e / BN, c = e % BN;
        int64_t gk = kt + kk, gj = n0 + c;
        rb[i] = (gk < k1 && gj < n) ? B[gk * rsb + gj * csb] : T(0);
      }
    };
    auto store = [&](int buf) {
#pragma unroll
      for (int i = 0; i < LA; ++i) {
        int e = tid + i * NT;
        As[buf][e % BK][e / BK] = ra[i];
      }
#pragma unroll
      for (int i = 0; i < LB; ++i) {
        int e = tid + i * NT;
        Bs[buf][e / BN][e % BN] = rb[i];
      }
    };
    const int64_t ktiles = (k1 - k0 + BK - 1) / BK;
    if (ktiles > 0) {
      load(k0);
      store(0);
    }
    __syncthreads();
    for (int64_t kt = 0; kt < ktiles; ++kt) {
      const int buf = (int)(kt & 1);
      if (kt + 1 < ktiles) load(k0 + (kt + 1) * BK);
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T a[TM], b[TN];
        if constexpr (kVec) {
#pragma unroll
          for (int g = 0; g < TM / 4; ++g) {
            const float4 v = *reinterpret_cast<const float4*>(&As[buf][kk][row_of(tr, 4 * g)]);
            a[4 * g] = v.x, a[4 * g + 1] = v.y, a[4 * g + 2] = v.z, a[4 * g + 3] = v.w;
          }
#pragma unroll
          for (int g = 0; g < TN / 4; ++g) {
            const float4 v = *reinterpret_cast<const float4*>(&Bs[buf][kk][col_of(tc, 4 * g)]);
            b[4 * g] = v.x, b[4 * g + 1] = v.y, b[4 * g + 2] = v.z, b[4 * g + 3] = v.w;
          }
        } else {
#pragma unroll
          for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][row_of(tr, i)];
#pragma unroll
          for (int j = 0; j < TN; ++j) b[j] = Bs[buf][kk][col_of(tc, j)];
        }
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      if (kt + 1 < ktiles) store(buf ^ 1);
      __syncthreads();
    }
  }
  __device__ __forceinline__ void coords(int e, int& r, int& c) const {
    const int tid = threadIdx.x;
    const int tr = tid / (BN / TN), tc = tid % (BN / TN);
    r = row_of(tr, e / TN);
    c = col_of(tc, e % TN);
  }
  __device__ __forceinline__ T value(int e) const { return acc[e / TN][e % TN]; }
  static constexpr int kPerThread = TM * TN;
};

// Writes (or, with accumulate, adds -- product rounded first) the tile to C.
template <typename T, typename Tile>
__device__ __forceinline__ void tile_store(const Tile& t, T* __restrict__ C, int64_t ldc, int64_t m,
                                           int64_t n, int64_t m0, int64_t n0, bool accumulate) {
#pragma unroll
  for (int e = 0; e < Tile::kPerThread; ++e) {
    int r, c;
    t.coords(e, r, c);
    const int64_t gi = m0 + r, gj = n0 + c;
    if (gi < m && gj < n) {
      T* p = C + gi * ldc + gj;
      const T v = (T)t.value(e);
      *p = accumulate ? (*p + v) : v;
    }
  }
}

}  // namespace nrs_tiles
