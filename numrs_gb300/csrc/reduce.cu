// Axis folds and flat reductions.
//
// Axis folds (math::sum/mean/max/min(axis), Array::sum_axis) fold every
// output lane sequentially, left to right, exactly as the reference's lane
// loops do (src/math/aggregation.rs:555-561, src/math/statistics/mod.rs:1066,
// src/math/aggregation.rs:250-263, src/array/operations.rs:137-153), so float
// results carry the reference's rounding bit for bit. Sequential lanes give
// far fewer independent loads than a tree, so the HBM stream is decoupled from
// the folding threads with a TMA pipeline: a CTA owns a block of lanes and
// walks the reduced axis through STAGES shared-memory tiles whose copies are
// in flight while earlier tiles are folded.
//
//  * fold_cols_tma : lanes are adjacent in memory (stride 1), the axis is
//                    strided -- e.g. axis 0 of a row-major matrix, or axis 1
//                    of its transposed view. Tile = 64 lanes x
//                    (8 KB / (64 * sizeof(T))) rows; thread t folds column t
//                    of every tile.
//  * fold_rows_tma : each lane is contiguous along the axis -- axis 1 of a
//                    row-major matrix, axis 0 of its transposed view. Tile =
//                    128 B along the axis x 64 lanes with the 128-byte
//                    swizzle, so thread t reading its own row with 16-byte
//                    loads is bank-conflict free.
//  * fold_generic  : any strides, one thread per lane (small or unaligned
//                    views).
//
// Flat reductions (kernels::reduce, src/kernels/reduce.rs:204-444) keep the
// reference's 8192-element chunking: one warp sums a chunk with a
// lane-striped tree (256 lanes, eight per thread, 16-byte loads), chunk
// partials go to workspace, and a single CTA folds them (in chunk order up to
// 1024 chunks, else as 1024 interleaved runs folded in order).
#include <cfloat>
#include <type_traits>
#include <climits>
#include <cmath>
#include <mutex>
#include <vector>

#include "reduce_common.cuh"

using namespace nrs_red;

namespace {

constexpr int kChunk = 8192;        // PARALLEL_CHUNK, src/kernels/mod.rs:92
constexpr int kParallelMin = 10000; // PARALLEL_MIN_LEN, src/kernels/mod.rs:74
constexpr int kVarParallelMin = 40000;  // VAR_PARALLEL_MIN_LEN, src/kernels/reduce.rs:202

// ---------------------------------------------------------------------------
// Generic strided fold: one thread per output lane.
// ---------------------------------------------------------------------------
struct KeptDims {
  int n;
  int64_t size[NRS_UFUNC_MAX_DIMS];
  int64_t stride[NRS_UFUNC_MAX_DIMS];
};

template <typename T, int OP>
__global__ void fold_generic(const T* __restrict__ x, KeptDims kd, int64_t n_out, int64_t alen,
                             int64_t astride, typename OutOf<T, OP>::type* __restrict__ out,
                             const T* __restrict__ lane_mean, T div) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n_out;
       o += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = o, base = 0;
    for (int d = kd.n - 1; d >= 0; --d) {
      int64_t c = rem % kd.size[d];
      rem /= kd.size[d];
      base += c * kd.stride[d];
    }
    const T* p = x + base;
    const T m = lane_mean ? lane_mean[o] : T(0);
    T acc = Fold<T, OP>::init();
    for (int64_t j = 0; j < alen; ++j) acc = Fold<T, OP>::step(acc, lane_xform<T, OP>(p[j * astride], m));
    out[o] = finish<T, OP>(acc, alen, div);
  }
}

// argmax / argmin along an axis (math::statistics::argmax/argmin,
// src/math/statistics/mod.rs:79, :218): the first element starts the lane,
// a later one replaces it only if strictly greater (smaller), so ties keep
// the first index and a NaN is never chosen unless it is element 0.
template <typename T, bool MAX>
__global__ void arg_generic(const T* __restrict__ x, KeptDims kd, int64_t n_out, int64_t alen,
                            int64_t astride, int64_t* __restrict__ out) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n_out;
       o += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = o, base = 0;
    for (int d = kd.n - 1; d >= 0; --d) {
      int64_t c = rem % kd.size[d];
      rem /= kd.size[d];
      base += c * kd.stride[d];
    }
    const T* p = x + base;
    T best = p[0];
    int64_t bi = 0;
    for (int64_t j = 1; j < alen; ++j) {
      const T v = p[j * astride];
      if (MAX ? (v > best) : (v < best)) {
        best = v;
        bi = j;
      }
    }
    out[o] = bi;
  }
}

// Flat argmax / argmin (axis = None): the reference scans left to right from
// element 0 keeping the first strictly greater (smaller) value. The same
// answer in parallel: a candidate (v, i) beats (w, j) if v is strictly
// better, or equal with i < j; NaNs never win; and if element 0 is NaN the
// answer is 0 (nothing compares greater than it). Chunk candidates go to
// workspace and one thread combines them.
template <typename T>
struct ArgCand {
  T v;  // unused when idx < 0
  int64_t idx;
};

template <typename T, bool MAX>
__device__ __forceinline__ bool arg_better(T v, int64_t i, T w, int64_t j) {
  if (v != v) return false;
  if (j < 0 || w != w) return true;
  if (MAX ? (v > w) : (v < w)) return true;
  return v == w && i < j;
}

// One warp per 8192-element chunk with eight consecutive elements per thread
// and step (the flat_partials layout below); each warp keeps the best of all
// its chunks and writes one candidate, part[global warp index] (idx -1: the
// warp had no chunk). arg_better is a strict preference, so the scan and
// combine order are free.
template <typename T, bool MAX, bool VEC>
__global__ void __launch_bounds__(256, 4)
    arg_partials(const T* __restrict__ x, int64_t n, ArgCand<T>* __restrict__ part) {
  constexpr int LPT = 8;
  constexpr int UNROLL = sizeof(T) == 8 ? 2 : 4;
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  const int t = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  T wbv = T(0);
  int64_t wgi = -1;
  for (int64_t c = wid; c < nchunks; c += nwarps) {
    const int64_t lo = c * kChunk;
    const int64_t len = (n - lo) < kChunk ? (n - lo) : kChunk;
    const T* p = x + lo + LPT * t;
    // A thread meets its elements in increasing index order and never keeps a
    // NaN, so arg_better reduces to "strictly better, or the first non-NaN":
    // ties keep the earlier index. `bi` is the offset 256k + 8t + j.
    T bv = T(0);
    int bi = -1;
    const int full = (int)(len / 256);
#pragma unroll UNROLL
    for (int k = 0; k < full; ++k) {
      T v[LPT];
      if constexpr (VEC) {
        constexpr int NV = LPT * (int)sizeof(T) / 16;
        uint4 u[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) u[q] = reinterpret_cast<const uint4*>(p + 256 * k)[q];
        memcpy(v, u, sizeof(v));
      } else {
#pragma unroll
        for (int j = 0; j < LPT; ++j) v[j] = p[256 * k + j];
      }
#pragma unroll
      for (int j = 0; j < LPT; ++j) {
        if ((MAX ? (v[j] > bv) : (v[j] < bv)) || (bi < 0 && v[j] == v[j])) {
          bv = v[j];
          bi = 256 * k + LPT * t + j;
        }
      }
    }
    const int rest = (int)(len - 256 * (int64_t)full);
#pragma unroll
    for (int j = 0; j < LPT; ++j) {
      if (LPT * t + j < rest) {
        const T v = p[256 * full + j];
        if ((MAX ? (v > bv) : (v < bv)) || (bi < 0 && v == v)) {
          bv = v;
          bi = 256 * full + LPT * t + j;
        }
      }
    }
    int64_t gi = bi < 0 ? -1 : lo + bi;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const T ov = __shfl_xor_sync(0xffffffffu, bv, off);
      const int64_t oi = __shfl_xor_sync(0xffffffffu, gi, off);
      if (oi >= 0 && arg_better<T, MAX>(ov, oi, bv, gi)) {
        bv = ov;
        gi = oi;
      }
    }
    if (gi >= 0 && arg_better<T, MAX>(bv, gi, wbv, wgi)) {
      wbv = bv;
      wgi = gi;
    }
  }
  if (t == 0) part[wid] = ArgCand<T>{wbv, wgi};
}

// Combines the chunk candidates. arg_better is a strict preference (better
// value, then smaller index; a NaN is never better), so picking the best
// candidate in any grouping gives the same answer: thread t takes candidates
// t, t+1024, ... (coalesced), then a shared-memory tree.
template <typename T, bool MAX>
__global__ void __launch_bounds__(1024)
    arg_finish(const T* __restrict__ x, const ArgCand<T>* __restrict__ part, int64_t nchunks,
               int64_t* out) {
  __shared__ T sv[1024];
  __shared__ int64_t si[1024];
  const int t = threadIdx.x;
  T bv = T(0);
  int64_t bi = -1;
#pragma unroll 4
  for (int64_t c = t; c < nchunks; c += 1024) {
    const ArgCand<T> q = part[c];
    if (q.idx >= 0 && arg_better<T, MAX>(q.v, q.idx, bv, bi)) {
      bv = q.v;
      bi = q.idx;
    }
  }
  sv[t] = bv;
  si[t] = bi;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (t < s && si[t + s] >= 0 && arg_better<T, MAX>(sv[t + s], si[t + s], sv[t], si[t])) {
      sv[t] = sv[t + s];
      si[t] = si[t + s];
    }
    __syncthreads();
  }
  if (t == 0) {
    const T x0 = x[0];
    // a NaN first element is never replaced; all-NaN tails give index 0
    out[0] = (x0 != x0 || si[0] < 0) ? 0 : si[0];
  }
}

// ---------------------------------------------------------------------------
// TMA pipelines
// ---------------------------------------------------------------------------
// Shared-memory layout: STAGES tiles (1024-byte aligned) then STAGES mbarriers.
template <int TILE_BYTES, int STAGES>
struct PipeSmem {
  static constexpr int kBytes = TILE_BYTES * STAGES + 8 * STAGES + 1024;  // + alignment slack
};

// Lanes adjacent (stride 1), axis strided. Tensor map dims (lanes, axis,
// batch), box (LW, RB, 1), no swizzle: tile row r holds lanes [l0, l0+LW) of
// axis position y0 + r. 64 lanes per CTA for every dtype, so a 16384-lane
// problem is 256 CTAs: one wave at the three 66 KB CTAs an SM holds.
constexpr int kColLanes = 64;
template <typename T>
constexpr int col_rows() { return 8192 / (kColLanes * (int)sizeof(T)); }

template <typename T, int OP, int STAGES>
__global__ void __launch_bounds__(kColLanes)
    fold_cols_tma(const __grid_constant__ CUtensorMap map, int64_t alen, int64_t lanes,
                  typename OutOf<T, OP>::type* __restrict__ out, uint32_t* err,
                  const T* __restrict__ lane_mean, T div, int64_t part_len, int64_t part_stride) {
  constexpr int LW = kColLanes;        // lanes per tile (= threads)
  constexpr int RB = col_rows<T>();    // axis positions per tile (8 KB tiles)
  constexpr int TILE = LW * RB * sizeof(T);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + TILE * STAGES);
  __shared__ int abort_flag;

  const int t = threadIdx.x;
  const int64_t l0 = (int64_t)blockIdx.x * LW;
  const int32_t batch = blockIdx.y;
  // axis part blockIdx.z: positions [a0, a0 + plen) (the whole axis unless
  // max / min split it across CTAs; part_len is a whole number of tiles)
  const int64_t a0 = (int64_t)blockIdx.z * part_len;
  const int64_t plen = (alen - a0) < part_len ? (alen - a0) : part_len;
  const int64_t n_tiles = (plen + RB - 1) / RB;
  // Wait-expiry test hook (nrs_test_expire_next_wait): err[1], when set,
  // makes the first CTA leave stage 0 unloaded, so its first wait is on a
  // barrier nothing completes, bounded to err[1] probes. Other CTAs and all
  // later launches run normally.
  __shared__ uint32_t wait_limit, skip_stage0;

  if (t == 0) {
    prefetch_tensormap(&map);
    for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
    abort_flag = 0;
    const uint32_t probes = (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) ? atomicExch(&err[1], 0u) : 0u;
    skip_stage0 = probes != 0;
    wait_limit = probes != 0 ? probes : NRS_WAIT_LIMIT;
  }
  __syncthreads();
  if (t == 0) {
    for (int s = 0; s < STAGES && s < n_tiles; ++s) {
      if (s == 0 && skip_stage0) continue;
      mbar_arrive_expect_tx(&full[s], TILE);
      tma_load_3d(smem + s * TILE, &map, &full[s], (int32_t)l0, (int32_t)(a0 + s * RB), batch);
    }
  }
  // A thread past the last lane folds lane 0's column (and discards it)
  // rather than the box's zero fill, whose zeros would send the max / min
  // chains to the ordered path on every tile and make this CTA the
  // launch's straggler (f64: 2.3x the launch time at 11586^2). f32 max /
  // min keep their own column: their ordered path is cheap, and the
  // substitution measured 14% slower for them.
  constexpr bool kSubst = !(std::is_same<T, float>::value && (OP == NRS_MAX || OP == NRS_MIN));
  const bool live = l0 + t < lanes;
  const int tl = (kSubst && !live) ? 0 : t;
  const T m = (lane_mean && l0 + tl < lanes) ? lane_mean[(int64_t)batch * lanes + l0 + tl] : T(0);
  T acc = Fold<T, OP>::init();
  int64_t it = 0;
  for (; it < n_tiles; ++it) {
    const int s = (int)(it % STAGES);
    const uint32_t phase = (uint32_t)((it / STAGES) & 1);
    if (!mbar_wait_bounded(&full[s], phase, wait_limit)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) break;
    const T* tile = reinterpret_cast<const T*>(smem + s * TILE);
    const int64_t y0 = it * RB;
    const int cnt = (int)((plen - y0) < RB ? (plen - y0) : RB);
    if (cnt == RB) {
      acc = RunFold<T, OP>::template run<RB>(
          acc, [&](int r) { return lane_xform<T, OP>(tile[r * LW + tl], m); });
    } else {
      for (int r = 0; r < cnt; ++r) acc = Fold<T, OP>::step(acc, lane_xform<T, OP>(tile[r * LW + tl], m));
    }
    __syncthreads();  // every thread is done with stage s
    if (t == 0 && it + STAGES < n_tiles) {
      mbar_arrive_expect_tx(&full[s], TILE);
      tma_load_3d(smem + s * TILE, &map, &full[s], (int32_t)l0, (int32_t)(a0 + (it + STAGES) * RB),
                  batch);
    }
  }
  if (abort_flag) {
    // Drain: wait (bounded) for every copy this CTA issued and has not
    // consumed (the stage the test hook left unloaded was never issued).
    if (t == 0) {
      atomicOr(err, NRS_DEVERR_REDUCE_TMA | (1u << 8));
      for (int64_t j = it; j < n_tiles && j < it + STAGES; ++j) {
        if (j == 0 && skip_stage0) continue;
        mbar_wait_bounded(&full[j % STAGES], (uint32_t)((j / STAGES) & 1), NRS_WAIT_LIMIT);
      }
    }
    return;
  }
  const int64_t lane = l0 + t;
  if (lane < lanes) out[blockIdx.z * part_stride + (int64_t)batch * lanes + lane] = finish<T, OP>(acc, alen, div);
}

// Lanes contiguous along the axis. Tensor map dims (axis, lanes, batch), box
// (128 B of axis, 64 lanes, 1), 128-byte swizzle: 16-byte chunk j of tile
// row r sits at r*128 + ((j ^ (r & 7)) * 16).
template <typename T, int OP, int STAGES>
__global__ void __launch_bounds__(64)
    fold_rows_tma(const __grid_constant__ CUtensorMap map, int64_t alen, int64_t lanes,
                  typename OutOf<T, OP>::type* __restrict__ out, uint32_t* err,
                  const T* __restrict__ lane_mean, T div, int64_t part_len, int64_t part_stride) {
  constexpr int LN = 64;                  // lanes per tile (= threads)
  constexpr int XB = 128 / sizeof(T);     // axis elements per tile row
  constexpr int PER16 = 16 / sizeof(T);   // elements per 16-byte chunk
  constexpr int TILE = LN * 128;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + TILE * STAGES);
  __shared__ int abort_flag;

  const int t = threadIdx.x;
  const int64_t l0 = (int64_t)blockIdx.x * LN;
  const int32_t batch = blockIdx.y;
  // axis part blockIdx.z: positions [a0, a0 + plen) (see fold_cols_tma)
  const int64_t a0 = (int64_t)blockIdx.z * part_len;
  const int64_t plen = (alen - a0) < part_len ? (alen - a0) : part_len;
  const int64_t n_tiles = (plen + XB - 1) / XB;

  if (t == 0) {
    prefetch_tensormap(&map);
    for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  if (t == 0) {
    for (int s = 0; s < STAGES && s < n_tiles; ++s) {
      mbar_arrive_expect_tx(&full[s], TILE);
      tma_load_3d(smem + s * TILE, &map, &full[s], (int32_t)(a0 + s * XB), (int32_t)l0, batch);
    }
  }
  // A thread past the last row folds row 0 of the tile (and discards it)
  // rather than the box's zero fill (see fold_cols_tma).
  const int tl = l0 + t < lanes ? t : 0;
  const T m = (lane_mean && l0 + tl < lanes) ? lane_mean[(int64_t)batch * lanes + l0 + tl] : T(0);
  T acc = Fold<T, OP>::init();
  const int sw = tl & 7;
  int64_t it = 0;
  for (; it < n_tiles; ++it) {
    const int s = (int)(it % STAGES);
    const uint32_t phase = (uint32_t)((it / STAGES) & 1);
    if (!mbar_wait_bounded(&full[s], phase, NRS_WAIT_LIMIT)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) break;
    const uint8_t* row = smem + s * TILE + tl * 128;
    const int64_t x0 = it * XB;
    const int cnt = (int)((plen - x0) < XB ? (plen - x0) : XB);
    if (cnt == XB) {
      T v[XB];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const T* c = reinterpret_cast<const T*>(row + ((j ^ sw) << 4));
        if constexpr (sizeof(T) == 4) {
          float4 q = *reinterpret_cast<const float4*>(c);
          memcpy(&v[j * PER16], &q, 16);
        } else {
          double2 q = *reinterpret_cast<const double2*>(c);
          memcpy(&v[j * PER16], &q, 16);
        }
      }
      acc = RunFold<T, OP>::template run<XB>(acc, [&](int e) { return lane_xform<T, OP>(v[e], m); });
    } else {
      for (int e = 0; e < cnt; ++e) {
        const int j = e / PER16;
        const T* c = reinterpret_cast<const T*>(row + ((j ^ sw) << 4));
        acc = Fold<T, OP>::step(acc, lane_xform<T, OP>(c[e % PER16], m));
      }
    }
    __syncthreads();
    if (t == 0 && it + STAGES < n_tiles) {
      mbar_arrive_expect_tx(&full[s], TILE);
      tma_load_3d(smem + s * TILE, &map, &full[s], (int32_t)(a0 + (it + STAGES) * XB), (int32_t)l0,
                  batch);
    }
  }
  if (abort_flag) {
    if (t == 0) {
      atomicOr(err, NRS_DEVERR_REDUCE_TMA | (2u << 8));
      for (int64_t j = it; j < n_tiles && j < it + STAGES; ++j)
        mbar_wait_bounded(&full[j % STAGES], (uint32_t)((j / STAGES) & 1), NRS_WAIT_LIMIT);
    }
    return;
  }
  const int64_t lane = l0 + t;
  if (lane < lanes) out[blockIdx.z * part_stride + (int64_t)batch * lanes + lane] = finish<T, OP>(acc, alen, div);
}

// The comparison argmax / argmin runs on: the value itself, except for f64,
// whose values map to int64 keys (integer pipe; GB300's FP64 pipe retires a
// few operations per clock per SM): the magnitude bits of negatives flipped,
// -0 folded onto +0 (equal values tie, the first index stays), a NaN element
// the key that never wins, and a lane that starts with NaN the key nothing
// beats.
template <typename T, bool MAX>
struct ArgOrd {
  using K = T;
  static __device__ __forceinline__ K key(T v) { return v; }
  static __device__ __forceinline__ K start(T v) { return v; }
  // the key an axis part after the first starts from: no element strictly
  // beats it unless it beats every non-NaN value
  static __device__ __forceinline__ K none() { return MAX ? Lim<T>::lowest() : Lim<T>::highest(); }
};
template <bool MAX>
struct ArgOrd<double, MAX> {
  using K = int64_t;
  static __device__ __forceinline__ K key(double v) {
    const uint64_t u = (uint64_t)__double_as_longlong(v);
    if (nrs_f64_is_nan(u)) return MAX ? INT64_MIN : INT64_MAX;
    if ((u << 1) == 0) return 0;
    return nrs_f64_key(u);
  }
  static __device__ __forceinline__ K start(double v) { return v != v ? (MAX ? INT64_MAX : INT64_MIN) : key(v); }
  static __device__ __forceinline__ K none() { return key(MAX ? -INFINITY : INFINITY); }
};

// argmax / argmin along lanes through the same TMA pipelines: each thread
// scans its lane in order keeping (best, index) -- the first element starts
// the lane, a later one replaces it only if strictly greater (smaller), so
// ties keep the first index and a NaN is chosen only as element 0.
template <typename T, bool MAX, bool COLS, int STAGES>
__global__ void __launch_bounds__(64)
    arg_lane_tma(const __grid_constant__ CUtensorMap map, int64_t alen, int64_t lanes,
                 int64_t* __restrict__ out, uint32_t* err, int64_t part_len,
                 typename ArgOrd<T, MAX>::K* __restrict__ part_key) {
  constexpr int TB = COLS ? col_rows<T>() : 128 / (int)sizeof(T);  // axis positions per tile
  constexpr int TILE = 8192;
  constexpr int PER16 = 16 / sizeof(T);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + TILE * STAGES);
  __shared__ int abort_flag;

  const int t = threadIdx.x;
  const int64_t l0 = (int64_t)blockIdx.x * 64;
  const int32_t batch = blockIdx.y;
  // axis part blockIdx.z: positions [a0, a0 + plen); with part_key set,
  // each part writes its best key and absolute index (-1: none) for
  // combine_arg_parts, and parts after the first start from no candidate
  // (only the lane's own first element may be a NaN winner)
  const int64_t a0 = (int64_t)blockIdx.z * part_len;
  const int64_t plen = (alen - a0) < part_len ? (alen - a0) : part_len;
  const int64_t n_tiles = (plen + TB - 1) / TB;
  auto load = [&](int s, int64_t tile) {
    mbar_arrive_expect_tx(&full[s], TILE);
    if (COLS)
      tma_load_3d(smem + s * TILE, &map, &full[s], (int32_t)l0, (int32_t)(a0 + tile * TB), batch);
    else
      tma_load_3d(smem + s * TILE, &map, &full[s], (int32_t)(a0 + tile * TB), (int32_t)l0, batch);
  };
  if (t == 0) {
    prefetch_tensormap(&map);
    for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  if (t == 0)
    for (int s = 0; s < STAGES && s < n_tiles; ++s) load(s, s);
  using Ord = ArgOrd<T, MAX>;
  typename Ord::K best = typename Ord::K(0);
  int bt = 0, be = 0;  // tile and position of the best so far (32-bit selects)
  bool found = blockIdx.z == 0;  // a later part: has any element beaten none()?
  const int sw = t & 7;
  int64_t it = 0;
  for (; it < n_tiles; ++it) {
    const int s = (int)(it % STAGES);
    if (!mbar_wait_bounded(&full[s], (uint32_t)((it / STAGES) & 1), NRS_WAIT_LIMIT)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) break;
    const int64_t j0 = it * TB;
    const int cnt = (int)((plen - j0) < TB ? (plen - j0) : TB);
    T v[TB];
    if (COLS) {
      const T* tile = reinterpret_cast<const T*>(smem + s * TILE);
#pragma unroll
      for (int r = 0; r < TB; ++r) v[r] = tile[r * 64 + t];
    } else {
      const uint8_t* row = smem + s * TILE + t * 128;
#pragma unroll
      for (int c = 0; c < 8; ++c) lds16(&v[c * PER16], row + ((c ^ sw) << 4));
    }
    // Unrolled over the tile with constant indices (v stays in registers);
    // positions past the end of the axis are skipped.
    // The lane's first element starts it (comparing it with itself then
    // changes nothing, NaN included), so full tiles need no per-element
    // checks beyond the compare.
    if (it == 0) best = blockIdx.z == 0 ? Ord::start(v[0]) : Ord::none();
    int bet = -1;  // position of this tile's improvement, if any
    if (cnt == TB) {
#pragma unroll
      for (int e = 0; e < TB; ++e) {
        const typename Ord::K k = Ord::key(v[e]);
        if (MAX ? (k > best) : (k < best)) {
          best = k;
          bet = e;
        }
      }
    } else {
#pragma unroll
      for (int e = 0; e < TB; ++e) {
        const typename Ord::K k = Ord::key(v[e]);
        if (e < cnt && (MAX ? (k > best) : (k < best))) {
          best = k;
          bet = e;
        }
      }
    }
    if (bet >= 0) {
      bt = (int)it;
      be = bet;
      found = true;
    }
    __syncthreads();  // every thread is done with stage s
    if (t == 0 && it + STAGES < n_tiles) load(s, it + STAGES);
  }
  if (abort_flag) {
    if (t == 0) {
      atomicOr(err, NRS_DEVERR_REDUCE_TMA | (7u << 8));
      for (int64_t j = it; j < n_tiles && j < it + STAGES; ++j)
        mbar_wait_bounded(&full[j % STAGES], (uint32_t)((j / STAGES) & 1), NRS_WAIT_LIMIT);
    }
    return;
  }
  const int64_t lane = l0 + t;
  if (lane < lanes) {
    const int64_t o = (int64_t)batch * lanes + lane;
    if (!part_key) {
      out[o] = (int64_t)bt * TB + be;
    } else {
      const int64_t po = (int64_t)blockIdx.z * lanes * gridDim.y + o;
      out[po] = found ? a0 + (int64_t)bt * TB + be : -1;
      part_key[po] = best;
    }
  }
}

constexpr int kStages = 8;

// ---------------------------------------------------------------------------
// Flat reductions
// ---------------------------------------------------------------------------
// Per-chunk partials in the lane-striped order of a 256-lane SIMD sum: lane L
// folds elements L, L+256, ... of its chunk in order, then the 256 lanes
// combine as eight groups of 32 (xor butterfly over offsets 16, 8, 4, 2, 1,
// the lower-index side first) whose eight results fold in group order
// (block_combine's tree). MIN/MAX fold with a NaN flag and ignore NaNs in
// the value, as chunk_min/chunk_max do (src/kernels/reduce.rs:337-350). SSD
// folds (x - mean)^2.
//
// One warp owns a chunk and each thread eight consecutive lanes (8t..8t+7),
// so a step of the order is one contiguous 256-element row read with 16-byte
// loads, and the combine needs no block barrier: butterfly offsets 16 and 8
// are thread xor 2 and 1, offsets 4, 2, 1 stay inside a thread, and group g's
// result sits in thread 4g.
constexpr int kFlatLanesPerThread = 8;
constexpr int kFlatBlocksPerSM = 4;

template <typename T, bool VEC>
__device__ __forceinline__ void load_lanes(const T* p, T (&v)[kFlatLanesPerThread]) {
  if constexpr (VEC) {
    constexpr int NV = kFlatLanesPerThread * (int)sizeof(T) / 16;
    uint4 u[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) u[i] = reinterpret_cast<const uint4*>(p)[i];
    memcpy(v, u, sizeof(v));
  } else {
#pragma unroll
    for (int j = 0; j < kFlatLanesPerThread; ++j) v[j] = p[j];
  }
}

template <typename T, int OP, bool SSD>
__device__ __forceinline__ void fold_lane(T& acc, int& nan, T v, T mean) {
  if constexpr (SSD) {
    T d = v - mean;
    v = d * d;
  }
  if constexpr (OP == NRS_MAX || OP == NRS_MIN) {
    nan |= is_nan(v);
    if (!is_nan(v)) acc = Fold<T, OP>::step(acc, v);
  } else {
    acc = Fold<T, OP>::step(acc, v);
  }
}

template <typename T, int OP, bool SSD, bool VEC>
__global__ void __launch_bounds__(256, kFlatBlocksPerSM)
    flat_partials(const T* __restrict__ x, int64_t n, int64_t chunk, const T* mean_ptr,
                  Partial<T>* __restrict__ part) {
  constexpr int LPT = kFlatLanesPerThread;
  constexpr int UNROLL = sizeof(T) == 8 ? 2 : 4;  // 128 bytes of loads in flight per thread
  const int64_t nchunks = (n + chunk - 1) / chunk;
  const T mean = SSD ? *mean_ptr : T(0);
  const int t = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nwarps) {
    const int64_t lo = c * chunk;
    const int64_t len = (n - lo) < chunk ? (n - lo) : chunk;
    const T* p = x + lo + LPT * t;
    if constexpr (std::is_same<T, double>::value && (OP == NRS_MAX || OP == NRS_MIN) && !SSD) {
      // f64 max / min on int64 keys (no FP64 instruction per element): the
      // chunk's extreme when it holds no NaN and no zero (the extreme is then
      // unique in bits and the order is free); otherwise the chunk is folded
      // again below with the ordered steps.
      using RF = RunFold<double, OP>;
      const int64_t k0 = RF::key64((uint64_t)__double_as_longlong(Fold<double, OP>::init()));
      int64_t kacc[LPT];
#pragma unroll
      for (int j = 0; j < LPT; ++j) kacc[j] = k0;
      bool odd = false;
      auto kfold = [&](int64_t& a, double v) {
        const uint64_t u = (uint64_t)__double_as_longlong(v);
        odd |= RF::nan_or_zero64(u);
        const int64_t k = RF::key64(u);
        a = (OP == NRS_MAX ? (k > a) : (k < a)) ? k : a;
      };
      const int64_t full = len / 256;
#pragma unroll UNROLL
      for (int64_t k = 0; k < full; ++k) {
        T v[LPT];
        load_lanes<T, VEC>(p + 256 * k, v);
#pragma unroll
        for (int j = 0; j < LPT; ++j) kfold(kacc[j], v[j]);
      }
      const int64_t rest = len - 256 * full;
#pragma unroll
      for (int j = 0; j < LPT; ++j)
        if (LPT * t + j < rest) kfold(kacc[j], p[256 * full + j]);
      if (!__any_sync(0xffffffffu, odd)) {
        int64_t b = kacc[0];
#pragma unroll
        for (int j = 1; j < LPT; ++j) b = (OP == NRS_MAX ? (kacc[j] > b) : (kacc[j] < b)) ? kacc[j] : b;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const int64_t o = __shfl_xor_sync(0xffffffffu, b, off);
          b = (OP == NRS_MAX ? (o > b) : (o < b)) ? o : b;
        }
        if (t == 0) part[c] = Partial<T>{__longlong_as_double((long long)RF::key64((uint64_t)b)), 0};
        continue;
      }
    }
    T acc[LPT];
#pragma unroll
    for (int j = 0; j < LPT; ++j) acc[j] = Fold<T, OP>::init();
    int nan = 0;
    const int64_t full = len / 256;  // steps in which all 256 lanes have an element
#pragma unroll UNROLL
    for (int64_t k = 0; k < full; ++k) {
      T v[LPT];
      load_lanes<T, VEC>(p + 256 * k, v);
#pragma unroll
      for (int j = 0; j < LPT; ++j) fold_lane<T, OP, SSD>(acc[j], nan, v[j], mean);
    }
    const int64_t rest = len - 256 * full;
#pragma unroll
    for (int j = 0; j < LPT; ++j)
      if (LPT * t + j < rest) fold_lane<T, OP, SSD>(acc[j], nan, p[256 * full + j], mean);
#pragma unroll
    for (int j = 0; j < LPT; ++j) {
      acc[j] = Fold<T, OP>::step(acc[j], __shfl_xor_sync(0xffffffffu, acc[j], 2));
      acc[j] = Fold<T, OP>::step(acc[j], __shfl_xor_sync(0xffffffffu, acc[j], 1));
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] = Fold<T, OP>::step(acc[j], acc[j + 4]);
#pragma unroll
    for (int j = 0; j < 2; ++j) acc[j] = Fold<T, OP>::step(acc[j], acc[j + 2]);
    acc[0] = Fold<T, OP>::step(acc[0], acc[1]);
    T r = __shfl_sync(0xffffffffu, acc[0], 0);
#pragma unroll
    for (int g = 1; g < 8; ++g) r = Fold<T, OP>::step(r, __shfl_sync(0xffffffffu, acc[0], 4 * g));
    if constexpr (std::is_floating_point<T>::value && (OP == NRS_MAX || OP == NRS_MIN) && !SSD) {
      // An extreme of zero: the left-to-right fold keeps the chunk's first
      // zero (-0.0 and +0.0 tie), which the lane order above does not
      // track; the warp looks it up (lane l checks l, l + 32, ...).
      if (r == T(0)) {
        int64_t fz = len;
        for (int64_t i = t; i < len; i += 32)
          if (x[lo + i] == T(0)) {
            fz = i;
            break;
          }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const int64_t o = __shfl_xor_sync(0xffffffffu, fz, off);
          fz = o < fz ? o : fz;
        }
        r = x[lo + fz];
      }
    }
    const int anynan = __any_sync(0xffffffffu, nan);
    if (t == 0) part[c] = Partial<T>{r, anynan};
  }
}

// Blocks of 256 threads for one warp per chunk: about the same number of
// chunks per warp, on a grid that is resident at once.
inline int flat_warp_grid(int64_t nchunks, int sms) {
  if (nchunks < 1) return 1;
  const int64_t cap = (int64_t)sms * kFlatBlocksPerSM * 8;  // resident warps
  const int64_t per = (nchunks + cap - 1) / cap;
  const int64_t warps = (nchunks + per - 1) / per;
  return (int)((warps + 7) / 8);
}

// Launches flat_partials: 16-byte loads when the array is 16-byte aligned
// (chunk starts then are too: a chunk is 8192 elements or the whole array).
template <typename T, int OP, bool SSD>
void launch_partials(cudaStream_t s, int sms, const T* x, int64_t n, int64_t chunk, const T* mean,
                     Partial<T>* part) {
  const int grid = flat_warp_grid((n + chunk - 1) / chunk, sms);
  if ((reinterpret_cast<uintptr_t>(x) & 15) == 0)
    flat_partials<T, OP, SSD, true><<<grid, 256, 0, s>>>(x, n, chunk, mean, part);
  else
    flat_partials<T, OP, SSD, false><<<grid, 256, 0, s>>>(x, n, chunk, mean, part);
}

// Folds the chunk partials: 1024 or fewer in chunk order by one thread (the
// reference's sequential fold of the collected Vec); more than 1024 first as
// 1024 interleaved runs (thread t folds partials t, t+1024, ... in order: a
// warp reads 32 consecutive partials per step), then the runs in order. The
// order does not depend on the grid or the device.
// `fin_op` says what to write: the folded value (SUM/MAX/MIN/PROD), the mean
// (MEAN; f64 for integers), the mean into `mean_out` for the variance's second
// pass (-1), or VAR/STD from the folded squared deviations.
template <typename T, int OP>
__global__ void __launch_bounds__(1024)
    flat_finish(const Partial<T>* __restrict__ part, int64_t nchunks, int64_t n, int fin_op,
                double ddof, T* mean_out, void* out) {
  __shared__ T run[1024];
  __shared__ int runnan[1024];
  const int t = threadIdx.x;
  T acc = Fold<T, OP>::init();
  int nan = 0;
#pragma unroll 8
  for (int64_t i = t; i < nchunks; i += 1024) {
    const Partial<T> p = part[i];
    acc = Fold<T, OP>::step(acc, p.v);
    nan |= p.nan;
  }
  T r = Fold<T, OP>::init();
  int anynan = 0;
  if constexpr (OP == NRS_MAX || OP == NRS_MIN) {
    // The partials hold no NaN (a flag carries it), and without NaNs max/min
    // depend on the grouping only in which of two equal zeros is kept: the
    // runs combine as a tree of (value, first chunk) pairs, equal values
    // keeping the smaller chunk, so the result is the left-to-right fold's.
    int64_t ai = nchunks;  // chunk of acc's value (none yet)
    {
      T a2 = Fold<T, OP>::init();
      for (int64_t i = t; i < nchunks; i += 1024) {
        const T v = part[i].v;
        if (OP == NRS_MAX ? (v > a2) : (v < a2)) {
          a2 = v;
          ai = i;
        }
      }
      acc = a2;
    }
    auto take = [](T v, int64_t i, T w, int64_t j) {
      return (OP == NRS_MAX ? (v > w) : (v < w)) || (v == w && i < j);
    };
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const T ov = __shfl_xor_sync(0xffffffffu, acc, off);
      const int64_t oi = __shfl_xor_sync(0xffffffffu, ai, off);
      if (take(ov, oi, acc, ai)) {
        acc = ov;
        ai = oi;
      }
    }
    __shared__ int64_t runi[32];
    if ((t & 31) == 0) {
      run[t >> 5] = acc;
      runi[t >> 5] = ai;
    }
    anynan = __syncthreads_or(nan);
    if (t != 0) return;
    r = run[0];
    int64_t ri = runi[0];
    for (int w = 1; w < 32; ++w)
      if (take(run[w], runi[w], r, ri)) {
        r = run[w];
        ri = runi[w];
      }
  } else {
    run[t] = acc;
    runnan[t] = nan;
    __syncthreads();
    if (t != 0) return;
    const int nruns = nchunks < 1024 ? (int)nchunks : 1024;
#pragma unroll 8
    for (int i = 0; i < nruns; ++i) {
      r = Fold<T, OP>::step(r, run[i]);
      anynan |= runnan[i];
    }
  }
  if constexpr (OP == NRS_MAX || OP == NRS_MIN) {
    if constexpr (std::is_floating_point<T>::value) {
      if (anynan) r = (T)NAN;
    }
    static_cast<T*>(out)[0] = r;
  } else if constexpr (OP == NRS_SUM) {
    if (fin_op == NRS_SUM) {
      static_cast<T*>(out)[0] = r;
    } else if (fin_op == NRS_MEAN) {
      if constexpr (std::is_floating_point<T>::value)
        static_cast<T*>(out)[0] = r / (T)n;
      else
        static_cast<double*>(out)[0] = (double)r / (double)n;
    } else if constexpr (std::is_floating_point<T>::value) {
      if (fin_op == -1) {
        *mean_out = r / (T)n;
      } else {  // VAR / STD from the sum of squared deviations
        T var = r / ((T)n - (T)ddof);
        static_cast<T*>(out)[0] = (fin_op == NRS_STD) ? sqrt(var) : var;
      }
    }
  } else {
    static_cast<T*>(out)[0] = r;
  }
}

template <typename T>
__global__ void write_scalar(T* out, T v) { out[0] = v; }

// Logical-order gather of a non-contiguous view into a contiguous buffer
// (kernels::borrow::operand, src/kernels/borrow.rs:59).
template <typename T>
__global__ void gather_view(const T* __restrict__ x, KeptDims kd, int64_t n, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = i, off = 0;
    for (int d = kd.n - 1; d >= 0; --d) {
      int64_t c = rem % kd.size[d];
      rem /= kd.size[d];
      off += c * kd.stride[d];
    }
    y[i] = x[off];
  }
}

template <typename T>
__global__ void fill_value(T* out, int64_t n, T v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = v;
}

// Max / min split along the axis: the parts' results fold in axis order
// with the lane fold's own step. The step is a monoid action (a lane's first
// NaN stays; strict comparisons keep the first of equal values), so the
// result is the unsplit fold's bit for bit.
template <typename T, int OP>
__global__ void __launch_bounds__(256)
    combine_parts(const T* __restrict__ part, int parts, int64_t n, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = Fold<T, OP>::init();
    for (int p = 0; p < parts; ++p) acc = Fold<T, OP>::step(acc, part[p * n + i]);
    out[i] = acc;
  }
}

// argmax / argmin split along the axis: part 0's candidate (the lane's
// first element seeds it, a leading NaN unbeatable), then each later part's
// candidate, if it has one, replaces it only when strictly better, so the
// first index of the extreme wins as in one left-to-right scan.
template <typename K, bool MAX>
__global__ void __launch_bounds__(256)
    combine_arg_parts(const K* __restrict__ key, const int64_t* __restrict__ idx, int parts, int64_t n,
                      int64_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    K best = key[i];
    int64_t bi = idx[i];
    for (int p = 1; p < parts; ++p) {
      const int64_t j = idx[p * n + i];
      const K k = key[p * n + i];
      if (j >= 0 && (MAX ? (k > best) : (k < best))) {
        best = k;
        bi = j;
      }
    }
    out[i] = bi;
  }
}

// ---------------------------------------------------------------------------
// Host dispatch
// ---------------------------------------------------------------------------
CUtensorMapDataType tma_dtype(int dtype) {
  switch (dtype) {
    case NRS_F32: return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    case NRS_F64: return CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    case NRS_I32: return CU_TENSOR_MAP_DATA_TYPE_INT32;
    default: return CU_TENSOR_MAP_DATA_TYPE_INT64;
  }
}

struct AxisProblem {
  int dtype, op;
  const void* x;
  void* out;
  int64_t alen, astride;
  KeptDims kept;  // collapsed kept dims, outer to inner
  int64_t n_out;
  const void* lane_mean;  // VAR/STD second pass: per-lane means (else null)
  double div;             // VAR/STD divisor: axis length - ddof
};

template <typename T, int OP>
int launch_generic(nrs_handle* h, const AxisProblem& p) {
  int64_t blocks = (p.n_out + 255) / 256;
  int grid = (int)(blocks < (int64_t)h->num_sms * 16 ? blocks : (int64_t)h->num_sms * 16);
  if (grid < 1) grid = 1;
  fold_generic<T, OP><<<grid, 256, 0, h->stream>>>(
      (const T*)p.x, p.kept, p.n_out, p.alen, p.astride, (typename OutOf<T, OP>::type*)p.out,
      (const T*)p.lane_mean, (T)p.div);
  return nrs_after_launch(h, "fold_generic");
}

template <typename T, bool MAX>
int launch_arg_tma(nrs_handle* h, const AxisProblem& p);

template <typename T, bool MAX>
int launch_arg(nrs_handle* h, const AxisProblem& p) {
  if (p.alen >= 256 && p.n_out >= 64) {
    const int st = launch_arg_tma<T, MAX>(h, p);
    if (st != NRS_ERR_UNSUPPORTED) return st;
  }
  int64_t blocks = (p.n_out + 255) / 256;
  int grid = (int)(blocks < (int64_t)h->num_sms * 16 ? blocks : (int64_t)h->num_sms * 16);
  if (grid < 1) grid = 1;
  arg_generic<T, MAX><<<grid, 256, 0, h->stream>>>((const T*)p.x, p.kept, p.n_out, p.alen,
                                                   p.astride, (int64_t*)p.out);
  return nrs_after_launch(h, "arg_generic");
}

// Builds a 3-D tensor map (dim0 contiguous). Returns false if TMA rules are
// not met (base or strides not multiples of 16 bytes, sizes beyond limits).
bool make_map(CUtensorMap* map, int dtype, const void* base, const uint64_t dims[3],
              const uint64_t strides_bytes[2], const uint32_t box[3], CUtensorMapSwizzle sw) {
  auto enc = nrs_get_encode_tiled();
  if (!enc) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
  for (int i = 0; i < 2; ++i)
    if ((strides_bytes[i] & 15) != 0 || strides_bytes[i] >= (1ull << 40) || strides_bytes[i] == 0)
      return false;
  for (int i = 0; i < 3; ++i)
    if (dims[i] == 0 || dims[i] > (1ull << 32)) return false;
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, tma_dtype(dtype), 3, const_cast<void*>(base), dims, strides_bytes, box,
                   estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Tries the TMA kernels for a (batch, lanes) x axis problem. Returns
// NRS_ERR_UNSUPPORTED (nothing launched) when the view does not qualify.
template <typename T, int OP>
int launch_tma(nrs_handle* h, const AxisProblem& p) {
  const int es = sizeof(T);
  const KeptDims& k = p.kept;
  if (k.n < 1 || k.n > 2 || p.alen < 1) return NRS_ERR_UNSUPPORTED;
  const int64_t lanes = k.size[k.n - 1], lstride = k.stride[k.n - 1];
  const int64_t batch = (k.n == 2) ? k.size[0] : 1;
  const int64_t bstride = (k.n == 2) ? k.stride[0] : 0;
  if (batch > 65535) return NRS_ERR_UNSUPPORTED;
  CUtensorMap map;
  const size_t tile_bytes = 8192;
  const size_t smem = PipeSmem<8192, kStages>::kBytes;
  using OutT = typename OutOf<T, OP>::type;
  // Max / min whose CTAs leave resident slots idle split the axis into up
  // to 8 parts of whole tiles (at least 8 tiles each), one CTA per (lanes,
  // part), as many parts as fit one wave of resident CTAs (a second, partial
  // wave costs more than it gains), and combine the parts in order
  // (combine_parts).
  const int64_t ctas = ((lanes + 63) / 64) * batch;
  int64_t parts = 1, part_len = p.alen;
  OutT* dst = (OutT*)p.out;
  const int64_t n_out = lanes * batch;
  auto plan_parts = [&](const void* kern, int threads, int64_t axis_tile) -> int {
    if constexpr (OP == NRS_MAX || OP == NRS_MIN) {
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
      }
      parts = ((int64_t)per_sm * h->num_sms) / ctas;
      const int64_t by_len = p.alen / (8 * axis_tile);
      if (parts > by_len) parts = by_len;
      if (parts > 8) parts = 8;
      if (parts < 1) parts = 1;
    }
    part_len = ((p.alen + parts - 1) / parts + axis_tile - 1) / axis_tile * axis_tile;
    parts = (p.alen + part_len - 1) / part_len;
    if (parts > 1) {
      int st;
      dst = (OutT*)nrs_workspace(h, (size_t)(parts * n_out) * sizeof(OutT) + 256, &st);
      if (!dst) return st;
    }
    return NRS_OK;
  };
  auto combine = [&]() -> int {
    if (parts > 1) {
      if constexpr (OP == NRS_MAX || OP == NRS_MIN) {
        const int64_t blocks = (n_out + 255) / 256;
        combine_parts<T, OP><<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, h->stream>>>(
            (const T*)dst, (int)parts, n_out, (T*)p.out);
      }
    }
    return NRS_OK;
  };
  if (lstride == 1 && p.astride > 1) {
    // Columns: dims (lanes, axis, batch).
    const uint64_t dims[3] = {(uint64_t)lanes, (uint64_t)p.alen, (uint64_t)batch};
    uint64_t sb = (uint64_t)(batch > 1 ? bstride : p.astride * p.alen) * es;
    const uint64_t strides[2] = {(uint64_t)p.astride * es, sb};
    const uint32_t box[3] = {(uint32_t)kColLanes, (uint32_t)col_rows<T>(), 1};
    if (!make_map(&map, p.dtype, p.x, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE))
      return NRS_ERR_UNSUPPORTED;
    auto kern = fold_cols_tma<T, OP, kStages>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (int st = plan_parts((const void*)kern, kColLanes, col_rows<T>())) return st;
    dim3 grid((unsigned)((lanes + kColLanes - 1) / kColLanes), (unsigned)batch, (unsigned)parts);
    kern<<<grid, kColLanes, smem, h->stream>>>(map, p.alen, lanes, dst, h->dev_error,
                                               (const T*)p.lane_mean, (T)p.div, part_len, n_out);
    combine();
    return nrs_after_launch(h, "fold_cols_tma");
  }
  if (p.astride == 1 && lstride > 1) {
    // Rows: dims (axis, lanes, batch), 128-byte swizzle.
    const uint64_t dims[3] = {(uint64_t)p.alen, (uint64_t)lanes, (uint64_t)batch};
    uint64_t sb = (uint64_t)(batch > 1 ? bstride : lstride * lanes) * es;
    const uint64_t strides[2] = {(uint64_t)lstride * es, sb};
    const uint32_t box[3] = {(uint32_t)(128 / es), 64, 1};
    if (!make_map(&map, p.dtype, p.x, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B))
      return NRS_ERR_UNSUPPORTED;
    auto kern = fold_rows_tma<T, OP, kStages>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (int st = plan_parts((const void*)kern, 64, 128 / es)) return st;
    dim3 grid((unsigned)((lanes + 63) / 64), (unsigned)batch, (unsigned)parts);
    kern<<<grid, 64, smem, h->stream>>>(map, p.alen, lanes, dst, h->dev_error,
                                        (const T*)p.lane_mean, (T)p.div, part_len, n_out);
    combine();
    return nrs_after_launch(h, "fold_rows_tma");
  }
  (void)tile_bytes;
  return NRS_ERR_UNSUPPORTED;
}

// argmax / argmin through the TMA lane pipelines (the fold kernels'
// geometry); NRS_ERR_UNSUPPORTED when the view does not qualify.
template <typename T, bool MAX>
int launch_arg_tma(nrs_handle* h, const AxisProblem& p) {
  const int es = sizeof(T);
  const KeptDims& k = p.kept;
  if (k.n < 1 || k.n > 2 || p.alen < 1) return NRS_ERR_UNSUPPORTED;
  const int64_t lanes = k.size[k.n - 1], lstride = k.stride[k.n - 1];
  const int64_t batch = (k.n == 2) ? k.size[0] : 1;
  const int64_t bstride = (k.n == 2) ? k.stride[0] : 0;
  if (batch > 65535) return NRS_ERR_UNSUPPORTED;
  const size_t smem = PipeSmem<8192, kStages>::kBytes;
  CUtensorMap map;
  // Too few CTAs for one wave of resident slots: split the axis into up to
  // 8 parts of whole tiles (at least 8 tiles each), as many as fit one wave,
  // and combine the parts' candidates in order (combine_arg_parts).
  using Key = typename ArgOrd<T, MAX>::K;
  const int64_t ctas = ((lanes + 63) / 64) * batch;
  const int64_t n_out = lanes * batch;
  int64_t parts = 1, part_len = p.alen;
  int64_t* idx = (int64_t*)p.out;
  Key* pkey = nullptr;
  auto plan_parts = [&](const void* kern, int64_t axis_tile) -> int {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 64, smem) != cudaSuccess) {
      cudaGetLastError();
      per_sm = 1;
    }
    parts = ((int64_t)per_sm * h->num_sms) / ctas;
    const int64_t by_len = p.alen / (8 * axis_tile);
    if (parts > by_len) parts = by_len;
    if (parts > 8) parts = 8;
    if (parts < 1) parts = 1;
    part_len = ((p.alen + parts - 1) / parts + axis_tile - 1) / axis_tile * axis_tile;
    parts = (p.alen + part_len - 1) / part_len;
    if (parts > 1) {
      int st;
      uint8_t* ws = (uint8_t*)nrs_workspace(h, (size_t)(parts * n_out) * (sizeof(int64_t) + sizeof(Key)) + 256, &st);
      if (!ws) return st;
      idx = reinterpret_cast<int64_t*>(ws);
      pkey = reinterpret_cast<Key*>(ws + (size_t)(parts * n_out) * sizeof(int64_t));
    }
    return NRS_OK;
  };
  auto combine = [&]() {
    if (parts > 1) {
      const int64_t blocks = (n_out + 255) / 256;
      combine_arg_parts<Key, MAX><<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, h->stream>>>(
          pkey, idx, (int)parts, n_out, (int64_t*)p.out);
    }
  };
  if (lstride == 1 && p.astride > 1) {
    const uint64_t dims[3] = {(uint64_t)lanes, (uint64_t)p.alen, (uint64_t)batch};
    const uint64_t strides[2] = {(uint64_t)p.astride * es, (uint64_t)(batch > 1 ? bstride : p.astride * p.alen) * es};
    const uint32_t box[3] = {(uint32_t)kColLanes, (uint32_t)col_rows<T>(), 1};
    if (!make_map(&map, p.dtype, p.x, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE)) return NRS_ERR_UNSUPPORTED;
    auto kern = arg_lane_tma<T, MAX, true, kStages>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (int st = plan_parts((const void*)kern, col_rows<T>())) return st;
    dim3 grid((unsigned)((lanes + 63) / 64), (unsigned)batch, (unsigned)parts);
    kern<<<grid, 64, smem, h->stream>>>(map, p.alen, lanes, idx, h->dev_error, part_len, pkey);
    combine();
    return nrs_after_launch(h, "arg_lane_tma");
  }
  if (p.astride == 1 && lstride > 1) {
    const uint64_t dims[3] = {(uint64_t)p.alen, (uint64_t)lanes, (uint64_t)batch};
    const uint64_t strides[2] = {(uint64_t)lstride * es, (uint64_t)(batch > 1 ? bstride : lstride * lanes) * es};
    const uint32_t box[3] = {(uint32_t)(128 / es), 64, 1};
    if (!make_map(&map, p.dtype, p.x, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B)) return NRS_ERR_UNSUPPORTED;
    auto kern = arg_lane_tma<T, MAX, false, kStages>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (int st = plan_parts((const void*)kern, 128 / es)) return st;
    dim3 grid((unsigned)((lanes + 63) / 64), (unsigned)batch, (unsigned)parts);
    kern<<<grid, 64, smem, h->stream>>>(map, p.alen, lanes, idx, h->dev_error, part_len, pkey);
    combine();
    return nrs_after_launch(h, "arg_lane_tma");
  }
  return NRS_ERR_UNSUPPORTED;
}

template <typename T, int OP>
int dispatch_axis_t(nrs_handle* h, const AxisProblem& p) {
  // The TMA pipelines pay off once lanes are long enough to fill a pipeline.
  if (p.alen >= 256 && p.n_out >= 64) {
    int st = launch_tma<T, OP>(h, p);
    if (st != NRS_ERR_UNSUPPORTED) return st;
  }
  return launch_generic<T, OP>(h, p);
}

template <typename T>
int dispatch_axis_ops(nrs_handle* h, const AxisProblem& p) {
  switch (p.op) {
    case NRS_SUM: return dispatch_axis_t<T, NRS_SUM>(h, p);
    case NRS_MEAN: return dispatch_axis_t<T, NRS_MEAN>(h, p);
    case NRS_MAX: return dispatch_axis_t<T, NRS_MAX>(h, p);
    case NRS_MIN: return dispatch_axis_t<T, NRS_MIN>(h, p);
    case NRS_PROD: return dispatch_axis_t<T, NRS_PROD>(h, p);
    case NRS_ARGMAX: return launch_arg<T, true>(h, p);
    case NRS_ARGMIN: return launch_arg<T, false>(h, p);
    default: {
      if constexpr (!std::is_floating_point<T>::value) {
        return nrs_fail(h, NRS_ERR_DTYPE, "VAR/STD need a float dtype");
      } else {
        // math::statistics::var(axis): per-lane mean first (the MEAN fold),
        // then the sum of squared deviations from it, / (axis length - ddof).
        int st;
        T* means = (T*)nrs_workspace(h, (size_t)p.n_out * sizeof(T) + 256, &st);
        if (!means) return st;
        AxisProblem pm = p;
        pm.out = means;
        pm.lane_mean = nullptr;
        if ((st = dispatch_axis_t<T, NRS_MEAN>(h, pm))) return st;
        AxisProblem pv = p;
        pv.lane_mean = means;
        return p.op == NRS_VAR ? dispatch_axis_t<T, NRS_VAR>(h, pv)
                               : dispatch_axis_t<T, NRS_STD>(h, pv);
      }
    }
  }
}

// Flat reduction of a contiguous buffer.
template <typename T>
int flat_reduce(nrs_handle* h, int op, int64_t n, int64_t ddof, const T* x, void* out) {
  // Tiering (src/kernels/reduce.rs): SUM/MEAN one simd_sum below 10k, else
  // 8192 chunks; VAR below 40k one pass each, else chunks; MIN/MAX (whose
  // partials keep the first of equal zeros) and PROD always use 8192 chunks.
  int64_t chunk;
  if (op == NRS_VAR || op == NRS_STD)
    chunk = (n < kVarParallelMin) ? (n > 0 ? n : 1) : kChunk;
  else if (op == NRS_SUM || op == NRS_MEAN)
    chunk = (n < kParallelMin) ? (n > 0 ? n : 1) : kChunk;
  else
    chunk = kChunk;
  const int64_t nchunks = n > 0 ? (n + chunk - 1) / chunk : 0;
  int st;
  size_t need = (size_t)(nchunks + 1) * sizeof(Partial<T>) + 256;
  uint8_t* ws = (uint8_t*)nrs_workspace(h, need, &st);
  if (!ws) return st;
  Partial<T>* part = reinterpret_cast<Partial<T>*>(ws);
  T* mean_slot = reinterpret_cast<T*>(ws + (size_t)(nchunks + 1) * sizeof(Partial<T>));
  if (n == 0) {
    T v = (op == NRS_PROD) ? T(1) : T(0);
    write_scalar<T><<<1, 1, 0, h->stream>>>((T*)out, v);
    return nrs_after_launch(h, "write_scalar");
  }
  switch (op) {
    case NRS_SUM:
    case NRS_MEAN:
      launch_partials<T, NRS_SUM, false>(h->stream, h->num_sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_SUM><<<1, 1024, 0, h->stream>>>(part, nchunks, n, op, 0.0, nullptr, out);
      break;
    case NRS_VAR:
    case NRS_STD:
      launch_partials<T, NRS_SUM, false>(h->stream, h->num_sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_SUM><<<1, 1024, 0, h->stream>>>(part, nchunks, n, -1, 0.0, mean_slot, nullptr);
      launch_partials<T, NRS_SUM, true>(h->stream, h->num_sms, x, n, chunk, mean_slot, part);
      flat_finish<T, NRS_SUM><<<1, 1024, 0, h->stream>>>(part, nchunks, n, op, (double)ddof, nullptr, out);
      break;
    case NRS_MAX:
      launch_partials<T, NRS_MAX, false>(h->stream, h->num_sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_MAX><<<1, 1024, 0, h->stream>>>(part, nchunks, n, op, 0.0, nullptr, out);
      break;
    case NRS_MIN:
      launch_partials<T, NRS_MIN, false>(h->stream, h->num_sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_MIN><<<1, 1024, 0, h->stream>>>(part, nchunks, n, op, 0.0, nullptr, out);
      break;
    case NRS_PROD:
      launch_partials<T, NRS_PROD, false>(h->stream, h->num_sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_PROD><<<1, 1024, 0, h->stream>>>(part, nchunks, n, op, 0.0, nullptr, out);
      break;
    default:
      return nrs_fail(h, NRS_ERR_INVALID, "unknown reduce op");
  }
  return nrs_after_launch(h, "flat reduction");
}

template <typename T, bool MAX>
int flat_arg(nrs_handle* h, int64_t n, const void* x, void* out) {
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  int st;
  const int grid = flat_warp_grid(nchunks, h->num_sms);
  const int64_t ncand = (int64_t)grid * 8;  // one candidate per warp
  ArgCand<T>* part = (ArgCand<T>*)nrs_workspace(h, (size_t)(ncand + 1) * sizeof(ArgCand<T>), &st);
  if (!part) return st;
  if ((reinterpret_cast<uintptr_t>(x) & 15) == 0)
    arg_partials<T, MAX, true><<<grid, 256, 0, h->stream>>>((const T*)x, n, part);
  else
    arg_partials<T, MAX, false><<<grid, 256, 0, h->stream>>>((const T*)x, n, part);
  arg_finish<T, MAX><<<1, 1024, 0, h->stream>>>((const T*)x, part, ncand, (int64_t*)out);
  return nrs_after_launch(h, "flat argmax/argmin");
}

// Integer flat reductions: any order is exact. MEAN writes f64.
template <typename T>
int flat_reduce_int(nrs_handle* h, int op, int64_t n, const T* x, void* out) {
  if (op != NRS_SUM && op != NRS_MAX && op != NRS_MIN && op != NRS_PROD && op != NRS_MEAN)
    return nrs_fail(h, NRS_ERR_DTYPE, "VAR/STD need a float dtype");
  if (n == 0) {
    if (op == NRS_MEAN) {
      write_scalar<double><<<1, 1, 0, h->stream>>>((double*)out, 0.0);
    } else {
      write_scalar<T><<<1, 1, 0, h->stream>>>((T*)out, op == NRS_PROD ? T(1) : T(0));
    }
    return nrs_after_launch(h, "write_scalar");
  }
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  int st;
  Partial<T>* part = (Partial<T>*)nrs_workspace(h, (size_t)(nchunks + 1) * sizeof(Partial<T>), &st);
  if (!part) return st;
  switch (op) {
    case NRS_SUM:
      launch_partials<T, NRS_SUM, false>(h->stream, h->num_sms, x, n, kChunk, nullptr, part);
      flat_finish<T, NRS_SUM><<<1, 1024, 0, h->stream>>>(part, nchunks, n, NRS_SUM, 0.0, nullptr, out);
      break;
    case NRS_MEAN:
      launch_partials<T, NRS_SUM, false>(h->stream, h->num_sms, x, n, kChunk, nullptr, part);
      flat_finish<T, NRS_SUM><<<1, 1024, 0, h->stream>>>(part, nchunks, n, NRS_MEAN, 0.0, nullptr, out);
      break;
    case NRS_MAX:
      launch_partials<T, NRS_MAX, false>(h->stream, h->num_sms, x, n, kChunk, nullptr, part);
      flat_finish<T, NRS_MAX><<<1, 1024, 0, h->stream>>>(part, nchunks, n, NRS_MAX, 0.0, nullptr, out);
      break;
    case NRS_MIN:
      launch_partials<T, NRS_MIN, false>(h->stream, h->num_sms, x, n, kChunk, nullptr, part);
      flat_finish<T, NRS_MIN><<<1, 1024, 0, h->stream>>>(part, nchunks, n, NRS_MIN, 0.0, nullptr, out);
      break;
    default:
      launch_partials<T, NRS_PROD, false>(h->stream, h->num_sms, x, n, kChunk, nullptr, part);
      flat_finish<T, NRS_PROD><<<1, 1024, 0, h->stream>>>(part, nchunks, n, NRS_PROD, 0.0, nullptr, out);
      break;
  }
  return nrs_after_launch(h, "flat integer reduction");
}

}  // namespace

extern "C" int nrs_reduce(nrs_handle* h, int dtype, int op, int ndim, const int64_t* shape,
                          const int64_t* strides, int64_t axis, int64_t ddof, const void* x,
                          void* out) {
  if (!h) return NRS_ERR_INVALID;
  h->last_error.clear();
  if (ndim < 0 || ndim > NRS_UFUNC_MAX_DIMS || (ndim > 0 && (!shape || !strides)))
    return nrs_fail(h, NRS_ERR_INVALID, "bad ndim/shape/strides");
  if (op < NRS_SUM || op > NRS_ARGMIN) return nrs_fail(h, NRS_ERR_INVALID, "unknown reduce op");
  const bool is_arg = (op == NRS_ARGMAX || op == NRS_ARGMIN);
  const size_t es = nrs_dtype_size(dtype);
  if (!es) return nrs_fail(h, NRS_ERR_DTYPE, "unknown dtype");
  const bool is_int = (dtype == NRS_I32 || dtype == NRS_I64);
  int64_t total = 1;
  for (int d = 0; d < ndim; ++d) {
    if (shape[d] < 0) return nrs_fail(h, NRS_ERR_SHAPE, "negative dimension");
    if (strides[d] < 0) return nrs_fail(h, NRS_ERR_STRIDE, "negative stride");
    total *= shape[d];
  }
  if (total > 0 && !x) return nrs_fail(h, NRS_ERR_INVALID, "null input");
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;

  if (axis == NRS_AXIS_NONE) {
    if (!out) return nrs_fail(h, NRS_ERR_INVALID, "null output");
    if (is_int && (op == NRS_VAR || op == NRS_STD))
      return nrs_fail(h, NRS_ERR_DTYPE, "VAR/STD need a float dtype");
    if (is_arg && total == 0)
      return nrs_fail(h, NRS_ERR_EMPTY, op == NRS_ARGMAX ? "Cannot find argmax of empty array"
                                                         : "Cannot find argmin of empty array");
    // Non-contiguous views are gathered into logical order first, as
    // kernels::borrow::operand does.
    bool contig = true;
    int64_t expect = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      if (shape[d] != 1 && strides[d] != expect) contig = false;
      expect *= shape[d];
    }
    const void* src = x;
    if (!contig && total > 0) {
      KeptDims kd{};
      kd.n = ndim;
      for (int d = 0; d < ndim; ++d) {
        kd.size[d] = shape[d];
        kd.stride[d] = strides[d];
      }
      // Reserve the gathered copy past the partials area of the workspace.
      size_t part_bytes = ((size_t)(total / kChunk + 2) * 16 + 4096 + 255) & ~size_t(255);
      uint8_t* ws = (uint8_t*)nrs_workspace(h, part_bytes + (size_t)total * es, &st);
      if (!ws) return st;
      void* dst = ws + part_bytes;
      int grid = h->num_sms * 8;
      if (es == 4)
        gather_view<uint32_t><<<grid, 256, 0, h->stream>>>((const uint32_t*)x, kd, total, (uint32_t*)dst);
      else
        gather_view<uint64_t><<<grid, 256, 0, h->stream>>>((const uint64_t*)x, kd, total, (uint64_t*)dst);
      if ((st = nrs_after_launch(h, "gather_view"))) return st;
      src = dst;
      // The flat kernels must not reuse the gathered region as partials: the
      // workspace is large enough that their partials (at offset 0) fit below.
    }
    if (is_arg) {
      switch (dtype) {
        case NRS_F32: return op == NRS_ARGMAX ? flat_arg<float, true>(h, total, src, out) : flat_arg<float, false>(h, total, src, out);
        case NRS_F64: return op == NRS_ARGMAX ? flat_arg<double, true>(h, total, src, out) : flat_arg<double, false>(h, total, src, out);
        case NRS_I64: return op == NRS_ARGMAX ? flat_arg<int64_t, true>(h, total, src, out) : flat_arg<int64_t, false>(h, total, src, out);
        default: return op == NRS_ARGMAX ? flat_arg<int32_t, true>(h, total, src, out) : flat_arg<int32_t, false>(h, total, src, out);
      }
    }
    switch (dtype) {
      case NRS_F32: return flat_reduce<float>(h, op, total, ddof, (const float*)src, out);
      case NRS_F64: return flat_reduce<double>(h, op, total, ddof, (const double*)src, out);
      case NRS_I64: return flat_reduce_int<int64_t>(h, op, total, (const int64_t*)src, out);
      default: return flat_reduce_int<int32_t>(h, op, total, (const int32_t*)src, out);
    }
  }

  if (ndim == 0) return nrs_fail(h, NRS_ERR_AXIS, "axis given for a 0-d array");
  int64_t ax = axis < 0 ? axis + ndim : axis;
  if (ax < 0 || ax >= ndim) {
    return nrs_fail(h, NRS_ERR_AXIS, "Axis " + std::to_string(axis) +
                                         " out of bounds for array of dimension " +
                                         std::to_string(ndim));
  }
  if (is_int && (op == NRS_VAR || op == NRS_STD))
    return nrs_fail(h, NRS_ERR_DTYPE, "VAR/STD need a float dtype");
  if (is_int && op == NRS_MEAN && dtype == NRS_I32)
    return nrs_fail(h, NRS_ERR_DTYPE, "i32 MEAN is not provided");
  if (total == 0 && (op == NRS_VAR || op == NRS_STD || is_arg))
    return nrs_fail(h, NRS_ERR_EMPTY, "Cannot reduce an empty array");
  if ((op == NRS_VAR || op == NRS_STD) && (ddof < 0 || shape[ax] <= ddof))
    return nrs_fail(h, NRS_ERR_EMPTY, "Degrees of freedom " + std::to_string(ddof) +
                                          " >= axis size " + std::to_string(shape[ax]));

  AxisProblem p{};
  p.dtype = dtype;
  p.op = op;
  p.x = x;
  p.out = out;
  p.alen = shape[ax];
  p.astride = strides[ax];
  p.lane_mean = nullptr;
  p.div = (double)(shape[ax] - ddof);
  // Collapse kept dims (outer to inner), dropping size-1 dims.
  KeptDims kd{};
  kd.n = 0;
  int64_t n_out = 1;
  for (int d = 0; d < ndim; ++d) {
    if (d == ax) continue;
    n_out *= shape[d];
    if (shape[d] == 1) continue;
    if (kd.n > 0 && kd.stride[kd.n - 1] == strides[d] * shape[d]) {
      kd.size[kd.n - 1] *= shape[d];
      kd.stride[kd.n - 1] = strides[d];
    } else {
      kd.size[kd.n] = shape[d];
      kd.stride[kd.n] = strides[d];
      kd.n++;
    }
  }
  p.kept = kd;
  p.n_out = n_out;
  if (total == 0) {
    if (n_out == 0 && (op == NRS_SUM || op == NRS_PROD)) return NRS_OK;
    // Empty array: math::sum gives zeros; max/min/mean error out.
    if (op == NRS_SUM || op == NRS_PROD) {
      if (!out) return nrs_fail(h, NRS_ERR_INVALID, "null output");
      int grid = h->num_sms * 4;
      if (dtype == NRS_F32) fill_value<float><<<grid, 256, 0, h->stream>>>((float*)out, n_out, op == NRS_PROD ? 1.f : 0.f);
      else if (dtype == NRS_F64) fill_value<double><<<grid, 256, 0, h->stream>>>((double*)out, n_out, op == NRS_PROD ? 1.0 : 0.0);
      else if (dtype == NRS_I64) fill_value<int64_t><<<grid, 256, 0, h->stream>>>((int64_t*)out, n_out, op == NRS_PROD ? 1 : 0);
      else fill_value<int32_t><<<grid, 256, 0, h->stream>>>((int32_t*)out, n_out, op == NRS_PROD ? 1 : 0);
      return nrs_after_launch(h, "fill_value");
    }
    return nrs_fail(h, NRS_ERR_EMPTY, "Cannot reduce an empty array");
  }
  if (!out) return nrs_fail(h, NRS_ERR_INVALID, "null output");
  switch (dtype) {
    case NRS_F32: return dispatch_axis_ops<float>(h, p);
    case NRS_F64: return dispatch_axis_ops<double>(h, p);
    case NRS_I64: return dispatch_axis_ops<int64_t>(h, p);
    default: {
      if (op == NRS_MEAN) return nrs_fail(h, NRS_ERR_DTYPE, "i32 MEAN is not provided");
      return dispatch_axis_ops<int32_t>(h, p);
    }
  }
}

// ---------------------------------------------------------------------------
// Allocation-free flat reduction
// ---------------------------------------------------------------------------
// Some callers cannot let this library call cudaMalloc: code that runs under
// another runtime's memory discipline (a serving stack or framework allocator
// that owns all device memory and budgets it), or latency-critical loops where
// the device-wide synchronisation an allocation can cause is not acceptable.
// nrs_reduce_flat_noalloc serves them: the same chunk-partial kernels as the
// flat path of nrs_reduce, with the partials in the file-scope array below
// instead of the handle's cudaMalloc'd workspace. The array is 128 KiB + 256 B
// and stays resident on every GPU that loads the library until the process
// exits. Its host-side name is only a stand-in, so the device address is
// fetched with cudaGetSymbolAddress once per device and cached.
namespace {
constexpr int64_t kNoAllocMaxChunks = 8192;  // partials of up to 8192 chunks
constexpr int64_t kNoAllocMaxElems = kNoAllocMaxChunks * kChunk;  // 67,108,864
constexpr int kNoAllocMaxDevices = 64;
static_assert(sizeof(Partial<double>) <= 16, "a chunk partial must fit 16 bytes");
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_partials[kNoAllocMaxChunks * 16 + 256];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {nullptr};
int g_noalloc_sms[kNoAllocMaxDevices] = {0};
// The context the cached address belongs to: after cudaDeviceReset (or with
// another context current) the module, and with it the array, can live at a
// new address, so a different current context repeats the lookup.
void* g_noalloc_ctx[kNoAllocMaxDevices] = {nullptr};

typedef int (*ctx_get_current_fn)(void**);
void* current_context() {
  static ctx_get_current_fn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<ctx_get_current_fn>(p);
    else
      cudaGetLastError();
  });
  void* ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

template <typename T>
int noalloc_flat(cudaStream_t s, int op, int64_t n, const T* x, void* out, void* scratch, int sms) {
  if (n == 0) {
    write_scalar<T><<<1, 1, 0, s>>>((T*)out, T(0));
    return cudaGetLastError() == cudaSuccess ? NRS_OK : NRS_ERR_CUDA;
  }
  // Same tiering as flat_reduce: SUM/MEAN use one chunk below 10000 elements.
  const int64_t chunk = ((op == NRS_SUM || op == NRS_MEAN) && n < kParallelMin) ? n : kChunk;
  const int64_t nchunks = (n + chunk - 1) / chunk;
  Partial<T>* part = static_cast<Partial<T>*>(scratch);
  switch (op) {
    case NRS_SUM:
    case NRS_MEAN:
      launch_partials<T, NRS_SUM, false>(s, sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_SUM><<<1, 1024, 0, s>>>(part, nchunks, n, op, 0.0, nullptr, out);
      break;
    case NRS_MAX:
      launch_partials<T, NRS_MAX, false>(s, sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_MAX><<<1, 1024, 0, s>>>(part, nchunks, n, op, 0.0, nullptr, out);
      break;
    default:
      launch_partials<T, NRS_MIN, false>(s, sms, x, n, chunk, nullptr, part);
      flat_finish<T, NRS_MIN><<<1, 1024, 0, s>>>(part, nchunks, n, op, 0.0, nullptr, out);
      break;
  }
  return cudaGetLastError() == cudaSuccess ? NRS_OK : NRS_ERR_CUDA;
}
}  // namespace

extern "C" int nrs_reduce_flat_noalloc(void* cuda_stream, int dtype, int op, int64_t n,
                                       const void* x, void* out) {
  if (dtype != NRS_F32 && dtype != NRS_F64) return NRS_ERR_DTYPE;
  if (op != NRS_SUM && op != NRS_MEAN && op != NRS_MAX && op != NRS_MIN) return NRS_ERR_INVALID;
  if (n < 0 || !out || (n > 0 && !x)) return NRS_ERR_INVALID;
  if (n > kNoAllocMaxElems) return NRS_ERR_TOO_LARGE;
  // An error left by earlier, unrelated work must not be reported as this
  // call's launch failure: clear it before the first launch.
  cudaGetLastError();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
    cudaGetLastError();
    return NRS_ERR_CUDA;
  }
  void* scratch;
  int sms;
  {
    // First call on a device (or in a new context of it): look up the
    // array's device address with this device current, and its SM count.
    // Later calls in the same context reuse both.
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    void* ctx = current_context();
    if (!g_noalloc_ptr[dev] || ctx != g_noalloc_ctx[dev]) {
      g_noalloc_ptr[dev] = nullptr;
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) {
        cudaGetLastError();
        return NRS_ERR_CUDA;
      }
      int count = 0;
      if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return NRS_ERR_CUDA;
      }
      g_noalloc_sms[dev] = count;
      g_noalloc_ptr[dev] = p;
      g_noalloc_ctx[dev] = ctx;
    }
    scratch = g_noalloc_ptr[dev];
    sms = g_noalloc_sms[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (dtype == NRS_F32) return noalloc_flat<float>(s, op, n, (const float*)x, out, scratch, sms);
  return noalloc_flat<double>(s, op, n, (const double*)x, out, scratch, sms);
}
