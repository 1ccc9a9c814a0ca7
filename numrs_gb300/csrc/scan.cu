// Seeded and running folds: ufunc reduce with `initial`, ufunc accumulate,
// cumsum and cumprod.
//
//   ufunc_ops::ufunc_reduce      src/ufunc_ops.rs:417 (reduce_full :265,
//                                reduce_along_axis :317, reduce_lane :230)
//   ufunc_ops::ufunc_accumulate  src/ufunc_ops.rs:523 (accumulate_flat :452,
//                                accumulate_along_axis :470)
//   math::cumsum / cumprod       src/math/statistics/mod.rs:584, :795
//
// Along an axis every lane is one sequential chain, exactly the reference's
// left-to-right fold, so results are bit-identical; lanes run in parallel
// through the same TMA pipelines as the axis reductions. A running fold
// (accumulate) rewrites each staged tile in shared memory with its prefix
// values and stores it back (a TMA store; per-row bulk copies for rows of
// 4-byte types): HBM traffic is one read and one write of the array.
//
// Over the flattened array (axis = None) the order-free cases use a
// reduce-then-scan over contiguous segments (8192-element chunks for
// unaligned arrays) whose combine always keeps the earlier operand on the
// left. maximum/minimum are associative under the
// reference's apply (NaN absorbs, ties take the right operand), so the
// parallel scan is exact; integer add/multiply wrap and are exact in any
// order; float add/multiply reassociate (tolerance-based, as the flat
// product is). subtract/divide are inherently serial and run as one lane.
#include <mutex>
#include <cmath>
#include <limits>
#include <string>
#include <type_traits>

#include "f64_round.cuh"
#include "nrs_internal.cuh"

namespace {

// ---------------------------------------------------------------------------
// UfuncOp::apply (src/ufunc_ops.rs:153-181)
// ---------------------------------------------------------------------------
template <typename T> NRS_DEV T qnan();
template <> NRS_DEV float qnan<float>() { return __int_as_float(0x7fc00000); }
template <> NRS_DEV double qnan<double>() { return __longlong_as_double(0x7ff8000000000000LL); }

// One rounding per op; maximum/minimum: NaN (Rust's quiet-NaN bits) if
// either side is NaN, else the left operand only if strictly greater
// (smaller). Integers wrap; integer division is rejected on the host.
template <typename T, int OP>
NRS_DEV T apply(T a, T b) {
  if constexpr (std::is_same<T, float>::value) {
    if constexpr (OP == NRS_OP_ADD) return __fadd_rn(a, b);
    else if constexpr (OP == NRS_OP_SUB) return __fsub_rn(a, b);
    else if constexpr (OP == NRS_OP_MUL) return __fmul_rn(a, b);
    else if constexpr (OP == NRS_OP_DIV) return __fdiv_rn(a, b);
    else if constexpr (OP == NRS_OP_MAX) return (a != a || b != b) ? qnan<float>() : (a > b ? a : b);
    else return (a != a || b != b) ? qnan<float>() : (a < b ? a : b);
  } else if constexpr (std::is_same<T, double>::value) {
    if constexpr (OP == NRS_OP_ADD) return __dadd_rn(a, b);
    else if constexpr (OP == NRS_OP_SUB) return __dsub_rn(a, b);
    else if constexpr (OP == NRS_OP_MUL) return __dmul_rn(a, b);
    else if constexpr (OP == NRS_OP_DIV) return __ddiv_rn(a, b);
    else if constexpr (OP == NRS_OP_MAX) return (a != a || b != b) ? qnan<double>() : (a > b ? a : b);
    else return (a != a || b != b) ? qnan<double>() : (a < b ? a : b);
  } else {
    using U = typename std::make_unsigned<T>::type;
    if constexpr (OP == NRS_OP_ADD) return (T)((U)a + (U)b);
    else if constexpr (OP == NRS_OP_SUB) return (T)((U)a - (U)b);
    else if constexpr (OP == NRS_OP_MUL) return (T)((U)a * (U)b);
    else if constexpr (OP == NRS_OP_MAX) return a > b ? a : b;
    else if constexpr (OP == NRS_OP_MIN) return a < b ? a : b;
    else return b == 0 ? T(0) : a / b;
  }
}

// A value e with apply(e, x) == x and apply(x, e) == x bit for bit, for the
// order-free ops: -0.0 for float add (-0 + -0 = -0, -0 + +0 = +0), 1 for
// multiply, -inf / +inf (integer extremes) for maximum / minimum.
template <typename T, int OP>
NRS_DEV T identity() {
  if constexpr (OP == NRS_OP_ADD) {
    if constexpr (std::is_floating_point<T>::value) return -T(0);
    else return T(0);
  } else if constexpr (OP == NRS_OP_MUL) {
    return T(1);
  } else if constexpr (OP == NRS_OP_MAX) {
    if constexpr (std::is_floating_point<T>::value) return -INFINITY;
    else return std::numeric_limits<T>::lowest();
  } else {
    if constexpr (std::is_floating_point<T>::value) return INFINITY;
    else return std::numeric_limits<T>::max();
  }
}

// ---------------------------------------------------------------------------
// Lanes
// ---------------------------------------------------------------------------
constexpr int kMaxDims = NRS_UFUNC_MAX_DIMS;

// Kept (non-axis) dimensions, outer to inner, with the input's strides and,
// for a running fold, the output's.
struct Lanes {
  int n;
  int64_t size[kMaxDims];
  int64_t xstride[kMaxDims];
  int64_t ostride[kMaxDims];
};

// How a lane starts: from `seed` folding every element, or from its first
// element (seed ignored).
struct Seed {
  int first;
  double fseed;   // f32/f64 seeds
  int64_t iseed;  // integer seeds
  template <typename T>
  __host__ __device__ T get() const {
    if constexpr (std::is_floating_point<T>::value) return (T)fseed;
    else return (T)iseed;
  }
};

// One thread per lane, any strides. RUNNING writes every prefix to
// out[obase + j * oastride]; otherwise the lane's result to out[o].
template <typename T, int OP, bool RUNNING>
__global__ void __launch_bounds__(256)
    lane_scan_generic(const T* __restrict__ x, Lanes g, int64_t n_lanes, int64_t alen,
                      int64_t xastride, T* __restrict__ out, int64_t oastride, Seed seed) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n_lanes;
       o += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = o, xb = 0, ob = 0;
    for (int d = g.n - 1; d >= 0; --d) {
      const int64_t c = rem % g.size[d];
      rem /= g.size[d];
      xb += c * g.xstride[d];
      ob += c * g.ostride[d];
    }
    T acc = seed.get<T>();
    int64_t j = 0;
    if (seed.first) {
      acc = x[xb];
      if (RUNNING) out[ob] = acc;
      j = 1;
    }
    for (; j < alen; ++j) {
      acc = apply<T, OP>(acc, x[xb + j * xastride]);
      if (RUNNING) out[ob + j * oastride] = acc;
    }
    if (!RUNNING) out[o] = acc;
  }
}

// Lanes adjacent in memory (stride 1), axis strided: tiles of 64 lanes x
// (8 KB / 64 / sizeof(T)) axis positions through an 8-stage TMA ring (the
// geometry of the column reductions). Thread t owns lane l0 + t.
constexpr int kLanesPerCta = 64;
constexpr int kScanStages = 8;
constexpr int kTileBytes = 8192;

template <typename T>
constexpr int col_rows() { return kTileBytes / (kLanesPerCta * (int)sizeof(T)); }

// 16-byte chunk j of row r of a 128-byte-swizzled tile.
NRS_DEV int swz(int r, int j) { return r * 128 + ((j ^ (r & 7)) << 4); }

// Folds one staged column (cols) / row (rows) of a tile into `acc`; with
// WRITE the prefix values replace the staged ones. `first` seeds the lane
// from its first element (the tile's element 0).
// Running fold of N staged values in place (v[e] becomes the prefix through
// e); `first` seeds the lane from v[0], which keeps its own bits. Float
// maximum / minimum give apply's result with a shorter dependent chain: a
// sticky flag records that a NaN has been seen (every later prefix is then
// the canonical NaN), so the value chain is one compare and select (ties keep
// the later operand, as apply does).
template <typename T, int OP, int N>
NRS_DEV T run_block(T (&v)[N], bool first, T acc);

// f32 maximum / minimum returning NaN when either operand is NaN (the
// instruction has no f64 form).
template <int OP>
NRS_DEV float nan_pick(float a, float b) {
  float d;
  if constexpr (OP == NRS_OP_MAX) asm("max.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
  else asm("min.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
  return d;
}

// The same fold's result without the prefixes (reductions). Float maximum /
// minimum are order-free over values that hold no NaN and no zero (equal
// values then have equal bits), so blocks fold as four independent chains:
// f32 with NaN-propagating max / min and one test of the result, f64 with
// fmax / fmin after a per-element NaN-or-zero test; a block with a NaN or
// a zero, or a NaN accumulator, takes the sequential chain. Other ops: the
// sequential chain.
template <typename T, int OP, int N>
NRS_DEV T reduce_block(T (&v)[N], bool first, T acc) {
  if constexpr (std::is_same<T, float>::value && (OP == NRS_OP_MAX || OP == NRS_OP_MIN) && N % 4 == 0) {
    // Four NaN-propagating chains, one instruction per element: a result
    // that is neither NaN nor zero is apply's fold bit for bit (equal nonzero
    // values have equal bits); a NaN (canonical in apply) or a zero (-0 and
    // +0 tie, the later wins) takes the ordered chain.
    if (first || acc == acc) {
      float a[4] = {first ? v[0] : nan_pick<OP>(acc, v[0]), v[1], v[2], v[3]};
#pragma unroll
      for (int e = 4; e < N; ++e) a[e & 3] = nan_pick<OP>(a[e & 3], v[e]);
      const float r = nan_pick<OP>(nan_pick<OP>(a[0], a[1]), nan_pick<OP>(a[2], a[3]));
      if (r == r && r != 0.0f) return r;
    }
  } else if constexpr (std::is_same<T, double>::value && (OP == NRS_OP_MAX || OP == NRS_OP_MIN) && N % 4 == 0) {
    // int64 keys (the magnitude bits of negatives flipped) order non-NaN,
    // nonzero doubles exactly, with no FP64 instruction per element.
    auto key = [](uint64_t u) { return nrs_f64_key(u); };
    auto odd = [](uint64_t u) { return nrs_f64_nan_or_zero(u); };
    auto better = [](int64_t k, int64_t a) { return OP == NRS_OP_MAX ? (k > a) : (k < a); };
    const uint64_t ua = (uint64_t)__double_as_longlong(acc);
    bool special = !first && odd(ua);
    int64_t a[4];
#pragma unroll
    for (int e = 0; e < N; ++e) {
      const uint64_t u = (uint64_t)__double_as_longlong(v[e]);
      special |= odd(u);
      const int64_t k = key(u);
      if (e < 4) a[e] = (e == 0 && !first) ? (better(k, key(ua)) ? k : key(ua)) : k;
      else a[e & 3] = better(k, a[e & 3]) ? k : a[e & 3];
    }
    if (!special) {
      const int64_t b0 = better(a[1], a[0]) ? a[1] : a[0];
      const int64_t b1 = better(a[3], a[2]) ? a[3] : a[2];
      return __longlong_as_double((long long)key((uint64_t)(better(b1, b0) ? b1 : b0)));
    }
  }
  return run_block<T, OP, N>(v, first, acc);
}

template <typename T, int OP, int N>
NRS_DEV T run_block(T (&v)[N], bool first, T acc) {
  if constexpr (std::is_floating_point<T>::value && (OP == NRS_OP_MAX || OP == NRS_OP_MIN)) {
    bool nanf = acc != acc;
    T a = acc;
#pragma unroll
    for (int e = 0; e < N; ++e) {
      const T xe = v[e];
      if (e == 0 && first) {
        a = xe;
        nanf = xe != xe;
      } else {
        nanf |= xe != xe;
        a = (OP == NRS_OP_MAX ? (a > xe) : (a < xe)) ? a : xe;
        v[e] = nanf ? qnan<T>() : a;
      }
    }
    return nanf ? qnan<T>() : a;
  } else {
#pragma unroll
    for (int e = 0; e < N; ++e) {
      acc = (e == 0 && first) ? v[0] : apply<T, OP>(acc, v[e]);
      v[e] = acc;
    }
    return acc;
  }
}

template <typename T, int OP, bool WRITE>
NRS_DEV T fold_col(T* tile, int t, int cnt, bool first, T acc) {
  constexpr int RB = col_rows<T>();
  constexpr int LW = kLanesPerCta;
  if (cnt == RB) {
    T v[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) v[r] = tile[r * LW + t];
    acc = WRITE ? run_block<T, OP, RB>(v, first, acc) : reduce_block<T, OP, RB>(v, first, acc);
    if (WRITE) {
#pragma unroll
      for (int r = 0; r < RB; ++r) tile[r * LW + t] = v[r];
    }
  } else {
    for (int r = 0; r < cnt; ++r) {
      acc = (r == 0 && first) ? tile[t] : apply<T, OP>(acc, tile[r * LW + t]);
      if (WRITE) tile[r * LW + t] = acc;
    }
  }
  return acc;
}

template <typename T, int OP, bool WRITE>
NRS_DEV T fold_row(uint8_t* tile, int t, int cnt, bool first, T acc) {
  constexpr int XB = 128 / sizeof(T);
  constexpr int PER16 = 16 / sizeof(T);
  if (cnt == XB) {
    // constant indices only, so v stays in registers
    T v[XB];
#pragma unroll
    for (int j = 0; j < 8; ++j) lds16(&v[j * PER16], tile + swz(t, j));
    acc = WRITE ? run_block<T, OP, XB>(v, first, acc) : reduce_block<T, OP, XB>(v, first, acc);
    if (WRITE) {
#pragma unroll
      for (int j = 0; j < 8; ++j) sts16(tile + swz(t, j), &v[j * PER16]);
    }
  } else {
    // the axis' last, short tile: element by element in the tile itself
    for (int e = 0; e < cnt; ++e) {
      T* p = reinterpret_cast<T*>(tile + swz(t, e / PER16)) + (e % PER16);
      acc = (e == 0 && first) ? *p : apply<T, OP>(acc, *p);
      if (WRITE) *p = acc;
    }
  }
  return acc;
}

// Reduction along lanes (one value per lane): the axis-reduction pipeline.
// COLS: lanes adjacent, map dims (lanes, axis, batch); else lanes along
// rows, map dims (axis, lanes, batch) with the 128-byte swizzle.
template <typename T, int OP, bool COLS>
__global__ void __launch_bounds__(kLanesPerCta)
    lane_reduce_tma(const __grid_constant__ CUtensorMap xmap, int64_t alen, int64_t lanes,
                    T* __restrict__ out, uint32_t* err, Seed seed) {
  constexpr int TB = COLS ? col_rows<T>() : 128 / (int)sizeof(T);  // axis positions per tile
  constexpr int S = kScanStages;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kTileBytes * S);
  __shared__ int abort_flag;

  const int t = threadIdx.x;
  const int64_t l0 = (int64_t)blockIdx.x * kLanesPerCta;
  // a thread past the last lane folds lane 0's data (and discards it)
  // rather than the box's zero fill, which would send the max / min chains
  // to the ordered path on every tile
  const int tl = l0 + t < lanes ? t : 0;
  const int32_t batch = blockIdx.y;
  const int64_t n_tiles = (alen + TB - 1) / TB;
  auto load = [&](int s, int64_t tile) {
    mbar_arrive_expect_tx(&full[s], kTileBytes);
    if (COLS)
      tma_load_3d(smem + s * kTileBytes, &xmap, &full[s], (int32_t)l0, (int32_t)(tile * TB), batch);
    else
      tma_load_3d(smem + s * kTileBytes, &xmap, &full[s], (int32_t)(tile * TB), (int32_t)l0, batch);
  };

  if (t == 0) {
    prefetch_tensormap(&xmap);
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  if (t == 0)
    for (int s = 0; s < S && s < n_tiles; ++s) load(s, s);
  T acc = seed.get<T>();
  int64_t it = 0;
  for (; it < n_tiles; ++it) {
    const int s = (int)(it % S);
    if (!mbar_wait_bounded(&full[s], (uint32_t)((it / S) & 1), NRS_WAIT_LIMIT)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) break;
    const int cnt = (int)((alen - it * TB) < TB ? (alen - it * TB) : TB);
    const bool first = (it == 0) && seed.first;
    if (COLS)
      acc = fold_col<T, OP, false>(reinterpret_cast<T*>(smem + s * kTileBytes), tl, cnt, first, acc);
    else
      acc = fold_row<T, OP, false>(smem + s * kTileBytes, tl, cnt, first, acc);
    __syncthreads();  // every thread is done with stage s
    if (t == 0 && it + S < n_tiles) load(s, it + S);
  }
  if (abort_flag) {
    if (t == 0) {
      atomicOr(err, NRS_DEVERR_REDUCE_TMA | ((COLS ? 3u : 4u) << 8));
      for (int64_t j = it; j < n_tiles && j < it + S; ++j)
        mbar_wait_bounded(&full[j % S], (uint32_t)((j / S) & 1), NRS_WAIT_LIMIT);
    }
    return;
  }
  const int64_t lane = l0 + t;
  if (lane < lanes) out[(int64_t)batch * lanes + lane] = acc;
}

// Running fold (accumulate) with warp-specialised roles, 96 threads:
//  * warps 0-1 (consumers), thread t owns lane l0 + t: wait for the stage,
//    rewrite its column / row with the prefix values, fence the writes for
//    the TMA (async) proxy and arrive on `done[s]`;
//  * warp 2, lane 0 (producer): keeps the ring full, TMA-stores each stage
//    once `done[s]` completes (positions outside the array are clipped by
//    the store) and refills a buffer only when its store has finished
//    reading it: after committing the store of stage i it waits until at
//    most LAG stores are still reading, then reloads the buffer of stage
//    i - LAG with stage i - LAG + S.
// A stage holds A consecutive 8 KB tiles along the axis (one barrier pair),
// so a row segment moved per stage is A x 128 B for lanes along rows.
// Every wait is bounded; a give-up sets the shared abort flag and the error
// word, and the producer drains its outstanding copies before returning.
// Ring shape (compile-time; measured on 16384^2 f32/f64 cumsum along both
// axes): 3 stages of 4 tiles (96 KB, two CTAs per SM), store lag 1. Deeper
// rings of single tiles, or a longer lag, were slower or no faster.
#ifndef NRS_RUN_STAGES
#define NRS_RUN_STAGES 3
#endif
#ifndef NRS_RUN_TILES_PER_STAGE
#define NRS_RUN_TILES_PER_STAGE 4
#endif
#ifndef NRS_RUN_STORE_LAG
#define NRS_RUN_STORE_LAG 1
#endif
constexpr int kRunStages = NRS_RUN_STAGES;
constexpr int kRunTiles = NRS_RUN_TILES_PER_STAGE;
constexpr int kStoreLag = NRS_RUN_STORE_LAG;
static_assert(kStoreLag >= 0 && kStoreLag < kRunStages, "the ring must run ahead of the store lag");

template <typename T, int OP, bool COLS>
__global__ void __launch_bounds__(96)
    lane_running_tma(const __grid_constant__ CUtensorMap xmap,
                     const __grid_constant__ CUtensorMap omap, int64_t alen, uint32_t* err,
                     Seed seed) {
  constexpr int TB = COLS ? col_rows<T>() : 128 / (int)sizeof(T);  // axis positions per tile
  constexpr int S = kRunStages;
  constexpr int A = kRunTiles;
  constexpr int STAGE = A * kTileBytes;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGE * S);
  uint64_t* done = full + S;
  __shared__ volatile int abort_flag;

  const int t = threadIdx.x;
  const int64_t l0 = (int64_t)blockIdx.x * kLanesPerCta;
  const int32_t batch = blockIdx.y;
  const int64_t n_tiles = (alen + TB - 1) / TB;       // 8 KB tiles along the axis
  const int64_t n_stages = (n_tiles + A - 1) / A;      // ring steps
  // tiles of step i inside the array
  auto tiles_in = [&](int64_t i) { return (int)((n_tiles - i * A) < A ? (n_tiles - i * A) : A); };
  auto xy = [&](int64_t tile, int32_t* x, int32_t* y) {
    if (COLS) {
      *x = (int32_t)l0;
      *y = (int32_t)(tile * TB);
    } else {
      *x = (int32_t)(tile * TB);
      *y = (int32_t)l0;
    }
  };

  if (t == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&done[s], kLanesPerCta);
    }
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();

  if (t >= kLanesPerCta) {  // producer warp
    if (t != kLanesPerCta) return;
    prefetch_tensormap(&xmap);
    prefetch_tensormap(&omap);
    auto load = [&](int s, int64_t i) {
      const int na = tiles_in(i);
      mbar_arrive_expect_tx(&full[s], (uint32_t)(na * kTileBytes));
      for (int a = 0; a < na; ++a) {
        int32_t x, y;
        xy(i * A + a, &x, &y);
        tma_load_3d(smem + s * STAGE + a * kTileBytes, &xmap, &full[s], x, y, batch);
      }
    };
    int64_t issued = 0;
    for (; issued < S && issued < n_stages; ++issued) load((int)issued, issued);
    bool ok = true;
    for (int64_t i = 0; i < n_stages; ++i) {
      const int s = (int)(i % S);
      if (abort_flag || !mbar_wait_bounded(&done[s], (uint32_t)((i / S) & 1), NRS_WAIT_LIMIT)) {
        ok = false;
        break;
      }
      const int na = tiles_in(i);
      for (int a = 0; a < na; ++a) {
        int32_t x, y;
        xy(i * A + a, &x, &y);
        tma_store_3d(&omap, smem + s * STAGE + a * kTileBytes, x, y, batch);
      }
      bulk_commit();
      const int64_t r = i - kStoreLag;  // its store has now finished reading
      if (r >= 0 && r + S < n_stages) {
        bulk_wait_read<kStoreLag>();
        load((int)(r % S), r + S);
        issued = r + S + 1;
      }
    }
    if (!ok) {
      abort_flag = 1;
      atomicOr(err, NRS_DEVERR_REDUCE_TMA | ((COLS ? 5u : 6u) << 8));
      // Loads issued into the ring: steps issued - S .. issued - 1.
      for (int64_t j = (issued > S ? issued - S : 0); j < issued; ++j)
        mbar_wait_bounded(&full[j % S], (uint32_t)((j / S) & 1), NRS_WAIT_LIMIT);
    }
    bulk_wait<0>();
    return;
  }

  // consumers
  T acc = seed.get<T>();
  for (int64_t i = 0; i < n_stages; ++i) {
    const int s = (int)(i % S);
    if (abort_flag || !mbar_wait_bounded(&full[s], (uint32_t)((i / S) & 1), NRS_WAIT_LIMIT)) {
      abort_flag = 1;
      return;
    }
    const int na = tiles_in(i);
    for (int a = 0; a < na; ++a) {
      const int64_t tile = i * A + a;
      const int cnt = (int)((alen - tile * TB) < TB ? (alen - tile * TB) : TB);
      const bool first = (tile == 0) && seed.first;
      uint8_t* base = smem + s * STAGE + a * kTileBytes;
      if (COLS)
        acc = fold_col<T, OP, true>(reinterpret_cast<T*>(base), t, cnt, first, acc);
      else
        acc = fold_row<T, OP, true>(base, t, cnt, first, acc);
    }
    fence_proxy_async_smem();
    mbar_arrive(&done[s]);
  }
}

// Running fold along rows whose positions are contiguous (axis stride 1) and
// 16-byte aligned: each stage holds kRowSegBytes of up to kRowLanes rows,
// moved per row by untiled bulk copies (one contiguous request per row and
// stage, where the tiled form issues 128-byte box rows), into rows padded to
// kRowSegBytes + 16 bytes so that thread t's 16-byte reads of its own row hit
// distinct banks across each quarter warp. The last warp moves data (lane i:
// rows i, i + 32, ...), the others fold (thread t: row t). The rows per CTA
// are chosen at launch so the CTAs fill whole waves. Waits are bounded as in
// lane_running_tma.
#ifndef NRS_ROW_SEG_BYTES
#define NRS_ROW_SEG_BYTES 1024
#endif
#ifndef NRS_ROW_STAGES
#define NRS_ROW_STAGES 3
#endif
#ifndef NRS_ROW_LANES
#define NRS_ROW_LANES 32
#endif
constexpr int kRowSegBytes = NRS_ROW_SEG_BYTES;
constexpr int kRowPitch = kRowSegBytes + 16;
constexpr int kRowStages = NRS_ROW_STAGES;
constexpr int kRowLanes = NRS_ROW_LANES;  // most rows per CTA, one folding thread each
constexpr size_t row_smem(int rows) { return (size_t)rows * kRowPitch * kRowStages + 16 * kRowStages + 16; }
static_assert(kRowSegBytes % 128 == 0, "segments are whole 128-byte blocks");
static_assert(kRowLanes % 32 == 0, "whole folding warps");
static_assert(kStoreLag < kRowStages, "the ring must run ahead of the store lag");

// Folds `cnt` staged values of one padded row in place (prefix values).
template <typename T, int OP>
NRS_DEV T fold_seg(uint8_t* row, int cnt, bool first, T acc) {
  constexpr int SUB = 128 / (int)sizeof(T);
  constexpr int PER16 = 16 / (int)sizeof(T);
#pragma unroll 1
  for (int b = 0; b < kRowSegBytes / 128; ++b) {
    const int c = cnt - b * SUB;
    if (c <= 0) break;
    uint8_t* blk = row + b * 128;
    const bool f = first && b == 0;
    if (c >= SUB) {
      T v[SUB];
#pragma unroll
      for (int j = 0; j < 8; ++j) lds16(&v[j * PER16], blk + 16 * j);
      acc = run_block<T, OP, SUB>(v, f, acc);
#pragma unroll
      for (int j = 0; j < 8; ++j) sts16(blk + 16 * j, &v[j * PER16]);
    } else {  // the row's last, short block: element by element in place
      T* pv = reinterpret_cast<T*>(blk);
      for (int e = 0; e < c; ++e) {
        acc = (e == 0 && f) ? pv[0] : apply<T, OP>(acc, pv[e]);
        pv[e] = acc;
      }
    }
  }
  return acc;
}

template <typename T, int OP>
__global__ void __launch_bounds__(kRowLanes + 32)
    lane_running_rows(const T* __restrict__ x, T* __restrict__ out, int64_t alen, int64_t lanes,
                      int64_t lstride, int64_t bstride, int rows_per_cta, uint32_t* err, Seed seed) {
  constexpr int S = kRowStages;
  const int stage_bytes = rows_per_cta * kRowPitch;
  constexpr int SEG = kRowSegBytes / (int)sizeof(T);  // positions per stage
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 15) & ~uintptr_t(15));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)stage_bytes * S);
  uint64_t* done = full + S;
  __shared__ volatile int abort_flag;

  const int t = threadIdx.x;
  const int64_t l0 = (int64_t)blockIdx.x * rows_per_cta;
  const int nrows = (int)((lanes - l0) < rows_per_cta ? (lanes - l0) : rows_per_cta);
  const int64_t off0 = (int64_t)blockIdx.y * bstride + l0 * lstride;
  const int64_t n_stages = (alen + SEG - 1) / SEG;
  auto seg_bytes = [&](int64_t i) {
    const int64_t left = alen - i * SEG;
    return (uint32_t)((left < SEG ? left : SEG) * (int64_t)sizeof(T));
  };

  if (t == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&done[s], kRowLanes);
    }
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();

  if (t >= kRowLanes) {  // producer warp
    const int lane = t - kRowLanes;
    auto load = [&](int s, int64_t i) {
      const uint32_t bytes = seg_bytes(i);
      if (lane == 0) mbar_arrive_expect_tx(&full[s], bytes * (uint32_t)nrows);
      __syncwarp();
      for (int r = lane; r < nrows; r += 32)
        bulk_load(smem + (size_t)s * stage_bytes + r * kRowPitch, x + off0 + r * lstride + i * SEG, bytes,
                  &full[s]);
    };
    int64_t issued = 0;
    for (; issued < S && issued < n_stages; ++issued) load((int)issued, issued);
    bool ok = true;
    for (int64_t i = 0; i < n_stages; ++i) {
      const int s = (int)(i % S);
      const bool got = !abort_flag && mbar_wait_bounded(&done[s], (uint32_t)((i / S) & 1), NRS_WAIT_LIMIT);
      if (!__all_sync(0xffffffffu, got)) {
        ok = false;
        break;
      }
      const uint32_t bytes = seg_bytes(i);
      for (int r = lane; r < nrows; r += 32)
        bulk_store(out + off0 + r * lstride + i * SEG, smem + (size_t)s * stage_bytes + r * kRowPitch, bytes);
      bulk_commit();
      const int64_t q = i - kStoreLag;  // its stores have now finished reading
      if (q >= 0 && q + S < n_stages) {
        bulk_wait_read<kStoreLag>();
        __syncwarp();
        load((int)(q % S), q + S);
        issued = q + S + 1;
      }
    }
    if (!ok) {
      if (lane == 0) {
        abort_flag = 1;
        atomicOr(err, NRS_DEVERR_REDUCE_TMA | (7u << 8));
      }
      // Loads issued into the ring: steps issued - S .. issued - 1.
      for (int64_t j = (issued > S ? issued - S : 0); j < issued; ++j)
        mbar_wait_bounded(&full[j % S], (uint32_t)((j / S) & 1), NRS_WAIT_LIMIT);
    }
    bulk_wait<0>();
    return;
  }

  // consumers: every thread takes every step (rows past the array only
  // arrive), so each phase of done[] counts exactly one arrival per thread
  T acc = seed.get<T>();
  uint8_t* myrow = smem + t * kRowPitch;
  for (int64_t i = 0; i < n_stages; ++i) {
    const int s = (int)(i % S);
    if (abort_flag || !mbar_wait_bounded(&full[s], (uint32_t)((i / S) & 1), NRS_WAIT_LIMIT)) {
      abort_flag = 1;
      return;
    }
    if (t < nrows) {
      const int cnt = (int)((alen - i * SEG) < SEG ? (alen - i * SEG) : SEG);
      acc = fold_seg<T, OP>(myrow + (size_t)s * stage_bytes, cnt, i == 0 && seed.first, acc);
    }
    fence_proxy_async_smem();
    mbar_arrive(&done[s]);
  }
}

// ---------------------------------------------------------------------------
// Flat scans (order-free ops)
// ---------------------------------------------------------------------------
// A block takes one chunk; warp w takes its sub-chunk as R rounds of 32
// consecutive elements (coalesced), held in registers: R = 32 for 4-byte
// types (8192-element chunks), 16 for 8-byte ones (4096). Every combine
// keeps the earlier operand on the left.
constexpr int kScanWarps = 8;
template <typename T>
constexpr int rounds_of() { return sizeof(T) == 4 ? 32 : 16; }
template <typename T>
constexpr int64_t flat_chunk() { return 32 * rounds_of<T>() * kScanWarps; }

template <typename T, int OP>
NRS_DEV T warp_inclusive(T v, int lane) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const T o = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v = apply<T, OP>(o, v);
  }
  return v;
}

// Loads the warp's rounds (identity past n), scans each round in place, and
// returns the warp total (the rounds' totals folded in order).
template <typename T, int OP>
NRS_DEV T warp_rounds(const T* __restrict__ x, int64_t wbase, int64_t n, int lane,
                      T (&v)[rounds_of<T>()]) {
  constexpr int kRounds = rounds_of<T>();
#pragma unroll
  for (int k = 0; k < kRounds; ++k) {
    const int64_t i = wbase + k * 32 + lane;
    v[k] = i < n ? x[i] : identity<T, OP>();
  }
#pragma unroll
  for (int k = 0; k < kRounds; ++k) v[k] = warp_inclusive<T, OP>(v[k], lane);
  T run = identity<T, OP>();
#pragma unroll
  for (int k = 0; k < kRounds; ++k) run = apply<T, OP>(run, __shfl_sync(0xffffffffu, v[k], 31));
  return run;
}

// Phase 1: the ordered total of every chunk.
template <typename T, int OP>
__global__ void __launch_bounds__(256)
    flat_chunk_totals(const T* __restrict__ x, int64_t n, T* __restrict__ totals) {
  constexpr int kRounds = rounds_of<T>();
  constexpr int64_t kChunk = flat_chunk<T>();
  __shared__ T wt[kScanWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    T v[kRounds];
    const T tot = warp_rounds<T, OP>(x, c * kChunk + (int64_t)w * 32 * kRounds, n, lane, v);
    if (lane == 0) wt[w] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
      T r = wt[0];
      for (int i = 1; i < kScanWarps; ++i) r = apply<T, OP>(r, wt[i]);
      totals[c] = r;
    }
    __syncthreads();
  }
}

// Phase 2 (one block of 1024): carries[c] = seed (op) totals[0] (op) ...
// (op) totals[c - 1] in order (identity in place of an absent seed); with
// `final_out` set, writes seed (op) all totals there instead.
template <typename T, int OP>
__global__ void __launch_bounds__(1024)
    flat_chunk_carries(const T* __restrict__ totals, int64_t nchunks, int has_seed, Seed seed,
                       T* __restrict__ carries, T* __restrict__ final_out) {
  __shared__ T runs[1024];
  const int t = threadIdx.x;
  const int64_t per = (nchunks + 1023) / 1024;
  const int64_t lo = t * per, hi = (lo + per < nchunks) ? lo + per : nchunks;
  T r = identity<T, OP>();
  for (int64_t i = lo; i < hi; ++i) r = apply<T, OP>(r, totals[i]);
  runs[t] = r;
  __syncthreads();
  if (t == 0) {
    T c = has_seed ? seed.get<T>() : identity<T, OP>();
    for (int i = 0; i < 1024; ++i) {
      const T ri = runs[i];
      runs[i] = c;  // exclusive prefix of run i
      c = apply<T, OP>(c, ri);
    }
    if (final_out) *final_out = c;
  }
  __syncthreads();
  if (final_out) return;
  T c = runs[t];
  for (int64_t i = lo; i < hi; ++i) {
    carries[i] = c;
    c = apply<T, OP>(c, totals[i]);
  }
}

// Phase 3: every element's prefix: the warp's carry, then the earlier
// rounds' totals, then the element's own round prefix.
template <typename T, int OP>
__global__ void __launch_bounds__(256)
    flat_chunk_scan(const T* __restrict__ x, int64_t n, const T* __restrict__ carries,
                    T* __restrict__ out) {
  constexpr int kRounds = rounds_of<T>();
  constexpr int64_t kChunk = flat_chunk<T>();
  __shared__ T wt[kScanWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int64_t wbase = c * kChunk + (int64_t)w * 32 * kRounds;
    T v[kRounds];
    const T tot = warp_rounds<T, OP>(x, wbase, n, lane, v);
    if (lane == 0) wt[w] = tot;
    __syncthreads();
    T run = carries[c];
    for (int i = 0; i < w; ++i) run = apply<T, OP>(run, wt[i]);
#pragma unroll
    for (int k = 0; k < kRounds; ++k) {
      const int64_t i = wbase + k * 32 + lane;
      if (i < n) out[i] = apply<T, OP>(run, v[k]);
      run = apply<T, OP>(run, __shfl_sync(0xffffffffu, v[k], 31));
    }
    __syncthreads();
  }
}

// Flat scans over 16-byte-aligned arrays, as three streaming passes over
// G <= 2 x SMs contiguous segments (each a whole number of CTA tiles):
// seg_totals folds each segment, seg_carries folds the G totals into each
// segment's carry, seg_scan rescans each segment from its carry. A CTA tile
// is kSegWarps warp sub-tiles of kSegRounds rounds of 32 lanes x 16 bytes;
// lane l of round r holds V = 16 / sizeof(T) consecutive elements, scanned in
// the lane, then across the warp (shuffles), then across rounds and warps in
// order. Every combine keeps the earlier operand on the left.
constexpr int kSegWarps = 8;
constexpr int kSegRounds = 8;
template <typename T>
constexpr int64_t seg_tile() { return (int64_t)kSegWarps * kSegRounds * 32 * (16 / (int)sizeof(T)); }

// Loads elements [e, e + V) (identity past `hi`) / stores them (none past `hi`).
template <typename T, int OP>
NRS_DEV void seg_load(const T* __restrict__ x, int64_t e, int64_t hi, T (&v)[16 / sizeof(T)]) {
  constexpr int V = 16 / (int)sizeof(T);
  if (e + V <= hi) {
    const uint4 u = *reinterpret_cast<const uint4*>(x + e);
    memcpy(v, &u, 16);
  } else {
#pragma unroll
    for (int j = 0; j < V; ++j) v[j] = (e + j < hi) ? x[e + j] : identity<T, OP>();
  }
}

// Float maximum / minimum in the segmented scans: values combine without
// NaN checks (ties keep the later operand, as apply does) and a separate
// flag, ORed along the same order, marks every prefix at or after a NaN;
// flagged results are the canonical NaN. Without a NaN this is apply bit for
// bit, and the flag makes the NaN cases so as well. Other ops use apply.
template <typename T, int OP>
constexpr bool seg_flagged() {
  return std::is_floating_point<T>::value && (OP == NRS_OP_MAX || OP == NRS_OP_MIN);
}
template <typename T, int OP>
NRS_DEV T seg_comb(T a, T b) {
  if constexpr (seg_flagged<T, OP>()) return (OP == NRS_OP_MAX ? (a > b) : (a < b)) ? a : b;
  else return apply<T, OP>(a, b);
}

// Segment totals in index order: warp w folds a contiguous run of 512-byte
// rounds (each round: lanes' V elements in order, then an ordered tree over
// the lanes), the warps' totals fold in order. Index order matters for float
// maximum / minimum, whose ties keep the later operand (+0.0 vs -0.0).
template <typename T, int OP>
__global__ void __launch_bounds__(256)
    seg_totals(const T* __restrict__ x, int64_t n, int64_t seg, T* __restrict__ totals) {
  constexpr int V = 16 / (int)sizeof(T);
  constexpr int64_t ROUND = 32 * V;
  __shared__ T wt[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t lo = (int64_t)blockIdx.x * seg;
  const int64_t hi = (lo + seg < n) ? lo + seg : n;
  const int64_t nr = (hi - lo + ROUND - 1) / ROUND;
  const int64_t per = (nr + 7) / 8;
  const int64_t r0 = w * per, r1 = (r0 + per < nr) ? r0 + per : nr;
  constexpr int U = 8;  // rounds loaded before any is folded
  T acc = identity<T, OP>();
  bool nanf = false;
  for (int64_t r = r0; r < r1; r += U) {
    T v[U][V];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (r + u < r1) {
        seg_load<T, OP>(x, lo + (r + u) * ROUND + lane * V, hi, v[u]);
      } else {
#pragma unroll
        for (int j = 0; j < V; ++j) v[u][j] = identity<T, OP>();
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if constexpr (seg_flagged<T, OP>()) {
#pragma unroll
        for (int j = 0; j < V; ++j) nanf |= v[u][j] != v[u][j];
      }
      T s = v[u][0];
#pragma unroll
      for (int j = 1; j < V; ++j) s = seg_comb<T, OP>(s, v[u][j]);
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const T o = __shfl_down_sync(0xffffffffu, s, off);
        if ((lane & (2 * off - 1)) == 0) s = seg_comb<T, OP>(s, o);
      }
      acc = seg_comb<T, OP>(acc, __shfl_sync(0xffffffffu, s, 0));
    }
  }
  if (lane == 0) wt[w] = acc;
  const int anynan = __syncthreads_or(nanf);
  if (threadIdx.x == 0) {
    T r = wt[0];
    for (int i = 1; i < 8; ++i) r = seg_comb<T, OP>(r, wt[i]);
    if constexpr (seg_flagged<T, OP>()) {
      if (anynan) r = qnan<T>();
    }
    totals[blockIdx.x] = r;
  }
}

// carries[g] = seed (op) totals[0] (op) ... (op) totals[g - 1] (identity in
// place of an absent seed); with `final_out`, seed (op) all totals there. One
// warp, g <= 1024: lane l folds the run [l*per, (l+1)*per) in order, an
// ordered warp scan gives each run's carry, then lane l writes its run's.
template <typename T, int OP>
__global__ void __launch_bounds__(32)
    seg_carries(const T* __restrict__ totals, int g, int has_seed, Seed seed,
                T* __restrict__ carries, T* __restrict__ final_out) {
  __shared__ T tot[1024];
  const int lane = threadIdx.x;
  for (int i = lane; i < g; i += 32) tot[i] = totals[i];
  __syncwarp();
  const int per = (g + 31) / 32;
  const int a = lane * per, b = (a + per < g) ? a + per : g;
  T run = identity<T, OP>();
  for (int i = a; i < b; ++i) run = apply<T, OP>(run, tot[i]);
  T inc = run;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const T o = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc = apply<T, OP>(o, inc);
  }
  const T s0 = has_seed ? seed.get<T>() : identity<T, OP>();
  const T ex = __shfl_up_sync(0xffffffffu, inc, 1);
  T c = lane == 0 ? s0 : apply<T, OP>(s0, ex);
  if (final_out) {
    if (lane == 31) *final_out = apply<T, OP>(s0, inc);
    return;
  }
  for (int i = a; i < b; ++i) {
    carries[i] = c;
    c = apply<T, OP>(c, tot[i]);
  }
}

template <typename T, int OP>
__global__ void __launch_bounds__(kSegWarps * 32)
    seg_scan(const T* __restrict__ x, int64_t n, int64_t seg, const T* __restrict__ carries,
             T* __restrict__ out) {
  constexpr int V = 16 / (int)sizeof(T);
  constexpr int R = kSegRounds;
  constexpr int64_t TILE = seg_tile<T>();
  constexpr int64_t SUB = (int64_t)R * 32 * V;  // elements per warp sub-tile
  __shared__ T wt[2][kSegWarps];
  __shared__ int wtf[2][kSegWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t lo = (int64_t)blockIdx.x * seg;
  const int64_t hi = (lo + seg < n) ? lo + seg : n;
  T carry = carries[blockIdx.x];
  int par = 0;
  for (int64_t base = lo; base < hi; base += TILE, par ^= 1) {
    const int64_t sb = base + w * SUB;
    T v[R][V];
#pragma unroll
    for (int r = 0; r < R; ++r) seg_load<T, OP>(x, sb + (int64_t)r * 32 * V + lane * V, hi, v[r]);
    // in-lane prefixes, then the lanes' exclusive prefix and each round's
    // total; with flags (float max / min): a per-element NaN-prefix bit in
    // `lf`, the lanes' exclusive NaN bit and each round's NaN bit
    constexpr bool FL = seg_flagged<T, OP>();
    T ex[R], rt[R];
    uint32_t lf[R], exf = 0, rtf = 0;  // bit j of lf[r]: a NaN at or before element j of the lane
#pragma unroll
    for (int r = 0; r < R; ++r) {
      lf[r] = 0;
      if constexpr (FL) {
        bool f = false;
#pragma unroll
        for (int j = 0; j < V; ++j) {
          f |= v[r][j] != v[r][j];
          lf[r] |= (uint32_t)f << j;
        }
        const uint32_t m = __ballot_sync(0xffffffffu, f);
        exf |= (uint32_t)((m & ((1u << lane) - 1u)) != 0) << r;
        rtf |= (uint32_t)(m != 0) << r;
      }
#pragma unroll
      for (int j = 1; j < V; ++j) v[r][j] = seg_comb<T, OP>(v[r][j - 1], v[r][j]);
      T inc = v[r][V - 1];
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const T o = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc = seg_comb<T, OP>(o, inc);
      }
      rt[r] = __shfl_sync(0xffffffffu, inc, 31);
      const T e = __shfl_up_sync(0xffffffffu, inc, 1);
      ex[r] = lane == 0 ? identity<T, OP>() : e;
    }
    T sub = rt[0];
#pragma unroll
    for (int r = 1; r < R; ++r) sub = seg_comb<T, OP>(sub, rt[r]);
    if (lane == 0) {
      wt[par][w] = sub;
      wtf[par][w] = rtf != 0;
    }
    __syncthreads();
    const bool cf = FL && carry != carry;  // the carry is the canonical NaN once flagged
    T run = carry;
    bool runf = cf;
    for (int i = 0; i < w; ++i) {
      run = seg_comb<T, OP>(run, wt[par][i]);
      runf |= wtf[par][i] != 0;
    }
    T next = carry;
    bool nextf = cf;
#pragma unroll
    for (int i = 0; i < kSegWarps; ++i) {
      next = seg_comb<T, OP>(next, wt[par][i]);
      nextf |= wtf[par][i] != 0;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const T b = lane == 0 ? run : seg_comb<T, OP>(run, ex[r]);
      const bool bf = runf || ((exf >> r) & 1u);
      T o[V];
#pragma unroll
      for (int j = 0; j < V; ++j) {
        o[j] = seg_comb<T, OP>(b, v[r][j]);
        if constexpr (FL) {
          if (bf || ((lf[r] >> j) & 1u)) o[j] = qnan<T>();
        }
      }
      const int64_t e = sb + (int64_t)r * 32 * V + lane * V;
      if (e + V <= hi) {
        uint4 u;
        memcpy(&u, o, 16);
        *reinterpret_cast<uint4*>(out + e) = u;
      } else {
#pragma unroll
        for (int j = 0; j < V; ++j)
          if (e + j < hi) out[e + j] = o[j];
      }
      run = seg_comb<T, OP>(run, rt[r]);
      runf = runf || ((rtf >> r) & 1u);
    }
    carry = next;
    if constexpr (FL) {
      if (nextf) carry = qnan<T>();
    }
  }
}

template <typename T, int OP>
__global__ void seed_combine(T* out, Seed seed) {
  out[0] = apply<T, OP>(seed.get<T>(), out[0]);
}

template <typename T>
__global__ void fill_seed(T* out, int64_t n, Seed seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = seed.get<T>();
}

template <typename T>
__global__ void gather_logical(const T* __restrict__ x, Lanes g, int64_t n, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = i, off = 0;
    for (int d = g.n - 1; d >= 0; --d) {
      off += (rem % g.size[d]) * g.xstride[d];
      rem /= g.size[d];
    }
    y[i] = x[off];
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
CUtensorMapDataType map_dtype(int dtype) {
  switch (dtype) {
    case NRS_F32: return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    case NRS_F64: return CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    case NRS_I32: return CU_TENSOR_MAP_DATA_TYPE_INT32;
    default: return CU_TENSOR_MAP_DATA_TYPE_INT64;
  }
}

bool encode_map(CUtensorMap* map, int dtype, const void* base, const uint64_t dims[3],
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
  return enc(map, map_dtype(dtype), 3, const_cast<void*>(base), dims, strides_bytes, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct LaneProblem {
  int dtype;
  const void* x;
  void* out;
  int64_t alen, xastride, oastride;
  Lanes lanes;
  int64_t n_lanes;
  bool running;
  bool same_layout;  // running fold: output strides equal the input's
  Seed seed;
};

int grid_for(nrs_handle* h, int64_t items, int per_block) {
  const int64_t blocks = (items + per_block - 1) / per_block;
  const int64_t cap = (int64_t)h->num_sms * 16;
  return (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

// TMA lane kernels for (batch, lanes) x axis views; NRS_ERR_UNSUPPORTED when
// the view does not qualify (nothing launched).
template <typename T, int OP, bool RUNNING>
int launch_lane_tma(nrs_handle* h, const LaneProblem& p) {
  const Lanes& k = p.lanes;
  if (k.n < 1 || k.n > 2 || p.alen < 1) return NRS_ERR_UNSUPPORTED;
  if (RUNNING && !p.same_layout) return NRS_ERR_UNSUPPORTED;
  const int es = sizeof(T);
  const int64_t lanes = k.size[k.n - 1], lstride = k.xstride[k.n - 1];
  const int64_t batch = (k.n == 2) ? k.size[0] : 1;
  const int64_t bstride = (k.n == 2) ? k.xstride[0] : 0;
  if (batch > 65535) return NRS_ERR_UNSUPPORTED;
  const size_t smem = (size_t)kTileBytes * kScanStages + 16 * kScanStages + 1024;
  const bool cols = (lstride == 1 && p.xastride > 1);
  const bool rows = (p.xastride == 1 && lstride > 1);
  if (!cols && !rows) return NRS_ERR_UNSUPPORTED;
  // 4-byte rows: bulk-copy ring. 8-byte rows stay on the tiled ring, which
  // keeps twice the rows per SM in flight (their folds were slower with
  // fewer, longer segments: 2.2-2.7 against 3.6 TB/s at 11586^2 f64).
  if (RUNNING && rows && es == 4 && ((uintptr_t)p.x & 15) == 0 && ((uintptr_t)p.out & 15) == 0 &&
      (lstride * es) % 16 == 0 && (bstride * es) % 16 == 0 && (p.alen * es) % 16 == 0) {
    auto kern = lane_running_rows<T, OP>;
    // The attribute belongs to the current device's context: set it on every
    // call (cheap), not once per process.
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem(kRowLanes));
    // CTAs resident per SM for each row count (depends only on the kernel).
    static int per_sm[kRowLanes + 1];
    static std::once_flag once;
    std::call_once(once, [&] {
      for (int r = kRowLanes / 2; r <= kRowLanes; ++r)
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[r], kern, kRowLanes + 32, row_smem(r)) !=
            cudaSuccess)
          per_sm[r] = 0;
    });
    // Rows per CTA: the count whose CTAs best fill whole waves (ties: more
    // rows); within one wave, the count that reaches the most SMs.
    int rows = kRowLanes;
    double best = -1.0;
    for (int r = kRowLanes; r >= kRowLanes / 2; --r) {
      if (per_sm[r] < 1) continue;
      const double ctas = (double)((lanes + r - 1) / r) * (double)batch;
      const double q = ctas / ((double)per_sm[r] * h->num_sms);
      const double eff = q <= 1.0 ? 0.999 * std::fmin(ctas, (double)h->num_sms) / h->num_sms : q / std::ceil(q);
      if (eff > best + 1e-9) {
        best = eff;
        rows = r;
      }
    }
    if (best < 0) return NRS_ERR_UNSUPPORTED;
    dim3 grid((unsigned)((lanes + rows - 1) / rows), (unsigned)batch);
    kern<<<grid, kRowLanes + 32, row_smem(rows), h->stream>>>((const T*)p.x, (T*)p.out, p.alen, lanes, lstride,
                                                              bstride, rows, h->dev_error, p.seed);
    return nrs_after_launch(h, "lane_running_rows");
  }
  uint64_t dims[3], strides[2];
  uint32_t box[3];
  if (cols) {
    dims[0] = (uint64_t)lanes; dims[1] = (uint64_t)p.alen; dims[2] = (uint64_t)batch;
    strides[0] = (uint64_t)p.xastride * es;
    strides[1] = (uint64_t)(batch > 1 ? bstride : p.xastride * p.alen) * es;
    box[0] = kLanesPerCta; box[1] = col_rows<T>(); box[2] = 1;
  } else {
    dims[0] = (uint64_t)p.alen; dims[1] = (uint64_t)lanes; dims[2] = (uint64_t)batch;
    strides[0] = (uint64_t)lstride * es;
    strides[1] = (uint64_t)(batch > 1 ? bstride : lstride * lanes) * es;
    box[0] = 128 / es; box[1] = kLanesPerCta; box[2] = 1;
  }
  const CUtensorMapSwizzle sw = cols ? CU_TENSOR_MAP_SWIZZLE_NONE : CU_TENSOR_MAP_SWIZZLE_128B;
  CUtensorMap xmap, omap;
  if (!encode_map(&xmap, p.dtype, p.x, dims, strides, box, sw)) return NRS_ERR_UNSUPPORTED;
  if (RUNNING && !encode_map(&omap, p.dtype, p.out, dims, strides, box, sw)) return NRS_ERR_UNSUPPORTED;
  dim3 grid((unsigned)((lanes + kLanesPerCta - 1) / kLanesPerCta), (unsigned)batch);
  if (RUNNING) {
    const size_t rsmem = (size_t)kTileBytes * kRunTiles * kRunStages + 16 * kRunStages + 1024;
    auto kern = cols ? lane_running_tma<T, OP, true> : lane_running_tma<T, OP, false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem);
    kern<<<grid, 96, rsmem, h->stream>>>(xmap, omap, p.alen, h->dev_error, p.seed);
    return nrs_after_launch(h, "lane_running_tma");
  }
  auto kern = cols ? lane_reduce_tma<T, OP, true> : lane_reduce_tma<T, OP, false>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kern<<<grid, kLanesPerCta, smem, h->stream>>>(xmap, p.alen, lanes, (T*)p.out, h->dev_error, p.seed);
  return nrs_after_launch(h, "lane_reduce_tma");
}

template <typename T, int OP, bool RUNNING>
int launch_lanes(nrs_handle* h, const LaneProblem& p) {
  if (p.alen >= 256 && p.n_lanes >= 64) {
    const int st = launch_lane_tma<T, OP, RUNNING>(h, p);
    if (st != NRS_ERR_UNSUPPORTED) return st;
  }
  lane_scan_generic<T, OP, RUNNING><<<grid_for(h, p.n_lanes, 256), 256, 0, h->stream>>>(
      (const T*)p.x, p.lanes, p.n_lanes, p.alen, p.xastride, (T*)p.out, p.oastride, p.seed);
  return nrs_after_launch(h, "lane_scan_generic");
}

template <typename T>
int lanes_by_op(nrs_handle* h, int op, const LaneProblem& p) {
#define NRS_LANE_CASE(OPC)                                                          \
  case OPC:                                                                         \
    return p.running ? launch_lanes<T, OPC, true>(h, p) : launch_lanes<T, OPC, false>(h, p);
  switch (op) {
    NRS_LANE_CASE(NRS_OP_ADD)
    NRS_LANE_CASE(NRS_OP_SUB)
    NRS_LANE_CASE(NRS_OP_MUL)
    NRS_LANE_CASE(NRS_OP_MAX)
    NRS_LANE_CASE(NRS_OP_MIN)
    default:
      if constexpr (std::is_floating_point<T>::value) {
        return p.running ? launch_lanes<T, NRS_OP_DIV, true>(h, p) : launch_lanes<T, NRS_OP_DIV, false>(h, p);
      } else {
        return nrs_fail(h, NRS_ERR_DTYPE, "integer divide has no ufunc reduce/accumulate");
      }
  }
#undef NRS_LANE_CASE
}

int run_lanes(nrs_handle* h, int op, const LaneProblem& p) {
  switch (p.dtype) {
    case NRS_F32: return lanes_by_op<float>(h, op, p);
    case NRS_F64: return lanes_by_op<double>(h, op, p);
    case NRS_I64: return lanes_by_op<int64_t>(h, op, p);
    default: return lanes_by_op<int32_t>(h, op, p);
  }
}

// Flat reduce-then-scan over a contiguous buffer. `final_out` set: only the
// seeded total is written there (reduce); otherwise out[0..n) gets every
// prefix (accumulate).
template <typename T, int OP>
int flat_scan_t(nrs_handle* h, const T* x, int64_t n, int has_seed, Seed seed, T* out,
                T* final_out) {
  const int64_t nchunks = (n + flat_chunk<T>() - 1) / flat_chunk<T>();
  int st;
  T* ws = (T*)nrs_workspace(h, (size_t)(2 * nchunks + 2) * sizeof(T) + 256, &st);
  if (!ws) return st;
  T* totals = ws;
  T* carries = ws + nchunks + 1;
  if ((reinterpret_cast<uintptr_t>(x) & 15) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
    // Segments: a whole number of tiles each, at most two per SM of the
    // planning SM count (the segments decide the float rounding, so they do
    // not follow the device or the handle's SM budget).
    const int64_t tiles = (n + seg_tile<T>() - 1) / seg_tile<T>();
    const int64_t gmax = (int64_t)NRS_PLAN_SMS * 2 < 1024 ? (int64_t)NRS_PLAN_SMS * 2 : 1024;
    const int64_t seg = ((tiles + gmax - 1) / gmax) * seg_tile<T>();
    const int g = (int)((n + seg - 1) / seg);
    seg_totals<T, OP><<<g, 256, 0, h->stream>>>(x, n, seg, totals);
    seg_carries<T, OP><<<1, 32, 0, h->stream>>>(totals, g, has_seed, seed, carries, final_out);
    if (!final_out) seg_scan<T, OP><<<g, kSegWarps * 32, 0, h->stream>>>(x, n, seg, carries, out);
    return nrs_after_launch(h, "flat scan");
  }
  const int grid = (int)(nchunks < (int64_t)h->num_sms * 8 ? nchunks : (int64_t)h->num_sms * 8);
  flat_chunk_totals<T, OP><<<grid, 256, 0, h->stream>>>(x, n, totals);
  flat_chunk_carries<T, OP><<<1, 1024, 0, h->stream>>>(totals, nchunks, has_seed, seed, carries, final_out);
  if (!final_out) flat_chunk_scan<T, OP><<<grid, 256, 0, h->stream>>>(x, n, carries, out);
  return nrs_after_launch(h, "flat scan");
}

template <typename T>
int flat_scan(nrs_handle* h, int op, const T* x, int64_t n, int has_seed, Seed seed, T* out,
              T* final_out) {
  switch (op) {
    case NRS_OP_ADD: return flat_scan_t<T, NRS_OP_ADD>(h, x, n, has_seed, seed, out, final_out);
    case NRS_OP_MUL: return flat_scan_t<T, NRS_OP_MUL>(h, x, n, has_seed, seed, out, final_out);
    case NRS_OP_MAX: return flat_scan_t<T, NRS_OP_MAX>(h, x, n, has_seed, seed, out, final_out);
    default: return flat_scan_t<T, NRS_OP_MIN>(h, x, n, has_seed, seed, out, final_out);
  }
}

int flat_scan_dtype(nrs_handle* h, int dtype, int op, const void* x, int64_t n, int has_seed, Seed seed,
                    void* out, void* final_out) {
  switch (dtype) {
    case NRS_F32: return flat_scan<float>(h, op, (const float*)x, n, has_seed, seed, (float*)out, (float*)final_out);
    case NRS_F64: return flat_scan<double>(h, op, (const double*)x, n, has_seed, seed, (double*)out, (double*)final_out);
    case NRS_I64: return flat_scan<int64_t>(h, op, (const int64_t*)x, n, has_seed, seed, (int64_t*)out, (int64_t*)final_out);
    default: return flat_scan<int32_t>(h, op, (const int32_t*)x, n, has_seed, seed, (int32_t*)out, (int32_t*)final_out);
  }
}

bool valid_op(int op) {
  return op == NRS_OP_ADD || op == NRS_OP_SUB || op == NRS_OP_MUL || op == NRS_OP_DIV ||
         op == NRS_OP_MAX || op == NRS_OP_MIN;
}

const char* op_name(int op) {
  switch (op) {
    case NRS_OP_ADD: return "add";
    case NRS_OP_SUB: return "subtract";
    case NRS_OP_MUL: return "multiply";
    case NRS_OP_DIV: return "divide";
    case NRS_OP_MAX: return "maximum";
    default: return "minimum";
  }
}

Seed seed_from(int dtype, const void* value) {
  Seed s{};
  s.first = 0;
  switch (dtype) {
    case NRS_F32: s.fseed = *(const float*)value; break;
    case NRS_F64: s.fseed = *(const double*)value; break;
    case NRS_I64: s.iseed = *(const int64_t*)value; break;
    default: s.iseed = *(const int32_t*)value; break;
  }
  return s;
}

Seed seed_const(double v) {
  Seed s{};
  s.first = 0;
  s.fseed = v;
  s.iseed = (int64_t)v;
  return s;
}

Seed seed_first() {
  Seed s{};
  s.first = 1;
  return s;
}

// Shared validation and the gather of a non-contiguous view into logical
// order (kernels::borrow::operand, src/kernels/borrow.rs:59).
struct View {
  int64_t total = 1;
  bool contig = true;
  Lanes all{};
};

int check_view(nrs_handle* h, int dtype, int op, int ndim, const int64_t* shape,
               const int64_t* strides, View* v) {
  if (ndim < 0 || ndim > kMaxDims || (ndim > 0 && (!shape || !strides)))
    return nrs_fail(h, NRS_ERR_INVALID, "bad ndim/shape/strides");
  if (!valid_op(op)) return nrs_fail(h, NRS_ERR_INVALID, "unknown ufunc op");
  if (!nrs_dtype_size(dtype)) return nrs_fail(h, NRS_ERR_DTYPE, "unknown dtype");
  if (op == NRS_OP_DIV && (dtype == NRS_I32 || dtype == NRS_I64))
    return nrs_fail(h, NRS_ERR_DTYPE, "integer divide has no ufunc reduce/accumulate");
  int64_t expect = 1;
  v->all.n = ndim;
  for (int d = ndim - 1; d >= 0; --d) {
    if (shape[d] < 0) return nrs_fail(h, NRS_ERR_SHAPE, "negative dimension");
    if (strides[d] < 0) return nrs_fail(h, NRS_ERR_STRIDE, "negative stride");
    if (shape[d] != 1 && strides[d] != expect) v->contig = false;
    expect *= shape[d];
    v->total *= shape[d];
    v->all.size[d] = shape[d];
    v->all.xstride[d] = strides[d];
  }
  return NRS_OK;
}

// Contiguous logical-order copy of a view in workspace, past `reserve` bytes.
int gathered(nrs_handle* h, int dtype, const void* x, const View& v, size_t reserve, const void** src) {
  if (v.contig || v.total == 0) {
    *src = x;
    return NRS_OK;
  }
  const size_t es = nrs_dtype_size(dtype);
  int st;
  uint8_t* ws = (uint8_t*)nrs_workspace(h, reserve + (size_t)v.total * es, &st);
  if (!ws) return st;
  void* dst = ws + reserve;
  const int grid = h->num_sms * 8;
  if (es == 4) gather_logical<uint32_t><<<grid, 256, 0, h->stream>>>((const uint32_t*)x, v.all, v.total, (uint32_t*)dst);
  else gather_logical<uint64_t><<<grid, 256, 0, h->stream>>>((const uint64_t*)x, v.all, v.total, (uint64_t*)dst);
  if ((st = nrs_after_launch(h, "gather_logical"))) return st;
  *src = dst;
  return NRS_OK;
}

int fill(nrs_handle* h, int dtype, void* out, int64_t n, Seed s) {
  const int grid = grid_for(h, n, 256);
  switch (dtype) {
    case NRS_F32: fill_seed<float><<<grid, 256, 0, h->stream>>>((float*)out, n, s); break;
    case NRS_F64: fill_seed<double><<<grid, 256, 0, h->stream>>>((double*)out, n, s); break;
    case NRS_I64: fill_seed<int64_t><<<grid, 256, 0, h->stream>>>((int64_t*)out, n, s); break;
    default: fill_seed<int32_t><<<grid, 256, 0, h->stream>>>((int32_t*)out, n, s); break;
  }
  return nrs_after_launch(h, "fill_seed");
}

template <int OP>
int seed_combine_dtype(nrs_handle* h, int dtype, void* out, Seed s) {
  switch (dtype) {
    case NRS_F32: seed_combine<float, OP><<<1, 1, 0, h->stream>>>((float*)out, s); break;
    case NRS_F64: seed_combine<double, OP><<<1, 1, 0, h->stream>>>((double*)out, s); break;
    case NRS_I64: seed_combine<int64_t, OP><<<1, 1, 0, h->stream>>>((int64_t*)out, s); break;
    default: seed_combine<int32_t, OP><<<1, 1, 0, h->stream>>>((int32_t*)out, s); break;
  }
  return nrs_after_launch(h, "seed_combine");
}

// Normalises `axis` and builds the lane problem: kept dims collapsed outer
// to inner where both the input's and the output's strides allow.
int lane_problem(nrs_handle* h, int ndim, const int64_t* shape, const int64_t* strides, int64_t axis,
                 const int64_t* out_strides, LaneProblem* p, int* ax_out) {
  if (ndim == 0) return nrs_fail(h, NRS_ERR_AXIS, "axis given for a 0-d array");
  const int64_t ax = axis < 0 ? axis + ndim : axis;
  if (ax < 0 || ax >= ndim)
    return nrs_fail(h, NRS_ERR_AXIS, "axis " + std::to_string(axis) +
                                         " out of bounds for array of dimension " +
                                         std::to_string(ndim));
  *ax_out = (int)ax;
  p->alen = shape[ax];
  p->xastride = strides[ax];
  p->oastride = out_strides ? out_strides[ax] : 0;
  Lanes& k = p->lanes;
  k.n = 0;
  p->n_lanes = 1;
  p->same_layout = true;
  for (int d = 0; d < ndim; ++d) {
    const int64_t os = out_strides ? out_strides[d] : 0;
    if (out_strides && shape[d] != 1 && os != strides[d]) p->same_layout = false;
    if (d == ax) continue;
    p->n_lanes *= shape[d];
    if (shape[d] == 1) continue;
    if (k.n > 0 && k.xstride[k.n - 1] == strides[d] * shape[d] &&
        k.ostride[k.n - 1] == os * shape[d]) {
      k.size[k.n - 1] *= shape[d];
      k.xstride[k.n - 1] = strides[d];
      k.ostride[k.n - 1] = os;
    } else {
      k.size[k.n] = shape[d];
      k.xstride[k.n] = strides[d];
      k.ostride[k.n] = os;
      k.n++;
    }
  }
  // A reduction writes lane o at out[o]: row-major kept dims.
  if (!out_strides) {
    int64_t c = 1;
    for (int d = k.n - 1; d >= 0; --d) {
      k.ostride[d] = c;
      c *= k.size[d];
    }
  }
  return NRS_OK;
}

}  // namespace

extern "C" int nrs_ufunc_reduce(nrs_handle* h, int dtype, int op, int ndim, const int64_t* shape,
                                const int64_t* strides, int64_t axis, const void* initial,
                                const void* x, void* out) {
  if (!h) return NRS_ERR_INVALID;
  h->last_error.clear();
  View v;
  int st = check_view(h, dtype, op, ndim, shape, strides, &v);
  if (st) return st;
  if (v.total > 0 && !x) return nrs_fail(h, NRS_ERR_INVALID, "null input");
  if ((st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice"))) return st;
  const bool has_init = initial != nullptr;
  const std::string no_identity =
      std::string("zero-size array to reduction operation ") + op_name(op) + " which has no identity";

  if (axis == NRS_AXIS_NONE) {
    if (!out) return nrs_fail(h, NRS_ERR_INVALID, "null output");
    // reduce_full: add / multiply are seed (op) the tiered flat sum / product.
    if (op == NRS_OP_ADD || op == NRS_OP_MUL) {
      const int64_t one = 1;
      const int64_t* shp = ndim ? shape : &one;
      const int64_t* strd = ndim ? strides : &one;
      if ((st = nrs_reduce(h, dtype, op == NRS_OP_ADD ? NRS_SUM : NRS_PROD, ndim ? ndim : 1, shp, strd,
                           NRS_AXIS_NONE, 0, x, out)))
        return st;
      const Seed s = has_init ? seed_from(dtype, initial) : seed_const(op == NRS_OP_ADD ? 0.0 : 1.0);
      return op == NRS_OP_ADD ? seed_combine_dtype<NRS_OP_ADD>(h, dtype, out, s)
                              : seed_combine_dtype<NRS_OP_MUL>(h, dtype, out, s);
    }
    if (v.total == 0) {
      if (!has_init) return nrs_fail(h, NRS_ERR_EMPTY, no_identity);
      return fill(h, dtype, out, 1, seed_from(dtype, initial));
    }
    const size_t reserve = (size_t)(2 * (v.total / 4096 + 2)) * 8 + 4096;
    const void* src;
    if ((st = gathered(h, dtype, x, v, reserve, &src))) return st;
    if (op == NRS_OP_MAX || op == NRS_OP_MIN)
      return flat_scan_dtype(h, dtype, op, src, v.total, has_init,
                             has_init ? seed_from(dtype, initial) : seed_const(0.0), nullptr, out);
    // subtract / divide: one serial lane.
    LaneProblem p{};
    p.dtype = dtype;
    p.x = src;
    p.out = out;
    p.alen = v.total;
    p.xastride = 1;
    p.lanes.n = 0;
    p.n_lanes = 1;
    p.running = false;
    p.seed = has_init ? seed_from(dtype, initial) : seed_first();
    return run_lanes(h, op, p);
  }

  LaneProblem p{};
  int ax;
  if ((st = lane_problem(h, ndim, shape, strides, axis, nullptr, &p, &ax))) return st;
  if (p.n_lanes == 0) return NRS_OK;
  if (!out) return nrs_fail(h, NRS_ERR_INVALID, "null output");
  if (p.alen == 0) {
    // reduce_lane on empty lanes: initial, else the identity, else an error.
    if (has_init) return fill(h, dtype, out, p.n_lanes, seed_from(dtype, initial));
    if (op == NRS_OP_ADD || op == NRS_OP_MUL)
      return fill(h, dtype, out, p.n_lanes, seed_const(op == NRS_OP_ADD ? 0.0 : 1.0));
    return nrs_fail(h, NRS_ERR_EMPTY, no_identity);
  }
  p.dtype = dtype;
  p.x = x;
  p.out = out;
  p.running = false;
  p.seed = has_init ? seed_from(dtype, initial) : seed_first();
  return run_lanes(h, op, p);
}

extern "C" int nrs_accumulate(nrs_handle* h, int dtype, int op, int ndim, const int64_t* shape,
                              const int64_t* strides, int64_t axis, const void* x, void* out,
                              const int64_t* out_strides) {
  if (!h) return NRS_ERR_INVALID;
  h->last_error.clear();
  View v;
  int st = check_view(h, dtype, op, ndim, shape, strides, &v);
  if (st) return st;
  if (v.total == 0) {
    if (axis != NRS_AXIS_NONE && ndim > 0) {
      const int64_t ax = axis < 0 ? axis + ndim : axis;
      if (ax < 0 || ax >= ndim)
        return nrs_fail(h, NRS_ERR_AXIS, "axis " + std::to_string(axis) +
                                             " out of bounds for array of dimension " +
                                             std::to_string(ndim));
    }
    return NRS_OK;
  }
  if (!x || !out) return nrs_fail(h, NRS_ERR_INVALID, "null input or output");
  if (out_strides)
    for (int d = 0; d < ndim; ++d)
      if (out_strides[d] < 0) return nrs_fail(h, NRS_ERR_STRIDE, "negative stride");
  if ((st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice"))) return st;
  // cumsum seeds lanes with 0, cumprod with 1; the other ufuncs with the
  // lane's first element.
  const Seed seed = op == NRS_OP_ADD ? seed_const(0.0) : op == NRS_OP_MUL ? seed_const(1.0) : seed_first();

  if (axis == NRS_AXIS_NONE) {
    // Flattened: out is the n values in logical order, contiguous.
    const size_t reserve = (size_t)(2 * (v.total / 4096 + 2)) * 8 + 4096;
    const void* src;
    if ((st = gathered(h, dtype, x, v, reserve, &src))) return st;
    const bool order_free = (op == NRS_OP_ADD || op == NRS_OP_MUL || op == NRS_OP_MAX || op == NRS_OP_MIN);
    if (order_free && v.total >= 64)
      return flat_scan_dtype(h, dtype, op, src, v.total, !seed.first, seed, out, nullptr);
    LaneProblem p{};
    p.dtype = dtype;
    p.x = src;
    p.out = out;
    p.alen = v.total;
    p.xastride = 1;
    p.oastride = 1;
    p.lanes.n = 0;
    p.n_lanes = 1;
    p.running = true;
    p.same_layout = false;
    p.seed = seed;
    return run_lanes(h, op, p);
  }

  int64_t cstr[kMaxDims];
  if (!out_strides) {
    int64_t c = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      cstr[d] = c;
      c *= shape[d];
    }
  }
  LaneProblem p{};
  int ax;
  if ((st = lane_problem(h, ndim, shape, strides, axis, out_strides ? out_strides : cstr, &p, &ax)))
    return st;
  p.dtype = dtype;
  p.x = x;
  p.out = out;
  p.running = true;
  p.seed = seed;
  return run_lanes(h, op, p);
}
