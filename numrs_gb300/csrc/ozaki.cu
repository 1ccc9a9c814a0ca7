// f64-accurate GEMM from BF16 slices on tcgen05 tensor cores (Ozaki scheme).
//
// C = A*B with A (m x k) and B (k x n) row-major f64. No reference
// counterpart: it stands in for the f64 tier of kernels::gemm::gemm_2d
// (src/kernels/gemm.rs:290) where GB300's FP64 rate (~1.2 TFLOP/s) makes a
// native FP64 GEMM slow.
//
// 1. Scaling: e_a[i] = frexp exponent of max_k |a_ik| (|a_ik| < 2^e_a[i]),
//    e_b[j] likewise over column j of B. Powers of two: exact.
// 2. Slicing: x = a_ik * 2^-e_a[i] in (-1, 1) becomes the 126-bit fixed-point
//    integer X = round(x * 2^126), split into S signed b-bit digits
//    (b = 8, 7 or 6: the widest whose exactness bounds below hold for the
//    call's K and S) whose weighted sum is X rounded to the nearest
//    multiple of 2^(127 - b - b(S-1)): each digit lies in [-2^(b-1), 2^(b-1)],
//    exactly representable in BF16, and x = sum_t digit_t * 2^-(b - 1 + bt)
//    up to 2^-(bS). Slices are stored K-major ([S][rows][kpad] bf16) for A
//    and for B^T (the B slicer transposes through shared memory).
// 3. Products: for every slice pair (s, t) with s + t <= S-1 (the pairs
//    whose weight 2^-(2b - 2 + b(s+t)) matters), P = A_s * B_t^T on the
//    tensor cores with FP32 accumulation. |digit products| <= 2^(2b-2), so
//    every partial sum of a K <= 2^(26-2b) chunk (4096 for b = 7) is an
//    integer of at most 2^24: the FP32 accumulation is EXACT.
// 4. Cross-slice accumulation: the exact products of one diagonal
//    (s + t = d) are summed as int32 and carried, from d = S-1 up to d = 0,
//    in one int32 per element: R <- floor(R / 2^b) + D_d, the low b bits of
//    the old R being final (digit S-2-d). After d = 0 the exact total is
//    T = R 2^(b(S-1)) + sum_t digit_t 2^(bt), rounded once to f64 with
//    integer operations (no FP64 op) and scaled by
//    2^(e_a[i] + e_b[j] + 2 - 2b - b(S-1)).
//
// The tensor-core kernel is persistent (one CTA per SM) and warp-specialised:
//   warp 0      : TMA producer, 4-stage ring of A (128x64) + B (256x64) bf16
//                 tiles, 128-byte swizzle;
//   warp 1      : TMEM allocator and single-thread tcgen05.mma issuer,
//                 M=128 N=256 K=16, FP32 accumulator in TMEM columns 0..255;
//   warps 2..9  : epilogue (one TMEM lane = one tile row per thread, two warps
//                 per lane quarter splitting the 256 columns): copy the
//                 finished accumulator to registers, hand it back to the MMA
//                 warp at once, fold the copy into the carried int32 sums R
//                 kept in TMEM columns 256..511, write each retired digit as
//                 a byte of the element's record in a per-CTA slot, and
//                 round every element's exact total once after d = 0.
// Grouped launches (many small problems, one tile list) use 128 x 128 tiles,
// a 6-stage ring and two accumulators in turn, and keep the digits in TMEM
// and registers (the grouped epilogue below describes it).
// Measured at 8192^3 (clock counters per warp): the MMA warp waits for TMA
// data ~29% of its time and for the epilogue ~8%.
// Every mbarrier wait is bounded; on give-up the kernel records an error
// word, drains its own copies and MMAs (bounded), frees TMEM and returns.
#include <mutex>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "f64_round.cuh"
#include "nrs_internal.cuh"

namespace {

constexpr int OZ_BM = 128;
constexpr int OZ_BN = 256;
// K per ring stage: 64 bf16 = one 128-byte swizzle row. (32 per stage with
// the 64-byte swizzle and 9 stages computed the same results but ran 28%
// slower at 8192^3: the per-stage barrier and issue work doubles.)
constexpr int OZ_BK = 64;
constexpr int OZ_STAGES = 4;
constexpr int OZ_A_BYTES = OZ_BM * OZ_BK * 2;  // 16 KB
constexpr int OZ_THREADS = 320;                 // 10 warps: TMA, MMA, 8 epilogue
constexpr int OZ_TMEM_COLS = 512;               // accumulator(s) + diagonal sums
// Signed digits of b bits: |digit| <= 2^(b-1), exact in BF16 (8-bit
// significand) for b <= 8; products <= 2^(2b-2), so a K chunk of 2^(26-2b)
// sums exactly in FP32 (at most 2^24). Wider digits need fewer slices for
// the same precision (S = ceil(54 / b): 7 slices and 28 pairs for b = 8,
// 8 and 36 for b = 7, 9 and 45 for b = 6) but shorter exact K chunks.
constexpr int kChunkOf(int b) { return 1 << (26 - 2 * b); }
constexpr int kTopOf(int b) { return 127 - b; }  // position of the top digit in X
constexpr int OZ_MAX_SLICES = 16;

// Tile geometry per launch kind. One large problem: 128 x 256 tiles, one
// accumulator, 4 stages (the constants above). Grouped launches, mostly
// small problems: 128 x 128 tiles (less padding for narrow problems), two
// accumulators in TMEM columns 0..255 so the MMAs of the next group run
// while the epilogue reads the last one, the diagonal sums in 256..383,
// and 6 stages of 32 KB.
template <bool G>
struct OzGeom {
  static constexpr int BN = G ? 128 : OZ_BN;
  static constexpr int STAGES = G ? 6 : OZ_STAGES;
  static constexpr int B_BYTES = BN * OZ_BK * 2;
  static constexpr int STAGE_BYTES = OZ_A_BYTES + B_BYTES;
  static constexpr int ACC_BUFS = G ? 2 : 1;
  // Grouped epilogue: the column exponents of each epilogue warp's 64 tile
  // columns, staged once per tile.
  static constexpr int EB_BYTES = G ? 8 * 64 * 4 : 0;
  static constexpr int SMEM = STAGES * STAGE_BYTES + EB_BYTES + 1024 /*align*/ + 256 /*barriers*/;
  // Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B bf16
  // (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
  // 17-22, M >> 4 at bits 24-28.
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                    ((uint32_t)(OZ_BM >> 4) << 24);
};
// Grouped launches with S > 9 keep digits 8..14 in a per-CTA 128 x 128 slot
// of 8-byte records (column-major: for one column a warp's 32 rows are 256
// contiguous bytes).
constexpr int OZ_DIGIT_BYTES = 8;


// ---------------------------------------------------------------------------
// tcgen05 / TMEM wrappers
// ---------------------------------------------------------------------------
NRS_DEV void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
NRS_DEV void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
NRS_DEV void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
NRS_DEV void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
NRS_DEV void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

NRS_DEV void tc_mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
NRS_DEV void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns.
NRS_DEV void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 32 lanes x 16 columns into v[0..15] without waiting: several loads can be
// in flight before one tcgen05.wait::ld.
NRS_DEV void tmem_ld16_nowait(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}
// 32 lanes x 8 columns into v[0..7] without waiting.
NRS_DEV void tmem_ld8_nowait(uint32_t taddr, uint32_t* v) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                 "=r"(v[7])
               : "r"(taddr)
               : "memory");
}
NRS_DEV void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

NRS_DEV void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
      "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
      : "memory");
}
NRS_DEV void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor, K-major operand with 128-byte swizzle:
// rows of 128 B, 8-row core-matrix groups 1024 B apart (SBO), descriptor
// version 1 (bits 46-47), swizzle mode 2 = 128B (bits 61-63).
NRS_DEV uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)(16 >> 4) << 16;    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

struct OzParams {
  int64_t m, n, k, kpad;
  int slices;
  int kchunks;
  int n_pairs;     // pairs x kchunks work units per tile
  int tiles_m, tiles_n;
  int group_m;     // tile rasterisation group height
  const int* ea;   // row exponents of A
  const int* eb;   // column exponents of B
  __int128* acc;   // per-CTA digit slots (16-byte aligned)
  double* C;
  int64_t ldc;
  int final_shift; // 2 - 2b - b(S-1) for b-bit digits
  int digit_bits;  // b
  int kchunk;      // exact FP32 K chunk, 2^(26-2b)
  int accumulate;  // C += result instead of C = result
  uint32_t* err;
  // Spread estimate only (EST kernel): row sums of |A'| and column sums of
  // |B'| (operands scaled by their row / column exponents), and the word
  // that collects max_ij of the ratio as float bits.
  const float* ra;
  const float* cb;
  uint32_t* est;
  // Grouped launch only: the tile list and the problems it points into.
  const struct OzTile* tiles;
  const struct OzProb* probs;
  int n_tiles;
};

// One problem of a grouped launch: its slices are rows [rowoff, rowoff + m)
// of the stacked A slices and [coloff, coloff + n) of the stacked B^T slices
// (row pitch = the group's largest kpad; this problem's rows are zero from
// its own k to its kpad), and its exponents sit at the same offsets.
struct OzProb {
  int64_t m, n, kpad;
  int64_t rowoff, coloff;
  void* C;  // double, or float when f32
  int64_t ldc;
  int32_t kchunks, n_pairs;
  int32_t accumulate, f32;
};
struct OzTile {
  int32_t prob, tm, tn, pad;
};

// Everything a CTA needs about the tile it works on.
struct TileCtx {
  int64_t m, n;        // the problem's C dimensions
  int64_t arow, brow;  // TMA row coordinates of the tile's A / B^T boxes
  int64_t row0, col0;  // tile origin inside the problem
  int kblocks, n_pairs, kchunks;
  const int* ea;
  const int* eb;
  void* C;  // double, or float when f32
  int64_t ldc;
  int accumulate, f32;
};

// Work units of a tile, in order: diagonals from the least significant
// (d = S-1) to the most significant (d = 0), within a diagonal the pairs
// (s, t = d - s) for s = 0..d, within a pair its K chunks; the last unit of a
// tile is pair (0,0). Walked incrementally (no search per unit).
struct PairIter {
  int d, s, chunk;
  __device__ __forceinline__ void start(int S) {
    d = S - 1;
    s = 0;
    chunk = 0;
  }
  __device__ __forceinline__ int t() const { return d - s; }
  __device__ __forceinline__ bool diag_first() const { return s == 0 && chunk == 0; }
  // units of the current diagonal from this one on, this one included
  __device__ __forceinline__ int left(int kchunks) const { return (d - s) * kchunks + (kchunks - chunk); }
  __device__ __forceinline__ void next(int kchunks) {
    if (++chunk == kchunks) {
      chunk = 0;
      if (s < d) {
        ++s;
      } else {
        --d;
        s = 0;
      }
    }
  }
};

__device__ __forceinline__ void tile_coords(int tile, const OzParams& P, int& tm, int& tn) {
  // Grouped rasterisation: consecutive tiles walk group_m tile rows before
  // moving along N, so concurrently active tiles share A and B panels in L2.
  const int per_group = P.group_m * P.tiles_n;
  const int g = tile / per_group;
  const int first_m = g * P.group_m;
  const int gm = (P.tiles_m - first_m) < P.group_m ? (P.tiles_m - first_m) : P.group_m;
  const int r = tile % per_group;
  tm = first_m + r % gm;
  tn = r / gm;
}

// Units of a tile that the tensor cores accumulate together. With one K
// chunk (kchunks == 1) consecutive units are consecutive pairs; the pairs of
// one diagonal can share the fp32 accumulator as long as the sum stays an
// exact integer: each pair's sum is at most kblocks * 64 * 2^(2b-2), so up
// to 2^24 / that many pairs. Several K chunks (and the spread estimate)
// keep one unit per accumulation.
__device__ __forceinline__ int merge_count(const TileCtx& c, const OzParams& P, bool est) {
  if (est || c.kchunks != 1) return 1;
  const int64_t per_pair = (int64_t)c.kblocks * OZ_BK << (2 * P.digit_bits - 2);
  const int64_t g = ((int64_t)1 << 24) / per_pair;
  return g < 1 ? 1 : (int)g;
}
// Units in the accumulation group that starts at `pi`: the same diagonal, at
// most `gm` units.
__device__ __forceinline__ int group_size(const PairIter& pi, int gm, int kchunks) {
  const int l = pi.left(kchunks);
  return l < gm ? l : gm;
}


// Writes 8 consecutive columns of one tile row of C (f64, or f32 when F32):
// R values w, digit words per column (S <= 5: digits 0..S-2 in lw; else
// digits 0..3 in lw and 4..7 in hw), digits 8..14 from the 8-byte records
// `pitch` apart (S > 9 only) and the column exponents; `left` of the 8
// columns lie inside the problem; the row starts at element `off` of C. The
// conversions run straight-line for all 8 (interleaved); zero, subnormal and
// overflowing results are redone by the exact path.
template <bool F32>
__device__ __forceinline__ void retire8(const uint32_t (&w)[8], const uint32_t (&lw)[8], const uint32_t (&hw)[8],
                                        const uint8_t* rec, size_t pitch, const int* eb, int left, int b, int S,
                                        int ebase, void* C, int64_t off, bool accumulate) {
  using Fmt = typename std::conditional<F32, NrsF32Fmt, NrsF64Fmt>::type;
  uint64_t hi[8], bits[8];
  int ex[8];
  unsigned special = 0;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    hi[e] = 0;
    ex[e] = 0;
    if (e < left) {
      if (S > 9) hi[e] = __ldcg(reinterpret_cast<const unsigned long long*>(rec + (size_t)e * pitch));
      ex[e] = eb[e];
    }
  }
  if (F32 && b == 8 && S <= 5) {
    // T = R 2^(8(S-1)) + digits < 2^63: one rounding int64 -> f32 in
    // hardware, the scale added to the exponent field (exact while the
    // result stays normal; otherwise the exact path below).
    const int sh = 8 * (S - 1);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int64_t t = (int64_t)(int32_t)w[e] * ((int64_t)1 << sh) + (int64_t)(lw[e] & (uint32_t)((1ull << sh) - 1));
      const uint32_t fb = __float_as_uint(__ll2float_rn(t));
      const int fe = (int)((fb >> 23) & 0xFF) + ebase + ex[e];
      bits[e] = fb + ((uint32_t)(ebase + ex[e]) << 23);
      special |= (unsigned)(t == 0 || fe < 1 || fe > 254) << e;
    }
  } else {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const uint64_t lo = S - 1 > 4 ? (uint64_t)lw[e] | (uint64_t)hw[e] << 32 : (uint64_t)lw[e];
      bool neg, sp;
      uint64_t mhi, mlo;
      ozaki_exact_total((int32_t)w[e], lo, hi[e], b, S, neg, mhi, mlo);
      bits[e] = int128_to_float_bits_fast<Fmt>(neg, mhi, mlo, ebase + ex[e], sp);
      special |= (unsigned)sp << e;
    }
  }
  if (special) {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      if (!((special >> e) & 1)) continue;
      const uint64_t lo = S - 1 > 4 ? (uint64_t)lw[e] | (uint64_t)hw[e] << 32 : (uint64_t)lw[e];
      bool neg;
      uint64_t mhi, mlo;
      ozaki_exact_total((int32_t)w[e], lo, hi[e], b, S, neg, mhi, mlo);
      bits[e] = int128_to_float_bits<Fmt>(neg, mhi, mlo, ebase + ex[e]);
    }
  }
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    if (e >= left) continue;
    if (F32) {
      float* cp = static_cast<float*>(C) + off + e;
      const float r = __uint_as_float((uint32_t)bits[e]);
      *cp = accumulate ? *cp + r : r;
    } else {
      double* cp = static_cast<double*>(C) + off + e;
      const double r = __longlong_as_double((long long)bits[e]);
      *cp = accumulate ? *cp + r : r;
    }
  }
}

template <bool G>
__device__ __forceinline__ TileCtx tile_ctx(const OzParams& P, int tile) {
  TileCtx c;
  if (G) {
    const OzTile t = P.tiles[tile];
    const OzProb& q = P.probs[t.prob];
    c.m = q.m;
    c.n = q.n;
    c.row0 = (int64_t)t.tm * OZ_BM;
    c.col0 = (int64_t)t.tn * OzGeom<true>::BN;
    c.arow = q.rowoff + c.row0;
    c.brow = q.coloff + c.col0;
    c.kblocks = (int)((q.kpad + OZ_BK - 1) / OZ_BK);
    c.n_pairs = q.n_pairs;
    c.kchunks = q.kchunks;
    c.ea = P.ea + q.rowoff;
    c.eb = P.eb + q.coloff;
    c.C = q.C;
    c.ldc = q.ldc;
    c.accumulate = q.accumulate;
    c.f32 = q.f32;
  } else {
    int tm, tn;
    tile_coords(tile, P, tm, tn);
    c.m = P.m;
    c.n = P.n;
    c.row0 = c.arow = (int64_t)tm * OZ_BM;
    c.col0 = c.brow = (int64_t)tn * OZ_BN;
    c.kblocks = (int)((P.kpad + OZ_BK - 1) / OZ_BK);
    c.n_pairs = P.n_pairs;
    c.kchunks = P.kchunks;
    c.ea = P.ea;
    c.eb = P.eb;
    c.C = P.C;
    c.ldc = P.ldc;
    c.accumulate = P.accumulate;
    c.f32 = 0;
  }
  return c;
}

// EST = false: the slice-pair GEMM described in the file header.
// EST = true : the same pipeline on the spread-estimate operands (one K chunk
//              covering all of K): pass 1 (slices = 1) runs the one product
//              D = |A'| |B'|^T; pass 2 (slices = 2) also runs the two cross
//              products N = |A'| 1_B^T + 1_A |B'|^T of slices 0 and 1 (|x'|
//              and the nonzero indicator). The epilogue folds
//              max_ij (numerator_ij / D_ij) into P.est instead of writing C.
template <bool EST, bool G>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    ozaki_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                    OzParams P) {
  using Geo = OzGeom<G>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Geo::STAGES * Geo::STAGE_BYTES + Geo::EB_BYTES);
  uint64_t* empty = full + Geo::STAGES;
  uint64_t* accf = empty + Geo::STAGES;
  uint64_t* acce = accf + 2;
  uint64_t* drain = acce + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tiles = G ? P.n_tiles : P.tiles_m * P.tiles_n;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Geo::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 8);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&mapA);
    prefetch_tensormap(&mapB);
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, OZ_TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  auto bounded = [&](uint64_t* bar, uint32_t phase, uint32_t site) -> bool {
    for (uint32_t i = 0; i < NRS_WAIT_LIMIT; ++i) {
      if (mbar_try_wait(bar, phase)) return true;
      if (*abort_flag) return false;
    }
    *abort_flag = 1;
    atomicOr(P.err, NRS_DEVERR_GEMM_TC | (site << 8));
    return false;
  };

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const TileCtx c = tile_ctx<G>(P, tile);
        PairIter pr;
        pr.start(P.slices);
        for (int u = 0; u < c.n_pairs && ok; ++u, pr.next(c.kchunks)) {
          const int kb0 = pr.chunk * (P.kchunk / OZ_BK);
          int kb1 = kb0 + P.kchunk / OZ_BK;
          if (kb1 > c.kblocks) kb1 = c.kblocks;
          for (int kb = kb0; kb < kb1; ++kb, ++it) {
            const int s = it % Geo::STAGES;
            const uint32_t ph = (it / Geo::STAGES) & 1;
            if (!bounded(&empty[s], ph ^ 1, 1)) { ok = false; break; }
            uint8_t* st = smem + s * Geo::STAGE_BYTES;
            mbar_arrive_expect_tx(&full[s], Geo::STAGE_BYTES);
            tma_load_3d(st, &mapA, &full[s], kb * OZ_BK, (int32_t)c.arow, pr.s);
            tma_load_3d(st + OZ_A_BYTES, &mapB, &full[s], kb * OZ_BK, (int32_t)c.brow, pr.t());
          }
        }
      }
      if (!ok) {
        // Drain: wait (bounded) for the copies still in flight.
        for (uint32_t j = (it >= Geo::STAGES ? it - Geo::STAGES : 0); j < it; ++j)
          mbar_wait_bounded(&full[j % Geo::STAGES], (j / Geo::STAGES) & 1, 1u << 16);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t it = 0, ai = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const TileCtx c = tile_ctx<G>(P, tile);
        const int gm = merge_count(c, P, EST);
        PairIter pr;
        pr.start(P.slices);
        for (int u = 0; u < c.n_pairs && ok; ++ai) {
          const int g = group_size(pr, gm, c.kchunks);
          // One accumulator (TMEM columns 0..255) or two (0..127, 128..255,
          // grouped launches), used in turn; the epilogue frees one as soon
          // as it has read it.
          const int buf = Geo::ACC_BUFS == 2 ? (int)(ai & 1) : 0;
          const uint32_t aph = (Geo::ACC_BUFS == 2 ? ai >> 1 : ai) & 1;
          if (!bounded(&acce[buf], aph ^ 1, 2)) { ok = false; break; }
          tc_fence_after();
          const uint32_t d_tmem = tmem_base + (uint32_t)(buf * Geo::BN);
          for (int j = 0; j < g && ok; ++j, pr.next(c.kchunks)) {
            const int kb0 = pr.chunk * (P.kchunk / OZ_BK);
            int kb1 = kb0 + P.kchunk / OZ_BK;
            if (kb1 > c.kblocks) kb1 = c.kblocks;
            for (int kb = kb0; kb < kb1; ++kb, ++it) {
              const int s = it % Geo::STAGES;
              const uint32_t ph = (it / Geo::STAGES) & 1;
              if (!bounded(&full[s], ph, 3)) { ok = false; break; }
              tc_fence_after();
              const uint32_t a_addr = smem_u32(smem + s * Geo::STAGE_BYTES);
              const uint32_t b_addr = a_addr + OZ_A_BYTES;
#pragma unroll
              for (int kk = 0; kk < OZ_BK / 16; ++kk) {
                tc_mma_bf16(d_tmem, smem_desc_sw128(a_addr + kk * 32), smem_desc_sw128(b_addr + kk * 32),
                            Geo::IDESC, (j > 0 || kb > kb0 || kk > 0) ? 1u : 0u);
              }
              tc_commit(&empty[s]);  // frees the stage once these MMAs have read it
            }
          }
          if (!ok) break;
          tc_commit(&accf[buf]);  // accumulator ready once every MMA above completes
          u += g;
        }
      }
      // Make sure no MMA is still running before TMEM is released.
      tc_commit(drain);
      mbar_wait_bounded(drain, 0, 1u << 20);
    }
  } else if (EST) {
    // ---------------- spread-estimate epilogue (warps 2..9) ----------------
    // Same TMEM geometry as below. Units of a tile: pass 1: (0,0) = D;
    // pass 2: (0,1), (1,0) summed in fp32 into columns 256..511 = N, then
    // (0,0) = D. Per element r = numerator / D (pass 1: numerator =
    // (ra_i + cb_j) 2^96, the operands' 2^48 scale factors); D = 0 gives
    // +inf unless the numerator is 0 too (every product then has a zero
    // factor and the result is exact). The running max is float bits.
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row_in_tile = q * 32 + lane;
    const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16) + half * (OZ_BN / 2);
    const uint32_t acc_t = lane_base;
    const uint32_t dsum_t = lane_base + OZ_BN;
    uint32_t ai = 0;
    float rmax = 0.0f;
    bool ok = true;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      const TileCtx tc = tile_ctx<G>(P, tile);
      const int64_t row = tc.row0 + row_in_tile;
      const bool row_ok = row < tc.m;
      const int64_t col0 = tc.col0 + half * (OZ_BN / 2);
      const float ra = row_ok ? P.ra[row] : 0.0f;
      PairIter pr;
      pr.start(P.slices);
      for (int u = 0; u < tc.n_pairs; ++u, ++ai, pr.next(1)) {
        if (!bounded(&accf[0], ai & 1, 4)) { ok = false; break; }
        tc_fence_after();
        uint32_t v[OZ_BN / 2];
#pragma unroll
        for (int c = 0; c < OZ_BN / 32; ++c) tmem_ld16_nowait(acc_t + c * 16, v + c * 16);
        tmem_wait_ld();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[0]);
        if (pr.d == 1) {
#pragma unroll
          for (int c = 0; c < OZ_BN / 32; ++c) {
            uint32_t w[16];
            if (pr.s == 1) {
              tmem_ld16(dsum_t + c * 16, w);
#pragma unroll
              for (int e = 0; e < 16; ++e)
                w[e] = __float_as_uint(__uint_as_float(w[e]) + __uint_as_float(v[c * 16 + e]));
            } else {
#pragma unroll
              for (int e = 0; e < 16; ++e) w[e] = v[c * 16 + e];
            }
            tmem_st16(dsum_t + c * 16, w);
          }
          tmem_wait_st();
          tc_fence_before();
          __syncwarp();
          continue;
        }
#pragma unroll
        for (int c = 0; c < OZ_BN / 32; ++c) {  // unrolled: v[] stays in registers
          uint32_t w[16];
          if (P.slices == 2) tmem_ld16(dsum_t + c * 16, w);  // warp-uniform
          if (!row_ok) continue;
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int64_t col = col0 + c * 16 + e;
            if (col >= tc.n) continue;
            const float D = __uint_as_float(v[c * 16 + e]);
            const float num = P.slices == 2 ? __uint_as_float(w[e]) : ra + P.cb[col];
            float r;
            if (D > 0.0f) {
              r = num / D;
              if (P.slices != 2) r *= 0x1p96f;
            } else {
              r = num > 0.0f ? __uint_as_float(0x7f800000u) : 0.0f;
            }
            rmax = fmaxf(rmax, r);
          }
        }
      }
    }
    for (int off = 16; off; off >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
    if (lane == 0 && ok) atomicMax(P.est, __float_as_uint(rmax));
  } else if (G) {
    // ---------------- grouped epilogue (warps 2..9) ----------------
    // Warp w reads TMEM lane quarter w % 4 (one tile row per thread); the
    // two warps of a quarter take alternate 16-column chunks (half h:
    // chunks h, h+2, h+4, h+6), so narrow problems keep both busy. Chunks
    // right of the problem's n and quarters below its m skip all TMEM work
    // (warp-uniform tests).
    //
    // Exact accumulation without a 128-bit read-modify-write: one int32 per
    // element, R (TMEM columns 256..383), runs over the diagonals from
    // d = S-1 (least significant) to d = 0. Moving from diagonal d+1 to d,
    // R <- floor(R / 2^b) + D_d and the low b bits of the old R are final:
    // digit S-2-d. After d = 0,
    //   T = R 2^(b(S-1)) + sum_t digit_t 2^(bt)
    // is the exact sum of D_d 2^(b(S-1-d)), converted once to f64.
    // |R| < 2^31: |D_d| <= 120 * 2^24 (host limit on K chunks x S) and the
    // carry adds at most |R| / 2^b + 1.
    // Digits are kept one byte each, four to a word per element: digits
    // 0..3 in a register word that moves to TMEM columns 384..511 once full,
    // digits 4..7 in the register word after it, digits 8..14 (S > 9 only)
    // in this CTA's slot of 8-byte records in global memory.
    constexpr int BN = Geo::BN;
    constexpr size_t kColPitch = (size_t)OZ_BM * OZ_DIGIT_BYTES;  // slot bytes per tile column
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row_in_tile = q * 32 + lane;
    const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16);
    const uint32_t dsum_t = lane_base + 2 * BN;  // R
    const uint32_t dig_t = lane_base + 3 * BN;   // digits 0..3
    const int b = P.digit_bits, S = P.slices, nd = S - 1;
    const uint32_t dmask = (1u << b) - 1;
    uint8_t* const slot = reinterpret_cast<uint8_t*>(P.acc) + (size_t)blockIdx.x * (kColPitch * BN) +
                          (size_t)row_in_tile * OZ_DIGIT_BYTES;
    uint32_t dreg[BN / 2];  // this thread's digit word per element (chunk i, column e: [i * 16 + e])
    // this warp's column exponents, [i * 16 + e] for chunk i, column e
    int* const sm_eb = reinterpret_cast<int*>(smem + Geo::STAGES * Geo::STAGE_BYTES) + (warp - 2) * 64;
    uint32_t ai = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      const TileCtx tc = tile_ctx<G>(P, tile);
      const int64_t row = tc.row0 + row_in_tile;
      const bool row_ok = row < tc.m;
      const int ncols = (int)(tc.n - tc.col0 < BN ? tc.n - tc.col0 : BN);
      int nch = (ncols - 16 * half + 31) / 32;  // chunks of this warp inside the problem
      if (nch < 0 || tc.row0 + q * 32 >= tc.m) nch = 0;
      const int ecol_base = row_ok ? tc.ea[row] + P.final_shift : 0;
      // Column exponents of this warp's columns j = lane, lane + 32 (chunk
      // j / 16, column j % 16): loaded now, used by the retire pass at the
      // end of the tile (their latency hides behind the tile's groups).
      int ebj[2];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int j = lane + 32 * t;
        const int64_t col = tc.col0 + (2 * (j >> 4) + half) * 16 + (j & 15);
        ebj[t] = col < tc.n ? tc.eb[col] : 0;
      }
      const int gm = merge_count(tc, P, false);
#pragma unroll
      for (int e = 0; e < BN / 2; ++e) dreg[e] = 0;  // (no value survives a tile)
      PairIter pr;
      pr.start(S);
      int last_buf = 0;
      for (int u = 0; u < tc.n_pairs && ok; ++ai) {
        const int g = group_size(pr, gm, tc.kchunks);
        const int d = pr.d;
        const bool diag_start = pr.diag_first();
        const bool tile_first = u == 0;
        u += g;
        for (int j = 0; j < g; ++j) pr.next(tc.kchunks);
        const bool final_group = u == tc.n_pairs;  // the last group of d = 0
        const int buf = (int)(ai & 1);
        if (!bounded(&accf[buf], (ai >> 1) & 1, 4)) { ok = false; break; }
        tc_fence_after();
        // Chunk by chunk: the accumulator and R in flight together, R
        // updated and stored back; the accumulator goes back to the MMA warp
        // after the last chunk is read (the other one is in use meanwhile).
        const int dig_i = nd - 1 - d;  // digit index of diagonal d + 1
        const int dsh = 8 * (dig_i & 3);
#pragma unroll
        for (int i = 0; i < BN / 32; ++i) {
          if (i >= nch) continue;
          const int col_t = (2 * i + half) * 16;
          uint32_t v[16], w[16];
          tmem_ld16_nowait(lane_base + buf * BN + col_t, v);
          if (!tile_first) tmem_ld16_nowait(dsum_t + col_t, w);
          tmem_wait_ld();
          if (tile_first) {
#pragma unroll
            for (int e = 0; e < 16; ++e) w[e] = (uint32_t)__float2int_rn(__uint_as_float(v[e]));
          } else if (diag_start) {
#pragma unroll
            for (int e = 0; e < 16; ++e) {
              const int32_t r = (int32_t)w[e];
              const uint32_t dg = (uint32_t)r & dmask;
              if (dig_i < 8) {
                dreg[i * 16 + e] = (dsh ? dreg[i * 16 + e] : 0u) | dg << dsh;
              } else if (row_ok && col_t + e < ncols) {
                slot[(size_t)(col_t + e) * kColPitch + (dig_i - 8)] = (uint8_t)dg;
              }
              w[e] = (uint32_t)((r >> b) + __float2int_rn(__uint_as_float(v[e])));
            }
            if (dig_i == 3) tmem_st16(dig_t + col_t, *reinterpret_cast<const uint32_t(*)[16]>(dreg + i * 16));
          } else {
#pragma unroll
            for (int e = 0; e < 16; ++e) w[e] = (uint32_t)((int32_t)w[e] + __float2int_rn(__uint_as_float(v[e])));
          }
          tmem_st16(dsum_t + col_t, w);
          // The last group parks the register digit word in TMEM for the
          // retire pass below: digits 4..7 in this accumulator's columns
          // (held until then), or digits 0..S-2 in 384..511 when S <= 5.
          if (final_group)
            tmem_st16(nd > 4 ? lane_base + buf * BN + col_t : dig_t + col_t,
                      *reinterpret_cast<const uint32_t(*)[16]>(dreg + i * 16));
        }
        if (!final_group) {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&acce[buf]);
        }
        tmem_wait_st();
        last_buf = buf;
      }
      if (!ok) break;
      // After the last group of d = 0 (whose accumulator is still held): read
      // R and the digit words back, add the digits 8.. of the records,
      // convert, write C, then free the accumulator.
      sm_eb[lane] = ebj[0];
      sm_eb[lane + 32] = ebj[1];
      __syncwarp();
#pragma unroll 1
      for (int i = 0; i < nch; ++i) {
#pragma unroll
        for (int h8 = 0; h8 < 16; h8 += 8) {
          const int col_t = (2 * i + half) * 16 + h8;
          uint32_t w[8], lw[8], hw[8];
          tmem_ld8_nowait(dsum_t + col_t, w);
          tmem_ld8_nowait(dig_t + col_t, lw);
          if (nd > 4) tmem_ld8_nowait(lane_base + last_buf * BN + col_t, hw);
          tmem_wait_ld();
          if (!row_ok) continue;
          const int64_t off = row * tc.ldc + tc.col0 + col_t;
          if (tc.f32)
            retire8<true>(w, lw, hw, slot + (size_t)col_t * kColPitch, kColPitch, sm_eb + i * 16 + h8,
                          ncols - col_t, b, S, ecol_base, tc.C, off, tc.accumulate);
          else
            retire8<false>(w, lw, hw, slot + (size_t)col_t * kColPitch, kColPitch, sm_eb + i * 16 + h8,
                           ncols - col_t, b, S, ecol_base, tc.C, off, tc.accumulate);
        }
      }
      tc_fence_before();
      __syncwarp();  // (also: sm_eb is rewritten by the next tile only after this)
      if (lane == 0) mbar_arrive(&acce[last_buf]);
    }
  } else {
    // ---------------- epilogue (warps 2..9) ----------------
    // Warp w reads TMEM lane quarter w % 4 (one tile row per thread) and
    // column half (w - 2) / 4 (128 columns). As in the grouped epilogue, one
    // int32 per element, R (TMEM columns 256..511), carries the exact
    // diagonal sums from d = S-1 to d = 0 (R <- floor(R / 2^b) + D_d) and
    // the low b bits retire as digit S-2-d, here as a byte of the element's
    // 16-byte record in this CTA's slot (column-major 128 x 256; written once
    // per diagonal, read once).
    // No global read-modify-write per diagonal; after d = 0 each element's
    // exact total R 2^(b(S-1)) + sum_t digit_t 2^(bt) is rounded once to
    // f64. Per group: copy the accumulator to registers, hand it back to the
    // MMA warp at once, fold the copy into R.
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row_in_tile = q * 32 + lane;
    const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16) + half * (OZ_BN / 2);
    const uint32_t acc_t = lane_base;           // accumulator columns
    const uint32_t dsum_t = lane_base + OZ_BN;  // R
    const int b = P.digit_bits, S = P.slices, nd = S - 1;
    const uint32_t dmask = (1u << b) - 1;
    constexpr size_t pitch = (size_t)OZ_BM * 16;  // record bytes between tile columns
    uint8_t* const slot = reinterpret_cast<uint8_t*>(P.acc) + (size_t)blockIdx.x * (OZ_BM * OZ_BN * 16) +
                          (size_t)(half * (OZ_BN / 2)) * pitch + (size_t)row_in_tile * 16;
    uint32_t ai = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      const TileCtx tc = tile_ctx<G>(P, tile);
      const int64_t row = tc.row0 + row_in_tile;
      const bool row_ok = row < tc.m;
      const int64_t col0 = tc.col0 + half * (OZ_BN / 2);
      const int ncols = (int)(tc.n - col0 < OZ_BN / 2 ? (tc.n - col0 > 0 ? tc.n - col0 : 0) : OZ_BN / 2);
      const int ecol_base = row_ok ? tc.ea[row] + P.final_shift : 0;
      const int gm = merge_count(tc, P, false);
      PairIter pr;
      pr.start(S);
      for (int u = 0; u < tc.n_pairs && ok; ++ai) {
        const int g = group_size(pr, gm, tc.kchunks);
        const int d = pr.d;
        const bool diag_start = pr.diag_first();
        const bool tile_first = u == 0;
        u += g;
        for (int j = 0; j < g; ++j) pr.next(tc.kchunks);
        const uint32_t aph = ai & 1;
        if (!bounded(&accf[0], aph, 4)) { ok = false; break; }
        tc_fence_after();
        // Copy this warp's 128 accumulator columns to registers (eight loads,
        // one wait) and hand the accumulator back at once, so the next unit's
        // MMAs run while the copy is folded into R.
        uint32_t v[OZ_BN / 2];
#pragma unroll
        for (int c = 0; c < OZ_BN / 32; ++c) tmem_ld16_nowait(acc_t + c * 16, v + c * 16);
        tmem_wait_ld();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[0]);
        const int dig_i = nd - 1 - d;  // digit index of diagonal d + 1
#pragma unroll
        for (int c = 0; c < OZ_BN / 32; ++c) {
          uint32_t w[16];
          if (tile_first) {
#pragma unroll
            for (int e = 0; e < 16; ++e) w[e] = (uint32_t)__float2int_rn(__uint_as_float(v[c * 16 + e]));
          } else {
            tmem_ld16(dsum_t + c * 16, w);
            if (diag_start) {
              uint8_t* sp = slot + (size_t)(c * 16) * pitch + dig_i;
              const int nv = row_ok ? ncols - c * 16 : 0;  // columns of this chunk inside the problem
#pragma unroll
              for (int e = 0; e < 16; ++e) {
                const int32_t r = (int32_t)w[e];
                if (e < nv) sp[(size_t)e * pitch] = (uint8_t)((uint32_t)r & dmask);
                w[e] = (uint32_t)((r >> b) + __float2int_rn(__uint_as_float(v[c * 16 + e])));
              }
            } else {
#pragma unroll
              for (int e = 0; e < 16; ++e)
                w[e] = (uint32_t)((int32_t)w[e] + __float2int_rn(__uint_as_float(v[c * 16 + e])));
            }
          }
          tmem_st16(dsum_t + c * 16, w);
        }
        tmem_wait_st();
        tc_fence_before();
        __syncwarp();
      }
      if (!ok) break;
      // After the last group of d = 0: R and the records of 8 columns at a
      // time (loads in flight together), rounded once, written to C.
#pragma unroll 1
      for (int c8 = 0; c8 < OZ_BN / 2; c8 += 8) {
        if (c8 >= ncols) break;  // warp-uniform
        uint32_t w[8], lw[8], hw[8];
        tmem_ld8_nowait(dsum_t + c8, w);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          uint64_t r = 0;
          if (row_ok && c8 + e < ncols)
            r = __ldcg(reinterpret_cast<const unsigned long long*>(slot + (size_t)(c8 + e) * pitch));
          lw[e] = (uint32_t)r;
          hw[e] = (uint32_t)(r >> 32);
        }
        tmem_wait_ld();
        if (!row_ok) continue;
        retire8<false>(w, lw, hw, slot + (size_t)c8 * pitch + 8, pitch, tc.eb + col0 + c8, ncols - c8, b, S,
                       ecol_base, tc.C, row * tc.ldc + col0 + c8, tc.accumulate);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, OZ_TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// Scaling exponents and slicing
// ---------------------------------------------------------------------------
// frexp-style exponent of max |x| over a row (one warp per row; T double or
// float, widened exactly). `flag` (may be null) gets bit 0 set when a row
// holds an Inf or a NaN.
template <typename T>
__global__ void row_exponents(const T* __restrict__ A, int64_t m, int64_t k, int64_t lda,
                              int* __restrict__ ea, uint32_t* __restrict__ flag) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= m) return;
  uint64_t mx = 0;
  for (int64_t j = lane; j < k; j += 32) {
    uint64_t b = (uint64_t)__double_as_longlong((double)A[row * lda + j]) & 0x7FFFFFFFFFFFFFFFULL;
    mx = b > mx ? b : mx;
  }
  for (int off = 16; off; off >>= 1) {
    uint64_t o = __shfl_xor_sync(0xffffffffu, mx, off);
    mx = o > mx ? o : mx;
  }
  if (lane == 0) {
    int e = (int)(mx >> 52) - 1022;  // |max| < 2^e
    if ((mx >> 52) == 0) e = -1021;  // zero or subnormal
    ea[row] = e;
    if (flag && (mx >> 52) == 0x7FF) atomicOr(flag, 1u);
  }
}

// Column maxima of |B| (k x n row-major) as IEEE bit patterns (ordered like
// the magnitudes): a 2-D grid of 256-row strips, coalesced across columns,
// combined with atomicMax on the bit pattern into a zeroed array.
constexpr int kColStrip = 256;
template <typename T>
__global__ void col_max_bits(const T* __restrict__ B, int64_t k, int64_t n, int64_t ldb,
                             unsigned long long* __restrict__ colmax) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n) return;
  const int64_t r0 = (int64_t)blockIdx.y * kColStrip;
  const int64_t r1 = (r0 + kColStrip) < k ? (r0 + kColStrip) : k;
  unsigned long long mx = 0;
  for (int64_t i = r0; i < r1; ++i) {
    const unsigned long long b =
        (unsigned long long)__double_as_longlong((double)B[i * ldb + col]) & 0x7FFFFFFFFFFFFFFFULL;
    mx = b > mx ? b : mx;
  }
  atomicMax(&colmax[col], mx);
}

// frexp-style exponent from a max-magnitude bit pattern.
__global__ void exponents_from_bits(const unsigned long long* __restrict__ mx, int64_t n,
                                    int* __restrict__ e, uint32_t* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long b = mx[i];
  e[i] = ((b >> 52) == 0) ? -1021 : (int)(b >> 52) - 1022;
  if (flag && (b >> 52) == 0x7FF) atomicOr(flag, 1u);
}

// X = round(x * 2^(126 - e)) as a signed 128-bit integer (|x| < 2^e).
__device__ __forceinline__ __int128 fixed126(double x, int e) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const bool neg = bits >> 63;
  const int biased = (int)((bits >> 52) & 0x7FF);
  uint64_t mant = bits & 0xFFFFFFFFFFFFFULL;
  int E;
  if (biased == 0) {
    E = -1022 - 52;  // subnormal: x = mant * 2^-1074
  } else {
    mant |= 1ULL << 52;
    E = biased - 1023 - 52;  // x = mant * 2^E
  }
  const int sh = E + 126 - e;
  __int128 X;
  if (mant == 0) {
    X = 0;
  } else if (sh >= 0) {
    X = (__int128)mant << sh;  // sh <= 73 because |x| < 2^e
  } else if (sh > -64) {
    X = (__int128)((mant + (1ULL << (-sh - 1))) >> (-sh));
  } else {
    X = 0;
  }
  return neg ? -X : X;
}

// Signed b-bit digits of X at positions p_t = 127 - b - b t, t < S, with
//   sum_t d_t 2^p_t = X rounded to the nearest multiple of 2^p_(S-1) (ties up).
// Z = X + h * sum_t 2^p_t + 2^(p_(S-1) - 1), h = 2^(b-1), makes every b-bit
// field of Z the digit plus h, so each digit is one shift and mask: d_t in
// [-h, h - 1] for t >= 1, the top digit (Z >> p_0) - h in [-h, h]. Every
// digit is exact in BF16 and |d_s d_t| <= 2^(2b-2), as the file header
// requires.
// Z is unsigned: X + C lies in (0, 2^127 + 2^122), beyond the signed range.
__device__ __forceinline__ unsigned __int128 digit_offset(int S, int b) {
  unsigned __int128 c = (unsigned __int128)1 << (kTopOf(b) - b * (S - 1) - 1);
  for (int t = 0; t < S; ++t) c += (unsigned __int128)(1u << (b - 1)) << (kTopOf(b) - b * t);
  return c;
}
// B is a template argument so that every digit position is a constant shift.
template <int B>
__device__ __forceinline__ int digit_at(unsigned __int128 Z, int t) {
  const int p = kTopOf(B) - B * t;
  const int f = (int)(uint32_t)(uint64_t)(Z >> p);
  return (t == 0 ? f : (f & ((1 << B) - 1))) - (1 << (B - 1));
}

__device__ __forceinline__ uint32_t bf16_of_int(int v) {
  // |v| <= 2^(b-1) <= 128: exact in bf16; its fp32 bit pattern's top half.
  return __float_as_uint((float)v) >> 16;
}

// A (m x k) -> slices [S][m][kpad], K-major; zero beyond k. A thread takes 8
// consecutive k of one row (kpad is a multiple of 8; four 16-byte loads when
// aligned) and writes one 16-byte vector per slice.
// SMALL (b S <= 64): the same digits from 64-bit arithmetic (ozaki_z64).
template <int b, bool VEC, bool SMALL>
__global__ void __launch_bounds__(256)
    slice_rows(const double* __restrict__ A, int64_t m, int64_t k, int64_t lda, int64_t kpad,
               const int* __restrict__ ea, int S, uint16_t* __restrict__ out) {
  const int64_t gpr = kpad / 8;
  const int64_t total = m * gpr;
  const unsigned __int128 C = digit_offset(S, b);
  const uint64_t C64 = ozaki_offset64(S, b);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = g / gpr, j0 = (g - i * gpr) * 8;
    const int e = ea[i];
    double x[8];
    const double* row = A + i * lda + j0;
    if (VEC && j0 + 8 <= k) {  // four 16-byte loads
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double2 d2 = reinterpret_cast<const double2*>(row)[q];
        x[2 * q] = d2.x;
        x[2 * q + 1] = d2.y;
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) x[q] = j0 + q < k ? row[q] : 0.0;
    }
    // The eight offset values, then one slice at a time (one 16-byte store
    // each), so only the current slice's packed words are live.
    uint16_t* o = out + i * kpad + j0;
    if constexpr (SMALL) {
      OzakiZ64 Z[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) Z[q] = ozaki_z64(x[q], e, b, S, C64);
#pragma unroll
      for (int t = 0; t < OZ_MAX_SLICES; ++t) {
        if (t < S) {
          uint32_t pk[4];
#pragma unroll
          for (int h = 0; h < 4; ++h)
            pk[h] = bf16_of_int(ozaki_digit64<b>(Z[2 * h], t)) |
                    (bf16_of_int(ozaki_digit64<b>(Z[2 * h + 1], t)) << 16);
          *reinterpret_cast<uint4*>(o + (int64_t)t * m * kpad) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    } else {
      unsigned __int128 Z[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) Z[q] = (unsigned __int128)fixed126(x[q], e) + C;
#pragma unroll
      for (int t = 0; t < OZ_MAX_SLICES; ++t) {
        if (t < S) {
          uint32_t pk[4];
#pragma unroll
          for (int h = 0; h < 4; ++h)
            pk[h] = bf16_of_int(digit_at<b>(Z[2 * h], t)) | (bf16_of_int(digit_at<b>(Z[2 * h + 1], t)) << 16);
          *reinterpret_cast<uint4*>(o + (int64_t)t * m * kpad) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
  }
}

// B (k x n row-major) -> slices of B^T [S][n][kpad]. A block takes 64 k x 32 n:
// thread (nn = tid % 32, kk pair) reads B coalesced along n, packs the digits
// of two consecutive k into one 32-bit word of a shared tile [S][32 n][33
// words] (the pad word keeps both phases free of bank conflicts), then every
// thread writes one 16-byte vector (8 k of one n row) per slice.
constexpr int kSliceColK = 64, kSliceColN = 32, kSliceColPitch = kSliceColK / 2 + 1;
template <int b, bool SMALL>
__global__ void __launch_bounds__(256)
    slice_cols(const double* __restrict__ B, int64_t k, int64_t n, int64_t ldb, int64_t kpad,
               const int* __restrict__ eb, int S, uint16_t* __restrict__ out) {
  extern __shared__ uint32_t tile[];  // [S][32][33]
  const int64_t k0 = (int64_t)blockIdx.y * kSliceColK, n0 = (int64_t)blockIdx.x * kSliceColN;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const unsigned __int128 C = digit_offset(S, b);
  const uint64_t C64 = ozaki_offset64(S, b);
  {
    const int64_t nn = n0 + tx;
    const int e = nn < n ? eb[nn] : 0;
#pragma unroll
    for (int r = 0; r < kSliceColK / 16; ++r) {  // word column w = ty + 8r: k rows 2w, 2w+1
      const int w = ty + 8 * r;
      const int64_t kk = k0 + 2 * w;
      const double x0 = kk < k && nn < n ? B[kk * ldb + nn] : 0.0;
      const double x1 = kk + 1 < k && nn < n ? B[(kk + 1) * ldb + nn] : 0.0;
      if constexpr (SMALL) {
        const OzakiZ64 Z0 = ozaki_z64(x0, e, b, S, C64), Z1 = ozaki_z64(x1, e, b, S, C64);
#pragma unroll
        for (int t = 0; t < OZ_MAX_SLICES; ++t)
          if (t < S)
            tile[(t * kSliceColN + tx) * kSliceColPitch + w] =
                bf16_of_int(ozaki_digit64<b>(Z0, t)) | (bf16_of_int(ozaki_digit64<b>(Z1, t)) << 16);
      } else {
        const unsigned __int128 Z0 = (unsigned __int128)fixed126(x0, e) + C;
        const unsigned __int128 Z1 = (unsigned __int128)fixed126(x1, e) + C;
#pragma unroll
        for (int t = 0; t < OZ_MAX_SLICES; ++t)
          if (t < S)
            tile[(t * kSliceColN + tx) * kSliceColPitch + w] =
                bf16_of_int(digit_at<b>(Z0, t)) | (bf16_of_int(digit_at<b>(Z1, t)) << 16);
      }
    }
  }
  __syncthreads();
  const int r = threadIdx.x >> 3, c = threadIdx.x & 7;  // n row, 16-byte chunk (8 k)
  const int64_t nn = n0 + r, kk = k0 + c * 8;
  if (nn < n && kk < kpad) {
    for (int t = 0; t < S; ++t) {
      const uint32_t* src = tile + (t * kSliceColN + r) * kSliceColPitch + c * 4;
      *reinterpret_cast<uint4*>(out + (int64_t)t * n * kpad + nn * kpad + kk) =
          make_uint4(src[0], src[1], src[2], src[3]);
    }
  }
}

// ---------------------------------------------------------------------------
// Spread estimate operands
// ---------------------------------------------------------------------------
// For the automatic slice count the operands are also written as two BF16
// "slices": slice 0 = |x'| 2^48 (x' = x 2^-e, so |x'| < 1; rounded to
// nearest) and slice 1 = 2^48 where x != 0, else 0. The 2^48 factors keep
// products of small |x'| above FP32's underflow threshold while every sum
// over K stays below 2^96 * 2^31 < 2^128. Row sums of |x'| (fp32, fixed
// order) give the pass-1 numerator.
constexpr uint32_t kBf16Two48 = 0x5780u;  // 2^48 in BF16

__device__ __forceinline__ bool nonzero(double x) {
  return ((uint64_t)__double_as_longlong(x) << 1) != 0;  // integer test, +-0 excluded
}

// |x| 2^-e from the bit pattern alone (no FP64 arithmetic: GB300's FP64 pipe
// is slow): *f = |x'| as fp32 (mantissa truncated), return value = |x'| 2^48
// as BF16 (round to nearest even). Subnormal x and values below the formats'
// normal ranges give 0 (the estimate then only grows).
__device__ __forceinline__ uint32_t est_bits(double x, int e, float* f) {
  const uint64_t u = (uint64_t)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFULL;
  const int be = (int)(u >> 52);
  const uint64_t mant = u & 0xFFFFFFFFFFFFFULL;
  const int fe = be - 1023 - e;  // unbiased exponent of |x'| (<= -1)
  if (be == 0) {
    *f = 0.0f;
    return 0u;
  }
  *f = (fe + 127 >= 1) ? __uint_as_float(((uint32_t)(fe + 127) << 23) | (uint32_t)(mant >> 29)) : 0.0f;
  if (fe + 48 + 127 < 1) return 0u;
  uint32_t h = ((uint32_t)(fe + 48 + 127) << 7) | (uint32_t)(mant >> 45);
  const uint64_t rem = mant & ((1ULL << 45) - 1), half = 1ULL << 44;
  if (rem > half || (rem == half && (h & 1u))) ++h;
  return h;
}

// X (rows x k, row pitch ld, contiguous along k) -> out [2][rows][kpad],
// sums[row] = sum_k |x'|. One warp per row, 8 consecutive k per lane step.
template <bool VEC, typename T>
__global__ void __launch_bounds__(256)
    est_rows(const T* __restrict__ X, int64_t rows, int64_t k, int64_t ld, int64_t kpad,
             const int* __restrict__ e, uint16_t* __restrict__ out, float* __restrict__ sums) {
  const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  const int er = e[row];
  const T* xr = X + row * ld;
  float s = 0.0f;
  for (int64_t j0 = (int64_t)lane * 8; j0 < kpad; j0 += 256) {
    double x[8];
    if (VEC && j0 + 8 <= k) {  // (T = double only)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double2 d2 = reinterpret_cast<const double2*>(xr + j0)[q];
        x[2 * q] = d2.x;
        x[2 * q + 1] = d2.y;
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) x[q] = j0 + q < k ? (double)xr[j0 + q] : 0.0;
    }
    uint32_t pa[4], pi[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      float f0, f1;
      const uint32_t b0 = est_bits(x[2 * h], er, &f0), b1 = est_bits(x[2 * h + 1], er, &f1);
      s += f0;
      s += f1;
      pa[h] = b0 | (b1 << 16);
      pi[h] = (nonzero(x[2 * h]) ? kBf16Two48 : 0u) | ((nonzero(x[2 * h + 1]) ? kBf16Two48 : 0u) << 16);
    }
    uint16_t* o = out + row * kpad + j0;
    *reinterpret_cast<uint4*>(o) = make_uint4(pa[0], pa[1], pa[2], pa[3]);
    *reinterpret_cast<uint4*>(o + rows * kpad) = make_uint4(pi[0], pi[1], pi[2], pi[3]);
  }
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) sums[row] = s;
}

// X (k x cols row-major) -> out [2][cols][kpad] (transposed through shared
// memory like slice_cols), part[strip][col] = sum of |x'| over the block's
// 64 k; est_strip_sums adds the strips in order (deterministic).
template <typename T>
__global__ void __launch_bounds__(256)
    est_cols(const T* __restrict__ X, int64_t k, int64_t cols, int64_t ld, int64_t kpad,
             const int* __restrict__ e, uint16_t* __restrict__ out, float* __restrict__ part) {
  __shared__ uint32_t tile[2][kSliceColN][kSliceColPitch];
  __shared__ float csum[8][kSliceColN];
  const int64_t k0 = (int64_t)blockIdx.y * kSliceColK, n0 = (int64_t)blockIdx.x * kSliceColN;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t nn = n0 + tx;
  const int ec = nn < cols ? e[nn] : 0;
  float s = 0.0f;
#pragma unroll
  for (int r = 0; r < kSliceColK / 16; ++r) {
    const int w = ty + 8 * r;
    const int64_t kk = k0 + 2 * w;
    const double x0 = kk < k && nn < cols ? (double)X[kk * ld + nn] : 0.0;
    const double x1 = kk + 1 < k && nn < cols ? (double)X[(kk + 1) * ld + nn] : 0.0;
    float f0, f1;
    const uint32_t b0 = est_bits(x0, ec, &f0), b1 = est_bits(x1, ec, &f1);
    s += f0;
    s += f1;
    tile[0][tx][w] = b0 | (b1 << 16);
    tile[1][tx][w] = (nonzero(x0) ? kBf16Two48 : 0u) | ((nonzero(x1) ? kBf16Two48 : 0u) << 16);
  }
  csum[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && nn < cols) {
    float t = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q) t += csum[q][tx];
    part[(int64_t)blockIdx.y * cols + nn] = t;
  }
  const int r = threadIdx.x >> 3, c = threadIdx.x & 7;
  const int64_t n2 = n0 + r, k2 = k0 + c * 8;
  if (n2 < cols && k2 < kpad) {
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const uint32_t* src = &tile[t][r][c * 4];
      *reinterpret_cast<uint4*>(out + (int64_t)t * cols * kpad + n2 * kpad + k2) =
          make_uint4(src[0], src[1], src[2], src[3]);
    }
  }
}

__global__ void est_strip_sums(const float* __restrict__ part, int64_t strips, int64_t cols,
                               float* __restrict__ sums) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float t = 0.0f;
  for (int64_t s = 0; s < strips; ++s) t += part[s * cols + c];
  sums[c] = t;
}

bool make_slice_map(CUtensorMap* map, const void* base, int64_t kpad, int64_t rows, int S,
                    uint32_t box_rows) {
  auto enc = nrs_get_encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)rows, (cuuint64_t)S};
  const cuuint64_t strides[2] = {(cuuint64_t)kpad * 2, (cuuint64_t)(kpad * rows * 2)};
  const cuuint32_t box[3] = {OZ_BK, box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}


// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// One operand as the kernels see it: `rows` output rows (m for A, n for B)
// along K. rows_contig: element (r, kk) at p[r * ld + kk] (A as given, or B
// passed transposed); otherwise at p[kk * ld + r] (B as given, or A passed
// transposed), which the column kernels read coalesced and transpose.
struct OzOperand {
  const void* p;  // double, or float when f32 (the spread estimate only)
  int64_t ld;
  int64_t rows;
  bool rows_contig;
  bool f32 = false;
  const double* d() const { return static_cast<const double*>(p); }
  const float* f() const { return static_cast<const float*>(p); }
};

int launch_exponents(nrs_handle* h, const OzOperand& o, int64_t k, int* e,
                     unsigned long long* colmax, uint32_t* flag) {
  cudaStream_t s = h->stream;
  if (o.rows_contig) {
    if (o.f32)
      row_exponents<float><<<(unsigned)((o.rows + 7) / 8), 256, 0, s>>>(o.f(), o.rows, k, o.ld, e, flag);
    else
      row_exponents<double><<<(unsigned)((o.rows + 7) / 8), 256, 0, s>>>(o.d(), o.rows, k, o.ld, e, flag);
  } else {
    int st = nrs_cuda_check(h, cudaMemsetAsync(colmax, 0, (size_t)o.rows * 8, s), "cudaMemsetAsync");
    if (st) return st;
    const dim3 grid((unsigned)((o.rows + 255) / 256), (unsigned)((k + kColStrip - 1) / kColStrip));
    if (o.f32)
      col_max_bits<float><<<grid, 256, 0, s>>>(o.f(), k, o.rows, o.ld, colmax);
    else
      col_max_bits<double><<<grid, 256, 0, s>>>(o.d(), k, o.rows, o.ld, colmax);
    exponents_from_bits<<<(unsigned)((o.rows + 255) / 256), 256, 0, s>>>(colmax, o.rows, e, flag);
  }
  return nrs_after_launch(h, "ozaki exponents");
}

template <int b, bool SMALL>
int launch_slices_bs(nrs_handle* h, const OzOperand& o, int64_t k, int64_t kpad, const int* e, int S,
                     uint16_t* out) {
  cudaStream_t s = h->stream;
  if (o.rows_contig) {
    const int64_t groups = o.rows * (kpad / 8);
    const int grid = (int)std::min<int64_t>((groups + 255) / 256, (int64_t)h->num_sms * 8);
    // 16-byte row loads when every row start is 16-byte aligned.
    if (((reinterpret_cast<uintptr_t>(o.p) & 15) == 0) && (o.ld % 2 == 0))
      slice_rows<b, true, SMALL><<<grid, 256, 0, s>>>(o.d(), o.rows, k, o.ld, kpad, e, S, out);
    else
      slice_rows<b, false, SMALL><<<grid, 256, 0, s>>>(o.d(), o.rows, k, o.ld, kpad, e, S, out);
  } else {
    const int smem = (int)((size_t)S * kSliceColN * kSliceColPitch * 4);
    int st = nrs_cuda_check(h,
                            cudaFuncSetAttribute(slice_cols<b, SMALL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 smem),
                            "cudaFuncSetAttribute(slice_cols)");
    if (st) return st;
    dim3 g((unsigned)((o.rows + kSliceColN - 1) / kSliceColN), (unsigned)((kpad + kSliceColK - 1) / kSliceColK));
    slice_cols<b, SMALL><<<g, 256, smem, s>>>(o.d(), k, o.rows, o.ld, kpad, e, S, out);
  }
  return nrs_after_launch(h, "ozaki slicing");
}
// b S <= 64: the 64-bit digit path (the same digits, fewer integer operations)
template <int b>
int launch_slices_b(nrs_handle* h, const OzOperand& o, int64_t k, int64_t kpad, const int* e, int S,
                    uint16_t* out) {
  return b * S <= 64 ? launch_slices_bs<b, true>(h, o, k, kpad, e, S, out)
                     : launch_slices_bs<b, false>(h, o, k, kpad, e, S, out);
}

int launch_slices(nrs_handle* h, const OzOperand& o, int64_t k, int64_t kpad, const int* e, int b, int S,
                  uint16_t* out) {
  return b == 8 ? launch_slices_b<8>(h, o, k, kpad, e, S, out)
                : b == 7 ? launch_slices_b<7>(h, o, k, kpad, e, S, out)
                         : launch_slices_b<6>(h, o, k, kpad, e, S, out);
}

int launch_est_operand(nrs_handle* h, const OzOperand& o, int64_t k, int64_t kpad, const int* e,
                       uint16_t* out, float* sums, float* part) {
  cudaStream_t s = h->stream;
  if (o.rows_contig) {
    const unsigned grid = (unsigned)((o.rows + 7) / 8);
    if (o.f32)
      est_rows<false, float><<<grid, 256, 0, s>>>(o.f(), o.rows, k, o.ld, kpad, e, out, sums);
    else if (((reinterpret_cast<uintptr_t>(o.p) & 15) == 0) && (o.ld % 2 == 0))
      est_rows<true, double><<<grid, 256, 0, s>>>(o.d(), o.rows, k, o.ld, kpad, e, out, sums);
    else
      est_rows<false, double><<<grid, 256, 0, s>>>(o.d(), o.rows, k, o.ld, kpad, e, out, sums);
  } else {
    const int64_t strips = (kpad + kSliceColK - 1) / kSliceColK;
    dim3 g((unsigned)((o.rows + kSliceColN - 1) / kSliceColN), (unsigned)strips);
    if (o.f32)
      est_cols<float><<<g, 256, 0, s>>>(o.f(), k, o.rows, o.ld, kpad, e, out, part);
    else
      est_cols<double><<<g, 256, 0, s>>>(o.d(), k, o.rows, o.ld, kpad, e, out, part);
    est_strip_sums<<<(unsigned)((o.rows + 255) / 256), 256, 0, s>>>(part, strips, o.rows, sums);
  }
  return nrs_after_launch(h, "ozaki spread operands");
}

// rows_a / rows_b: rows of the (stacked) slice buffers; P.kpad: their pitch.
template <bool EST, bool G>
int launch_tc(nrs_handle* h, const void* sa, const void* sb, int S, const OzParams& P, int64_t rows_a,
              int64_t rows_b, cudaStream_t stream) {
  CUtensorMap mapA, mapB;
  if (!make_slice_map(&mapA, sa, P.kpad, rows_a, S, OZ_BM) ||
      !make_slice_map(&mapB, sb, P.kpad, rows_b, S, OzGeom<G>::BN))
    return nrs_fail(h, NRS_ERR_CUDA, "cuTensorMapEncodeTiled failed for the slices");
  // Set on every call: the attribute belongs to the current device's context.
  int st = nrs_cuda_check(h, cudaFuncSetAttribute(ozaki_tc_kernel<EST, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  OzGeom<G>::SMEM),
                          "cudaFuncSetAttribute(ozaki)");
  if (st) return st;
  const int n_tiles = G ? P.n_tiles : P.tiles_m * P.tiles_n;
  const int ctas = n_tiles < h->num_sms ? n_tiles : h->num_sms;
  if (ctas < 1) return NRS_OK;
  ozaki_tc_kernel<EST, G><<<ctas, OZ_THREADS, OzGeom<G>::SMEM, stream>>>(mapA, mapB, P);
  return nrs_after_launch(h, EST ? "ozaki_tc_kernel<est>" : "ozaki_tc_kernel");
}

OzParams base_params(nrs_handle* h, int64_t m, int64_t n, int64_t k, int64_t kpad) {
  OzParams P{};
  P.m = m;
  P.n = n;
  P.k = k;
  P.kpad = kpad;
  P.tiles_m = (int)((m + OZ_BM - 1) / OZ_BM);
  P.tiles_n = (int)((n + OZ_BN - 1) / OZ_BN);
  P.group_m = 12;
  P.err = h->dev_error;
  return P;
}

// Limits of b-bit digits with S slices over kpad: S <= 16, every digit
// inside the 126 fraction bits (b S <= 126), int32-exact diagonal sums (at
// most kc S K-chunk sums of |x| <= 2^24 each, kc = ceil(kpad / 2^(26-2b)):
// kc S <= 127 for one problem, <= 120 for grouped launches, whose carried
// sums need the headroom), and the exact total inside a signed 128-bit
// integer (|total| < 2^(31 + b(S-1)) with b(S-1) <= 95).
constexpr int64_t kMaxChunkSlices = 127;
constexpr int64_t kMaxChunkSlicesGrouped = 120;
bool digits_fit(int b, int S, int64_t kpad, int64_t max_kcs) {
  const int64_t kc = std::max<int64_t>(1, (kpad + kChunkOf(b) - 1) / kChunkOf(b));
  return S >= 1 && S <= OZ_MAX_SLICES && b * S <= 126 && b * (S - 1) <= 95 && kc * S <= max_kcs;
}

// Digit width and count for `bits` bits of each operand's fixed-point value:
// the widest b (8, 7, 6) with S = ceil(bits / b) inside digits_fit's limits.
// false if no width qualifies.
bool choose_digits(int64_t kpad, double bits, int* b, int* S, int* kchunks,
                   int64_t max_kcs = kMaxChunkSlices) {
  for (int cand = 8; cand >= 6; --cand) {
    int s_c = (int)std::ceil(bits / cand - 1e-9);
    if (s_c < 1) s_c = 1;
    const int64_t kc = (kpad + kChunkOf(cand) - 1) / kChunkOf(cand);
    if (digits_fit(cand, s_c, kpad, max_kcs)) {
      *b = cand;
      *S = s_c;
      *kchunks = (int)kc;
      return true;
    }
  }
  return false;
}

// Bits of the fixed-point operands that keep the slicing error at FP64's
// unit roundoff relative to (|A||B|)_ij: each operand element is rounded at
// 2^-(bS) (scaled units), so |C - AB|_ij <~ 2^-(bS) (sum_k |a'_ik| + |b'_kj|)
// = 2^-(bS) R_ij (|A'||B'|)_ij, and bS >= 53 + log2 max_ij R_ij.
constexpr double kTargetBits = 53.0;

struct SpreadResult {
  float rmax;
  uint32_t flags;  // bit 0: an operand holds Inf or NaN
};

// Runs the spread estimate: exponents, estimate operands and one (pass 1) or
// three (pass 2) BF16 products, then reads max_ij R_ij back (one stream
// synchronisation).
int spread_estimate(nrs_handle* h, const OzOperand& a, const OzOperand& bT, int64_t m, int64_t n, int64_t k,
                    int64_t kpad, int pass, SpreadResult* res) {
  auto al = [](size_t v) { return (v + 1023) & ~size_t(1023); };
  const int64_t strips = (kpad + kSliceColK - 1) / kSliceColK;
  const size_t ea_b = al((size_t)m * 4), eb_b = al((size_t)n * 4), ra_b = al((size_t)m * 4),
               cb_b = al((size_t)n * 4), cm_b = al((size_t)std::max(m, n) * 8),
               part_b = al((size_t)strips * std::max(m, n) * 4), sa_b = al((size_t)2 * m * kpad * 2),
               sb_b = al((size_t)2 * n * kpad * 2), word_b = 1024;
  int st;
  uint8_t* ws = (uint8_t*)nrs_workspace(h, ea_b + eb_b + ra_b + cb_b + cm_b + part_b + sa_b + sb_b + word_b, &st);
  if (!ws) return st;
  int* ea = (int*)ws;
  int* eb = (int*)(ws + ea_b);
  float* ra = (float*)(ws + ea_b + eb_b);
  float* cb = (float*)(ws + ea_b + eb_b + ra_b);
  unsigned long long* colmax = (unsigned long long*)(ws + ea_b + eb_b + ra_b + cb_b);
  float* part = (float*)(ws + ea_b + eb_b + ra_b + cb_b + cm_b);
  uint16_t* sa = (uint16_t*)(ws + ea_b + eb_b + ra_b + cb_b + cm_b + part_b);
  uint16_t* sb = (uint16_t*)((uint8_t*)sa + sa_b);
  uint32_t* word = (uint32_t*)((uint8_t*)sb + sb_b);  // [0] max R bits, [1] flags
  cudaStream_t s = h->stream;
  if ((st = nrs_cuda_check(h, cudaMemsetAsync(word, 0, 8, s), "cudaMemsetAsync"))) return st;
  if ((st = launch_exponents(h, a, k, ea, colmax, word + 1))) return st;
  if ((st = launch_exponents(h, bT, k, eb, colmax, word + 1))) return st;
  if ((st = launch_est_operand(h, a, k, kpad, ea, sa, ra, part))) return st;
  if ((st = launch_est_operand(h, bT, k, kpad, eb, sb, cb, part))) return st;
  OzParams P = base_params(h, m, n, k, kpad);
  P.slices = pass;
  P.kchunks = 1;
  P.n_pairs = pass == 1 ? 1 : 3;
  P.kchunk = (int)(((kpad + OZ_BK - 1) / OZ_BK) * OZ_BK);
  P.ra = ra;
  P.cb = cb;
  P.est = word;
  if ((st = launch_tc<true, false>(h, sa, sb, 2, P, m, n, s))) return st;
  uint32_t host[2] = {0, 0};
  if ((st = nrs_cuda_check(h, cudaMemcpyAsync(host, word, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync")))
    return st;
  if ((st = nrs_cuda_check(h, cudaStreamSynchronize(s), "cudaStreamSynchronize"))) return st;
  uint32_t derr = 0;
  if ((st = nrs_cuda_check(h, cudaMemcpy(&derr, h->dev_error, 4, cudaMemcpyDeviceToHost), "cudaMemcpy")))
    return st;
  if (derr) return nrs_fail(h, NRS_ERR_TIMEOUT, "ozaki spread estimate: a device-side bounded wait gave up");
  float r;
  std::memcpy(&r, &host[0], 4);
  res->rmax = r;
  res->flags = host[1];
  return NRS_OK;
}

int ozaki_run(nrs_handle* h, const OzOperand& a, const OzOperand& bT, int64_t m, int64_t n, int64_t k,
              int64_t kpad, int b, int S, int kchunks, double* C, int64_t ldc, bool accumulate) {
  auto al = [](size_t v) { return (v + 1023) & ~size_t(1023); };
  // Workspace: exponents | A slices | B slices | digit slots, one 128 x 256
  // x 16-byte slot per CTA (the column maxima of a column-major operand go
  // through the slots first).
  const size_t ea_b = al((size_t)m * 4), eb_b = al((size_t)n * 4);
  const size_t sa_b = al((size_t)S * m * kpad * 2), sb_b = al((size_t)S * n * kpad * 2);
  const int64_t tiles = ((m + OZ_BM - 1) / OZ_BM) * ((n + OZ_BN - 1) / OZ_BN);
  const int64_t ctas = std::min<int64_t>(tiles, h->hw_sms);
  const size_t acc_b = al(std::max((size_t)ctas * OZ_BM * OZ_BN * 16, (size_t)std::max(m, n) * 8));
  int st;
  uint8_t* ws = (uint8_t*)nrs_workspace(h, ea_b + eb_b + sa_b + sb_b + acc_b, &st);
  if (!ws) return st;
  int* ea = (int*)ws;
  int* eb = (int*)(ws + ea_b);
  uint16_t* sa = (uint16_t*)(ws + ea_b + eb_b);
  uint16_t* sb = (uint16_t*)(ws + ea_b + eb_b + sa_b);
  __int128* acc = (__int128*)(ws + ea_b + eb_b + sa_b + sb_b);
  unsigned long long* colmax = reinterpret_cast<unsigned long long*>(acc);
  if ((st = launch_exponents(h, a, k, ea, colmax, nullptr))) return st;
  if ((st = launch_exponents(h, bT, k, eb, colmax, nullptr))) return st;
  if ((st = launch_slices(h, a, k, kpad, ea, b, S, sa))) return st;
  if ((st = launch_slices(h, bT, k, kpad, eb, b, S, sb))) return st;
  OzParams P = base_params(h, m, n, k, kpad);
  P.slices = S;
  P.kchunks = kchunks;
  P.n_pairs = S * (S + 1) / 2 * (kchunks > 0 ? kchunks : 1);
  P.ea = ea;
  P.eb = eb;
  P.acc = acc;
  P.C = C;
  P.ldc = ldc;
  P.final_shift = 2 - 2 * b - b * (S - 1);
  P.digit_bits = b;
  P.kchunk = kChunkOf(b);
  P.accumulate = accumulate ? 1 : 0;
  return launch_tc<false, false>(h, sa, sb, S, P, m, n, h->stream);
}

// ---------------------------------------------------------------------------
// Grouped launch: many f64 problems in one pass of each kernel
// ---------------------------------------------------------------------------
// The problems' slices are stacked: problem p owns rows [rowoff, rowoff + m)
// of the A slices and [coloff, coloff + n) of the B^T slices, all with the
// group's pitch KP (the largest kpad, a multiple of 64); columns [k, kpad) of
// its rows are zero and columns beyond its kpad are never read. One launch
// of each pre-processing kernel covers every problem through a chunk table,
// and one persistent tensor-core launch covers every tile.
struct OzIn {
  const void* A;  // double or float, as the group's element type T
  int64_t lda;
  const void* B;
  int64_t ldb;
  int64_t m, n, k, kpad;
  int64_t rowoff, coloff;
};
struct OzChunk {
  int32_t prob, r0, k0, pad;  // problem, first row (column), first k
};

// Row exponents of every A: one warp per row, 8 rows per block. T (double or
// float) is the group's element type; floats widen to double exactly.
template <typename T>
__global__ void __launch_bounds__(256)
    g_row_exponents(const OzIn* __restrict__ in, const OzChunk* __restrict__ ch, int* __restrict__ ea) {
  const OzChunk c = ch[blockIdx.x];
  const OzIn q = in[c.prob];
  const int64_t row = (int64_t)c.r0 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= q.m) return;
  uint64_t mx = 0;
  for (int64_t j = lane; j < q.k; j += 32) {
    const uint64_t v =
        (uint64_t)__double_as_longlong((double)static_cast<const T*>(q.A)[row * q.lda + j]) & 0x7FFFFFFFFFFFFFFFULL;
    mx = v > mx ? v : mx;
  }
  for (int off = 16; off; off >>= 1) {
    const uint64_t o = __shfl_xor_sync(0xffffffffu, mx, off);
    mx = o > mx ? o : mx;
  }
  if (lane == 0) ea[q.rowoff + row] = ((mx >> 52) == 0) ? -1021 : (int)(mx >> 52) - 1022;
}

// Column maxima of every B: 256 columns x 256 k per block, atomicMax on the
// bit patterns (of the values widened to double) into a zeroed array.
template <typename T>
__global__ void __launch_bounds__(256)
    g_col_max_bits(const OzIn* __restrict__ in, const OzChunk* __restrict__ ch, unsigned long long* __restrict__ colmax) {
  const OzChunk c = ch[blockIdx.x];
  const OzIn q = in[c.prob];
  const int64_t col = (int64_t)c.r0 + threadIdx.x;
  if (col >= q.n) return;
  const int64_t r1 = (c.k0 + kColStrip) < q.k ? (c.k0 + kColStrip) : q.k;
  unsigned long long mx = 0;
  for (int64_t i = c.k0; i < r1; ++i) {
    const unsigned long long v =
        (unsigned long long)__double_as_longlong((double)static_cast<const T*>(q.B)[i * q.ldb + col]) &
        0x7FFFFFFFFFFFFFFFULL;
    mx = v > mx ? v : mx;
  }
  atomicMax(&colmax[q.coloff + col], mx);
}

// A slices of every problem: a block takes 8 rows of one problem, a thread 8
// consecutive k of one row (zero beyond k, up to the problem's kpad).
template <typename T, int b, bool SMALL>
__global__ void __launch_bounds__(256)
    g_slice_rows(const OzIn* __restrict__ in, const OzChunk* __restrict__ ch, const int* __restrict__ ea, int S,
                 int64_t pitch, int64_t plane, uint16_t* __restrict__ out) {
  const OzChunk c = ch[blockIdx.x];
  const OzIn q = in[c.prob];
  const int64_t groups = q.kpad / 8;
  const unsigned __int128 C = digit_offset(S, b);
  const uint64_t C64 = ozaki_offset64(S, b);
  for (int64_t w = threadIdx.x; w < 8 * groups; w += blockDim.x) {
    const int64_t row = (int64_t)c.r0 + w / groups, j0 = (w % groups) * 8;
    if (row >= q.m) break;  // w only grows: every later item is beyond m too
    const int e = ea[q.rowoff + row];
    const T* src = static_cast<const T*>(q.A) + row * q.lda + j0;
    uint16_t* o = out + (q.rowoff + row) * pitch + j0;
    if constexpr (SMALL) {
      OzakiZ64 Z[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) Z[t] = ozaki_z64(j0 + t < q.k ? (double)src[t] : 0.0, e, b, S, C64);
#pragma unroll
      for (int t = 0; t < OZ_MAX_SLICES; ++t) {
        if (t < S) {
          uint32_t pk[4];
#pragma unroll
          for (int hh = 0; hh < 4; ++hh)
            pk[hh] = bf16_of_int(ozaki_digit64<b>(Z[2 * hh], t)) |
                     (bf16_of_int(ozaki_digit64<b>(Z[2 * hh + 1], t)) << 16);
          *reinterpret_cast<uint4*>(o + (int64_t)t * plane) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    } else {
      unsigned __int128 Z[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) Z[t] = (unsigned __int128)fixed126(j0 + t < q.k ? (double)src[t] : 0.0, e) + C;
#pragma unroll
      for (int t = 0; t < OZ_MAX_SLICES; ++t) {
        if (t < S) {
          uint32_t pk[4];
#pragma unroll
          for (int hh = 0; hh < 4; ++hh)
            pk[hh] = bf16_of_int(digit_at<b>(Z[2 * hh], t)) | (bf16_of_int(digit_at<b>(Z[2 * hh + 1], t)) << 16);
          *reinterpret_cast<uint4*>(o + (int64_t)t * plane) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
  }
}

// B^T slices of every problem: slice_cols' 64 k x 32 n transposing tile.
template <typename T, int b, bool SMALL>
__global__ void __launch_bounds__(256)
    g_slice_cols(const OzIn* __restrict__ in, const OzChunk* __restrict__ ch, const int* __restrict__ eb, int S,
                 int64_t pitch, int64_t plane, uint16_t* __restrict__ out) {
  extern __shared__ uint32_t tile[];  // [S][32][33]
  const OzChunk c = ch[blockIdx.x];
  const OzIn q = in[c.prob];
  const int64_t k0 = c.k0, n0 = c.r0;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const unsigned __int128 C = digit_offset(S, b);
  const uint64_t C64 = ozaki_offset64(S, b);
  const T* const Bq = static_cast<const T*>(q.B);
  {
    const int64_t nn = n0 + tx;
    const int e = nn < q.n ? eb[q.coloff + nn] : 0;
#pragma unroll
    for (int r = 0; r < kSliceColK / 16; ++r) {
      const int w = ty + 8 * r;
      const int64_t kk = k0 + 2 * w;
      const double x0 = kk < q.k && nn < q.n ? (double)Bq[kk * q.ldb + nn] : 0.0;
      const double x1 = kk + 1 < q.k && nn < q.n ? (double)Bq[(kk + 1) * q.ldb + nn] : 0.0;
      if constexpr (SMALL) {
        const OzakiZ64 Z0 = ozaki_z64(x0, e, b, S, C64), Z1 = ozaki_z64(x1, e, b, S, C64);
#pragma unroll
        for (int t = 0; t < OZ_MAX_SLICES; ++t)
          if (t < S)
            tile[(t * kSliceColN + tx) * kSliceColPitch + w] =
                bf16_of_int(ozaki_digit64<b>(Z0, t)) | (bf16_of_int(ozaki_digit64<b>(Z1, t)) << 16);
      } else {
        const unsigned __int128 Z0 = (unsigned __int128)fixed126(x0, e) + C;
        const unsigned __int128 Z1 = (unsigned __int128)fixed126(x1, e) + C;
#pragma unroll
        for (int t = 0; t < OZ_MAX_SLICES; ++t)
          if (t < S)
            tile[(t * kSliceColN + tx) * kSliceColPitch + w] =
                bf16_of_int(digit_at<b>(Z0, t)) | (bf16_of_int(digit_at<b>(Z1, t)) << 16);
      }
    }
  }
  __syncthreads();
  const int r = threadIdx.x >> 3, cc = threadIdx.x & 7;
  const int64_t nn = n0 + r, kk = k0 + cc * 8;
  if (nn < q.n && kk < q.kpad) {
    for (int t = 0; t < S; ++t) {
      const uint32_t* src = tile + (t * kSliceColN + r) * kSliceColPitch + cc * 4;
      *reinterpret_cast<uint4*>(out + (int64_t)t * plane + (q.coloff + nn) * pitch + kk) =
          make_uint4(src[0], src[1], src[2], src[3]);
    }
  }
}

}  // namespace

extern "C" int nrs_gemm_ozaki(nrs_handle* h, int64_t m, int64_t k, int64_t n, const double* A,
                              int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc,
                              unsigned flags, int slices, nrs_ozaki_info* info) {
  if (!h) return NRS_ERR_INVALID;
  h->last_error.clear();
  if (m < 0 || k < 0 || n < 0) return nrs_fail(h, NRS_ERR_SHAPE, "negative GEMM dimension");
  if (flags & ~(NRS_GEMM_ACCUMULATE | NRS_GEMM_TRANS_A | NRS_GEMM_TRANS_B))
    return nrs_fail(h, NRS_ERR_INVALID, "unknown GEMM flag");
  const bool ta = flags & NRS_GEMM_TRANS_A, tb = flags & NRS_GEMM_TRANS_B;
  const bool accumulate = flags & NRS_GEMM_ACCUMULATE;
  if (ldc < (n > 0 ? n : 1)) return nrs_fail(h, NRS_ERR_SHAPE, "ldc < n");
  if (lda < ((ta ? m : k) > 0 ? (ta ? m : k) : 1)) return nrs_fail(h, NRS_ERR_SHAPE, "lda too small");
  if (ldb < ((tb ? k : n) > 0 ? (tb ? k : n) : 1)) return nrs_fail(h, NRS_ERR_SHAPE, "ldb too small");
  if (slices < 0 || slices > OZ_MAX_SLICES)
    return nrs_fail(h, NRS_ERR_INVALID, "slices must be 0 (auto) or 1..16");
  const int64_t kpad = ((k + 7) / 8) * 8;
  if (info) std::memset(info, 0, sizeof(*info));
  int b = 0, S = 0, kchunks = 0;
  if (slices > 0) {
    // Widest digits whose int32 diagonal sums stay exact for this K and S.
    for (int cand = 8; cand >= 6 && !b; --cand) {
      const int kc = (int)((kpad + kChunkOf(cand) - 1) / kChunkOf(cand));
      if (digits_fit(cand, slices, kpad, kMaxChunkSlices)) {
        b = cand;
        S = slices;
        kchunks = kc;
      }
    }
    if (!b)
      return nrs_fail(h, NRS_ERR_TOO_LARGE,
                      "k too large for this slice count (ceil(k / 16384) * S must be < 128)");
  }
  if (m == 0 || n == 0) return NRS_OK;
  if (k == 0) {
    if (accumulate) return NRS_OK;
    return nrs_gemm(h, NRS_F64, m, 0, n, A, lda, B, ldb, C, ldc, 0, NRS_GEMM_GENERIC);
  }
  if (!A || !B || !C) return nrs_fail(h, NRS_ERR_INVALID, "null operand");
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  if (m > (1LL << 31) || n > (1LL << 31) || kpad > (1LL << 31))
    return nrs_fail(h, NRS_ERR_TOO_LARGE, "dimension beyond 2^31");
  const OzOperand a{A, lda, m, !ta};
  const OzOperand bT{B, ldb, n, tb};

  auto fallback = [&](const char*) {
    // Native FP64 (DMMA) GEMM: non-finite operands, or a spread that no
    // slice count within the limits covers.
    if (info) {
      info->slices = 0;
      info->products = 0;
      info->est_rel_error = 0.0;
    }
    return nrs_gemm(h, NRS_F64, m, k, n, A, lda, B, ldb, C, ldc, flags, NRS_GEMM_DMMA);
  };

  double spread = 0.0;
  if (slices == 0) {
    SpreadResult r{};
    if ((st = spread_estimate(h, a, bT, m, n, k, kpad, 1, &r))) return st;
    if (r.flags & 1u) return fallback("non-finite operand");
    double need = kTargetBits + (r.rmax > 1.0f ? std::log2((double)r.rmax) : 0.0);
    if (!(std::isfinite((double)r.rmax) && choose_digits(kpad, need, &b, &S, &kchunks))) {
      // The pass-1 numerator counts every k; pass 2 counts only the k where
      // the other operand is nonzero (sparse and structured operands).
      if ((st = spread_estimate(h, a, bT, m, n, k, kpad, 2, &r))) return st;
      need = kTargetBits + (r.rmax > 1.0f ? std::log2((double)r.rmax) : 0.0);
      if (!(std::isfinite((double)r.rmax) && choose_digits(kpad, need, &b, &S, &kchunks))) {
        if (info) info->spread = std::isfinite((double)r.rmax) ? (double)r.rmax : HUGE_VAL;
        return fallback("spread beyond the slice limits");
      }
    }
    spread = r.rmax;
  }
  if (info) {
    info->slices = S;
    info->products = S * (S + 1) / 2 * (kchunks > 0 ? kchunks : 1);
    info->slice_bits = b;
    info->k_chunk = kChunkOf(b);
    info->spread = spread;
    // auto: 2^-(bS) R_max (+ the final rounding); explicit: relative to
    // rowmax|A| colmax|B| k, as no spread was measured
    info->est_rel_error = slices == 0 ? std::ldexp(std::max(spread, 1.0), -b * S) + std::ldexp(1.0, -53)
                                      : std::ldexp(2.0, -b * S);
  }
  return ozaki_run(h, a, bT, m, n, k, kpad, b, S, kchunks, C, ldc, accumulate);
}

// ---------------------------------------------------------------------------
// Grouped launch: host side
// ---------------------------------------------------------------------------
struct nrs_ozaki_group {
  int S = 0, b = 0;
  int f32 = 0;  // element type of the group's problems: float (1) or double (0)
  int64_t pitch = 0, rows_a = 0, rows_b = 0, n_tiles = 0;
  int64_t n_rowch = 0, n_colch = 0, n_slcol = 0;
  void* arena = nullptr;
  OzIn* d_in = nullptr;
  OzChunk *d_rowch = nullptr, *d_colch = nullptr, *d_slcol = nullptr;
  OzProb* d_probs = nullptr;
  OzTile* d_tiles = nullptr;
  int *d_ea = nullptr, *d_eb = nullptr;
  unsigned long long* d_colmax = nullptr;
  uint16_t *d_sa = nullptr, *d_sb = nullptr;
  __int128* d_acc = nullptr;
};

void nrs_ozaki_group_free(nrs_ozaki_group* g) {
  if (!g) return;
  cudaFree(g->arena);
  delete g;
}

int nrs_ozaki_group_info(const nrs_ozaki_group* g, int* slices, int* bits, int64_t* tiles) {
  if (!g) return NRS_ERR_INVALID;
  if (slices) *slices = g->S;
  if (bits) *bits = g->b;
  if (tiles) *tiles = g->n_tiles;
  return NRS_OK;
}

// The row-major GEMMs of element type `dtype` (NRS_F64 or NRS_F32) as one
// group. Slice count for `slices` = 0: each problem's spread measured now
// (one read-back each); the group takes the largest count, carrying each
// operand to 53 + log2(max R) bits for f64 and 26 + log2(max R) (f32's 24
// and two guard bits) for f32. Problems whose spread no count covers, or
// with Inf / NaN, are left out (they stay on the persistent kernel's DMMA or
// FP32 tiles). digit_bits 0 = the widest width the group's K allows.
constexpr double kTargetBits32 = 26.0;
int nrs_ozaki_group_build(nrs_handle* h, int64_t count, const nrs_gemm_desc* d, int dtype, int slices,
                          int digit_bits, int* accepted, nrs_ozaki_group** out) {
  *out = nullptr;
  if (slices < 0 || slices > OZ_MAX_SLICES) return nrs_fail(h, NRS_ERR_INVALID, "slices must be 0 (auto) or 1..16");
  if (digit_bits != 0 && (digit_bits < 6 || digit_bits > 8))
    return nrs_fail(h, NRS_ERR_INVALID, "digit bits must be 0 (widest) or 6..8");
  std::vector<int64_t> idx;
  int64_t kp_max = 0;
  for (int64_t i = 0; i < count; ++i) {
    accepted[i] = 0;
    const nrs_gemm_desc& g = d[i];
    if (g.dtype != dtype || (g.flags & (NRS_GEMM_TRANS_A | NRS_GEMM_TRANS_B)) || g.m <= 0 || g.n <= 0 || g.k <= 0)
      continue;
    idx.push_back(i);
    kp_max = std::max(kp_max, (g.k + OZ_BK - 1) / OZ_BK * OZ_BK);
  }
  if (idx.empty()) return NRS_OK;
  const bool f32 = dtype == NRS_F32;
  const double target = f32 ? kTargetBits32 : kTargetBits;
  double bits_max = target;
  std::vector<int64_t> keep;
  for (int64_t i : idx) {
    const nrs_gemm_desc& g = d[i];
    if (slices > 0) {
      keep.push_back(i);
      continue;
    }
    const int64_t kpad8 = (g.k + 7) / 8 * 8;
    SpreadResult r{};
    const OzOperand a{g.A, g.lda, g.m, true, f32}, bT{g.B, g.ldb, g.n, false, f32};
    int st = spread_estimate(h, a, bT, g.m, g.n, g.k, kpad8, 1, &r);
    if (st) return st;
    if (r.flags & 1u) continue;
    double need = target + (r.rmax > 1.0f ? std::log2((double)r.rmax) : 0.0);
    int bb, SS, kc;
    if (!(std::isfinite((double)r.rmax) && choose_digits(kp_max, need, &bb, &SS, &kc, kMaxChunkSlicesGrouped))) {
      if ((st = spread_estimate(h, a, bT, g.m, g.n, g.k, kpad8, 2, &r))) return st;
      need = target + (r.rmax > 1.0f ? std::log2((double)r.rmax) : 0.0);
      if (!(std::isfinite((double)r.rmax) && choose_digits(kp_max, need, &bb, &SS, &kc, kMaxChunkSlicesGrouped)))
        continue;
    }
    bits_max = std::max(bits_max, need);
    keep.push_back(i);
  }
  if (keep.empty()) return NRS_OK;
  int b = 0, S = 0, kc_max = 0;
  if (digit_bits) {
    // a given width: S from the bits (or as given), if the width's limits hold
    const int s_c = slices > 0 ? slices : std::max(1, (int)std::ceil(bits_max / digit_bits - 1e-9));
    if (digits_fit(digit_bits, s_c, kp_max, kMaxChunkSlicesGrouped)) {
      b = digit_bits;
      S = s_c;
    } else {
      return NRS_OK;  // this width cannot carry the bits: all stay on DMMA
    }
  } else if (slices > 0) {
    for (int cand = 8; cand >= 6 && !b; --cand) {
      const int kc = (int)((kp_max + kChunkOf(cand) - 1) / kChunkOf(cand));
      if (digits_fit(cand, slices, kp_max, kMaxChunkSlicesGrouped)) {
        b = cand;
        S = slices;
        kc_max = kc;
      }
    }
    if (!b) return nrs_fail(h, NRS_ERR_TOO_LARGE, "k too large for this slice count");
  } else if (!choose_digits(kp_max, bits_max, &b, &S, &kc_max, kMaxChunkSlicesGrouped)) {
    return NRS_OK;  // nothing qualifies together: all stay on DMMA
  }
  (void)kc_max;
  // Layout: offsets, chunk tables, tiles (most work first: the persistent
  // kernel hands tiles out round-robin).
  std::vector<OzIn> ins;
  std::vector<OzProb> probs;
  std::vector<OzChunk> rowch, colch, slcol;
  struct TileW {
    double w;
    OzTile t;
  };
  std::vector<TileW> tiles;
  int64_t rowoff = 0, coloff = 0;
  for (int64_t i : keep) {
    const nrs_gemm_desc& g = d[i];
    const int64_t kpad = (g.k + OZ_BK - 1) / OZ_BK * OZ_BK;
    const int p = (int)ins.size();
    ins.push_back(OzIn{g.A, g.lda, g.B, g.ldb, g.m, g.n, g.k, kpad, rowoff, coloff});
    const int kc = (int)((kpad + kChunkOf(b) - 1) / kChunkOf(b));
    probs.push_back(OzProb{g.m, g.n, kpad, rowoff, coloff, g.C, g.ldc, kc, S * (S + 1) / 2 * kc,
                           (g.flags & NRS_GEMM_ACCUMULATE) ? 1 : 0, f32 ? 1 : 0});
    for (int64_t r = 0; r < g.m; r += 8) rowch.push_back(OzChunk{p, (int32_t)r, 0, 0});
    for (int64_t c0 = 0; c0 < g.n; c0 += 256)
      for (int64_t k0 = 0; k0 < g.k; k0 += kColStrip) colch.push_back(OzChunk{p, (int32_t)c0, (int32_t)k0, 0});
    for (int64_t c0 = 0; c0 < g.n; c0 += kSliceColN)
      for (int64_t k0 = 0; k0 < kpad; k0 += kSliceColK) slcol.push_back(OzChunk{p, (int32_t)c0, (int32_t)k0, 0});
    constexpr int kBN = OzGeom<true>::BN;
    const int tm_n = (int)((g.m + OZ_BM - 1) / OZ_BM), tn_n = (int)((g.n + kBN - 1) / kBN);
    for (int a = 0; a < tm_n; ++a)
      for (int c = 0; c < tn_n; ++c) tiles.push_back({(double)kpad * (S * (S + 1) / 2), OzTile{p, a, c, 0}});
    rowoff += g.m;
    coloff += g.n;
  }
  std::stable_sort(tiles.begin(), tiles.end(), [](const TileW& x, const TileW& y) { return x.w > y.w; });
  std::vector<OzTile> tl(tiles.size());
  for (size_t i = 0; i < tiles.size(); ++i) tl[i] = tiles[i].t;
  if (rowoff > (1LL << 31) || coloff > (1LL << 31) || (int64_t)tl.size() > (1LL << 30))
    return NRS_OK;  // beyond the tensor maps' coordinate range: stay on DMMA
  auto al = [](size_t v) { return (v + 255) & ~size_t(255); };
  const size_t b_in = al(ins.size() * sizeof(OzIn)), b_rc = al(rowch.size() * sizeof(OzChunk)),
               b_cc = al(colch.size() * sizeof(OzChunk)), b_sc = al(slcol.size() * sizeof(OzChunk)),
               b_pr = al(probs.size() * sizeof(OzProb)), b_tl = al(tl.size() * sizeof(OzTile)),
               b_ea = al((size_t)rowoff * 4), b_eb = al((size_t)coloff * 4), b_cm = al((size_t)coloff * 8),
               b_sa = al((size_t)S * rowoff * kp_max * 2), b_sb = al((size_t)S * coloff * kp_max * 2),
               b_acc = al((size_t)h->hw_sms * OZ_BM * OzGeom<true>::BN * OZ_DIGIT_BYTES);  // a digit slot per CTA
  const size_t total = b_in + b_rc + b_cc + b_sc + b_pr + b_tl + b_ea + b_eb + b_cm + b_sa + b_sb + b_acc;
  nrs_ozaki_group* G = new nrs_ozaki_group();
  if (cudaMalloc(&G->arena, total) != cudaSuccess) {
    cudaGetLastError();
    delete G;
    return nrs_fail(h, NRS_ERR_ALLOC, "grouped Ozaki buffers");
  }
  uint8_t* q = (uint8_t*)G->arena;
  auto take = [&](size_t bytes) {
    uint8_t* p = q;
    q += bytes;
    return p;
  };
  G->d_in = (OzIn*)take(b_in);
  G->d_rowch = (OzChunk*)take(b_rc);
  G->d_colch = (OzChunk*)take(b_cc);
  G->d_slcol = (OzChunk*)take(b_sc);
  G->d_probs = (OzProb*)take(b_pr);
  G->d_tiles = (OzTile*)take(b_tl);
  G->d_ea = (int*)take(b_ea);
  G->d_eb = (int*)take(b_eb);
  G->d_colmax = (unsigned long long*)take(b_cm);
  G->d_sa = (uint16_t*)take(b_sa);
  G->d_sb = (uint16_t*)take(b_sb);
  G->d_acc = (__int128*)take(b_acc);
  G->S = S;
  G->b = b;
  G->f32 = f32 ? 1 : 0;
  G->pitch = kp_max;
  G->rows_a = rowoff;
  G->rows_b = coloff;
  G->n_tiles = (int64_t)tl.size();
  G->n_rowch = (int64_t)rowch.size();
  G->n_colch = (int64_t)colch.size();
  G->n_slcol = (int64_t)slcol.size();
  cudaError_t e = cudaSuccess;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (!e && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  };
  up(G->d_in, ins.data(), ins.size() * sizeof(OzIn));
  up(G->d_rowch, rowch.data(), rowch.size() * sizeof(OzChunk));
  up(G->d_colch, colch.data(), colch.size() * sizeof(OzChunk));
  up(G->d_slcol, slcol.data(), slcol.size() * sizeof(OzChunk));
  up(G->d_probs, probs.data(), probs.size() * sizeof(OzProb));
  up(G->d_tiles, tl.data(), tl.size() * sizeof(OzTile));
  if (e) {
    nrs_ozaki_group_free(G);
    return nrs_cuda_check(h, e, "cudaMemcpy(grouped Ozaki tables)");
  }
  for (int64_t i : keep) accepted[i] = 1;
  *out = G;
  return NRS_OK;
}

template <typename T, int b, bool SMALL>
int group_slices_s(nrs_handle* h, nrs_ozaki_group* G, cudaStream_t s) {
  const int64_t plane_a = G->rows_a * G->pitch, plane_b = G->rows_b * G->pitch;
  g_slice_rows<T, b, SMALL><<<(unsigned)G->n_rowch, 256, 0, s>>>(G->d_in, G->d_rowch, G->d_ea, G->S, G->pitch,
                                                                 plane_a, G->d_sa);
  const int smem = (int)((size_t)G->S * kSliceColN * kSliceColPitch * 4);
  int st = nrs_cuda_check(
      h, cudaFuncSetAttribute(g_slice_cols<T, b, SMALL>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
      "cudaFuncSetAttribute(g_slice_cols)");
  if (st) return st;
  g_slice_cols<T, b, SMALL><<<(unsigned)G->n_slcol, 256, smem, s>>>(G->d_in, G->d_slcol, G->d_eb, G->S, G->pitch,
                                                                   plane_b, G->d_sb);
  return nrs_after_launch(h, "grouped ozaki slicing");
}
template <typename T, int b>
int group_slices(nrs_handle* h, nrs_ozaki_group* G, cudaStream_t s) {
  return b * G->S <= 64 ? group_slices_s<T, b, true>(h, G, s) : group_slices_s<T, b, false>(h, G, s);
}

template <typename T>
int group_prepare(nrs_handle* h, nrs_ozaki_group* G, cudaStream_t s) {
  g_row_exponents<T><<<(unsigned)G->n_rowch, 256, 0, s>>>(G->d_in, G->d_rowch, G->d_ea);
  g_col_max_bits<T><<<(unsigned)G->n_colch, 256, 0, s>>>(G->d_in, G->d_colch, G->d_colmax);
  exponents_from_bits<<<(unsigned)((G->rows_b + 255) / 256), 256, 0, s>>>(G->d_colmax, G->rows_b, G->d_eb, nullptr);
  int st = nrs_after_launch(h, "grouped ozaki exponents");
  if (st) return st;
  return G->b == 8 ? group_slices<T, 8>(h, G, s) : G->b == 7 ? group_slices<T, 7>(h, G, s)
                                                             : group_slices<T, 6>(h, G, s);
}

// Enqueues the whole group on `s` (no host synchronisation).
int nrs_ozaki_group_launch(nrs_handle* h, nrs_ozaki_group* G, cudaStream_t s) {
  if (!G || G->n_tiles == 0) return NRS_OK;
  int st = nrs_cuda_check(h, cudaMemsetAsync(G->d_colmax, 0, (size_t)G->rows_b * 8, s), "cudaMemsetAsync");
  if (st) return st;
  st = G->f32 ? group_prepare<float>(h, G, s) : group_prepare<double>(h, G, s);
  if (st) return st;
  OzParams P{};
  P.kpad = G->pitch;
  P.slices = G->S;
  P.group_m = 1;
  P.ea = G->d_ea;
  P.eb = G->d_eb;
  P.acc = G->d_acc;
  P.final_shift = 2 - 2 * G->b - G->b * (G->S - 1);
  P.digit_bits = G->b;
  P.kchunk = kChunkOf(G->b);
  P.err = h->dev_error;
  P.tiles = G->d_tiles;
  P.probs = G->d_probs;
  P.n_tiles = (int)G->n_tiles;
  return launch_tc<false, true>(h, G->d_sa, G->d_sb, G->S, P, G->rows_a, G->rows_b, s);
}

extern "C" int nrs_gemm_ozaki_grouped(nrs_handle* h, int64_t count, const nrs_gemm_desc* descs, int slices,
                                      int* on_tensor_cores, nrs_ozaki_info* info) {
  if (!h || count < 0 || (count && !descs)) return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  for (int64_t i = 0; i < count; ++i) {
    const nrs_gemm_desc& g = descs[i];
    if (g.dtype != NRS_F64) return nrs_fail(h, NRS_ERR_DTYPE, "grouped Ozaki takes f64 GEMMs");
    if (g.flags & ~(NRS_GEMM_ACCUMULATE | NRS_GEMM_TRANS_A | NRS_GEMM_TRANS_B))
      return nrs_fail(h, NRS_ERR_INVALID, "unknown GEMM flag");
    const bool ta = g.flags & NRS_GEMM_TRANS_A, tb = g.flags & NRS_GEMM_TRANS_B;
    if (g.m < 0 || g.k < 0 || g.n < 0) return nrs_fail(h, NRS_ERR_SHAPE, "negative GEMM dimension");
    if (g.ldc < (g.n > 0 ? g.n : 1) || g.lda < ((ta ? g.m : g.k) > 0 ? (ta ? g.m : g.k) : 1) ||
        g.ldb < ((tb ? g.k : g.n) > 0 ? (tb ? g.k : g.n) : 1))
      return nrs_fail(h, NRS_ERR_SHAPE, "leading dimension too small");
    if (g.m * g.n > 0 && (!g.C || (g.k > 0 && (!g.A || !g.B)))) return nrs_fail(h, NRS_ERR_INVALID, "null operand");
  }
  std::vector<int> acc((size_t)count);
  nrs_ozaki_group* G = nullptr;
  if ((st = nrs_ozaki_group_build(h, count, descs, NRS_F64, slices, 0, acc.data(), &G))) return st;
  if (info) {
    std::memset(info, 0, sizeof(*info));
    if (G) {
      info->slices = G->S;
      info->slice_bits = G->b;
      info->k_chunk = kChunkOf(G->b);
      info->products = (int32_t)G->n_tiles;
    }
  }
  // the problems the group does not take run one by one on DMMA
  for (int64_t i = 0; i < count && st == NRS_OK; ++i) {
    if (on_tensor_cores) on_tensor_cores[i] = acc[i];
    if (!acc[i]) {
      const nrs_gemm_desc& g = descs[i];
      st = nrs_gemm(h, NRS_F64, g.m, g.k, g.n, g.A, g.lda, g.B, g.ldb, g.C, g.ldc, g.flags, NRS_GEMM_DMMA);
    }
  }
  if (st == NRS_OK && G) st = nrs_ozaki_group_launch(h, G, h->stream);
  if (G) {
    cudaStreamSynchronize(h->stream);  // the group's buffers are freed below
    nrs_ozaki_group_free(G);
  }
  return st;
}
