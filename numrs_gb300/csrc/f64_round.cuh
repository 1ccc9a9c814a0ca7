// The grouped Ozaki epilogue's exact total of a C element and its 128-bit
// integer to f64 / f32 conversion, and the int64 order keys of doubles used
// by the max / min / argmax kernels, written for host and device alike so
// that the CPU tests check the same code the kernels run.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define NRS_HD __host__ __device__ __forceinline__
#else
#define NRS_HD inline
#endif

NRS_HD int nrs_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

NRS_HD double nrs_f64_from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

NRS_HD float nrs_f32_from_bits(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, sizeof f);
  return f;
#endif
}

// Binary floating-point formats: WIDTH bits, MANT stored mantissa bits, BIAS
// exponent bias, EMAX the all-ones biased exponent (infinity).
struct NrsF64Fmt {
  static constexpr int WIDTH = 64, MANT = 52, BIAS = 1023, EMAX = 2047;
};
struct NrsF32Fmt {
  static constexpr int WIDTH = 32, MANT = 23, BIAS = 127, EMAX = 255;
};

// (-1)^neg (mhi:mlo) 2^e rounded to nearest (ties to even) in format F, the
// bit pattern assembled with integer operations: GB300's FP64 pipe runs a
// few operations per clock per SM, which a per-element int-to-double
// conversion and scaling would saturate. Subnormal results take an exact
// 128-bit shift-and-round path; overflow gives infinity.
template <typename F>
NRS_HD uint64_t int128_to_float_bits(bool neg, uint64_t mhi, uint64_t mlo, int e) {
  constexpr int W = F::WIDTH;
  const uint64_t sign = (uint64_t)neg << (W - 1);
  if ((mhi | mlo) == 0) return sign;
  int p;         // position of the leading one
  uint64_t top;  // the 64 bits from the leading one down, left-aligned
  bool below;    // any one bit below those 64
  if (mhi) {
    const int lz = nrs_clz64(mhi);
    p = 127 - lz;
    top = lz ? (mhi << lz) | (mlo >> (64 - lz)) : mhi;
    below = (lz ? mlo << lz : mlo) != 0;
  } else {
    const int lz = nrs_clz64(mlo);
    p = 63 - lz;
    top = mlo << lz;
    below = false;
  }
  constexpr int DROP = 63 - F::MANT;  // bits of `top` below the mantissa
  const int be = p + e + F::BIAS;     // biased exponent of the leading one
  if (be > 0) {
    uint64_t mant = top >> DROP;  // MANT + 1 bits
    const bool rnd = (top >> (DROP - 1)) & 1, sticky = (top & ((1ull << (DROP - 1)) - 1)) != 0 || below;
    int pe = be;
    if (rnd && (sticky || (mant & 1))) {
      if (++mant >> (F::MANT + 1)) {
        mant >>= 1;
        ++pe;
      }
    }
    if (pe >= F::EMAX) return sign | (uint64_t)F::EMAX << F::MANT;
    return sign | (uint64_t)pe << F::MANT | (mant & ((1ull << F::MANT) - 1));
  }
  // subnormal (or zero after rounding): the value in units of the smallest
  // subnormal, 2^(1 - BIAS - MANT)
  const unsigned __int128 m = (unsigned __int128)mhi << 64 | mlo;
  const int sh = -(e + F::BIAS - 1 + F::MANT);  // right shift onto the subnormal grid
  uint64_t q;
  if (sh <= 0) {
    q = (uint64_t)(m << -sh);  // exact: below 2^MANT here
  } else if (sh >= 128) {
    q = sh == 128 && m > ((unsigned __int128)1 << 127) ? 1 : 0;  // at most one unit
  } else {
    q = (uint64_t)(m >> sh);
    const unsigned __int128 rem = m & (((unsigned __int128)1 << sh) - 1), half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) ++q;
  }
  return sign | q;
}

NRS_HD double int128_to_f64(bool neg, uint64_t mhi, uint64_t mlo, int e) {
  return nrs_f64_from_bits(int128_to_float_bits<NrsF64Fmt>(neg, mhi, mlo, e));
}
NRS_HD float int128_to_f32(bool neg, uint64_t mhi, uint64_t mlo, int e) {
  return nrs_f32_from_bits((uint32_t)int128_to_float_bits<NrsF32Fmt>(neg, mhi, mlo, e));
}

// The same conversion without branches for the common case, so that several
// elements' operation chains interleave: returns the bits when the magnitude
// is nonzero and the result normal and finite; otherwise sets `special` (the
// caller then uses int128_to_float_bits).
template <typename F>
NRS_HD uint64_t int128_to_float_bits_fast(bool neg, uint64_t mhi, uint64_t mlo, int e, bool& special) {
  constexpr int W = F::WIDTH;
  constexpr int DROP = 63 - F::MANT;
  const bool hz = mhi == 0;
  const uint64_t x = hz ? mlo : mhi;
  const int lz = nrs_clz64(x | 1);  // (x = 0 is special below)
  const int p = (hz ? 63 : 127) - lz;
  const uint64_t hi_part = (mhi << lz) | ((mlo >> 1) >> (63 - lz));
  const uint64_t top = hz ? mlo << lz : hi_part;
  const uint64_t below = hz ? 0 : mlo << lz;
  uint64_t mant = top >> DROP;
  const uint64_t rnd = (top >> (DROP - 1)) & 1;
  const uint64_t sticky = ((top & ((1ull << (DROP - 1)) - 1)) | below) != 0;
  mant += rnd & (sticky | (mant & 1));
  const uint64_t carry = mant >> (F::MANT + 1);
  mant >>= carry;
  const int pe = p + e + F::BIAS + (int)carry;
  special = (x == 0) | (pe <= 0) | (pe >= F::EMAX);
  return (uint64_t)neg << (W - 1) | (uint64_t)(pe & F::EMAX) << F::MANT | (mant & ((1ull << F::MANT) - 1));
}
NRS_HD uint64_t int128_to_f64_bits_fast(bool neg, uint64_t mhi, uint64_t mlo, int e, bool& special) {
  return int128_to_float_bits_fast<NrsF64Fmt>(neg, mhi, mlo, e, special);
}

// The exact total T = R 2^(b(S-1)) + sum_t digit_t 2^(bt) of a grouped Ozaki
// element (R: the carried int32 sum, digit t = byte t of lo | hi << 64,
// digits below 2^b) as sign and 128-bit magnitude. For b = 8 the digits are
// the bytes themselves: T = R 2^(8(S-1)) + (the record's low 8(S-1) bits),
// straight-line; other widths fold them in by Horner's rule,
// T = ((R 2^b + digit_{S-2}) 2^b + ...) 2^b + digit_0.
NRS_HD void ozaki_exact_total(int32_t R, uint64_t lo, uint64_t hi, int b, int S, bool& neg, uint64_t& mhi,
                              uint64_t& mlo) {
  const int nd = S - 1;
  const uint64_t r64 = (uint64_t)(int64_t)R;
  const uint64_t high = (uint64_t)((int64_t)R >> 63);
  uint64_t th, tl;
  if (b == 8) {
    const int sh = 8 * nd;  // 0..112
    const bool small = sh < 64;
    const int s1 = small ? sh : 0, s2 = small ? 0 : sh - 64;
    const uint64_t lmask = (~0ull >> 1) >> (63 - s1);  // the low s1 bits
    const uint64_t hmask = (~0ull >> 1) >> (63 - s2);  // the low s2 bits
    tl = small ? (r64 << s1) | (lo & lmask) : lo;
    th = small ? (high << s1) | ((r64 >> 1) >> (63 - s1)) : (r64 << s2) | (hi & hmask);
  } else {
    th = high;
    tl = r64;
    for (int t = nd - 1; t >= 0; --t) {
      const uint64_t dg = (t < 8 ? lo >> (8 * t) : hi >> (8 * (t - 8))) & 0xFF;
      th = (th << b) | (tl >> (64 - b));
      tl = (tl << b) | dg;
    }
  }
  neg = (int64_t)th < 0;
  mlo = neg ? ~tl + 1 : tl;
  mhi = neg ? ~th + (tl == 0 ? 1 : 0) : th;
}

// ---------------------------------------------------------------------------
// Slicing with 64-bit integers when b S <= 64
// ---------------------------------------------------------------------------
// The slicers round X = x 2^(126-e) (exact for |x| < 2^e) to a multiple of
// 2^p, p = 127 - bS (ties up), and read S signed b-bit digits off
// Z = X + 2^(p-1) + h sum_t 2^(p_t) (h = 2^(b-1), p_t = 127 - b - bt). With
// b S <= 64 the same digits come from 64-bit arithmetic:
//   Y = floor((X + 2^(p-1)) / 2^p) = round-half-up(x 2^(bS-1-e)), |Y| < 2^63,
//   Z' = Y + h sum_t 2^(b(S-1-t)) = Z >> p  (0 <= Z' < 2^(bS+1)),
// digit t = field t of Z' minus h; the top field can need a ninth bit (bit
// bS of Z', or for b S = 64 the carry-out of the add).
NRS_HD int64_t ozaki_round_y(double x, int e, int bS) {
  uint64_t bits;
  memcpy(&bits, &x, sizeof bits);
  const bool neg = bits >> 63;
  const int biased = (int)((bits >> 52) & 0x7FF);
  uint64_t mant = bits & 0xFFFFFFFFFFFFFull;
  int E;
  if (biased == 0) {
    E = -1074;
  } else {
    mant |= 1ull << 52;
    E = biased - 1075;  // x = mant 2^E
  }
  if (mant == 0) return 0;
  const int sh = E + bS - 1 - e;
  if (sh >= 0) {  // exact; below 2^63 because |x| < 2^e
    const int64_t m = (int64_t)(mant << sh);
    return neg ? -m : m;
  }
  const int k = -sh;
  if (k >= 64) return 0;  // |x 2^(bS-1-e)| < 2^-11
  const uint64_t half = 1ull << (k - 1);
  // floor((+-mant 2^-k) + 1/2): up for a positive half, toward zero for a negative one
  return neg ? -(int64_t)((mant + half - 1) >> k) : (int64_t)((mant + half) >> k);
}

NRS_HD uint64_t ozaki_offset64(int S, int b) {
  uint64_t c = 0;
  for (int t = 0; t < S; ++t) c += (uint64_t)1 << (b - 1) << (b * (S - 1 - t));
  return c;
}

// Z' left-aligned (digit t in bits [64 - b(t+1), 64 - bt)) and the carry-out
// of Y + offset, from which ozaki_digit64 reads digit t.
struct OzakiZ64 {
  uint64_t z;
  uint32_t carry;
};
NRS_HD OzakiZ64 ozaki_z64(double x, int e, int b, int S, uint64_t offset) {
  const int bS = b * S;
  const int64_t Y = ozaki_round_y(x, e, bS);
  const uint64_t z = (uint64_t)Y + offset;
  OzakiZ64 r;
  // the top field's ninth bit: bit bS of Z' (below 2^(bS+1)), or for
  // b S = 64 the carry-out of the 64-bit add
  r.carry = bS < 64 ? (uint32_t)((z >> bS) & 1) : (uint32_t)((Y >= 0) && (z < offset));
  r.z = bS < 64 ? z << (64 - bS) : z;
  return r;
}
template <int B>
NRS_HD int ozaki_digit64(const OzakiZ64& z, int t) {
  const int f = (int)(uint32_t)(z.z >> (64 - B * (t + 1)));
  return (t == 0 ? (f | (int)(z.carry << B)) : (f & ((1 << B) - 1))) - (1 << (B - 1));
}

// ---------------------------------------------------------------------------
// f64 order on the integer pipe
// ---------------------------------------------------------------------------
// For doubles that are neither NaN nor zero, a < b exactly when
// nrs_f64_key(a) < nrs_f64_key(b) as int64 (the magnitude bits of negatives
// flipped), and equal keys mean equal bits; the key maps back to the bits by
// the same operation.
NRS_HD int64_t nrs_f64_key(uint64_t u) { return (int64_t)(u ^ ((uint64_t)((int64_t)u >> 63) >> 1)); }
// NaN or a zero: the magnitude bits minus one, unsigned, reach the infinity
// pattern (zero wraps around).
NRS_HD bool nrs_f64_nan_or_zero(uint64_t u) {
  return ((u & 0x7FFFFFFFFFFFFFFFull) - 1u) >= 0x7FF0000000000000ull;
}
NRS_HD bool nrs_f64_is_nan(uint64_t u) { return (u & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull; }
