"""The grouped Ozaki epilogue's exact element total and its 128-bit integer
-> f64 / f32 conversions (numrs_gb300/csrc/f64_round.cuh, host/device code),
compiled for the host with g++: the exact path and the straight-line fast
path against exact rational rounding (round to nearest, ties to even) over
random magnitudes and scales, ties, carries into the next binade, overflow
to infinity and the subnormal range; the total T = R 2^(b(S-1)) +
sum_t digit_t 2^(bt) against Python integers for every digit width; and
the int64 order keys of doubles (max / min / argmax kernels) against
Python's float order."""
import ctypes
import os
import random
import shutil
import struct
import subprocess
from fractions import Fraction

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(HERE, "..", "numrs_gb300", "csrc", "f64_round.cuh")

HARNESS = r"""
#include "f64_round.cuh"
extern "C" double nrs_test_int128_to_f64(uint64_t hi, uint64_t lo, int e, int neg) {
  return int128_to_f64(neg != 0, hi, lo, e);
}
extern "C" uint64_t nrs_test_fast(uint64_t hi, uint64_t lo, int e, int neg, int* special) {
  bool sp = false;
  const uint64_t r = int128_to_f64_bits_fast(neg != 0, hi, lo, e, sp);
  *special = sp;
  return r;
}
extern "C" uint32_t nrs_test_f32(uint64_t hi, uint64_t lo, int e, int neg, int fast, int* special) {
  bool sp = false;
  uint64_t r;
  if (fast) {
    r = int128_to_float_bits_fast<NrsF32Fmt>(neg != 0, hi, lo, e, sp);
  } else {
    r = int128_to_float_bits<NrsF32Fmt>(neg != 0, hi, lo, e);
  }
  *special = sp;
  return (uint32_t)r;
}
extern "C" void nrs_test_digits64(double x, int e, int b, int S, int* out) {
  const OzakiZ64 z = ozaki_z64(x, e, b, S, ozaki_offset64(S, b));
  for (int t = 0; t < S; ++t)
    out[t] = b == 8 ? ozaki_digit64<8>(z, t) : b == 7 ? ozaki_digit64<7>(z, t) : ozaki_digit64<6>(z, t);
}
extern "C" int64_t nrs_test_key(uint64_t u) { return nrs_f64_key(u); }
extern "C" int nrs_test_nan_or_zero(uint64_t u) { return nrs_f64_nan_or_zero(u); }
extern "C" int nrs_test_is_nan(uint64_t u) { return nrs_f64_is_nan(u); }
extern "C" void nrs_test_total(int32_t R, uint64_t lo, uint64_t hi, int b, int S, int* neg, uint64_t* mhi,
                               uint64_t* mlo) {
  bool n = false;
  ozaki_exact_total(R, lo, hi, b, S, n, *mhi, *mlo);
  *neg = n;
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("f64round")
    src, so = d / "h.cpp", d / "h.so"
    src.write_text(HARNESS)
    subprocess.run([cxx, "-O2", "-shared", "-fPIC", "-I", os.path.dirname(HDR), str(src), "-o", str(so)],
                   check=True, capture_output=True)
    return ctypes.CDLL(str(so))


@pytest.fixture(scope="module")
def conv(lib):
    f = lib.nrs_test_int128_to_f64
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
    return lambda m, e, neg: f(m >> 64, m & ((1 << 64) - 1), e, neg)


def _exact(m, e, neg):
    if m == 0:
        return -0.0 if neg else 0.0
    try:
        v = float(Fraction(m) * Fraction(2) ** e)
    except OverflowError:
        v = float("inf")
    return -v if neg else v


def _cases():
    r = random.Random(5)
    out = []
    for _ in range(60000):
        bits = r.randint(0, 128)
        m = r.getrandbits(bits) if bits else r.randint(0, 3)
        e = r.choice([r.randint(-200, 200), r.randint(-1250, -1000), r.randint(900, 1100)])
        out.append((m, e, r.randint(0, 1)))
    for k in range(54, 128):
        base = 1 << k
        for e in (-1100, -1074, -1022 - k, -1023 - k, 0, 1023 - k, 1024 - k):
            for m in (base | (1 << (k - 53)), base | (3 << (k - 54)), (1 << (k + 1)) - 1,
                      base | (1 << (k - 53)) | 1, base + (1 << (k - 53)) - 1):
                out += [(m, e, 0), (m, e, 1)]
    out += [((1 << 127) + 1, -1202, 0), (1 << 127, -1202, 0), ((1 << 128) - 1, -1202, 1)]
    return out


def test_int128_to_f64_rounds_exactly(conv):
    bad = []
    for m, e, neg in _cases():
        got, want = conv(m, e, neg), _exact(m, e, neg)
        if not (got == want and repr(got) == repr(want)):
            bad.append((hex(m), e, neg, got, want))
    assert not bad, bad[:5]


def test_fast_path_matches_exact_or_defers(lib, conv):
    """The straight-line path gives the exact path's bits, or flags the
    element (zero, subnormal, overflow) for it."""
    f = lib.nrs_test_fast
    f.restype = ctypes.c_uint64
    f.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    sp = ctypes.c_int()
    n_fast = 0
    for m, e, neg in _cases():
        bits = f(m >> 64, m & ((1 << 64) - 1), e, neg, ctypes.byref(sp))
        if sp.value:
            continue
        n_fast += 1
        want = struct.unpack("<Q", struct.pack("<d", _exact(m, e, neg)))[0]
        assert bits == want, (hex(m), e, neg, hex(bits), hex(want))
    assert n_fast > 30000  # the rest: zero, subnormal or overflowing (a third of the mix)


@pytest.mark.parametrize("b", [8, 7, 6])
def test_exact_total_every_width(lib, b):
    f = lib.nrs_test_total
    f.restype = None
    f.argtypes = [ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    r = random.Random(b)
    neg, mhi, mlo = ctypes.c_int(), ctypes.c_uint64(), ctypes.c_uint64()
    for S in range(1, 17):
        if b * (S - 1) > 95:
            continue
        for _ in range(400):
            R = r.choice([r.randint(-(1 << 31), (1 << 31) - 1), r.randint(-3, 3)])
            digits = [r.randrange(1 << b) for _ in range(S - 1)]
            rec = sum(d << (8 * t) for t, d in enumerate(digits))
            rec |= r.getrandbits(128) >> (8 * (S - 1)) << (8 * (S - 1)) if S - 1 < 16 else 0  # junk above
            T = R * (1 << (b * (S - 1))) + sum(d << (b * t) for t, d in enumerate(digits))
            f(R, rec & ((1 << 64) - 1), rec >> 64, b, S, ctypes.byref(neg), ctypes.byref(mhi), ctypes.byref(mlo))
            got = (mhi.value << 64 | mlo.value) * (-1 if neg.value else 1)
            assert got == T and bool(neg.value) == (T < 0), (b, S, R, digits)


def _f32_bits(m, e, neg):
    """Round m 2^e to binary32 (nearest, ties to even) with integers only."""
    sign = (1 << 31) if neg else 0
    if m == 0:
        return sign

    def rne(num, sh):  # round(num / 2^sh), ties to even (sh may be <= 0)
        if sh <= 0:
            return num << -sh
        q, r = num >> sh, num & ((1 << sh) - 1)
        half = 1 << (sh - 1)
        return q + 1 if r > half or (r == half and q & 1) else q

    p = m.bit_length() - 1
    if p + e >= -126:
        mant = rne(m, p - 23)  # 24 bits (or 2^24 after a carry)
        E = p + e
        if mant >> 24:
            mant >>= 1
            E += 1
        if E > 127:
            return sign | 0x7F800000
        return sign | (E + 127) << 23 | (mant & 0x7FFFFF)
    return sign | rne(m, -(e + 149))  # subnormal grid 2^-149 (2^-126 after a carry)


def test_int128_to_f32_exact_and_fast(lib):
    f = lib.nrs_test_f32
    f.restype = ctypes.c_uint32
    f.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.POINTER(ctypes.c_int)]
    r = random.Random(9)
    sp = ctypes.c_int()
    cases = []
    for _ in range(40000):
        bits = r.randint(0, 128)
        m = r.getrandbits(bits) if bits else r.randint(0, 3)
        cases.append((m, r.choice([r.randint(-100, 60), r.randint(-300, -130), r.randint(-40, 140)]), r.randint(0, 1)))
    for k in range(25, 127):
        for e in (-149 - k, -126 - k, -127 - k, 0, 127 - k, 128 - k):
            base = 1 << k
            for m in (base | (1 << (k - 24)), base | (3 << (k - 25)), (1 << (k + 1)) - 1, base | (1 << (k - 24)) | 1):
                cases += [(m, e, 0), (m, e, 1)]
    n_fast = 0
    for m, e, neg in cases:
        want = _f32_bits(m, e, neg)
        got = f(m >> 64, m & ((1 << 64) - 1), e, neg, 0, ctypes.byref(sp))
        assert got == want, ("exact", hex(m), e, neg, hex(got), hex(want))
        got = f(m >> 64, m & ((1 << 64) - 1), e, neg, 1, ctypes.byref(sp))
        if not sp.value:
            n_fast += 1
            assert got == want, ("fast", hex(m), e, neg, hex(got), hex(want))
    assert n_fast > 10000


def _digits128(x, e, b, S):
    """The slicers' 128-bit digits: X = x 2^(126-e), Z = X + 2^(p-1) +
    h sum_t 2^(p_t), digit t = field t of Z minus h (p_t = 127 - b - bt)."""
    X = int(Fraction(x) * Fraction(2) ** (126 - e))  # exact for |x| < 2^e
    h = 1 << (b - 1)
    p = [127 - b - b * t for t in range(S)]
    Z = X + (1 << (p[S - 1] - 1)) + sum(h << pt for pt in p)
    return [((Z >> p[t]) if t == 0 else ((Z >> p[t]) & ((1 << b) - 1))) - h for t in range(S)]


@pytest.mark.parametrize("b", [8, 7, 6])
def test_slice_digits64_equal_the_128bit_digits(lib, b):
    """The 64-bit slicing form gives the 128-bit form's digits for every
    b S <= 64: random doubles of every magnitude below 2^e (subnormals and
    zeros included), rounding ties, and values next to the row maximum."""
    import math
    f = lib.nrs_test_digits64
    f.restype = None
    f.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    out = (ctypes.c_int * 16)()
    r = random.Random(100 + b)
    for S in range(1, 17):
        if b * S > 64:
            continue
        xs = []
        for _ in range(300):
            e = r.randint(-1060, 1000)
            xs.append((r.uniform(-1, 1) * 2.0 ** (e - r.choice([0, 0, 1, 5, 20, 60])), e))
        xs += [(0.0, 3), (-0.0, 3), (5e-324, -1021), (-5e-324, -1021), (math.ldexp(1 - 2 ** -53, 7), 7),
               (-math.ldexp(1 - 2 ** -53, 7), 7), (math.ldexp(1, -b * S), 1), (-math.ldexp(1, -b * S), 1),
               (math.ldexp(3, -b * S - 1), 1), (-math.ldexp(3, -b * S - 1), 1)]
        for x, e in xs:
            assert abs(x) < 2.0 ** e
            f(x, e, b, S, out)
            assert list(out[:S]) == _digits128(x, e, b, S), (x, e, b, S)


def test_f64_order_keys(lib):
    """nrs_f64_key orders doubles that are neither NaN nor zero exactly as
    floats, equal keys only for equal bits, and maps back to the bits by the
    same operation; nrs_f64_nan_or_zero / nrs_f64_is_nan classify every
    class of double (signed zeros, subnormals, infinities, quiet and
    signalling NaNs of both signs)."""
    key, noz, isn = lib.nrs_test_key, lib.nrs_test_nan_or_zero, lib.nrs_test_is_nan
    key.restype = ctypes.c_int64
    key.argtypes = [ctypes.c_uint64]
    for f in (noz, isn):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_uint64]
    bits_of = lambda d: struct.unpack("<Q", struct.pack("<d", d))[0]  # noqa: E731
    r = random.Random(17)
    vals = [r.uniform(-1, 1) * 2.0 ** r.randint(-1074, 1023) for _ in range(4000)]
    vals += [5e-324, -5e-324, 2.2250738585072014e-308, -2.2250738585072014e-308, 1.7976931348623157e308,
             -1.7976931348623157e308, float("inf"), float("-inf"), 1.0, -1.0, 0.5, -0.5]
    vals = [v for v in vals if v != 0.0]
    keyed = [(key(bits_of(v)), v) for v in vals]
    for k, v in keyed:
        assert key(k & ((1 << 64) - 1)) & ((1 << 64) - 1) == bits_of(v)  # involution
    keyed.sort()
    for (k1, v1), (k2, v2) in zip(keyed, keyed[1:]):
        assert v1 <= v2 and (k1 == k2) == (bits_of(v1) == bits_of(v2))
    nans = [0x7FF8000000000000, 0xFFF8000000000000, 0x7FF0000000000001, 0xFFF0000000000001, 0x7FFFFFFFFFFFFFFF]
    for u in nans:
        assert noz(u) and isn(u)
    for u in (0, 1 << 63):
        assert noz(u) and not isn(u)
    for v in vals:
        assert not noz(bits_of(v)) and not isn(bits_of(v))
