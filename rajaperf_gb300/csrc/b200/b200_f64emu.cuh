// Exactly rounded FP64 add and multiply on the integer pipe.
//
// GB300 issues about 0.53 T FP64 instructions/s but about 20 T integer
// multiply-adds/s, and the FP64-bound stencils leave the integer pipe idle.
// These routines compute IEEE-754 binary64 round-to-nearest-even results
// with 32/64-bit integer arithmetic only, bit-identical to the FP64 pipe's
// a + b and a * b, so a kernel can hand part of its points to integer-pipe
// warps without changing a single result bit.
//
// Fast path: both operands normal (biased exponent 1..2046) and a normal
// result.  Everything else -- zeros, subnormals, infinities, NaNs, overflow,
// underflow -- falls back to the native operation, so every input gives the
// native result.  Exact cancellation returns +0 (round-to-nearest rule).
//
// Rounding: operands are aligned with 10 guard bits below the 53-bit
// significand and a sticky bit (OR of every bit shifted out) in bit 0.  Any
// inexact alignment makes the working sum odd, so it can never equal the
// exact half-way value; after at most one normalising shift the guard/sticky
// comparison against half an ulp decides round-to-nearest-even correctly.
#pragma once

#include <cstdint>

namespace b200 {
namespace f64emu {

constexpr uint64_t kSign = 0x8000000000000000ULL;
constexpr uint64_t kFrac = 0x000FFFFFFFFFFFFFULL;
constexpr uint64_t kHidden = 0x0010000000000000ULL;

__device__ __forceinline__ uint64_t bits(double x) {
  return static_cast<uint64_t>(__double_as_longlong(x));
}
__device__ __forceinline__ double from_bits(uint64_t u) {
  return __longlong_as_double(static_cast<long long>(u));
}
// The bits of x through a move the compiler cannot see into: integer masks
// on them (|x| as x & ~sign, -x as x ^ sign) stay integer instructions
// instead of being recognised as fabs / fneg and issued on the FP64 pipe.
__device__ __forceinline__ uint64_t bits_opaque(double x) {
  uint64_t u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
}

// a + b, correctly rounded (RN-even), integer pipe on the fast path.
__device__ __forceinline__ double add(double a, double b) {
  const uint64_t A = bits(a), B = bits(b);
  const uint32_t eA = static_cast<uint32_t>(A >> 52) & 0x7ffu;
  const uint32_t eB = static_cast<uint32_t>(B >> 52) & 0x7ffu;
  if (eA - 1u >= 2046u || eB - 1u >= 2046u) return a + b;  // zero/subnormal/inf/nan
  const bool swap = (B & ~kSign) > (A & ~kSign);
  const uint64_t X = swap ? B : A, Y = swap ? A : B;
  const int ex = static_cast<int>(swap ? eB : eA);
  const uint32_t d = swap ? (eB - eA) : (eA - eB);
  const uint64_t MX = ((X & kFrac) | kHidden) << 10;
  const uint64_t my = ((Y & kFrac) | kHidden) << 10;
  uint64_t MY;
  if (d >= 63u) {
    MY = 1u;  // only the sticky bit survives
  } else {
    MY = my >> d;
    MY |= ((my & ((1ULL << d) - 1u)) != 0u) ? 1u : 0u;
  }
  uint64_t S;
  int e = ex;
  if (((X ^ Y) & kSign) == 0u) {
    S = MX + MY;
    if (S >> 63) {
      S = (S >> 1) | (S & 1u);
      e += 1;
    }
  } else {
    S = MX - MY;
    if (S == 0u) return 0.0;
    const int lz = __clzll(static_cast<long long>(S)) - 1;  // leading one to bit 62
    S <<= lz;
    e -= lz;
  }
  uint64_t mant = S >> 10;
  const uint32_t rem = static_cast<uint32_t>(S) & 0x3ffu;
  if (rem > 0x200u || (rem == 0x200u && (mant & 1u))) {
    mant += 1u;
    if (mant >> 53) {
      mant >>= 1;
      e += 1;
    }
  }
  if (e <= 0 || e >= 2047) return a + b;  // result under/overflows: native
  return from_bits((X & kSign) | ((static_cast<uint64_t>(e - 1) << 52) + mant));
}

__device__ __forceinline__ double sub(double a, double b) { return add(a, -b); }

// a * b, correctly rounded (RN-even), integer pipe on the fast path.
__device__ __forceinline__ double mul(double a, double b) {
  const uint64_t A = bits(a), B = bits(b);
  const uint32_t eA = static_cast<uint32_t>(A >> 52) & 0x7ffu;
  const uint32_t eB = static_cast<uint32_t>(B >> 52) & 0x7ffu;
  if (eA - 1u >= 2046u || eB - 1u >= 2046u) return a * b;
  const uint64_t mA = (A & kFrac) | kHidden, mB = (B & kFrac) | kHidden;
  const uint64_t lo = mA * mB;
  const uint64_t hi = __umul64hi(mA, mB);  // product < 2^106: hi < 2^42
  int e = static_cast<int>(eA) + static_cast<int>(eB) - 1023;
  uint64_t mant, rem, half;
  if (hi >> 41) {  // product in [2^105, 2^106): keep bits 105..53
    mant = (hi << 11) | (lo >> 53);
    rem = lo & ((1ULL << 53) - 1u);
    half = 1ULL << 52;
    e += 1;
  } else {         // product in [2^104, 2^105): keep bits 104..52
    mant = (hi << 12) | (lo >> 52);
    rem = lo & ((1ULL << 52) - 1u);
    half = 1ULL << 51;
  }
  if (rem > half || (rem == half && (mant & 1u))) {
    mant += 1u;
    if (mant >> 53) {
      mant >>= 1;
      e += 1;
    }
  }
  if (e <= 0 || e >= 2047) return a * b;
  return from_bits(((A ^ B) & kSign) | ((static_cast<uint64_t>(e - 1) << 52) + mant));
}

// a + b for operands of the same sign, both normal, with biased exponents at
// most 3 apart and below 2046: aligned to the larger exponent with 3 guard
// bits, both significands are exact (no bit of the smaller one is shifted
// out), so their sum is exact and one round-to-nearest-even on the low 3 bits
// (4 when the sum carried into a new binade) gives the FP64 pipe's result.
// The rounding carry runs into the exponent field by itself; the largest
// exponent allowed makes the carry's overflow the correctly rounded infinity.
// About 40 integer instructions against one FP64 add: worth it only where the
// FP64 pipe is the bound and the integer pipes have room (JACOBI_2D's sums
// of values of one sign and similar size).  Anything else sets `slow` (the
// caller adds natively).
__device__ __forceinline__ double add_close_fast(double a, double b, bool& slow) {
  const uint64_t A = bits(a), B = bits(b);
  const uint32_t ahi = static_cast<uint32_t>(A >> 32), bhi = static_cast<uint32_t>(B >> 32);
  const uint32_t ea = (ahi >> 20) & 0x7ffu, eb = (bhi >> 20) & 0x7ffu;
  const bool a_big = ea >= eb;
  const uint32_t emax = a_big ? ea : eb, emin = a_big ? eb : ea;
  const uint32_t d = emax - emin;
  if (((ahi ^ bhi) >> 31) != 0u || emin == 0u || emax > 2045u || d > 3u) {
    slow = true;
    return 0.0;
  }
  const uint64_t X = a_big ? A : B, Y = a_big ? B : A;
  const uint64_t mx = ((X & kFrac) | kHidden) << 3;
  const uint64_t my = ((Y & kFrac) | kHidden) << (3u - d);
  const uint64_t S = mx + my;                         // < 2^57, exact
  const uint32_t c = static_cast<uint32_t>(S >> 56);  // carried into the next binade
  const uint32_t k = 3u + c;                          // bits dropped
  // round to nearest even in one add: with q = S >> k, S + (half an ulp - 1)
  // + (q & 1) carries into q exactly when the dropped bits exceed half an ulp,
  // or equal it and q is odd
  const uint64_t mant = (S + ((4ull << c) - 1u) + ((S >> k) & 1u)) >> k;  // 53 bits (54 on a carry)
  return from_bits((X & kSign) | ((static_cast<uint64_t>(emax + c - 1u) << 52) + mant));
}

// a + b (bit patterns A and B) for normal operands of either sign with biased
// exponents at most 3 apart and below 2046.  The operand of larger magnitude
// is X; aligned to its exponent with 3 guard bits both significands are
// exact, so S = |X| +- |Y| (never negative) is the exact result's magnitude
// in units of 2^(ex - 1078).  A difference may cancel any number of leading
// bits: S is shifted up until its leading one is bit 62 (a leading-zero
// count), which keeps every bit, and the 10 bits below the 53 kept ones
// decide round to nearest even (at most 4 of them can be set).  An exact
// zero is +0 (round to nearest).  `slow` is set when an operand is zero,
// subnormal, infinite or NaN, the exponents are further apart, or the result
// falls below the normal range; the caller then adds natively.  About 50
// integer instructions against one FP64 add (HEAT_3D's b(+1) - 2a, whose
// operands are within a binade or two of each other).  SUB gives a - b: b's
// sign is flipped in the sign logic.  The callers pass bits_opaque() bits, so
// the masks below stay on the integer pipes.
template <bool SUB>
__device__ __forceinline__ double add_near_bits(uint64_t A, uint64_t B, bool& slow) {
  const uint64_t ma = A & ~kSign, mb = B & ~kSign;
  const bool a_big = ma >= mb;
  const uint64_t X = a_big ? ma : mb, Y = a_big ? mb : ma;
  const uint32_t ex = static_cast<uint32_t>(X >> 52), ey = static_cast<uint32_t>(Y >> 52);
  const uint32_t d = ex - ey;
  if (ey == 0u || ex > 2045u || d > 3u) {
    slow = true;
    return 0.0;
  }
  const uint64_t mx = ((X & kFrac) | kHidden) << 3;
  const uint64_t my = ((Y & kFrac) | kHidden) << (3u - d);
  const bool opp = (((A ^ B) >> 63) != 0u) != SUB;
  const uint64_t S = opp ? mx - my : mx + my;            // < 2^57, exact
  if (S == 0u) return 0.0;
  const uint32_t lz = static_cast<uint32_t>(__clzll(static_cast<long long>(S)));  // 7..63
  const int e = static_cast<int>(ex) + 8 - static_cast<int>(lz);  // the result's biased exponent
  if (e <= 0) {
    slow = true;
    return 0.0;
  }
  // leading one at bit 62 (lz >= 7, so no bit is lost); the 53 bits from there
  // down are kept, and adding (half an ulp - 1) plus the kept part's last bit
  // before the shift rounds to nearest even (a carry to 2^53 runs into the
  // exponent field when packed)
  const uint64_t W = S << (lz - 1u);
  const uint64_t mant = (W + 0x1ffu + ((W >> 10) & 1u)) >> 10;
  const uint64_t sign = a_big ? (A & kSign) : (SUB ? (~B & kSign) : (B & kSign));
  return from_bits(sign | ((static_cast<uint64_t>(e - 1) << 52) + mant));
}
__device__ __forceinline__ double add_near_fast(double a, double b, bool& slow) {
  return add_near_bits<false>(bits_opaque(a), bits_opaque(b), slow);
}
__device__ __forceinline__ double sub_near_fast(double a, double b, bool& slow) {
  return add_near_bits<true>(bits_opaque(a), bits_opaque(b), slow);
}

// a * b + c with one rounding (the FP64 pipe's fma) on the integer pipes, for
// positive normal operands with c's last bit at or above the product's
// (D = ec + 1075 - ea - eb, the shift of c's significand to the product's
// scale, in [0, 74]).  The 106-bit product of the significands and c's
// shifted significand add exactly in 128 bits (their sum stays below 2^128);
// the sum is shifted up until its leading one is bit 127 (the product alone
// is at least 2^104, so the high word is never zero), the top 53 bits are
// kept, and bit 74 with the OR of the bits below decides round to nearest
// even.  `slow` is set for every other input (a zero, subnormal, negative,
// infinite or NaN operand; c too far below the product or too far above
// it; a result leaving the normal range), for which the caller uses the FP64
// pipe.  About 60 integer instructions against one DFMA (EOS's r * y + z,
// whose addends exceed their products by a few binades).
__device__ __forceinline__ double fma_pos_fast(double a, double b, double c, bool& slow) {
  const uint64_t A = bits_opaque(a), B = bits_opaque(b), C = bits_opaque(c);
  // biased exponents with the sign bit above them: a negative operand gives
  // a value of 2048 or more and fails the range test
  const uint32_t ea = static_cast<uint32_t>(A >> 52), eb = static_cast<uint32_t>(B >> 52);
  const uint32_t ec = static_cast<uint32_t>(C >> 52);
  const int D = static_cast<int>(ec) + 1075 - static_cast<int>(ea) - static_cast<int>(eb);
  if (ea - 1u > 2045u || eb - 1u > 2045u || ec - 1u > 2045u ||
      static_cast<unsigned>(D) > 74u) {
    slow = true;
    return 0.0;
  }
  const uint64_t ma = (A & kFrac) | kHidden, mb = (B & kFrac) | kHidden, mc = (C & kFrac) | kHidden;
  using u128 = unsigned __int128;
  const u128 S = static_cast<u128>(ma) * mb + (static_cast<u128>(mc) << D);  // exact, < 2^128
  const uint32_t lz = static_cast<uint32_t>(__clzll(static_cast<long long>(S >> 64)));  // 0..23
  const u128 V = S << lz;                                    // leading one at bit 127
  const uint64_t vh = static_cast<uint64_t>(V >> 64), vl = static_cast<uint64_t>(V);
  const uint64_t mant = vh >> 11;                            // 53 bits with the hidden one
  const uint32_t rest = static_cast<uint32_t>(vh) & 0x7ffu;  // round bit 0x400, sticky below
  const uint64_t up = (rest > 0x400u || (rest == 0x400u && (vl != 0u || (mant & 1u)))) ? 1u : 0u;
  const int e = static_cast<int>(ea + eb) - 1000 - static_cast<int>(lz);  // the result's biased exponent
  if (e <= 0 || e >= 2046) {
    slow = true;
    return 0.0;
  }
  return from_bits((static_cast<uint64_t>(e - 1) << 52) + mant + up);
}

// x * 2^k for a small |k|: exact exponent arithmetic; native when the result
// would leave the normal range (or x is not a normal number).
__device__ __forceinline__ double scale2(double x, int k) {
  const uint64_t X = bits(x);
  const int e = static_cast<int>((X >> 52) & 0x7ffu);
  if (e == 0 || e == 2047 || e + k <= 0 || e + k >= 2047) return x * scalbn(1.0, k);
  return from_bits(X + (static_cast<uint64_t>(static_cast<int64_t>(k)) << 52));
}

// a * b, correctly rounded (RN-even), on the integer pipe: the 106-bit
// product of the significands (64-bit multiply and high half), one
// normalising shift, then round-to-nearest-even on the bits shifted out.
// `slow` is set for zeros, subnormals, infinities, NaNs and products outside
// the normal range; the caller then multiplies natively.  With a constant b
// the compiler folds b's fields.
__device__ __forceinline__ double mul_fast(double a, double b, bool& slow) {
  const uint64_t A = bits(a), B = bits(b);
  const uint32_t eA = static_cast<uint32_t>(A >> 52) & 0x7ffu;
  const uint32_t eB = static_cast<uint32_t>(B >> 52) & 0x7ffu;
  const uint64_t mA = (A & kFrac) | kHidden, mB = (B & kFrac) | kHidden;
  const uint64_t lo = mA * mB;
  const uint64_t hi = __umul64hi(mA, mB);  // product < 2^106: hi < 2^42
  const uint32_t top = static_cast<uint32_t>(hi >> 41);  // 1: product in [2^105, 2^106)
  const int e = static_cast<int>(eA) + static_cast<int>(eB) - 1023 + static_cast<int>(top);
  const uint32_t s = 52u + top;  // bits dropped
  // round to nearest even in one 128-bit add: half an ulp - 1, plus the kept
  // part's low bit, carries into the kept part exactly when it should; a
  // carry to 2^53 runs into the exponent field when packed below
  const uint64_t bias = ((1ULL << (s - 1u)) - 1u) + ((lo >> s) & 1u);
  const uint64_t lo2 = lo + bias;
  const uint64_t hi2 = hi + (lo2 < lo ? 1u : 0u);
  const uint64_t mant = (hi2 << (64u - s)) | (lo2 >> s);  // 53 bits (54 on a carry)
  slow |= (eA - 1u >= 2046u) || (eB - 1u >= 2046u) || e <= 0 || e >= 2047;
  return from_bits(((A ^ B) & kSign) | ((static_cast<uint64_t>(e & 0x7ff) - 1u) << 52) + mant);
}

// x * 2^K for a constant K as an exponent move on the integer pipe.  Exact
// and equal to the FP64 pipe's x * 2^K while x and the result are normal
// numbers; `slow` is set for every other input (zeros, subnormals,
// infinities, NaNs, results leaving the normal range), for which the caller
// recomputes with the FP64 pipe.
template <int K>
__device__ __forceinline__ double mul_pow2_fast(double x, bool& slow) {
  static_assert(K > -1000 && K < 1000 && K != 0, "small nonzero K");
  constexpr unsigned kLo = (K < 0) ? static_cast<unsigned>(1 - K) : 1u;  // smallest kept normal
  constexpr unsigned kHi = (K > 0) ? static_cast<unsigned>(2046 - K) : 2046u;  // largest
  const int hi = __double2hiint(x);
  const unsigned e = (static_cast<unsigned>(hi) >> 20) & 0x7ffu;
  slow |= (e - kLo) > (kHi - kLo);
  return __hiloint2double(hi + K * (1 << 20), __double2loint(x));
}

// a + b for a b far below a's last bit, without the FP64 pipe: returns a,
// which is RN(a + b) when a is normal and a's biased exponent exceeds b's by
// at least 55.  Then |b| < 2^(eb - 1022) <= 2^(ea - 1077), a quarter of a's
// ulp, below half the gap to a's neighbours on either side (the gap below a
// power of two is half an ulp), so rounding to nearest gives back a.  `slow`
// is set for every other pair (a zero, subnormal, infinite or NaN a; an
// infinite or NaN b; a gap under 55), for which the caller adds natively.
__device__ __forceinline__ double add_negligible(double a, double b, bool& slow) {
  const unsigned ea = (static_cast<unsigned>(__double2hiint(a)) >> 20) & 0x7ffu;
  const unsigned eb = (static_cast<unsigned>(__double2hiint(b)) >> 20) & 0x7ffu;
  slow |= (ea - 1u >= 2046u) || (ea < eb + 55u);
  return a;
}

// x < 0.0 on the integer pipe: the sign bit is set and the magnitude is
// neither zero (-0.0 is not below 0) nor a NaN (no NaN compares below 0);
// -inf counts.  Equal to the FP64 compare for every input.
__device__ __forceinline__ bool lt_zero(double x) {
  const uint64_t u = bits(x);
  return (u >> 63) && ((u & ~kSign) - 1u) < 0x7FF0000000000000ULL;
}

// One round of the significand long division in div_fast: appends K quotient
// bits to Q and leaves the exact remainder in R (0 <= R < mb on entry and on
// exit).  The digit q = floor(R * 2^K / mb) is estimated in FP32 from the top
// 32 bits of R and the FP32 reciprocal rf of mb's top 32 bits; with K <= 20
// the estimate is within one of q (relative error of the FP32 product below
// 2^-22), and the exact remainder R * 2^K - q * mb -- computed modulo 2^64,
// exact because its true value lies in (-mb, 2 mb) -- corrects it.
template <int K>
__device__ __forceinline__ void div_round(uint64_t& Q, uint64_t& R, uint64_t mb, float rf) {
  static_assert(K >= 1 && K <= 20, "digit size");
  const float rfk = rf * static_cast<float>(1u << K);  // exact scaling
  uint32_t q = __float2uint_rz(__uint2float_rn(static_cast<uint32_t>(R >> 21)) * rfk);
  long long r = static_cast<long long>((R << K) - static_cast<uint64_t>(q) * mb);
  if (r < 0) {
    q -= 1u;
    r += static_cast<long long>(mb);
  } else if (r >= static_cast<long long>(mb)) {
    q += 1u;
    r -= static_cast<long long>(mb);
  }
  Q = (Q << K) | q;
  R = static_cast<uint64_t>(r);
}

// a / b, correctly rounded (RN-even), without FP64 instructions: integer long
// division of the significands (schoolbook division with estimated digits,
// Knuth TAOCP vol. 2, 4.3.1, here with FP32 digit estimates).  For a, b
// normal, M = ma or 2 ma with M / mb in [1, 2); Q = floor(M 2^53 / mb) has 54
// bits (53 significand bits and a guard bit) and the final remainder R is
// exact, so guard bit, sticky bit (R != 0) and the last bit decide
// round-to-nearest-even exactly.  `slow` is set for zeros, subnormals,
// infinities, NaNs and quotients outside the normal range; the caller then
// divides natively.
__device__ __forceinline__ double div_fast(double a, double b, bool& slow) {
  const uint64_t A = bits(a), B = bits(b);
  const uint32_t ea = static_cast<uint32_t>(A >> 52) & 0x7ffu;
  const uint32_t eb = static_cast<uint32_t>(B >> 52) & 0x7ffu;
  const uint64_t ma = (A & kFrac) | kHidden, mb = (B & kFrac) | kHidden;
  const uint32_t sh = ma < mb ? 1u : 0u;
  const uint64_t M = ma << sh;
  int e = static_cast<int>(ea) - static_cast<int>(eb) + 1023 - static_cast<int>(sh);
  const float rf = __frcp_rn(__uint2float_rn(static_cast<uint32_t>(mb >> 21)));
  uint64_t Q = 1u, R = M - mb;  // the leading quotient bit is 1
  div_round<20>(Q, R, mb, rf);
  div_round<20>(Q, R, mb, rf);
  div_round<13>(Q, R, mb, rf);
  const uint64_t m0 = Q >> 1;  // [2^52, 2^53)
  const bool up = (Q & 1u) && (R != 0u || (m0 & 1u));
  uint64_t mant = m0 + (up ? 1u : 0u);
  if (mant >> 53) {
    mant >>= 1;
    e += 1;
  }
  slow |= (ea - 1u >= 2046u) || (eb - 1u >= 2046u) || e <= 0 || e >= 2047;
  return from_bits(((A ^ B) & kSign) | (static_cast<uint64_t>(e & 0x7ff) << 52) |
                   (mant & kFrac));
}

}  // namespace f64emu
}  // namespace b200
