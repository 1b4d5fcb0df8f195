// Correctly rounded FP64 add, multiply and divide on the integer pipes.
//
// GB300 issues about two FP64 lanes per clock per SM, against 128 lanes of
// 32-bit integer and FP32 work, so every stencil kernel of the solve waits
// on its FP64 instructions while most issue slots stay empty.  These
// functions compute IEEE 754 binary64 results with round-to-nearest-even
// from the operands' bit patterns, with integer instructions (and, for the
// division's reciprocal seed, one FP32 reciprocal), so a kernel can move
// part of its FP64 work off the FP64 pipe and still produce the hardware's
// results bit for bit.  A correctly rounded FP64 division takes many FP64
// instructions; emu_ddiv and emu_ddiv_var take none.
//
// Method (textbook IEEE 754 arithmetic, as in Muller et al., Handbook of
// Floating-Point Arithmetic): align the significands in 64-bit integers with
// guard bits and a sticky bit, add, multiply or divide exactly, normalise,
// round to nearest even on the guard bits.  Operands or results outside the
// normal range (zeros, subnormals, infinities, NaNs, overflow, underflow)
// take the hardware instruction instead, so those cases are the hardware's
// by construction.
#pragma once

#include <stdint.h>

namespace tea {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kFrac = 0x000fffffffffffffull;
constexpr uint64_t kHidden = 0x0010000000000000ull;

// Round the 64-bit significand f (leading one at bit 63) to 53 bits with
// sticky information s below bit 0 and pack it with biased exponent e and
// sign bit sg, as a bit pattern.  A carry out of the rounding moves into
// the exponent field.
__device__ __forceinline__ uint64_t emu_pack(uint64_t sg, int e, uint64_t f, bool s) {
  uint64_t m = f >> 11;
  const uint32_t rest = (uint32_t)f & 0x7ffu;
  m += (rest > 0x400u || (rest == 0x400u && (s || (m & 1)))) ? 1 : 0;
  return sg + ((uint64_t)(e - 1) << 52) + m;
}

// a + b, rounded to nearest even.
__device__ __forceinline__ double emu_dadd(double a, double b) {
  const uint64_t ia = (uint64_t)__double_as_longlong(a);
  const uint64_t ib = (uint64_t)__double_as_longlong(b);
  const bool swap = (ia & ~kSign) < (ib & ~kSign);
  const uint64_t x = swap ? ib : ia;  // larger magnitude
  const uint64_t y = swap ? ia : ib;
  const int ex = (int)(x >> 52) & 0x7ff, ey = (int)(y >> 52) & 0x7ff;
  // With ex >= 64 even total cancellation (at most 63 leading zeros) leaves
  // a normal result, so every case for the hardware is known here.
  if (ex < 64 || ex >= 0x7fe || ey == 0) return __dadd_rn(a, b);
  const uint64_t fx = ((x & kFrac) | kHidden) << 10;  // leading one at bit 62
  uint64_t fy = ((y & kFrac) | kHidden) << 10;
  const int d = ex - ey;
  if (d >= 64) {
    fy = 1;  // only the sticky bit is left
  } else if (d > 0) {
    const uint64_t lost = fy << (64 - d);
    fy = (fy >> d) | (lost != 0 ? 1 : 0);
  }
  const uint64_t f = ((x ^ y) & kSign) ? fx - fy : fx + fy;
  // Exact cancellation gives +0.  The zero is selected as a bit pattern:
  // a floating-point select would go through the FP64 pipe.
  const uint64_t fs = f | (f == 0 ? 1 : 0);
  const int lz = __clzll((long long)fs);  // 0 after a carry, 1, or more after cancellation
  const uint64_t r = emu_pack(x & kSign, ex + 1 - lz, fs << lz, false);
  return __longlong_as_double((long long)(f == 0 ? 0 : r));
}

// a * b, rounded to nearest even.
__device__ __forceinline__ double emu_dmul(double a, double b) {
  const uint64_t ia = (uint64_t)__double_as_longlong(a);
  const uint64_t ib = (uint64_t)__double_as_longlong(b);
  const int ea = (int)(ia >> 52) & 0x7ff, eb = (int)(ib >> 52) & 0x7ff;
  const int e0 = ea + eb - 1023;  // biased exponent of a product in [1, 2)
  if (ea == 0 || eb == 0 || ea == 0x7ff || eb == 0x7ff || e0 < 1 || e0 > 0x7fd)
    return __dmul_rn(a, b);
  const uint64_t ma = ((ia & kFrac) | kHidden) << 11;  // [2^63, 2^64)
  const uint64_t mb = ((ib & kFrac) | kHidden) << 11;
  const uint64_t hi = __umul64hi(ma, mb);  // product in [2^126, 2^128)
  const uint64_t lo = ma * mb;
  const int top = (int)(hi >> 63);  // 1 when the product is in [2, 4)
  const uint64_t f = top ? hi : ((hi << 1) | (lo >> 63));
  const uint64_t below = top ? lo : (lo << 1);
  return __longlong_as_double((long long)emu_pack((ia ^ ib) & kSign, e0 + top, f, below != 0));
}

// Division by a divisor that is the same for every element of a launch
// (the Chebyshev / PPCG theta), exactly rounded, on the integer pipes.
// The significand quotient is an integer division by an invariant divisor:
// Moller and Granlund, "Improved division by invariant integers" (IEEE
// Trans. Computers 60(2), 2011), algorithm 4 (2/1 division with a
// precomputed reciprocal), applied to the 128-bit numerator mx * 2^(65|66)
// and the normalised divisor significand d = my * 2^11.  Its 55-bit
// quotient and the remainder give the 53-bit significand, the round bit and
// the sticky bit.
struct DivConst {
  double y;    // the divisor
  uint64_t d;  // significand of y with its leading one at bit 63
  uint64_t v;  // floor((2^128 - 1) / d) - 2^64
  int ey;      // biased exponent of y
  int ok;      // y is a normal number; otherwise the hardware divides
};

// The reciprocal constants of y (host code: 128-bit integer division).
inline DivConst div_const(double y) {
  DivConst k;
  uint64_t iy;
  static_assert(sizeof(iy) == sizeof(y), "binary64");
  __builtin_memcpy(&iy, &y, sizeof(iy));
  k.y = y;
  k.ey = (int)(iy >> 52) & 0x7ff;
  k.ok = k.ey != 0 && k.ey != 0x7ff;
  k.d = ((iy & kFrac) | kHidden) << 11;
  const unsigned __int128 all = ~(unsigned __int128)0;
  k.v = (uint64_t)(all / k.d);  // the quotient is below 2^65: its low word
  return k;
}

// x / k.y, rounded to nearest even.
__device__ __forceinline__ double emu_ddiv(double x, const DivConst& k) {
  const uint64_t ix = (uint64_t)__double_as_longlong(x);
  const int ex = (int)(ix >> 52) & 0x7ff;
  const uint64_t mx = (ix & kFrac) | kHidden;
  const uint64_t my = k.d >> 11;
  const int lt = mx < my ? 1 : 0;  // significand quotient below 1
  const int e = ex - k.ey + 1023 - lt;  // biased exponent of the result
  if (!k.ok || ex == 0 || ex == 0x7ff || e < 1 || e > 0x7fe) return x / k.y;
  // numerator u1 * 2^64 with u1 = mx * 2^(1 + lt) < d: quotient in [2^54, 2^55)
  const uint64_t u1 = mx << (1 + lt);
  const uint64_t q0 = k.v * u1;
  uint64_t q1 = __umul64hi(k.v, u1) + u1 + 1;
  uint64_t r = 0 - q1 * k.d;
  if (r > q0) {
    q1 -= 1;
    r += k.d;
  }
  if (r >= k.d) {
    q1 += 1;
    r -= k.d;
  }
  // q1 has 55 bits: 53 for the significand, a round bit, and one more
  // below it that joins the remainder in the sticky bit
  uint64_t m = q1 >> 2;
  const bool rb = (q1 >> 1) & 1;
  const bool sticky = (q1 & 1) || r != 0;
  m += (rb && (sticky || (m & 1))) ? 1 : 0;
  const uint64_t sg = (ix ^ (uint64_t)__double_as_longlong(k.y)) & kSign;
  return __longlong_as_double((long long)(sg + ((uint64_t)(e - 1) << 52) + m));
}

// x / y for divisors that change from element to element, exactly rounded,
// on the integer and FP32 pipes.  The significand quotient
// Q = floor(mx 2^(54|55) / my) comes from a reciprocal R ~ 2^116 / my: an
// FP32 seed (1 / the top 24 bits of my, correctly rounded) refined by two
// fixed-point Newton-Raphson steps for the reciprocal,
// R += R (2^116 - my R) / 2^116, each doubling the correct bits, then
// Q ~ mx R / 2^(62|61).  The remainder N - Q my is then formed exactly and Q
// corrected until 0 <= remainder < my, so the quotient is exact whatever
// the reciprocal's error; if three corrections each way do not get there
// (they always do: the estimate is within two of Q), the hardware divides.
// Rounding is as in emu_ddiv.
__device__ __forceinline__ double emu_ddiv_var(double x, double y) {
  const uint64_t ix = (uint64_t)__double_as_longlong(x);
  const uint64_t iy = (uint64_t)__double_as_longlong(y);
  const int ex = (int)(ix >> 52) & 0x7ff, ey = (int)(iy >> 52) & 0x7ff;
  const uint64_t mx = (ix & kFrac) | kHidden, my = (iy & kFrac) | kHidden;
  const int lt = mx < my ? 1 : 0;
  const int e = ex - ey + 1023 - lt;  // biased exponent of the result
  if (ex == 0 || ex == 0x7ff || ey == 0 || ey == 0x7ff || e < 1 || e > 0x7fe) return x / y;
  // seed: f ~ 2^29 / my to about 2^-22; R0 ~ 2^116 / my, below 2^64
  const float f = __frcp_rn((float)(uint32_t)(my >> 29));
  uint64_t R = (__float2ull_rz(f * 0x1p86f) << 1) - 1;
#pragma unroll
  for (int it = 0; it < 2; it++) {
    // err = 2^116 - my R as a 128-bit two's complement value; e52 = err >> 52
    const uint64_t plo = my * R, phi = __umul64hi(my, R);
    const uint64_t elo = 0 - plo;
    const uint64_t ehi = (1ull << 52) - phi - (plo != 0 ? 1 : 0);
    const long long e52 = (long long)((ehi << 12) | (elo >> 52));
    if (e52 >= 0) {
      const uint64_t c = __umul64hi(R, (uint64_t)e52);
      R = c > ~R ? ~0ull : R + c;
    } else {
      R -= __umul64hi(R, (uint64_t)(-e52));
    }
  }
  // Q ~ mx R / 2^(62 - lt), then the exact remainder N - Q my modulo 2^64
  const uint64_t qlo = mx * R, qhi = __umul64hi(mx, R);
  uint64_t q = (qhi << (2 + lt)) | (qlo >> (62 - lt));
  long long rem = (long long)((mx << (54 + lt)) - q * my);
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (rem < 0) {
      q -= 1;
      rem += (long long)my;
    }
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (rem >= (long long)my) {
      q += 1;
      rem -= (long long)my;
    }
  if (rem < 0 || rem >= (long long)my) return x / y;
  uint64_t m = q >> 2;
  const bool rb = (q >> 1) & 1;
  const bool sticky = (q & 1) || rem != 0;
  m += (rb && (sticky || (m & 1))) ? 1 : 0;
  return __longlong_as_double((long long)(((ix ^ iy) & kSign) + ((uint64_t)(e - 1) << 52) + m));
}

}  // namespace tea
