// cbns_ff.cuh — float-float arithmetic for the binary64-grade face kernel.
//
// A value is the unevaluated sum hi + lo of two binary32 numbers with
// |lo| <= ulp(hi)/2: about 47 significant bits (binary64 has 53), in binary32's
// exponent range.  GB300 issues binary32 fused multiply-adds at about 64 times
// its binary64 rate, so a face in float-float arithmetic (10-15 binary32
// operations per binary64 one) runs several times faster than in binary64.
//
// Published algorithms, written here from their descriptions:
// * TwoSum (Knuth, TAOCP vol. 2, 4.2.2) and Fast2Sum (Dekker 1971): the sum of
//   two binary32 numbers and its exact rounding error;
// * the exact product by one fused multiply-add: a*b - fl(a*b) = fma(a, b, -fl(a*b));
// * the double-word sum and product of Joldes, Muller and Popescu, "Tight and
//   rigorous error bounds for basic building blocks of double-word arithmetic",
//   ACM TOMS 44(2), 2017: SloppyDWPlusDW (relative to |x| + |y|, about 2^-46)
//   and DWTimesDW with fused multiply-adds (about 5 * 2^-48);
// * reciprocal and reciprocal square root by one Newton-Raphson step on the
//   hardware estimate with the residual formed in float-float (Karp and
//   Markstein, "High-precision division and square root", ACM TOMS 23(4), 1997),
//   here with the residual's second-order term added, so the estimate's error e
//   leaves O(e^3).
//
// The hardware estimates are PTX rcp.approx.ftz.f32 and rsqrt.approx.ftz.f32
// (MUFU), used on positive normal operands only.
#pragma once

#include <cstdint>

namespace cbns {

struct ff {
  float hi, lo;
};

// A binary64 constant as float-float (compile time).
__host__ __device__ constexpr ff ff_const(double x) {
  return ff{(float)x, (float)(x - (double)(float)x)};
}

// The binary32 additions and multiplications below are __fadd_rn, __fsub_rn and
// __fmul_rn: the compiler never merges these into a fused multiply-add, which
// would change what the error-free transformations compute (and make the
// results depend on how the surrounding code compiles).
#define FF_ADD(a, b) __fadd_rn((a), (b))
#define FF_SUB(a, b) __fsub_rn((a), (b))
#define FF_MUL(a, b) __fmul_rn((a), (b))

__device__ __forceinline__ ff ff_fast2sum(float a, float b) {  // |a| >= |b| or a = 0
  const float s = FF_ADD(a, b);
  return ff{s, FF_SUB(b, FF_SUB(s, a))};
}

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = FF_ADD(a, b);
  const float v = FF_SUB(s, a);
  return ff{s, FF_ADD(FF_SUB(a, FF_SUB(s, v)), FF_SUB(b, v))};
}

// The sum of two non-negative binary32 values with its exact error: Fast2Sum
// (Dekker) on the larger and the smaller gives the same pair as TwoSum in three
// additions instead of six (the max and the min go to the ALU pipe, not the FMA
// pipe).  s is formed from the operands as given, so a NaN still propagates.
__device__ __forceinline__ ff ff_two_sum_nonneg(float a, float b) {
  const float s = FF_ADD(a, b);
  return ff{s, FF_SUB(fminf(a, b), FF_SUB(s, fmaxf(a, b)))};
}
template <bool NONNEG>
__device__ __forceinline__ ff ff_two_sum_as(float a, float b) {
  if constexpr (NONNEG) {
    return ff_two_sum_nonneg(a, b);
  } else {
    return ff_two_sum(a, b);
  }
}

__device__ __forceinline__ ff operator-(ff a) { return ff{-a.hi, -a.lo}; }

// SloppyDWPlusDW: TwoSum of the high parts, the low parts added, renormalised.
__device__ __forceinline__ ff operator+(ff a, ff b) {
  const ff s = ff_two_sum(a.hi, b.hi);
  return ff_fast2sum(s.hi, FF_ADD(s.lo, FF_ADD(a.lo, b.lo)));
}
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }

// DWTimesDW: the exact product of the high parts plus the two cross terms.  The
// pair (p, e) is returned without renormalising: a product has no cancellation,
// so |e| stays within about one ulp of p (at most ulp(p)/2 from the exact
// product's error plus two cross terms each below 2^-23 |p|), which every
// operation here accepts as a float-float operand (the renormalising Fast2Sum
// would cost three additions per product).
__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = FF_MUL(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.lo, b.hi, fmaf(a.hi, b.lo, e));
  return ff{p, e};
}

// Times a power of two: exact.
__device__ __forceinline__ ff ff_scale(ff a, float p2) { return ff{FF_MUL(a.hi, p2), FF_MUL(a.lo, p2)}; }

// a * b + c, the product's error terms folded into one sloppy sum.
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) {
  const float p = FF_MUL(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.lo, b.hi, fmaf(a.hi, b.lo, e));
  const ff s = ff_two_sum(p, c.hi);
  return ff_fast2sum(s.hi, FF_ADD(s.lo, FF_ADD(e, c.lo)));
}

// c * b + d for a binary32 constant c.
__device__ __forceinline__ ff ff_fma(float c, ff b, ff d) {
  const float p = FF_MUL(c, b.hi);
  const float e = fmaf(c, b.lo, fmaf(c, b.hi, -p));
  const ff s = ff_two_sum(p, d.hi);
  return ff_fast2sum(s.hi, FF_ADD(s.lo, FF_ADD(e, d.lo)));
}

// Accumulating forms: the same results without the final Fast2Sum, for a value
// that is used only as the addend of another float-float operation (whose TwoSum
// takes any high part exactly and folds the low part into its error term) or is
// widened to binary64.  A chain of multiply-adds renormalises once, at its end.
// NONNEG: both the product's and the addend's high parts are known to be >= 0
// (sums of squares and of products of them), so the TwoSum is the cheaper
// ff_two_sum_nonneg; the result is the same.
template <bool NONNEG = false>
__device__ __forceinline__ ff ff_fma_acc(ff a, ff b, ff c) {
  const float p = FF_MUL(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.lo, b.hi, fmaf(a.hi, b.lo, e));
  const ff s = ff_two_sum_as<NONNEG>(p, c.hi);
  return ff{s.hi, FF_ADD(s.lo, FF_ADD(e, c.lo))};
}
template <bool NONNEG = false>
__device__ __forceinline__ ff ff_fma_acc(float c, ff b, ff d) {
  const float p = FF_MUL(c, b.hi);
  const float e = fmaf(c, b.lo, fmaf(c, b.hi, -p));
  const ff s = ff_two_sum_as<NONNEG>(p, d.hi);
  return ff{s.hi, FF_ADD(s.lo, FF_ADD(e, d.lo))};
}
__device__ __forceinline__ ff ff_add_acc(ff a, ff b) {
  const ff s = ff_two_sum(a.hi, b.hi);
  return ff{s.hi, FF_ADD(s.lo, FF_ADD(a.lo, b.lo))};
}
// a^2 + c with c.hi >= 0 (sums of squares: the cheaper TwoSum).
__device__ __forceinline__ ff ff_sqr_add_acc(ff a, ff c) {
  const float p = FF_MUL(a.hi, a.hi);
  const float e = fmaf(FF_ADD(a.hi, a.hi), a.lo, fmaf(a.hi, a.hi, -p));
  const ff s = ff_two_sum_nonneg(p, c.hi);
  return ff{s.hi, FF_ADD(s.lo, FF_ADD(e, c.lo))};
}

// a^2 + c with c.hi >= 0.
__device__ __forceinline__ ff ff_sqr_add(ff a, ff c) {
  const float p = FF_MUL(a.hi, a.hi);
  const float e = fmaf(FF_ADD(a.hi, a.hi), a.lo, fmaf(a.hi, a.hi, -p));
  const ff s = ff_two_sum_nonneg(p, c.hi);
  return ff_fast2sum(s.hi, FF_ADD(s.lo, FF_ADD(e, c.lo)));
}

__device__ __forceinline__ ff ff_sqr(ff a) {  // unrenormalised, as operator*
  const float p = FF_MUL(a.hi, a.hi);
  const float e = fmaf(FF_ADD(a.hi, a.hi), a.lo, fmaf(a.hi, a.hi, -p));
  return ff{p, e};
}

// 1/a for a positive normal float-float a.  y = estimate of 1/a.hi; the residual
// r = 1 - a y is formed exactly up to the last term (1 - fl(a.hi y) is exact by
// Sterbenz's lemma, the product's error comes from a fused multiply-add), and
// 1/a = y (1 + r + r^2 + ...) is taken to r^2.
__device__ __forceinline__ ff ff_rcp(ff a) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(a.hi));
  const float p = FF_MUL(a.hi, y);
  const float pe = fmaf(a.hi, y, -p);
  const float r = fmaf(-a.lo, y, FF_SUB(FF_SUB(1.0f, p), pe));
  return ff_fast2sum(y, FF_MUL(y, fmaf(r, r, r)));
}

// 1/sqrt(a) for a positive normal float-float a: y = estimate of 1/sqrt(a.hi),
// r = 1 - a y^2 formed as above, 1/sqrt(a) = y (1 + r/2 + 3 r^2/8 + ...).
__device__ __forceinline__ ff ff_rsqrt(ff a) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(a.hi));
  const float s = FF_MUL(y, y);
  const float se = fmaf(y, y, -s);  // y^2 = s + se exactly
  const float p = FF_MUL(a.hi, s);
  float e = fmaf(a.hi, s, -p);
  e = fmaf(a.hi, se, fmaf(a.lo, s, e));  // a y^2 = p + e to float-float accuracy
  const float r = FF_SUB(FF_SUB(1.0f, p), e);
  return ff_fast2sum(y, FF_MUL(y, FF_MUL(r, fmaf(0.375f, r, 0.5f))));
}

__device__ __forceinline__ ff ff_abs(ff a) { return a.hi < 0.0f ? -a : a; }

__device__ __forceinline__ ff ff_max(ff a, ff b) {
  return (a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo)) ? a : b;
}

// ---------------------------------------------------------------------------
// Conversions, on the integer pipe (binary64 conversions would take the FP64
// pipe the float-float kernel exists to spare).

// A binary64 value as float-float (stored as float2 {hi, lo}): hi is x truncated
// to binary32's 24 significant bits, lo the next 23 bits, also truncated (x to
// about 2^-46 relative).  Exact bit manipulation, valid for 2^-103 <= |x| < 2^128
// (below about 2^-79 lo is a binary32 subnormal, still exact); below 2^-103 lo
// is 0, below binary32's normal range both parts are 0 (an absolute error under
// 2^-126), and |x| >= 2^128 (or Inf/NaN) gives NaN.
__device__ __forceinline__ float2 ff_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const unsigned sign = h32 & 0x80000000u;
  const unsigned e = (h32 >> 20) & 0x7ffu;  // biased binary64 exponent
  // exponent rebased from 1023 to 127 (bias difference 896), then the 20 + 3
  // leading fraction bits: (h32 - 896 * 2^20) << 3 keeps exponent and fraction in
  // bits 30..0 when 897 <= e <= 1150
  const unsigned hb = sign | ((((h32 & 0x7fffffffu) - (896u << 20)) << 3) | (l32 >> 29));
  // the remaining 29 fraction bits m = l32 & (2^29 - 1) are worth m * 2^(E-52),
  // E the unbiased exponent: put their top 23 bits under the exponent of
  // 2^(E-23) and subtract 2^(E-23) (exact)
  const unsigned pe = (hb & 0xff800000u) - (23u << 23);
  float hi = __uint_as_float(hb);
  float lo = FF_SUB(__uint_as_float(pe | ((l32 >> 6) & 0x7fffffu)), __uint_as_float(pe));
  if (e < 920u) {
    lo = __uint_as_float(sign);  // a zero of x's sign, so -0.0 stays -0.0
    if (e < 897u) hi = __uint_as_float(sign);
  }
  if (e > 1150u) {
    hi = __uint_as_float(0x7fffffffu);
    lo = 0.0f;
  }
  return make_float2(hi, lo);
}

// A binary32 value widened to binary64 exactly: normal values and zeros by
// bits (exponent rebased from 127 to 1023, fraction shifted up 29 places);
// subnormals, Inf and NaN, which the kernels' values rarely are, by the
// hardware conversion.
__device__ __forceinline__ double ff_widen(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned a = b & 0x7fffffffu, sign = b & 0x80000000u;
  if (a - 0x00800000u < 0x7f000000u)
    return __hiloint2double((int)(sign | ((a >> 3) + (896u << 20))), (int)(b << 29));
  if (a == 0u) return __hiloint2double((int)sign, 0);
  return (double)f;
}

// The float-float value rounded to binary64 (one binary64 addition).
__device__ __forceinline__ double ff_to_double(ff a) { return ff_widen(a.hi) + ff_widen(a.lo); }

}  // namespace cbns
