// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats with |lo| <= ulp(hi) / 2 (about 48 significant bits, relative
// rounding error of a few 2^-48 per operation), evaluated on the FP32 pipe.
//
// Error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum and the
// FMA-based exact product.  Double-word algorithms: those analysed by
// M. Joldes, J.-M. Muller and V. Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic", ACM Trans. Math.
// Softw. 44(2), 2017 (Algorithms 4, 6, 8 and 12: DWPlusFP, AccurateDWPlusDW,
// DWTimesFP3, DWTimesDW3; relative error bounds 2u^2, 3u^2, 2u^2 and 4u^2 with
// u = 2^-24); division and square root by one Newton correction of a float
// estimate in double-word arithmetic.
//
// Every operation goes through an explicitly rounded intrinsic on the device
// (no contraction, no reassociation); on the host the same header compiles
// with ordinary float operations and fmaf (build without FP contraction), so
// host tests reproduce the device's results bit for bit.
#pragma once

#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace htr {

struct dfloat {
  float hi, lo;
};

DF_HD float df_add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
DF_HD float df_sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
DF_HD float df_mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
DF_HD float df_fma_rn(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}
// correctly rounded reciprocal and square root of a float (the Newton
// corrections below only need an estimate, but a deterministic one)
DF_HD float df_rcp_rn(float a) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(a);
#else
  return 1.0f / a;
#endif
}
DF_HD float df_sqrt_rn(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return sqrtf(a);
#endif
}

// --- error-free transformations -------------------------------------------
// s + t = a + b exactly (TwoSum, 6 operations)
DF_HD dfloat two_sum(float a, float b) {
  const float s = df_add_rn(a, b);
  const float ap = df_sub_rn(s, b);
  const float bp = df_sub_rn(s, ap);
  return {s, df_add_rn(df_sub_rn(a, ap), df_sub_rn(b, bp))};
}
// the same for |a| >= |b| (or a == 0)  (Fast2Sum, 3 operations)
DF_HD dfloat fast_two_sum(float a, float b) {
  const float s = df_add_rn(a, b);
  return {s, df_sub_rn(b, df_sub_rn(s, a))};
}
// p + e = a * b exactly
DF_HD dfloat two_prod(float a, float b) {
  const float p = df_mul_rn(a, b);
  return {p, df_fma_rn(a, b, -p)};
}

// --- conversions ------------------------------------------------------------
DF_HD dfloat df_from(float a) { return {a, 0.0f}; }
// nearest float, then the nearest float of the remainder (exact remainder in
// double); relative representation error below 2^-48 for |x| in the normal
// range of float above 2^-102, zero below 2^-126
DF_HD dfloat df_from(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
// exact: hi and lo have 24 bits each and |lo| <= ulp(hi)/2
DF_HD double df_to_double(dfloat a) { return (double)a.hi + (double)a.lo; }

// The same conversions on the integer pipe.  Conversion instructions between
// double and float run at the FP64 rate on this part, so the hot paths build
// the float and double bit patterns with integer operations instead.
DF_HD unsigned long long df_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, 8);
  return b;
#endif
}
DF_HD double df_double(unsigned long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
DF_HD unsigned df_fbits(float x) {
#if defined(__CUDA_ARCH__)
  return (unsigned)__float_as_uint(x);
#else
  unsigned b;
  memcpy(&b, &x, 4);
  return b;
#endif
}
DF_HD float df_float(unsigned b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, 4);
  return x;
#endif
}
// 2^e as a float, -126 <= e <= 127
DF_HD float df_pow2(int e) { return df_float((unsigned)(e + 127) << 23); }

// double -> double-float: hi = the top 24 significand bits (truncated), the
// remaining 29 bits split into two exact floats A * 2^23 + B (each below
// 2^23, turned into floats by the 2^23 bias trick) and summed into lo with
// one rounding, then the pair renormalised.  Error at most 2^-48 relative
// for 2^-74 <= |x| < 2^128; 2^-126 <= |x| < 2^-74 keeps hi only (2^-23);
// smaller |x| (and zero) gives 0.  x must be finite.
DF_HD dfloat df_from_bits(double x) {
  const unsigned long long b = df_bits(x);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -126) return {0.0f, 0.0f};
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long m = b & 0xfffffffffffffULL;
  const float hi = df_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29));
  if (e < -74) return {hi, 0.0f};
  const unsigned r = (unsigned)(m & 0x1fffffffu);
  // exact floats: A = r >> 23 (6 bits), B = r & (2^23 - 1), by 2^23 + n - 2^23
  const float A = df_sub_rn(df_float(0x4b000000u | (r >> 23)), 8388608.0f);
  const float B = df_sub_rn(df_float(0x4b000000u | (r & 0x7fffffu)), 8388608.0f);
  // lo = A 2^(e-29) + B 2^(e-52), one rounding (both products are exact)
  float lo = df_fma_rn(A, df_pow2(e - 29), df_mul_rn(B, df_pow2(e - 52)));
  if (sign) lo = -lo;
  return fast_two_sum(hi, lo);
}
// double -> float rounded to nearest, ties to even, on the integer pipe:
// the same value as the conversion instruction for |x| in float's normal
// range (including the carry into the exponent and overflow to infinity);
// |x| below 2^-126 gives a zero of x's sign (the instruction would give a
// subnormal: an absolute difference below 2^-126).  x must not be NaN.
DF_HD float df_round_float(double x) {
  const unsigned long long b = df_bits(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -126) return df_float(sign);
  if (e > 127) return df_float(sign | 0x7f800000u);
  const unsigned long long m = b & 0xfffffffffffffULL;
  unsigned t = ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29);
  const unsigned rem = (unsigned)(m & 0x1fffffffu);
  t += (rem > 0x10000000u || (rem == 0x10000000u && (t & 1u))) ? 1u : 0u;
  return df_float(sign | t);
}
// float -> double by its bit pattern (normal floats; zero and subnormal
// floats give 0, infinities and NaN go through the conversion instruction)
DF_HD double df_widen(float f) {
  const unsigned u = df_fbits(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u) return 0.0;
  if (e == 0xffu) return (double)f;
  return df_double(((unsigned long long)(u & 0x80000000u) << 32) | ((unsigned long long)(e + 896u) << 52) |
                   ((unsigned long long)(u & 0x7fffffu) << 29));
}
// double-float -> double (exact for normal parts; one FP64 addition)
DF_HD double df_to_double_bits(dfloat a) { return df_widen(a.hi) + df_widen(a.lo); }

// --- arithmetic ---------------------------------------------------------------
// a + b, b a float (DWPlusFP)
DF_HD dfloat df_add(dfloat a, float b) {
  const dfloat s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, df_add_rn(a.lo, s.lo));
}
// a + b (AccurateDWPlusDW)
DF_HD dfloat df_add(dfloat a, dfloat b) {
  const dfloat s = two_sum(a.hi, b.hi);
  const dfloat t = two_sum(a.lo, b.lo);
  const dfloat v = fast_two_sum(s.hi, df_add_rn(s.lo, t.hi));
  return fast_two_sum(v.hi, df_add_rn(t.lo, v.lo));
}
// a + b for operands of the same sign (SloppyDWPlusDW: 11 operations; for
// same-sign operands no cancellation occurs and the relative error stays
// within 3u^2, checked by the host test)
DF_HD dfloat df_add_same(dfloat a, dfloat b) {
  const dfloat s = two_sum(a.hi, b.hi);
  const float v = df_add_rn(a.lo, b.lo);
  return fast_two_sum(s.hi, df_add_rn(s.lo, v));
}
DF_HD dfloat df_neg(dfloat a) { return {-a.hi, -a.lo}; }
DF_HD dfloat df_sub(dfloat a, dfloat b) { return df_add(a, df_neg(b)); }
// a * b, b a float (DWTimesFP3)
DF_HD dfloat df_mul(dfloat a, float b) {
  const dfloat c = two_prod(a.hi, b);
  return fast_two_sum(c.hi, df_fma_rn(a.lo, b, c.lo));
}
// a * b (DWTimesDW3)
DF_HD dfloat df_mul(dfloat a, dfloat b) {
  const dfloat c = two_prod(a.hi, b.hi);
  const float t0 = df_mul_rn(a.lo, b.lo);
  const float t1 = df_fma_rn(a.hi, b.lo, t0);
  const float c2 = df_fma_rn(a.lo, b.hi, t1);
  return fast_two_sum(c.hi, df_add_rn(c.lo, c2));
}
// a * b + c
DF_HD dfloat df_fma(dfloat a, dfloat b, dfloat c) { return df_add(df_mul(a, b), c); }
// 1 / a: r0 = rcp(hi), r = r0 + r0 (1 - a r0) with the residual in
// double-word arithmetic (two_prod makes a.hi * r0 exact)
DF_HD dfloat df_rcp(dfloat a) {
  const float r0 = df_rcp_rn(a.hi);
  const dfloat p = two_prod(a.hi, r0);                    // a.hi r0 exactly
  const float e = df_sub_rn(df_sub_rn(df_sub_rn(1.0f, p.hi), p.lo), df_mul_rn(a.lo, r0));  // 1 - a r0
  return fast_two_sum(r0, df_mul_rn(r0, e));
}
// a / b: q0 = a.hi rcp(b.hi), q = q0 + (a - b q0) / b.hi
DF_HD dfloat df_div(dfloat a, dfloat b) {
  const float r0 = df_rcp_rn(b.hi);
  const float q0 = df_mul_rn(a.hi, r0);
  const dfloat bq = df_mul(b, q0);        // b q0 (error 2u^2 relative)
  const dfloat d = df_sub(a, bq);         // a - b q0: cancels to ~u |a|
  return fast_two_sum(q0, df_mul_rn(d.hi, r0));
}
// sqrt(a), a > 0: s0 = sqrt(hi), s = s0 + (a - s0^2) / (2 s0)
DF_HD dfloat df_sqrt(dfloat a) {
  const float s0 = df_sqrt_rn(a.hi);
  const dfloat sq = two_prod(s0, s0);
  const float d = df_add_rn(df_sub_rn(df_sub_rn(a.hi, sq.hi), sq.lo), a.lo);
  return fast_two_sum(s0, df_mul_rn(d, df_mul_rn(0.5f, df_rcp_rn(s0))));
}

// a double constant split into its double-float form at compile time
#define HTR_DF_CONST(c) (::htr::dfloat{(float)(c), (float)((double)(c) - (double)(float)(c))})

}  // namespace htr
