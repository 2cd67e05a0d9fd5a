// Table-driven exponential for the explicit chemistry sources.
//
// Method: P. T. P. Tang, "Table-driven implementation of the exponential
// function in IEEE floating-point arithmetic", ACM Trans. Math. Softw. 15(2),
// 1989.  x = (64 m + j) ln2/64 + r with integers m, j (0 <= j < 64) and
// |r| <= ln2/128, so exp(x) = 2^m * 2^(j/64) * exp(r):
//   * k = 64 m + j = round(x * 64/ln2) by adding 1.5 * 2^52 (the sum's low
//     word is k in two's complement);
//   * r = x - k ln2/64 with ln2/64 split into a double L1 and its remainder
//     L2 (fused multiply-adds, so k * L1 is not rounded before the
//     subtraction);
//   * exp(r) - 1 by its Taylor polynomial of degree 5: the first omitted term
//     r^6/720 is below 3.5e-17;
//   * 2^(j/64) from a table of the correctly rounded doubles (below), the
//     product with 1 + p(r) as one fused multiply-add, and 2^m added to the
//     exponent field.
// Ten FP64 instructions; the error is below one ulp plus the table's half
// ulp.  Arguments with |x| >= 700 (results outside [1e-304, 1e304]) and NaN go
// to the math library's exp.
#pragma once

#include "common.cuh"

namespace htr {

// 2^(j/64), j = 0..63, rounded to the nearest double
static __device__ const double kExp2Frac[64] = {
    0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, 0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0,
    0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, 0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0,
    0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, 0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0,
    0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, 0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0,
    0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, 0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0,
    0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, 0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0,
    0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, 0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0,
    0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, 0x1.6247eb03a5585p+0, 0x1.6623882552225p+0,
    0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, 0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0,
    0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, 0x1.82589994cce13p+0, 0x1.868d99b4492edp+0,
    0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, 0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0,
    0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, 0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0,
    0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, 0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0,
    0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, 0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0,
    0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, 0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0,
    0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, 0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0,
};

HTR_D double exp_table(double x) {
  // |x| >= 700 or NaN: the bit pattern of |x| is at least that of 700.0
  if ((__double_as_longlong(x) & 0x7fffffffffffffffLL) >= 0x4085e00000000000LL) return exp(x);
  const double shifted = fma(x, 0x1.71547652b82fep+6, 0x1.8p52);  // 64/ln2
  const int k = __double2loint(shifted);
  const double kd = shifted - 0x1.8p52;
  double r = fma(-kd, 0x1.62e42fefa39efp-7, x);   // L1 = ln2/64 rounded
  r = fma(-kd, 0x1.abc9e3b39803fp-62, r);         // L2 = ln2/64 - L1
  double s = fma(r, 1.0 / 120, 1.0 / 24);
  s = fma(r, s, 1.0 / 6);
  s = fma(r, s, 0.5);
  const double p = fma(r * r, s, r);  // exp(r) - 1
  const double t = __ldg(&kExp2Frac[k & 63]);
  const double y = fma(t, p, t);      // in [0.99, 2): a normal double
  return __longlong_as_double(__double_as_longlong(y) + ((long long)(k >> 6) << 52));
}

}  // namespace htr
