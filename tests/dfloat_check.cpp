// Test harness: double-float operations (htr-solver_gb300/csrc/dfloat.cuh) on
// random operands against double arithmetic; prints the largest relative
// error of each operation in units of u^2 = 2^-48.
#include <cmath>
#include <cstdio>
#include <cstdint>

#include "dfloat.cuh"

using htr::dfloat;

static uint64_t state = 0x9e3779b97f4a7c15ull;
static double uniform() {  // splitmix64 -> [0, 1)
  uint64_t z = (state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  return (z >> 11) * 0x1.0p-53;
}
static dfloat rnd(double lo_exp, double hi_exp, bool sign) {
  double m = std::exp2(lo_exp + (hi_exp - lo_exp) * uniform()) * (1.0 + uniform());
  if (sign && uniform() < 0.5) m = -m;
  return htr::df_from(m);
}

int main() {
  const double u2 = std::ldexp(1.0, -48);
  double e_add = 0, e_addpos = 0, e_mul = 0, e_mulf = 0, e_div = 0, e_rcp = 0, e_sqrt = 0, e_conv = 0;
  double e_bits = 0, e_bits_small = 0, e_same = 0;
  long bits_back_mismatch = 0, round_mismatch = 0;
  for (int k = 0; k < 2000000; k++) {
    const dfloat a = rnd(-20, 20, true), b = rnd(-20, 20, true);
    const dfloat p = rnd(-20, 20, false), q = rnd(-20, 20, false);
    const double A = htr::df_to_double(a), B = htr::df_to_double(b);
    const double P = htr::df_to_double(p), Q = htr::df_to_double(q);
    auto rel = [](dfloat got, double want) {
      return want == 0 ? 0.0 : std::fabs(htr::df_to_double(got) - want) / std::fabs(want);
    };
    // sums of opposite signs that cancel badly are measured against |a|+|b|
    const double s = A + B;
    const double es = std::fabs(htr::df_to_double(htr::df_add(a, b)) - s) / (std::fabs(A) + std::fabs(B));
    e_add = std::fmax(e_add, es / u2);
    e_addpos = std::fmax(e_addpos, rel(htr::df_add(p, q), P + Q) / u2);
    e_same = std::fmax(e_same, rel(htr::df_add_same(p, q), P + Q) / u2);
    e_same = std::fmax(e_same, rel(htr::df_add_same(htr::df_neg(p), htr::df_neg(q)), -(P + Q)) / u2);
    e_mul = std::fmax(e_mul, rel(htr::df_mul(a, b), A * B) / u2);
    e_mulf = std::fmax(e_mulf, rel(htr::df_mul(a, b.hi), A * (double)b.hi) / u2);
    e_div = std::fmax(e_div, rel(htr::df_div(a, b), A / B) / u2);
    e_rcp = std::fmax(e_rcp, rel(htr::df_rcp(b), 1.0 / B) / u2);
    e_sqrt = std::fmax(e_sqrt, rel(htr::df_sqrt(p), std::sqrt(P)) / u2);
    const double x = std::exp2(-60 + 120 * uniform()) * (1.0 + uniform());
    e_conv = std::fmax(e_conv, std::fabs(htr::df_to_double(htr::df_from(x)) - x) / x / u2);
    // integer-pipe conversions: 2^-74 <= |x| < 2^100 within 2^-48; below that
    // range hi alone (2^-23 relative); back to double equals the plain sum
    const double y = (uniform() < 0.5 ? -1 : 1) * std::exp2(-74 + 174 * uniform()) * (1.0 + uniform());
    const dfloat fy = htr::df_from_bits(y);
    e_bits = std::fmax(e_bits, std::fabs(htr::df_to_double(fy) - y) / std::fabs(y) / u2);
    if (htr::df_to_double_bits(fy) != htr::df_to_double(fy)) bits_back_mismatch++;
    // round-to-nearest conversion on the integer pipe: the conversion's value
    // in float's normal range, ties (x built on a half-ulp) included
    const double w = (uniform() < 0.5 ? -1 : 1) * std::exp2(-125 + 252 * uniform()) * (1.0 + uniform());
    if (htr::df_round_float(w) != (float)w) round_mismatch++;
    const float f = (float)std::exp2(-120 + 240 * uniform()) * (1.0f + (float)uniform());
    const double tie = (double)f + 0.5 * ((double)std::nextafter(f, 2.0f * f) - (double)f);
    if (htr::df_round_float(tie) != (float)tie || htr::df_round_float(-tie) != (float)-tie) round_mismatch++;
    const double z = std::exp2(-126 + 52 * uniform()) * (1.0 + uniform());
    e_bits_small = std::fmax(e_bits_small, std::fabs(htr::df_to_double(htr::df_from_bits(z)) - z) / z);
  }
  std::printf("same %.3f round_mismatch %ld ", e_same, round_mismatch);
  std::printf("add %.3f addpos %.3f mul %.3f mulf %.3f div %.3f rcp %.3f sqrt %.3f conv %.3f bits %.3f "
              "bits_small %.3e bits_back_mismatch %ld zero %d\n", e_add, e_addpos, e_mul, e_mulf, e_div, e_rcp, e_sqrt,
              e_conv, e_bits, e_bits_small, bits_back_mismatch,
              (int)(htr::df_to_double_bits(htr::df_from_bits(0.0)) == 0.0 && htr::df_from_bits(1e-40).hi == 0.0f));
  return 0;
}
