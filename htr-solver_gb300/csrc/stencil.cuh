// Stencil tables, exact integer powers and the TENO / Kennedy-Gruber
// operators on the device.
//
// Node types, offsets and coefficients are those of HTR
// (src/prometeo_metric_coeffs.h:54-66, src/prometeo_metric_coeffs_macros.h);
// the operators follow src/prometeo_metric.inl.  Translation units that
// include this header and evaluate TENO selection flags are compiled with
// -fmad=false: every + - * / and sqrt is then rounded exactly as the
// reference's host build rounds it, and the only non-elementary operation,
// x^n with n in {4, 6, 12}, is evaluated in double-double arithmetic
// (Dekker two-product via fma) and rounded once, i.e. correctly rounded.
#pragma once

#include "common.cuh"
#include "dfloat.cuh"

namespace htr {

// ---------------------------------------------------------------------------
// Decision counters (diagnostic, off unless htr_decision_counters enables
// them): how many selections the single-precision filters decided and how
// many went to the exact double-precision path, and how many faces the
// positivity limiter blended.  Every translation unit is its own module, so
// each holds its own copy; HTR_DECISION_COUNTERS_ACCESS(name) defines the
// host function through which htr_decision_counters reads, clears and
// switches the copy of one translation unit.
// ---------------------------------------------------------------------------
enum DecisionCounter {
  kTenoFiltered = 0,  // TENO / TENO-A / TENO-LAD stencil selection taken by fast_mask
  kTenoExact,         // ... by the exact FP64 expression
  kSensorFiltered,    // shock-sensor node decided by an FP32 filter
  kSensorExact,       // ... by the exact FP64 expression
  kCutFiltered,       // sensor cut-off exponent taken from the FP32 argument
  kCutExact,          // ... from the exact FP64 argument
  kLimiterBlend,      // multi-species TENO face blended with the first-order flux
  kDecisionCounters
};
static_assert(kDecisionCounters == HTR_DECISION_COUNTERS, "counter count of the C ABI");
static __device__ unsigned long long g_decisions[kDecisionCounters];
static __device__ int g_count_decisions;
HTR_D void count_decision(int k) {
  if (g_count_decisions) atomicAdd(&g_decisions[k], 1ull);
}
#define HTR_DECISION_COUNTERS_ACCESS(NAME)                                                              \
  cudaError_t NAME(int enable, unsigned long long *out) {                                             \
    unsigned long long c[kDecisionCounters];                                                          \
    cudaError_t e = cudaMemcpyFromSymbol(c, g_decisions, sizeof(c));                                  \
    if (e != cudaSuccess) return e;                                                                   \
    for (int k = 0; k < kDecisionCounters; k++) out[k] += c[k];                                       \
    for (int k = 0; k < kDecisionCounters; k++) c[k] = 0ull;                                          \
    if ((e = cudaMemcpyToSymbol(g_decisions, c, sizeof(c))) != cudaSuccess) return e;                 \
    return cudaMemcpyToSymbol(g_count_decisions, &enable, sizeof(int));                               \
  }

enum NodeType { Std = 0, L_S, Lp1_S, Lp2_S, Rm3_S, Rm2_S, Rm1_S, R_S, L_C, Lp1_C, Rm2_C, Rm1_C, R_C };

// Boundary (ghost) nodes: their state is imposed by the boundary condition,
// never advanced by the RHS.
HTR_HD bool ghost_node(int t) { return t == L_S || t == R_S || t == L_C || t == R_C; }
// A face whose left node is a right-boundary ghost lies outside the domain.
HTR_HD bool outside_face(int t) { return t == R_S || t == R_C; }

// Per-cell kernels run over a whole grid of packed instances skip the
// boundary ghost nodes (in any direction with more than one cell).
struct GhostSkip {
  Fd<int> nt[3];
  unsigned active = 0;  // 0: skip nothing
  HTR_D bool at(const long long *p) const {
    bool g = false;
#pragma unroll
    for (int d = 0; d < 3; d++)
      if (active & (1u << d)) g = g || ghost_node(ld(nt[d].at(p)));
    return g;
  }
};
inline GhostSkip ghost_skip(const htr_fluid_view &v, unsigned active) {
  GhostSkip g;
  g.nt[0] = fd<int>(v.nType_x);
  g.nt[1] = fd<int>(v.nType_y);
  g.nt[2] = fd<int>(v.nType_z);
  g.active = active;
  return g;
}

struct NodeDev {
  int8_t off[5];
  int8_t kgOrder;
  double rp[4][6], rm[4][6];
  double cp[4], cm[4];
  double interp[2], grad[2];  // the reference's float tables (metric_coeffs.h:85-88), promoted
  double kg[3];
};

#define HTR_Z6 {0, 0, 0, 0, 0, 0}
#define HTR_STD_W {9.0 / 20.0, 6.0 / 20.0, 1.0 / 20.0, 4.0 / 20.0}
static __constant__ NodeDev kNode[13] = {
    {{-2, -1, 1, 2, 3}, 3,
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {2.0 / 6.0, -7.0 / 6.0, 11.0 / 6.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 3.0 / 12.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 11.0 / 6.0, -7.0 / 6.0, 2.0 / 6.0}, {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 3.0 / 12.0, 0.0, 0.0}},
     HTR_STD_W, HTR_STD_W, {0.5f, 0.5f}, {0.5f, 0.5f}, {3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0}},
    {{0, 0, 1, 1, 1}, 0,
     {{0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}},
     {{0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}},
     HTR_STD_W, HTR_STD_W, {1.0f, 0.0f}, {0.0f, 2.0f}, {0.0, 0.0, 0.0}},
    {{-1, -1, 1, 2, 3}, 1,
     {{0.0, -2.0 / 4.0, 5.0 / 4.0, 1.0 / 4.0, 0.0, 0.0}, {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      HTR_Z6, {0.0, 0.0, 3.0 / 12.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, {0.0, -2.0 / 4.0, 5.0 / 4.0, 1.0 / 4.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 11.0 / 6.0, -7.0 / 6.0, 2.0 / 6.0}, HTR_Z6},
     {2.0 / 4.0, 1.0 / 4.0, 0.0, 1.0 / 4.0}, {7.0 / 16.0, 8.0 / 16.0, 1.0 / 16.0, 0.0},
     {0.5f, 0.5f}, {1.0f, 0.5f}, {0.5, 0.0, 0.0}},
    {{-2, -1, 1, 2, 3}, 2,
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {1.0, -2.0, 2.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 3.0 / 12.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 11.0 / 6.0, -7.0 / 6.0, 2.0 / 6.0}, {3.0 / 9.0, -7.0 / 9.0, 11.0 / 9.0, 2.0 / 9.0, 0.0, 0.0}},
     {47.0 / 100.0, 27.0 / 100.0, 10.0 / 100.0, 16.0 / 100.0},
     {39.0 / 100.0, 27.0 / 100.0, 4.0 / 100.0, 30.0 / 100.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, {2.0 / 3.0, -1.0 / 12.0, 0.0}},
    {{-2, -1, 1, 2, 3}, 2,
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {2.0 / 6.0, -7.0 / 6.0, 11.0 / 6.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 2.0 / 9.0, 11.0 / 9.0, -7.0 / 9.0, 3.0 / 9.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 2.0, -2.0, 1.0}, {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 3.0 / 12.0, 0.0, 0.0}},
     {39.0 / 100.0, 27.0 / 100.0, 4.0 / 100.0, 30.0 / 100.0},
     {47.0 / 100.0, 27.0 / 100.0, 10.0 / 100.0, 16.0 / 100.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, {2.0 / 3.0, -1.0 / 12.0, 0.0}},
    {{-2, -1, 1, 2, 2}, 1,
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, {0.0, 0.0, 1.0 / 4.0, 5.0 / 4.0, -2.0 / 4.0, 0.0},
      {2.0 / 6.0, -7.0 / 6.0, 11.0 / 6.0, 0.0, 0.0, 0.0}, HTR_Z6},
     {{0.0, 0.0, 1.0 / 4.0, 5.0 / 4.0, -2.0 / 4.0, 0.0}, {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      HTR_Z6, {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 3.0 / 12.0, 0.0, 0.0}},
     {7.0 / 16.0, 8.0 / 16.0, 1.0 / 16.0, 0.0}, {2.0 / 4.0, 1.0 / 4.0, 0.0, 1.0 / 4.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, {0.5, 0.0, 0.0}},
    {{-1, -1, 1, 1, 1}, 0,
     {{0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}},
     {{0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}},
     HTR_STD_W, HTR_STD_W, {0.0f, 1.0f}, {0.5f, 1.0f}, {0.0, 0.0, 0.0}},
    {{-1, -1, 0, 0, 0}, 0, {HTR_Z6, HTR_Z6, HTR_Z6, HTR_Z6}, {HTR_Z6, HTR_Z6, HTR_Z6, HTR_Z6},
     {0, 0, 0, 0}, {0, 0, 0, 0}, {0.5f, 0.5f}, {2.0f, 0.0f}, {0.0, 0.0, 0.0}},
    {{0, 0, 1, 2, 2}, 1, {{0, 0, 1.0, 0, 0, 0}, HTR_Z6, HTR_Z6, HTR_Z6},
     {{0, 0, 0, 1.0, 0, 0}, HTR_Z6, HTR_Z6, HTR_Z6}, {1.0, 0.0, 0.0, 0.0}, {1.0, 0.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.0f, 1.0f}, {0.5, 0.0, 0.0}},
    {{-1, -1, 1, 2, 2}, 2,
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, HTR_Z6, HTR_Z6},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, HTR_Z6, HTR_Z6},
     {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0}, {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, {2.0 / 3.0, -1.0 / 12.0, 0.0}},
    {{-1, -1, 1, 2, 2}, 2,
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, HTR_Z6, HTR_Z6},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, HTR_Z6, HTR_Z6},
     {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0}, {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, {2.0 / 3.0, -1.0 / 12.0, 0.0}},
    {{-1, -1, 1, 1, 1}, 1, {{0, 0, 1.0, 0, 0, 0}, HTR_Z6, HTR_Z6, HTR_Z6},
     {{0, 0, 0, 1.0, 0, 0}, HTR_Z6, HTR_Z6, HTR_Z6}, {1.0, 0.0, 0.0, 0.0}, {1.0, 0.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, {0.5, 0.0, 0.0}},
    {{-1, -1, 0, 0, 0}, 0, {HTR_Z6, HTR_Z6, HTR_Z6, HTR_Z6}, {HTR_Z6, HTR_Z6, HTR_Z6, HTR_Z6},
     {0, 0, 0, 0}, {0, 0, 0, 0}, {0.5f, 0.5f}, {1.0f, 0.0f}, {0.0, 0.0, 0.0}},
};
#undef HTR_Z6
#undef HTR_STD_W

// Powers of ten as float (TENO cut-offs).
static __constant__ float kP10[14] = {1,    1e-1, 1e-2, 1e-3,  1e-4,  1e-5,  1e-6,
                                      1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12, 1e-13};

HTR_D double interp2(int t, double a, double b) {
  return __dadd_rn(__dmul_rn(kNode[t].interp[0], a), __dmul_rn(kNode[t].interp[1], b));
}
HTR_D double deriv(int t, double xm1, double x, double xp1, double m) {
  return __dmul_rn(__dadd_rn(__dmul_rn(kNode[t].grad[0], __dsub_rn(x, xm1)),
                             __dmul_rn(kNode[t].grad[1], __dsub_rn(xp1, x))),
                   m);
}

// ---------------------------------------------------------------------------
// correctly rounded x^n in double-double (Dekker / Knuth error-free products)
// ---------------------------------------------------------------------------
struct DD {
  double h, l;
};
HTR_D DD dd_sq(double x) {
  DD r;
  r.h = __dmul_rn(x, x);
  r.l = __fma_rn(x, x, -r.h);
  return r;
}
HTR_D DD dd_mul_d(DD a, double x) {  // (a.h + a.l) * x
  DD r;
  const double p = __dmul_rn(a.h, x);
  const double e = __fma_rn(a.h, x, -p);
  const double l = __fma_rn(a.l, x, e);
  r.h = __dadd_rn(p, l);
  r.l = __dsub_rn(l, __dsub_rn(r.h, p));
  return r;
}
HTR_D DD dd_square(DD a) {  // (a.h + a.l)^2, dropping a.l^2
  DD r;
  const double p = __dmul_rn(a.h, a.h);
  const double e = __fma_rn(a.h, a.h, -p);
  const double l = __fma_rn(__dadd_rn(a.h, a.h), a.l, e);
  r.h = __dadd_rn(p, l);
  r.l = __dsub_rn(l, __dsub_rn(r.h, p));
  return r;
}
HTR_D double dd_round(DD a) {
  // an overflowed leading term is returned as is (the error terms are NaN there)
  return isinf(a.h) ? a.h : __dadd_rn(a.h, a.l);
}
HTR_D double pow4_exact(double x) { return dd_round(dd_square(dd_sq(x))); }
HTR_D DD pow6_dd(double x) { return dd_square(dd_mul_d(dd_sq(x), x)); }
HTR_D double pow6_exact(double x) { return dd_round(pow6_dd(x)); }
HTR_D double pow12_exact(double x) {
  const DD s = pow6_dd(x);
  if (isinf(s.h)) return s.h;
  return dd_round(dd_square(s));
}

// ---------------------------------------------------------------------------
// smoothness measures of the four TENO candidates (metric.inl:442-449)
// ---------------------------------------------------------------------------
struct Smooth {
  double s1, s2, s3, s4, tau6;
};
HTR_D Smooth smoothness(double ym2, double ym1, double y, double yp1, double yp2, double yp3) {
  const double C13 = 13.0 / 12.0, C23 = 3.0 / 12.0, C14 = 1.0 / 36.0, C24 = 13.0 / 12.0,
               C34 = 781.0 / 720.0;
  Smooth s;
  double a1, a2, a3;
  a1 = (ym1 - 2 * y + yp1);
  a2 = (ym1 - yp1);
  s.s1 = C13 * a1 * a1 + C23 * a2 * a2;
  a1 = (y - 2 * yp1 + yp2);
  a2 = (3 * y - 4 * yp1 + yp2);
  s.s2 = C13 * a1 * a1 + C23 * a2 * a2;
  a1 = (ym2 - 2 * ym1 + y);
  a2 = (3 * y - 4 * ym1 + ym2);
  s.s3 = C13 * a1 * a1 + C23 * a2 * a2;
  a1 = (-11 * y + 18 * yp1 - 9 * yp2 + 2 * yp3);
  a2 = (2 * y - 5 * yp1 + 4 * yp2 - yp3);
  a3 = (-y + 3 * yp1 - 3 * yp2 + yp3);
  s.s4 = C14 * a1 * a1 + C24 * a2 * a2 + C34 * a3 * a3;
  s.tau6 = fabs(s.s4 - (s.s3 + s.s2 + 4 * s.s1) / 6);
  return s;
}

// ---------------------------------------------------------------------------
// FP32 decision filter for TENO stencil selection.
//
// The selection flag of candidate k is  a_k * (1 / sum_j a_j) >= cut  with
// a_k = (1 + tau6/(s_k + eps))^6.  The weights' values are never used, only
// the flags.  This filter evaluates q_k = a_k / sum_j a_j in single precision
// as (x_k/m)^6 / sum_j (x_j/m)^6 (m = max x_j, so nothing overflows) from the
// exact double-precision smoothness measures.  Every single-precision
// operation is correctly rounded (u = 2^-24), so |q_k - exact| <= 142 u q_k
// (conversion, add and divide 5u on x_k, 11u on the ratio, 69u on its sixth
// power, 72u on the sum, 142u on the quotient).  A flag is taken from the
// filter only when q_k is further than 1e-4 * cut from cut (70x that bound);
// otherwise the caller evaluates the exact double-precision expression.  The
// flags therefore equal the reference's bit for bit while most faces skip
// the 5 double divisions and 4 double sixth powers.
// ---------------------------------------------------------------------------
struct FastX {
  float x[4];
  bool ok;
};
HTR_D FastX fast_x(const Smooth &s, double eps) {
  FastX f;
  const double big = 1e30;
  f.ok = (s.tau6 < big) && (s.s1 < big) && (s.s2 < big) && (s.s3 < big) && (s.s4 < big);
  // round-to-nearest conversions on the integer pipe; values below 2^-126
  // become zero, negligible against eps >= 1e-16
  const float t = df_round_float(s.tau6);
  const float e = __double2float_rn(eps);
  f.x[0] = __fadd_rn(1.0f, __fdiv_rn(t, __fadd_rn(df_round_float(s.s1), e)));
  f.x[1] = __fadd_rn(1.0f, __fdiv_rn(t, __fadd_rn(df_round_float(s.s2), e)));
  f.x[2] = __fadd_rn(1.0f, __fdiv_rn(t, __fadd_rn(df_round_float(s.s3), e)));
  f.x[3] = __fadd_rn(1.0f, __fdiv_rn(t, __fadd_rn(df_round_float(s.s4), e)));
  return f;
}
HTR_D float pow6f(float r) {
  const float r2 = __fmul_rn(r, r);
  const float r3 = __fmul_rn(r2, r);
  return __fmul_rn(r3, r3);
}
// Flags (bit k = stencil k kept) for the `used` candidates, or -1 when any
// flag lies inside the safety margin.  Unused candidates get flag 0.
HTR_D int fast_mask(const FastX &f, unsigned used, double cut) {
  if (!f.ok || used == 0u) return -1;
  float m = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (used & (1u << k)) m = fmaxf(m, f.x[k]);
  if (!(m >= 1.0f)) return -1;  // NaN guard
  float q[4], S = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    q[k] = (used & (1u << k)) ? pow6f(__fdiv_rn(f.x[k], m)) : 0.0f;
    S = __fadd_rn(S, q[k]);
  }
  const float c = (float)cut;
  const float hi = c * 1.0001f, lo = c * 0.9999f;
  int mask = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (!(used & (1u << k))) continue;
    const float qk = __fdiv_rn(q[k], S);
    if (qk >= hi)
      mask |= 1 << k;
    else if (!(qk <= lo))
      return -1;
  }
  return mask;
}



// ---------------------------------------------------------------------------
// Smoothness measures in single precision with a rigorous bound on their
// absolute error, from six point values v[] already converted to float
// (conversion error at most u |v| <= uM): every stencil difference with
// integer coefficients c_i and k rounded operations is within (k + 2) u C M
// of its exact value (C = sum |c_i|; the +2 covers the conversion), squares
// and sums add at most a few u relative to the (positive) terms.  Used by
// the shock sensor's interval filter below.
// ---------------------------------------------------------------------------
struct SmoothF {
  float s[4], e[4];  // s_k and the bound on its error
  float tau, et;     // tau6 and its bound
};
HTR_D SmoothF smooth_f32(float v0, float v1, float v2, float v3, float v4, float v5, float uM) {
  const float u = 5.9604645e-08f;
  // s = A a^2 + B b^2 and the bound on its error
  auto sq2 = [&](float A, float a, float ea, float B, float b, float eb, float &e) {
    const float t = __fadd_rn(__fmul_rn(__fmul_rn(A, a), a), __fmul_rn(__fmul_rn(B, b), b));
    e = A * ea * (2.0f * fabsf(a) + ea) + B * eb * (2.0f * fabsf(b) + eb) + 8.0f * u * t;
    return t;
  };
  const float C13 = 13.0f / 12.0f, C23 = 3.0f / 12.0f, C14 = 1.0f / 36.0f, C24 = 13.0f / 12.0f,
              C34 = 781.0f / 720.0f;
  SmoothF r;
  // s1: a = ym1 - 2y + yp1 (C 4, 2 ops), b = ym1 - yp1 (C 2, 1 op)
  r.s[0] = sq2(C13, __fadd_rn(__fsub_rn(v1, 2.0f * v2), v3), 4.0f * 4.0f * uM, C23, __fsub_rn(v1, v3),
               3.0f * 2.0f * uM, r.e[0]);
  // s2: a = y - 2yp1 + yp2 (C 4, 2), b = 3y - 4yp1 + yp2 (C 8, 3)
  r.s[1] = sq2(C13, __fadd_rn(__fsub_rn(v2, 2.0f * v3), v4), 4.0f * 4.0f * uM, C23,
               __fadd_rn(__fsub_rn(__fmul_rn(3.0f, v2), 4.0f * v3), v4), 5.0f * 8.0f * uM, r.e[1]);
  // s3: a = ym2 - 2ym1 + y (C 4, 2), b = 3y - 4ym1 + ym2 (C 8, 3)
  r.s[2] = sq2(C13, __fadd_rn(__fsub_rn(v0, 2.0f * v1), v2), 4.0f * 4.0f * uM, C23,
               __fadd_rn(__fsub_rn(__fmul_rn(3.0f, v2), 4.0f * v1), v0), 5.0f * 8.0f * uM, r.e[2]);
  // s4: a = -11y + 18yp1 - 9yp2 + 2yp3 (C 40, 6), b = 2y - 5yp1 + 4yp2 - yp3 (C 12, 4),
  //     c = -y + 3yp1 - 3yp2 + yp3 (C 8, 5)
  const float a4 = __fadd_rn(__fsub_rn(__fadd_rn(__fmul_rn(-11.0f, v2), __fmul_rn(18.0f, v3)), __fmul_rn(9.0f, v4)),
                             2.0f * v5);
  const float b4 = __fsub_rn(__fadd_rn(__fsub_rn(2.0f * v2, __fmul_rn(5.0f, v3)), 4.0f * v4), v5);
  const float c4 = __fadd_rn(__fsub_rn(__fadd_rn(-v2, __fmul_rn(3.0f, v3)), __fmul_rn(3.0f, v4)), v5);
  const float ea4 = 8.0f * 40.0f * uM, eb4 = 6.0f * 12.0f * uM, ec4 = 7.0f * 8.0f * uM;
  r.s[3] = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(C14, a4), a4), __fmul_rn(__fmul_rn(C24, b4), b4)),
                     __fmul_rn(__fmul_rn(C34, c4), c4));
  r.e[3] = C14 * ea4 * (2.0f * fabsf(a4) + ea4) + C24 * eb4 * (2.0f * fabsf(b4) + eb4) +
           C34 * ec4 * (2.0f * fabsf(c4) + ec4) + 10.0f * u * r.s[3];
  const float comb = __fdiv_rn(__fadd_rn(__fadd_rn(r.s[2], r.s[1]), 4.0f * r.s[0]), 6.0f);
  r.tau = fabsf(__fsub_rn(r.s[3], comb));
  r.et = r.e[3] + (r.e[2] + r.e[1] + 4.0f * r.e[0]) / 6.0f + 6.0f * u * (r.s[3] + comb);
  return r;
}

// One TENO reconstruction at face c+1/2 from y = (c-2 .. c+3); MINUS gives
// the right-biased value (metric.inl:431-1038).  Returns the 4 selection
// flags in *mask (bit k = stencil k kept).
// FMA: contract the reconstruction from the selected stencils (it feeds no
// selection) into fused multiply-adds; false keeps the reference's rounding.
template <int KIND, bool MINUS, bool FMA = false>
HTR_D double teno(double ym2, double ym1, double y, double yp1, double yp2, double yp3, int t,
                  unsigned *mask) {
  // optimal weights of this side (tables indexed directly: constant space)
  const double W0 = MINUS ? kNode[t].cm[0] : kNode[t].cp[0];
  const double W1 = MINUS ? kNode[t].cm[1] : kNode[t].cp[1];
  const double W2 = MINUS ? kNode[t].cm[2] : kNode[t].cp[2];
  const double W3 = MINUS ? kNode[t].cm[3] : kNode[t].cp[3];
  const double eps = KIND == kTENO ? 1e-10 : (KIND == kTENOA ? 1e-8 : 1e-16);
  int fmask = -1;
  const unsigned used_all = (W0 < 1e-10 ? 0u : 1u) | (W1 < 1e-10 ? 0u : 2u) | (W2 < 1e-10 ? 0u : 4u) |
                            (W3 < 1e-10 ? 0u : 8u);
  const Smooth s = MINUS ? smoothness(yp3, yp2, yp1, y, ym1, ym2) : smoothness(ym2, ym1, y, yp1, yp2, yp3);
  if (KIND != kTENOA || t != Std) {
    // second filter on the double-precision smoothness measures (see
    // fast_mask); TENO-A on standard nodes adapts its cut-off to a Ren
    // sensor and always takes the exact path
    const unsigned used = used_all;
    const FastX fx = fast_x(s, eps);
    double fcut = 1e-6;
    bool cut_ok = true;
    if (KIND == kTENOA) {
      fcut = double(kP10[4]);
    } else if (KIND == kTENOLAD) {
      const float e = __double2float_rn(eps), tt = df_round_float(s.tau6);
      float cm = __fdiv_rn(tt, __fadd_rn(df_round_float(s.s1), e));
      cm = fmaxf(cm, __fdiv_rn(tt, __fadd_rn(df_round_float(s.s2), e)));
      cm = fmaxf(cm, __fdiv_rn(tt, __fadd_rn(df_round_float(s.s3), e)));
      cm = fmaxf(cm, __fdiv_rn(tt, __fadd_rn(df_round_float(s.s4), e)));
      const float arg = 3.0f + 9.5f / (1.0f + cm * 0.1f);
      const float fl = floorf(arg);
      // the exact argument 3 + 9.5 theta is never below 3 (theta > 0), so a
      // power of 3 needs the margin only towards 4 (smooth regions, where
      // chi is huge, sit just above 3)
      cut_ok = fx.ok && (fl <= 3.0f || arg - fl > 1e-3f) && (fl + 1.0f - arg > 1e-3f);
      fcut = double(kP10[min(max(int(fl), 0), 13)]);
    }
    if (cut_ok) fmask = fast_mask(fx, used, fcut);
  }
  if (fmask >= 0) {
    if (mask) *mask = unsigned(fmask);
  }
  int b1, b2, b3, b4;
  if (fmask >= 0) {
    count_decision(kTenoFiltered);
    b1 = fmask & 1;
    b2 = (fmask >> 1) & 1;
    b3 = (fmask >> 2) & 1;
    b4 = (fmask >> 3) & 1;
  } else {
  count_decision(kTenoExact);
  const double chi1 = s.tau6 / (s.s1 + eps);
  const double chi2 = s.tau6 / (s.s2 + eps);
  const double chi3 = s.tau6 / (s.s3 + eps);
  const double chi4 = s.tau6 / (s.s4 + eps);
  double a1 = pow6_exact(1 + chi1);
  double a2 = pow6_exact(1 + chi2);
  double a3 = pow6_exact(1 + chi3);
  double a4 = pow6_exact(1 + chi4);
  double cut;
  bool zero_unused = true;
  if (KIND == kTENO) {
    cut = 1e-6;
  } else if (KIND == kTENOA) {
    if (t == Std) {
      zero_unused = false;
      const double rc = 0.2;
      const double Ren_eps = 0.9 * rc * 1e-16 / (1.0 - 0.9 * rc);
      const double Ren_irc = 1.0 / rc;
      const double v2 = fabs(ym1 - ym2), v3 = fabs(y - ym1), v4 = fabs(yp1 - y);
      const double v5 = fabs(yp2 - yp1), v6 = fabs(yp3 - yp2);
      double eta = smin((2 * v2 * v3 + Ren_eps) / (v2 * v2 + v3 * v3 + Ren_eps),
                        (2 * v3 * v4 + Ren_eps) / (v3 * v3 + v4 * v4 + Ren_eps));
      eta = smin(eta, (2 * v4 * v5 + Ren_eps) / (v4 * v4 + v5 * v5 + Ren_eps));
      eta = smin(eta, (2 * v5 * v6 + Ren_eps) / (v5 * v5 + v6 * v6 + Ren_eps));
      const double delta = 1 - smin(eta * Ren_irc, 1.0);
      const double decay = pow4_exact(1 - delta) * (1 + 4 * delta);
      const int power = min(max(int(floor(9.5 - 3.5 * (1 - decay))), 0), 13);
      cut = double(kP10[power]);
    } else {
      cut = double(kP10[4]);
    }
  } else {
    const double chiMax = smax(chi1, smax(chi2, smax(chi3, chi4)));
    const double theta = 1.0 / (1 + chiMax * 1e-1);
    const int power = min(max(int(floor(3.0 + 9.5 * theta)), 0), 13);
    cut = double(kP10[power]);
  }
  if (zero_unused) {
    if (W0 < 1e-10) a1 = 0.0;
    if (W1 < 1e-10) a2 = 0.0;
    if (W2 < 1e-10) a3 = 0.0;
    if (W3 < 1e-10) a4 = 0.0;
  }
  const double a = 1.0 / (a1 + a2 + a3 + a4);
  b1 = (a1 * a < cut) ? 0 : 1;
  b2 = (a2 * a < cut) ? 0 : 1;
  b3 = (a3 * a < cut) ? 0 : 1;
  b4 = (a4 * a < cut) ? 0 : 1;
  if (mask) *mask = unsigned(b1) | (unsigned(b2) << 1) | (unsigned(b3) << 2) | (unsigned(b4) << 3);
  }
  const double base = MINUS ? yp1 : y;
  double v[4];
  if (FMA && t == Std) {
    if (!MINUS) {
      v[0] = __fma_rn(ym1, -1.0 / 6.0, __fma_rn(y, 5.0 / 6.0, __fma_rn(yp1, 2.0 / 6.0, -base)));
      v[1] = __fma_rn(y, 2.0 / 6.0, __fma_rn(yp1, 5.0 / 6.0, __fma_rn(yp2, -1.0 / 6.0, -base)));
      v[2] = __fma_rn(ym2, 2.0 / 6.0, __fma_rn(ym1, -7.0 / 6.0, __fma_rn(y, 11.0 / 6.0, -base)));
      v[3] = __fma_rn(y, 3.0 / 12.0,
                      __fma_rn(yp1, 13.0 / 12.0, __fma_rn(yp2, -5.0 / 12.0, __fma_rn(yp3, 1.0 / 12.0, -base))));
    } else {
      v[0] = __fma_rn(y, 2.0 / 6.0, __fma_rn(yp1, 5.0 / 6.0, __fma_rn(yp2, -1.0 / 6.0, -base)));
      v[1] = __fma_rn(ym1, -1.0 / 6.0, __fma_rn(y, 5.0 / 6.0, __fma_rn(yp1, 2.0 / 6.0, -base)));
      v[2] = __fma_rn(yp1, 11.0 / 6.0, __fma_rn(yp2, -7.0 / 6.0, __fma_rn(yp3, 2.0 / 6.0, -base)));
      v[3] = __fma_rn(ym2, 1.0 / 12.0,
                      __fma_rn(ym1, -5.0 / 12.0, __fma_rn(y, 13.0 / 12.0, __fma_rn(yp1, 3.0 / 12.0, -base))));
    }
  } else if (t == Std) {
    // zero entries of the standard stencils skipped: adding an exact zero
    // does not change a rounded sum.
    if (!MINUS) {
      v[0] = ym1 * (-1.0 / 6.0) + y * (5.0 / 6.0) + yp1 * (2.0 / 6.0) - base;
      v[1] = y * (2.0 / 6.0) + yp1 * (5.0 / 6.0) + yp2 * (-1.0 / 6.0) - base;
      v[2] = ym2 * (2.0 / 6.0) + ym1 * (-7.0 / 6.0) + y * (11.0 / 6.0) - base;
      v[3] = y * (3.0 / 12.0) + yp1 * (13.0 / 12.0) + yp2 * (-5.0 / 12.0) + yp3 * (1.0 / 12.0) - base;
    } else {
      v[0] = y * (2.0 / 6.0) + yp1 * (5.0 / 6.0) + yp2 * (-1.0 / 6.0) - base;
      v[1] = ym1 * (-1.0 / 6.0) + y * (5.0 / 6.0) + yp1 * (2.0 / 6.0) - base;
      v[2] = yp1 * (11.0 / 6.0) + yp2 * (-7.0 / 6.0) + yp3 * (2.0 / 6.0) - base;
      v[3] = ym2 * (1.0 / 12.0) + ym1 * (-5.0 / 12.0) + y * (13.0 / 12.0) + yp1 * (3.0 / 12.0) - base;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const double r0 = MINUS ? kNode[t].rm[k][0] : kNode[t].rp[k][0];
      const double r1 = MINUS ? kNode[t].rm[k][1] : kNode[t].rp[k][1];
      const double r2 = MINUS ? kNode[t].rm[k][2] : kNode[t].rp[k][2];
      const double r3 = MINUS ? kNode[t].rm[k][3] : kNode[t].rp[k][3];
      const double r4 = MINUS ? kNode[t].rm[k][4] : kNode[t].rp[k][4];
      const double r5 = MINUS ? kNode[t].rm[k][5] : kNode[t].rp[k][5];
      v[k] = ym2 * r0 + ym1 * r1 + y * r2 + yp1 * r3 + yp2 * r4 + yp3 * r5 - base;
    }
  }
  double w1, w2, w3, w4;
  if (t == Std && b1 && b2 && b3 && b4) {
    // every standard candidate kept (smooth flow): the normalised optimal
    // weights, the same operations as below evaluated once
    constexpr double ia = 1.0 / (((9.0 / 20.0 + 6.0 / 20.0) + 1.0 / 20.0) + 4.0 / 20.0);
    w1 = (9.0 / 20.0) * ia;
    w2 = (6.0 / 20.0) * ia;
    w3 = (1.0 / 20.0) * ia;
    w4 = (4.0 / 20.0) * ia;
  } else {
    const double c1 = W0 * b1, c2 = W1 * b2, c3 = W2 * b3, c4 = W3 * b4;
    const double ia = 1.0 / (c1 + c2 + c3 + c4);
    w1 = c1 * ia;
    w2 = c2 * ia;
    w3 = c3 * ia;
    w4 = c4 * ia;
  }
  if (FMA) return __fma_rn(w4, v[3], __fma_rn(w3, v[2], __fma_rn(w2, v[1], __fma_rn(w1, v[0], base))));
  return base + w1 * v[0] + w2 * v[1] + w3 * v[2] + w4 * v[3];
}

// Cut-off of the hybrid shock sensor from the Ducros value of the stencil
// (metric.inl:395-397); shared by every species of a cell and direction.
HTR_D double sensor_cut(double Phi) {
  const double decay = pow12_exact(1 - Phi) * (1 + 12 * Phi);
  const int power = min(max(int(floor(12.5 - 11.5 * (1 - decay))), 0), 13);
  return double(kP10[power]);
}

// ---------------------------------------------------------------------------
// FP32 pre-decision of the shock sensor with rigorous error bounds.
//
// The sensor of a node is true iff a_k / sum_j a_j > cut for its four
// candidates, a_k = (1 + tau6 / (s_k + eps))^6, with the smoothness measures
// s_k and tau6 of six point values.  sensor_prefilter evaluates s_k and tau6
// in single precision together with an upper bound on the absolute error of
// each: every stencil difference with integer coefficients c_i and k
// rounded operations is within (k + 2) u C M of its exact value (C = sum
// |c_i|, M = max |y_i|, u = 2^-24; the +2 covers the conversion of the
// inputs), squares and sums add at most a few u relative to the (positive)
// terms.  From those bounds it forms intervals for x_k = 1 + tau6/(s_k+eps)
// and for q_k = x_k^6 / sum_j x_j^6, and returns a decision only when every
// interval lies on one side of cut by more than 1e-3 cut, far above the
// relative rounding of the interval arithmetic itself (below 1e-5).  It
// returns -1 otherwise (and for large or non-finite inputs); the caller then
// evaluates the sensor exactly in double precision.  Decisions therefore equal
// the double-precision ones.
// ---------------------------------------------------------------------------
HTR_D int sensor_prefilter(double ym2, double ym1, double y0, double yp1, double yp2, double yp3,
                           double cut) {
  const float u = 5.9604645e-08f;
  // round-to-nearest conversions on the integer pipe (the conversion
  // instruction runs at the FP64 rate on this part); values below 2^-126
  // become zero, within the u M conversion bound as long as M >= 2^-100
  const float v0 = df_round_float(ym2), v1 = df_round_float(ym1), v2 = df_round_float(y0),
              v3 = df_round_float(yp1), v4 = df_round_float(yp2), v5 = df_round_float(yp3);
  float M = fmaxf(fmaxf(fmaxf(fabsf(v0), fabsf(v1)), fmaxf(fabsf(v2), fabsf(v3))), fmaxf(fabsf(v4), fabsf(v5)));
  if (!(M < 1e6f) || !(M >= 7.88860905e-31f)) return -1;  // 2^-100
  const SmoothF sm = smooth_f32(v0, v1, v2, v3, v4, v5, u * M);
  const float tau = sm.tau, et = sm.et;
  const float s1 = sm.s[0], s2 = sm.s[1], s3 = sm.s[2], s4 = sm.s[3];
  const float e1 = sm.e[0], e2 = sm.e[1], e3 = sm.e[2], e4 = sm.e[3];
  const float eps = 1e-8f;
  const float tlo = fmaxf(tau - et, 0.0f), thi = tau + et;
  const float sv[4] = {s1, s2, s3, s4}, ev[4] = {e1, e2, e3, e4};
  float xl[4], xh[4], m = 1.0f;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    xl[k] = 1.0f + tlo / (sv[k] + ev[k] + eps);
    xh[k] = 1.0f + thi / (fmaxf(sv[k] - ev[k], 0.0f) + eps);
    m = fmaxf(m, xh[k]);
  }
  float pl[4], ph[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    pl[k] = pow6f(xl[k] / m);
    ph[k] = pow6f(xh[k] / m);
  }
  const float cf = (float)cut;
  bool all_smooth = true, any_shock = false;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float ol = 0.0f, oh = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (j != k) {
        ol += pl[j];
        oh += ph[j];
      }
    const float qlo = pl[k] / (pl[k] + oh);
    const float qhi = ph[k] / (ph[k] + ol);
    all_smooth = all_smooth && (qlo > cf * 1.001f);
    any_shock = any_shock || (qhi < cf * 0.999f);
  }
  if (all_smooth) return 1;
  if (any_shock) return 0;
  return -1;
}

// sensor_cut with an FP32 pre-decision: decay and the exponent argument in
// single precision (absolute error of the argument below 3e-4 for Phi in
// [0, 1]); the integer part is taken from it when the argument is further
// than 1e-3 from an integer, otherwise the exact double-precision path runs.
HTR_D double sensor_cut_fast(double Phi) {
  if (Phi >= 0.0 && Phi <= 1.0) {
    const float P = df_round_float(Phi);
    const float w = __fsub_rn(1.0f, P);
    const float w2 = __fmul_rn(w, w), w3 = __fmul_rn(w2, w), w6 = __fmul_rn(w3, w3), w12 = __fmul_rn(w6, w6);
    const float d = __fmul_rn(w12, __fadd_rn(1.0f, __fmul_rn(12.0f, P)));
    const float z = __fsub_rn(12.5f, __fmul_rn(11.5f, __fsub_rn(1.0f, d)));
    const float fl = floorf(z), fr = z - fl;
    if (fr > 1e-3f && fr < 1.0f - 1e-3f) {
      count_decision(kCutFiltered);
      return double(kP10[min(max(int(fl), 0), 13)]);
    }
  }
  count_decision(kCutExact);
  return sensor_cut(Phi);
}

// Shock sensor of the hybrid scheme on a positive scalar (metric.inl:351-403),
// true = smooth; `cut` from sensor_cut.
HTR_D bool teno_a_sensor(double ym2, double ym1, double y, double yp1, double yp2, double yp3,
                         int t, double cut) {
  const double rc = 0.2;
  const double Ren_eps = 0.9 * rc * 1e-6 / (1.0 - 0.9 * rc);
  const double Ren_irc = 1.0 / rc;
  if (t == L_S || t == Rm1_S) return true;
  if (t == L_C || t == Rm1_C) {
    const double v1 = (t == L_C) ? yp1 - y : y - ym1;
    const double v2 = (t == L_C) ? yp2 - yp1 : yp1 - y;
    const double eta = (fabs(2.0 * v1 * v2) + Ren_eps) / (v1 * v1 + v2 * v2 + Ren_eps);
    return ((1.0 - smin(1.0, Ren_irc * eta)) < 0.5);
  }
  const int pre = sensor_prefilter(ym2, ym1, y, yp1, yp2, yp3, cut);
  if (pre >= 0) {
    count_decision(kSensorFiltered);
    return pre == 1;
  }
  const Smooth s = smoothness(ym2, ym1, y, yp1, yp2, yp3);
  const double eps = 1e-8;
  // strict comparison a_k*a > cut: the filter's flag "q >= cut(1+1e-4)"
  // implies it, "q <= cut(1-1e-4)" refutes it
  const int fm = fast_mask(fast_x(s, eps), 15u, cut);
  if (fm >= 0) {
    count_decision(kSensorFiltered);
    return fm == 15;
  }
  count_decision(kSensorExact);
  const double a1 = pow6_exact(1 + s.tau6 / (s.s1 + eps));
  const double a2 = pow6_exact(1 + s.tau6 / (s.s2 + eps));
  const double a3 = pow6_exact(1 + s.tau6 / (s.s3 + eps));
  const double a4 = pow6_exact(1 + s.tau6 / (s.s4 + eps));
  const double a = 1.0 / (a1 + a2 + a3 + a4);
  return ((a1 * a > cut) && (a2 * a > cut) && (a3 * a > cut) && (a4 * a > cut));
}

}  // namespace htr
