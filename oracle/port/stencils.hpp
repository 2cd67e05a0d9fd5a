// CPU oracle port: stencil tables and reconstruction operators.
// TEST INFRASTRUCTURE ONLY.
//
// The 13 node types of the reference (src/prometeo_metric_coeffs.h:54-66)
// with their offsets, TENO candidate stencils, optimal weights,
// staggered-interpolation / gradient weights and Kennedy-Gruber orders,
// restated as one record per node type (values of
// src/prometeo_metric_coeffs_macros.h and src/prometeo_metric_coeffs.cc:36-232).
// Operators follow src/prometeo_metric.inl.
#ifndef HTR_ORACLE_PORT_STENCILS_HPP
#define HTR_ORACLE_PORT_STENCILS_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace oport {

enum NodeType {
  Std = 0, L_S, Lp1_S, Lp2_S, Rm3_S, Rm2_S, Rm1_S, R_S, L_C, Lp1_C, Rm2_C, Rm1_C, R_C, kNodeTypes
};

struct NodeRec {
  int8_t off[5];      // stencil offsets of points m2, m1, p1, p2, p3
  double rp[4][6];    // candidate stencils, plus side, applied to [c-2 .. c+3]
  double rm[4][6];    // candidate stencils, minus side
  double cp[4];       // optimal weights, plus side
  double cm[4];       // optimal weights, minus side
  float interp[2];    // staggered interpolation [c, c+1]
  float grad[2];      // cell-centre gradient [c - c-1, c+1 - c]
  int8_t kgOrder;     // Kennedy-Gruber order (1 = 2nd, 2 = 4th, 3 = 6th)
  double kg[3];       // Kennedy-Gruber coefficients
  int8_t kgNSum;      // number of running sums refreshed per point
};

#define Z6 {0, 0, 0, 0, 0, 0}

static const NodeRec kNodes[kNodeTypes] = {
    // Std
    {{-2, -1, 1, 2, 3},
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {2.0 / 6.0, -7.0 / 6.0, 11.0 / 6.0, 0.0, 0.0, 0.0},
      {0.0, 0.0, 3.0 / 12.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 11.0 / 6.0, -7.0 / 6.0, 2.0 / 6.0},
      {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 3.0 / 12.0, 0.0, 0.0}},
     {9.0 / 20.0, 6.0 / 20.0, 1.0 / 20.0, 4.0 / 20.0},
     {9.0 / 20.0, 6.0 / 20.0, 1.0 / 20.0, 4.0 / 20.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, 3, {3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0}, 3},
    // L_S: boundary node sitting on the face
    {{0, 0, 1, 1, 1},
     {{0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}},
     {{0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}, {0, 0, 1.0, 0, 0, 0}},
     {9.0 / 20.0, 6.0 / 20.0, 1.0 / 20.0, 4.0 / 20.0},
     {9.0 / 20.0, 6.0 / 20.0, 1.0 / 20.0, 4.0 / 20.0},
     {1.0f, 0.0f}, {0.0f, 2.0f}, 0, {0.0, 0.0, 0.0}, 0},
    // Lp1_S
    {{-1, -1, 1, 2, 3},
     {{0.0, -2.0 / 4.0, 5.0 / 4.0, 1.0 / 4.0, 0.0, 0.0},
      {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      Z6,
      {0.0, 0.0, 3.0 / 12.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {0.0, -2.0 / 4.0, 5.0 / 4.0, 1.0 / 4.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 11.0 / 6.0, -7.0 / 6.0, 2.0 / 6.0},
      Z6},
     {2.0 / 4.0, 1.0 / 4.0, 0.0, 1.0 / 4.0},
     {7.0 / 16.0, 8.0 / 16.0, 1.0 / 16.0, 0.0},
     {0.5f, 0.5f}, {1.0f, 0.5f}, 1, {0.5, 0.0, 0.0}, 3},
    // Lp2_S
    {{-2, -1, 1, 2, 3},
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {1.0, -2.0, 2.0, 0.0, 0.0, 0.0},
      {0.0, 0.0, 3.0 / 12.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 11.0 / 6.0, -7.0 / 6.0, 2.0 / 6.0},
      {3.0 / 9.0, -7.0 / 9.0, 11.0 / 9.0, 2.0 / 9.0, 0.0, 0.0}},
     {47.0 / 100.0, 27.0 / 100.0, 10.0 / 100.0, 16.0 / 100.0},
     {39.0 / 100.0, 27.0 / 100.0, 4.0 / 100.0, 30.0 / 100.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, 2, {2.0 / 3.0, -1.0 / 12.0, 0.0}, 3},
    // Rm3_S
    {{-2, -1, 1, 2, 3},
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {2.0 / 6.0, -7.0 / 6.0, 11.0 / 6.0, 0.0, 0.0, 0.0},
      {0.0, 0.0, 2.0 / 9.0, 11.0 / 9.0, -7.0 / 9.0, 3.0 / 9.0}},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 2.0, -2.0, 1.0},
      {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 3.0 / 12.0, 0.0, 0.0}},
     {39.0 / 100.0, 27.0 / 100.0, 4.0 / 100.0, 30.0 / 100.0},
     {47.0 / 100.0, 27.0 / 100.0, 10.0 / 100.0, 16.0 / 100.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, 2, {2.0 / 3.0, -1.0 / 12.0, 0.0}, 2},
    // Rm2_S
    {{-2, -1, 1, 2, 2},
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 1.0 / 4.0, 5.0 / 4.0, -2.0 / 4.0, 0.0},
      {2.0 / 6.0, -7.0 / 6.0, 11.0 / 6.0, 0.0, 0.0, 0.0},
      Z6},
     {{0.0, 0.0, 1.0 / 4.0, 5.0 / 4.0, -2.0 / 4.0, 0.0},
      {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      Z6,
      {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 3.0 / 12.0, 0.0, 0.0}},
     {7.0 / 16.0, 8.0 / 16.0, 1.0 / 16.0, 0.0},
     {2.0 / 4.0, 1.0 / 4.0, 0.0, 1.0 / 4.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, 1, {0.5, 0.0, 0.0}, 1},
    // Rm1_S: the next node sits on the face
    {{-1, -1, 1, 1, 1},
     {{0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}},
     {{0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}, {0, 0, 0, 1.0, 0, 0}},
     {9.0 / 20.0, 6.0 / 20.0, 1.0 / 20.0, 4.0 / 20.0},
     {9.0 / 20.0, 6.0 / 20.0, 1.0 / 20.0, 4.0 / 20.0},
     {0.0f, 1.0f}, {0.5f, 1.0f}, 0, {0.0, 0.0, 0.0}, 0},
    // R_S
    {{-1, -1, 0, 0, 0}, {Z6, Z6, Z6, Z6}, {Z6, Z6, Z6, Z6}, {0, 0, 0, 0}, {0, 0, 0, 0},
     {0.5f, 0.5f}, {2.0f, 0.0f}, 0, {0.0, 0.0, 0.0}, 0},
    // L_C
    {{0, 0, 1, 2, 2},
     {{0, 0, 1.0, 0, 0, 0}, Z6, Z6, Z6},
     {{0, 0, 0, 1.0, 0, 0}, Z6, Z6, Z6},
     {1.0, 0.0, 0.0, 0.0}, {1.0, 0.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.0f, 1.0f}, 1, {0.5, 0.0, 0.0}, 3},
    // Lp1_C
    {{-1, -1, 1, 2, 2},
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, Z6, Z6},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, Z6, Z6},
     {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0}, {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, 2, {2.0 / 3.0, -1.0 / 12.0, 0.0}, 3},
    // Rm2_C
    {{-1, -1, 1, 2, 2},
     {{0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0},
      {0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0}, Z6, Z6},
     {{0.0, 0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0},
      {0.0, -1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0}, Z6, Z6},
     {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0}, {1.0 / 2.0, 1.0 / 2.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, 2, {2.0 / 3.0, -1.0 / 12.0, 0.0}, 2},
    // Rm1_C
    {{-1, -1, 1, 1, 1},
     {{0, 0, 1.0, 0, 0, 0}, Z6, Z6, Z6},
     {{0, 0, 0, 1.0, 0, 0}, Z6, Z6, Z6},
     {1.0, 0.0, 0.0, 0.0}, {1.0, 0.0, 0.0, 0.0},
     {0.5f, 0.5f}, {0.5f, 0.5f}, 1, {0.5, 0.0, 0.0}, 1},
    // R_C
    {{-1, -1, 0, 0, 0}, {Z6, Z6, Z6, Z6}, {Z6, Z6, Z6, Z6}, {0, 0, 0, 0}, {0, 0, 0, 0},
     {0.5f, 0.5f}, {1.0f, 0.0f}, 0, {0.0, 0.0, 0.0}, 0},
};
#undef Z6

// TENO cut-off table (powers of ten as float, src/prometeo_metric_coeffs.cc:228-229).
static const float kP10[14] = {1,    1e-1, 1e-2, 1e-3,  1e-4,  1e-5,  1e-6,
                               1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12, 1e-13};

inline double interp2(int t, double a, double b) {
  return kNodes[t].interp[0] * (a) + kNodes[t].interp[1] * (b);
}
inline double deriv(int t, double xm1, double x, double xp1, double m) {
  return (kNodes[t].grad[0] * (x - xm1) + kNodes[t].grad[1] * (xp1 - x)) * m;
}

// Kennedy-Gruber split-form reconstructions (src/prometeo_metric.inl:210-292).
inline double kg3(const double *rho, const double *u, const double *phi, int t) {
  if (t == L_S) return rho[2] * u[2] * phi[2];
  if (t == Rm1_S) return rho[3] * u[3] * phi[3];
  double flux = 0.0;
  for (int l = 0; l < kNodes[t].kgOrder; l++) {
    const int lp = l + 1;
    double acc = 0.0;
    for (int m = 0; m < lp; m++)
      acc += ((rho[2 - m] + rho[2 - m + lp]) * (u[2 - m] + u[2 - m + lp]) *
              (phi[2 - m] + phi[2 - m + lp]));
    flux += kNodes[t].kg[l] * acc;
  }
  return flux * 0.25;
}
inline double kg1(const double *phi, int t) {
  if (t == L_S) return phi[2];
  if (t == Rm1_S) return phi[3];
  double flux = 0.0;
  for (int l = 0; l < kNodes[t].kgOrder; l++) {
    const int lp = l + 1;
    double acc = 0.0;
    for (int m = 0; m < lp; m++) acc += (phi[2 - m] + phi[2 - m + lp]);
    flux += kNodes[t].kg[l] * acc;
  }
  return flux;
}

// Jiang-Shu-type smoothness measures of the four TENO candidates, for the
// stencil y[0..5] = (c-2 .. c+3) oriented towards the face c+1/2.
struct Smooth {
  double s1, s2, s3, s4, tau6;
};
constexpr double C13 = 13.0 / 12.0, C23 = 3.0 / 12.0, C14 = 1.0 / 36.0, C24 = 13.0 / 12.0,
                 C34 = 781.0 / 720.0;
inline Smooth smooth(double ym2, double ym1, double y, double yp1, double yp2, double yp3) {
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
  s.tau6 = std::fabs(s.s4 - (s.s3 + s.s2 + 4 * s.s1) / 6);
  return s;
}

enum TenoKind { kTENO, kTENOA, kTENOLAD };

// One TENO reconstruction (src/prometeo_metric.inl:431-1038).  `minus`
// reconstructs the right-biased value; its smoothness measures use the
// mirrored stencil.  `sel` (optional) receives the 4 stencil-selection flags.
inline double teno(TenoKind kind, bool minus, double ym2, double ym1, double y, double yp1,
                   double yp2, double yp3, int t, int *sel = nullptr) {
  const NodeRec &nr = kNodes[t];
  const double *W = minus ? nr.cm : nr.cp;
  const double(*R)[6] = minus ? nr.rm : nr.rp;
  const Smooth s = minus ? smooth(yp3, yp2, yp1, y, ym1, ym2) : smooth(ym2, ym1, y, yp1, yp2, yp3);
  const double eps = kind == kTENO ? 1e-10 : (kind == kTENOA ? 1e-8 : 1e-16);
  const double chi1 = s.tau6 / (s.s1 + eps);
  const double chi2 = s.tau6 / (s.s2 + eps);
  const double chi3 = s.tau6 / (s.s3 + eps);
  const double chi4 = s.tau6 / (s.s4 + eps);
  double a1 = std::pow(1 + chi1, 6);
  double a2 = std::pow(1 + chi2, 6);
  double a3 = std::pow(1 + chi3, 6);
  double a4 = std::pow(1 + chi4, 6);
  float cut;
  if (kind == kTENO) {
    if (W[0] < 1e-10) a1 = 0.0;
    if (W[1] < 1e-10) a2 = 0.0;
    if (W[2] < 1e-10) a3 = 0.0;
    if (W[3] < 1e-10) a4 = 0.0;
    cut = 1e-6;  // a double constant in the reference; 1e-6 compared as double below
  } else if (kind == kTENOA) {
    if (t == Std) {
      // Ren et al. smoothness indicator over the 6 points (metric.inl:635-660);
      // this operator's regularisation is 1e-16 (metric.inl:811-813)
      const double rc = 0.2;
      const double Ren_eps = 0.9 * rc * 1e-16 / (1.0 - 0.9 * rc);
      const double Ren_irc = 1.0 / rc;
      const double v2 = std::fabs(ym1 - ym2), v3 = std::fabs(y - ym1), v4 = std::fabs(yp1 - y);
      const double v5 = std::fabs(yp2 - yp1), v6 = std::fabs(yp3 - yp2);
      double eta = std::min((2 * v2 * v3 + Ren_eps) / (v2 * v2 + v3 * v3 + Ren_eps),
                            (2 * v3 * v4 + Ren_eps) / (v3 * v3 + v4 * v4 + Ren_eps));
      eta = std::min(eta, (2 * v4 * v5 + Ren_eps) / (v4 * v4 + v5 * v5 + Ren_eps));
      eta = std::min(eta, (2 * v5 * v6 + Ren_eps) / (v5 * v5 + v6 * v6 + Ren_eps));
      const double delta = 1 - std::min(eta * Ren_irc, 1.0);
      const double decay = std::pow((1 - delta), 4) * (1 + 4 * delta);
      const int power = std::min(std::max(int(std::floor(9.5 - 3.5 * (1 - decay))), 0), 13);
      cut = kP10[power];
    } else {
      if (W[0] < 1e-10) a1 = 0.0;
      if (W[1] < 1e-10) a2 = 0.0;
      if (W[2] < 1e-10) a3 = 0.0;
      if (W[3] < 1e-10) a4 = 0.0;
      cut = kP10[4];
    }
  } else {
    if (W[0] < 1e-10) a1 = 0.0;
    if (W[1] < 1e-10) a2 = 0.0;
    if (W[2] < 1e-10) a3 = 0.0;
    if (W[3] < 1e-10) a4 = 0.0;
    const double chiMax = std::max(chi1, std::max(chi2, std::max(chi3, chi4)));
    const double theta = 1.0 / (1 + chiMax * 1e-1);
    const int power = std::min(std::max(int(std::floor(3.0 + 9.5 * theta)), 0), 13);
    cut = kP10[power];
  }
  double a = 1.0 / (a1 + a2 + a3 + a4);
  int b1, b2, b3, b4;
  if (kind == kTENO) {
    const double c = 1e-6;
    b1 = (a1 * a < c) ? 0 : 1;
    b2 = (a2 * a < c) ? 0 : 1;
    b3 = (a3 * a < c) ? 0 : 1;
    b4 = (a4 * a < c) ? 0 : 1;
  } else {
    b1 = (a1 * a < cut) ? 0 : 1;
    b2 = (a2 * a < cut) ? 0 : 1;
    b3 = (a3 * a < cut) ? 0 : 1;
    b4 = (a4 * a < cut) ? 0 : 1;
  }
  if (sel) {
    sel[0] = b1;
    sel[1] = b2;
    sel[2] = b3;
    sel[3] = b4;
  }
  const double base = minus ? yp1 : y;
  double var[4];
  for (int k = 0; k < 4; k++)
    var[k] = ym2 * R[k][0] + ym1 * R[k][1] + y * R[k][2] + yp1 * R[k][3] + yp2 * R[k][4] +
             yp3 * R[k][5] - base;
  a1 = W[0] * b1;
  a2 = W[1] * b2;
  a3 = W[2] * b3;
  a4 = W[3] * b4;
  a = 1.0 / (a1 + a2 + a3 + a4);
  const double w1 = a1 * a, w2 = a2 * a, w3 = a3 * a, w4 = a4 * a;
  return base + w1 * var[0] + w2 * var[1] + w3 * var[2] + w4 * var[3];
}

// Shock sensor of the hybrid scheme: TENO-A-style selection on a positive
// scalar with a cut-off adapted to the Ducros value Phi
// (src/prometeo_metric.inl:351-403).  True = smooth.
inline bool teno_a_sensor(double ym2, double ym1, double y, double yp1, double yp2, double yp3,
                          int t, double Phi) {
  const double rc = 0.2;
  const double Ren_eps = 0.9 * rc * 1e-6 / (1.0 - 0.9 * rc);
  const double Ren_irc = 1.0 / rc;
  if (t == L_S || t == Rm1_S) return true;
  if (t == L_C || t == Rm1_C) {
    const double v1 = (t == L_C) ? yp1 - y : y - ym1;
    const double v2 = (t == L_C) ? yp2 - yp1 : yp1 - y;
    const double eta = (std::fabs(2.0 * v1 * v2) + Ren_eps) / (v1 * v1 + v2 * v2 + Ren_eps);
    return ((1.0 - std::min(1.0, Ren_irc * eta)) < 0.5);
  }
  const Smooth s = smooth(ym2, ym1, y, yp1, yp2, yp3);
  const double eps = 1e-8;
  const double a1 = std::pow(1 + s.tau6 / (s.s1 + eps), 6);
  const double a2 = std::pow(1 + s.tau6 / (s.s2 + eps), 6);
  const double a3 = std::pow(1 + s.tau6 / (s.s3 + eps), 6);
  const double a4 = std::pow(1 + s.tau6 / (s.s4 + eps), 6);
  const double a = 1.0 / (a1 + a2 + a3 + a4);
  const double decay = std::pow((1 - Phi), 12) * (1 + 12 * Phi);
  const int power = std::min(std::max(int(std::floor(12.5 - 11.5 * (1 - decay))), 0), 13);
  const float cut = kP10[power];
  return ((a1 * a > cut) && (a2 * a > cut) && (a3 * a > cut) && (a4 * a > cut));
}

// Periodic wrap of a stencil point (src/Utils/PointDomain_helper.hpp:160-190).
inline long long wrap_minus(long long p, long long lo, long long size, int off) {
  return ((p + off - lo) % size + size) % size + lo;
}
inline long long wrap_plus(long long p, long long lo, long long size, int off) {
  return (p + off - lo) % size + lo;
}

}  // namespace oport

#endif
