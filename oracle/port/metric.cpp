// CPU oracle port: grid metrics of a stretched Cartesian grid.
// TEST INFRASTRUCTURE ONLY.
//
//   InitializeMetricTask         src/prometeo_metric.hpp:93-181, src/prometeo_metric.cc:36-178
//   CorrectGhostMetricTask<dir>  src/prometeo_metric.hpp:183-268, src/prometeo_metric.cc:180-213
//
// Every metric is the inverse of a coordinate difference.  The Euler metric
// of point i is 1 / (x_{i+1/2} - x_{i-1/2}), where x_{i+1/2} is the linear
// (optimal-weight) reconstruction of the centre coordinate to the face
// (src/prometeo_metric.inl:193-208) with the node type's candidate stencils;
// the diffusion metrics use the node's two-point gradient weights and the
// forward difference.  Periodic stencils see coordinates shifted by the
// domain width (src/prometeo_metric.hpp:48-86).
#include <cstdint>

#include "htr_rhs.h"
#include "stencils.hpp"

using namespace oport;

namespace {

struct Field {
  char *b;
  int64_t s[3];
  explicit Field(const htr_field &f) : b(static_cast<char *>(f.base)) {
    for (int i = 0; i < 3; i++) s[i] = f.stride[i];
  }
  template <class T> T *at(const long long *p) const {
    return reinterpret_cast<T *>(b + p[0] * s[0] + p[1] * s[1] + p[2] * s[2]);
  }
};

// Coordinate of the stencil point reached from p with offset `off` after the
// periodic wrap, moved back by whole widths next to p.
double unwarp(double x, double w, int off, long long p, long long lo, long long hi) {
  p += off;
  if (p < lo) {
    x -= w;
    p += 1;
  }
  return x + w * static_cast<long long>((p - lo) / (hi - lo + 1));
}

struct Line {
  Field cc, nt;
  int d;
  long long lo, hi, size;
  double w;
  double coord(const long long *p) const { return cc.at<double>(p)[d]; }
  int type(const long long *p) const { return *nt.at<int>(p); }
  // coordinate of the point p + off (wrapped), unwarped relative to p
  double at_off(const long long *p, int off, bool minus) const {
    long long q[3] = {p[0], p[1], p[2]};
    q[d] = minus ? wrap_minus(p[d], lo, size, off) : wrap_plus(p[d], lo, size, off);
    return unwarp(coord(q), w, off, p[d], lo, hi);
  }
  // face coordinate x_{p+1/2}
  double face(const long long *p) const {
    const int t = type(p);
    const int8_t *o = kNodes[t].off;
    const double y[6] = {at_off(p, o[0], true), at_off(p, o[1], true), coord(p),
                         at_off(p, o[2], false), at_off(p, o[3], false), at_off(p, o[4], false)};
    if (t == R_C) return 0.0;
    if (t == L_C || t == Rm1_C) return 0.5 * y[2] + 0.5 * y[3];
    const NodeRec &n = kNodes[t];
    double acc = 0.0;
    for (int j = 0; j < 6; j++) {
      const double a = n.rp[0][j] * n.cp[0] + n.rp[1][j] * n.cp[1] + n.rp[2][j] * n.cp[2] + n.rp[3][j] * n.cp[3];
      acc = (j == 0) ? y[0] * a : acc + y[j] * a;
    }
    return acc;
  }
};

template <class F> void for_points(const htr_rect3 &r, F &&f) {
#pragma omp parallel for collapse(3)
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        const long long p[3] = {i, j, k};
        f(p);
      }
}

bool bad_rect(const htr_rect3 &r) {
  for (int d = 0; d < 3; d++)
    if (r.hi[d] < r.lo[d]) return true;
  return false;
}

int correct(const htr_fluid_view *v, htr_field cc, htr_rect3 myf, int d) {
  if (v == nullptr || cc.base == nullptr || bad_rect(myf)) return HTR_ERR_ARGUMENT;
  const htr_field *nts[3] = {&v->nType_x, &v->nType_y, &v->nType_z};
  const htr_field *ms[3] = {&v->dcsi_e, &v->deta_e, &v->dzet_e};
  const Field c(cc), nt(*nts[d]), m(*ms[d]);
  for_points(myf, [&](const long long *p) {
    const int t = *nt.at<int>(p);
    if (t != L_S && t != L_C && t != R_S && t != R_C) return;
    const int dir = (t == L_S || t == L_C) ? 1 : -1;
    long long q1[3] = {p[0], p[1], p[2]}, q2[3] = {p[0], p[1], p[2]};
    q1[d] += dir;
    q2[d] += 2 * dir;
    if (q2[d] < myf.lo[d] || q2[d] > myf.hi[d]) return;  // an axis too short for a one-sided difference
    const double x0 = c.at<double>(p)[d], x1 = c.at<double>(q1)[d], x2 = c.at<double>(q2)[d];
    double den;
    if (t == L_S)
      den = (-(8.0 / 3.0) * x0 + 3.0 * x1) - (1.0 / 3.0) * x2;
    else if (t == L_C)
      den = (-1.5 * x0 + 2.0 * x1) - 0.5 * x2;
    else if (t == R_S)
      den = ((8.0 / 3.0) * x0 - 3.0 * x1) + (1.0 / 3.0) * x2;
    else
      den = (1.5 * x0 - 2.0 * x1) + 0.5 * x2;
    *m.at<double>(p) = 1.0 / den;
  });
  return HTR_OK;
}

}  // namespace

extern "C" {

int htr_InitializeMetric(const htr_fluid_view *v, htr_field cc, htr_rect3 myf, htr_rect3 fb, const double width[3],
                         htr_stream_t) {
  if (v == nullptr || cc.base == nullptr || width == nullptr || bad_rect(myf) || bad_rect(fb))
    return HTR_ERR_ARGUMENT;
  const htr_field *nts[3] = {&v->nType_x, &v->nType_y, &v->nType_z};
  const htr_field *me[3] = {&v->dcsi_e, &v->deta_e, &v->dzet_e};
  const htr_field *md[3] = {&v->dcsi_d, &v->deta_d, &v->dzet_d};
  const htr_field *msg[3] = {&v->dcsi_s, &v->deta_s, &v->dzet_s};
  for (int d = 0; d < 3; d++) {
    const Line L{Field(cc), Field(*nts[d]), d, fb.lo[d], fb.hi[d], fb.hi[d] - fb.lo[d] + 1, width[d]};
    const Field e(*me[d]), dd(*md[d]), s(*msg[d]);
    for_points(myf, [&](const long long *p) {
      const double xp = L.face(p);
      double xm;
      if (p[d] > myf.lo[d]) {
        long long q[3] = {p[0], p[1], p[2]};
        q[d] -= 1;
        xm = L.face(q);
      } else {
        long long q[3] = {p[0], p[1], p[2]};
        q[d] = wrap_minus(p[d], L.lo, L.size, kNodes[L.type(p)].off[1]);
        xm = unwarp(L.face(q), L.w, -1, p[d], L.lo, L.hi);
      }
      *e.at<double>(p) = 1.0 / (xp - xm);
      const int t = L.type(p);
      long long qm[3] = {p[0], p[1], p[2]}, qp[3] = {p[0], p[1], p[2]};
      qm[d] = wrap_minus(p[d], L.lo, L.size, kNodes[t].off[1]);
      qp[d] = wrap_plus(p[d], L.lo, L.size, kNodes[t].off[2]);
      const double x = L.coord(p);
      const double xm1 = unwarp(L.coord(qm), L.w, -1, p[d], L.lo, L.hi);
      const double xp1 = unwarp(L.coord(qp), L.w, 1, p[d], L.lo, L.hi);
      *s.at<double>(p) = 1.0 / (xp1 - x);
      *dd.at<double>(p) = 1.0 / deriv(t, xm1, x, xp1, 1.0);
    });
  }
  return HTR_OK;
}

int htr_CorrectGhostMetricX(const htr_fluid_view *v, htr_field cc, htr_rect3 myf, htr_stream_t) {
  return correct(v, cc, myf, 0);
}
int htr_CorrectGhostMetricY(const htr_fluid_view *v, htr_field cc, htr_rect3 myf, htr_stream_t) {
  return correct(v, cc, myf, 1);
}
int htr_CorrectGhostMetricZ(const htr_fluid_view *v, htr_field cc, htr_rect3 myf, htr_stream_t) {
  return correct(v, cc, myf, 2);
}

}  // extern "C"
