// Grid metrics of a stretched Cartesian grid on the device.
//
// Replaces InitializeMetricTask (src/prometeo_metric.hpp:93-181,
// src/prometeo_metric.cc:36-178) and CorrectGhostMetricTask<dir>
// (src/prometeo_metric.hpp:183-268, src/prometeo_metric.cc:180-213).
// One thread per point.  The Euler metric is 1 / (x_{i+1/2} - x_{i-1/2}) with
// the faces reconstructed linearly (optimal weights of the node's candidate
// stencils, src/prometeo_metric.inl:193-208); the reference carries the
// previous point's face along its line, a thread here reconstructs both
// faces, with the same operations.  This translation unit is compiled with
// -fmad=false, so the results are bit-identical to the CPU builds.
#include "kernels.cuh"
#include "stencil.cuh"

namespace htr {

namespace {

struct MetricArgs {
  Fd<double> cc;  // Vec3 per point
  Fd<int> nt[3];
  Fd<double> me[3], md[3], ms[3];
  Box my, fb;
  double w[3];
};

HTR_D double unwarp(double x, double w, int off, long long p, long long lo, long long hi) {
  p += off;
  if (p < lo) {
    x -= w;
    p += 1;
  }
  return x + w * (double)((p - lo) / (hi - lo + 1));
}

template <int D> HTR_D double coord_at(const MetricArgs &a, const long long *p, int off, bool minus) {
  long long q[3] = {p[0], p[1], p[2]};
  const long long lo = a.fb.lo[D], size = a.fb.size(D);
  q[D] = minus ? wrap_minus(p[D], lo, size, off) : wrap_plus(p[D], lo, size, off);
  return unwarp(a.cc.at(q)[D], a.w[D], off, p[D], lo, a.fb.hi[D]);
}

template <int D> HTR_D double face(const MetricArgs &a, const long long *p) {
  const int t = *a.nt[D].at(p);
  const NodeDev &n = kNode[t];
  const double y[6] = {coord_at<D>(a, p, n.off[0], true), coord_at<D>(a, p, n.off[1], true), a.cc.at(p)[D],
                       coord_at<D>(a, p, n.off[2], false), coord_at<D>(a, p, n.off[3], false),
                       coord_at<D>(a, p, n.off[4], false)};
  if (t == R_C) return 0.0;
  if (t == L_C || t == Rm1_C) return 0.5 * y[2] + 0.5 * y[3];
  double acc = 0.0;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const double c = n.rp[0][j] * n.cp[0] + n.rp[1][j] * n.cp[1] + n.rp[2][j] * n.cp[2] + n.rp[3][j] * n.cp[3];
    acc = (j == 0) ? y[0] * c : acc + y[j] * c;
  }
  return acc;
}

template <int D> HTR_D void metrics(const MetricArgs &a, const long long *p) {
  const double xp = face<D>(a, p);
  const int t = *a.nt[D].at(p);
  long long q[3] = {p[0], p[1], p[2]};
  double xm;
  if (p[D] > a.my.lo[D]) {
    q[D] = p[D] - 1;
    xm = face<D>(a, q);
  } else {
    q[D] = wrap_minus(p[D], a.fb.lo[D], a.fb.size(D), kNode[t].off[1]);
    xm = unwarp(face<D>(a, q), a.w[D], -1, p[D], a.fb.lo[D], a.fb.hi[D]);
  }
  *a.me[D].at(p) = 1.0 / (xp - xm);
  long long qm[3] = {p[0], p[1], p[2]}, qp[3] = {p[0], p[1], p[2]};
  qm[D] = wrap_minus(p[D], a.fb.lo[D], a.fb.size(D), kNode[t].off[1]);
  qp[D] = wrap_plus(p[D], a.fb.lo[D], a.fb.size(D), kNode[t].off[2]);
  const double x = a.cc.at(p)[D];
  const double xm1 = unwarp(a.cc.at(qm)[D], a.w[D], -1, p[D], a.fb.lo[D], a.fb.hi[D]);
  const double xp1 = unwarp(a.cc.at(qp)[D], a.w[D], 1, p[D], a.fb.lo[D], a.fb.hi[D]);
  *a.ms[D].at(p) = 1.0 / (xp1 - x);
  *a.md[D].at(p) = 1.0 / deriv(t, xm1, x, xp1, 1.0);
}

HTR_D bool point_of(const Box &b, long long idx, long long *p) {
  const long long nx = b.size(0), ny = b.size(1), n = nx * ny * b.size(2);
  if (idx >= n) return false;
  p[0] = b.lo[0] + idx % nx;
  p[1] = b.lo[1] + (idx / nx) % ny;
  p[2] = b.lo[2] + idx / (nx * ny);
  return true;
}

__global__ void init_metric_kernel(const MetricArgs a) {
  long long p[3];
  if (!point_of(a.my, blockIdx.x * (long long)blockDim.x + threadIdx.x, p)) return;
  metrics<0>(a, p);
  metrics<1>(a, p);
  metrics<2>(a, p);
}

template <int D> __global__ void correct_metric_kernel(const MetricArgs a) {
  long long p[3];
  if (!point_of(a.my, blockIdx.x * (long long)blockDim.x + threadIdx.x, p)) return;
  const int t = *a.nt[D].at(p);
  if (t != L_S && t != L_C && t != R_S && t != R_C) return;
  const int dir = (t == L_S || t == L_C) ? 1 : -1;
  long long q1[3] = {p[0], p[1], p[2]}, q2[3] = {p[0], p[1], p[2]};
  q1[D] += dir;
  q2[D] += 2 * dir;
  if (q2[D] < a.my.lo[D] || q2[D] > a.my.hi[D]) return;  // an axis too short for a one-sided difference
  const double x0 = a.cc.at(p)[D], x1 = a.cc.at(q1)[D], x2 = a.cc.at(q2)[D];
  double den;
  if (t == L_S)
    den = (-(8.0 / 3.0) * x0 + 3.0 * x1) - (1.0 / 3.0) * x2;
  else if (t == L_C)
    den = (-1.5 * x0 + 2.0 * x1) - 0.5 * x2;
  else if (t == R_S)
    den = ((8.0 / 3.0) * x0 - 3.0 * x1) + (1.0 / 3.0) * x2;
  else
    den = (1.5 * x0 - 2.0 * x1) + 0.5 * x2;
  *a.me[D].at(p) = 1.0 / den;
}

MetricArgs metric_args(const htr_fluid_view &v, const htr_field &cc, const htr_rect3 &my, const htr_rect3 &fb,
                       const double *w) {
  MetricArgs a;
  a.cc = fd<double>(cc);
  a.nt[0] = fd<int>(v.nType_x);
  a.nt[1] = fd<int>(v.nType_y);
  a.nt[2] = fd<int>(v.nType_z);
  a.me[0] = fd<double>(v.dcsi_e);
  a.me[1] = fd<double>(v.deta_e);
  a.me[2] = fd<double>(v.dzet_e);
  a.md[0] = fd<double>(v.dcsi_d);
  a.md[1] = fd<double>(v.deta_d);
  a.md[2] = fd<double>(v.dzet_d);
  a.ms[0] = fd<double>(v.dcsi_s);
  a.ms[1] = fd<double>(v.deta_s);
  a.ms[2] = fd<double>(v.dzet_s);
  a.my = box(my);
  a.fb = box(fb);
  for (int d = 0; d < 3; d++) a.w[d] = w ? w[d] : 0.0;
  return a;
}

unsigned blocks_for(const Box &b, int threads) {
  const long long n = b.size(0) * b.size(1) * b.size(2);
  return (unsigned)((n + threads - 1) / threads);
}

}  // namespace

cudaError_t launch_init_metric(const htr_fluid_view &v, const htr_field &cc, const htr_rect3 &my, const htr_rect3 &fb,
                               const double *width, cudaStream_t s) {
  const MetricArgs a = metric_args(v, cc, my, fb, width);
  init_metric_kernel<<<blocks_for(a.my, 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_correct_metric(const htr_fluid_view &v, const htr_field &cc, const htr_rect3 &my, int dir,
                                  cudaStream_t s) {
  const MetricArgs a = metric_args(v, cc, my, my, nullptr);
  const unsigned g = blocks_for(a.my, 128);
  if (dir == 0) correct_metric_kernel<0><<<g, 128, 0, s>>>(a);
  else if (dir == 1) correct_metric_kernel<1><<<g, 128, 0, s>>>(a);
  else correct_metric_kernel<2><<<g, 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace htr
