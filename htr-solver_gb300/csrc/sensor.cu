// Shock sensors of the hybrid scheme.
//
// Replaces UpdateDucrosSensorTask and UpdateShockSensorTask<dir>
// (src/prometeo_sensor.hpp:49-131, src/prometeo_sensor.inl:47-76,
// src/prometeo_sensor.cc:33-128).  Compiled with -fmad=false so the Ducros
// value and the TENO-A selection are rounded exactly as on the CPU and the
// boolean sensors agree bit for bit.
#include "kernels.cuh"
#include "stencil.cuh"

namespace htr {

struct SensorArgs {
  Fd<double> u, C, duc, mx, my_, mz;
  Fd<int> nx, ny, nz;
  Fd<bool> sx, sy, sz;
  Box my, fb;
  long long nyz, n0;
};

HTR_D void cell_of(const SensorArgs &a, long long idx, long long *p) {
  const long long nx = a.my.size(0), ny = a.my.size(1);
  p[0] = a.my.lo[0] + idx % nx;
  p[1] = a.my.lo[1] + (idx / nx) % ny;
  p[2] = a.my.lo[2] + idx / (nx * ny);
}

HTR_D void shift(const SensorArgs &a, long long *q, const long long *p, int e, int off, bool plus) {
  q[0] = p[0];
  q[1] = p[1];
  q[2] = p[2];
  q[e] = plus ? wrap_plus(p[e], a.fb.lo[e], a.fb.size(e), off)
              : wrap_minus(p[e], a.fb.lo[e], a.fb.size(e), off);
}

__global__ void ducros_kernel(const SensorArgs a, double eps, long long n) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    cell_of(a, idx, p);
    double g[3][3];
#pragma unroll
    for (int e = 0; e < 3; e++) {
      const Fd<int> &nt = e == 0 ? a.nx : (e == 1 ? a.ny : a.nz);
      const Fd<double> &m = e == 0 ? a.mx : (e == 1 ? a.my_ : a.mz);
      const int t = ld(nt.at(p));
      long long pm[3], pp[3];
      shift(a, pm, p, e, kNode[t].off[1], false);
      shift(a, pp, p, e, kNode[t].off[2], true);
      const double mm = ld(m.at(p));
#pragma unroll
      for (int i = 0; i < 3; i++)
        g[e][i] = deriv(t, ld(&a.u.at(pm)[i]), ld(&a.u.at(p)[i]), ld(&a.u.at(pp)[i]), mm);
    }
    const double div = g[0][0] + g[1][1] + g[2][2];
    const double div2 = div * div;
    const double omz = g[0][1] - g[1][0];
    const double omy = g[1][2] - g[2][1];
    const double omx = g[2][0] - g[0][2];
    const double om2 = omx * omx + omy * omy + omz * omz;
    *a.duc.at(p) = div2 / (div2 + om2 + eps);
  }
}

// The sensor test of one species as one out-of-line copy shared by the
// three directions: unrolled over 5 species and 3 directions the kernel
// stalled on instruction-cache misses more than on anything else, and three
// inlined copies still did (a 256^3 step: 222.0 ms with those, 219.4 ms with
// this one).
static __device__ __noinline__ bool sensor_test(double ym2, double ym1, double y, double yp1, double yp2,
                                                double yp3, int t, double cut) {
  return teno_a_sensor(ym2, ym1, y, yp1, yp2, yp3, t, cut);
}

// The TENO-A shock sensor of one direction E at cell p: true when every
// species' partial density is smooth there.
template <int NS, int E>
HTR_D bool shock_dir(const SensorArgs &a, const long long *p) {
  const Fd<int> &nt = E == 0 ? a.nx : (E == 1 ? a.ny : a.nz);
  const int t = ld(nt.at(p));
  long long q[6][3];
  shift(a, q[0], p, E, kNode[t].off[0], false);
  shift(a, q[1], p, E, kNode[t].off[1], false);
  q[2][0] = p[0];
  q[2][1] = p[1];
  q[2][2] = p[2];
  shift(a, q[3], p, E, kNode[t].off[2], true);
  shift(a, q[4], p, E, kNode[t].off[3], true);
  shift(a, q[5], p, E, kNode[t].off[4], true);
  double Phi = ld(a.duc.at(q[0]));
#pragma unroll
  for (int k = 1; k < 6; k++) Phi = smax(Phi, ld(a.duc.at(q[k])));
  const double cut = sensor_cut_fast(Phi);
  const double *c[6];
#pragma unroll
  for (int k = 0; k < 6; k++) c[k] = a.C.at(q[k]);
  bool s = true;
#pragma unroll 1
  for (int h = 0; h < NS && s; h++)
    s = sensor_test(ld(&c[0][h]), ld(&c[1][h]), ld(&c[2][h]), ld(&c[3][h]), ld(&c[4][h]), ld(&c[5][h]), t, cut);
  return s;
}

template <int NS>
__global__ void __launch_bounds__(256, 4) shock_kernel(const SensorArgs a, int dirmask, long long n) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    cell_of(a, idx, p);
    if (dirmask & 1) *a.sx.at(p) = shock_dir<NS, 0>(a, p);
    if (dirmask & 2) *a.sy.at(p) = shock_dir<NS, 1>(a, p);
    if (dirmask & 4) *a.sz.at(p) = shock_dir<NS, 2>(a, p);
  }
}

static SensorArgs sensor_args(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb) {
  SensorArgs a;
  a.u = fd<double>(v.velocity);
  a.C = fd<double>(v.Conserved);
  a.duc = fd<double>(v.DucrosSensor);
  a.mx = fd<double>(v.dcsi_d);
  a.my_ = fd<double>(v.deta_d);
  a.mz = fd<double>(v.dzet_d);
  a.nx = fd<int>(v.nType_x);
  a.ny = fd<int>(v.nType_y);
  a.nz = fd<int>(v.nType_z);
  a.sx = fd<bool>(v.shockSensorX);
  a.sy = fd<bool>(v.shockSensorY);
  a.sz = fd<bool>(v.shockSensorZ);
  a.my = box(my);
  a.fb = box(fb);
  return a;
}

// One cell per thread (the grid-stride loops only matter past the launch
// limit; a grid capped at 152 x 64 blocks was slower on a 256^3 box).
static dim3 grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 0x7fffffffLL) b = 0x7fffffffLL;
  return dim3((unsigned)(b > 0 ? b : 1));
}

cudaError_t launch_ducros(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                          double vorticityScale, cudaStream_t s) {
  const SensorArgs a = sensor_args(v, my, fb);
  const long long n = a.my.size(0) * a.my.size(1) * a.my.size(2);
  const double eps = smax(vorticityScale * vorticityScale, 1e-6);
  ducros_kernel<<<grid_for(n, 256), 256, 0, s>>>(a, eps, n);
  return cudaGetLastError();
}

cudaError_t launch_shock_sensor(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                                int nspec, int dirmask, cudaStream_t s) {
  const SensorArgs a = sensor_args(v, my, fb);
  const long long n = a.my.size(0) * a.my.size(1) * a.my.size(2);
  if (nspec == 1)
    shock_kernel<1><<<grid_for(n, 256), 256, 0, s>>>(a, dirmask, n);
  else if (nspec == 5)
    shock_kernel<5><<<grid_for(n, 256), 256, 0, s>>>(a, dirmask, n);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// decision counters of this translation unit (htr_decision_counters)
HTR_DECISION_COUNTERS_ACCESS(decision_counters_sensor)

}  // namespace htr
