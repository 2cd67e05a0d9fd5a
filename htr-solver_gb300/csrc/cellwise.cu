// Per-cell kernels: chemistry sources, implicit chemistry, state refresh,
// spectral radius and the SSP-RK3 bookkeeping.
//
//   AddChemistrySources           src/prometeo_chem.cc:71-110
//   UpdatePropertiesFromPrimitive src/prometeo_variables.hpp:52-89
//   UpdateConservedFromPrimitive  src/prometeo_variables.hpp:115-137
//   UpdatePrimitiveFromConserved  src/prometeo_variables.hpp:163-193
//   CalculateMaxSpectralRadius    src/prometeo_cfl.hpp:55-190
//   RK bookkeeping                src/prometeo_rk.rg:47-112
//
// One thread per cell, grid-stride loops sized to the SM count.  Iterative
// loops keep the reference's caps and report a hit through a status word
// instead of asserting.
#include "kernels.cuh"
#include "mixture.cuh"
#include "stencil.cuh"

namespace htr {

struct CellRange {
  Box my;
  long long n;
  HTR_D void point(long long idx, long long *p) const {
    const long long nx = my.size(0), ny = my.size(1);
    p[0] = my.lo[0] + idx % nx;
    p[1] = my.lo[1] + (idx / nx) % ny;
    p[2] = my.lo[2] + idx / (nx * ny);
  }
};

static CellRange cells(const htr_rect3 &r) {
  CellRange c;
  c.my = box(r);
  c.n = c.my.size(0) * c.my.size(1) * c.my.size(2);
  return c;
}

// One cell per thread (the grid-stride loops only matter past the launch
// limit).
static dim3 grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 0x7fffffffLL) b = 0x7fffffffLL;
  return dim3((unsigned)(b > 0 ? b : 1));
}

#define HTR_FOR_CELLS(R, IDX) \
  for (long long IDX = blockIdx.x * (long long)blockDim.x + threadIdx.x; IDX < (R).n; IDX += (long long)gridDim.x * blockDim.x)

HTR_D void flag_status(int *status, int code) {
  if (status) atomicMax(status, code);
}

// --- chemistry sources ------------------------------------------------------
template <class Mix>
__global__ void chem_sources_kernel(CellRange R, Fd<double> rho, Fd<double> P, Fd<double> T,
                                    Fd<double> Y, Fd<double> Ct, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    double y[NS], w[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) y[i] = ld(&Y.at(p)[i]);
    mix.ProductionRates(w, ld(rho.at(p)), ld(P.at(p)), ld(T.at(p)), y);
    double *ct = Ct.at(p);
#pragma unroll
    for (int i = 0; i < NS; i++) ct[i] += w[i];
  }
}

template <class Mix>
cudaError_t launch_chem_sources(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                                cudaStream_t s) {
  const CellRange R = cells(my);
  chem_sources_kernel<Mix><<<grid_for(R.n, 256), 256, 0, s>>>(
      R, fd<double>(v.rho), fd<double>(v.pressure), fd<double>(v.temperature),
      fd<double>(v.MassFracs), fd<double>(v.Conserved_t), mix);
  return cudaGetLastError();
}

// --- properties -------------------------------------------------------------
template <class Mix>
__global__ void properties_kernel(CellRange R, Fd<double> P, Fd<double> T, Fd<double> X,
                                  Fd<double> Y, Fd<double> rho, Fd<double> mu, Fd<double> lam,
                                  Fd<double> Di, Fd<double> SoS, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    double x[NS], y[NS], d[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) x[i] = ld(&X.at(p)[i]);
    const double Tp = ld(T.at(p)), Pp = ld(P.at(p));
    const double MixW = mix.MolarWeightFromXi(x);
    *rho.at(p) = mix.Rho(Pp, Tp, MixW);
    if constexpr (NS > 1) {
      double m, l;
      mix.TransportAt(Tp, Pp, MixW, x, m, l, d);
      *mu.at(p) = m;
      *lam.at(p) = l;
    } else {
      *mu.at(p) = mix.Viscosity(Tp, x);
      *lam.at(p) = mix.HeatConductivity(Tp, x);
      mix.Diffusivity(d, Pp, Tp, MixW, x);
    }
    mix.MassFractions(y, MixW, x);
    const double gamma = mix.Gamma(Tp, MixW, y);
    *SoS.at(p) = mix.SpeedOfSound(Tp, gamma, MixW);
    double *dp = Di.at(p), *yp = Y.at(p);
#pragma unroll
    for (int i = 0; i < NS; i++) {
      dp[i] = d[i];
      yp[i] = y[i];
    }
  }
}

template <class Mix>
cudaError_t launch_properties(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                              cudaStream_t s) {
  const CellRange R = cells(my);
  properties_kernel<Mix><<<grid_for(R.n, 128), 128, 0, s>>>(
      R, fd<double>(v.pressure), fd<double>(v.temperature), fd<double>(v.MolarFracs),
      fd<double>(v.MassFracs), fd<double>(v.rho), fd<double>(v.mu), fd<double>(v.lam),
      fd<double>(v.Di), fd<double>(v.SoS), mix);
  return cudaGetLastError();
}

// --- conserved from primitive -------------------------------------------------
template <class Mix>
__global__ void conserved_kernel(CellRange R, Fd<double> Y, Fd<double> T, Fd<double> u,
                                 Fd<double> rho, Fd<double> C, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    double y[NS], vel[3];
#pragma unroll
    for (int i = 0; i < NS; i++) y[i] = ld(&Y.at(p)[i]);
#pragma unroll
    for (int i = 0; i < 3; i++) vel[i] = ld(&u.at(p)[i]);
    const double r = ld(rho.at(p));
    double *c = C.at(p);
#pragma unroll
    for (int i = 0; i < NS; i++) c[i] = r * y[i];
#pragma unroll
    for (int i = 0; i < 3; i++) c[NS + i] = r * vel[i];
    c[NS + 3] = r * (0.5 * mod2(vel) + mix.InternalEnergy(ld(T.at(p)), y));
  }
}

template <class Mix>
cudaError_t launch_conserved(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                             cudaStream_t s) {
  const CellRange R = cells(my);
  conserved_kernel<Mix><<<grid_for(R.n, 256), 256, 0, s>>>(
      R, fd<double>(v.MassFracs), fd<double>(v.temperature), fd<double>(v.velocity),
      fd<double>(v.rho), fd<double>(v.Conserved), mix);
  return cudaGetLastError();
}

// --- primitive from conserved (Newton temperature solve) ----------------------
template <class Mix>
__global__ void primitive_kernel(CellRange R, Fd<double> C, Fd<double> T, Fd<double> P,
                                 Fd<double> X, Fd<double> u, int *status, const GhostSkip G,
                                 const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    if (G.active && G.at(p)) continue;
    const double *c = C.at(p);
    double rhoYi[NS], Yi[NS], x[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) rhoYi[i] = ld(&c[i]);
    const double rho = mix.RhoFromRhoYi(rhoYi);
    mix.YiFromRhoYi(Yi, rho, rhoYi);
    mix.ClipYi(Yi);
    const double MixW = mix.MolarWeightFromYi(Yi);
    mix.MolarFractions(x, MixW, Yi);
    const double rhoInv = 1.0 / rho;
    double vel[3];
#pragma unroll
    for (int i = 0; i < 3; i++) vel[i] = ld(&c[NS + i]) * rhoInv;
    const double e = ld(&c[NS + 3]) * rhoInv - 0.5 * mod2(vel);
    int its = 0;
    const double Tn = mix.TFromInternalEnergyFast(e, *T.at(p), Yi, &its);
    if (its >= 1000) flag_status(status, HTR_ERR_ITERATION_CAP);
    *T.at(p) = Tn;
    *P.at(p) = mix.PFromRhoAndT(rho, MixW, Tn);
    double *xp = X.at(p), *up = u.at(p);
#pragma unroll
    for (int i = 0; i < NS; i++) xp[i] = x[i];
#pragma unroll
    for (int i = 0; i < 3; i++) up[i] = vel[i];
  }
}

template <class Mix>
cudaError_t launch_primitive(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                             int *status, cudaStream_t s, unsigned skip_ghosts) {
  const CellRange R = cells(my);
  primitive_kernel<Mix><<<grid_for(R.n, 256), 256, 0, s>>>(
      R, fd<double>(v.Conserved), fd<double>(v.temperature), fd<double>(v.pressure),
      fd<double>(v.MolarFracs), fd<double>(v.velocity), status, ghost_skip(v, skip_ghosts), mix);
  return cudaGetLastError();
}

// --- spectral radius ------------------------------------------------------------
// Non-negative doubles order like their bit patterns, so an unsigned 64-bit
// atomicMax reduces them exactly (and independently of the order).
template <class Mix>
__global__ void spectral_kernel(CellRange R, Fd<double> dx, Fd<double> dy, Fd<double> dz,
                                Fd<double> T, Fd<double> Y, Fd<double> u, Fd<double> rho,
                                Fd<double> mu, Fd<double> lam, Fd<double> Di, Fd<double> SoS,
                                unsigned long long *out, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  double best = 0.0;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    const double a = ld(dx.at(p)), b = ld(dy.at(p)), c = ld(dz.at(p));
    const double s0 = ld(SoS.at(p));
    const double vx = fabs(ld(&u.at(p)[0])), vy = fabs(ld(&u.at(p)[1])), vz = fabs(ld(&u.at(p)[2]));
    double r = (vx + s0) * a;
    r = smax(r, (vy + s0) * b);
    r = smax(r, (vz + s0) * c);
    const double rh = ld(rho.at(p));
    const double nu = ld(mu.at(p)) / rh;
    double rv = nu * a * a;
    rv = smax(rv, nu * b * b);
    rv = smax(rv, nu * c * c);
    rv *= 4;
    r = smax(r, rv);
    double y[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) y[i] = ld(&Y.at(p)[i]);
    const double cp = mix.HeatCapacity(ld(T.at(p)), y);
    const double DifT = ld(lam.at(p)) / (cp * rh);
    double rt = DifT * a * a;
    rt = smax(rt, DifT * b * b);
    rt = smax(rt, DifT * c * c);
    rt *= 4;
    r = smax(r, rt);
    double rs = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
      const double d = ld(&Di.at(p)[i]);
      rs = smax(rs, d * a * a);
      rs = smax(rs, d * b * b);
      rs = smax(rs, d * c * c);
    }
    rs *= 4;
    r = smax(r, rs);
    best = smax(best, r);
  }
  // warp then block reduction, one atomic per block
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = smax(best, __shfl_xor_sync(0xffffffffu, best, o));
  __shared__ double wmax[32];
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x < 32) {
    double b = (threadIdx.x < (blockDim.x + 31) / 32) ? wmax[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = smax(b, __shfl_xor_sync(0xffffffffu, b, o));
    if (threadIdx.x == 0 && b > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(b));
  }
}

template <class Mix>
cudaError_t launch_spectral_radius(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                                   double *result, cudaStream_t s) {
  const CellRange R = cells(my);
  cudaError_t e = cudaMemsetAsync(result, 0, sizeof(double), s);
  if (e != cudaSuccess) return e;
  spectral_kernel<Mix><<<grid_for(R.n, 256), 256, 0, s>>>(
      R, fd<double>(v.dcsi_d), fd<double>(v.deta_d), fd<double>(v.dzet_d), fd<double>(v.temperature),
      fd<double>(v.MassFracs), fd<double>(v.velocity), fd<double>(v.rho), fd<double>(v.mu),
      fd<double>(v.lam), fd<double>(v.Di), fd<double>(v.SoS),
      reinterpret_cast<unsigned long long *>(result), mix);
  return cudaGetLastError();
}

// --- RK bookkeeping -----------------------------------------------------------------
__global__ void copy_conserved_kernel(CellRange R, Fd<double> C, Fd<double> Cold, int neq) {
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    const double *c = C.at(p);
    double *o = Cold.at(p);
    for (int i = 0; i < neq; i++) o[i] = c[i];
  }
}
__global__ void init_rhs_kernel(CellRange R, Fd<double> Ct, Fd<double> Ctold, int neq, int implicit) {
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    double *t = Ct.at(p);
    if (implicit) {
      const double *o = Ctold.at(p);
      for (int i = 0; i < neq; i++) t[i] = -o[i];
    } else {
      for (int i = 0; i < neq; i++) t[i] = 0.0;
    }
  }
}
__global__ void rk_update_kernel(CellRange R, Fd<double> C, Fd<double> Cold, Fd<double> Ct, int neq,
                                 double c1, double c2, double c3, double dt) {
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    double *c = C.at(p);
    const double *o = Cold.at(p), *t = Ct.at(p);
    for (int i = 0; i < neq; i++) c[i] = c1 * o[i] + c2 * c[i] + c3 * t[i] * dt;
  }
}

cudaError_t launch_copy_conserved(const htr_fluid_view &v, const htr_rect3 &my, int neq, cudaStream_t s) {
  const CellRange R = cells(my);
  copy_conserved_kernel<<<grid_for(R.n, 256), 256, 0, s>>>(R, fd<double>(v.Conserved),
                                                          fd<double>(v.Conserved_old), neq);
  return cudaGetLastError();
}
cudaError_t launch_init_rhs(const htr_fluid_view &v, const htr_rect3 &my, int neq, int implicit,
                            cudaStream_t s) {
  const CellRange R = cells(my);
  init_rhs_kernel<<<grid_for(R.n, 256), 256, 0, s>>>(R, fd<double>(v.Conserved_t),
                                                     fd<double>(v.Conserved_t_old), neq, implicit);
  return cudaGetLastError();
}
cudaError_t launch_rk_update(const htr_fluid_view &v, const htr_rect3 &my, int neq, int stage,
                             double dt, int implicit, cudaStream_t s) {
  const double RK[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
  if (stage < 1 || stage > 3) return cudaErrorInvalidValue;
  if (implicit) dt *= 0.5;
  const CellRange R = cells(my);
  rk_update_kernel<<<grid_for(R.n, 256), 256, 0, s>>>(R, fd<double>(v.Conserved), fd<double>(v.Conserved_old),
                                                      fd<double>(v.Conserved_t), neq, RK[stage - 1][0],
                                                      RK[stage - 1][1], RK[stage - 1][2], dt);
  return cudaGetLastError();
}

#define HTR_INST(MIX)                                                                                     \
  template cudaError_t launch_chem_sources<MIX>(const htr_fluid_view &, const htr_rect3 &, const MIX &,   \
                                                cudaStream_t);                                           \
  template cudaError_t launch_properties<MIX>(const htr_fluid_view &, const htr_rect3 &, const MIX &,     \
                                              cudaStream_t);                                             \
  template cudaError_t launch_conserved<MIX>(const htr_fluid_view &, const htr_rect3 &, const MIX &,      \
                                             cudaStream_t);                                              \
  template cudaError_t launch_primitive<MIX>(const htr_fluid_view &, const htr_rect3 &, const MIX &, int *, \
                                             cudaStream_t, unsigned);                                    \
  template cudaError_t launch_spectral_radius<MIX>(const htr_fluid_view &, const htr_rect3 &, const MIX &, \
                                                   double *, cudaStream_t);
HTR_INST(ConstPropDev)
HTR_INST(AirDev)
#undef HTR_INST

}  // namespace htr
