// Per-cell kernels: chemistry sources, implicit chemistry, state refresh,
// spectral radius and the SSP-RK3 bookkeeping.
//
//   AddChemistrySources           src/prometeo_chem.cc:71-110
//   UpdateChemistry (Rosenbrock)  src/prometeo_chem.hpp:53-93, src/Utils/math_utils.hpp:88-441
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

static dim3 grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152LL * 32) b = 152LL * 32;
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
      mix.Transport(Tp, Pp, MixW, x, m, l, d);
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
                                 Fd<double> X, Fd<double> u, int *status,
                                 const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
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
    const double Tn = mix.TFromInternalEnergy(e, *T.at(p), Yi, &its);
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
                             int *status, cudaStream_t s) {
  const CellRange R = cells(my);
  primitive_kernel<Mix><<<grid_for(R.n, 256), 256, 0, s>>>(
      R, fd<double>(v.Conserved), fd<double>(v.temperature), fd<double>(v.pressure),
      fd<double>(v.MolarFracs), fd<double>(v.velocity), status, mix);
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

// --- implicit chemistry: Rosenbrock with finite-difference Jacobian ---------------
template <class Mix> struct Rosen {
  static constexpr int N = Mix::NS + 4;
  static constexpr int MAXSTP = 100000, MAXITS = 100;
  const Mix &mix;
  const double *Ct_old;  // Conserved_t_old of the cell (N values)
  double T;              // running temperature guess (shared by every rhs call)
  double Jac[N * N], LU[N * N];
  int ind[N];
  double err[N], dx[N], xsav[N], dxsav[N];

  // chem.hpp:66-88
  HTR_D void rhs(double *r, const double *x) {
    constexpr int NS = Mix::NS;
    double rhoYi[NS], Yi[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) rhoYi[i] = x[i];
    const double rho = mix.RhoFromRhoYi(rhoYi);
    mix.YiFromRhoYi(Yi, rho, rhoYi);
    mix.ClipYi(Yi);
    const double MixW = mix.MolarWeightFromYi(Yi);
    const double rhoInv = 1.0 / rho;
    double vel[3];
#pragma unroll
    for (int i = 0; i < 3; i++) vel[i] = x[i + NS] * rhoInv;
    const double e = x[NS + 3] * rhoInv - 0.5 * mod2(vel);
    T = mix.TFromInternalEnergy(e, T, Yi, nullptr);
    const double P = mix.PFromRhoAndT(rho, MixW, T);
    double w[NS];
    mix.ProductionRates(w, rho, P, T, Yi);
#pragma unroll
    for (int i = 0; i < NS; i++) r[i] = w[i] + Ct_old[i];
#pragma unroll
    for (int i = NS; i < N; i++) r[i] = Ct_old[i];
  }
  // math_utils.hpp:248-272
  HTR_D void jacobian(double *x) {
    double tmp[N], fp[N], fm[N];
    for (int i = 0; i < N; i++) tmp[i] = x[i];
    for (int j = 0; j < N; j++) {
      const double h = x[j] * 1.0e-6 + 1.0e-14;
      x[j] = tmp[j] + h;
      const double hp = x[j] - tmp[j];
      rhs(fp, x);
      x[j] = tmp[j] - h;
      const double hm = tmp[j] - x[j];
      rhs(fm, x);
      x[j] = tmp[j];
      for (int i = 0; i < N; i++) Jac[i * N + j] = (fp[i] - fm[i]) / (hp + hm);
    }
  }
  // Crout LU with implicit partial pivoting (math_utils.hpp:105-156)
  HTR_D void ludcmp() {
    double vv[N];
    int imax = 0;
    for (int i = 0; i < N; i++) {
      double big = 0.0;
      for (int j = 0; j < N; j++) big = smax(fabs(LU[i * N + j]), big);
      vv[i] = 1.0 / big;
    }
    for (int j = 0; j < N; j++) {
      for (int i = 0; i < j; i++) {
        double sum = LU[i * N + j];
        for (int k = 0; k < i; k++) sum -= LU[i * N + k] * LU[k * N + j];
        LU[i * N + j] = sum;
      }
      double big = 0.0;
      for (int i = j; i < N; i++) {
        double sum = LU[i * N + j];
        for (int k = 0; k < j; k++) sum -= LU[i * N + k] * LU[k * N + j];
        LU[i * N + j] = sum;
        const double dum = vv[i] * fabs(sum);
        if (dum >= big) {
          big = dum;
          imax = i;
        }
      }
      if (j != imax) {
        for (int k = 0; k < N; k++) {
          const double dum = LU[imax * N + k];
          LU[imax * N + k] = LU[j * N + k];
          LU[j * N + k] = dum;
        }
        vv[imax] = vv[j];
      }
      ind[j] = imax;
      if (LU[j * N + j] == 0.0) LU[j * N + j] = 1.0e-20;
      if (j != N - 1) {
        const double dum = 1.0 / (LU[j * N + j]);
        for (int i = j + 1; i < N; i++) LU[i * N + j] *= dum;
      }
    }
  }
  HTR_D void lubksb(double *b) const {  // math_utils.hpp:158-180
    int ii = 0;
    for (int i = 0; i < N; i++) {
      const int ip = ind[i];
      double sum = b[ip];
      b[ip] = b[i];
      if (ii != 0)
        for (int j = ii - 1; j < i; j++) sum -= LU[i * N + j] * b[j];
      else if (sum != 0.0)
        ii = i + 1;
      b[i] = sum;
    }
    for (int i = N - 1; i > -1; i--) {
      double sum = b[i];
      for (int j = i + 1; j < N; j++) sum -= LU[i * N + j] * b[j];
      b[i] = sum / LU[i * N + i];
    }
  }
  // math_utils.hpp:275-338 (4-stage Rosenbrock, Shampine coefficients)
  HTR_D double step(double *x, double dt, double t0) {
    const double GAM = 1.0 / 2.0, A21 = 2.0, A31 = 48.0 / 25.0, A32 = 6.0 / 25.0, C21 = -8.0,
                 C31 = 372.0 / 25.0, C32 = 12.0 / 5.0, C41 = -112.0 / 125.0, C42 = -54.0 / 125.0,
                 C43 = -2.0 / 5.0, B1 = 19.0 / 9.0, B2 = 1.0 / 2.0, B3 = 25.0 / 108.0,
                 B4 = 125.0 / 108.0, E1 = 17.0 / 54.0, E2 = 7.0 / 36.0, E3 = 0.0, E4 = 125.0 / 108.0,
                 C1X = 1.0 / 2.0, C2X = -3.0 / 2.0, C3X = 121.0 / 50.0, C4X = 29.0 / 250.0;
    double g1[N], g2[N], g3[N], g4[N];
    for (int i = 0; i < N; i++) {
      for (int j = 0; j < N; j++) LU[i * N + j] = -Jac[i * N + j];
      LU[i * N + i] += 1.0 / (GAM * dt);
    }
    ludcmp();
    for (int i = 0; i < N; i++) g1[i] = dxsav[i] + dt * C1X * dx[i];
    lubksb(g1);
    for (int i = 0; i < N; i++) x[i] = xsav[i] + A21 * g1[i];
    rhs(dx, x);
    for (int i = 0; i < N; i++) g2[i] = dx[i] + dt * C2X * dx[i] + C21 * g1[i] / dt;
    lubksb(g2);
    for (int i = 0; i < N; i++) x[i] = xsav[i] + A31 * g1[i] + A32 * g2[i];
    rhs(dx, x);
    for (int i = 0; i < N; i++) g3[i] = dx[i] + dt * C3X * dx[i] + (C31 * g1[i] + C32 * g2[i]) / dt;
    lubksb(g3);
    for (int i = 0; i < N; i++) g4[i] = dx[i] + dt * C4X * dx[i] + (C41 * g1[i] + C42 * g2[i] + C43 * g3[i]) / dt;
    lubksb(g4);
    for (int i = 0; i < N; i++) x[i] = xsav[i] + B1 * g1[i] + B2 * g2[i] + B3 * g3[i] + B4 * g4[i];
    for (int i = 0; i < N; i++) err[i] = E1 * g1[i] + E2 * g2[i] + E3 * g3[i] + E4 * g4[i];
    return t0 + dt;
  }
  // returns 0 ok, HTR_ERR_ITERATION_CAP if a cap was hit (math_utils.hpp:208-244, 340-400)
  HTR_D int solve(double *x, double dtTry, double DelT) {
    const double iTOL = 1.0 / 1e-10, SAFETY = 0.9, GROW = 1.5, PGROW = -0.25, SHRNK = 0.5,
                 PSHRNK = -1.0 / 3.0, ERRCON = 0.1296;
    bool finish = false;
    double time = 0.0, dt = dtTry;
    for (int s = 0; s < MAXSTP; s++) {
      const double t0 = time;
      double dtNext = dt;
      jacobian(x);
      rhs(dx, x);
      for (int i = 0; i < N; i++) {
        xsav[i] = x[i];
        dxsav[i] = dx[i];
      }
      bool ok = false;
      for (int jtry = 0; jtry < MAXITS; jtry++) {
        time = step(x, dt, t0);
        double errmax = 0.0;
        for (int i = 0; i < N; i++) errmax = smax(errmax, fabs(err[i]));
        errmax *= iTOL;
        if ((errmax < 1.0) || finish) {
          dtNext = (errmax > ERRCON) ? SAFETY * dt * pow(errmax, PGROW) : GROW * dt;
          ok = true;
          break;
        }
        dtNext = SAFETY * dt * pow(errmax, PSHRNK);
        dt = (dt > 0.0) ? smax(dtNext, SHRNK * dt) : smin(dtNext, SHRNK * dt);
      }
      if (!ok) return HTR_ERR_ITERATION_CAP;
      const double Remainder = DelT - time;
      if (finish || (Remainder < 1e-12 * DelT)) return HTR_OK;
      if (dtNext * 1.5 > Remainder) {
        dt = Remainder;
        finish = true;
      } else {
        dt = dtNext;
        finish = false;
      }
    }
    return HTR_ERR_ITERATION_CAP;
  }
};

template <class Mix>
__global__ void update_chemistry_kernel(CellRange R, Fd<double> Ct, Fd<double> C, Fd<double> Ctold,
                                        Fd<double> T, double dt, int *status,
                                        const __grid_constant__ Mix mix) {
  constexpr int N = Mix::NS + 4;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    double old[N], x[N];
    double *co = Ctold.at(p);
    double *c = C.at(p);
    for (int i = 0; i < N; i++) {
      old[i] = ld(&Ct.at(p)[i]);
      co[i] = old[i];
      x[i] = c[i];
    }
    Rosen<Mix> rb{mix, old};
    rb.T = *T.at(p);
    const int st = rb.solve(x, dt, dt);
    if (st != HTR_OK) flag_status(status, st);
    for (int i = 0; i < N; i++) c[i] = x[i];
    *T.at(p) = rb.T;
  }
}

template <class Mix>
cudaError_t launch_update_chemistry(const htr_fluid_view &v, const htr_rect3 &my, double dt,
                                    const Mix &mix, int *status, cudaStream_t s) {
  const CellRange R = cells(my);
  update_chemistry_kernel<Mix><<<grid_for(R.n, 64), 64, 0, s>>>(
      R, fd<double>(v.Conserved_t), fd<double>(v.Conserved), fd<double>(v.Conserved_t_old),
      fd<double>(v.temperature), dt, status, mix);
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
                                             cudaStream_t);                                              \
  template cudaError_t launch_spectral_radius<MIX>(const htr_fluid_view &, const htr_rect3 &, const MIX &, \
                                                   double *, cudaStream_t);                              \
  template cudaError_t launch_update_chemistry<MIX>(const htr_fluid_view &, const htr_rect3 &, double,    \
                                                    const MIX &, int *, cudaStream_t);
HTR_INST(ConstPropDev)
HTR_INST(AirDev)
#undef HTR_INST

}  // namespace htr
