// Implicit chemistry: UpdateChemistryTask (src/prometeo_chem.cc:31-68,
// src/prometeo_chem.hpp:53-93) with the reference's Rosenbrock solver and LU
// decomposition (src/Utils/math_utils.hpp:88-441), one thread per cell.
//
// The solver's adaptive step control turns any difference of rounding in the
// right-hand side it integrates into a different sequence of steps, whose
// results then differ at the level of its own error tolerance (1e-10).  This
// translation unit is therefore compiled without FMA contraction and
// evaluates the right-hand side in the reference's operation order
// (AirDev::ProductionRatesRef), so that it follows the reference's sequence of
// steps unless the math library's exp / log / pow round differently.
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
// limit): a grid capped at 152 x 32 blocks made the implicit step of a 96^3
// air box 10 % slower (257 / 240 ms against 233 / 216 ms on two states).
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
    mix.ProductionRatesRef(w, rho, P, T, Yi);
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
                                        Fd<double> T, double dt, const double *dt_cell, int *status,
                                        const GhostSkip G, const __grid_constant__ Mix mix) {
  constexpr int N = Mix::NS + 4;
  HTR_FOR_CELLS(R, idx) {
    long long p[3];
    R.point(idx, p);
    if (G.active && G.at(p)) continue;
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
    // per-cell step sizes are indexed densely over the range (x fastest)
    const double h = dt_cell ? dt_cell[idx] : dt;
    const int st = rb.solve(x, h, h);
    if (st != HTR_OK) flag_status(status, st);
    for (int i = 0; i < N; i++) c[i] = x[i];
    *T.at(p) = rb.T;
  }
}

template <class Mix>
cudaError_t launch_update_chemistry(const htr_fluid_view &v, const htr_rect3 &my, double dt,
                                    const Mix &mix, int *status, cudaStream_t s, unsigned skip_ghosts,
                                    const double *dt_cell) {
  const CellRange R = cells(my);
  update_chemistry_kernel<Mix><<<grid_for(R.n, 64), 64, 0, s>>>(
      R, fd<double>(v.Conserved_t), fd<double>(v.Conserved), fd<double>(v.Conserved_t_old),
      fd<double>(v.temperature), dt, dt_cell, status, ghost_skip(v, skip_ghosts), mix);
  return cudaGetLastError();
}

template cudaError_t launch_update_chemistry<ConstPropDev>(const htr_fluid_view &, const htr_rect3 &, double,
                                                          const ConstPropDev &, int *, cudaStream_t, unsigned,
                                                          const double *);
template cudaError_t launch_update_chemistry<AirDev>(const htr_fluid_view &, const htr_rect3 &, double,
                                                    const AirDev &, int *, cudaStream_t, unsigned, const double *);

}  // namespace htr
