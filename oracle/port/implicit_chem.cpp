// CPU oracle port: implicit chemistry (UpdateChemistry).  TEST INFRASTRUCTURE ONLY.
//
// Restates ImplicitSolver (src/prometeo_chem.hpp:53-93) on top of the
// 4-stage Rosenbrock method with finite-difference Jacobian and Crout LU
// (src/Utils/math_utils.hpp:88-441), and the task body of
// src/prometeo_chem.cc:31-68.  Iteration caps report HTR_ERR_ITERATION_CAP
// through the status word instead of asserting.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "htr_rhs.h"
#include "mixtures.hpp"
#include "port.hpp"

using namespace oport;


namespace {

template <class Mix> struct Rosenbrock {
  static constexpr int N = Mix::NS + 4;
  const Mix &mix;
  const double *Ct_old;
  double &T;
  double Jac[N][N], LU[N][N], err[N], dx[N], xsav[N], dxsav[N];
  int ind[N];

  Rosenbrock(const Mix &m, const double *c, double &t) : mix(m), Ct_old(c), T(t) {}

  void rhs(double *r, const double *x) {
    constexpr int NS = Mix::NS;
    double rhoYi[NS], Yi[NS];
    for (int i = 0; i < NS; i++) rhoYi[i] = x[i];
    const double rho = mix.RhoFromRhoYi(rhoYi);
    mix.YiFromRhoYi(Yi, rho, rhoYi);
    mix.ClipYi(Yi);
    const double MixW = mix.MolarWeightFromYi(Yi);
    const double rhoInv = 1.0 / rho;
    double vel[3];
    for (int i = 0; i < 3; i++) vel[i] = x[i + NS] * rhoInv;
    double ke = 0.0;
    for (int i = 0; i < 3; i++) ke += vel[i] * vel[i];
    ke *= 0.5;
    const double e = x[NS + 3] * rhoInv - ke;
    T = mix.TFromInternalEnergy(e, T, Yi);
    const double P = mix.PFromRhoAndT(rho, MixW, T);
    double w[NS];
    mix.ProductionRates(w, rho, P, T, Yi);
    for (int i = 0; i < NS; i++) r[i] = w[i] + Ct_old[i];
    for (int i = NS; i < N; i++) r[i] = Ct_old[i];
  }

  void jacobian(double *x) {
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
      for (int i = 0; i < N; i++) Jac[i][j] = (fp[i] - fm[i]) / (hp + hm);
    }
  }

  void ludcmp() {
    double vv[N];
    int imax = 0;
    for (int i = 0; i < N; i++) {
      double big = 0.0;
      for (int j = 0; j < N; j++) big = std::max(std::fabs(LU[i][j]), big);
      vv[i] = 1.0 / big;
    }
    for (int j = 0; j < N; j++) {
      for (int i = 0; i < j; i++) {
        double sum = LU[i][j];
        for (int k = 0; k < i; k++) sum -= LU[i][k] * LU[k][j];
        LU[i][j] = sum;
      }
      double big = 0.0;
      for (int i = j; i < N; i++) {
        double sum = LU[i][j];
        for (int k = 0; k < j; k++) sum -= LU[i][k] * LU[k][j];
        LU[i][j] = sum;
        const double dum = vv[i] * std::fabs(sum);
        if (dum >= big) {
          big = dum;
          imax = i;
        }
      }
      if (j != imax) {
        for (int k = 0; k < N; k++) std::swap(LU[imax][k], LU[j][k]);
        vv[imax] = vv[j];
      }
      ind[j] = imax;
      if (LU[j][j] == 0.0) LU[j][j] = 1.0e-20;
      if (j != N - 1) {
        const double dum = 1.0 / (LU[j][j]);
        for (int i = j + 1; i < N; i++) LU[i][j] *= dum;
      }
    }
  }

  void lubksb(double *b) const {
    int ii = 0;
    for (int i = 0; i < N; i++) {
      const int ip = ind[i];
      double sum = b[ip];
      b[ip] = b[i];
      if (ii != 0)
        for (int j = ii - 1; j < i; j++) sum -= LU[i][j] * b[j];
      else if (sum != 0.0)
        ii = i + 1;
      b[i] = sum;
    }
    for (int i = N - 1; i > -1; i--) {
      double sum = b[i];
      for (int j = i + 1; j < N; j++) sum -= LU[i][j] * b[j];
      b[i] = sum / LU[i][i];
    }
  }

  double step(double *x, double dt, double t0) {
    const double GAM = 1.0 / 2.0, A21 = 2.0, A31 = 48.0 / 25.0, A32 = 6.0 / 25.0, C21 = -8.0,
                 C31 = 372.0 / 25.0, C32 = 12.0 / 5.0, C41 = -112.0 / 125.0, C42 = -54.0 / 125.0,
                 C43 = -2.0 / 5.0, B1 = 19.0 / 9.0, B2 = 1.0 / 2.0, B3 = 25.0 / 108.0,
                 B4 = 125.0 / 108.0, E1 = 17.0 / 54.0, E2 = 7.0 / 36.0, E3 = 0.0, E4 = 125.0 / 108.0,
                 C1X = 1.0 / 2.0, C2X = -3.0 / 2.0, C3X = 121.0 / 50.0, C4X = 29.0 / 250.0;
    double g1[N], g2[N], g3[N], g4[N];
    for (int i = 0; i < N; i++) {
      for (int j = 0; j < N; j++) LU[i][j] = -Jac[i][j];
      LU[i][i] += 1.0 / (GAM * dt);
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
    for (int i = 0; i < N; i++)
      g4[i] = dx[i] + dt * C4X * dx[i] + (C41 * g1[i] + C42 * g2[i] + C43 * g3[i]) / dt;
    lubksb(g4);
    for (int i = 0; i < N; i++) x[i] = xsav[i] + B1 * g1[i] + B2 * g2[i] + B3 * g3[i] + B4 * g4[i];
    for (int i = 0; i < N; i++) err[i] = E1 * g1[i] + E2 * g2[i] + E3 * g3[i] + E4 * g4[i];
    return t0 + dt;
  }

  int solve(double *x, double dtTry, double DelT) {
    const int MAXSTP = 100000, MAXITS = 100;
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
        for (int i = 0; i < N; i++) errmax = std::max(errmax, std::fabs(err[i]));
        errmax *= iTOL;
        if ((errmax < 1.0) || finish) {
          dtNext = (errmax > ERRCON) ? SAFETY * dt * std::pow(errmax, PGROW) : GROW * dt;
          ok = true;
          break;
        }
        dtNext = SAFETY * dt * std::pow(errmax, PSHRNK);
        dt = (dt > 0.0) ? std::max(dtNext, SHRNK * dt) : std::min(dtNext, SHRNK * dt);
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

inline double *at(const htr_field &f, long long x, long long y, long long z) {
  return reinterpret_cast<double *>(static_cast<char *>(f.base) + x * f.stride[0] +
                                    y * f.stride[1] + z * f.stride[2]);
}

template <class Mix>
int run(const Mix &mix, const htr_fluid_view *v, htr_rect3 r, double dt, int *status) {
  constexpr int N = Mix::NS + 4;
  int worst = HTR_OK;
#pragma omp parallel for collapse(3) reduction(max : worst)
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        double *ct = at(v->Conserved_t, i, j, k);
        double *old = at(v->Conserved_t_old, i, j, k);
        double *c = at(v->Conserved, i, j, k);
        double *T = at(v->temperature, i, j, k);
        for (int e = 0; e < N; e++) old[e] = ct[e];
        Rosenbrock<Mix> rb(mix, old, *T);
        const int st = rb.solve(c, dt, dt);
        worst = std::max(worst, st);
      }
  if (status) *status = worst;
  return HTR_OK;
}

}  // namespace

extern "C" int htr_UpdateChemistry(const htr_fluid_view *v, htr_rect3 r, double dt, htr_mixture_t mix,
                                   int *status, htr_stream_t) {
  if (v == nullptr || mix == nullptr) return HTR_ERR_ARGUMENT;
  if (mix->eos == HTR_EOS_AIRMIX) return run(mix->air, v, r, dt, status);
  if (mix->eos == HTR_EOS_CONSTPROPMIX) return run(mix->cp, v, r, dt, status);
  return HTR_ERR_UNSUPPORTED;
}
