// CPU oracle port: the RHS-path tasks over the htr_rhs.h field view.
// TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).
//
// A from-scratch restatement of the reference's CPU task bodies:
//   Euler fluxes     src/prometeo_rhs.inl:37-1052, src/prometeo_rhs.cc:35-406
//   diffusion flux   src/prometeo_rhs.inl:1054-1282, src/prometeo_rhs.cc:408-527
//   shock sensors    src/prometeo_sensor.inl:47-76, src/prometeo_sensor.cc:33-128
//   chemistry        src/prometeo_chem.hpp:53-93, src/prometeo_chem.cc:31-110
//   state refresh    src/prometeo_variables.hpp:52-210
//   spectral radius  src/prometeo_cfl.hpp:55-190
// Loops over pencils are parallel (OpenMP) like the reference's CPU
// variants; each pencil is swept sequentially with running face fluxes.
#include <omp.h>

#include <cstdint>
#include <cstring>
#include <string>

#include "htr_rhs.h"
#include "mixtures.hpp"
#include "port.hpp"
#include "stencils.hpp"

using namespace oport;


namespace {

thread_local std::string g_err;

template <class T> struct Fld {
  char *b;
  int64_t s[3];
  explicit Fld(const htr_field &f) : b(static_cast<char *>(f.base)) {
    s[0] = f.stride[0];
    s[1] = f.stride[1];
    s[2] = f.stride[2];
  }
  T *at(const long long *p) const { return reinterpret_cast<T *>(b + p[0] * s[0] + p[1] * s[1] + p[2] * s[2]); }
  T &operator()(const long long *p) const { return *at(p); }
};

struct Box {
  long long lo[3], hi[3];
  long long size(int d) const { return hi[d] - lo[d] + 1; }
};
inline Box box(const htr_rect3 &r) {
  Box b;
  for (int i = 0; i < 3; i++) {
    b.lo[i] = r.lo[i];
    b.hi[i] = r.hi[i];
  }
  return b;
}

inline void shiftp(long long *q, const long long *p, int d, const Box &fb, int off) {
  q[0] = p[0];
  q[1] = p[1];
  q[2] = p[2];
  q[d] = wrap_plus(p[d], fb.lo[d], fb.size(d), off);
}
inline void shiftm(long long *q, const long long *p, int d, const Box &fb, int off) {
  q[0] = p[0];
  q[1] = p[1];
  q[2] = p[2];
  q[d] = wrap_minus(p[d], fb.lo[d], fb.size(d), off);
}

template <class F> void for_pencils(const Box &r, int d, F &&f) {
  const int a = (d == 0) ? 1 : 0, b = (d == 2) ? 1 : 2;
  const long long na = r.size(a), nb = r.size(b);
#pragma omp parallel for collapse(2) schedule(static)
  for (long long jb = 0; jb < nb; jb++)
    for (long long ja = 0; ja < na; ja++) {
      long long p[3];
      p[d] = r.lo[d];
      p[a] = r.lo[a] + ja;
      p[b] = r.lo[b] + jb;
      f(p);
    }
}

template <class F> void for_cells(const Box &r, F &&f) {
#pragma omp parallel for collapse(3) schedule(static)
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        const long long p[3] = {i, j, k};
        f(p);
      }
}

inline const htr_field &ntype_of(const htr_fluid_view *v, int d) {
  return d == 0 ? v->nType_x : (d == 1 ? v->nType_y : v->nType_z);
}
inline const htr_field &me_of(const htr_fluid_view *v, int d) {
  return d == 0 ? v->dcsi_e : (d == 1 ? v->deta_e : v->dzet_e);
}
inline const htr_field &md_of(const htr_fluid_view *v, int d) {
  return d == 0 ? v->dcsi_d : (d == 1 ? v->deta_d : v->dzet_d);
}
inline const htr_field &ms_of(const htr_fluid_view *v, int d) {
  return d == 0 ? v->dcsi_s : (d == 1 ? v->deta_s : v->dzet_s);
}
inline const htr_field &sensor_of(const htr_fluid_view *v, int d) {
  return d == 0 ? v->shockSensorX : (d == 1 ? v->shockSensorY : v->shockSensorZ);
}

inline double mod2(const double *v) {
  double r = 0.0;
  for (int i = 0; i < 3; i++) r += v[i] * v[i];
  return r;
}

// ===========================================================================
// Euler fluxes
// ===========================================================================
template <class Mix> struct Euler {
  static constexpr int NS = Mix::NS, NE = NS + 4, iU = NS, iE = NS + 3;
  const Mix &mix;
  int d, t1, t2;
  Box fb;
  Fld<double> C, Cold, SoS, rho, Y, u, P, me, Ct;
  Fld<int> nt;
  Fld<bool> sen;
  double rk0, rk1, dt;

  Euler(const Mix &m, const htr_fluid_view *v, int dir, const Box &b, const double *rk, double delta)
      : mix(m), d(dir), t1(dir == 0 ? 1 : 0), t2(dir == 2 ? 1 : 2), fb(b), C(v->Conserved),
        Cold(v->Conserved_old), SoS(v->SoS), rho(v->rho), Y(v->MassFracs), u(v->velocity),
        P(v->pressure), me(me_of(v, dir)), Ct(v->Conserved_t), nt(ntype_of(v, dir)),
        sen(sensor_of(v, dir)), rk0(rk ? rk[0] : 0.0), rk1(rk ? rk[1] : 1.0), dt(delta) {}

  struct Roe {
    double rho, Yi[NS], vel[3], H, e, dpde, dpdrhoi[NS], a2, a;
  };

  // rhs.inl:40-75: sums over the pairs (p, p+l+1), l < KennedyNSum.
  void kg_sums(double *S, const long long *p, int t) const {
    const double H = (C.at(p)[iE] + P(p)) / rho(p);
    for (int l = 0; l < kNodes[t].kgNSum; l++) {
      long long pp[3];
      shiftp(pp, p, d, fb, l + 1);
      const int o = l * (NE + 1);
      const double rhom = rho(p) + rho(pp);
      const double vm = -(u.at(p)[d] + u.at(pp)[d]);
      for (int i = 0; i < NS; i++) S[o + i] = rhom * vm * (Y.at(p)[i] + Y.at(pp)[i]);
      for (int i = 0; i < 3; i++) S[o + iU + i] = rhom * vm * (u.at(p)[i] + u.at(pp)[i]);
      S[o + iE] = rhom * vm * (H + (C.at(pp)[iE] + P(pp)) / rho(pp));
      S[o + NE] = (P(p) + P(pp));
    }
  }

  // rhs.inl:77-135
  void kg_flux(double *F, const double *S, const long long *p, int t) const {
    if (t == L_S || t == Rm1_S) {
      long long q[3];
      if (t == L_S) {
        q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
      } else {
        shiftp(q, p, d, fb, kNodes[t].off[2]);
      }
      for (int i = 0; i < NE; i++) F[i] = -(C.at(q)[i] * u.at(q)[d]);
      F[iU + d] -= P(q);
      F[iE] -= P(q) * u.at(q)[d];
      return;
    }
    double f[NE + 1], acc[NE + 1];
    for (int i = 0; i < NE + 1; i++) f[i] = 0.0;
    for (int l = 0; l < kNodes[t].kgOrder; l++) {
      for (int i = 0; i < NE + 1; i++) acc[i] = 0.0;
      for (int m = 0; m < l + 1; m++) {
        const int o = (NE + 1) * ((5 - m) * m / 2 + l);
        for (int i = 0; i < NE + 1; i++) acc[i] += S[o + i];
      }
      for (int i = 0; i < NE + 1; i++) f[i] += kNodes[t].kg[l] * acc[i];
    }
    for (int i = 0; i < NE; i++) F[i] = 0.25 * f[i];
    F[iU + d] -= f[NE];
  }

  // rhs.inl:198-279
  void roe(Roe &R, const long long *pL, const long long *pR) const {
    const double *CL = C.at(pL), *CR = C.at(pR), *YL = Y.at(pL), *YR = Y.at(pR);
    const double *uL = u.at(pL), *uR = u.at(pR);
    const double rhoL = rho(pL), rhoR = rho(pR), PL = P(pL), PR = P(pR);
    const double eL = CL[iE] / rhoL - 0.5 * mod2(uL);
    const double eR = CR[iE] / rhoR - 0.5 * mod2(uR);
    const double HL = (CL[iE] + PL) / rhoL;
    const double HR = (CR[iE] + PR) / rhoR;
    const double fL = std::sqrt(rhoL) / (std::sqrt(rhoL) + std::sqrt(rhoR));
    const double fR = std::sqrt(rhoR) / (std::sqrt(rhoL) + std::sqrt(rhoR));
    R.rho = std::sqrt(rhoL * rhoR);
    for (int i = 0; i < NS; i++) R.Yi[i] = YL[i] * fL + YR[i] * fR;
    for (int i = 0; i < 3; i++) R.vel[i] = uL[i] * fL + uR[i] * fR;
    R.H = HL * fL + HR * fR;
    R.e = eL * fL + eR * fR;
    const double PovRho = R.H - R.e - 0.5 * mod2(R.vel);
    const double MixW = mix.MolarWeightFromYi(R.Yi);
    const double Teos = mix.TFromRhoAndP(R.rho, MixW, PovRho * R.rho);
    const double T = mix.TFromInternalEnergy(R.e, Teos, R.Yi);
    const double gamma = mix.Gamma(T, MixW, R.Yi);
    R.dpde = mix.dpde(R.rho, gamma);
    mix.dpdrhoi(R.dpdrhoi, gamma, T, R.Yi);
    const double dp = PR - PL;
    const double de = eR - eL;
    double drhoi[NS];
    for (int i = 0; i < NS; i++) drhoi[i] = rhoR * YR[i] - rhoL * YL[i];
    double dpError = dp - de * R.dpde;
    double fact = de * R.dpde;
    fact *= fact;
    for (int i = 0; i < NS; i++) {
      const double dpi = drhoi[i] * R.dpdrhoi[i];
      dpError -= dpi;
      fact += dpi * dpi;
    }
    fact = dpError / std::max(fact, 1e-6);
    for (int i = 0; i < NS; i++) R.dpdrhoi[i] = R.dpdrhoi[i] * (1.0 + R.dpdrhoi[i] * drhoi[i] * fact);
    R.dpde = R.dpde * (1.0 + R.dpde * de * fact);
    R.a2 = PovRho / R.rho * R.dpde;
    for (int i = 0; i < NS; i++) R.a2 += R.Yi[i] * R.dpdrhoi[i];
    R.a = std::sqrt(R.a2);
  }

  // rhs.inl:433-505: left eigenvectors applied to q
  void to_char(double *r, const double *q, const Roe &R) const {
    const double ia = 1.0 / R.a;
    const double ia2 = 1.0 / R.a2;
    const double Coeff = (R.e - 0.5 * mod2(R.vel)) * R.dpde / R.rho;
    double sum1 = 0.0;
    for (int i = 0; i < NS; i++) sum1 += (Coeff - R.dpdrhoi[i]) * ia2 * q[i];
    double sq = 0.0;
    for (int i = 0; i < NS; i++) sq += q[i];
    const double dd = R.dpde / (R.rho * R.a2);
    double c[3];
    for (int i = 0; i < 3; i++) c[i] = R.vel[i] * dd;
    r[0] = sq * R.vel[d] * ia - sum1;
    r[0] -= (c[d] + ia) * q[NS + d];
    r[0] -= c[t1] * q[NS + t1];
    r[0] -= c[t2] * q[NS + t2];
    r[0] += dd * q[NS + 3];
    r[0] *= 0.5;
    for (int i = 1; i < NS + 1; i++) {
      r[i] = R.Yi[i - 1] * sum1;
      r[i] += q[i - 1];
      for (int j = 0; j < 3; j++) r[i] += R.Yi[i - 1] * c[j] * q[NS + j];
      r[i] += -R.Yi[i - 1] * dd * q[NS + 3];
    }
    r[NS + 1] = -R.vel[t1] * sq;
    r[NS + 1] += q[NS + t1];
    r[NS + 2] = -R.vel[t2] * sq;
    r[NS + 2] += q[NS + t2];
    r[NS + 3] = -sq * R.vel[d] * ia - sum1;
    r[NS + 3] -= (c[d] - ia) * q[NS + d];
    r[NS + 3] -= c[t1] * q[NS + t1];
    r[NS + 3] -= c[t2] * q[NS + t2];
    r[NS + 3] += dd * q[NS + 3];
    r[NS + 3] *= 0.5;
  }

  // rhs.inl:507-572: right eigenvectors applied to q
  void from_char(double *r, const double *q, const Roe &R) const {
    for (int i = 0; i < NE; i++) r[i] = 0.0;
    double sq = 0.0;
    for (int i = 0; i < NS; i++) sq += q[i + 1];
    for (int i = 0; i < NS; i++) {
      r[i] += R.Yi[i] * q[0];
      r[i] += q[i + 1];
      r[i] += R.Yi[i] * q[NS + 3];
    }
    r[NS + d] += (R.vel[d] - R.a) * q[0];
    r[NS + d] += R.vel[d] * sq;
    r[NS + d] += (R.vel[d] + R.a) * q[NS + 3];
    r[NS + t1] += R.vel[t1] * q[0];
    r[NS + t1] += R.vel[t1] * sq;
    r[NS + t1] += q[NS + 1];
    r[NS + t1] += R.vel[t1] * q[NS + 3];
    r[NS + t2] += R.vel[t2] * q[0];
    r[NS + t2] += R.vel[t2] * sq;
    r[NS + t2] += q[NS + 2];
    r[NS + t2] += R.vel[t2] * q[NS + 3];
    r[NS + 3] += (R.H - R.vel[d] * R.a) * q[0];
    const double dedp = 1.0 / R.dpde;
    const double E = R.e + 0.5 * mod2(R.vel);
    for (int i = 0; i < NS; i++) r[NS + 3] += (E - R.rho * R.dpdrhoi[i] * dedp) * q[i + 1];
    r[NS + 3] += R.vel[t1] * q[NS + 1];
    r[NS + 3] += R.vel[t2] * q[NS + 2];
    r[NS + 3] += (R.H + R.vel[d] * R.a) * q[NS + 3];
  }

  // rhs.inl:584-620: local Lax-Friedrichs split in characteristic space
  void pm_flux(double *Fp, double *Fm, const Roe &R, const long long *q, double L1, double L,
               double LN) const {
    const double *Cq = C.at(q);
    const double un = u.at(q)[d], pq = P(q);
    double F[NE];
    for (int i = 0; i < NE; i++) F[i] = Cq[i] * un;
    F[iU + d] += pq;
    F[iE] += pq * un;
    double Qc[NE], Fc[NE];
    to_char(Qc, Cq, R);
    to_char(Fc, F, R);
    Fp[0] = Fc[0] + L1 * Qc[0];
    for (int i = 1; i < NE - 1; i++) Fp[i] = Fc[i] + L * Qc[i];
    Fp[NE - 1] = Fc[NE - 1] + LN * Qc[NE - 1];
    Fm[0] = Fc[0] - L1 * Qc[0];
    for (int i = 1; i < NE - 1; i++) Fm[i] = Fc[i] - L * Qc[i];
    Fm[NE - 1] = Fc[NE - 1] - LN * Qc[NE - 1];
  }

  // rhs.inl:622-759: characteristic TENO flux at face p+1/2 (+ positivity limiter)
  void teno_flux(double *Flux, TenoKind kind, const long long *p, int t, double lim_f) const {
    long long pts[6][3];
    shiftm(pts[0], p, d, fb, kNodes[t].off[0]);
    shiftm(pts[1], p, d, fb, kNodes[t].off[1]);
    pts[2][0] = p[0]; pts[2][1] = p[1]; pts[2][2] = p[2];
    shiftp(pts[3], p, d, fb, kNodes[t].off[2]);
    shiftp(pts[4], p, d, fb, kNodes[t].off[3]);
    shiftp(pts[5], p, d, fb, kNodes[t].off[4]);
    double e1[6], e0[6], eN[6];
    for (int k = 0; k < 6; k++) {
      const double un = u.at(pts[k])[d], a = SoS(pts[k]);
      e1[k] = std::fabs(un - a);
      e0[k] = std::fabs(un);
      eN[k] = std::fabs(un + a);
    }
    double L1 = e1[0], L = e0[0], LN = eN[0];
    for (int k = 1; k < 6; k++) {
      L1 = std::max(L1, e1[k]);
      L = std::max(L, e0[k]);
      LN = std::max(LN, eN[k]);
    }
    Roe R;
    roe(R, pts[2], pts[3]);
    double Fp[6][NE], Fm[6][NE];
    for (int k = 0; k < 6; k++) pm_flux(Fp[k], Fm[k], R, pts[k], L1, L, LN);
    double F[NE];
    for (int i = 0; i < NE; i++) {
      const double fplus = teno(kind, false, Fp[0][i], Fp[1][i], Fp[2][i], Fp[3][i], Fp[4][i], Fp[5][i], t);
      const double fminus = teno(kind, true, Fm[0][i], Fm[1][i], Fm[2][i], Fm[3][i], Fm[4][i], Fm[5][i], t);
      F[i] = -0.5 * (fplus + fminus);
    }
    from_char(Flux, F, R);
    if (NS > 1) {
      const long long *pc = pts[2], *pn = pts[3];
      const double eps_l = -1e-8;
      bool limit = false;
      for (int i = 0; i < NS; i++) {
        const double dr = lim_f * Flux[i];
        if (((rk0 * Cold.at(pc)[i] + rk1 * C.at(pc)[i] + dr) < eps_l) ||
            ((rk0 * Cold.at(pn)[i] + rk1 * C.at(pn)[i] - dr) < eps_l))
          limit = true;
      }
      if (limit) {
        const double eps = 1e-60;
        double theta = 1.0;
        double Flo_c[NE], Flo[NE];
        for (int i = 0; i < NE; i++) Flo_c[i] = (Fp[2][i] + Fm[3][i]) * -0.5;
        from_char(Flo, Flo_c, R);
        for (int i = 0; i < NS; i++) {
          const double dr = lim_f * Flux[i];
          const double dr_lo = lim_f * Flo[i];
          double th_p = 1.0;
          const double rp = rk0 * Cold.at(pc)[i] + rk1 * C.at(pc)[i];
          const double hp = rp + dr;
          if (hp < eps) {
            const double lo = rp + dr_lo;
            th_p = (std::fabs(hp - lo) > eps) ? std::max(0.0, (eps - lo) / (hp - lo)) : 1.0;
          }
          double th_n = 1.0;
          const double rn = rk0 * Cold.at(pn)[i] + rk1 * C.at(pn)[i];
          const double hn = rn - dr;
          if (hn < eps) {
            const double lo = rn - dr_lo;
            th_n = (std::fabs(hn - lo) > eps) ? std::max(0.0, (eps - lo) / (hn - lo)) : 1.0;
          }
          theta = std::min(std::min(th_p, th_n), theta);
        }
        for (int i = 0; i < NE; i++) Flux[i] = Flux[i] * theta + Flo[i] * (1 - theta);
      }
    }
  }

  void accumulate(const long long *p, const double *Fp, const double *Fm) const {
    double *ct = Ct.at(p);
    const double m = me(p);
    for (int i = 0; i < NE; i++) ct[i] += m * (Fp[i] - Fm[i]);
  }

  // rhs.inl:765-889 (hybrid), :979-1052 (skew-symmetric = hybrid with KG everywhere)
  void sweep_kg(const long long *p0, long long n, bool hybrid) const {
    double S[6 * (NE + 1)];
    double Fm[NE], Fp[NE];
    {
      long long p[3], pM1[3], pM2[3];
      shiftm(p, p0, d, fb, kNodes[nt(p0)].off[1]);
      const int t = nt(p);
      shiftm(pM1, p, d, fb, kNodes[t].off[1]);
      shiftm(pM2, p, d, fb, kNodes[t].off[0]);
      kg_sums(&S[3 * (NE + 1)], pM2, t);
      kg_sums(&S[2 * (NE + 1)], pM1, t);
      kg_sums(&S[0], p, t);
      if (!hybrid || (sen(pM1) && sen(p) && sen(p0)))
        kg_flux(Fm, S, p, t);
      else
        teno_flux(Fm, kTENO, p, t, dt * (me(p) + me(p0)));
    }
    for (long long i = 0; i < n; i++) {
      long long p[3] = {p0[0], p0[1], p0[2]};
      p[d] += i;
      const int t = nt(p);
      long long pM1[3], pP1[3];
      shiftm(pM1, p, d, fb, kNodes[t].off[1]);
      shiftp(pP1, p, d, fb, kNodes[t].off[2]);
      for (int l = 0; l < NE + 1; l++) S[5 * (NE + 1) + l] = S[4 * (NE + 1) + l];
      for (int l = 0; l < NE + 1; l++) S[4 * (NE + 1) + l] = S[2 * (NE + 1) + l];
      for (int l = 0; l < NE + 1; l++) S[3 * (NE + 1) + l] = S[1 * (NE + 1) + l];
      kg_sums(&S[0], p, t);
      if (!hybrid || (sen(pM1) && sen(p) && sen(pP1)))
        kg_flux(Fp, S, p, t);
      else
        teno_flux(Fp, kTENO, p, t, dt * (me(p) + me(pP1)));
      accumulate(p, Fp, Fm);
      for (int l = 0; l < NE; l++) Fm[l] = Fp[l];
    }
  }

  // rhs.inl:895-973 (TENO / TENO-A / TENO-LAD everywhere)
  void sweep_teno(const long long *p0, long long n, TenoKind kind) const {
    double Fm[NE], Fp[NE];
    {
      long long pm1[3];
      shiftm(pm1, p0, d, fb, kNodes[nt(p0)].off[1]);
      teno_flux(Fm, kind, pm1, nt(pm1), dt * (me(pm1) + me(p0)));
    }
    for (long long i = 0; i < n; i++) {
      long long p[3] = {p0[0], p0[1], p0[2]};
      p[d] += i;
      const int t = nt(p);
      long long pP1[3];
      shiftp(pP1, p, d, fb, kNodes[t].off[2]);
      teno_flux(Fp, kind, p, t, dt * (me(p) + me(pP1)));
      accumulate(p, Fp, Fm);
      for (int l = 0; l < NE; l++) Fm[l] = Fp[l];
    }
  }
};

// ===========================================================================
// Diffusion flux (rhs.inl:1054-1282)
// ===========================================================================
template <class Mix> struct Diffusion {
  static constexpr int NS = Mix::NS, NE = NS + 4, iU = NS, iE = NS + 3;
  const Mix &mix;
  int d, t1, t2;
  Box fb;
  Fld<double> C, T, X, rho, mu, lam, Di, u, ms, md, md1, md2, Ct;
  Fld<int> nt, nt1, nt2;

  Diffusion(const Mix &m, const htr_fluid_view *v, int dir, const Box &b)
      : mix(m), d(dir), t1(dir == 0 ? 1 : 0), t2(dir == 2 ? 1 : 2), fb(b), C(v->Conserved),
        T(v->temperature), X(v->MolarFracs), rho(v->rho), mu(v->mu), lam(v->lam), Di(v->Di),
        u(v->velocity), ms(ms_of(v, dir)), md(md_of(v, dir)), md1(md_of(v, dir == 0 ? 1 : 0)),
        md2(md_of(v, dir == 2 ? 1 : 2)), Ct(v->Conserved_t), nt(ntype_of(v, dir)),
        nt1(ntype_of(v, dir == 0 ? 1 : 0)), nt2(ntype_of(v, dir == 2 ? 1 : 2)) {}

  // velocity gradient along direction e at point p (metric.inl:103-134)
  void grad(double *g, const long long *p, int e, const Fld<int> &ntt, const Fld<double> &mm) const {
    const int t = ntt(p);
    long long pm[3], pp[3];
    shiftm(pm, p, e, fb, kNodes[t].off[1]);
    shiftp(pp, p, e, fb, kNodes[t].off[2]);
    for (int i = 0; i < 3; i++) g[i] = deriv(t, u.at(pm)[i], u.at(p)[i], u.at(pp)[i], mm(p));
  }

  void face(double *F, const long long *p, double g1[2][3], double g2[2][3]) const {
    const int t = nt(p);
    const double m_s = ms(p);
    long long q[3];
    shiftp(q, p, d, fb, 1);
    grad(g1[1], q, t1, nt1, md1);
    grad(g2[1], q, t2, nt2, md2);
    const double rho_s = interp2(t, rho(p), rho(q));
    const double iMixW_s = 1.0 / interp2(t, mix.MolarWeightFromXi(X.at(p)), mix.MolarWeightFromXi(X.at(q)));
    const double T_s = interp2(t, T(p), T(q));
    double heat = interp2(t, lam(p), lam(q)) * m_s * (T(p) - T(q));
    double ViCorr = 0.0;
    for (int i = 0; i < NS; i++) {
      const double YiVi = interp2(t, Di.at(p)[i], Di.at(q)[i]) * m_s * (X.at(p)[i] - X.at(q)[i]) *
                          mix.SpeciesMolarWeight(i) * iMixW_s;
      F[i] = -rho_s * YiVi;
      heat += rho_s * YiVi * mix.SpeciesEnthalpy(i, T_s);
      ViCorr += YiVi;
    }
    for (int i = 0; i < NS; i++) {
      const double c = interp2(t, C.at(p)[i], C.at(q)[i]) * ViCorr;
      F[i] += c;
      heat -= c * mix.SpeciesEnthalpy(i, T_s);
    }
    // viscous stress (rhs.inl:1058-1137, one formula for the three directions)
    const double mu_s = interp2(t, mu(p), mu(q));
    const double *up = u.at(p), *uq = u.at(q);
    const double dn_n = m_s * (uq[d] - up[d]);
    const double dn_t1 = m_s * (uq[t1] - up[t1]);
    const double dn_t2 = m_s * (uq[t2] - up[t2]);
    const double d1_n = interp2(t, g1[0][d], g1[1][d]);
    const double d1_t1 = interp2(t, g1[0][t1], g1[1][t1]);
    const double d2_n = interp2(t, g2[0][d], g2[1][d]);
    const double d2_t2 = interp2(t, g2[0][t2], g2[1][t2]);
    double sigma[3];
    sigma[d] = mu_s * (4 * dn_n - 2 * d1_t1 - 2 * d2_t2) / 3;
    sigma[t1] = mu_s * (dn_t1 + d1_n);
    sigma[t2] = mu_s * (dn_t2 + d2_n);
    for (int i = 0; i < 3; i++) F[iU + i] = sigma[i];
    double uSigma = 0.0;
    for (int i = 0; i < 3; i++) uSigma += interp2(t, up[i], uq[i]) * sigma[i];
    F[iE] = (uSigma - heat);
    for (int i = 0; i < 3; i++) {
      g1[0][i] = g1[1][i];
      g2[0][i] = g2[1][i];
    }
  }

  void sweep(const long long *p0, long long n) const {
    double Fm[NE], Fp[NE], g1[2][3], g2[2][3];
    {
      long long pm1[3];
      shiftm(pm1, p0, d, fb, kNodes[nt(p0)].off[1]);
      grad(g1[0], pm1, t1, nt1, md1);
      grad(g2[0], pm1, t2, nt2, md2);
      face(Fm, pm1, g1, g2);
    }
    for (long long i = 0; i < n; i++) {
      long long p[3] = {p0[0], p0[1], p0[2]};
      p[d] += i;
      face(Fp, p, g1, g2);
      double *ct = Ct.at(p);
      const double m = md(p);
      for (int k = 0; k < NE; k++) ct[k] += m * (Fp[k] - Fm[k]);
      for (int k = 0; k < NE; k++) Fm[k] = Fp[k];
    }
  }
};

// ===========================================================================
// dispatch helpers
// ===========================================================================
template <class F> int with_mix(htr_mixture_t mix, F &&f) {
  if (mix == nullptr) return HTR_ERR_ARGUMENT;
  if (mix->eos == HTR_EOS_CONSTPROPMIX) return f(mix->cp);
  if (mix->eos == HTR_EOS_AIRMIX) return f(mix->air);
  return HTR_ERR_UNSUPPORTED;
}

enum Scheme { kHybrid, kSkew, kTenoOnly };

int euler(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fbr, const double *rk, double dt,
          htr_mixture_t mix, int d, Scheme scheme, TenoKind kind) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    using M = std::decay_t<decltype(m)>;
    Euler<M> E(m, v, d, box(fbr), rk, dt);
    const Box r = box(myf);
    const long long n = r.size(d);
    for_pencils(r, d, [&](const long long *p0) {
      if (scheme == kTenoOnly)
        E.sweep_teno(p0, n, kind);
      else
        E.sweep_kg(p0, n, scheme == kHybrid);
    });
    return int(HTR_OK);
  });
}

int diffusion(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fbr, htr_mixture_t mix, int d) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    using M = std::decay_t<decltype(m)>;
    Diffusion<M> D(m, v, d, box(fbr));
    const Box r = box(myf);
    const long long n = r.size(d);
    for_pencils(r, d, [&](const long long *p0) { D.sweep(p0, n); });
    return int(HTR_OK);
  });
}

}  // namespace

// ===========================================================================
// exported entry points
// ===========================================================================
extern "C" {

const char *htr_last_error(void) { return g_err.c_str(); }

int htr_oracle_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}

int htr_load_mixture(int eos, const void *mixp, size_t bytes, htr_mixture_t *out) {
  if (mixp == nullptr || out == nullptr) return HTR_ERR_ARGUMENT;
  htr_mixture_s *m = new htr_mixture_s();
  m->eos = eos;
  if (eos == HTR_EOS_CONSTPROPMIX && bytes == sizeof(htr_constpropmix_t)) {
    std::memcpy(&m->cp.m, mixp, bytes);
  } else if (eos == HTR_EOS_AIRMIX && bytes == sizeof(htr_airmix_t)) {
    std::memcpy(&m->air.m, mixp, bytes);
  } else {
    delete m;
    g_err = "htr_load_mixture: unknown EOS or wrong struct size";
    return HTR_ERR_ARGUMENT;
  }
  *out = m;
  return HTR_OK;
}
int htr_free_mixture(htr_mixture_t m) {
  delete m;
  return HTR_OK;
}
int htr_mixture_eos(htr_mixture_t m) { return m ? m->eos : 0; }

#define ORACLE_EULER(NAME, D, SCHEME, KIND)                                                   \
  int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, const double rk[2], double dt, \
           htr_mixture_t mix, htr_stream_t) {                                                 \
    return euler(v, m, b, rk, dt, mix, D, SCHEME, KIND);                                      \
  }
ORACLE_EULER(htr_UpdateUsingHybridEulerFluxX, 0, kHybrid, kTENO)
ORACLE_EULER(htr_UpdateUsingHybridEulerFluxY, 1, kHybrid, kTENO)
ORACLE_EULER(htr_UpdateUsingHybridEulerFluxZ, 2, kHybrid, kTENO)
ORACLE_EULER(htr_UpdateUsingTENOEulerFluxX, 0, kTenoOnly, kTENO)
ORACLE_EULER(htr_UpdateUsingTENOEulerFluxY, 1, kTenoOnly, kTENO)
ORACLE_EULER(htr_UpdateUsingTENOEulerFluxZ, 2, kTenoOnly, kTENO)
ORACLE_EULER(htr_UpdateUsingTENOAEulerFluxX, 0, kTenoOnly, kTENOA)
ORACLE_EULER(htr_UpdateUsingTENOAEulerFluxY, 1, kTenoOnly, kTENOA)
ORACLE_EULER(htr_UpdateUsingTENOAEulerFluxZ, 2, kTenoOnly, kTENOA)
ORACLE_EULER(htr_UpdateUsingTENOLADEulerFluxX, 0, kTenoOnly, kTENOLAD)
ORACLE_EULER(htr_UpdateUsingTENOLADEulerFluxY, 1, kTenoOnly, kTENOLAD)
ORACLE_EULER(htr_UpdateUsingTENOLADEulerFluxZ, 2, kTenoOnly, kTENOLAD)

#define ORACLE_SKEW(NAME, D)                                                                 \
  int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t mix,            \
           htr_stream_t) {                                                                   \
    return euler(v, m, b, nullptr, 0.0, mix, D, kSkew, kTENO);                               \
  }
ORACLE_SKEW(htr_UpdateUsingSkewSymmetricEulerFluxX, 0)
ORACLE_SKEW(htr_UpdateUsingSkewSymmetricEulerFluxY, 1)
ORACLE_SKEW(htr_UpdateUsingSkewSymmetricEulerFluxZ, 2)

#define ORACLE_DIFF(NAME, D)                                                                 \
  int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t mix,            \
           htr_stream_t) {                                                                   \
    return diffusion(v, m, b, mix, D);                                                       \
  }
ORACLE_DIFF(htr_UpdateUsingDiffusionFluxX, 0)
ORACLE_DIFF(htr_UpdateUsingDiffusionFluxY, 1)
ORACLE_DIFF(htr_UpdateUsingDiffusionFluxZ, 2)

// --- sensors (sensor.inl:47-76, sensor.cc:76-128) --------------------------
int htr_UpdateDucrosSensor(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fbr,
                           double vorticityScale, htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  const Box fb = box(fbr);
  const Fld<double> u(v->velocity), out(v->DucrosSensor);
  const Fld<int> n[3] = {Fld<int>(v->nType_x), Fld<int>(v->nType_y), Fld<int>(v->nType_z)};
  const Fld<double> m[3] = {Fld<double>(v->dcsi_d), Fld<double>(v->deta_d), Fld<double>(v->dzet_d)};
  const double eps = std::max(vorticityScale * vorticityScale, 1e-6);
  for_cells(box(myf), [&](const long long *p) {
    double g[3][3];
    for (int e = 0; e < 3; e++) {
      const int t = n[e](p);
      long long pm[3], pp[3];
      shiftm(pm, p, e, fb, kNodes[t].off[1]);
      shiftp(pp, p, e, fb, kNodes[t].off[2]);
      for (int i = 0; i < 3; i++) g[e][i] = deriv(t, u.at(pm)[i], u.at(p)[i], u.at(pp)[i], m[e](p));
    }
    const double div = g[0][0] + g[1][1] + g[2][2];
    const double div2 = div * div;
    const double omz = g[0][1] - g[1][0];
    const double omy = g[1][2] - g[2][1];
    const double omx = g[2][0] - g[0][2];
    const double om2 = omx * omx + omy * omy + omz * omz;
    out(p) = div2 / (div2 + om2 + eps);
  });
  return HTR_OK;
}

static int shock_sensor(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fbr, htr_mixture_t mix,
                        int d) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  const int ns = (mix && mix->eos == HTR_EOS_AIRMIX) ? 5 : 1;
  const Box fb = box(fbr);
  const Fld<double> C(v->Conserved), duc(v->DucrosSensor);
  const Fld<int> nt(ntype_of(v, d));
  const Fld<bool> out(sensor_of(v, d));
  for_cells(box(myf), [&](const long long *p) {
    const int t = nt(p);
    long long q[6][3];
    shiftm(q[0], p, d, fb, kNodes[t].off[0]);
    shiftm(q[1], p, d, fb, kNodes[t].off[1]);
    q[2][0] = p[0]; q[2][1] = p[1]; q[2][2] = p[2];
    shiftp(q[3], p, d, fb, kNodes[t].off[2]);
    shiftp(q[4], p, d, fb, kNodes[t].off[3]);
    shiftp(q[5], p, d, fb, kNodes[t].off[4]);
    double Phi = duc(q[0]);
    for (int k = 1; k < 6; k++) Phi = std::max(Phi, duc(q[k]));
    bool s = true;
    for (int h = 0; h < ns && s; h++)
      s = teno_a_sensor(C.at(q[0])[h], C.at(q[1])[h], C.at(q[2])[h], C.at(q[3])[h], C.at(q[4])[h],
                        C.at(q[5])[h], t, Phi);
    out(p) = s;
  });
  return HTR_OK;
}
int htr_UpdateShockSensorX(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t x,
                           htr_stream_t) { return shock_sensor(v, m, b, x, 0); }
int htr_UpdateShockSensorY(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t x,
                           htr_stream_t) { return shock_sensor(v, m, b, x, 1); }
int htr_UpdateShockSensorZ(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t x,
                           htr_stream_t) { return shock_sensor(v, m, b, x, 2); }

// --- chemistry sources (chem.cc:71-110) -----------------------------------
int htr_AddChemistrySources(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix,
                            htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    using M = std::decay_t<decltype(m)>;
    constexpr int NS = M::NS;
    const Fld<double> rho(v->rho), P(v->pressure), T(v->temperature), Y(v->MassFracs),
        Ct(v->Conserved_t);
    for_cells(box(myf), [&](const long long *p) {
      double w[NS];
      m.ProductionRates(w, rho(p), P(p), T(p), Y.at(p));
      for (int i = 0; i < NS; i++) Ct.at(p)[i] += w[i];
    });
    return int(HTR_OK);
  });
}

// --- state refresh (variables.hpp:52-210) ----------------------------------
int htr_UpdatePropertiesFromPrimitive(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix,
                                      htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    const Fld<double> P(v->pressure), T(v->temperature), X(v->MolarFracs), Y(v->MassFracs),
        rho(v->rho), mu(v->mu), lam(v->lam), Di(v->Di), SoS(v->SoS);
    for_cells(box(myf), [&](const long long *p) {
      const double MixW = m.MolarWeightFromXi(X.at(p));
      rho(p) = m.Rho(P(p), T(p), MixW);
      mu(p) = m.Viscosity(T(p), X.at(p));
      lam(p) = m.HeatConductivity(T(p), X.at(p));
      m.Diffusivity(Di.at(p), P(p), T(p), MixW, X.at(p));
      m.MassFractions(Y.at(p), MixW, X.at(p));
      const double gamma = m.Gamma(T(p), MixW, Y.at(p));
      SoS(p) = m.SpeedOfSound(T(p), gamma, MixW);
    });
    return int(HTR_OK);
  });
}

int htr_UpdateConservedFromPrimitive(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix,
                                     htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    using M = std::decay_t<decltype(m)>;
    constexpr int NS = M::NS;
    const Fld<double> Y(v->MassFracs), T(v->temperature), u(v->velocity), rho(v->rho),
        C(v->Conserved);
    for_cells(box(myf), [&](const long long *p) {
      double *c = C.at(p);
      const double r = rho(p);
      for (int i = 0; i < NS; i++) c[i] = r * Y.at(p)[i];
      for (int i = 0; i < 3; i++) c[NS + i] = r * u.at(p)[i];
      c[NS + 3] = r * (0.5 * mod2(u.at(p)) + m.InternalEnergy(T(p), Y.at(p)));
    });
    return int(HTR_OK);
  });
}

int htr_UpdatePrimitiveFromConserved(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix,
                                     htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    using M = std::decay_t<decltype(m)>;
    constexpr int NS = M::NS;
    const Fld<double> C(v->Conserved), T(v->temperature), P(v->pressure), X(v->MolarFracs),
        u(v->velocity);
    for_cells(box(myf), [&](const long long *p) {
      const double *c = C.at(p);
      double rhoYi[NS], Yi[NS];
      for (int i = 0; i < NS; i++) rhoYi[i] = c[i];
      const double rho = m.RhoFromRhoYi(rhoYi);
      m.YiFromRhoYi(Yi, rho, rhoYi);
      m.ClipYi(Yi);
      const double MixW = m.MolarWeightFromYi(Yi);
      m.MolarFractions(X.at(p), MixW, Yi);
      const double rhoInv = 1.0 / rho;
      double *vel = u.at(p);
      for (int i = 0; i < 3; i++) vel[i] = c[NS + i] * rhoInv;
      const double ke = 0.5 * mod2(vel);
      const double e = c[NS + 3] * rhoInv - ke;
      T(p) = m.TFromInternalEnergy(e, T(p), Yi);
      P(p) = m.PFromRhoAndT(rho, MixW, T(p));
    });
    return int(HTR_OK);
  });
}

// --- spectral radius (cfl.hpp:70-190) --------------------------------------
int htr_CalculateMaxSpectralRadius(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix,
                                   double *result, htr_stream_t) {
  if (v == nullptr || result == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    using M = std::decay_t<decltype(m)>;
    constexpr int NS = M::NS;
    const Fld<double> dx(v->dcsi_d), dy(v->deta_d), dz(v->dzet_d), T(v->temperature),
        Y(v->MassFracs), u(v->velocity), rho(v->rho), mu(v->mu), lam(v->lam), Di(v->Di),
        SoS(v->SoS);
    const Box r = box(myf);
    double best = 0.0;
#pragma omp parallel for collapse(3) reduction(max : best)
    for (long long k = r.lo[2]; k <= r.hi[2]; k++)
      for (long long j = r.lo[1]; j <= r.hi[1]; j++)
        for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
          const long long p[3] = {i, j, k};
          const double a = dx(p), b = dy(p), c = dz(p);
          const double *vel = u.at(p);
          double s = (std::fabs(vel[0]) + SoS(p)) * a;
          s = std::max(s, (std::fabs(vel[1]) + SoS(p)) * b);
          s = std::max(s, (std::fabs(vel[2]) + SoS(p)) * c);
          const double nu = mu(p) / rho(p);
          double rv = nu * a * a;
          rv = std::max(rv, nu * b * b);
          rv = std::max(rv, nu * c * c);
          rv *= 4;
          s = std::max(s, rv);
          const double cp = m.HeatCapacity(T(p), Y.at(p));
          const double DifT = lam(p) / (cp * rho(p));
          double rh = DifT * a * a;
          rh = std::max(rh, DifT * b * b);
          rh = std::max(rh, DifT * c * c);
          rh *= 4;
          s = std::max(s, rh);
          double rs = 0.0;
          for (int q = 0; q < NS; q++) {
            rs = std::max(rs, Di.at(p)[q] * a * a);
            rs = std::max(rs, Di.at(p)[q] * b * b);
            rs = std::max(rs, Di.at(p)[q] * c * c);
          }
          rs *= 4;
          s = std::max(s, rs);
          best = std::max(best, s);
        }
    *result = best;
    return int(HTR_OK);
  });
}

}  // extern "C"
