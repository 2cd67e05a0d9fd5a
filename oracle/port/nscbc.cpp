// CPU oracle port: NSCBC boundary terms and the maximum Mach number.
// TEST INFRASTRUCTURE ONLY.
//
// Restates, operation by operation,
//   UpdateUsingFluxNSCBCInflow{Minus,Plus}SideTask   src/prometeo_rhs.inl:1288-1419,
//                                                     src/prometeo_rhs.cc:531-580
//   UpdateUsingFluxNSCBCOutflow{Minus,Plus}SideTask  src/prometeo_rhs.inl:1424-1628,
//                                                     src/prometeo_rhs.cc:685-740
//   CalculateMaxMachNumber                            src/prometeo_stat.rg:223-234
// with the one-sided boundary derivatives of src/prometeo_metric.inl:95-102
// and the first interior point of src/Utils/PointDomain_helper.hpp:115-133.
#include <cmath>
#include <cstdint>
#include <limits>

#include "htr_rhs.h"
#include "mixtures.hpp"
#include "port.hpp"
#include "stencils.hpp"

using namespace oport;

namespace {

template <class T> struct F3 {
  char *b;
  int64_t s[3];
  explicit F3(const htr_field &f) : b(static_cast<char *>(f.base)) {
    for (int i = 0; i < 3; i++) s[i] = f.stride[i];
  }
  T *at(const long long *p) const { return reinterpret_cast<T *>(b + p[0] * s[0] + p[1] * s[1] + p[2] * s[2]); }
};

const htr_field &ntype(const htr_fluid_view *v, int d) {
  return d == 0 ? v->nType_x : (d == 1 ? v->nType_y : v->nType_z);
}
const htr_field &mdiff(const htr_fluid_view *v, int d) {
  return d == 0 ? v->dcsi_d : (d == 1 ? v->deta_d : v->dzet_d);
}

// one-sided boundary derivatives (getDerivLeftBC / getDerivRightBC)
inline double dleft(int t, double x, double xp1, double m) { return (kNodes[t].grad[1] * (xp1 - x)) * m; }
inline double dright(int t, double xm1, double x, double m) { return (kNodes[t].grad[0] * (x - xm1)) * m; }

// getDeriv<e> of component c of the velocity at p (warpPeriodic stencil)
inline double vderiv(const F3<double> &u, const long long *p, int c, int e, int t, double m, const htr_rect3 &fb) {
  const long long size = fb.hi[e] - fb.lo[e] + 1;
  long long pm[3] = {p[0], p[1], p[2]}, pp[3] = {p[0], p[1], p[2]};
  pm[e] = wrap_minus(p[e], fb.lo[e], size, kNodes[t].off[1]);
  pp[e] = wrap_plus(p[e], fb.lo[e], size, kNodes[t].off[2]);
  return deriv(t, u.at(pm)[c], u.at(p)[c], u.at(pp)[c], m);
}

template <class Mix> void inflow(const Mix &mix, const htr_fluid_view *v, const htr_rect3 &bc, int dir, bool minus) {
  constexpr int NS = Mix::NS, NE = NS + 4;
  const int iN = dir;
  F3<double> Y(v->MassFracs), P(v->pressure), u(v->velocity), rho(v->rho), SoS(v->SoS), T(v->temperature),
      dudt(v->dudtBoundary), dTdt(v->dTdtBoundary), m_d(mdiff(v, dir)), Ct(v->Conserved_t);
  F3<int> nt(ntype(v, dir));
#pragma omp parallel for collapse(3)
  for (long long k = bc.lo[2]; k <= bc.hi[2]; k++)
    for (long long j = bc.lo[1]; j <= bc.hi[1]; j++)
      for (long long i = bc.lo[0]; i <= bc.hi[0]; i++) {
        const long long p[3] = {i, j, k};
        double *RHS = Ct.at(p);
        const double un = u.at(p)[iN], c = *SoS.at(p), r = *rho.at(p), Tp = *T.at(p);
        if (minus ? (un >= c) : (un <= -c)) {
          for (int l = 0; l < NE; l++) RHS[l] = 0.0;
          continue;
        }
        long long q[3] = {i, j, k};
        q[dir] += minus ? 1 : -1;
        const int t = *nt.at(p);
        const double m = *m_d.at(p);
        const double MixW_bnd = mix.MolarWeightFromYi(Y.at(p));
        const double Cp_bnd = mix.HeatCapacity(Tp, Y.at(p));
        const double lambda = un;
        double LS[NS];
        double L1, LN;
        if (minus) {
          const double lambda_1 = un - c;
          const double dp_dn = dleft(t, *P.at(p), *P.at(q), m);
          const double du_dn = dleft(t, u.at(p)[iN], u.at(q)[iN], m);
          L1 = lambda_1 * (dp_dn - r * c * du_dn);
          for (int s = 0; s < NS; s++) LS[s] = lambda * dleft(t, Y.at(p)[s], Y.at(q)[s], m);
          LN = L1 - 2 * r * c * dudt.at(p)[iN];
        } else {
          const double lambda_N = un + c;
          const double dp_dn = dright(t, *P.at(q), *P.at(p), m);
          const double du_dn = dright(t, u.at(q)[iN], u.at(p)[iN], m);
          LN = lambda_N * (dp_dn + r * c * du_dn);
          for (int s = 0; s < NS; s++) LS[s] = lambda * dright(t, Y.at(q)[s], Y.at(p)[s], m);
          L1 = LN + 2 * r * c * dudt.at(p)[iN];
        }
        double L2 = *dTdt.at(p) / Tp + (LN + L1) / (2 * r * Cp_bnd * Tp);
        for (int s = 0; s < NS; s++) L2 -= MixW_bnd / mix.SpeciesMolarWeight(s) * LS[s];
        L2 *= -r * c * c;
        const double d1 = (0.5 * (L1 + LN) - L2) / (c * c);
        for (int s = 0; s < NS; s++) RHS[s] -= (d1 * Y.at(p)[s] + r * LS[s]);
      }
}

template <class Mix>
void outflow(const Mix &mix, const htr_fluid_view *v, const htr_rect3 &bc, const htr_rect3 &fb, int dir, bool minus,
             double MaxMach, double LengthScale, double PInf) {
  constexpr int NS = Mix::NS;
  const int iN = dir, iT1 = (dir == 0) ? 1 : 0, iT2 = (dir == 2) ? 1 : 2;
  const int eT1 = iT1, eT2 = iT2;  // tangential directions getT1/getT2
  const int irU = NS, irE = NS + 3;
  F3<double> Y(v->MassFracs), P(v->pressure), u(v->velocity), rho(v->rho), mu(v->mu), SoS(v->SoS),
      T(v->temperature), C(v->Conserved), Ct(v->Conserved_t), mN(mdiff(v, dir)), mT1(mdiff(v, eT1)),
      mT2(mdiff(v, eT2));
  F3<int> nN(ntype(v, dir)), nT1(ntype(v, eT1)), nT2(ntype(v, eT2));
#pragma omp parallel for collapse(3)
  for (long long k = bc.lo[2]; k <= bc.hi[2]; k++)
    for (long long j = bc.lo[1]; j <= bc.hi[1]; j++)
      for (long long i = bc.lo[0]; i <= bc.hi[0]; i++) {
        const long long p[3] = {i, j, k};
        long long q[3] = {i, j, k};
        q[dir] += minus ? 1 : -1;
        double *RHS = Ct.at(p);
        const double *Cp = C.at(p);
        const double c = *SoS.at(p), Tp = *T.at(p), rp = *rho.at(p), mup = *mu.at(p);
        const int t = *nN.at(p);
        const double m = *mN.at(p);
        auto D = [&](double bnd, double in) { return minus ? dleft(t, bnd, in, m) : dright(t, in, bnd, m); };
        const double dp_dn = D(*P.at(p), *P.at(q));
        const double dun_dn = D(u.at(p)[iN], u.at(q)[iN]);
        const double duT1dn = D(u.at(p)[iT1], u.at(q)[iT1]);
        const double duT2dn = D(u.at(p)[iT2], u.at(q)[iT2]);
        const double un = u.at(p)[iN];
        const double lambda_1 = un - c;
        const double lambda = un;
        const double lambda_s = minus ? std::min(un, 0.0) : std::max(un, 0.0);
        const double lambda_N = un + c;
        const double sigma = 0.25;
        auto relax = [&]() {
          const double K = (MaxMach < 0.99) ? sigma * (1.0 - MaxMach * MaxMach) * c / LengthScale
                                            : sigma * (c - (un * un) / c) / LengthScale;
          return K * (*P.at(p) - PInf);
        };
        double L1, LN, LM;
        double LS[NS];
        if (minus) {
          L1 = lambda_1 * (dp_dn - rp * c * dun_dn);
          LM = lambda * (dp_dn - c * c * D(rp, *rho.at(q)));
          for (int s = 0; s < NS; s++) LS[s] = lambda_s * D(Y.at(p)[s], Y.at(q)[s]);
          if (lambda_N < 0)
            LN = lambda_N * (dp_dn + rp * c * dun_dn);
          else
            LN = relax();
        } else {
          if (lambda_1 > 0)
            L1 = lambda_1 * (dp_dn - rp * c * dun_dn);
          else
            L1 = relax();
          LM = lambda * (dp_dn - c * c * D(rp, *rho.at(q)));
          for (int s = 0; s < NS; s++) LS[s] = lambda_s * D(Y.at(p)[s], Y.at(q)[s]);
          LN = lambda_N * (dp_dn + rp * c * dun_dn);
        }
        const double d1 = (0.5 * (L1 + LN) - LM) / (c * c);
        double dM[3];
        dM[iN] = (LN - L1) / (2 * rp * c);
        dM[iT1] = lambda * duT1dn;
        dM[iT2] = lambda * duT2dn;
        const double dN = LM / (c * c);
        double vT1[3], vT2[3];
        for (int cc = 0; cc < 3; cc++) {
          vT1[cc] = vderiv(u, p, cc, eT1, *nT1.at(p), *mT1.at(p), fb);
          vT2[cc] = vderiv(u, p, cc, eT2, *nT2.at(p), *mT2.at(p), fb);
        }
        const double tauNN_bnd = mup * (4 * dun_dn - 2 * vT1[iT1] - 2 * vT2[iT2]) / 3;
        const double tauNN_int = *mu.at(q) * (4 * vderiv(u, q, iN, dir, *nN.at(q), *mN.at(q), fb)
                                            - 2 * vderiv(u, q, iT1, eT1, *nT1.at(q), *mT1.at(q), fb)
                                            - 2 * vderiv(u, q, iT2, eT2, *nT2.at(q), *mT2.at(q), fb)) / 3;
        const double dtau_dn = D(tauNN_bnd, tauNN_int);
        const double viscous_heating = D(un * tauNN_bnd, u.at(q)[iN] * tauNN_int) +
                                       duT1dn * mup * (duT1dn + vT1[iN]) +
                                       duT2dn * mup * (duT2dn + vT2[iN]);
        const double cpT = mix.HeatCapacity(Tp, Y.at(p)) * Tp;
        for (int s = 0; s < NS; s++) RHS[s] -= (d1 * Y.at(p)[s] + rp * LS[s]);
        RHS[irU + iN] -= (u.at(p)[iN] * d1 + rp * dM[iN] - dtau_dn);
        RHS[irU + iT1] -= (u.at(p)[iT1] * d1 + rp * dM[iT1]);
        RHS[irU + iT2] -= (u.at(p)[iT2] * d1 + rp * dM[iT2]);
        RHS[irE] -= ((Cp[irE] + *P.at(p)) * d1 / rp
                     + Cp[irU + iN] * dM[iN]
                     + Cp[irU + iT1] * dM[iT1]
                     + Cp[irU + iT2] * dM[iT2]
                     + cpT * dN
                     - viscous_heating);
        const double cpT_Wmix = cpT * mix.MolarWeightFromYi(Y.at(p));
        for (int s = 0; s < NS; s++) {
          const double dEdYi = mix.SpeciesEnthalpy(s, Tp) - cpT_Wmix / mix.SpeciesMolarWeight(s);
          RHS[irE] -= (rp * LS[s] * dEdYi);
        }
      }
}

template <class F> int with_mix(htr_mixture_t mix, F &&f) {
  if (mix == nullptr) return HTR_ERR_ARGUMENT;
  if (mix->eos == HTR_EOS_CONSTPROPMIX) return f(mix->cp);
  if (mix->eos == HTR_EOS_AIRMIX) return f(mix->air);
  return HTR_ERR_UNSUPPORTED;
}

int run_inflow(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t mix, int dir, bool minus) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    inflow(m, v, bc, dir, minus);
    return HTR_OK;
  });
}
int run_outflow(const htr_fluid_view *v, htr_rect3 bc, htr_rect3 fb, htr_mixture_t mix, int dir, bool minus,
                double MaxMach, double LengthScale, double PInf) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    outflow(m, v, bc, fb, dir, minus, MaxMach, LengthScale, PInf);
    return HTR_OK;
  });
}

}  // namespace

#define HTR_PORT_NSCBC(SIDE, DIR, MINUS)                                                                    \
  extern "C" int htr_UpdateUsingFluxNSCBCInflow##SIDE(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, \
                                                      htr_stream_t) {                                       \
    return run_inflow(v, bc, m, DIR, MINUS);                                                                \
  }                                                                                                         \
  extern "C" int htr_UpdateUsingFluxNSCBCOutflow##SIDE(const htr_fluid_view *v, htr_rect3 bc, htr_rect3 fb,  \
                                                       htr_mixture_t m, double MaxMach, double LengthScale, \
                                                       double PInf, htr_stream_t) {                          \
    return run_outflow(v, bc, fb, m, DIR, MINUS, MaxMach, LengthScale, PInf);                               \
  }
HTR_PORT_NSCBC(XNeg, 0, true)
HTR_PORT_NSCBC(XPos, 0, false)
HTR_PORT_NSCBC(YNeg, 1, true)
HTR_PORT_NSCBC(YPos, 1, false)
HTR_PORT_NSCBC(ZNeg, 2, true)
HTR_PORT_NSCBC(ZPos, 2, false)
#undef HTR_PORT_NSCBC

extern "C" int htr_CalculateMaxMachNumber(const htr_fluid_view *v, htr_rect3 r, int dir, double *result,
                                          htr_stream_t) {
  if (v == nullptr || result == nullptr || dir < 0 || dir > 2) return HTR_ERR_ARGUMENT;
  F3<double> u(v->velocity), SoS(v->SoS);
  double acc = -std::numeric_limits<double>::infinity();
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        const long long p[3] = {i, j, k};
        acc = std::max(acc, std::fabs(u.at(p)[dir]) / *SoS.at(p));
      }
  *result = acc;
  return HTR_OK;
}
