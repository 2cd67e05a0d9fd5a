// CPU oracle port: boundary-condition state updates.
// TEST INFRASTRUCTURE ONLY.
//
//   SetNSCBC_InflowBCTask<dir>   src/prometeo_bc.hpp:108-150, src/prometeo_bc.cc:84-135
//   SetNSCBC_OutflowBCTask       src/prometeo_bc.cc:160-197 (the per-cell primitive
//                                recovery of src/prometeo_variables.hpp:163-193)
//   SetIsothermalWallBC / SetAdiabaticWallBC   src/prometeo_bc.rg:1207-1263 (Regent)
//   UpdateNSCBCGhostCellTimeDerivatives        src/prometeo_bc.rg:1794-1810 (Regent)
#include <cmath>
#include <cstdint>

#include "htr_rhs.h"
#include "mixtures.hpp"
#include "port.hpp"

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

template <class F> void for_cells(const htr_rect3 &r, F &&f) {
#pragma omp parallel for collapse(3)
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        const long long p[3] = {i, j, k};
        f(p);
      }
}

template <class F> int with_mix(htr_mixture_t mix, F &&f) {
  if (mix == nullptr) return HTR_ERR_ARGUMENT;
  if (mix->eos == HTR_EOS_CONSTPROPMIX) return f(mix->cp);
  if (mix->eos == HTR_EOS_AIRMIX) return f(mix->air);
  return HTR_ERR_UNSUPPORTED;
}

int inflow_bc(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t mix, double Pbc, int dir) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  return with_mix(mix, [&](const auto &m) {
    using M = std::decay_t<decltype(m)>;
    constexpr int NS = M::NS;
    F3<double> C(v->Conserved), SoS(v->SoS), Xp(v->MolarFracs_profile), Tp(v->temperature_profile),
        up(v->velocity_profile), P(v->pressure), T(v->temperature), X(v->MolarFracs), u(v->velocity);
    for_cells(bc, [&](const long long *p) {
      for (int s = 0; s < NS; s++) X.at(p)[s] = Xp.at(p)[s];
      *T.at(p) = *Tp.at(p);
      for (int i = 0; i < 3; i++) u.at(p)[i] = up.at(p)[i];
      if (std::fabs(up.at(p)[dir]) >= *SoS.at(p)) {
        *P.at(p) = Pbc;  // supersonic: everything imposed
      } else {
        double rhoYi[NS];
        for (int s = 0; s < NS; s++) rhoYi[s] = C.at(p)[s];
        const double rho = m.RhoFromRhoYi(rhoYi);
        const double MixW = m.MolarWeightFromXi(Xp.at(p));
        *P.at(p) = m.PFromRhoAndT(rho, MixW, *Tp.at(p));
      }
    });
    return int(HTR_OK);
  });
}

int wall_bc(const htr_fluid_view *v, htr_rect3 bc, int side, htr_mixture_t mix, bool isothermal) {
  if (v == nullptr || mix == nullptr || side < 0 || side > 5) return HTR_ERR_ARGUMENT;
  const int d = side / 2;
  const int step = (side % 2 == 0) ? 1 : -1;  // towards the interior
  const int ns = (mix->eos == HTR_EOS_AIRMIX) ? 5 : 1;
  F3<double> X(v->MolarFracs), P(v->pressure), T(v->temperature), u(v->velocity), Tp(v->temperature_profile);
  for_cells(bc, [&](const long long *p) {
    long long q[3] = {p[0], p[1], p[2]};
    q[d] += step;
    for (int s = 0; s < ns; s++) X.at(p)[s] = X.at(q)[s];
    *P.at(p) = *P.at(q);
    *T.at(p) = isothermal ? *Tp.at(p) : *T.at(q);
    for (int i = 0; i < 3; i++) u.at(p)[i] = 0.0;
  });
  return HTR_OK;
}

}  // namespace

extern "C" {

int htr_SetNSCBC_InflowBCX(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t) {
  return inflow_bc(v, bc, m, Pbc, 0);
}
int htr_SetNSCBC_InflowBCY(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t) {
  return inflow_bc(v, bc, m, Pbc, 1);
}
int htr_SetNSCBC_InflowBCZ(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t) {
  return inflow_bc(v, bc, m, Pbc, 2);
}
int htr_UpdatePrimitiveFromConserved(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix, htr_stream_t);
int htr_SetNSCBC_OutflowBC(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, int *status, htr_stream_t s) {
  if (status) *status = 0;
  return htr_UpdatePrimitiveFromConserved(v, bc, m, s);
}
int htr_SetIsothermalWallBC(const htr_fluid_view *v, htr_rect3 bc, int side, htr_mixture_t m, htr_stream_t) {
  return wall_bc(v, bc, side, m, true);
}
int htr_SetAdiabaticWallBC(const htr_fluid_view *v, htr_rect3 bc, int side, htr_mixture_t m, htr_stream_t) {
  return wall_bc(v, bc, side, m, false);
}
int htr_UpdateNSCBCGhostCellTimeDerivatives(const htr_fluid_view *v, htr_rect3 bc, double dt, htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  F3<double> u(v->velocity), T(v->temperature), dudt(v->dudtBoundary), dTdt(v->dTdtBoundary),
      uo(v->velocity_old_NSCBC), To(v->temperature_old_NSCBC);
  for_cells(bc, [&](const long long *p) {
    for (int i = 0; i < 3; i++) dudt.at(p)[i] = (u.at(p)[i] - uo.at(p)[i]) / dt;
    *dTdt.at(p) = (*T.at(p) - *To.at(p)) / dt;
    for (int i = 0; i < 3; i++) uo.at(p)[i] = u.at(p)[i];
    *To.at(p) = *T.at(p);
  });
  return HTR_OK;
}

}  // extern "C"
