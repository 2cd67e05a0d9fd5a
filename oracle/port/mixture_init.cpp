// CPU oracle port: mixture construction and RK bookkeeping.
// TEST INFRASTRUCTURE ONLY.
//
// htr_airmix_init fills the 5-species air data (NASA-9 polynomials,
// Lennard-Jones data, Park-type reactions) of src/Mixtures/AirMix.hpp:58-317
// and the reference scales of StoreReferenceQuantities
// (src/Mixtures/MultiComponent.inl:438-487).  The SSP-RK3 helpers restate
// the Regent tasks of src/prometeo_rk.rg:47-112.
#include <omp.h>

#include <cmath>
#include <cstring>

#include "htr_rhs.h"
#include "mixtures.hpp"

using namespace oport;

namespace {

constexpr double kATom = 1e-10;
constexpr double kDToCm = 3.33564e-30;

void species(htr_species_t &s, const char *name, double W, int inx, const double H[9],
             const double M[9], const double L[9], int geom, double sigma, double kbOveps,
             double mu, double alpha, double Z298) {
  std::memset(&s, 0, sizeof(s));
  std::strncpy(s.Name, name, sizeof(s.Name) - 1);
  s.W = W;
  s.inx = uint8_t(inx);
  s.cpCoeff.TSwitch1 = 1000.0007f;
  s.cpCoeff.TSwitch2 = 6000.0007f;
  s.cpCoeff.TMin = 200.0000f;
  s.cpCoeff.TMax = 20000.0007f;
  for (int i = 0; i < 9; i++) {
    s.cpCoeff.cpH[i] = H[i];
    s.cpCoeff.cpM[i] = M[i];
    s.cpCoeff.cpL[i] = L[i];
  }
  s.DiffCoeff.Geom = uint8_t(geom);
  s.DiffCoeff.sigma = sigma;
  s.DiffCoeff.kbOveps = kbOveps;
  s.DiffCoeff.mu = mu;
  s.DiffCoeff.alpha = alpha;
  s.DiffCoeff.Z298 = Z298;
}

void arrh(htr_arrhenius_t &a, double A, float n, float EovR) {
  a.A = A;
  a.n = n;
  a.EovR = EovR;
}

thread_local double g_dummy = 0.0;

inline double *at(const htr_field &f, long long x, long long y, long long z) {
  return reinterpret_cast<double *>(static_cast<char *>(f.base) + x * f.stride[0] +
                                    y * f.stride[1] + z * f.stride[2]);
}

}  // namespace

extern "C" {

int htr_constpropmix_init(double gasConstant, double gamma, double prandtl, int viscosityModel,
                          double p0, double p1, double p2, htr_constpropmix_t *out) {
  if (out == nullptr) return HTR_ERR_ARGUMENT;
  std::memset(out, 0, sizeof(*out));
  out->R = gasConstant;
  out->gamma = gamma;
  out->viscosityModel = viscosityModel;
  out->Prandtl = prandtl;
  if (viscosityModel == HTR_VISC_CONSTANT) {
    out->constantVisc = p0;
  } else if (viscosityModel == HTR_VISC_POWERLAW) {
    out->powerlawTempRef = p0;
    out->powerlawViscRef = p1;
  } else if (viscosityModel == HTR_VISC_SUTHERLAND) {
    out->sutherlandSRef = p0;
    out->sutherlandTempRef = p1;
    out->sutherlandViscRef = p2;
  } else {
    return HTR_ERR_ARGUMENT;
  }
  return HTR_OK;
}

int htr_airmix_init(double PRef, double TRef, double LRef, const double XiRef[5], htr_airmix_t *m) {
  if (m == nullptr || XiRef == nullptr || !(PRef > 0) || !(TRef > 0) || !(LRef > 0))
    return HTR_ERR_ARGUMENT;
  std::memset(m, 0, sizeof(*m));
  // --- species: N2, O2, NO, N, O -------------------------------------------
  {
    const double H[9] = {8.310139160e+08, -6.420733540e+05, 2.020264635e+02, -3.065092046e-02,
                         2.486903333e-06, -9.705954110e-11, 1.437538881e-15, 4.938707040e+06,
                         -1.672099740e+03};
    const double M[9] = {5.877124060e+05, -2.239249073e+03, 6.066949220e+00, -6.139685500e-04,
                         1.491806679e-07, -1.923105485e-11, 1.061954386e-15, 1.283210415e+04,
                         -1.586640027e+01};
    const double L[9] = {2.210371497e+04, -3.818461820e+02, 6.082738360e+00, -8.530914410e-03,
                         1.384646189e-05, -9.625793620e-09, 2.519705809e-12, 7.108460860e+02,
                         -1.076003744e+01};
    species(m->species[0], "N2", 2 * 14.0067e-3, 0, H, M, L, 1, 3.621 * kATom, 1.0 / 97.530,
            0.000 * kDToCm, 1.760 * kATom * kATom * kATom, 4.000);
  }
  {
    const double H[9] = {4.975294300e+08, -2.866106874e+05, 6.690352250e+01, -6.169959020e-03,
                         3.016396027e-07, -7.421416600e-12, 7.278175770e-17, 2.293554027e+06,
                         -5.530621610e+02};
    const double M[9] = {-1.037939022e+06, 2.344830282e+03, 1.819732036e+00, 1.267847582e-03,
                         -2.188067988e-07, 2.053719572e-11, -8.193467050e-16, -1.689010929e+04,
                         1.738716506e+01};
    const double L[9] = {-3.425563420e+04, 4.847000970e+02, 1.119010961e+00, 4.293889240e-03,
                         -6.836300520e-07, -2.023372700e-09, 1.039040018e-12, -3.391454870e+03,
                         1.849699470e+01};
    species(m->species[1], "O2", 2 * 15.9994e-3, 1, H, M, L, 1, 3.458 * kATom, 1.0 / 107.40,
            0.000 * kDToCm, 1.600 * kATom * kATom * kATom, 3.8000);
  }
  {
    const double H[9] = {-9.575303540e+08, 5.912434480e+05, -1.384566826e+02, 1.694339403e-02,
                         -1.007351096e-06, 2.912584076e-11, -3.295109350e-16, -4.677501240e+06,
                         1.242081216e+03};
    const double M[9] = {2.239018716e+05, -1.289651623e+03, 5.433936030e+00, -3.656034900e-04,
                         9.880966450e-08, -1.416076856e-11, 9.380184620e-16, 1.750317656e+04,
                         -8.501669090e+00};
    const double L[9] = {-1.143916503e+04, 1.536467592e+02, 3.431468730e+00, -2.668592368e-03,
                         8.481399120e-06, -7.685111050e-09, 2.386797655e-12, 9.098214410e+03,
                         6.728725490e+00};
    species(m->species[2], "NO", 14.0067e-3 + 15.9994e-3, 2, H, M, L, 1, 3.621 * kATom,
            1.0 / 97.530, 0.000 * kDToCm, 1.760 * kATom * kATom * kATom, 4.000);
  }
  {
    const double H[9] = {5.475181050e+08, -3.107574980e+05, 6.916782740e+01, -6.847988130e-03,
                         3.827572400e-07, -1.098367709e-11, 1.277986024e-16, 2.550585618e+06,
                         -5.848769753e+02};
    const double M[9] = {8.876501380e+04, -1.071231500e+02, 2.362188287e+00, 2.916720081e-04,
                         -1.729515100e-07, 4.012657880e-11, -2.677227571e-15, 5.697351330e+04,
                         4.865231506e+00};
    const double L[9] = {0.000000000e+00, 0.000000000e+00, 2.500000000e+00, 0.000000000e+00,
                         0.000000000e+00, 0.000000000e+00, 0.000000000e+00, 5.610463780e+04,
                         4.193905036e+00};
    species(m->species[3], "N", 14.0067e-3, 3, H, M, L, 0, 3.298 * kATom, 1.0 / 71.400,
            0.000 * kDToCm, 0.000 * kATom * kATom * kATom, 0.000);
  }
  {
    const double H[9] = {1.779004264e+08, -1.082328257e+05, 2.810778365e+01, -2.975232262e-03,
                         1.854997534e-07, -5.796231540e-12, 7.191720164e-17, 8.890942630e+05,
                         -2.181728151e+02};
    const double M[9] = {2.619020262e+05, -7.298722030e+02, 3.317177270e+00, -4.281334360e-04,
                         1.036104594e-07, -9.438304330e-12, 2.725038297e-16, 3.392428060e+04,
                         -6.679585350e-01};
    const double L[9] = {-7.953611300e+03, 1.607177787e+02, 1.966226438e+00, 1.013670310e-03,
                         -1.110415423e-06, 6.517507500e-10, -1.584779251e-13, 2.840362437e+04,
                         8.404241820e+00};
    species(m->species[4], "O", 15.9994e-3, 4, H, M, L, 0, 2.750 * kATom, 1.0 / 80.000,
            0.000 * kDToCm, 0.000 * kATom * kATom * kATom, 0.000);
  }
  enum { iN2 = 0, iO2 = 1, iNO = 2, iN = 3, iO = 4 };
  // --- standard reactions: Zeldovich N2 + O <-> NO + N, NO + O <-> O2 + N ----
  {
    htr_reaction_t &r = m->reactions[0];
    arrh(r.ArrCoeff, 6.4e11, -1.0f, 38400.0f);
    r.has_backward = true;
    r.Neducts = 2;
    r.Npducts = 2;
    r.educts[0] = {iN2, 1.0f};
    r.educts[1] = {iO, 1.0f};
    r.pducts[0] = {iNO, 1.0f};
    r.pducts[1] = {iN, 1.0f};
  }
  {
    htr_reaction_t &r = m->reactions[1];
    arrh(r.ArrCoeff, 8.4e6, 0.0f, 19400.0f);
    r.has_backward = true;
    r.Neducts = 2;
    r.Npducts = 2;
    r.educts[0] = {iNO, 1.0f};
    r.educts[1] = {iO, 1.0f};
    r.pducts[0] = {iO2, 1.0f};
    r.pducts[1] = {iN, 1.0f};
  }
  // --- third-body dissociations of O2, NO, N2 ---------------------------------
  {
    htr_tbreaction_t &r = m->ThirdbodyReactions[0];
    arrh(r.ArrCoeff, 2.0e15, -1.5f, 59500.0f);
    r.has_backward = true;
    r.Neducts = 1;
    r.Npducts = 1;
    r.Nthirdb = 5;
    r.educts[0] = {iO2, 1.0f};
    r.pducts[0] = {iO, 2.0f};
    r.thirdb[0] = {iO2, 1.0f};
    r.thirdb[1] = {iNO, 1.0f};
    r.thirdb[2] = {iN2, 1.0f};
    r.thirdb[3] = {iO, 5.0f};
    r.thirdb[4] = {iN, 5.0f};
  }
  {
    htr_tbreaction_t &r = m->ThirdbodyReactions[1];
    arrh(r.ArrCoeff, 5e9, 0.0f, 75500.0f);
    r.has_backward = true;
    r.Neducts = 1;
    r.Npducts = 2;
    r.Nthirdb = 5;
    r.educts[0] = {iNO, 1.0f};
    r.pducts[0] = {iN, 1.0f};
    r.pducts[1] = {iO, 1.0f};
    r.thirdb[0] = {iO2, 1.0f};
    r.thirdb[1] = {iNO, 22.0f};
    r.thirdb[2] = {iN2, 1.0f};
    r.thirdb[3] = {iO, 22.0f};
    r.thirdb[4] = {iN, 22.0f};
  }
  {
    htr_tbreaction_t &r = m->ThirdbodyReactions[2];
    arrh(r.ArrCoeff, 7e15, -1.6f, 113200.0f);
    r.has_backward = true;
    r.Neducts = 1;
    r.Npducts = 1;
    r.Nthirdb = 5;
    r.educts[0] = {iN2, 1.0f};
    r.pducts[0] = {iN, 2.0f};
    r.thirdb[0] = {iO2, 1.0f};
    r.thirdb[1] = {iNO, 1.0f};
    r.thirdb[2] = {iN2, 1.0f};
    r.thirdb[3] = {iO, float(30.0 / 7)};
    r.thirdb[4] = {iN, float(30.0 / 7)};
  }
  // --- reference quantities (MultiComponent.inl:438-487) ---------------------
  m->PRef = PRef;
  m->TRef = TRef;
  double check = 0.0;
  for (int i = 0; i < 5; i++) {
    m->XiRef[i] = 1.0e-60;
    if (XiRef[i] > 0.0) {
      m->XiRef[i] = XiRef[i];
      check += XiRef[i];
    }
  }
  if (std::fabs(check - 1.0) >= 1e-3) return HTR_ERR_ARGUMENT;
  double MixW = 0.0;
  for (int i = 0; i < 5; i++) MixW += m->XiRef[i] * m->species[i].W;
  m->MixWRef = MixW;
  m->iMixWRef = 1.0 / m->MixWRef;
  m->rhoRef = PRef * m->MixWRef / (kRGAS * TRef);
  m->ieRef = m->rhoRef / PRef;
  m->iuRef = std::sqrt(m->ieRef);
  m->iCpRef = m->MixWRef / kRGAS;
  m->imuRef = 1.0 / (LRef * std::sqrt(PRef * m->rhoRef));
  m->ilamRef = m->MixWRef / (LRef * std::sqrt(PRef * m->rhoRef) * kRGAS);
  m->iDiRef = std::sqrt(m->rhoRef / PRef) / (LRef);
  m->iwiRef = LRef / std::sqrt(m->rhoRef * PRef);
  m->iKiRef = std::sqrt(PRef / m->rhoRef) * m->MixWRef / (kNa * LRef * kECrg);
  m->Eps0 = m->MixWRef / (m->rhoRef * kNa * kECrg * LRef);
  m->Eps0 = kEps0 * PRef * m->Eps0 * m->Eps0;
  m->TMax = 1e20;
  m->TMin = 0.0;
  for (int i = 0; i < 5; i++) {
    m->TMax = std::min(m->TMax, m->species[i].cpCoeff.TMax / TRef);
    m->TMin = std::max(m->TMin, m->species[i].cpCoeff.TMin / TRef);
  }
  (void)g_dummy;
  return HTR_OK;
}

// --- SSP-RK3 bookkeeping (prometeo_rk.rg:47-112; coefficients prometeo_const.rg:54-58) --
int htr_InitializeTemporaries(const htr_fluid_view *v, htr_rect3 r, htr_mixture_t mix,
                              htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  const int ne = (mix && htr_mixture_eos(mix) == HTR_EOS_AIRMIX) ? 9 : 5;
#pragma omp parallel for collapse(3)
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        const double *c = at(v->Conserved, i, j, k);
        double *o = at(v->Conserved_old, i, j, k);
        for (int e = 0; e < ne; e++) o[e] = c[e];
      }
  return HTR_OK;
}

int htr_InitializeTimeDerivatives(const htr_fluid_view *v, htr_rect3 r, int implicit,
                                  htr_mixture_t mix, htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  const int ne = (mix && htr_mixture_eos(mix) == HTR_EOS_AIRMIX) ? 9 : 5;
#pragma omp parallel for collapse(3)
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        double *t = at(v->Conserved_t, i, j, k);
        if (implicit) {
          const double *o = at(v->Conserved_t_old, i, j, k);
          for (int e = 0; e < ne; e++) t[e] = -o[e];
        } else {
          for (int e = 0; e < ne; e++) t[e] = 0.0;
        }
      }
  return HTR_OK;
}

int htr_UpdateVars(const htr_fluid_view *v, htr_rect3 r, int stage, double deltaTime,
                   int implicit, htr_mixture_t mix, htr_stream_t) {
  static const double RK[3][3] = {
      {1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
  if (v == nullptr || stage < 1 || stage > 3) return HTR_ERR_ARGUMENT;
  const int ne = (mix && htr_mixture_eos(mix) == HTR_EOS_AIRMIX) ? 9 : 5;
  double dt = deltaTime;
  if (implicit) dt *= 0.5;
  const double c1 = RK[stage - 1][0], c2 = RK[stage - 1][1], c3 = RK[stage - 1][2];
#pragma omp parallel for collapse(3)
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        double *c = at(v->Conserved, i, j, k);
        const double *o = at(v->Conserved_old, i, j, k);
        const double *t = at(v->Conserved_t, i, j, k);
        for (int e = 0; e < ne; e++) c[e] = c1 * o[e] + c2 * c[e] + c3 * t[e] * dt;
      }
  return HTR_OK;
}

}  // extern "C"
