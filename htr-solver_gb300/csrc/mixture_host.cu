// Host side of the mixtures: builders of the reference-compatible mixture
// structs and derivation of the constants the kernels use.
//
// htr_airmix_init carries the 5-species air data of HTR
// (src/Mixtures/AirMix.hpp:58-317: NASA-9 polynomials, Lennard-Jones /
// Stockmayer data, Park-type kinetics) and the reference scales of
// StoreReferenceQuantities (src/Mixtures/MultiComponent.inl:438-487).
#include <cmath>
#include <cstring>

#include "mixture_host.h"

namespace {

constexpr double kPI = 3.1415926535898;
constexpr double kRGAS = 8.3144598;
constexpr double kNa = 6.02214086e23;
constexpr double kKb = 1.38064852e-23;
constexpr double kEps0 = 8.8541878128e-12;
constexpr double kECrg = 1.60217662e-19;
constexpr double kATom = 1e-10;

struct SpeciesData {
  const char *name;
  double W;
  int geom;
  double sigma, kbOveps, mu, alpha, Z298;
  double poly[3][9];  // high, mid, low temperature ranges
};

// N2, O2, NO, N, O
const SpeciesData kAir[5] = {
    {"N2", 2 * 14.0067e-3, 1, 3.621 * kATom, 1.0 / 97.530, 0.0, 1.760 * kATom * kATom * kATom, 4.000,
     {{8.310139160e+08, -6.420733540e+05, 2.020264635e+02, -3.065092046e-02, 2.486903333e-06,
       -9.705954110e-11, 1.437538881e-15, 4.938707040e+06, -1.672099740e+03},
      {5.877124060e+05, -2.239249073e+03, 6.066949220e+00, -6.139685500e-04, 1.491806679e-07,
       -1.923105485e-11, 1.061954386e-15, 1.283210415e+04, -1.586640027e+01},
      {2.210371497e+04, -3.818461820e+02, 6.082738360e+00, -8.530914410e-03, 1.384646189e-05,
       -9.625793620e-09, 2.519705809e-12, 7.108460860e+02, -1.076003744e+01}}},
    {"O2", 2 * 15.9994e-3, 1, 3.458 * kATom, 1.0 / 107.40, 0.0, 1.600 * kATom * kATom * kATom, 3.8000,
     {{4.975294300e+08, -2.866106874e+05, 6.690352250e+01, -6.169959020e-03, 3.016396027e-07,
       -7.421416600e-12, 7.278175770e-17, 2.293554027e+06, -5.530621610e+02},
      {-1.037939022e+06, 2.344830282e+03, 1.819732036e+00, 1.267847582e-03, -2.188067988e-07,
       2.053719572e-11, -8.193467050e-16, -1.689010929e+04, 1.738716506e+01},
      {-3.425563420e+04, 4.847000970e+02, 1.119010961e+00, 4.293889240e-03, -6.836300520e-07,
       -2.023372700e-09, 1.039040018e-12, -3.391454870e+03, 1.849699470e+01}}},
    {"NO", 14.0067e-3 + 15.9994e-3, 1, 3.621 * kATom, 1.0 / 97.530, 0.0, 1.760 * kATom * kATom * kATom, 4.000,
     {{-9.575303540e+08, 5.912434480e+05, -1.384566826e+02, 1.694339403e-02, -1.007351096e-06,
       2.912584076e-11, -3.295109350e-16, -4.677501240e+06, 1.242081216e+03},
      {2.239018716e+05, -1.289651623e+03, 5.433936030e+00, -3.656034900e-04, 9.880966450e-08,
       -1.416076856e-11, 9.380184620e-16, 1.750317656e+04, -8.501669090e+00},
      {-1.143916503e+04, 1.536467592e+02, 3.431468730e+00, -2.668592368e-03, 8.481399120e-06,
       -7.685111050e-09, 2.386797655e-12, 9.098214410e+03, 6.728725490e+00}}},
    {"N", 14.0067e-3, 0, 3.298 * kATom, 1.0 / 71.400, 0.0, 0.0 * kATom * kATom * kATom, 0.0,
     {{5.475181050e+08, -3.107574980e+05, 6.916782740e+01, -6.847988130e-03, 3.827572400e-07,
       -1.098367709e-11, 1.277986024e-16, 2.550585618e+06, -5.848769753e+02},
      {8.876501380e+04, -1.071231500e+02, 2.362188287e+00, 2.916720081e-04, -1.729515100e-07,
       4.012657880e-11, -2.677227571e-15, 5.697351330e+04, 4.865231506e+00},
      {0.0, 0.0, 2.500000000e+00, 0.0, 0.0, 0.0, 0.0, 5.610463780e+04, 4.193905036e+00}}},
    {"O", 15.9994e-3, 0, 2.750 * kATom, 1.0 / 80.000, 0.0, 0.0 * kATom * kATom * kATom, 0.0,
     {{1.779004264e+08, -1.082328257e+05, 2.810778365e+01, -2.975232262e-03, 1.854997534e-07,
       -5.796231540e-12, 7.191720164e-17, 8.890942630e+05, -2.181728151e+02},
      {2.619020262e+05, -7.298722030e+02, 3.317177270e+00, -4.281334360e-04, 1.036104594e-07,
       -9.438304330e-12, 2.725038297e-16, 3.392428060e+04, -6.679585350e-01},
      {-7.953611300e+03, 1.607177787e+02, 1.966226438e+00, 1.013670310e-03, -1.110415423e-06,
       6.517507500e-10, -1.584779251e-13, 2.840362437e+04, 8.404241820e+00}}},
};

enum { iN2 = 0, iO2 = 1, iNO = 2, iN = 3, iO = 4 };

struct ReacData {  // educts / products as (species, nu), colliders as (species, efficiency)
  double A;
  float n, EovR;
  int nEd, ed[2];
  float nuEd[2];
  int nPd, pd[2];
  float nuPd[2];
  int nTb, tb[5];
  float eff[5];
};

// standard reactions (Zeldovich) then third-body dissociations
const ReacData kReac[5] = {
    {6.4e11, -1.0f, 38400.0f, 2, {iN2, iO}, {1.0f, 1.0f}, 2, {iNO, iN}, {1.0f, 1.0f}, 0, {0}, {0}},
    {8.4e6, 0.0f, 19400.0f, 2, {iNO, iO}, {1.0f, 1.0f}, 2, {iO2, iN}, {1.0f, 1.0f}, 0, {0}, {0}},
    {2.0e15, -1.5f, 59500.0f, 1, {iO2, 0}, {1.0f, 0.0f}, 1, {iO, 0}, {2.0f, 0.0f}, 5,
     {iO2, iNO, iN2, iO, iN}, {1.0f, 1.0f, 1.0f, 5.0f, 5.0f}},
    {5e9, 0.0f, 75500.0f, 1, {iNO, 0}, {1.0f, 0.0f}, 2, {iN, iO}, {1.0f, 1.0f}, 5,
     {iO2, iNO, iN2, iO, iN}, {1.0f, 22.0f, 1.0f, 22.0f, 22.0f}},
    {7e15, -1.6f, 113200.0f, 1, {iN2, 0}, {1.0f, 0.0f}, 1, {iN, 0}, {2.0f, 0.0f}, 5,
     {iO2, iNO, iN2, iO, iN}, {1.0f, 1.0f, 1.0f, float(30.0 / 7), float(30.0 / 7)}},
};

}  // namespace

extern "C" int htr_constpropmix_init(double gasConstant, double gamma, double prandtl,
                                     int viscosityModel, double p0, double p1, double p2,
                                     htr_constpropmix_t *out) {
  if (out == nullptr || !(gamma > 1.0) || !(gasConstant > 0.0)) return HTR_ERR_ARGUMENT;
  std::memset(out, 0, sizeof(*out));
  out->R = gasConstant;
  out->gamma = gamma;
  out->Prandtl = prandtl;
  out->viscosityModel = viscosityModel;
  switch (viscosityModel) {
    case HTR_VISC_CONSTANT: out->constantVisc = p0; break;
    case HTR_VISC_POWERLAW:
      out->powerlawTempRef = p0;
      out->powerlawViscRef = p1;
      break;
    case HTR_VISC_SUTHERLAND:
      out->sutherlandSRef = p0;
      out->sutherlandTempRef = p1;
      out->sutherlandViscRef = p2;
      break;
    default: return HTR_ERR_ARGUMENT;
  }
  return HTR_OK;
}

extern "C" int htr_airmix_init(double PRef, double TRef, double LRef, const double XiRef[HTR_AIR_NSPEC],
                               htr_airmix_t *m) {
  if (m == nullptr || XiRef == nullptr || !(PRef > 0) || !(TRef > 0) || !(LRef > 0))
    return HTR_ERR_ARGUMENT;
  std::memset(m, 0, sizeof(*m));
  for (int i = 0; i < 5; i++) {
    const SpeciesData &d = kAir[i];
    htr_species_t &s = m->species[i];
    std::strncpy(s.Name, d.name, sizeof(s.Name) - 1);
    s.W = d.W;
    s.inx = uint8_t(i);
    s.cpCoeff.TSwitch1 = 1000.0007f;
    s.cpCoeff.TSwitch2 = 6000.0007f;
    s.cpCoeff.TMin = 200.0f;
    s.cpCoeff.TMax = 20000.0007f;
    for (int k = 0; k < 9; k++) {
      s.cpCoeff.cpH[k] = d.poly[0][k];
      s.cpCoeff.cpM[k] = d.poly[1][k];
      s.cpCoeff.cpL[k] = d.poly[2][k];
    }
    s.DiffCoeff.Geom = uint8_t(d.geom);
    s.DiffCoeff.sigma = d.sigma;
    s.DiffCoeff.kbOveps = d.kbOveps;
    s.DiffCoeff.mu = d.mu;
    s.DiffCoeff.alpha = d.alpha;
    s.DiffCoeff.Z298 = d.Z298;
  }
  auto fill = [](auto &r, const ReacData &d) {
    r.ArrCoeff.A = d.A;
    r.ArrCoeff.n = d.n;
    r.ArrCoeff.EovR = d.EovR;
    r.has_backward = true;
    r.Neducts = uint8_t(d.nEd);
    r.Npducts = uint8_t(d.nPd);
    for (int i = 0; i < d.nEd; i++) r.educts[i] = {uint8_t(d.ed[i]), d.nuEd[i]};
    for (int i = 0; i < d.nPd; i++) r.pducts[i] = {uint8_t(d.pd[i]), d.nuPd[i]};
  };
  fill(m->reactions[0], kReac[0]);
  fill(m->reactions[1], kReac[1]);
  for (int k = 0; k < 3; k++) {
    htr_tbreaction_t &r = m->ThirdbodyReactions[k];
    fill(r, kReac[2 + k]);
    r.Nthirdb = uint8_t(kReac[2 + k].nTb);
    for (int i = 0; i < r.Nthirdb; i++) r.thirdb[i] = {uint8_t(kReac[2 + k].tb[i]), kReac[2 + k].eff[i]};
  }
  m->PRef = PRef;
  m->TRef = TRef;
  double check = 0.0;
  for (int i = 0; i < 5; i++) {
    m->XiRef[i] = (XiRef[i] > 0.0) ? XiRef[i] : 1.0e-60;
    if (XiRef[i] > 0.0) check += XiRef[i];
  }
  if (std::fabs(check - 1.0) >= 1e-3) return HTR_ERR_ARGUMENT;
  double MixW = 0.0;
  for (int i = 0; i < 5; i++) MixW += m->XiRef[i] * m->species[i].W;
  m->MixWRef = MixW;
  m->iMixWRef = 1.0 / MixW;
  m->rhoRef = PRef * MixW / (kRGAS * TRef);
  m->ieRef = m->rhoRef / PRef;
  m->iuRef = std::sqrt(m->ieRef);
  m->iCpRef = MixW / kRGAS;
  m->imuRef = 1.0 / (LRef * std::sqrt(PRef * m->rhoRef));
  m->ilamRef = MixW / (LRef * std::sqrt(PRef * m->rhoRef) * kRGAS);
  m->iDiRef = std::sqrt(m->rhoRef / PRef) / (LRef);
  m->iwiRef = LRef / std::sqrt(m->rhoRef * PRef);
  m->iKiRef = std::sqrt(PRef / m->rhoRef) * MixW / (kNa * LRef * kECrg);
  const double e0 = MixW / (m->rhoRef * kNa * kECrg * LRef);
  m->Eps0 = kEps0 * PRef * e0 * e0;
  m->TMax = 1e20;
  m->TMin = 0.0;
  for (int i = 0; i < 5; i++) {
    m->TMax = std::fmin(m->TMax, m->species[i].cpCoeff.TMax / TRef);
    m->TMin = std::fmax(m->TMin, m->species[i].cpCoeff.TMin / TRef);
  }
  return HTR_OK;
}

namespace htr {

bool derive(const htr_constpropmix_t &s, ConstPropDev &d) {
  d.R = s.R;
  d.gamma = s.gamma;
  d.Prandtl = s.Prandtl;
  d.visc = s.viscosityModel;
  d.cVisc = s.constantVisc;
  d.plTRef = s.powerlawTempRef;
  d.plVRef = s.powerlawViscRef;
  d.suS = s.sutherlandSRef;
  d.suT = s.sutherlandTempRef;
  d.suV = s.sutherlandViscRef;
  return s.gamma > 1.0 && s.R > 0.0 && s.viscosityModel >= 0 && s.viscosityModel <= 2;
}

bool derive(const htr_airmix_t &s, AirDev &d) {
  std::memset(&d, 0, sizeof(d));
  for (int i = 0; i < 5; i++) {
    const htr_species_t &sp = s.species[i];
    if (!(sp.W > 0.0)) return false;
    d.W[i] = sp.W;
    d.rOvW[i] = kRGAS / sp.W;
    d.TS1[i] = sp.cpCoeff.TSwitch1;
    d.TS2[i] = sp.cpCoeff.TSwitch2;
    std::memcpy(&d.TS1b[i], &d.TS1[i], sizeof(double));
    std::memcpy(&d.TS2b[i], &d.TS2[i], sizeof(double));
    const double *poly[3] = {sp.cpCoeff.cpH, sp.cpCoeff.cpM, sp.cpCoeff.cpL};
    for (int r = 0; r < 3; r++) {
      const double *c = poly[r];
      for (int k = 0; k < 7; k++) d.cp[i][r][k] = c[k];
      const double h[8] = {-c[0], c[1], c[7], c[2], c[3] * 0.50, c[4] / 3, c[5] * 0.25, c[6] / 5};
      for (int k = 0; k < 8; k++) d.hc[i][r][k] = h[k];
      const double g[9] = {-0.5 * c[0], c[1], c[2], c[7], c[8], c[3], c[4] / 3, c[5] / 6, c[6]};
      for (int k = 0; k < 9; k++) d.gc[i][r][k] = g[k];
      const double gf[9] = {g[0], g[1] + g[3], g[1], g[2], g[2] - g[4], 0.5 * g[5], 0.5 * g[6], 0.5 * g[7], 0.05 * g[8]};
      for (int k = 0; k < 9; k++) d.gf[i][r][k] = gf[k];
    }
    d.muNum[i] = kPI * sp.W / kNa * kKb;
    d.muDen[i] = 16 * kPI * std::pow(sp.DiffCoeff.sigma, 2);
    d.kbOveps[i] = sp.DiffCoeff.kbOveps;
    d.geom[i] = sp.DiffCoeff.Geom;
    d.sdDen[i] = 8 * kPI * std::pow(sp.DiffCoeff.sigma, 2);
    d.muC[i] = 5 * std::sqrt(d.muNum[i]) / d.muDen[i];
    d.sdC[i] = 3 * std::sqrt(kPI * kKb * sp.W / kNa) / d.sdDen[i];
    d.isqKbOveps[i] = 1.0 / std::sqrt(sp.DiffCoeff.kbOveps);
    d.iW[i] = 1.0 / sp.W;
    const double tmp = 1.0 / (sp.DiffCoeff.kbOveps * 298);
    const double fz298 = 1 + 0.5 * std::pow(kPI, 1.5) * std::sqrt(tmp) + (2 + 0.25 * kPI * kPI) * tmp +
                         std::pow(kPI, 1.5) * std::pow(tmp, 1.5);
    d.zrot298[i] = sp.DiffCoeff.Z298 * fz298;
    d.fvK[i] = d.sdC[i] / d.muC[i];
    d.iKbOveps[i] = 1.0 / sp.DiffCoeff.kbOveps;
    d.lamMono[i] = 15.0 / 4 * kRGAS / sp.W;
    const double CvROvR = (sp.DiffCoeff.Geom == 1) ? 1.0 : 1.5;
    d.CvRot[i] = CvROvR * kRGAS;
    d.CvVoff[i] = ((sp.DiffCoeff.Geom == 1) ? 3.5 : 4.0) * kRGAS;
    d.lamB0[i] = 2 / kPI * (5. / 3 * CvROvR);
    d.lamK5[i] = 5 * d.CvRot[i] / (kPI * 1.5 * kRGAS);
  }
  d.pi15 = std::pow(kPI, 1.5);
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 5; j++) {
      const htr_ljdata_t &a = s.species[i].DiffCoeff, &b = s.species[j].DiffCoeff;
      d.wilkeA[i][j] = std::pow(s.species[j].W / s.species[i].W, 0.25);
      d.wilkeB[i][j] = std::sqrt(8 * (1 + s.species[i].W / s.species[j].W));
      d.wilkeBi[i][j] = 1.0 / d.wilkeB[i][j];
      // Stockmayer collision parameters (Species.inl:152-181)
      double xi = 1.0;
      if ((a.mu * b.mu == 0.0) && (a.mu + b.mu != 0.0)) {
        const htr_ljdata_t &pol = (a.mu != 0.0) ? a : b, &non = (a.mu != 0.0) ? b : a;
        const double mup = pol.mu / std::sqrt(4 * kPI * kEps0 * kKb * std::pow(pol.sigma, 3) / pol.kbOveps);
        const double alp = non.alpha / std::pow(non.sigma, 3);
        const double epr = std::sqrt(non.kbOveps / pol.kbOveps);
        xi = 1 + 0.25 * mup * alp * epr;
      }
      const double sigmaij = 0.5 * (a.sigma + b.sigma) * std::pow(xi, -1. / 6);
      d.difEps[i][j] = std::sqrt(a.kbOveps * b.kbOveps) / (xi * xi);
      const double Wa = s.species[i].W, Wb = s.species[j].W;
      const double invWij = (Wa + Wb) / (Wa * Wb);
      d.difNum[i][j] = 2 * kPI * std::pow(kKb, 3) * kNa * invWij;
      d.difDen[i][j] = 16 * kPI * sigmaij * sigmaij;
      d.difK[i][j] = d.difDen[i][j] / (3 * std::sqrt(d.difNum[i][j]));
    }
  auto fill = [&](AirReac &r, const htr_arrhenius_t &A, bool bw, int ne, int np, int nt,
                  const htr_stoich_t *ed, const htr_stoich_t *pd, const htr_collider_t *tb) {
    r.A = A.A;
    r.n = A.n;
    r.EovR = A.EovR;
    r.useN = A.n != 0.0f;
    r.useE = std::fabs(A.EovR) > 1e-5f;
    r.backward = bw;
    r.nEd = ne;
    r.nPd = np;
    r.nTb = nt;
    for (int i = 0; i < 2; i++) {
      r.ed[i] = (i < ne) ? ed[i].ind : 0;
      r.nuE[i] = (i < ne) ? ed[i].nu : 0.0f;
      r.pd[i] = (i < np) ? pd[i].ind : 0;
      r.nuP[i] = (i < np) ? pd[i].nu : 0.0f;
    }
    for (int i = 0; i < 5; i++) {
      r.tb[i] = (i < nt) ? tb[i].ind : 0;
      r.effm1[i] = (i < nt) ? double(tb[i].eff) - 1.0 : 0.0;
    }
    for (int i = 0; i < 2; i++) {
      const double nuE = r.nuE[i], nuP = r.nuP[i];
      r.nuEk[i] = nuE == 1.0 ? 1 : (nuE == 2.0 ? 2 : 0);
      r.nuPk[i] = nuP == 1.0 ? 1 : (nuP == 2.0 ? 2 : 0);
    }
    r.sumNu = 0.0;
    for (int i = 0; i < ne; i++) r.sumNu -= double(ed[i].nu);
    for (int i = 0; i < np; i++) r.sumNu += double(pd[i].nu);
  };
  for (int k = 0; k < 2; k++) {
    const htr_reaction_t &r = s.reactions[k];
    if (r.Neducts > 2 || r.Npducts > 2) return false;
    fill(d.reac[k], r.ArrCoeff, r.has_backward, r.Neducts, r.Npducts, 0, r.educts, r.pducts, nullptr);
  }
  for (int k = 0; k < 3; k++) {
    const htr_tbreaction_t &r = s.ThirdbodyReactions[k];
    if (r.Neducts > 2 || r.Npducts > 2 || r.Nthirdb > 5) return false;
    fill(d.reac[2 + k], r.ArrCoeff, r.has_backward, r.Neducts, r.Npducts, r.Nthirdb, r.educts, r.pducts,
         r.thirdb);
  }
  d.TRef = s.TRef;
  d.PRef = s.PRef;
  d.rhoRef = s.rhoRef;
  d.iMixWRef = s.iMixWRef;
  d.ieRef = s.ieRef;
  d.iCpRef = s.iCpRef;
  d.imuRef = s.imuRef;
  d.ilamRef = s.ilamRef;
  d.iDiRef = s.iDiRef;
  d.iwiRef = s.iwiRef;
  d.MixWRef = 1.0 / s.iMixWRef;
  for (int i = 0; i < 5; i++) d.rOvWe[i] = d.rOvW[i] * d.ieRef;
  // double-float copies for TransportDF
  for (int i = 0; i < 5; i++) {
    d.xkbOveps[i] = df_from(d.kbOveps[i]);
    d.xmuC[i] = df_from(d.muC[i]);
    d.xfvK[i] = df_from(d.fvK[i]);
    d.xiKbOveps[i] = df_from(d.iKbOveps[i]);
    d.xisqKbOveps[i] = df_from(d.isqKbOveps[i]);
    d.xzrot298[i] = df_from(d.zrot298[i]);
    d.xlamB0[i] = df_from(d.lamB0[i]);
    d.xlamK5[i] = df_from(d.lamK5[i]);
    d.xlamMono[i] = df_from(d.lamMono[i]);
    d.xCvRot[i] = df_from(d.CvRot[i]);
    d.xCvVoff[i] = df_from(d.CvVoff[i]);
    d.xW[i] = df_from(d.W[i]);
    d.xiW[i] = df_from(d.iW[i]);
    for (int j = 0; j < 5; j++) {
      d.xwilkeA[i][j] = df_from(d.wilkeA[i][j]);
      d.xwilkeBi[i][j] = df_from(d.wilkeBi[i][j]);
      d.xdifEps[i][j] = df_from(d.difEps[i][j]);
      d.xdifK[i][j] = df_from(d.difK[i][j]);
    }
  }
  d.xpi15 = df_from(d.pi15);
  d.xPRef = df_from(d.PRef);
  d.ximuRef = df_from(d.imuRef);
  d.xilamRef = df_from(d.ilamRef);
  d.xiDiRef = df_from(d.iDiRef);
  // range() compares temperatures with the switches as bit patterns
  for (int i = 0; i < 5; i++)
    if (!(d.TS1[i] > 0.0) || !(d.TS2[i] > 0.0)) return false;
  return s.TRef > 0 && s.PRef > 0;
}

}  // namespace htr
