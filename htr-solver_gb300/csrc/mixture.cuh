// Device-side mixture models: thermodynamics, transport and kinetics.
//
// The physics is that of HTR's Mixtures (src/Mixtures/ConstPropMix.inl,
// Species.inl, MultiComponent.inl, Reaction.inl).  Host code
// (mixture.cpp) folds every temperature-independent sub-expression of those
// formulas into the constants below once per loaded mixture, keeping the
// operand order of the reference wherever a value can feed a TENO selection
// flag (enthalpy, heat capacity, the Newton temperature solve, the pressure
// derivatives), so those stay bit-identical to the CPU.
#pragma once

#include "common.cuh"
#include "dfloat.cuh"
#include "fastexp.cuh"

namespace htr {

constexpr double kRGAS = 8.3144598;

// ---------------------------------------------------------------------------
struct ConstPropDev {
  static constexpr int NS = 1;
  static constexpr int NE = 5;
  static constexpr bool kReactive = false;
  double R, gamma, Prandtl;
  int visc;
  double cVisc, plTRef, plVRef, suS, suT, suV;

  HTR_HD double MolarWeightFromYi(const double *) const { return kRGAS / R; }
  HTR_HD double MolarWeightFromXi(const double *) const { return kRGAS / R; }
  HTR_HD void MolarFractions(double *X, double, const double *Y) const { X[0] = Y[0]; }
  HTR_HD void MassFractions(double *Y, double, const double *X) const { Y[0] = X[0]; }
  HTR_HD double RhoFromRhoYi(const double *r) const { return r[0]; }
  HTR_HD void YiFromRhoYi(double *Y, double rho, const double *r) const { Y[0] = r[0] / rho; }
  HTR_HD void ClipYi(double *) const {}
  HTR_HD double Rho(double P, double T, double) const { return P / (R * T); }
  HTR_HD double HeatCapacity(double, const double *) const { return gamma / (gamma - 1) * R; }
  HTR_HD double SpeciesEnthalpy(int, double T) const { return gamma / (gamma - 1) * R * T; }
  HTR_HD double SpeciesMolarWeight(int) const { return kRGAS / R; }
  HTR_HD double InternalEnergy(double T, const double *) const { return T * R / (gamma - 1.0); }
  HTR_HD double TFromInternalEnergy(double e0, double, const double *, int *) const {
    return e0 * (gamma - 1.0) / R;
  }
  HTR_HD double TFromInternalEnergyFast(double e0, double T, const double *Y, int *its) const {
    return TFromInternalEnergy(e0, T, Y, its);
  }
  HTR_HD double TFromRhoAndP(double rho, double MixW, double P) const { return P * MixW / (rho * kRGAS); }
  HTR_HD double PFromRhoAndT(double rho, double MixW, double T) const { return rho * kRGAS * T / MixW; }
  HTR_D double Viscosity(double T, const double *) const {
    if (visc == HTR_VISC_CONSTANT) return cVisc;
    if (visc == HTR_VISC_POWERLAW) return plVRef * pow((T / plTRef), 0.7);
    return (suV * pow((T / suT), 1.5)) * ((suT + suS) / (T + suS));
  }
  HTR_D double HeatConductivity(double T, const double *X) const {
    const double cp = gamma / (gamma - 1) * R;
    return cp / Prandtl * Viscosity(T, X);
  }
  HTR_HD double Gamma(double, double, const double *) const { return gamma; }
  HTR_D double SpeedOfSound(double T, double g, double) const { return sqrt(g * R * T); }
  HTR_HD void Diffusivity(double *D, double, double, double, const double *) const { D[0] = 0.0; }
  HTR_HD void ProductionRates(double *w, double, double, double, const double *) const { w[0] = 0.0; }
  HTR_HD void ProductionRatesRef(double *w, double, double, double, const double *) const { w[0] = 0.0; }
  HTR_HD double dpde(double rho, double g) const { return rho * (g - 1); }
  // temperature, gamma and dp/drho_i of a Roe-averaged state (the Euler flux)
  HTR_D double RoeThermo(double e, double Teos, double MixW, const double *Y, double &gamma_, double *dpdrhoi_) const {
    const double T = TFromInternalEnergy(e, Teos, Y, nullptr);
    gamma_ = Gamma(T, MixW, Y);
    dpdrhoi(dpdrhoi_, gamma_, T, Y);
    return T;
  }
  HTR_HD void dpdrhoi(double *d, double, double T, const double *) const { d[0] = R * T; }
};

// ---------------------------------------------------------------------------
struct AirReac {  // one reaction, standard or third-body
  // The reference stores n, E/R, the stoichiometric coefficients and the
  // collider efficiencies as float; they are kept here promoted to double
  // (exact), so the kernels convert nothing.
  double A, n, EovR;
  double nuE[2], nuP[2];
  double effm1[5];  // efficiency - 1
  double sumNu;     // sum nuP - sum nuE
  int nuEk[2], nuPk[2];  // 1 or 2 where nu is exactly that, else 0 (tested on the integer pipe)
  int nEd, nPd, nTb;
  int ed[2], pd[2], tb[5];
  bool backward;
  bool useN, useE;  // n != 0, |E/R| > 1e-5 (the reference's float tests)
};

struct AirDev {
  static constexpr int NS = 5;
  static constexpr int NE = 9;
  static constexpr bool kReactive = true;
  // species
  double W[NS], rOvW[NS];  // rOvW = RGAS/W
  double rOvWe[NS];        // rOvW * ieRef
  double TS1[NS], TS2[NS]; // NASA range switches (the reference's floats, promoted)
  long long TS1b[NS], TS2b[NS];  // their bit patterns (range)
  double cp[NS][3][7];   // NASA coefficients c0..c6 per range (0 high, 1 mid, 2 low)
  double hc[NS][3][8];   // enthalpy: -c0, c1, c7, c2, c3*0.50, c4/3, c5*0.25, c6/5
  double gc[NS][3][9];   // free enthalpy: -0.5*c0, c1, c2, c7, c8, c3, c4/3, c5/6, c6
  double gf[NS][3][9];   // the same regrouped (FreeEnthalpyFast): g0, g1+g3, g1, g2, g2-g4, g5/2, g6/2, g7/2, g8/20
  // transport (T-independent factors of Species.inl:145-351, MultiComponent.inl:231-311)
  double muNum[NS];      // PI*W/Na*kb  (mu numerator is 5*sqrt(muNum*T))
  double muDen[NS];      // 16*PI*sigma^2
  double muC[NS];        // 5*sqrt(muNum)/muDen:  mu_i = muC * sqrt(T) / omega_mu
  double kbOveps[NS];
  double isqKbOveps[NS]; // 1/sqrt(kbOveps)
  double iW[NS];         // 1/W
  int geom[NS];
  double sdDen[NS];      // 8*PI*sigma^2 (self diffusion denominator)
  double sdC[NS];        // 3*sqrt(PI*kb*W/Na)/sdDen:  Dkk = sdC * sqrt(T) / omega_D
  double zrot298[NS];    // Z298*FZrot(298)
  double pi15;           // PI^1.5
  double wilkeA[NS][NS]; // (W_j/W_i)^0.25
  double wilkeB[NS][NS]; // sqrt(8*(1 + W_i/W_j))
  double wilkeBi[NS][NS];// 1/wilkeB
  double difNum[NS][NS]; // 2*PI*kb^3*Na*invWij  (num = 3*sqrt(difNum*T^3))
  double difDen[NS][NS]; // 16*PI*sigma_ij^2
  double difK[NS][NS];   // difDen/(3*sqrt(difNum)):  1/D_ij = difK * P * omega_D / T^1.5
  double difEps[NS][NS]; // kb/eps_ij
  // factors of the fused property refresh (TransportFast)
  double fvK[NS];        // sdC/muC:  Dkk/mu_k = fvK * omega_mu / omega_D
  double iKbOveps[NS];   // 1/kbOveps
  double lamMono[NS];    // 15/4 R/W (monatomic conductivity / viscosity)
  double CvRot[NS];      // CvROvR R
  double CvVoff[NS];     // 3.5 R (linear) or 4 R (non-linear)
  double lamB0[NS];      // 2/PI * 5/3 * CvROvR
  double lamK5[NS];      // 5 CvR / (PI CvT)
  // double-float copies of the transport factors (TransportDF)
  dfloat xkbOveps[NS], xmuC[NS], xfvK[NS], xiKbOveps[NS], xisqKbOveps[NS], xzrot298[NS], xlamB0[NS],
      xlamK5[NS], xlamMono[NS], xCvRot[NS], xCvVoff[NS], xW[NS], xiW[NS];
  dfloat xwilkeA[NS][NS], xwilkeBi[NS][NS], xdifEps[NS][NS], xdifK[NS][NS];
  dfloat xpi15, xPRef, ximuRef, xilamRef, xiDiRef;
  // kinetics (2 standard + 3 third-body)
  AirReac reac[5];
  // reference scales
  double TRef, PRef, rhoRef, iMixWRef, ieRef, iCpRef, imuRef, ilamRef, iDiRef, iwiRef;
  double MixWRef;  // 1 / iMixWRef

  // T > TS2 ? 0 : (T > TS1 ? 1 : 2), compared on the integer pipe: the bit
  // patterns of doubles order like their values when the switch
  // temperatures are positive (a negative T is below both, as compared in
  // double)
  HTR_HD int range(int i, double T) const {
    const long long b = (long long)df_bits(T);
    return (b > TS2b[i]) ? 0 : ((b > TS1b[i]) ? 1 : 2);
  }

  // Species.inl:84-101
  HTR_D double Cp(int i, double T, double Tinv) const {
    const double *c = cp[i][range(i, T)];
    return rOvW[i] * (c[0] * Tinv * Tinv + c[1] * Tinv + c[2] +
                      T * (c[3] + T * (c[4] + T * (c[5] + T * c[6]))));
  }
  // Species.inl:125-143 (logT = log(T), Tinv = 1/T)
  HTR_D double Enthalpy(int i, double T, double Tinv, double logT) const {
    const double *c = hc[i][range(i, T)];
    const double E = c[0] * Tinv + c[1] * logT + c[2] + T * (c[3] + T * (c[4] + T * (c[5] + T * (c[6] + c[7] * T))));
    return E * rOvW[i];
  }
  // Species.inl:103-123
  HTR_D double FreeEnthalpy(int i, double T, double Tinv, double logT) const {
    const double *c = gc[i][range(i, T)];
    const double G = c[0] * Tinv * Tinv + c[1] * Tinv * (1.0 + logT) + c[2] * (1.0 - logT) + c[3] * Tinv - c[4];
    return G - 0.5 * T * (c[5] + T * (c[6] + T * (c[7] + 0.1 * T * c[8])));
  }

  // The same free enthalpy with its T-independent combinations folded on the
  // host: G = Tinv (g0 Tinv + g1 + g3) + logT (g1 Tinv - g2) + (g2 - g4)
  //         - T (g5/2 + T (g6/2 + T (g7/2 + T g8/20)))
  // (nine operations; the explicit chemistry sources)
  HTR_D double FreeEnthalpyFast(int i, double T, double Tinv, double logT) const {
    const double *c = gf[i][range(i, T)];
    const double a = fma(c[0], Tinv, c[1]) * Tinv;
    const double b = fma(fma(c[2], Tinv, -c[3]), logT, a) + c[4];
    const double q = fma(fma(fma(c[8], T, c[7]), T, c[6]), T, c[5]);
    return fma(-T, q, b);
  }

  HTR_HD void ClipYi(double *Y) const {
#pragma unroll
    for (int i = 0; i < NS; i++) {
      Y[i] = smax(Y[i], 1e-60);
      Y[i] = smin(Y[i], 1.0);
    }
  }
  HTR_HD double MolarWeightFromYi(const double *Y) const {
    double w = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) w += Y[i] / W[i];
    return 1.0 / w;
  }
  HTR_HD double MolarWeightFromXi(const double *X) const {
    double w = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) w += X[i] * W[i];
    return w;
  }
  HTR_HD void MolarFractions(double *X, double MixW, const double *Y) const {
#pragma unroll
    for (int i = 0; i < NS; i++) X[i] = Y[i] * MixW / W[i];
  }
  HTR_HD void MassFractions(double *Y, double MixW, const double *X) const {
#pragma unroll
    for (int i = 0; i < NS; i++) Y[i] = X[i] * W[i] / MixW;
  }
  HTR_HD double RhoFromRhoYi(const double *r) const {
    double rho = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) rho += r[i];
    return rho;
  }
  HTR_HD void YiFromRhoYi(double *Y, double rho, const double *r) const {
    const double irho = 1.0 / rho;
#pragma unroll
    for (int i = 0; i < NS; i++) Y[i] = irho * r[i];
  }
  HTR_HD double Rho(double P, double T, double MixW) const { return P * MixW * iMixWRef / T; }
  HTR_D double HeatCapacity(double Tn, const double *Y) const {
    const double T = Tn * TRef;
    const double Tinv = 1.0 / T;
    double c = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) c += Y[i] * Cp(i, T, Tinv);
    return c * iCpRef;
  }
  HTR_D double SpeciesEnthalpy(int i, double Tn) const {
    const double T = Tn * TRef;
    return Enthalpy(i, T, 1.0 / T, log(T)) * ieRef;
  }
  // nondimensional species enthalpies at T (dimensional) with 1/T and log T
  // supplied (R/W and the energy scale folded into one factor)
  HTR_D void SpeciesEnthalpiesAt(double *h, double T, double Tinv, double logT) const {
#pragma unroll
    for (int i = 0; i < NS; i++) {
      const double *c = hc[i][range(i, T)];
      h[i] = (c[0] * Tinv + c[1] * logT + c[2] + T * (c[3] + T * (c[4] + T * (c[5] + T * (c[6] + c[7] * T))))) *
             rOvWe[i];
    }
  }
  HTR_D void SpeciesEnthalpies(double *h, double Tn) const {
    const double T = Tn * TRef;
    const double Tinv = 1.0 / T, logT = log(T);
#pragma unroll
    for (int i = 0; i < NS; i++) h[i] = Enthalpy(i, T, Tinv, logT) * ieRef;
  }
  HTR_HD double SpeciesMolarWeight(int i) const { return W[i]; }
  HTR_D double InternalEnergy(double Tn, const double *Y) const {
    const double T = Tn * TRef;
    const double Tinv = 1.0 / T, logT = log(T);
    double e = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) e += Y[i] * (Enthalpy(i, T, Tinv, logT) - kRGAS * T / W[i]);
    return e * ieRef;
  }
  // MultiComponent.inl:188-209; *its (optional) receives the iteration count.
  HTR_D double TFromInternalEnergy(double e0, double T, const double *Y, int *its) const {
    const int MAXITS = 1000;
    const double TOL = 1e-8;
    double dfdT = 1.0;
    int j = 0;
    for (; j < MAXITS; j++) {
      const double f = e0 - InternalEnergy(T, Y);
      if (fabs(f / dfdT) < TOL) break;
      dfdT = 0.0;
      const double Td = T * TRef;
      const double Tinv = 1.0 / Td;
#pragma unroll
      for (int i = 0; i < NS; i++) dfdT += Y[i] * (Cp(i, Td, Tinv) - kRGAS / W[i]) * iCpRef;
      T += f / dfdT;
    }
    if (its) *its = j;
    return T;
  }
  HTR_HD double TFromRhoAndP(double rho, double MixW, double P) const { return P * MixW * iMixWRef / rho; }
  HTR_HD double PFromRhoAndT(double rho, double MixW, double T) const { return rho * T / (MixW * iMixWRef); }
  HTR_D double Gamma(double T, double MixW, const double *Y) const {
    const double c = HeatCapacity(T, Y);
    const double Wr = MixW * iMixWRef;
    return c / (c - 1.0 / Wr);
  }
  HTR_D double SpeedOfSound(double T, double g, double MixW) const { return sqrt(g * T / (MixW * iMixWRef)); }
  HTR_HD double dpde(double rho, double g) const { return rho * (g - 1); }
  HTR_D void dpdrhoi(double *d, double g, double Tn, const double *Y) const {
    const double T = Tn * TRef;
    const double Tinv = 1.0 / T, logT = log(T);
    double e = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
      d[i] = Enthalpy(i, T, Tinv, logT) - kRGAS * T / W[i];
      e += Y[i] * d[i];
    }
#pragma unroll
    for (int i = 0; i < NS; i++) d[i] = (kRGAS * T / W[i] + (g - 1) * (e - d[i])) * ieRef;
  }

  // The reference's Newton for T from e with the fused species h and c_p
  // (the task kernels' primitive recovery)
  HTR_D double TFromInternalEnergyFast(double e0, double T, const double *Y, int *its) const {
    double cpk[NS], Td, Tinv, logT;
    return TFromInternalEnergyCp(e0, T, Y, its, cpk, Td, Tinv, logT);
  }
  // Temperature, gamma and dp/drho_i of a Roe-averaged state (the Euler
  // flux, rhs.inl:198-279): the reference's Newton from Teos
  // (TFromInternalEnergy: same start, tolerance and test) evaluated with the
  // fused species h and c_p of TFromInternalEnergyCp, whose values at the
  // returned temperature then give gamma (HeatCapacity) and dp/drho_i
  // (dpdrhoi) without evaluating them again.
  HTR_D double RoeThermo(double e, double Teos, double MixW, const double *Y, double &gamma_,
                         double *dpdrhoi_) const {
    double cpk[NS], h[NS], Td, Tinv, logT;
    const double T = TFromInternalEnergyCp(e, Teos, Y, nullptr, cpk, Td, Tinv, logT, false, nullptr, nullptr, h);
    double c = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) c += Y[i] * cpk[i];
    c *= iCpRef;
    gamma_ = c / (c - 1.0 / (MixW * iMixWRef));
    double ed = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
      dpdrhoi_[i] = h[i] - rOvW[i] * Td;
      ed += Y[i] * dpdrhoi_[i];
    }
#pragma unroll
    for (int i = 0; i < NS; i++) dpdrhoi_[i] = (rOvW[i] * Td + (gamma_ - 1) * (ed - dpdrhoi_[i])) * ieRef;
    return T;
  }

  // --- transport (Species.inl:145-351, MultiComponent.inl:231-311) ----------
  // rational fits as numerator / denominator pairs (one division saved per use)
  static HTR_D void omega_mu_nd(double T, double &n, double &d) {
    n = 3.3530622607 + T * (2.53272006 + T * (2.9024238575 + T * 0.11186138893));
    d = 0.8662326188 + T * (1.3913958626 + T * (3.158490576 + T * (0.18973411754 + T * 0.00018682962894)));
  }
  static HTR_D void omega_D_nd(double T, double &n, double &d) {
    n = 6.8728271691 + T * (9.4122316321 + T * (7.7442359037 + T * 0.23424661229));
    d = 1.45337701568 + T * (5.2269794238 + T * (9.7108519575 + T * (0.46539437353 + T * 0.00041908394781)));
  }
  // --- fused per-cell refresh (the update kernel of the fused stage) -------
  // The same physics as TFromInternalEnergy / Transport / HeatCapacity, with
  // the arithmetic regrouped for fewer FP64 operations: species enthalpies
  // and heat capacities share 1/T and the range lookup, the Newton loop keeps
  // the species c_p of its final temperature for the property refresh, and
  // transport replaces its ~50 divisions by a few batched inversions.
  // Results differ from the reference's operation order by rounding only.

  // Species enthalpies and heat capacities (mass units) at T (dimensional).
  HTR_D void EnthalpyCp(double T, double Tinv, double logT, double *h, double *cpk) const {
#pragma unroll
    for (int i = 0; i < NS; i++) {
      const int r = range(i, T);
      const double *a = hc[i][r];
      const double *c = cp[i][r];
      h[i] = (a[0] * Tinv + a[1] * logT + a[2] +
              T * (a[3] + T * (a[4] + T * (a[5] + T * (a[6] + a[7] * T))))) * rOvW[i];
      cpk[i] = rOvW[i] * (c[0] * Tinv * Tinv + c[1] * Tinv + c[2] +
                          T * (c[3] + T * (c[4] + T * (c[5] + T * c[6]))));
    }
  }
  // Newton for T from e (MultiComponent.inl:188-209: same tolerance, cap and
  // convergence test).  On return cpk holds the species c_p at the returned
  // temperature, Td = T * TRef and Tinv = 1 / Td.
  // With `have`, Td = T * TRef, Tinv and logT = log(Td) of the initial T are
  // supplied; later iterates take log T from the previous one through a
  // log1p series when they moved by less than 2^-10 (|r|^7/7 < 1e-22).
  // With h0 / cp0, the species enthalpies and heat capacities at the initial
  // T (computed by the previous refresh that ended on this very T) replace
  // its evaluation; hout (optional) receives the enthalpies at the returned T.
  HTR_D double TFromInternalEnergyCp(double e0, double T, const double *Y, int *its, double *cpk,
                                     double &Td, double &Tinv, double &logT, bool have = false,
                                     const double *h0 = nullptr, const double *cp0 = nullptr,
                                     double *hout = nullptr) const {
    const int MAXITS = 1000;
    const double TOL = 1e-8;
    double dfdT = 1.0, h[NS];
    int j = 0;
    if (!have) {
      Td = T * TRef;
      Tinv = 1.0 / Td;
      logT = log(Td);
    }
    for (; j < MAXITS; j++) {
      if (j > 0) {
        const double Tn = T * TRef;
        const double r = (Tn - Td) * Tinv;
        if (fabs(r) < 0.0009765625) {
          logT += r * (1.0 + r * (-0.5 + r * (1.0 / 3 + r * (-0.25 + r * (0.2 + r * (-1.0 / 6))))));
          // 1/(T (1 + r)) = (1/T) (1 - r + r^2 - ... - r^5), remainder below 2^-60
          Tinv *= 1.0 + r * (-1.0 + r * (1.0 + r * (-1.0 + r * (1.0 - r))));
        } else {
          logT = log(Tn);
          Tinv = 1.0 / Tn;
        }
        Td = Tn;
      }
      if (j == 0 && h0 != nullptr) {
#pragma unroll
        for (int i = 0; i < NS; i++) {
          h[i] = h0[i];
          cpk[i] = cp0[i];
        }
      } else {
        EnthalpyCp(Td, Tinv, logT, h, cpk);
      }
      double e = 0.0;
#pragma unroll
      for (int i = 0; i < NS; i++) e += Y[i] * (h[i] - rOvW[i] * Td);
      const double f = e0 - e * ieRef;
      // |f / dfdT| < TOL without the division (dfdT, a heat capacity, is
      // positive)
      if (fabs(f) < TOL * dfdT) break;
      double d = 0.0;
#pragma unroll
      for (int i = 0; i < NS; i++) d += Y[i] * (cpk[i] - rOvW[i]);
      dfdT = d * iCpRef;
      T += f / dfdT;
    }
    if (j == MAXITS) {
      Td = T * TRef;
      Tinv = 1.0 / Td;
      logT = log(Td);
      EnthalpyCp(Td, Tinv, logT, h, cpk);
    }
    if (hout != nullptr) {
#pragma unroll
      for (int i = 0; i < NS; i++) hout[i] = h[i];
    }
    if (its) *its = j;
    return T;
  }
  // Viscosity, conductivity, diffusivities (Species.inl:145-351,
  // MultiComponent.inl:231-311) at T = Td with 1/T = Tinv, species c_p given.
  HTR_D void TransportFast(double Td, double Tinv, double Pn, double MixW, const double *X,
                           const double *cpk, double &mu, double &lam, double *D) const {
    const double T = Td;
    const double P = Pn * PRef;
    const double isT = rsqrt(T);
    const double sT = T * isT;
    double nmu[NS], dmu[NS], nD[NS], dD[NS], inv1[2 * NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      omega_mu_nd(T * kbOveps[i], nmu[i], dmu[i]);
      inv1[i] = nmu[i];
      if (geom[i] != 0) {
        omega_D_nd(T * kbOveps[i], nD[i], dD[i]);
        inv1[NS + i] = nD[i] * dmu[i];
      } else {
        nD[i] = dD[i] = 1.0;
        inv1[NS + i] = 1.0;
      }
    }
    batch_inverse<2 * NS>(inv1);
    double muk[NS], smu[NS], ismu[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      muk[i] = muC[i] * sT * dmu[i] * inv1[i];
      ismu[i] = rsqrt(muk[i]);
      smu[i] = muk[i] * ismu[i];
    }
    // Wilke denominators (Phi_ii = 1 exactly) and the rotational relaxation
    // denominators of the polyatomic species, inverted together
    double inv2[2 * NS], fV[NS], fz[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      double den = X[i];
#pragma unroll
      for (int j = 0; j < NS; j++) {
        if (j == i) continue;
        double Phi = 1 + smu[i] * ismu[j] * wilkeA[i][j];
        Phi *= Phi * wilkeBi[i][j];
        den += X[j] * Phi;
      }
      inv2[i] = den;
      if (geom[i] != 0) {
        fV[i] = fvK[i] * dD[i] * nmu[i] * inv1[NS + i];  // Dkk / mu_k
        const double tmp = Tinv * iKbOveps[i];
        const double st = isT * isqKbOveps[i];
        fz[i] = 1 + 0.5 * pi15 * st + (2 + 0.25 * 3.1415926535898 * 3.1415926535898) * tmp + pi15 * (tmp * st);
        inv2[NS + i] = zrot298[i] + fz[i] * (lamB0[i] + (2 / 3.1415926535898) * fV[i]);
      } else {
        fV[i] = fz[i] = 0.0;
        inv2[NS + i] = 1.0;
      }
    }
    batch_inverse<2 * NS>(inv2);
    double m = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) m += X[i] * muk[i] * inv2[i];
    mu = m * imuRef;
    // species conductivities; lam = (sum X l + 1 / sum X/l) / 2 with the
    // second sum taken over a common denominator (one division)
    double l[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      if (geom[i] == 0) {
        l[i] = muk[i] * lamMono[i];
      } else {
        const double CvT = 1.5 * kRGAS;
        const double CvV = cpk[i] * W[i] - CvVoff[i];
        const double AiB = (2.5 - fV[i]) * fz[i] * inv2[NS + i];  // A / B
        const double fT = 2.5 - lamK5[i] * AiB;
        const double fR = fV[i] * (1. + (2 / 3.1415926535898) * AiB);
        l[i] = muk[i] * iW[i] * (fT * CvT + fR * CvRot[i] + fV[i] * CvV);
      }
    }
    double a = 0.0, pre[NS], suf[NS];
    pre[0] = 1.0;
#pragma unroll
    for (int i = 1; i < NS; i++) pre[i] = pre[i - 1] * l[i - 1];
    suf[NS - 1] = 1.0;
#pragma unroll
    for (int i = NS - 2; i >= 0; i--) suf[i] = suf[i + 1] * l[i + 1];
    double sx = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
      a += X[i] * l[i];
      sx += X[i] * (pre[i] * suf[i]);
    }
    lam = 0.5 * (a + pre[NS - 1] * l[NS - 1] / sx) * ilamRef;
    // binary diffusion coefficients, inverted together
    const double PisT3 = P * Tinv * isT;  // P / T^1.5
    double nb[NS * (NS - 1) / 2], db[NS * (NS - 1) / 2];
    {
      int k = 0;
#pragma unroll
      for (int i = 0; i < NS; i++)
#pragma unroll
        for (int j = 0; j < i; j++, k++) omega_D_nd(T * difEps[i][j], nb[k], db[k]);
    }
    batch_inverse<NS * (NS - 1) / 2>(db);
    double Ds[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) Ds[i] = 0.0;
    {
      int k = 0;
#pragma unroll
      for (int i = 0; i < NS; i++)
#pragma unroll
        for (int j = 0; j < i; j++, k++) {
          const double inv = difK[i][j] * PisT3 * nb[k] * db[k];  // 1 / D_ij
          Ds[i] += X[j] * inv;
          Ds[j] += X[i] * inv;
        }
    }
    double den[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) den[i] = MixW * Ds[i];
    batch_inverse<NS>(den);
#pragma unroll
    for (int i = 0; i < NS; i++) {
      double num = 0.0;
#pragma unroll
      for (int j = 0; j < NS; j++)
        if (j != i) num += X[j] * W[j];
      D[i] = num * den[i] * iDiRef;
    }
  }

  // The same viscosity, conductivity and diffusivities in double-float
  // arithmetic (dfloat.cuh) on the FP32 pipe, whose rate on this part is
  // ~70 times the FP64 rate: every factor is a T- or pair-dependent quantity
  // of bounded range, so about 48 significant bits carry the formulas of
  // TransportFast to a relative error of a few 1e-14 (measured), against the
  // 1e-11 bar.  Inputs and outputs cross between double and double-float on
  // the integer pipe.  Mole fractions below 2^-74 lose bits and below 2^-126
  // vanish; their terms are negligible in every sum as long as each
  // species' diffusion partner sum keeps a partner of mole fraction >= 1e-20,
  // i.e. at least two species have such a mole fraction.  A (near) pure
  // mixture takes the FP64 TransportFast.
  // Horner with positive coefficients at t > 0: every partial sum adds
  // operands of one sign
  static HTR_D dfloat df_poly(dfloat t, const dfloat *c, int n) {
    dfloat r = c[n - 1];
    for (int k = n - 2; k >= 0; k--) r = df_add_same(df_mul(r, t), c[k]);
    return r;
  }
  // omega_mu and omega_D as numerator / denominator (the fits of
  // Species.inl:198-239; constants split at compile time)
  static HTR_D void omega_mu_df(dfloat t, dfloat &n, dfloat &d) {
    const dfloat cn[4] = {HTR_DF_CONST(3.3530622607), HTR_DF_CONST(2.53272006), HTR_DF_CONST(2.9024238575),
                          HTR_DF_CONST(0.11186138893)};
    const dfloat cd[5] = {HTR_DF_CONST(0.8662326188), HTR_DF_CONST(1.3913958626), HTR_DF_CONST(3.158490576),
                          HTR_DF_CONST(0.18973411754), HTR_DF_CONST(0.00018682962894)};
    n = df_poly(t, cn, 4);
    d = df_poly(t, cd, 5);
  }
  static HTR_D void omega_D_df(dfloat t, dfloat &n, dfloat &d) {
    const dfloat cn[4] = {HTR_DF_CONST(6.8728271691), HTR_DF_CONST(9.4122316321), HTR_DF_CONST(7.7442359037),
                          HTR_DF_CONST(0.23424661229)};
    const dfloat cd[5] = {HTR_DF_CONST(1.45337701568), HTR_DF_CONST(5.2269794238), HTR_DF_CONST(9.7108519575),
                          HTR_DF_CONST(0.46539437353), HTR_DF_CONST(0.00041908394781)};
    n = df_poly(t, cn, 4);
    d = df_poly(t, cd, 5);
  }
  HTR_D void TransportDF(double Td, double Tinv_d, double Pn, double MixW_d, const double *X,
                         const double *cpk, double &mu, double &lam, double *D) const {
    // mole fractions are non-negative: their bit patterns order like them
    const unsigned long long kTiny = 0x3bc79ca10c924223ULL;  // 1e-20
    int big = 0;
#pragma unroll
    for (int i = 0; i < NS; i++) big += (df_bits(X[i]) >= kTiny) ? 1 : 0;
    if (big < 2) {
      TransportFast(Td, Tinv_d, Pn, MixW_d, X, cpk, mu, lam, D);
      return;
    }
    const dfloat T = df_from_bits(Td);
    const dfloat Tinv = df_from_bits(Tinv_d);
    const dfloat sT = df_sqrt(T);
    const dfloat isT = df_rcp(sT);
    const dfloat P = df_mul(df_from_bits(Pn), xPRef);
    dfloat x[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) x[i] = df_from_bits(X[i]);
    // species viscosities and the collision integrals of self diffusion
    dfloat muk[NS], smu[NS], ismu[NS], nmu[NS], dmu[NS], nD[NS], dD[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      const dfloat ts = df_mul(T, xkbOveps[i]);
      omega_mu_df(ts, nmu[i], dmu[i]);
      muk[i] = df_div(df_mul(df_mul(xmuC[i], sT), dmu[i]), nmu[i]);
      smu[i] = df_sqrt(muk[i]);
      ismu[i] = df_rcp(smu[i]);
      if (geom[i] != 0) {
        omega_D_df(ts, nD[i], dD[i]);
      } else {
        nD[i] = dD[i] = df_from(1.0f);
      }
    }
    // Wilke's mixing rule (Phi_ii = 1)
    dfloat m = df_from(0.0f);
#pragma unroll
    for (int i = 0; i < NS; i++) {
      dfloat den = x[i];
#pragma unroll
      for (int j = 0; j < NS; j++) {
        if (j == i) continue;
        dfloat phi = df_add(df_mul(df_mul(smu[i], ismu[j]), xwilkeA[i][j]), 1.0f);
        phi = df_mul(df_mul(phi, phi), xwilkeBi[i][j]);
        den = df_add_same(den, df_mul(x[j], phi));
      }
      m = df_add_same(m, df_div(df_mul(x[i], muk[i]), den));
    }
    mu = df_to_double_bits(df_mul(m, ximuRef));
    // species conductivities (Eucken with the rotational and vibrational
    // relaxation of the polyatomic species) and the mixing rule
    // lam = (sum X l + 1 / sum X / l) / 2
    const dfloat twoOvPi = HTR_DF_CONST(2 / 3.1415926535898);
    const dfloat fzK = HTR_DF_CONST(2 + 0.25 * 3.1415926535898 * 3.1415926535898);
    const dfloat CvT = HTR_DF_CONST(1.5 * kRGAS);
    dfloat a = df_from(0.0f), sxl = df_from(0.0f);
#pragma unroll
    for (int i = 0; i < NS; i++) {
      dfloat l;
      if (geom[i] == 0) {
        l = df_mul(muk[i], xlamMono[i]);
      } else {
        const dfloat fV = df_div(df_mul(df_mul(xfvK[i], nmu[i]), dD[i]), df_mul(dmu[i], nD[i]));  // Dkk / mu_k
        const dfloat tmp = df_mul(Tinv, xiKbOveps[i]);
        const dfloat st = df_mul(isT, xisqKbOveps[i]);
        const dfloat hp = df_mul(xpi15, st);
        dfloat fz = df_add(df_mul(hp, 0.5f), 1.0f);
        fz = df_add_same(fz, df_mul(fzK, tmp));
        fz = df_add_same(fz, df_mul(hp, tmp));
        const dfloat Bd = df_add_same(xzrot298[i], df_mul(fz, df_add_same(xlamB0[i], df_mul(twoOvPi, fV))));
        const dfloat AiB = df_div(df_mul(df_add(df_neg(fV), 2.5f), fz), Bd);  // A / B
        const dfloat fT = df_add(df_neg(df_mul(xlamK5[i], AiB)), 2.5f);
        const dfloat fR = df_mul(fV, df_add(df_mul(twoOvPi, AiB), 1.0f));
        const dfloat CvV = df_sub(df_mul(df_from_bits(cpk[i]), xW[i]), xCvVoff[i]);
        const dfloat s = df_add(df_add(df_mul(fT, CvT), df_mul(fR, xCvRot[i])), df_mul(fV, CvV));
        l = df_mul(df_mul(muk[i], xiW[i]), s);
      }
      a = df_add_same(a, df_mul(x[i], l));
      sxl = df_add_same(sxl, df_div(x[i], l));
    }
    lam = df_to_double_bits(df_mul(df_mul(df_add_same(a, df_rcp(sxl)), 0.5f), xilamRef));
    // binary diffusion coefficients: 1 / D_ij = difK P omega_D(T kb/eps_ij) / T^1.5
    const dfloat PisT3 = df_mul(df_mul(P, Tinv), isT);
    dfloat Ds[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) Ds[i] = df_from(0.0f);
#pragma unroll
    for (int i = 0; i < NS; i++)
#pragma unroll
      for (int j = 0; j < i; j++) {
        dfloat nb, db;
        omega_D_df(df_mul(T, xdifEps[i][j]), nb, db);
        const dfloat inv = df_div(df_mul(df_mul(xdifK[i][j], PisT3), nb), db);
        Ds[i] = df_add_same(Ds[i], df_mul(x[j], inv));
        Ds[j] = df_add_same(Ds[j], df_mul(x[i], inv));
      }
    const dfloat MixW = df_from_bits(MixW_d);
#pragma unroll
    for (int i = 0; i < NS; i++) {
      dfloat num = df_from(0.0f);
#pragma unroll
      for (int j = 0; j < NS; j++)
        if (j != i) num = df_add_same(num, df_mul(x[j], xW[j]));
      D[i] = df_to_double_bits(df_mul(df_div(num, df_mul(MixW, Ds[i])), xiDiRef));
    }
  }

  // TransportDF at a nondimensional temperature and pressure whose species
  // heat capacities are not at hand (the task kernels' property refresh)
  HTR_D void TransportAt(double Tn, double Pn, double MixW, const double *X, double &mu, double &lam,
                         double *D) const {
    const double Td = Tn * TRef, Tinv = 1.0 / Td;
    double cpk[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) cpk[i] = Cp(i, Td, Tinv);
    TransportDF(Td, Tinv, Pn, MixW, X, cpk, mu, lam, D);
  }

  // --- kinetics (Reaction.inl, MultiComponent.inl:370-415) ------------------
  // The reference's own operation order and function calls (pow, exp of
  // -E/RT, the backward rate through exp(-ln Kc), concentrations Y rho / W),
  // for the implicit solver: its adaptive step control amplifies any
  // difference of rounding into a different sequence of steps, so the
  // right-hand side it integrates is evaluated as the reference evaluates it
  // (in a translation unit without FMA contraction).
  HTR_D void ProductionRatesRef(double *w, double rhon, double Pn, double Tn, const double *Y) const {
    const double T = Tn * TRef;
    const double P = Pn * PRef;
    const double rho = rhon * rhoRef;
    double G[NS], C[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      w[i] = 0.0;
      C[i] = Y[i] * rho / W[i];
      G[i] = FreeEnthalpy(i, T, 1.0 / T, log(T));
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const AirReac &r = reac[k];
      double Kf = r.A;
      if (r.useN) Kf *= pow(T, r.n);
      if (r.useE) Kf *= exp(-r.EovR / T);
      double a = 1.0;
#pragma unroll
      for (int i = 0; i < 2; i++)
        if (i < r.nEd) a *= (r.nuEk[i] == 1) ? C[r.ed[i]] : pow(C[r.ed[i]], r.nuE[i]);
      double Kb = 0.0, b = 1.0;
      if (r.backward) {
        double sumNu = 0.0, sumNuG = 0.0;
#pragma unroll
        for (int i = 0; i < 2; i++)
          if (i < r.nEd) {
            sumNu -= r.nuE[i];
            sumNuG -= r.nuE[i] * G[r.ed[i]];
          }
#pragma unroll
        for (int i = 0; i < 2; i++)
          if (i < r.nPd) {
            sumNu += r.nuP[i];
            sumNuG += r.nuP[i] * G[r.pd[i]];
          }
        const double lnKc = -sumNuG - sumNu * (log(T) + log(kRGAS / P));
        Kb = Kf * exp(-lnKc);
#pragma unroll
        for (int i = 0; i < 2; i++)
          if (i < r.nPd) b *= (r.nuPk[i] == 1) ? C[r.pd[i]] : pow(C[r.pd[i]], r.nuP[i]);
      }
      double R = Kf * a - Kb * b;
      if (r.nTb > 0) {
        double c = P / (kRGAS * T);
#pragma unroll
        for (int i = 0; i < 5; i++)
          if (i < r.nTb) c += C[r.tb[i]] * r.effm1[i];
        R = c * (Kf * a - Kb * b);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
        if (i < r.nEd) w[r.ed[i]] -= r.nuE[i] * R;
#pragma unroll
      for (int i = 0; i < 2; i++)
        if (i < r.nPd) w[r.pd[i]] += r.nuP[i] * R;
    }
#pragma unroll
    for (int i = 0; i < NS; i++) w[i] *= W[i] * iwiRef;
  }

  HTR_D void ProductionRates(double *w, double rhon, double Pn, double Tn, const double *Y) const {
    const double T = Tn * TRef;
    ProductionRatesT(w, rhon, Pn, T, 1.0 / T, log(T), Y);
  }
  // the same with T = Tn * TRef, 1/T and log T supplied by the caller
  HTR_D void ProductionRatesT(double *w, double rhon, double Pn, double T, double Tinv, double logT,
                              const double *Y) const {
    const double P = Pn * PRef;
    const double rho = rhon * rhoRef;
    // collider concentration P / (R T), and log(R T / P) = -log(cM) for the
    // equilibrium constants
    const double cM = P * Tinv * (1.0 / kRGAS);
    const double lncM = log(cM);
    double G[NS], C[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      w[i] = 0.0;
      C[i] = Y[i] * rho * iW[i];
      G[i] = FreeEnthalpyFast(i, T, Tinv, logT);
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const AirReac &r = reac[k];
      // A T^n exp(-E/RT) and its backward partner as single exponentials
      // (table-driven exp: fastexp.cuh)
      double arg = 0.0;
      if (r.useN) arg += r.n * logT;
      if (r.useE) arg -= r.EovR * Tinv;
      const double Kf = r.A * exp_table(arg);
      double a = 1.0;
#pragma unroll
      for (int i = 0; i < 2; i++)
        if (i < r.nEd) a *= (r.nuEk[i] == 1) ? C[r.ed[i]] : ((r.nuEk[i] == 2) ? C[r.ed[i]] * C[r.ed[i]] : pow(C[r.ed[i]], r.nuE[i]));
      double Kb = 0.0, b = 1.0;
      if (r.backward) {
        double sumNuG = 0.0;
#pragma unroll
        for (int i = 0; i < 2; i++)
          if (i < r.nEd) sumNuG -= r.nuE[i] * G[r.ed[i]];
#pragma unroll
        for (int i = 0; i < 2; i++)
          if (i < r.nPd) sumNuG += r.nuP[i] * G[r.pd[i]];
        // ln Kc = -sum nu G - sum nu log(R T / P)
        const double lnKc = r.sumNu * lncM - sumNuG;
        Kb = r.A * exp_table(arg - lnKc);
#pragma unroll
        for (int i = 0; i < 2; i++)
          if (i < r.nPd) b *= (r.nuPk[i] == 1) ? C[r.pd[i]] : ((r.nuPk[i] == 2) ? C[r.pd[i]] * C[r.pd[i]] : pow(C[r.pd[i]], r.nuP[i]));
      }
      double c = 1.0;
      if (r.nTb > 0) {
        c = cM;
#pragma unroll
        for (int i = 0; i < 5; i++)
          if (i < r.nTb) c += C[r.tb[i]] * r.effm1[i];
      }
      const double R = c * (Kf * a - Kb * b);
#pragma unroll
      for (int i = 0; i < 2; i++)
        if (i < r.nEd) w[r.ed[i]] -= r.nuE[i] * R;
#pragma unroll
      for (int i = 0; i < 2; i++)
        if (i < r.nPd) w[r.pd[i]] += r.nuP[i] * R;
    }
#pragma unroll
    for (int i = 0; i < NS; i++) w[i] *= W[i] * iwiRef;
  }
};

}  // namespace htr
