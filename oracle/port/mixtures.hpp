// CPU oracle port: thermodynamics, transport and kinetics of the two
// mixtures on the RHS path.  TEST INFRASTRUCTURE ONLY.
//
// Restated from the reference's Mixtures (src/Mixtures/ConstPropMix.inl,
// Species.inl, MultiComponent.inl, Reaction.inl).  Every expression keeps the
// reference's operand order so that, compiled without FMA contraction, the
// results are bit-identical to the compiled reference.
#ifndef HTR_ORACLE_PORT_MIXTURES_HPP
#define HTR_ORACLE_PORT_MIXTURES_HPP

#include <algorithm>
#include <cmath>

#include "htr_mix.h"

namespace oport {

// Physical constants (src/Utils/constants.h:35-60).
constexpr double kPI = 3.1415926535898;
constexpr double kRGAS = 8.3144598;
constexpr double kNa = 6.02214086e23;
constexpr double kKb = 1.38064852e-23;
constexpr double kEps0 = 8.8541878128e-12;
constexpr double kECrg = 1.60217662e-19;

// ---------------------------------------------------------------------------
// Single-species calorically perfect gas (src/Mixtures/ConstPropMix.inl:57-168)
// ---------------------------------------------------------------------------
struct ConstProp {
  static constexpr int NS = 1;
  static constexpr bool kHasReactions = false;
  htr_constpropmix_t m;

  double MolarWeightFromYi(const double *) const { return kRGAS / m.R; }
  double MolarWeightFromXi(const double *) const { return kRGAS / m.R; }
  void MolarFractions(double *X, double, const double *Y) const { X[0] = Y[0]; }
  void MassFractions(double *Y, double, const double *X) const { Y[0] = X[0]; }
  double RhoFromRhoYi(const double *r) const { return r[0]; }
  void YiFromRhoYi(double *Y, double rho, const double *r) const { Y[0] = r[0] / rho; }
  void ClipYi(double *) const {}
  double Rho(double P, double T, double) const { return P / (m.R * T); }
  double HeatCapacity(double, const double *) const { return m.gamma / (m.gamma - 1) * m.R; }
  double SpeciesEnthalpy(int, double T) const { return m.gamma / (m.gamma - 1) * m.R * T; }
  double SpeciesMolarWeight(int) const { return kRGAS / m.R; }
  double InternalEnergy(double T, const double *) const { return T * m.R / (m.gamma - 1.0); }
  double TFromInternalEnergy(double e0, double, const double *) const {
    return e0 * (m.gamma - 1.0) / m.R;
  }
  double TFromRhoAndP(double rho, double MixW, double P) const { return P * MixW / (rho * kRGAS); }
  double PFromRhoAndT(double rho, double MixW, double T) const { return rho * kRGAS * T / MixW; }
  double Viscosity(double T, const double *) const {
    if (m.viscosityModel == HTR_VISC_CONSTANT) return m.constantVisc;
    if (m.viscosityModel == HTR_VISC_POWERLAW)
      return m.powerlawViscRef * std::pow((T / m.powerlawTempRef), 0.7);
    return (m.sutherlandViscRef * std::pow((T / m.sutherlandTempRef), 1.5)) *
           ((m.sutherlandTempRef + m.sutherlandSRef) / (T + m.sutherlandSRef));
  }
  double HeatConductivity(double T, const double *X) const {
    const double cp = m.gamma / (m.gamma - 1) * m.R;
    return cp / m.Prandtl * Viscosity(T, X);
  }
  double Gamma(double, double, const double *) const { return m.gamma; }
  double SpeedOfSound(double T, double gamma, double) const { return std::sqrt(gamma * m.R * T); }
  void Diffusivity(double *D, double, double, double, const double *) const { D[0] = 0.0; }
  void ProductionRates(double *w, double, double, double, const double *) const { w[0] = 0.0; }
  double dpde(double rho, double gamma) const { return rho * (gamma - 1); }
  void dpdrhoi(double *d, double, double T, const double *) const { d[0] = m.R * T; }
};

// ---------------------------------------------------------------------------
// Five-species air (src/Mixtures/Species.inl, MultiComponent.inl, Reaction.inl)
// ---------------------------------------------------------------------------
struct Air {
  static constexpr int NS = 5;
  static constexpr bool kHasReactions = true;
  htr_airmix_t m;

  // --- species (Species.inl) ---------------------------------------------
  const double *poly(int i, double T) const {
    const htr_nasa9_t &c = m.species[i].cpCoeff;
    if (T > c.TSwitch2) return c.cpH;
    if (T > c.TSwitch1) return c.cpM;
    return c.cpL;
  }
  // Species.inl:84-101
  double Cp(int i, double T) const {
    const double rOvW = kRGAS / m.species[i].W;
    const double Tinv = 1.0 / T;
    const double *c = poly(i, T);
    return rOvW * (c[0] * Tinv * Tinv + c[1] * Tinv + c[2] +
                   T * (c[3] + T * (c[4] + T * (c[5] + T * c[6]))));
  }
  // Species.inl:103-123
  double FreeEnthalpy(int i, double T) const {
    const double Tinv = 1.0 / T;
    const double logT = std::log(T);
    const double *c = poly(i, T);
    const double G = -0.5 * c[0] * Tinv * Tinv + c[1] * Tinv * (1.0 + logT) +
                     c[2] * (1.0 - logT) + c[7] * Tinv - c[8];
    return G - 0.5 * T * (c[3] + T * (c[4] / 3 + T * (c[5] / 6 + 0.1 * T * c[6])));
  }
  // Species.inl:125-143
  double Enthalpy(int i, double T) const {
    const double rOvW = kRGAS / m.species[i].W;
    const double Tinv = 1.0 / T;
    const double *c = poly(i, T);
    const double E = -c[0] * Tinv + c[1] * std::log(T) + c[7] +
                     T * (c[2] + T * (c[3] * 0.50 + T * (c[4] / 3 + T * (c[5] * 0.25 + c[6] / 5 * T))));
    return E * rOvW;
  }
  static double omega_mu(double T) {  // Species.inl:33-48
    const double m1 = 3.3530622607, m2 = 2.53272006, m3 = 2.9024238575, m4 = 0.11186138893;
    const double m5 = 0.8662326188, m6 = 1.3913958626, m7 = 3.158490576, m8 = 0.18973411754;
    const double m9 = 0.00018682962894;
    const double num = m1 + T * (m2 + T * (m3 + T * m4));
    const double den = m5 + T * (m6 + T * (m7 + T * (m8 + T * m9)));
    return num / den;
  }
  static double omega_D(double T) {  // Species.inl:50-66
    const double m1 = 6.8728271691, m2 = 9.4122316321, m3 = 7.7442359037, m4 = 0.23424661229;
    const double m5 = 1.45337701568, m6 = 5.2269794238, m7 = 9.7108519575, m8 = 0.46539437353;
    const double m9 = 0.00041908394781;
    const double num = m1 + T * (m2 + T * (m3 + T * m4));
    const double den = m5 + T * (m6 + T * (m7 + T * (m8 + T * m9)));
    return num / den;
  }
  // Species.inl:145-150
  double Mu(int i, double T) const {
    const htr_species_t &s = m.species[i];
    const double num = 5 * std::sqrt(kPI * s.W / kNa * kKb * T);
    const double den = 16 * kPI * std::pow(s.DiffCoeff.sigma, 2) * omega_mu(T * s.DiffCoeff.kbOveps);
    return num / den;
  }
  // Species.inl:152-181 (Stockmayer collision parameters)
  void CollParam(int a, int b, double T, double &sigmaij, double &omega11) const {
    const htr_ljdata_t &s1 = m.species[a].DiffCoeff;
    const htr_ljdata_t &s2 = m.species[b].DiffCoeff;
    double xi = 1.0;
    if ((s1.mu * s2.mu == 0.0) && (s1.mu + s2.mu != 0.0)) {
      double mup, alp, epr;
      if (s1.mu != 0.0) {
        mup = s1.mu / std::sqrt(4 * kPI * kEps0 * kKb * std::pow(s1.sigma, 3) / s1.kbOveps);
        alp = s2.alpha / std::pow(s2.sigma, 3);
        epr = std::sqrt(s2.kbOveps / s1.kbOveps);
      } else {
        mup = s2.mu / std::sqrt(4 * kPI * kEps0 * kKb * std::pow(s2.sigma, 3) / s2.kbOveps);
        alp = s1.alpha / std::pow(s1.sigma, 3);
        epr = std::sqrt(s1.kbOveps / s2.kbOveps);
      }
      xi = 1 + 0.25 * mup * alp * epr;
    }
    sigmaij = 0.5 * (s1.sigma + s2.sigma) * std::pow(xi, -1. / 6);
    const double kboEpsij = std::sqrt(s1.kbOveps * s2.kbOveps) / (xi * xi);
    omega11 = omega_D(T * kboEpsij);
  }
  // Species.inl:216-242 (binary diffusion coefficient)
  double Dif(int a, int b, double P, double T) const {
    double sigmaij, omega11;
    CollParam(a, b, T, sigmaij, omega11);
    const double Wa = m.species[a].W, Wb = m.species[b].W;
    const double invWij = (Wa + Wb) / (Wa * Wb);
    const double num = 3 * std::sqrt(2 * kPI * std::pow(kKb, 3) * std::pow(T, 3) * kNa * invWij);
    const double den = 16 * kPI * P * sigmaij * sigmaij * omega11;
    return num / den;
  }
  double SelfDiffusion(int i, double T) const {  // Species.inl:271-276
    const htr_species_t &s = m.species[i];
    const double num = 3 * std::sqrt(kPI * kKb * T * s.W / kNa);
    const double den = 8 * kPI * std::pow(s.DiffCoeff.sigma, 2) * omega_D(T * s.DiffCoeff.kbOveps);
    return num / den;
  }
  double FZrot(int i, double T) const {  // Species.inl:278-284
    const double tmp = 1.0 / (m.species[i].DiffCoeff.kbOveps * T);
    return 1 + 0.5 * std::pow(kPI, 1.5) * std::sqrt(tmp) + (2 + 0.25 * kPI * kPI) * tmp +
           std::pow(kPI, 1.5) * std::pow(tmp, 1.5);
  }
  // Species.inl:286-351 (Eucken-type conductivity with Mason-Monchick corrections)
  double Lam(int i, double T) const {
    const htr_species_t &s = m.species[i];
    if (s.DiffCoeff.Geom == 0) {
      const double mu = Mu(i, T);
      return 15.0 / 4 * mu * kRGAS / s.W;
    }
    const double CvTOvR = 1.5;
    const double CvROvR = (s.DiffCoeff.Geom == 1) ? 1.0 : 1.5;
    const double CvT = CvTOvR * kRGAS;
    const double CvR = CvROvR * kRGAS;
    const double CvV = Cp(i, T) * s.W - ((s.DiffCoeff.Geom == 1) ? 3.5 : 4.0) * kRGAS;
    const double Dkk = SelfDiffusion(i, T);
    const double mu = Mu(i, T);
    const double fV = Dkk / mu;
    const double Zrot = s.DiffCoeff.Z298 * FZrot(i, 298.0) / FZrot(i, T);
    const double A = 2.5 - fV;
    const double B = Zrot + 2 / kPI * (5. / 3 * CvROvR + fV);
    const double fT = 2.5 * (1. - 2 * CvR * A / (kPI * CvT * B));
    const double fR = fV * (1. + 2 * A / (kPI * B));
    return mu / s.W * (fT * CvT + fR * CvR + fV * CvV);
  }

  // --- mixture (MultiComponent.inl) ----------------------------------------
  void ClipYi(double *Y) const {
    for (int i = 0; i < NS; i++) {
      Y[i] = std::max(Y[i], 1e-60);
      Y[i] = std::min(Y[i], 1.0);
    }
  }
  double MolarWeightFromYi(const double *Y) const {
    double w = 0.0;
    for (int i = 0; i < NS; i++) w += Y[i] / m.species[i].W;
    return 1.0 / w;
  }
  double MolarWeightFromXi(const double *X) const {
    double w = 0.0;
    for (int i = 0; i < NS; i++) w += X[i] * m.species[i].W;
    return w;
  }
  void MolarFractions(double *X, double MixW, const double *Y) const {
    for (int i = 0; i < NS; i++) X[i] = Y[i] * MixW / m.species[i].W;
  }
  void MassFractions(double *Y, double MixW, const double *X) const {
    for (int i = 0; i < NS; i++) Y[i] = X[i] * m.species[i].W / MixW;
  }
  double RhoFromRhoYi(const double *r) const {
    double rho = 0.0;
    for (int i = 0; i < NS; i++) rho += r[i];
    return rho;
  }
  void YiFromRhoYi(double *Y, double rho, const double *r) const {
    const double irho = 1.0 / rho;
    for (int i = 0; i < NS; i++) Y[i] = irho * r[i];
  }
  double Rho(double P, double T, double MixW) const { return P * MixW * m.iMixWRef / T; }
  double HeatCapacity(double Tn, const double *Y) const {
    const double T = Tn * m.TRef;
    double cp = 0.0;
    for (int i = 0; i < NS; i++) cp += Y[i] * Cp(i, T);
    return cp * m.iCpRef;
  }
  double SpeciesEnthalpy(int i, double T) const { return Enthalpy(i, T * m.TRef) * m.ieRef; }
  double SpeciesMolarWeight(int i) const { return m.species[i].W; }
  double InternalEnergy(double Tn, const double *Y) const {
    const double T = Tn * m.TRef;
    double e = 0.0;
    for (int i = 0; i < NS; i++) e += Y[i] * (Enthalpy(i, T) - kRGAS * T / m.species[i].W);
    return e * m.ieRef;
  }
  // MultiComponent.inl:188-209 (Newton, 1000 iterations, tolerance 1e-8)
  double TFromInternalEnergy(double e0, double T, const double *Y) const {
    const int MAXITS = 1000;
    const double TOL = 1e-8;
    double dfdT = 1.0;
    for (int j = 0; j < MAXITS; j++) {
      const double f = e0 - InternalEnergy(T, Y);
      if (std::fabs(f / dfdT) < TOL) break;
      dfdT = 0.0;
      for (int i = 0; i < NS; i++)
        dfdT += Y[i] * (Cp(i, T * m.TRef) - kRGAS / m.species[i].W) * m.iCpRef;
      T += f / dfdT;
    }
    return T;
  }
  double TFromRhoAndP(double rho, double MixW, double P) const {
    return P * MixW * m.iMixWRef / rho;
  }
  double PFromRhoAndT(double rho, double MixW, double T) const {
    return rho * T / (MixW * m.iMixWRef);
  }
  // MultiComponent.inl:231-255 (Wilke)
  double Viscosity(double Tn, const double *X) const {
    const double T = Tn * m.TRef;
    double muk[NS];
    for (int i = 0; i < NS; i++) muk[i] = Mu(i, T);
    double mu = 0.0;
    for (int i = 0; i < NS; i++) {
      double den = 0.0;
      for (int j = 0; j < NS; j++) {
        double Phi = 1 + std::sqrt(muk[i] / muk[j]) *
                             std::pow(m.species[j].W / m.species[i].W, 0.25);
        Phi *= Phi / std::sqrt(8 * (1 + m.species[i].W / m.species[j].W));
        den += X[j] * Phi;
      }
      mu += X[i] * muk[i] / den;
    }
    return mu * m.imuRef;
  }
  // MultiComponent.inl:258-271
  double HeatConductivity(double Tn, const double *X) const {
    const double T = Tn * m.TRef;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < NS; i++) {
      const double l = Lam(i, T);
      a += X[i] * l;
      b += X[i] / l;
    }
    return 0.5 * (a + 1.0 / b) * m.ilamRef;
  }
  double Gamma(double T, double MixW, const double *Y) const {
    const double cp = HeatCapacity(T, Y);
    const double Wr = MixW * m.iMixWRef;
    return cp / (cp - 1.0 / Wr);
  }
  double SpeedOfSound(double T, double gamma, double MixW) const {
    return std::sqrt(gamma * T / (MixW * m.iMixWRef));
  }
  // MultiComponent.inl:288-311 (mixture-averaged diffusivities)
  void Diffusivity(double *D, double Pn, double Tn, double MixW, const double *X) const {
    const double T = Tn * m.TRef;
    const double P = Pn * m.PRef;
    for (int i = 0; i < NS; i++) D[i] = 0.0;
    for (int i = 0; i < NS; i++)
      for (int j = 0; j < i; j++) {
        const double invDij = 1.0 / Dif(i, j, P, T);
        D[i] += X[j] * invDij;
        D[j] += X[i] * invDij;
      }
    for (int i = 0; i < NS; i++) {
      double num = 0.0;
      for (int j = 0; j < NS; j++)
        if (j != i) num += X[j] * m.species[j].W;
      D[i] = num / (MixW * D[i]) * m.iDiRef;
    }
  }
  double dpde(double rho, double gamma) const { return rho * (gamma - 1); }
  void dpdrhoi(double *d, double gamma, double Tn, const double *Y) const {
    const double T = Tn * m.TRef;
    double e = 0.0;
    for (int i = 0; i < NS; i++) {
      d[i] = Enthalpy(i, T) - kRGAS * T / m.species[i].W;
      e += Y[i] * d[i];
    }
    for (int i = 0; i < NS; i++)
      d[i] = (kRGAS * T / m.species[i].W + (gamma - 1) * (e - d[i])) * m.ieRef;
  }

  // --- kinetics (Reaction.inl) ----------------------------------------------
  static double RateCoeff(const htr_arrhenius_t &a, double T) {  // Reaction.inl:33-41
    double Kf = a.A;
    if (a.n != 0.0) Kf *= std::pow(T, a.n);
    if (std::fabs(a.EovR) > 1e-5) Kf *= std::exp(-a.EovR / T);
    return Kf;
  }
  template <class R>
  static double BackwardCoeff(const R &r, double Kf, double P, double T, const double *G) {
    double sumNu = 0.0, sumNuG = 0.0;  // Reaction.inl:84-101
    for (int i = 0; i < r.Neducts; i++) {
      sumNu -= r.educts[i].nu;
      sumNuG -= r.educts[i].nu * G[r.educts[i].ind];
    }
    for (int i = 0; i < r.Npducts; i++) {
      sumNu += r.pducts[i].nu;
      sumNuG += r.pducts[i].nu * G[r.pducts[i].ind];
    }
    const double lnKc = -sumNuG - sumNu * (std::log(T) + std::log(kRGAS / P));
    return Kf * std::exp(-lnKc);
  }
  template <class R>
  static double MassAction(const R &r, double Kf, double P, double T, const double *C,
                           const double *G, double &Kb, double &b) {
    double a = 1.0;
    for (int i = 0; i < r.Neducts; i++) {
      const int ind = r.educts[i].ind;
      if (r.educts[i].nu == 1)
        a *= C[ind];
      else
        a *= std::pow(C[ind], r.educts[i].nu);
    }
    Kb = 0.0;
    b = 1.0;
    if (r.has_backward) {
      Kb = BackwardCoeff(r, Kf, P, T, G);
      for (int i = 0; i < r.Npducts; i++) {
        const int ind = r.pducts[i].ind;
        if (r.pducts[i].nu == 1)
          b *= C[ind];
        else
          b *= std::pow(C[ind], r.pducts[i].nu);
      }
    }
    return a;
  }
  template <class R> static void Apply(const R &r, double Rr, double *w) {
    for (int i = 0; i < r.Neducts; i++) w[r.educts[i].ind] -= r.educts[i].nu * Rr;
    for (int i = 0; i < r.Npducts; i++) w[r.pducts[i].ind] += r.pducts[i].nu * Rr;
  }
  // MultiComponent.inl:370-415
  void ProductionRates(double *w, double rhon, double Pn, double Tn, const double *Y) const {
    const double T = Tn * m.TRef;
    const double P = Pn * m.PRef;
    const double rho = rhon * m.rhoRef;
    double G[NS], C[NS];
    for (int i = 0; i < NS; i++) {
      w[i] = 0.0;
    }
    for (int i = 0; i < NS; i++) {
      C[i] = Y[i] * rho / m.species[i].W;
      G[i] = FreeEnthalpy(i, T);
    }
    for (int k = 0; k < HTR_AIR_NREAC; k++) {  // Reaction.inl:105-151
      const htr_reaction_t &r = m.reactions[k];
      const double Kf = RateCoeff(r.ArrCoeff, T);
      double Kb, b;
      const double a = MassAction(r, Kf, P, T, C, G, Kb, b);
      Apply(r, (Kf * a - Kb * b), w);
    }
    for (int k = 0; k < HTR_AIR_NTBREAC; k++) {  // Reaction.inl:153-222
      const htr_tbreaction_t &r = m.ThirdbodyReactions[k];
      const double Kf = RateCoeff(r.ArrCoeff, T);
      double Kb, b;
      const double a = MassAction(r, Kf, P, T, C, G, Kb, b);
      double c = 1.0;
      if (r.Nthirdb > 0) {
        c = P / (kRGAS * T);
        for (int i = 0; i < r.Nthirdb; i++) c += C[r.thirdb[i].ind] * (r.thirdb[i].eff - 1.0);
      }
      Apply(r, c * (Kf * a - Kb * b), w);
    }
    for (int i = 0; i < NS; i++) w[i] *= m.species[i].W * m.iwiRef;
  }
};

}  // namespace oport

#endif
