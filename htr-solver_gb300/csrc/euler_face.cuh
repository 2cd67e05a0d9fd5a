// Face fluxes of the Euler schemes, shared by the per-direction task kernels
// (euler.cu) and the fused stage pipeline (stage_euler.cu).  Both translation
// units are compiled with -fmad=false (see stencil.cuh).
#pragma once

#include "mixture.cuh"
#include "stencil.cuh"

namespace htr {

struct EulerArgs {
  Fd<double> C, Cold, SoS, rho, Y, u, P, me, Ct;
  Fd<int> nt;
  Fd<bool> sen;
  Box my, fb;
  double rk0, rk1, dt;
  // per-cell step sizes (batched instances): the limiter's deltaTime of a
  // face is (dtc[left cell] * dtc_c3) * dtc_h, the stage's dt * RK_C[3]
  // (halved with implicit chemistry); null: dt above for every face
  const double *dtc = nullptr;
  double dtc_c3 = 1.0, dtc_h = 1.0;
  HTR_D double face_dt(const long long *p) const { return dtc ? (dtc[my.dense(p)] * dtc_c3) * dtc_h : dt; }
};

enum { kSchemeHybrid = 0, kSchemeSkew = 1, kSchemeTeno = 2 };

template <class Mix, int D> struct EulerFace {
  static constexpr int NS = Mix::NS, NE = NS + 4, iU = NS, iE = NS + 3;
  static constexpr int T1 = (D == 0) ? 1 : 0, T2 = (D == 2) ? 1 : 2;

  const EulerArgs &a;
  const Mix &mix;

  HTR_D void shift(long long *q, const long long *p, int off, bool plus) const {
    q[0] = p[0];
    q[1] = p[1];
    q[2] = p[2];
    q[D] = plus ? wrap_plus(p[D], a.fb.lo[D], a.fb.size(D), off)
                : wrap_minus(p[D], a.fb.lo[D], a.fb.size(D), off);
  }

  // Kennedy-Gruber split-form flux at face p+1/2 (rhs.inl:77-196)
  HTR_D void kg(double *F, const long long *p, int t) const {
    if (t == L_S || t == Rm1_S) {
      long long q[3];
      shift(q, p, (t == L_S) ? 0 : kNode[t].off[2], true);
      const double *Cq = a.C.at(q);
      const double un = ld(&a.u.at(q)[D]);
      const double pq = ld(a.P.at(q));
#pragma unroll
      for (int i = 0; i < NE; i++) F[i] = -(ld(&Cq[i]) * un);
      F[iU + D] -= pq;
      F[iE] -= pq * un;
      return;
    }
    long long q[6][3];
    shift(q[0], p, kNode[t].off[0], false);
    shift(q[1], p, kNode[t].off[1], false);
    q[2][0] = p[0];
    q[2][1] = p[1];
    q[2][2] = p[2];
    shift(q[3], p, kNode[t].off[2], true);
    shift(q[4], p, kNode[t].off[3], true);
    shift(q[5], p, kNode[t].off[4], true);
    double r[6], v[6], h[6], pr[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      r[k] = ld(a.rho.at(q[k]));
      v[k] = -ld(&a.u.at(q[k])[D]);
      pr[k] = ld(a.P.at(q[k]));
      h[k] = (ld(&a.C.at(q[k])[iE]) + pr[k]) / r[k];
    }
    const int order = kNode[t].kgOrder;
    const double kg0 = kNode[t].kg[0], kg1 = kNode[t].kg[1], kg2 = kNode[t].kg[2];
    const double kgc[3] = {kg0, kg1, kg2};
    // products (rho_a + rho_b)(v_a + v_b) shared by every transported scalar
    double rv[3][3];
#pragma unroll
    for (int l = 0; l < 3; l++)
#pragma unroll
      for (int m = 0; m < 3; m++)
        if (m <= l && l < order) rv[l][m] = (r[2 - m] + r[2 - m + l + 1]) * (v[2 - m] + v[2 - m + l + 1]);
    auto triple = [&](const double *phi) {
      double flux = 0.0;
#pragma unroll
      for (int l = 0; l < 3; l++) {
        if (l < order) {
          double acc = 0.0;
#pragma unroll
          for (int m = 0; m <= l; m++) acc += rv[l][m] * (phi[2 - m] + phi[2 - m + l + 1]);
          flux += kgc[l] * acc;
        }
      }
      return flux * 0.25;
    };
    double phi[6];
#pragma unroll
    for (int i = 0; i < NS; i++) {
#pragma unroll
      for (int k = 0; k < 6; k++) phi[k] = ld(&a.Y.at(q[k])[i]);
      F[i] = triple(phi);
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
#pragma unroll
      for (int k = 0; k < 6; k++) phi[k] = ld(&a.u.at(q[k])[c]);
      F[iU + c] = triple(phi);
    }
    {
      double flux = 0.0;
#pragma unroll
      for (int l = 0; l < 3; l++) {
        if (l < order) {
          double acc = 0.0;
#pragma unroll
          for (int m = 0; m <= l; m++) acc += (pr[2 - m] + pr[2 - m + l + 1]);
          flux += kgc[l] * acc;
        }
      }
      F[iU + D] -= flux;
    }
    F[iE] = triple(h);
  }

  struct Roe {
    double rho, Yi[NS], vel[3], H, e, dpde, dpdrhoi[NS], a2, a;
  };

  // rhs.inl:198-279
  HTR_D void roe(Roe &R, const long long *pL, const long long *pR) const {
    double CL[NE], CR[NE], YL[NS], YR[NS], uL[3], uR[3];
#pragma unroll
    for (int i = 0; i < NE; i++) {
      CL[i] = ld(&a.C.at(pL)[i]);
      CR[i] = ld(&a.C.at(pR)[i]);
    }
#pragma unroll
    for (int i = 0; i < NS; i++) {
      YL[i] = ld(&a.Y.at(pL)[i]);
      YR[i] = ld(&a.Y.at(pR)[i]);
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
      uL[i] = ld(&a.u.at(pL)[i]);
      uR[i] = ld(&a.u.at(pR)[i]);
    }
    const double rhoL = ld(a.rho.at(pL)), rhoR = ld(a.rho.at(pR));
    const double PL = ld(a.P.at(pL)), PR = ld(a.P.at(pR));
    const double eL = CL[iE] / rhoL - 0.5 * mod2(uL);
    const double eR = CR[iE] / rhoR - 0.5 * mod2(uR);
    const double HL = (CL[iE] + PL) / rhoL;
    const double HR = (CR[iE] + PR) / rhoR;
    const double sL = sqrt(rhoL), sR = sqrt(rhoR);
    const double fL = sL / (sL + sR);
    const double fR = sR / (sL + sR);
    R.rho = sqrt(rhoL * rhoR);
#pragma unroll
    for (int i = 0; i < NS; i++) R.Yi[i] = YL[i] * fL + YR[i] * fR;
#pragma unroll
    for (int i = 0; i < 3; i++) R.vel[i] = uL[i] * fL + uR[i] * fR;
    R.H = HL * fL + HR * fR;
    R.e = eL * fL + eR * fR;
    const double PovRho = R.H - R.e - 0.5 * mod2(R.vel);
    const double MixW = mix.MolarWeightFromYi(R.Yi);
    const double Teos = mix.TFromRhoAndP(R.rho, MixW, PovRho * R.rho);
    double gamma;
    mix.RoeThermo(R.e, Teos, MixW, R.Yi, gamma, R.dpdrhoi);
    R.dpde = mix.dpde(R.rho, gamma);
    const double dp = PR - PL;
    const double de = eR - eL;
    double drhoi[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) drhoi[i] = rhoR * YR[i] - rhoL * YL[i];
    double dpError = dp - de * R.dpde;
    double fact = de * R.dpde;
    fact *= fact;
#pragma unroll
    for (int i = 0; i < NS; i++) {
      const double dpi = drhoi[i] * R.dpdrhoi[i];
      dpError -= dpi;
      fact += dpi * dpi;
    }
    fact = dpError / smax(fact, 1e-6);
#pragma unroll
    for (int i = 0; i < NS; i++) R.dpdrhoi[i] = R.dpdrhoi[i] * (1.0 + R.dpdrhoi[i] * drhoi[i] * fact);
    R.dpde = R.dpde * (1.0 + R.dpde * de * fact);
    R.a2 = PovRho / R.rho * R.dpde;
#pragma unroll
    for (int i = 0; i < NS; i++) R.a2 += R.Yi[i] * R.dpdrhoi[i];
    R.a = sqrt(R.a2);
  }

  // Face constants of the left-eigenvector projection (rhs.inl:433-505);
  // each is the value the reference recomputes per projection.
  struct Proj {
    double ia, bsp[NS], c[3], dd, Ycj[NS][3], mYd[NS];
  };
  HTR_D void proj_init(Proj &Pj, const Roe &R) const {
    Pj.ia = 1.0 / R.a;
    const double ia2 = 1.0 / R.a2;
    const double Coeff = (R.e - 0.5 * mod2(R.vel)) * R.dpde / R.rho;
#pragma unroll
    for (int i = 0; i < NS; i++) Pj.bsp[i] = (Coeff - R.dpdrhoi[i]) * ia2;
    Pj.dd = R.dpde / (R.rho * R.a2);
#pragma unroll
    for (int i = 0; i < 3; i++) Pj.c[i] = R.vel[i] * Pj.dd;
#pragma unroll
    for (int i = 0; i < NS; i++) {
#pragma unroll
      for (int j = 0; j < 3; j++) Pj.Ycj[i][j] = R.Yi[i] * Pj.c[j];
      Pj.mYd[i] = -R.Yi[i] * Pj.dd;
    }
  }
  HTR_D void to_char(double *r, const double *q, const Roe &R, const Proj &Pj) const {
    double sum1 = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) sum1 += Pj.bsp[i] * q[i];
    double sq = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) sq += q[i];
    r[0] = sq * R.vel[D] * Pj.ia - sum1;
    r[0] -= (Pj.c[D] + Pj.ia) * q[NS + D];
    r[0] -= Pj.c[T1] * q[NS + T1];
    r[0] -= Pj.c[T2] * q[NS + T2];
    r[0] += Pj.dd * q[NS + 3];
    r[0] *= 0.5;
#pragma unroll
    for (int i = 1; i < NS + 1; i++) {
      r[i] = R.Yi[i - 1] * sum1;
      r[i] += q[i - 1];
#pragma unroll
      for (int j = 0; j < 3; j++) r[i] += Pj.Ycj[i - 1][j] * q[NS + j];
      r[i] += Pj.mYd[i - 1] * q[NS + 3];
    }
    r[NS + 1] = -R.vel[T1] * sq;
    r[NS + 1] += q[NS + T1];
    r[NS + 2] = -R.vel[T2] * sq;
    r[NS + 2] += q[NS + T2];
    r[NS + 3] = -sq * R.vel[D] * Pj.ia - sum1;
    r[NS + 3] -= (Pj.c[D] - Pj.ia) * q[NS + D];
    r[NS + 3] -= Pj.c[T1] * q[NS + T1];
    r[NS + 3] -= Pj.c[T2] * q[NS + T2];
    r[NS + 3] += Pj.dd * q[NS + 3];
    r[NS + 3] *= 0.5;
  }

  // rhs.inl:507-572
  HTR_D void from_char(double *r, const double *q, const Roe &R) const {
    double sq = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) sq += q[i + 1];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      double t = 0.0;
      t += R.Yi[i] * q[0];
      t += q[i + 1];
      t += R.Yi[i] * q[NS + 3];
      r[i] = t;
    }
    double rn = 0.0, r1 = 0.0, r2 = 0.0, re = 0.0;
    rn += (R.vel[D] - R.a) * q[0];
    rn += R.vel[D] * sq;
    rn += (R.vel[D] + R.a) * q[NS + 3];
    r1 += R.vel[T1] * q[0];
    r1 += R.vel[T1] * sq;
    r1 += q[NS + 1];
    r1 += R.vel[T1] * q[NS + 3];
    r2 += R.vel[T2] * q[0];
    r2 += R.vel[T2] * sq;
    r2 += q[NS + 2];
    r2 += R.vel[T2] * q[NS + 3];
    re += (R.H - R.vel[D] * R.a) * q[0];
    const double dedp = 1.0 / R.dpde;
    const double E = R.e + 0.5 * mod2(R.vel);
#pragma unroll
    for (int i = 0; i < NS; i++) re += (E - R.rho * R.dpdrhoi[i] * dedp) * q[i + 1];
    re += R.vel[T1] * q[NS + 1];
    re += R.vel[T2] * q[NS + 2];
    re += (R.H + R.vel[D] * R.a) * q[NS + 3];
    r[NS + D] = rn;
    r[NS + T1] = r1;
    r[NS + T2] = r2;
    r[NS + 3] = re;
  }

  // Characteristic TENO flux at face p+1/2 with left point p (rhs.inl:622-759,
  // positivity limiter :710-758; lim_f = dt * (m_e[p] + m_e[right cell])).
  //
  // The reference projects the conserved vector and the flux of each of the
  // six stencil points on every characteristic field, splits them, then
  // reconstructs field by field.  Here the fields are streamed: the per-point
  // quantities every projection row needs (normal velocity, pressure,
  // momentum and energy, and the two species sums of the projection) are
  // kept, and each row is projected, split and reconstructed in turn, with
  // the reference's operations in the reference's order, so every value is
  // bit-identical while only one field's twelve split values are live.
  template <int KIND>
  HTR_D void teno_flux(double *Flux, const long long *p, int t, double lim_f) const {
    long long pts[6][3];
    shift(pts[0], p, kNode[t].off[0], false);
    shift(pts[1], p, kNode[t].off[1], false);
    pts[2][0] = p[0];
    pts[2][1] = p[1];
    pts[2][2] = p[2];
    shift(pts[3], p, kNode[t].off[2], true);
    shift(pts[4], p, kNode[t].off[3], true);
    shift(pts[5], p, kNode[t].off[4], true);
    const double *Cpt[6];
#pragma unroll
    for (int k = 0; k < 6; k++) Cpt[k] = a.C.at(pts[k]);
    double L1 = 0, L0 = 0, LN = 0;
    double un[6], pq[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      un[k] = ld(&a.u.at(pts[k])[D]);
      pq[k] = ld(a.P.at(pts[k]));
      const double c = ld(a.SoS.at(pts[k]));
      const double e1 = fabs(un[k] - c), e0 = fabs(un[k]), eN = fabs(un[k] + c);
      if (k == 0) {
        L1 = e1;
        L0 = e0;
        LN = eN;
      } else {
        L1 = smax(L1, e1);
        L0 = smax(L0, e0);
        LN = smax(LN, eN);
      }
    }
    Roe R;
    roe(R, pts[2], pts[3]);
    Proj Pj;
    proj_init(Pj, R);
    // per point: the species sums of the projection (sum1 = sum bsp_i q_i,
    // sq = sum q_i) of C and of the flux
    double s1Q[6], sqQ[6], s1F[6], sqF[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      double a1 = 0.0, a2 = 0.0, b1 = 0.0, b2 = 0.0;
#pragma unroll
      for (int i = 0; i < NS; i++) {
        const double q = ld(&Cpt[k][i]);
        const double f = q * un[k];
        a1 += Pj.bsp[i] * q;
        a2 += q;
        b1 += Pj.bsp[i] * f;
        b2 += f;
      }
      s1Q[k] = a1;
      sqQ[k] = a2;
      s1F[k] = b1;
      sqF[k] = b2;
    }
    double F[NE], Flc[NE];
    // one characteristic field per iteration (not unrolled: the point data
    // are reloaded from cache, keeping one field's values live)
#pragma unroll 1
    for (int i = 0; i < NE; i++) {
      double fp[6], fm[6];
      const double Lam = (i == 0) ? L1 : ((i == NE - 1) ? LN : L0);
#pragma unroll
      for (int k = 0; k < 6; k++) {
        double cq[4], fq[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          cq[j] = ld(&Cpt[k][NS + j]);
          fq[j] = cq[j] * un[k];
        }
        fq[D] += pq[k];
        fq[3] += pq[k] * un[k];
        double qc, fc;
        if (i == 0 || i == NE - 1) {
          // to_char rows 0 and NS+3
          const double cD = (i == 0) ? (Pj.c[D] + Pj.ia) : (Pj.c[D] - Pj.ia);
          qc = (i == 0 ? sqQ[k] : -sqQ[k]) * R.vel[D] * Pj.ia - s1Q[k];
          qc -= cD * cq[D];
          qc -= Pj.c[T1] * cq[T1];
          qc -= Pj.c[T2] * cq[T2];
          qc += Pj.dd * cq[3];
          qc *= 0.5;
          fc = (i == 0 ? sqF[k] : -sqF[k]) * R.vel[D] * Pj.ia - s1F[k];
          fc -= cD * fq[D];
          fc -= Pj.c[T1] * fq[T1];
          fc -= Pj.c[T2] * fq[T2];
          fc += Pj.dd * fq[3];
          fc *= 0.5;
        } else if (i <= NS) {
          const int sp = i - 1;
          const double q = ld(&Cpt[k][sp]);
          const double f = q * un[k];
          qc = R.Yi[sp] * s1Q[k];
          qc += q;
          fc = R.Yi[sp] * s1F[k];
          fc += f;
#pragma unroll
          for (int j = 0; j < 3; j++) {
            qc += Pj.Ycj[sp][j] * cq[j];
            fc += Pj.Ycj[sp][j] * fq[j];
          }
          qc += Pj.mYd[sp] * cq[3];
          fc += Pj.mYd[sp] * fq[3];
        } else {
          const int tj = (i == NS + 1) ? T1 : T2;
          qc = -R.vel[tj] * sqQ[k];
          qc += cq[tj];
          fc = -R.vel[tj] * sqF[k];
          fc += fq[tj];
        }
        fp[k] = fc + Lam * qc;
        fm[k] = fc - Lam * qc;
      }
      // multi-species fluxes are compared within a tolerance (their Roe
      // state already comes from a Newton solve), so their reconstruction
      // from the selected stencils is contracted; single-species fluxes keep
      // the reference's rounding bit for bit
      const double rp = teno<KIND, false, (NS > 1)>(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], t, nullptr);
      const double rm = teno<KIND, true, (NS > 1)>(fm[0], fm[1], fm[2], fm[3], fm[4], fm[5], t, nullptr);
      F[i] = -0.5 * (rp + rm);
      Flc[i] = (fp[2] + fm[3]) * -0.5;
    }
    from_char(Flux, F, R);
    if (NS > 1) {
      // limiter points: the face's two stencil cells (rhs.inl:717-721)
      const long long *pc = pts[2], *pn = pts[3];
      bool limit = false;
#pragma unroll
      for (int i = 0; i < NS; i++) {
        const double dr = lim_f * Flux[i];
        if (((a.rk0 * ld(&a.Cold.at(pc)[i]) + a.rk1 * ld(&a.C.at(pc)[i]) + dr) < -1e-8) ||
            ((a.rk0 * ld(&a.Cold.at(pn)[i]) + a.rk1 * ld(&a.C.at(pn)[i]) - dr) < -1e-8))
          limit = true;
      }
      if (limit) {
        count_decision(kLimiterBlend);
        const double eps = 1e-60;
        double theta = 1.0;
        double Fl[NE];
        from_char(Fl, Flc, R);
#pragma unroll
        for (int i = 0; i < NS; i++) {
          const double dr = lim_f * Flux[i];
          const double drl = lim_f * Fl[i];
          double thp = 1.0;
          const double rp = a.rk0 * ld(&a.Cold.at(pc)[i]) + a.rk1 * ld(&a.C.at(pc)[i]);
          const double hp = rp + dr;
          if (hp < eps) {
            const double lo = rp + drl;
            thp = (fabs(hp - lo) > eps) ? smax(0.0, (eps - lo) / (hp - lo)) : 1.0;
          }
          double thn = 1.0;
          const double rn = a.rk0 * ld(&a.Cold.at(pn)[i]) + a.rk1 * ld(&a.C.at(pn)[i]);
          const double hn = rn - dr;
          if (hn < eps) {
            const double lo = rn - drl;
            thn = (fabs(hn - lo) > eps) ? smax(0.0, (eps - lo) / (hn - lo)) : 1.0;
          }
          theta = smin(smin(thp, thn), theta);
        }
#pragma unroll
        for (int i = 0; i < NE; i++) Flux[i] = Flux[i] * theta + Fl[i] * (1 - theta);
      }
    }
  }
};

}  // namespace htr
