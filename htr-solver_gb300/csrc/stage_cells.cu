// Per-cell kernels and orchestration of the fused stage pipeline.
//
//   stage_prepass    per cell: velocity-gradient tensor (the reference's
//                    getDeriv, bit-identical), mixture molar weight and total
//                    enthalpy H, each computed once and shared by every face
//                    that needs them
//   diffusion_faces  viscous / heat / species face fluxes of one direction
//   stage_update     per cell: chemistry sources, then the face-flux
//                    differences in the reference's order (Euler Z, Y, X,
//                    diffusion Z, Y, X), the SSP-RK3 update, the primitive
//                    recovery (Newton) and the property refresh
#include "kernels.cuh"
#include "mixture.cuh"
#include "stage.cuh"
#include "stencil.cuh"

namespace htr {

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

StageTuning &stage_tuning() {
  static StageTuning t;
  return t;
}

size_t stage_workspace_bytes(const htr_rect3 &r, int neq) {
  const FaceGrid g = face_grid(r);
  const long long ncell = (r.hi[0] - r.lo[0] + 1) * (r.hi[1] - r.lo[1] + 1) * (r.hi[2] - r.lo[2] + 1);
  size_t b = 0;
  for (int D = 0; D < 3; D++) b += 2 * align256(sizeof(double) * neq * g.nf[D]);
  b += align256(sizeof(TenoEntry) * (g.nf[0] + g.nf[1] + g.nf[2]));
  b += align256(sizeof(unsigned));
  b += align256(sizeof(double) * kPrepVals * ncell);
  b += align256(sizeof(double) * (3 + 2 * (neq - 4)) * ncell);
  return b;
}

bool stage_workspace_carve(void *base, size_t bytes, const htr_rect3 &r, int neq, StageWorkspace &w) {
  if (base == nullptr || bytes < stage_workspace_bytes(r, neq)) return false;
  const FaceGrid g = face_grid(r);
  char *p = static_cast<char *>(base);
  for (int D = 0; D < 3; D++) {
    w.fe[D] = reinterpret_cast<double *>(p);
    p += align256(sizeof(double) * neq * g.nf[D]);
    w.fd[D] = reinterpret_cast<double *>(p);
    p += align256(sizeof(double) * neq * g.nf[D]);
  }
  w.queue = reinterpret_cast<TenoEntry *>(p);
  p += align256(sizeof(TenoEntry) * (g.nf[0] + g.nf[1] + g.nf[2]));
  w.count = reinterpret_cast<unsigned *>(p);
  w.scalars = reinterpret_cast<double *>(p + 48);
  p += align256(sizeof(unsigned));
  w.prep = reinterpret_cast<double *>(p);
  {
    const long long ncell = (r.hi[0] - r.lo[0] + 1) * (r.hi[1] - r.lo[1] + 1) * (r.hi[2] - r.lo[2] + 1);
    p += align256(sizeof(double) * kPrepVals * ncell);
  }
  w.tcache = reinterpret_cast<double *>(p);
  return true;
}

struct Dense {  // dense per-cell indexing of the interior
  long long lo[3], n[3];
  HTR_HD long long idx(const long long *p) const {
    return (p[0] - lo[0]) + n[0] * ((p[1] - lo[1]) + n[1] * (p[2] - lo[2]));
  }
  HTR_HD long long count() const { return n[0] * n[1] * n[2]; }
  HTR_HD void point(long long i, long long *p) const {
    p[0] = lo[0] + i % n[0];
    p[1] = lo[1] + (i / n[0]) % n[1];
    p[2] = lo[2] + i / (n[0] * n[1]);
  }
};
static Dense dense(const htr_rect3 &r) {
  Dense d;
  for (int i = 0; i < 3; i++) {
    d.lo[i] = r.lo[i];
    d.n[i] = r.hi[i] - r.lo[i] + 1;
  }
  return d;
}

// One cell (or face) per thread.  The grid-stride loops of the kernels only
// matter past the launch limit: grids capped at 152 x 32 blocks, each thread
// striding over ~27 cells of a 256^3 box, made its fused step 219.1 ms
// against 213.1 ms (with the shock sensor's grid uncapped too).
static dim3 grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 0x7fffffffLL) b = 0x7fffffffLL;
  return dim3((unsigned)(b > 0 ? b : 1));
}

// ---------------------------------------------------------------------------
struct PrepArgs {
  Fd<double> u, X, C, P, rho, m[3];
  Fd<int> nt[3];
  Box fb;
  Dense dn;
  double *prep;
};

template <class Mix>
__global__ void stage_prepass(const PrepArgs A, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  const long long n = A.dn.count();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    A.dn.point(i, p);
#pragma unroll
    for (int e = 0; e < 3; e++) {
      const int t = ld(A.nt[e].at(p));
      long long pm[3] = {p[0], p[1], p[2]}, pp[3] = {p[0], p[1], p[2]};
      pm[e] = wrap_minus(p[e], A.fb.lo[e], A.fb.size(e), kNode[t].off[1]);
      pp[e] = wrap_plus(p[e], A.fb.lo[e], A.fb.size(e), kNode[t].off[2]);
      const double mm = ld(A.m[e].at(p));
#pragma unroll
      for (int c = 0; c < 3; c++)
        A.prep[(e * 3 + c) * n + i] = deriv(t, ld(&A.u.at(pm)[c]), ld(&A.u.at(p)[c]), ld(&A.u.at(pp)[c]), mm);
    }
    double x[NS];
#pragma unroll
    for (int k = 0; k < NS; k++) x[k] = ld(&A.X.at(p)[k]);
    A.prep[9 * n + i] = mix.MolarWeightFromXi(x);
    A.prep[10 * n + i] = (ld(&A.C.at(p)[NS + 3]) + ld(A.P.at(p))) / ld(A.rho.at(p));
  }
}

// ---------------------------------------------------------------------------
struct DiffFaceArgs {
  Fd<double> C, T, X, rho, mu, lam, Di, u, ms;
  Fd<int> nt;
  Box my, fb;
  Dense dn;
  const double *prep;
  FaceGrid g;
  double *fd;
  const double *tcache;  // the update kernel's stage cache (multi-species)
};

// log T and 1/T at a face temperature Ts (dimensional) next to cell p whose
// stage cache holds log(Tp) and 1/Tp for its current temperature: by series
// in r = (Ts - Tp) / Tp when |r| < 2^-7 (eight terms of log(1 + r) and
// 1/(1 + r), remainders below 2^-59), else from the math library.
HTR_D void face_log_inv(double Ts, double Tp, const double *tcache, long long n, long long ip, double &logT,
                        double &Tinv) {
  if (tcache != nullptr && __double_as_longlong(tcache[ip]) == __double_as_longlong(Tp)) {
    const double Tinvp = tcache[2 * n + ip];
    const double r = (Ts * Tinvp) - 1.0;
    if (fabs(r) < 0.0078125) {
      logT = tcache[n + ip] +
             r * (1.0 + r * (-0.5 + r * (1.0 / 3 + r * (-0.25 + r * (0.2 + r * (-1.0 / 6 + r * (1.0 / 7 - 0.125 * r)))))));
      Tinv = Tinvp * (1.0 + r * (-1.0 + r * (1.0 + r * (-1.0 + r * (1.0 + r * (-1.0 + r * (1.0 + r * (-1.0 + r))))))));
      return;
    }
  }
  Tinv = 1.0 / Ts;
  logT = log(Ts);
}

template <class Mix, int D>
__global__ void __launch_bounds__(128) diffusion_faces(const DiffFaceArgs A, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS, NE = NS + 4, iU = NS, iE = NS + 3;
  constexpr int T1 = (D == 0) ? 1 : 0, T2 = (D == 2) ? 1 : 2;
  const long long nf = A.g.nf[D];
  const long long ncell = A.dn.count();
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
    long long c[3];
    const long long e0 = A.g.ext[D][0], e1 = A.g.ext[D][1];
    c[0] = A.g.lo[0] + f % e0;
    c[1] = A.g.lo[1] + (f / e0) % e1;
    c[2] = A.g.lo[2] + f / (e0 * e1);
    long long p[3] = {c[0], c[1], c[2]};
    if (c[D] == A.my.lo[D]) {
      const int t0 = ld(A.nt.at(c));
      p[D] = wrap_minus(c[D], A.fb.lo[D], A.fb.size(D), kNode[t0].off[1]);
    } else {
      p[D] = c[D] - 1;
    }
    long long q[3] = {p[0], p[1], p[2]};
    q[D] = wrap_plus(p[D], A.fb.lo[D], A.fb.size(D), 1);
    const int t = ld(A.nt.at(p));
    if (outside_face(t)) {
#pragma unroll
      for (int i = 0; i < NE; i++) A.fd[i * nf + f] = 0.0;
      continue;
    }
    const double m_s = ld(A.ms.at(p));
    // interior-dense indices of p and q (periodic interior == bounds)
    const long long ip = A.dn.idx(p), iq = A.dn.idx(q);
    double g1p[3], g1q[3], g2p[3], g2q[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      g1p[k] = A.prep[(T1 * 3 + k) * ncell + ip];
      g1q[k] = A.prep[(T1 * 3 + k) * ncell + iq];
      g2p[k] = A.prep[(T2 * 3 + k) * ncell + ip];
      g2q[k] = A.prep[(T2 * 3 + k) * ncell + iq];
    }
    const double rho_s = interp2(t, ld(A.rho.at(p)), ld(A.rho.at(q)));
    const double iMixW_s = 1.0 / interp2(t, A.prep[9 * ncell + ip], A.prep[9 * ncell + iq]);
    const double Tp = ld(A.T.at(p)), Tq = ld(A.T.at(q));
    const double T_s = interp2(t, Tp, Tq);
    double heat = interp2(t, ld(A.lam.at(p)), ld(A.lam.at(q))) * m_s * (Tp - Tq);
    double F[NE];
    if constexpr (NS > 1) {
      double h[NS], logTs, Tinvs;
      const double Tsd = T_s * mix.TRef;
      face_log_inv(Tsd, Tp, A.tcache, ncell, ip, logTs, Tinvs);
      mix.SpeciesEnthalpiesAt(h, Tsd, Tinvs, logTs);
      double ViCorr = 0.0;
#pragma unroll
      for (int i = 0; i < NS; i++) {
        const double YiVi = interp2(t, ld(&A.Di.at(p)[i]), ld(&A.Di.at(q)[i])) * m_s *
                            (ld(&A.X.at(p)[i]) - ld(&A.X.at(q)[i])) * mix.SpeciesMolarWeight(i) * iMixW_s;
        F[i] = -rho_s * YiVi;
        heat += rho_s * YiVi * h[i];
        ViCorr += YiVi;
      }
#pragma unroll
      for (int i = 0; i < NS; i++) {
        const double cc = interp2(t, ld(&A.C.at(p)[i]), ld(&A.C.at(q)[i])) * ViCorr;
        F[i] += cc;
        heat -= cc * h[i];
      }
    } else {
      const double h0 = mix.SpeciesEnthalpy(0, T_s);
      const double YiVi = interp2(t, ld(&A.Di.at(p)[0]), ld(&A.Di.at(q)[0])) * m_s *
                          (ld(&A.X.at(p)[0]) - ld(&A.X.at(q)[0])) * mix.SpeciesMolarWeight(0) * iMixW_s;
      F[0] = -rho_s * YiVi;
      heat += rho_s * YiVi * h0;
      const double cc = interp2(t, ld(&A.C.at(p)[0]), ld(&A.C.at(q)[0])) * YiVi;
      F[0] += cc;
      heat -= cc * h0;
    }
    const double mu_s = interp2(t, ld(A.mu.at(p)), ld(A.mu.at(q)));
    double up[3], uq[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      up[i] = ld(&A.u.at(p)[i]);
      uq[i] = ld(&A.u.at(q)[i]);
    }
    const double dn_n = m_s * (uq[D] - up[D]);
    const double dn_t1 = m_s * (uq[T1] - up[T1]);
    const double dn_t2 = m_s * (uq[T2] - up[T2]);
    const double d1_n = interp2(t, g1p[D], g1q[D]);
    const double d1_t1 = interp2(t, g1p[T1], g1q[T1]);
    const double d2_n = interp2(t, g2p[D], g2q[D]);
    const double d2_t2 = interp2(t, g2p[T2], g2q[T2]);
    double sigma[3];
    sigma[D] = mu_s * (4 * dn_n - 2 * d1_t1 - 2 * d2_t2) / 3;
    sigma[T1] = mu_s * (dn_t1 + d1_n);
    sigma[T2] = mu_s * (dn_t2 + d2_n);
    double uSigma = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      F[iU + i] = sigma[i];
      uSigma += interp2(t, up[i], uq[i]) * sigma[i];
    }
    F[iE] = (uSigma - heat);
#pragma unroll
    for (int i = 0; i < NE; i++) A.fd[i * nf + f] = F[i];
  }
}

// ---------------------------------------------------------------------------
struct UpdateArgs {
  Fd<double> C, Cold, Ct, Ctold, rho, P, T, X, Y, u, mu, lam, Di, SoS, me[3], md[3];
  Fd<int> nt[3];
  unsigned active;
  Dense dn;
  FaceGrid g;
  const double *fe[3], *fd[3];
  double c1, c2, c3, dt;
  int chemistry;
  int mode;        // StageMode
  const double *dt_cell;  // per-cell step sizes (dense), or null: dt
  double dt_h;            // factor of dt_cell (1/2 with implicit chemistry)
  int *status;
  // [3 + 2 NS][ncell] of the last refresh: T, log(T TRef), 1/(T TRef), the
  // species enthalpies and heat capacities at that T
  double *tcache;
  // boundary step only
  Fd<double> Xp, Tp, up;  // NSCBC inflow profiles
  int bc[6];
  double Pbc[6];
};

// Primitive recovery and property refresh of one cell from its new
// conserved vector u_.  Single-species gas: the task kernels' arithmetic.
// Air: the fused thermo/transport of the mixture (one Newton pass that also
// yields the species c_p of the final temperature, batched inversions).
// cached: the cache holds this cell's species enthalpies and heat
// capacities at the current T (the Newton's first evaluation is skipped).
template <class Mix>
HTR_D void refresh_cell(const UpdateArgs &A, const Mix &mix, const long long *p, const double *u_, long long i,
                        double Td, double Tinv, double logT, bool cached = false) {
  constexpr int NS = Mix::NS;
  double rhoYi[NS], Yi[NS], x[NS], vel[3], d[NS], y2[NS];
#pragma unroll
  for (int k = 0; k < NS; k++) rhoYi[k] = u_[k];
  const double rho = mix.RhoFromRhoYi(rhoYi);
  const double rhoInv = 1.0 / rho;
  int its = 0;
  if constexpr (NS > 1) {
#pragma unroll
    for (int k = 0; k < NS; k++) Yi[k] = rhoInv * rhoYi[k];
    mix.ClipYi(Yi);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NS; k++) s += Yi[k] * mix.iW[k];
    const double MixW = 1.0 / s;  // 1 / MixW = sum Y/W
#pragma unroll
    for (int k = 0; k < NS; k++) x[k] = Yi[k] * MixW * mix.iW[k];
#pragma unroll
    for (int k = 0; k < 3; k++) vel[k] = u_[NS + k] * rhoInv;
    const double e = u_[NS + 3] * rhoInv - 0.5 * mod2(vel);
    double cpk[NS], hk[NS], h0[NS], cp0[NS];
    const long long n = A.dn.count();
    if (cached) {
#pragma unroll
      for (int k = 0; k < NS; k++) {
        h0[k] = A.tcache[(3 + k) * n + i];
        cp0[k] = A.tcache[(3 + NS + k) * n + i];
      }
    }
    const double Tn = mix.TFromInternalEnergyCp(e, *A.T.at(p), Yi, &its, cpk, Td, Tinv, logT, true,
                                                cached ? h0 : nullptr, cp0, hk);
    A.tcache[i] = Tn;
    A.tcache[n + i] = logT;
    A.tcache[2 * n + i] = Tinv;
#pragma unroll
    for (int k = 0; k < NS; k++) {
      A.tcache[(3 + k) * n + i] = hk[k];
      A.tcache[(3 + NS + k) * n + i] = cpk[k];
    }
    const double Pn = rho * Tn * s * mix.MixWRef;
    *A.T.at(p) = Tn;
    *A.P.at(p) = Pn;
    double *xp = A.X.at(p), *up = A.u.at(p);
#pragma unroll
    for (int k = 0; k < NS; k++) xp[k] = x[k];
#pragma unroll
    for (int k = 0; k < 3; k++) up[k] = vel[k];
    // the molar weight and the mass fractions recomputed from X, as the
    // reference's property refresh does: they normalise the clipped Yi,
    // whose sum differs from 1 where clipping raised negative partial
    // densities
    const double MixWx = mix.MolarWeightFromXi(x);
    const double Wr = MixWx * mix.iMixWRef;
    const double iTn = Tinv * mix.TRef;
    *A.rho.at(p) = Pn * Wr * iTn;
    // viscosity, conductivity and diffusivities: stage_transport, from the
    // T, P, X and cached c_p written here
    const double iMixWx = 1.0 / MixWx;
    const double iWr = iMixWx * mix.MixWRef;
    double c = 0.0;
#pragma unroll
    for (int k = 0; k < NS; k++) {
      y2[k] = x[k] * mix.W[k] * iMixWx;
      c += y2[k] * cpk[k];
    }
    c *= mix.iCpRef;
    const double gamma = c / (c - iWr);
    *A.SoS.at(p) = sqrt(gamma * Tn * iWr);
  } else {
    mix.YiFromRhoYi(Yi, rho, rhoYi);
    mix.ClipYi(Yi);
    const double MixW = mix.MolarWeightFromYi(Yi);
    mix.MolarFractions(x, MixW, Yi);
#pragma unroll
    for (int k = 0; k < 3; k++) vel[k] = u_[NS + k] * rhoInv;
    const double e = u_[NS + 3] * rhoInv - 0.5 * mod2(vel);
    const double Tn = mix.TFromInternalEnergy(e, *A.T.at(p), Yi, &its);
    const double Pn = mix.PFromRhoAndT(rho, MixW, Tn);
    *A.T.at(p) = Tn;
    *A.P.at(p) = Pn;
    double *xp = A.X.at(p), *up = A.u.at(p);
#pragma unroll
    for (int k = 0; k < NS; k++) xp[k] = x[k];
#pragma unroll
    for (int k = 0; k < 3; k++) up[k] = vel[k];
    const double MixWx = mix.MolarWeightFromXi(x);
    *A.rho.at(p) = mix.Rho(Pn, Tn, MixWx);
    *A.mu.at(p) = mix.Viscosity(Tn, x);
    *A.lam.at(p) = mix.HeatConductivity(Tn, x);
    mix.Diffusivity(d, Pn, Tn, MixWx, x);
    mix.MassFractions(y2, MixWx, x);
    const double gamma = mix.Gamma(Tn, MixWx, y2);
    *A.SoS.at(p) = mix.SpeedOfSound(Tn, gamma, MixWx);
  }
  if (its >= 1000 && A.status) atomicMax(A.status, (int)HTR_ERR_ITERATION_CAP);
  double *yp = A.Y.at(p);
#pragma unroll
  for (int k = 0; k < NS; k++) yp[k] = y2[k];
  if constexpr (NS == 1) A.Di.at(p)[0] = d[0];
}

// Viscosity, conductivity and mixture-averaged diffusivities of the cells
// that refresh_cell just refreshed (multi-species mixtures): those whose
// temperature cache entry holds their current temperature.  The inputs are
// the values refresh_cell wrote and used (T, P, X, 1/T and the species c_p
// of the final Newton temperature), so the results are those it would have
// computed.  A kernel of its own because the double-float transport
// (TransportDF) runs on the FP32 pipe in long dependent chains that the
// FP64-bound update kernel, at its register count, has too few warps to
// hide (inside the update kernel: 52.2 ms per 256^3 stage; split: 36.1 ms
// update + 6.7 ms here).  Five blocks per SM (96 registers, a few hundred
// bytes of spills) run it 9 % faster than four without spills.
template <class Mix>
__global__ void __launch_bounds__(128, 5) stage_transport(const UpdateArgs A, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  const long long n = A.dn.count();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    A.dn.point(i, p);
    const double Tn = *A.T.at(p);
    if (__double_as_longlong(A.tcache[i]) != __double_as_longlong(Tn)) continue;
    double x[NS], cpk[NS], d[NS], m_, l_;
    const double *xp = A.X.at(p);
#pragma unroll
    for (int k = 0; k < NS; k++) {
      x[k] = xp[k];
      cpk[k] = A.tcache[(3 + NS + k) * n + i];
    }
    mix.TransportDF(Tn * mix.TRef, A.tcache[2 * n + i], *A.P.at(p), mix.MolarWeightFromXi(x), x, cpk, m_, l_, d);
    *A.mu.at(p) = m_;
    *A.lam.at(p) = l_;
    double *dp = A.Di.at(p);
#pragma unroll
    for (int k = 0; k < NS; k++) dp[k] = d[k];
  }
}

// Properties of a boundary point from its primitives (the arithmetic of
// UpdatePropertiesFromPrimitive, src/prometeo_variables.hpp:62-89), then its
// conserved variables (UpdateConservedFromPrimitive, :91-130).
template <class Mix>
__device__ __noinline__ void boundary_properties(const UpdateArgs &A, const Mix &mix, const long long *p, double Pp,
                                                 double Tp, const double *x, const double *vel) {
  constexpr int NS = Mix::NS;
  double y[NS], d[NS];
  const double MixW = mix.MolarWeightFromXi(x);
  const double r = mix.Rho(Pp, Tp, MixW);
  *A.rho.at(p) = r;
  if constexpr (NS > 1) {
    double m, l;
    mix.TransportAt(Tp, Pp, MixW, x, m, l, d);
    *A.mu.at(p) = m;
    *A.lam.at(p) = l;
  } else {
    *A.mu.at(p) = mix.Viscosity(Tp, x);
    *A.lam.at(p) = mix.HeatConductivity(Tp, x);
    mix.Diffusivity(d, Pp, Tp, MixW, x);
  }
  mix.MassFractions(y, MixW, x);
  const double gamma = mix.Gamma(Tp, MixW, y);
  *A.SoS.at(p) = mix.SpeedOfSound(Tp, gamma, MixW);
  double *dp = A.Di.at(p), *yp = A.Y.at(p), *c = A.C.at(p);
#pragma unroll
  for (int k = 0; k < NS; k++) {
    dp[k] = d[k];
    yp[k] = y[k];
    c[k] = r * y[k];
  }
#pragma unroll
  for (int k = 0; k < 3; k++) c[NS + k] = r * vel[k];
  c[NS + 3] = r * (0.5 * mod2(vel) + mix.InternalEnergy(Tp, y));
}

// NSCBC inflow point after the RK update (SetNSCBC_InflowBCTask,
// src/prometeo_bc.hpp:108-150): imposed composition, temperature and
// velocity; pressure from the advanced density, or the imposed pressure of a
// supersonic inflow.
template <class Mix>
__device__ __noinline__ void inflow_refresh(const UpdateArgs &A, const Mix &mix, const long long *p, const double *u_,
                                            int side) {
  constexpr int NS = Mix::NS;
  double x[NS], vel[3];
#pragma unroll
  for (int k = 0; k < NS; k++) x[k] = ld(&A.Xp.at(p)[k]);
#pragma unroll
  for (int k = 0; k < 3; k++) vel[k] = ld(&A.up.at(p)[k]);
  const double T = ld(A.Tp.at(p));
  double P;
  if (fabs(vel[side / 2]) >= *A.SoS.at(p)) {
    P = A.Pbc[side];
  } else {
    double rhoYi[NS];
#pragma unroll
    for (int k = 0; k < NS; k++) rhoYi[k] = u_[k];
    P = mix.PFromRhoAndT(mix.RhoFromRhoYi(rhoYi), mix.MolarWeightFromXi(x), T);
  }
  double *xp = A.X.at(p), *vp = A.u.at(p);
#pragma unroll
  for (int k = 0; k < NS; k++) xp[k] = x[k];
#pragma unroll
  for (int k = 0; k < 3; k++) vp[k] = vel[k];
  *A.T.at(p) = T;
  *A.P.at(p) = P;
  boundary_properties(A, mix, p, P, T, x, vel);
}

// NSCBC outflow point after the first primitive recovery: the recovery again
// for each further outflow plane holding the point, then its properties and
// conserved variables (out of line: the boundary paths stay out of the
// per-cell kernel's hot instruction stream).
template <class Mix>
__device__ __noinline__ void outflow_refresh(const UpdateArgs &A, const Mix &mix, const long long *p, const double *u_,
                                             long long i, int n_out) {
  constexpr int NS = Mix::NS;
  const long long n = A.dn.count();
  for (int r = 1; r < n_out; r++) {
    double Td = 0.0, Ti = 0.0, lT = 0.0;
    if constexpr (NS > 1) {
      Td = *A.T.at(p) * mix.TRef;
      Ti = A.tcache[2 * n + i];
      lT = A.tcache[n + i];
    }
    refresh_cell(A, mix, p, u_, i, Td, Ti, lT, NS > 1);
  }
  double x[NS], vel[3];
  const double *xp = A.X.at(p), *vp = A.u.at(p);
#pragma unroll
  for (int k = 0; k < NS; k++) x[k] = xp[k];
#pragma unroll
  for (int k = 0; k < 3; k++) vel[k] = vp[k];
  boundary_properties(A, mix, p, *A.P.at(p), *A.T.at(p), x, vel);
}

// BC = false: periodic grids and Dirichlet ghosts (ghost nodes keep their
// state).  BC = true: the boundary step; a point with a staggered (wall)
// ghost node is not solved (the wall kernels refresh it after this kernel);
// a collocated NSCBC boundary point is solved without the flux divergence
// normal to its side(s), adds the NSCBC terms its plane kernels left in
// Conserved_t (zero at a supersonic inflow) and is refreshed by its side's
// rule: inflow (inflow wins an edge with an outflow), else the outflow's
// primitive recovery; then its properties and conserved variables.
template <class Mix, bool BC>
__global__ void __launch_bounds__(128) stage_update(const UpdateArgs A, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS, NE = NS + 4;
  const long long n = A.dn.count();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    A.dn.point(i, p);
    double ct[NE];
    if (A.mode == kStageImplicit) {
      // InitializeTimeDerivatives of implicit chemistry (src/prometeo_rk.rg:59-70)
      const double *o = A.Ctold.at(p);
#pragma unroll
      for (int k = 0; k < NE; k++) ct[k] = -ld(&o[k]);
    } else {
#pragma unroll
      for (int k = 0; k < NE; k++) ct[k] = 0.0;
    }
    unsigned div = A.active;  // directions whose flux divergence applies here
    bool bnd = false;         // on an NSCBC plane
    int inflow_side = -1;
    int n_out = 0;            // outflow planes holding this point
    bool skip = false;
    if constexpr (BC) {
#pragma unroll
      for (int D = 0; D < 3; D++) {
        if (!(A.active & (1u << D))) continue;
        const int t = ld(A.nt[D].at(p));
        if (t == L_S || t == R_S) skip = true;
        if (t == L_C || t == R_C) {
          div &= ~(1u << D);
          bnd = true;
          const int side = 2 * D + (t == R_C ? 1 : 0);
          if (A.bc[side] == kBcInflow && inflow_side < 0) inflow_side = side;
          if (A.bc[side] == kBcOutflow) n_out++;
        }
      }
    } else {
      // boundary ghosts keep their imposed state; their RHS is zero
#pragma unroll
      for (int D = 0; D < 3; D++)
        if (A.active & (1u << D)) skip = skip || ghost_node(ld(A.nt[D].at(p)));
    }
    if (skip) {
      double *ctp = A.Ct.at(p);
#pragma unroll
      for (int k = 0; k < NE; k++) ctp[k] = A.mode == kStageImplicit ? ct[k] : 0.0;
      continue;
    }
    // T, 1/T and log T of the current state: from the previous stage's
    // refresh when it computed them for this very T, else evaluated here
    double Td0 = 0.0, Tinv0 = 0.0, logT0 = 0.0;
    bool cached = false;
    if constexpr (NS > 1) {
      const double Tn0 = *A.T.at(p);
      Td0 = Tn0 * mix.TRef;
      if (__double_as_longlong(A.tcache[i]) == __double_as_longlong(Tn0)) {
        logT0 = A.tcache[n + i];
        Tinv0 = A.tcache[2 * n + i];
        cached = true;
      } else {
        Tinv0 = 1.0 / Td0;
        logT0 = log(Td0);
      }
    }
    if (A.chemistry) {
      double y[NS], w[NS];
#pragma unroll
      for (int k = 0; k < NS; k++) y[k] = ld(&A.Y.at(p)[k]);
      if constexpr (NS > 1)
        mix.ProductionRatesT(w, ld(A.rho.at(p)), ld(A.P.at(p)), Td0, Tinv0, logT0, y);
      else
        mix.ProductionRates(w, ld(A.rho.at(p)), ld(A.P.at(p)), ld(A.T.at(p)), y);
#pragma unroll
      for (int k = 0; k < NS; k++) ct[k] = __dadd_rn(ct[k], w[k]);
    }
    // flux differences: Euler Z, Y, X then diffusion Z, Y, X
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
#pragma unroll
      for (int dd = 2; dd >= 0; dd--) {
        if (!(div & (1u << dd))) continue;
        long long c1[3] = {p[0], p[1], p[2]};
        c1[dd] += 1;
        const long long nf = A.g.nf[dd];
        const long long fm = A.g.index(dd, p), fp = A.g.index(dd, c1);
        const double *F = pass == 0 ? A.fe[dd] : A.fd[dd];
        const double m = pass == 0 ? ld(A.me[dd].at(p)) : ld(A.md[dd].at(p));
#pragma unroll
        for (int k = 0; k < NE; k++) ct[k] = __fma_rn(m, __dsub_rn(F[k * nf + fp], F[k * nf + fm]), ct[k]);
      }
    }
    if constexpr (BC) {
      if (bnd) {
        // the NSCBC terms (src/prometeo.rg:592-605), added last
        const double *nb = A.Ct.at(p);
#pragma unroll
        for (int k = 0; k < NE; k++) ct[k] = __dadd_rn(ct[k], nb[k]);
        if (inflow_side >= 0) {
          const double un = A.u.at(p)[inflow_side / 2], c = A.SoS.at(p)[0];
          if ((inflow_side % 2 == 0) ? (un >= c) : (un <= -c)) {
#pragma unroll
            for (int k = 0; k < NE; k++) ct[k] = 0.0;
          }
        }
      }
    }
    double *ctp = A.Ct.at(p);
    if (A.mode == kStageRhsOnly) {
#pragma unroll
      for (int k = 0; k < NE; k++) ctp[k] = ct[k];
      continue;
    }
    // SSP-RK3 update (prometeo_rk.rg:88-112)
    double *cons = A.C.at(p);
    const double *old = A.Cold.at(p);
    double u_[NE];
    const double dtu = A.dt_cell ? ld(&A.dt_cell[i]) * A.dt_h : A.dt;
    // c1 old + c2 cons + c3 dt ct, contracted (rounding-level against the
    // reference's product-then-sum order)
    const double c3dt = A.c3 * dtu;
#pragma unroll
    for (int k = 0; k < NE; k++) {
      ctp[k] = ct[k];
      u_[k] = fma(A.c1, ld(&old[k]), fma(A.c2, cons[k], c3dt * ct[k]));
      cons[k] = u_[k];
    }
    if constexpr (BC) {
      // an NSCBC point keeps its stage state until boundary_refresh (after
      // this kernel) applies its side's rule, so no warp here diverges
      if (bnd) continue;
    }
    // primitive recovery (variables.hpp:163-193) and property refresh
    // (variables.hpp:62-89) of the new state
    refresh_cell(A, mix, p, u_, i, Td0, Tinv0, logT0, cached);
  }
}

// The NSCBC points of one boundary plane after the update, each refreshed
// once by the first NSCBC plane (in side order) that holds it: the inflow
// rule (inflow wins an edge with an outflow), else the outflow's primitive
// recovery, repeated once per outflow plane holding the point (an edge
// shared by two outflows is recovered twice, the second Newton starting
// from the first's temperature), then properties and conserved variables.
template <class Mix>
__global__ void boundary_refresh(const UpdateArgs A, const __grid_constant__ Mix mix, const Box plane, int side) {
  constexpr int NS = Mix::NS, NE = NS + 4;
  const long long np = plane.size(0) * plane.size(1) * plane.size(2);
  const long long n = A.dn.count();
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < np; q += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    p[0] = plane.lo[0] + q % plane.size(0);
    p[1] = plane.lo[1] + (q / plane.size(0)) % plane.size(1);
    p[2] = plane.lo[2] + q / (plane.size(0) * plane.size(1));
    int first_out = -1, inflow_side = -1, n_out = 0;
    bool wall = false;
#pragma unroll
    for (int D = 0; D < 3; D++) {
      if (!(A.active & (1u << D))) continue;
      const int t = ld(A.nt[D].at(p));
      if (t == L_S || t == R_S) wall = true;
      if (t == L_C || t == R_C) {
        const int s = 2 * D + (t == R_C ? 1 : 0);
        if (A.bc[s] == kBcInflow && inflow_side < 0) inflow_side = s;
        if (A.bc[s] == kBcOutflow) {
          if (first_out < 0) first_out = s;
          n_out++;
        }
      }
    }
    // the planes holding the point: its first inflow side alone (an inflow
    // wins an edge), else every outflow side; the first of them refreshes it
    const int owner = inflow_side >= 0 ? inflow_side : first_out;
    if (wall || owner != side) continue;
    double u_[NE];
    const double *cp = A.C.at(p);
#pragma unroll
    for (int k = 0; k < NE; k++) u_[k] = cp[k];
    if (inflow_side >= 0) {
      inflow_refresh(A, mix, p, u_, inflow_side);
      continue;
    }
    const long long i = A.dn.idx(p);
    double Td0 = 0.0, Tinv0 = 0.0, logT0 = 0.0;
    bool cached = false;
    if constexpr (NS > 1) {
      const double Tn0 = *A.T.at(p);
      Td0 = Tn0 * mix.TRef;
      if (__double_as_longlong(A.tcache[i]) == __double_as_longlong(Tn0)) {
        logT0 = A.tcache[n + i];
        Tinv0 = A.tcache[2 * n + i];
        cached = true;
      } else {
        Tinv0 = 1.0 / Td0;
        logT0 = log(Td0);
      }
    }
    refresh_cell(A, mix, p, u_, i, Td0, Tinv0, logT0, cached);
    outflow_refresh(A, mix, p, u_, i, n_out);
  }
}

// ---------------------------------------------------------------------------
template <class Mix>
cudaError_t launch_stage(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb, const Mix &mix,
                         const StageWorkspace &w, const StageParams &sp, int *status, cudaStream_t s,
                         cudaEvent_t *ev) {
  // ev (optional): ev[0] before the first kernel, ev[1 + k] after kernel k (StageKernel)
  auto mark = [&](int i) { return ev ? cudaEventRecord(ev[i], s) : cudaSuccess; };
  static const double RK[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
  const double c1 = RK[sp.stage - 1][0], c2 = RK[sp.stage - 1][1], c3 = RK[sp.stage - 1][2];
  const Dense dn = dense(my);
  const FaceGrid g = face_grid(my);
  const long long n = dn.count();
  double *prep = w.prep;
  cudaError_t e;
  if ((e = mark(0)) != cudaSuccess) return e;
  {
    PrepArgs A;
    A.u = fd<double>(v.velocity);
    A.X = fd<double>(v.MolarFracs);
    A.C = fd<double>(v.Conserved);
    A.P = fd<double>(v.pressure);
    A.rho = fd<double>(v.rho);
    A.m[0] = fd<double>(v.dcsi_d);
    A.m[1] = fd<double>(v.deta_d);
    A.m[2] = fd<double>(v.dzet_d);
    A.nt[0] = fd<int>(v.nType_x);
    A.nt[1] = fd<int>(v.nType_y);
    A.nt[2] = fd<int>(v.nType_z);
    A.fb = box(fb);
    A.dn = dn;
    A.prep = prep;
    const int pb = stage_tuning().prepass_block;
    stage_prepass<Mix><<<grid_for(n, pb), pb, 0, s>>>(A, mix);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(1 + kPrepass)) != cudaSuccess) return e;
  }
  Fd<double> H;
  H.b = reinterpret_cast<char *>(prep + 10 * n);
  H.s0 = sizeof(double);
  H.s1 = sizeof(double) * dn.n[0];
  H.s2 = sizeof(double) * dn.n[0] * dn.n[1];
  H.b -= (dn.lo[0] * H.s0 + dn.lo[1] * H.s1 + dn.lo[2] * H.s2);
  // RK_coeffs and deltaTime of the Euler limiter: the stage's; halved with
  // implicit chemistry; {0, 1} and dt/2 for the RHS of the implicit pre-step
  // (src/prometeo.rg:1363-1376, :1406-1419, UpdateDerivatives :498-512)
  double rk0 = c1, rk1 = c2, sdt = sp.dt * c3;
  StageParams ep = sp;
  ep.dtc_c3 = c3;
  ep.dtc_h = 1.0;
  if (sp.mode == kStageImplicit) {
    sdt = (sp.dt * c3) * 0.5;
    ep.dtc_h = 0.5;
  }
  if (sp.mode == kStageRhsOnly) {
    rk0 = 0.0;
    rk1 = 1.0;
    sdt = sp.dt * 0.5;
    ep.dtc_c3 = 1.0;
    ep.dtc_h = 0.5;
  }
  if ((e = launch_stage_euler(v, my, fb, mix, w, H, ep, rk0, rk1, sdt, s, ev ? ev + 1 + kKgZ : nullptr)) !=
      cudaSuccess)
    return e;
  const htr_field *ms[3] = {&v.dcsi_s, &v.deta_s, &v.dzet_s};
  const htr_field *nt[3] = {&v.nType_x, &v.nType_y, &v.nType_z};
  for (int D = 2; D >= 0; D--) {
    if (!(sp.active & (1u << D))) {
      if ((e = mark(1 + kDiffZ + (2 - D))) != cudaSuccess) return e;
      continue;
    }
    DiffFaceArgs A;
    A.C = fd<double>(v.Conserved);
    A.T = fd<double>(v.temperature);
    A.X = fd<double>(v.MolarFracs);
    A.rho = fd<double>(v.rho);
    A.mu = fd<double>(v.mu);
    A.lam = fd<double>(v.lam);
    A.Di = fd<double>(v.Di);
    A.u = fd<double>(v.velocity);
    A.ms = fd<double>(*ms[D]);
    A.nt = fd<int>(*nt[D]);
    A.my = box(my);
    A.fb = box(fb);
    A.dn = dn;
    A.prep = prep;
    A.g = g;
    A.fd = w.fd[D];
    A.tcache = w.tcache;
    const int db = stage_tuning().diffusion_block;
    const dim3 gr = grid_for(g.nf[D], db);
    if (D == 0) diffusion_faces<Mix, 0><<<gr, db, 0, s>>>(A, mix);
    else if (D == 1) diffusion_faces<Mix, 1><<<gr, db, 0, s>>>(A, mix);
    else diffusion_faces<Mix, 2><<<gr, db, 0, s>>>(A, mix);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(1 + kDiffZ + (2 - D))) != cudaSuccess) return e;
  }
  UpdateArgs U;
  U.C = fd<double>(v.Conserved);
  U.Cold = fd<double>(v.Conserved_old);
  U.Ct = fd<double>(v.Conserved_t);
  U.Ctold = fd<double>(v.Conserved_t_old);
  U.rho = fd<double>(v.rho);
  U.P = fd<double>(v.pressure);
  U.T = fd<double>(v.temperature);
  U.X = fd<double>(v.MolarFracs);
  U.Y = fd<double>(v.MassFracs);
  U.u = fd<double>(v.velocity);
  U.mu = fd<double>(v.mu);
  U.lam = fd<double>(v.lam);
  U.Di = fd<double>(v.Di);
  U.SoS = fd<double>(v.SoS);
  U.me[0] = fd<double>(v.dcsi_e);
  U.me[1] = fd<double>(v.deta_e);
  U.me[2] = fd<double>(v.dzet_e);
  U.md[0] = fd<double>(v.dcsi_d);
  U.md[1] = fd<double>(v.deta_d);
  U.md[2] = fd<double>(v.dzet_d);
  U.nt[0] = fd<int>(v.nType_x);
  U.nt[1] = fd<int>(v.nType_y);
  U.nt[2] = fd<int>(v.nType_z);
  U.active = sp.active;
  U.dn = dn;
  U.g = g;
  for (int D = 0; D < 3; D++) {
    U.fe[D] = w.fe[D];
    U.fd[D] = w.fd[D];
  }
  U.c1 = c1;
  U.c2 = c2;
  U.c3 = c3;
  // UpdateVars halves the step with implicit chemistry (src/prometeo_rk.rg:95-97)
  U.dt = sp.mode == kStageImplicit ? sp.dt * 0.5 : sp.dt;
  U.chemistry = sp.mode == kStageExplicit ? sp.chemistry : 0;
  U.mode = sp.mode;
  U.dt_cell = sp.dt_cell;
  U.dt_h = sp.mode == kStageImplicit ? 0.5 : 1.0;
  U.status = status;
  U.tcache = w.tcache;
  U.Xp = fd<double>(v.MolarFracs_profile);
  U.Tp = fd<double>(v.temperature_profile);
  U.up = fd<double>(v.velocity_profile);
  for (int k = 0; k < 6; k++) {
    U.bc[k] = sp.bc[k];
    U.Pbc[k] = sp.Pbc[k];
  }
  const int ub = stage_tuning().update_block;
  if (sp.boundary) {
    stage_update<Mix, true><<<grid_for(n, ub), ub, 0, s>>>(U, mix);
    for (int k = 0; k < 6; k++) {
      if (sp.bc[k] != kBcInflow && sp.bc[k] != kBcOutflow) continue;
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      const Box pl = box(sp.plane[k]);
      boundary_refresh<Mix><<<grid_for(pl.size(0) * pl.size(1) * pl.size(2), 128), 128, 0, s>>>(U, mix, pl, k);
    }
  } else {
    stage_update<Mix, false><<<grid_for(n, ub), ub, 0, s>>>(U, mix);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = mark(1 + kUpdate)) != cudaSuccess) return e;
  if constexpr (Mix::NS > 1) {
    if (sp.mode != kStageRhsOnly) {
      stage_transport<Mix><<<grid_for(n, 128), 128, 0, s>>>(U, mix);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  }
  return mark(1 + kTransport);
}

template cudaError_t launch_stage<ConstPropDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                                const ConstPropDev &, const StageWorkspace &, const StageParams &,
                                                int *, cudaStream_t, cudaEvent_t *);
template cudaError_t launch_stage<AirDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                          const AirDev &, const StageWorkspace &, const StageParams &, int *,
                                          cudaStream_t, cudaEvent_t *);

}  // namespace htr
