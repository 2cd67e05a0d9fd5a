// Diffusion fluxes: viscous stress, Fourier heat flux and mixture-averaged
// species diffusion with mass-conserving correction and enthalpy transport.
//
// Replaces UpdateUsingDiffusionFluxTask<dir> (src/prometeo_rhs.hpp:368-473,
// src/prometeo_rhs.inl:1054-1282, GPU variant src/prometeo_rhs.cu:482-627).
//
// Same tiling as the Euler kernel: each face of a block's tile is computed
// once into shared memory, then every cell takes m_d * (F(i+1/2) - F(i-1/2)).
// The species enthalpies at the face temperature are evaluated once per face
// (the reference evaluates them twice, with identical results).
#include "kernels.cuh"
#include "mixture.cuh"
#include "stencil.cuh"

namespace htr {

struct DiffArgs {
  Fd<double> C, T, X, rho, mu, lam, Di, u, ms, md, md1, md2, Ct;
  Fd<int> nt, nt1, nt2;
  Box my, fb;
};

template <int D> struct DTile {
  static constexpr int L = (D == 0) ? 1 : 32;
  static constexpr int S = (D == 0) ? 256 : 8;
  static constexpr int NF = L * (S + 1);
};

template <class Mix, int D>
__global__ void __launch_bounds__(256) diffusion_kernel(const DiffArgs a, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS, NE = NS + 4, iU = NS, iE = NS + 3;
  constexpr int T1 = (D == 0) ? 1 : 0, T2 = (D == 2) ? 1 : 2;
  using TL = DTile<D>;
  extern __shared__ double smem[];
  double *Fs = smem;  // [NE][NF]

  long long o[3];
  if (D == 0) {
    o[0] = a.my.lo[0] + (long long)blockIdx.x * TL::S;
    o[1] = a.my.lo[1] + blockIdx.y;
    o[2] = a.my.lo[2] + blockIdx.z;
  } else if (D == 1) {
    o[0] = a.my.lo[0] + (long long)blockIdx.x * TL::L;
    o[1] = a.my.lo[1] + (long long)blockIdx.y * TL::S;
    o[2] = a.my.lo[2] + blockIdx.z;
  } else {
    o[0] = a.my.lo[0] + (long long)blockIdx.x * TL::L;
    o[1] = a.my.lo[1] + blockIdx.y;
    o[2] = a.my.lo[2] + (long long)blockIdx.z * TL::S;
  }
  const long long nseg = min((long long)TL::S, a.my.hi[D] - o[D] + 1);
  const int nlines = (D == 0) ? 1 : (int)min((long long)TL::L, a.my.hi[0] - o[0] + 1);
  const int nface = nlines * (int)(nseg + 1);

  auto shifted = [&](long long *q, const long long *p, int e, int off, bool plus) {
    q[0] = p[0];
    q[1] = p[1];
    q[2] = p[2];
    q[e] = plus ? wrap_plus(p[e], a.fb.lo[e], a.fb.size(e), off)
                : wrap_minus(p[e], a.fb.lo[e], a.fb.size(e), off);
  };
  // velocity gradient along e at point p (metric.inl:103-134)
  auto grad = [&](double *g, const long long *p, int e, const Fd<int> &ntt, const Fd<double> &mm) {
    const int t = ld(ntt.at(p));
    long long pm[3], pp[3];
    shifted(pm, p, e, kNode[t].off[1], false);
    shifted(pp, p, e, kNode[t].off[2], true);
    const double m = ld(mm.at(p));
#pragma unroll
    for (int i = 0; i < 3; i++)
      g[i] = deriv(t, ld(&a.u.at(pm)[i]), ld(&a.u.at(p)[i]), ld(&a.u.at(pp)[i]), m);
  };

  for (int f = threadIdx.x; f < nface; f += blockDim.x) {
    const int l = (D == 0) ? 0 : f % nlines;
    const int j = (D == 0) ? f : f / nlines;
    long long c[3] = {o[0], o[1], o[2]};
    if (D != 0) c[0] += l;
    c[D] += j;  // cell right of the face
    long long p[3];
    if (j == 0 && c[D] == a.my.lo[D]) {
      const int t0 = ld(a.nt.at(c));
      shifted(p, c, D, kNode[t0].off[1], false);
    } else {
      p[0] = c[0];
      p[1] = c[1];
      p[2] = c[2];
      p[D] = c[D] - 1;
    }
    long long q[3];
    shifted(q, p, D, 1, true);
    const int t = ld(a.nt.at(p));
    const double m_s = ld(a.ms.at(p));
    double g1p[3], g1q[3], g2p[3], g2q[3];
    grad(g1p, p, T1, a.nt1, a.md1);
    grad(g2p, p, T2, a.nt2, a.md2);
    grad(g1q, q, T1, a.nt1, a.md1);
    grad(g2q, q, T2, a.nt2, a.md2);
    double Xp[NS], Xq[NS];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      Xp[i] = ld(&a.X.at(p)[i]);
      Xq[i] = ld(&a.X.at(q)[i]);
    }
    const double rho_s = interp2(t, ld(a.rho.at(p)), ld(a.rho.at(q)));
    const double iMixW_s = 1.0 / interp2(t, mix.MolarWeightFromXi(Xp), mix.MolarWeightFromXi(Xq));
    const double Tp = ld(a.T.at(p)), Tq = ld(a.T.at(q));
    const double T_s = interp2(t, Tp, Tq);
    double heat = interp2(t, ld(a.lam.at(p)), ld(a.lam.at(q))) * m_s * (Tp - Tq);
    double F[NE];
    if constexpr (NS > 1) {
      double h[NS];
      mix.SpeciesEnthalpies(h, T_s);
      double ViCorr = 0.0;
#pragma unroll
      for (int i = 0; i < NS; i++) {
        const double YiVi = interp2(t, ld(&a.Di.at(p)[i]), ld(&a.Di.at(q)[i])) * m_s * (Xp[i] - Xq[i]) *
                            mix.SpeciesMolarWeight(i) * iMixW_s;
        F[i] = -rho_s * YiVi;
        heat += rho_s * YiVi * h[i];
        ViCorr += YiVi;
      }
#pragma unroll
      for (int i = 0; i < NS; i++) {
        const double cc = interp2(t, ld(&a.C.at(p)[i]), ld(&a.C.at(q)[i])) * ViCorr;
        F[i] += cc;
        heat -= cc * h[i];
      }
    } else {
      // single species: Di == 0 in the reference mixture (ConstPropMix.inl:149)
      const double h0 = mix.SpeciesEnthalpy(0, T_s);
      const double YiVi = interp2(t, ld(&a.Di.at(p)[0]), ld(&a.Di.at(q)[0])) * m_s * (Xp[0] - Xq[0]) *
                          mix.SpeciesMolarWeight(0) * iMixW_s;
      F[0] = -rho_s * YiVi;
      heat += rho_s * YiVi * h0;
      const double cc = interp2(t, ld(&a.C.at(p)[0]), ld(&a.C.at(q)[0])) * YiVi;
      F[0] += cc;
      heat -= cc * h0;
    }
    // viscous stress (rhs.inl:1058-1137)
    const double mu_s = interp2(t, ld(a.mu.at(p)), ld(a.mu.at(q)));
    double up[3], uq[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      up[i] = ld(&a.u.at(p)[i]);
      uq[i] = ld(&a.u.at(q)[i]);
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
    for (int i = 0; i < NE; i++) Fs[i * TL::NF + f] = F[i];
  }
  __syncthreads();
  const int ncell = nlines * (int)nseg;
  for (int cidx = threadIdx.x; cidx < ncell; cidx += blockDim.x) {
    const int l = (D == 0) ? 0 : cidx % nlines;
    const int j = (D == 0) ? cidx : cidx / nlines;
    long long p[3] = {o[0], o[1], o[2]};
    if (D != 0) p[0] += l;
    p[D] += j;
    const int fm = (D == 0) ? j : j * nlines + l;
    const int fp = (D == 0) ? j + 1 : (j + 1) * nlines + l;
    double *ct = a.Ct.at(p);
    const double m = ld(a.md.at(p));
#pragma unroll
    for (int i = 0; i < NE; i++) ct[i] += m * (Fs[i * TL::NF + fp] - Fs[i * TL::NF + fm]);
  }
}

template <class Mix, int D>
static cudaError_t launch_dir(const DiffArgs &a, const Mix &mix, cudaStream_t s) {
  using TL = DTile<D>;
  const long long n[3] = {a.my.size(0), a.my.size(1), a.my.size(2)};
  dim3 grid;
  if (D == 0) grid = dim3((unsigned)((n[0] + TL::S - 1) / TL::S), (unsigned)n[1], (unsigned)n[2]);
  else if (D == 1) grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)((n[1] + TL::S - 1) / TL::S), (unsigned)n[2]);
  else grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)n[1], (unsigned)((n[2] + TL::S - 1) / TL::S));
  const size_t sm = sizeof(double) * (Mix::NS + 4) * TL::NF;
  auto k = diffusion_kernel<Mix, D>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, 256, sm, s>>>(a, mix);
  return cudaGetLastError();
}

template <class Mix>
cudaError_t launch_diffusion(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                             const Mix &mix, int dir, cudaStream_t s) {
  DiffArgs a;
  a.C = fd<double>(v.Conserved);
  a.T = fd<double>(v.temperature);
  a.X = fd<double>(v.MolarFracs);
  a.rho = fd<double>(v.rho);
  a.mu = fd<double>(v.mu);
  a.lam = fd<double>(v.lam);
  a.Di = fd<double>(v.Di);
  a.u = fd<double>(v.velocity);
  a.Ct = fd<double>(v.Conserved_t);
  const htr_field *ms[3] = {&v.dcsi_s, &v.deta_s, &v.dzet_s};
  const htr_field *md[3] = {&v.dcsi_d, &v.deta_d, &v.dzet_d};
  const htr_field *nt[3] = {&v.nType_x, &v.nType_y, &v.nType_z};
  const int t1 = dir == 0 ? 1 : 0, t2 = dir == 2 ? 1 : 2;
  a.ms = fd<double>(*ms[dir]);
  a.md = fd<double>(*md[dir]);
  a.md1 = fd<double>(*md[t1]);
  a.md2 = fd<double>(*md[t2]);
  a.nt = fd<int>(*nt[dir]);
  a.nt1 = fd<int>(*nt[t1]);
  a.nt2 = fd<int>(*nt[t2]);
  a.my = box(my);
  a.fb = box(fb);
  if (dir == 0) return launch_dir<Mix, 0>(a, mix, s);
  if (dir == 1) return launch_dir<Mix, 1>(a, mix, s);
  return launch_dir<Mix, 2>(a, mix, s);
}

template cudaError_t launch_diffusion<ConstPropDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                                    const ConstPropDev &, int, cudaStream_t);
template cudaError_t launch_diffusion<AirDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                              const AirDev &, int, cudaStream_t);

}  // namespace htr
