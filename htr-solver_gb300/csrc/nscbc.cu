// NSCBC boundary terms and the maximum Mach number of a direction.
//
// Replaces UpdateUsingFluxNSCBCInflow{Minus,Plus}SideTask and
// UpdateUsingFluxNSCBCOutflow{Minus,Plus}SideTask (src/prometeo_rhs.hpp:476-719,
// src/prometeo_rhs.inl:1284-1629, src/prometeo_rhs.cc:531-900) and
// CalculateMaxMachNumber (src/prometeo_stat.rg:223-234).
//
// One thread per point of the boundary plane (grid-stride).  Each point adds
// the LODI wave terms of a characteristic boundary to its Conserved_t using
// one-sided derivatives towards the first interior point
// (src/prometeo_metric.inl:95-102, src/Utils/PointDomain_helper.hpp:115-133).
#include "kernels.cuh"
#include "mixture.cuh"
#include "stencil.cuh"

namespace htr {

struct BcArgs {
  Fd<double> Y, P, u, rho, mu, SoS, T, C, Ct, dudt, dTdt, m[3];
  Fd<int> nt[3];
  Box bc, fb;
  long long n;  // points of the plane
  double MaxMach, LengthScale, PInf;
  const double *MaxMachDev;  // if set, MaxMach is read from device memory
};

HTR_D void plane_point(const BcArgs &a, long long idx, long long *p) {
  const long long nx = a.bc.size(0), ny = a.bc.size(1);
  p[0] = a.bc.lo[0] + idx % nx;
  p[1] = a.bc.lo[1] + (idx / nx) % ny;
  p[2] = a.bc.lo[2] + idx / (nx * ny);
}

HTR_D double dleft(int t, double x, double xp1, double m) { return (kNode[t].grad[1] * (xp1 - x)) * m; }
HTR_D double dright(int t, double xm1, double x, double m) { return (kNode[t].grad[0] * (x - xm1)) * m; }

// d(u_c)/dx_e at p with the node's periodic-wrapped stencil (metric.inl:104-135)
HTR_D double vderiv(const BcArgs &a, const long long *p, int c, int e) {
  const int t = ld(a.nt[e].at(p));
  const double m = ld(a.m[e].at(p));
  const long long size = a.fb.size(e);
  long long pm[3] = {p[0], p[1], p[2]}, pp[3] = {p[0], p[1], p[2]};
  pm[e] = wrap_minus(p[e], a.fb.lo[e], size, kNode[t].off[1]);
  pp[e] = wrap_plus(p[e], a.fb.lo[e], size, kNode[t].off[2]);
  return deriv(t, ld(&a.u.at(pm)[c]), ld(&a.u.at(p)[c]), ld(&a.u.at(pp)[c]), m);
}

template <class Mix, int DIR, bool MINUS>
__global__ void nscbc_inflow(const BcArgs a, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS, NE = NS + 4, iN = DIR;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < a.n;
       idx += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    plane_point(a, idx, p);
    double *RHS = a.Ct.at(p);
    const double un = ld(&a.u.at(p)[iN]), c = ld(a.SoS.at(p)), r = ld(a.rho.at(p)), T = ld(a.T.at(p));
    if (MINUS ? (un >= c) : (un <= -c)) {
#pragma unroll
      for (int l = 0; l < NE; l++) RHS[l] = 0.0;
      continue;
    }
    long long q[3] = {p[0], p[1], p[2]};
    q[DIR] += MINUS ? 1 : -1;
    const int t = ld(a.nt[DIR].at(p));
    const double m = ld(a.m[DIR].at(p));
    double Yp[NS], Yq[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) {
      Yp[s] = ld(&a.Y.at(p)[s]);
      Yq[s] = ld(&a.Y.at(q)[s]);
    }
    const double MixW_bnd = mix.MolarWeightFromYi(Yp);
    const double Cp_bnd = mix.HeatCapacity(T, Yp);
    const double lambda = un;
    double LS[NS], L1, LN;
    if (MINUS) {
      const double dp_dn = dleft(t, ld(a.P.at(p)), ld(a.P.at(q)), m);
      const double du_dn = dleft(t, un, ld(&a.u.at(q)[iN]), m);
      L1 = (un - c) * (dp_dn - r * c * du_dn);
#pragma unroll
      for (int s = 0; s < NS; s++) LS[s] = lambda * dleft(t, Yp[s], Yq[s], m);
      LN = L1 - 2 * r * c * ld(&a.dudt.at(p)[iN]);
    } else {
      const double dp_dn = dright(t, ld(a.P.at(q)), ld(a.P.at(p)), m);
      const double du_dn = dright(t, ld(&a.u.at(q)[iN]), un, m);
      LN = (un + c) * (dp_dn + r * c * du_dn);
#pragma unroll
      for (int s = 0; s < NS; s++) LS[s] = lambda * dright(t, Yq[s], Yp[s], m);
      L1 = LN + 2 * r * c * ld(&a.dudt.at(p)[iN]);
    }
    double L2 = ld(a.dTdt.at(p)) / T + (LN + L1) / (2 * r * Cp_bnd * T);
#pragma unroll
    for (int s = 0; s < NS; s++) L2 -= MixW_bnd / mix.SpeciesMolarWeight(s) * LS[s];
    L2 *= -r * c * c;
    const double d1 = (0.5 * (L1 + LN) - L2) / (c * c);
#pragma unroll
    for (int s = 0; s < NS; s++) RHS[s] -= (d1 * Yp[s] + r * LS[s]);
  }
}

template <class Mix, int DIR, bool MINUS>
__global__ void nscbc_outflow(const BcArgs a, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS, iN = DIR, iT1 = (DIR == 0) ? 1 : 0, iT2 = (DIR == 2) ? 1 : 2;
  constexpr int irU = NS, irE = NS + 3;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < a.n;
       idx += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    plane_point(a, idx, p);
    long long q[3] = {p[0], p[1], p[2]};
    q[DIR] += MINUS ? 1 : -1;
    double *RHS = a.Ct.at(p);
    const double *Cp = a.C.at(p);
    const double c = ld(a.SoS.at(p)), T = ld(a.T.at(p)), rp = ld(a.rho.at(p)), mup = ld(a.mu.at(p));
    const int t = ld(a.nt[DIR].at(p));
    const double m = ld(a.m[DIR].at(p));
    auto D = [&](double bnd, double in) { return MINUS ? dleft(t, bnd, in, m) : dright(t, in, bnd, m); };
    double up[3], uq[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      up[k] = ld(&a.u.at(p)[k]);
      uq[k] = ld(&a.u.at(q)[k]);
    }
    const double Pp = ld(a.P.at(p));
    const double dp_dn = D(Pp, ld(a.P.at(q)));
    const double dun_dn = D(up[iN], uq[iN]);
    const double duT1dn = D(up[iT1], uq[iT1]);
    const double duT2dn = D(up[iT2], uq[iT2]);
    const double un = up[iN];
    const double lambda_1 = un - c, lambda = un, lambda_N = un + c;
    const double lambda_s = MINUS ? smin(un, 0.0) : smax(un, 0.0);
    const double sigma = 0.25;
    const double MaxMach = a.MaxMachDev ? *a.MaxMachDev : a.MaxMach;
    const double K = (MaxMach < 0.99) ? sigma * (1.0 - MaxMach * MaxMach) * c / a.LengthScale
                                        : sigma * (c - (un * un) / c) / a.LengthScale;
    double Yp[NS], LS[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) {
      Yp[s] = ld(&a.Y.at(p)[s]);
      LS[s] = lambda_s * D(Yp[s], ld(&a.Y.at(q)[s]));
    }
    const double LM = lambda * (dp_dn - c * c * D(rp, ld(a.rho.at(q))));
    double L1, LN;
    if (MINUS) {
      L1 = lambda_1 * (dp_dn - rp * c * dun_dn);
      LN = (lambda_N < 0) ? lambda_N * (dp_dn + rp * c * dun_dn) : K * (Pp - a.PInf);
    } else {
      L1 = (lambda_1 > 0) ? lambda_1 * (dp_dn - rp * c * dun_dn) : K * (Pp - a.PInf);
      LN = lambda_N * (dp_dn + rp * c * dun_dn);
    }
    const double d1 = (0.5 * (L1 + LN) - LM) / (c * c);
    double dM[3];
    dM[iN] = (LN - L1) / (2 * rp * c);
    dM[iT1] = lambda * duT1dn;
    dM[iT2] = lambda * duT2dn;
    const double dN = LM / (c * c);
    const double vT1_T1 = vderiv(a, p, iT1, iT1), vT2_T2 = vderiv(a, p, iT2, iT2);
    const double vT1_N = vderiv(a, p, iN, iT1), vT2_N = vderiv(a, p, iN, iT2);
    const double tauNN_bnd = mup * (4 * dun_dn - 2 * vT1_T1 - 2 * vT2_T2) / 3;
    const double tauNN_int = ld(a.mu.at(q)) *
                             (4 * vderiv(a, q, iN, DIR) - 2 * vderiv(a, q, iT1, iT1) - 2 * vderiv(a, q, iT2, iT2)) / 3;
    const double dtau_dn = D(tauNN_bnd, tauNN_int);
    const double viscous_heating = D(un * tauNN_bnd, uq[iN] * tauNN_int) + duT1dn * mup * (duT1dn + vT1_N) +
                                   duT2dn * mup * (duT2dn + vT2_N);
    const double cpT = mix.HeatCapacity(T, Yp) * T;
#pragma unroll
    for (int s = 0; s < NS; s++) RHS[s] -= (d1 * Yp[s] + rp * LS[s]);
    RHS[irU + iN] -= (up[iN] * d1 + rp * dM[iN] - dtau_dn);
    RHS[irU + iT1] -= (up[iT1] * d1 + rp * dM[iT1]);
    RHS[irU + iT2] -= (up[iT2] * d1 + rp * dM[iT2]);
    double dE = (ld(&Cp[irE]) + Pp) * d1 / rp + ld(&Cp[irU + iN]) * dM[iN] + ld(&Cp[irU + iT1]) * dM[iT1] +
                ld(&Cp[irU + iT2]) * dM[iT2] + cpT * dN - viscous_heating;
    RHS[irE] -= dE;
    const double cpT_Wmix = cpT * mix.MolarWeightFromYi(Yp);
#pragma unroll
    for (int s = 0; s < NS; s++) {
      const double dEdYi = mix.SpeciesEnthalpy(s, T) - cpT_Wmix / mix.SpeciesMolarWeight(s);
      RHS[irE] -= (rp * LS[s] * dEdYi);
    }
  }
}

// Non-negative doubles order like their bit patterns: an unsigned 64-bit
// atomicMax reduces them exactly.
__global__ void max_mach_kernel(const BcArgs a, int dir, unsigned long long *out) {
  double best = 0.0;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < a.n;
       idx += (long long)gridDim.x * blockDim.x) {
    long long p[3];
    plane_point(a, idx, p);
    best = smax(best, fabs(ld(&a.u.at(p)[dir])) / ld(a.SoS.at(p)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = smax(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

static BcArgs bc_args(const htr_fluid_view &v, const htr_rect3 &bc, const htr_rect3 &fb) {
  BcArgs a;
  a.Y = fd<double>(v.MassFracs);
  a.P = fd<double>(v.pressure);
  a.u = fd<double>(v.velocity);
  a.rho = fd<double>(v.rho);
  a.mu = fd<double>(v.mu);
  a.SoS = fd<double>(v.SoS);
  a.T = fd<double>(v.temperature);
  a.C = fd<double>(v.Conserved);
  a.Ct = fd<double>(v.Conserved_t);
  a.dudt = fd<double>(v.dudtBoundary);
  a.dTdt = fd<double>(v.dTdtBoundary);
  a.m[0] = fd<double>(v.dcsi_d);
  a.m[1] = fd<double>(v.deta_d);
  a.m[2] = fd<double>(v.dzet_d);
  a.nt[0] = fd<int>(v.nType_x);
  a.nt[1] = fd<int>(v.nType_y);
  a.nt[2] = fd<int>(v.nType_z);
  a.bc = box(bc);
  a.fb = box(fb);
  a.n = a.bc.size(0) * a.bc.size(1) * a.bc.size(2);
  a.MaxMach = a.LengthScale = a.PInf = 0.0;
  a.MaxMachDev = nullptr;
  return a;
}

static dim3 plane_grid(long long n) {
  long long b = (n + 127) / 128;
  if (b > 152LL * 16) b = 152LL * 16;
  return dim3((unsigned)(b > 0 ? b : 1));
}

template <class Mix, int DIR, bool MINUS>
static cudaError_t inflow_dir(const BcArgs &a, const Mix &mix, cudaStream_t s) {
  nscbc_inflow<Mix, DIR, MINUS><<<plane_grid(a.n), 128, 0, s>>>(a, mix);
  return cudaGetLastError();
}
template <class Mix, int DIR, bool MINUS>
static cudaError_t outflow_dir(const BcArgs &a, const Mix &mix, cudaStream_t s) {
  nscbc_outflow<Mix, DIR, MINUS><<<plane_grid(a.n), 128, 0, s>>>(a, mix);
  return cudaGetLastError();
}

template <class Mix>
cudaError_t launch_nscbc_inflow(const htr_fluid_view &v, const htr_rect3 &bc, const Mix &mix, int dir, bool minus,
                                cudaStream_t s) {
  const BcArgs a = bc_args(v, bc, bc);
  if (dir == 0) return minus ? inflow_dir<Mix, 0, true>(a, mix, s) : inflow_dir<Mix, 0, false>(a, mix, s);
  if (dir == 1) return minus ? inflow_dir<Mix, 1, true>(a, mix, s) : inflow_dir<Mix, 1, false>(a, mix, s);
  return minus ? inflow_dir<Mix, 2, true>(a, mix, s) : inflow_dir<Mix, 2, false>(a, mix, s);
}

template <class Mix>
cudaError_t launch_nscbc_outflow(const htr_fluid_view &v, const htr_rect3 &bc, const htr_rect3 &fb, const Mix &mix,
                                 int dir, bool minus, double MaxMach, double LengthScale, double PInf,
                                 cudaStream_t s, const double *MaxMachDev) {
  BcArgs a = bc_args(v, bc, fb);
  a.MaxMach = MaxMach;
  a.MaxMachDev = MaxMachDev;
  a.LengthScale = LengthScale;
  a.PInf = PInf;
  if (dir == 0) return minus ? outflow_dir<Mix, 0, true>(a, mix, s) : outflow_dir<Mix, 0, false>(a, mix, s);
  if (dir == 1) return minus ? outflow_dir<Mix, 1, true>(a, mix, s) : outflow_dir<Mix, 1, false>(a, mix, s);
  return minus ? outflow_dir<Mix, 2, true>(a, mix, s) : outflow_dir<Mix, 2, false>(a, mix, s);
}

cudaError_t launch_max_mach(const htr_fluid_view &v, const htr_rect3 &my, int dir, double *result, cudaStream_t s) {
  const BcArgs a = bc_args(v, my, my);
  cudaError_t e = cudaMemsetAsync(result, 0, sizeof(double), s);
  if (e != cudaSuccess) return e;
  max_mach_kernel<<<plane_grid(a.n), 128, 0, s>>>(a, dir, reinterpret_cast<unsigned long long *>(result));
  return cudaGetLastError();
}

#define HTR_INST(MIX)                                                                                         \
  template cudaError_t launch_nscbc_inflow<MIX>(const htr_fluid_view &, const htr_rect3 &, const MIX &, int,  \
                                                bool, cudaStream_t);                                         \
  template cudaError_t launch_nscbc_outflow<MIX>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &, \
                                                 const MIX &, int, bool, double, double, double, cudaStream_t, \
                                                 const double *);
HTR_INST(ConstPropDev)
HTR_INST(AirDev)
#undef HTR_INST

}  // namespace htr
