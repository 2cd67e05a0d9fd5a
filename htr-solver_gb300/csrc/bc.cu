// Boundary-condition state updates of the boundary points after a stage.
//
//   SetNSCBC_InflowBCTask<dir>   src/prometeo_bc.hpp:108-150, src/prometeo_bc.cc:84-135
//   SetNSCBC_OutflowBCTask       src/prometeo_bc.cc:160-197 (per-cell primitive
//                                recovery, src/prometeo_variables.hpp:163-193)
//   SetIsothermalWallBC / SetAdiabaticWallBC   src/prometeo_bc.rg:1207-1263
//   UpdateNSCBCGhostCellTimeDerivatives        src/prometeo_bc.rg:1794-1810
// One thread per boundary point (grid-stride over the plane).
#include "kernels.cuh"
#include "mixture.cuh"

namespace htr {

struct StateArgs {
  Fd<double> C, SoS, Xp, Tp, up, P, T, X, u, dudt, dTdt, uo, To;
  Box bc;
  long long n;
};

HTR_D void bc_point(const StateArgs &a, long long idx, long long *p) {
  const long long nx = a.bc.size(0), ny = a.bc.size(1);
  p[0] = a.bc.lo[0] + idx % nx;
  p[1] = a.bc.lo[1] + (idx / nx) % ny;
  p[2] = a.bc.lo[2] + idx / (nx * ny);
}

#define HTR_FOR_PLANE(A, IDX) \
  for (long long IDX = blockIdx.x * (long long)blockDim.x + threadIdx.x; IDX < (A).n; IDX += (long long)gridDim.x * blockDim.x)

template <class Mix>
__global__ void inflow_state(const StateArgs a, double Pbc, int dir, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS;
  HTR_FOR_PLANE(a, idx) {
    long long p[3];
    bc_point(a, idx, p);
    double xp[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) {
      xp[s] = ld(&a.Xp.at(p)[s]);
      a.X.at(p)[s] = xp[s];
    }
    const double Tp = ld(a.Tp.at(p));
    *a.T.at(p) = Tp;
    double up[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      up[i] = ld(&a.up.at(p)[i]);
      a.u.at(p)[i] = up[i];
    }
    if (fabs(up[dir]) >= ld(a.SoS.at(p))) {
      *a.P.at(p) = Pbc;
    } else {
      double rhoYi[NS];
#pragma unroll
      for (int s = 0; s < NS; s++) rhoYi[s] = ld(&a.C.at(p)[s]);
      const double rho = mix.RhoFromRhoYi(rhoYi);
      *a.P.at(p) = mix.PFromRhoAndT(rho, mix.MolarWeightFromXi(xp), Tp);
    }
  }
}

template <int NS>
__global__ void wall_state(const StateArgs a, int d, int step, bool isothermal) {
  HTR_FOR_PLANE(a, idx) {
    long long p[3];
    bc_point(a, idx, p);
    long long q[3] = {p[0], p[1], p[2]};
    q[d] += step;
#pragma unroll
    for (int s = 0; s < NS; s++) a.X.at(p)[s] = ld(&a.X.at(q)[s]);
    *a.P.at(p) = ld(a.P.at(q));
    *a.T.at(p) = isothermal ? ld(a.Tp.at(p)) : ld(a.T.at(q));
#pragma unroll
    for (int i = 0; i < 3; i++) a.u.at(p)[i] = 0.0;
  }
}

__global__ void nscbc_time_derivatives(const StateArgs a, double dt) {
  HTR_FOR_PLANE(a, idx) {
    long long p[3];
    bc_point(a, idx, p);
    double *uo = a.uo.at(p), *du = a.dudt.at(p);
    const double *u = a.u.at(p);
#pragma unroll
    for (int i = 0; i < 3; i++) du[i] = (u[i] - uo[i]) / dt;
    *a.dTdt.at(p) = (*a.T.at(p) - *a.To.at(p)) / dt;
#pragma unroll
    for (int i = 0; i < 3; i++) uo[i] = u[i];
    *a.To.at(p) = *a.T.at(p);
  }
}

static StateArgs state_args(const htr_fluid_view &v, const htr_rect3 &bc) {
  StateArgs a;
  a.C = fd<double>(v.Conserved);
  a.SoS = fd<double>(v.SoS);
  a.Xp = fd<double>(v.MolarFracs_profile);
  a.Tp = fd<double>(v.temperature_profile);
  a.up = fd<double>(v.velocity_profile);
  a.P = fd<double>(v.pressure);
  a.T = fd<double>(v.temperature);
  a.X = fd<double>(v.MolarFracs);
  a.u = fd<double>(v.velocity);
  a.dudt = fd<double>(v.dudtBoundary);
  a.dTdt = fd<double>(v.dTdtBoundary);
  a.uo = fd<double>(v.velocity_old_NSCBC);
  a.To = fd<double>(v.temperature_old_NSCBC);
  a.bc = box(bc);
  a.n = a.bc.size(0) * a.bc.size(1) * a.bc.size(2);
  return a;
}

static dim3 plane_blocks(long long n) {
  long long b = (n + 127) / 128;
  if (b > 152LL * 16) b = 152LL * 16;
  return dim3((unsigned)(b > 0 ? b : 1));
}

template <class Mix>
cudaError_t launch_inflow_state(const htr_fluid_view &v, const htr_rect3 &bc, const Mix &mix, double Pbc, int dir,
                                cudaStream_t s) {
  const StateArgs a = state_args(v, bc);
  inflow_state<Mix><<<plane_blocks(a.n), 128, 0, s>>>(a, Pbc, dir, mix);
  return cudaGetLastError();
}

cudaError_t launch_wall_state(const htr_fluid_view &v, const htr_rect3 &bc, int nspec, int side, bool isothermal,
                              cudaStream_t s) {
  const StateArgs a = state_args(v, bc);
  const int d = side / 2, step = (side % 2 == 0) ? 1 : -1;
  if (nspec == 1) wall_state<1><<<plane_blocks(a.n), 128, 0, s>>>(a, d, step, isothermal);
  else if (nspec == 5) wall_state<5><<<plane_blocks(a.n), 128, 0, s>>>(a, d, step, isothermal);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_nscbc_time_derivatives(const htr_fluid_view &v, const htr_rect3 &bc, double dt, cudaStream_t s) {
  const StateArgs a = state_args(v, bc);
  nscbc_time_derivatives<<<plane_blocks(a.n), 128, 0, s>>>(a, dt);
  return cudaGetLastError();
}

template cudaError_t launch_inflow_state<ConstPropDev>(const htr_fluid_view &, const htr_rect3 &, const ConstPropDev &,
                                                       double, int, cudaStream_t);
template cudaError_t launch_inflow_state<AirDev>(const htr_fluid_view &, const htr_rect3 &, const AirDev &, double,
                                                 int, cudaStream_t);

}  // namespace htr
