// Launchers of the htr_gb300 kernels (host-callable, one per kernel family).
#pragma once

#include "common.cuh"

namespace htr {

struct ConstPropDev;
struct AirDev;

// scheme: 0 hybrid, 1 skew-symmetric, 2 TENO-only; kind: 0 TENO, 1 TENO-A, 2 TENO-LAD
template <class Mix>
cudaError_t launch_euler(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                         const double *rk, double dt, const Mix &mix, int dir, int scheme, int kind,
                         cudaStream_t s);

template <class Mix>
cudaError_t launch_diffusion(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                             const Mix &mix, int dir, cudaStream_t s);

// grid metrics (metric.cu): all three directions over my; Euler metric of the
// boundary nodes of direction dir
cudaError_t launch_init_metric(const htr_fluid_view &v, const htr_field &cc, const htr_rect3 &my,
                               const htr_rect3 &fb, const double *width, cudaStream_t s);
cudaError_t launch_correct_metric(const htr_fluid_view &v, const htr_field &cc, const htr_rect3 &my, int dir,
                                  cudaStream_t s);

cudaError_t launch_ducros(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                          double vorticityScale, cudaStream_t s);
// dirmask: bit d set = compute the sensor of direction d
cudaError_t launch_shock_sensor(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                                int nspec, int dirmask, cudaStream_t s);

template <class Mix>
cudaError_t launch_chem_sources(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                                cudaStream_t s);
template <class Mix>
cudaError_t launch_properties(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                              cudaStream_t s);
template <class Mix>
cudaError_t launch_conserved(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                             cudaStream_t s);
// skip_ghosts (bit d: direction d has more than one cell): leave boundary
// ghost nodes alone (packed instances; 0 = every cell of my)
template <class Mix>
cudaError_t launch_primitive(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                             int *status, cudaStream_t s, unsigned skip_ghosts = 0);
template <class Mix>
cudaError_t launch_spectral_radius(const htr_fluid_view &v, const htr_rect3 &my, const Mix &mix,
                                   double *result, cudaStream_t s);
template <class Mix>
// dt_cell (optional): one step size per cell of `my`, dense with x fastest,
// replacing dt
cudaError_t launch_update_chemistry(const htr_fluid_view &v, const htr_rect3 &my, double dt,
                                    const Mix &mix, int *status, cudaStream_t s, unsigned skip_ghosts = 0,
                                    const double *dt_cell = nullptr);

// NSCBC boundary terms on the plane `bc` (dir 0..2, minus = the "Neg" side)
template <class Mix>
cudaError_t launch_nscbc_inflow(const htr_fluid_view &v, const htr_rect3 &bc, const Mix &mix, int dir, bool minus,
                                cudaStream_t s);
template <class Mix>
cudaError_t launch_nscbc_outflow(const htr_fluid_view &v, const htr_rect3 &bc, const htr_rect3 &fb, const Mix &mix,
                                 int dir, bool minus, double MaxMach, double LengthScale, double PInf,
                                 cudaStream_t s, const double *MaxMachDev = nullptr);
cudaError_t launch_max_mach(const htr_fluid_view &v, const htr_rect3 &my, int dir, double *result, cudaStream_t s);

// boundary-point state updates (side: 0 XNeg .. 5 ZPos)
template <class Mix>
cudaError_t launch_inflow_state(const htr_fluid_view &v, const htr_rect3 &bc, const Mix &mix, double Pbc, int dir,
                                cudaStream_t s);
cudaError_t launch_wall_state(const htr_fluid_view &v, const htr_rect3 &bc, int nspec, int side, bool isothermal,
                              cudaStream_t s);
cudaError_t launch_nscbc_time_derivatives(const htr_fluid_view &v, const htr_rect3 &bc, double dt, cudaStream_t s);

// SSP-RK3 bookkeeping; neq = number of conserved components
cudaError_t launch_copy_conserved(const htr_fluid_view &v, const htr_rect3 &my, int neq, cudaStream_t s);
cudaError_t launch_init_rhs(const htr_fluid_view &v, const htr_rect3 &my, int neq, int implicit,
                            cudaStream_t s);
cudaError_t launch_rk_update(const htr_fluid_view &v, const htr_rect3 &my, int neq, int stage,
                             double dt, int implicit, cudaStream_t s);

// decision counters of the translation units that take filtered decisions
// (stencil.cuh): add this unit's counts to out[], clear them, set counting
cudaError_t decision_counters_euler(int enable, unsigned long long *out);
cudaError_t decision_counters_stage_euler(int enable, unsigned long long *out);
cudaError_t decision_counters_sensor(int enable, unsigned long long *out);

}  // namespace htr
