/* htr_gb300 — C ABI of the GB300 (sm_103a) explicit right-hand side of HTR.
 *
 * Each entry point replaces one HTR Legion task on the RHS path.  The
 * reference task bodies are `T::cpu_base_impl` / `T::gpu_base_impl`
 * (signature src/Utils/task_helper.hpp:108-122) registered from
 * register_rhs_tasks() (src/prometeo_rhs.h:39), register_sensor_tasks(),
 * register_chem_tasks() and register_variables_tasks().  Where a task reads
 * its arguments from `Args` and its data from Legion regions, the entry
 * point here takes:
 *
 *   - `view`         per-field device pointers with byte strides (the Realm
 *                    AffineAccessor of every field of Fluid_columns,
 *                    src/prometeo_types.h:49-114);
 *   - `my_fluid`     the task's execution rectangle (`r_MyFluid`, the index
 *                    space of the region the task writes);
 *   - `fluid_bounds` `Args::Fluid_bounds` (the whole grid, used for periodic
 *                    wrap by warpPeriodic, src/Utils/PointDomain_helper.hpp:160-190);
 *   - `mix`          a handle made by htr_load_mixture (replaces `Args::mix`
 *                    and the `__constant__ Mix` that LoadMixtureTask fills,
 *                    src/prometeo_mixture.cu:32-47);
 *   - scalar task arguments (`RK_coeffs`, the `deltaTime` future, ...);
 *   - `stream`       the CUDA stream to run on (the task's stream in Legion).
 *
 * Every call is asynchronous on `stream`, allocates nothing in steady state
 * and returns an htr_status.  Buffers are owned by the caller and must stay
 * valid until the stream has passed the call.  A field element is the
 * reference's element type (double, int nType, bool sensor, or an array of
 * double for VecNEq / VecNSp / Vec3) with components contiguous; strides
 * are free (Legion's default layout is x fastest, one array per field).
 */
#ifndef HTR_RHS_H
#define HTR_RHS_H

#include <stddef.h>
#include <stdint.h>

#include "htr_mix.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *htr_stream_t;

typedef enum {
  HTR_OK = 0,
  HTR_ERR_ARGUMENT = 1,      /* null pointer, inverted rectangle, wrong EOS */
  HTR_ERR_LAYOUT = 2,        /* stride not a multiple of the element size, misaligned base */
  HTR_ERR_CUDA = 3,          /* a CUDA call failed (message in htr_last_error) */
  HTR_ERR_ITERATION_CAP = 4, /* a device Newton / Rosenbrock loop hit its cap */
  HTR_ERR_UNSUPPORTED = 5,   /* configuration the library does not support (e.g. other mixtures) */
  HTR_ERR_NO_DEVICE = 6,     /* no usable sm_103 device */
  HTR_ERR_IO = 7,            /* a file could not be opened, read or written */
  HTR_ERR_FORMAT = 8         /* a file is not HDF5, is truncated, or lacks what a restart holds */
} htr_status;

/* One field: address of grid point (0,0,0) (it may lie outside the
 * allocation when the instance does not start at the origin) and byte
 * strides between neighbouring points in x, y and z. */
typedef struct {
  void *base;
  int64_t stride[3];
} htr_field;

/* Inclusive rectangle, like Legion::Rect<3>. */
typedef struct {
  int64_t lo[3];
  int64_t hi[3];
} htr_rect3;

/* The fields of Fluid_columns that the RHS path touches, in declaration
 * order (src/prometeo_types.h:49-114).  Unused fields may be left null. */
typedef struct {
  htr_field nType_x, nType_y, nType_z;       /* int  */
  htr_field dcsi_e, deta_e, dzet_e;          /* double, Euler metrics */
  htr_field dcsi_d, deta_d, dzet_d;          /* double, diffusion metrics */
  htr_field dcsi_s, deta_s, dzet_s;          /* double, staggered metrics */
  htr_field rho, mu, lam, Di, SoS;           /* Di: VecNSp */
  htr_field pressure, temperature;
  htr_field MassFracs, MolarFracs, velocity; /* VecNSp, VecNSp, Vec3 */
  htr_field Conserved, Conserved_old, Conserved_t, Conserved_t_old; /* VecNEq */
  htr_field shockSensorX, shockSensorY, shockSensorZ;               /* bool */
  htr_field DucrosSensor;
  htr_field dudtBoundary, dTdtBoundary;  /* Vec3, double: NSCBC inflow data */
  htr_field velocity_old_NSCBC, temperature_old_NSCBC;  /* Vec3, double */
  htr_field MolarFracs_profile, velocity_profile, temperature_profile; /* VecNSp, Vec3, double */
} htr_fluid_view;

typedef struct htr_mixture_s *htr_mixture_t;

/* --- device / mixture management ---------------------------------------- */

/* Text of the last error on the calling thread ("" if none). */
const char *htr_last_error(void);

/* Replaces LoadMixtureTask (src/prometeo_mixture.cu:32-47): copies the
 * mixture (a htr_constpropmix_t or htr_airmix_t, `bytes` = its size) to the
 * current device and derives the per-species constants the kernels use. */
int htr_load_mixture(int eos, const void *mix, size_t bytes, htr_mixture_t *out);
int htr_free_mixture(htr_mixture_t mix);
int htr_mixture_eos(htr_mixture_t mix);

/* Builders for callers without the reference struct.  They restate the
 * mixture constructors Mix(const Config&) of src/Mixtures/ConstPropMix.inl:31-51
 * and src/Mixtures/AirMix.hpp:319-332 (+ StoreReferenceQuantities,
 * src/Mixtures/MultiComponent.inl:438-487). */
int htr_constpropmix_init(double gasConstant, double gamma, double prandtl, int viscosityModel,
                          double p0, double p1, double p2, htr_constpropmix_t *out);
int htr_airmix_init(double PRef, double TRef, double LRef, const double XiRef[HTR_AIR_NSPEC],
                    htr_airmix_t *out);

/* --- Euler fluxes (src/prometeo_rhs.hpp:171-366, src/prometeo_rhs.cc:35-406) --
 * Conserved_t[p] += m_e[p] * (F(p+1/2) - F(p-1/2)) over `my_fluid`.
 * Hybrid: KG split form where shockSensor is true at p-1, p, p+1, TENO
 * otherwise.  rk_coeffs / delta_time feed the positivity limiter of
 * multi-species mixtures (the `deltaTime` future of the reference task). */
int htr_UpdateUsingHybridEulerFluxX(const htr_fluid_view *view, htr_rect3 my_fluid,
                                    htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                    double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingHybridEulerFluxY(const htr_fluid_view *view, htr_rect3 my_fluid,
                                    htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                    double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingHybridEulerFluxZ(const htr_fluid_view *view, htr_rect3 my_fluid,
                                    htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                    double delta_time, htr_mixture_t mix, htr_stream_t stream);
/* TENO (eps 1e-10), TENO-A (eps 1e-8) and TENO-LAD (eps 1e-16) everywhere
 * (UpdateUsingTENOEulerFluxTask<dir, Op>, src/prometeo_rhs.hpp:243-310). */
int htr_UpdateUsingTENOEulerFluxX(const htr_fluid_view *view, htr_rect3 my_fluid,
                                  htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                  double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOEulerFluxY(const htr_fluid_view *view, htr_rect3 my_fluid,
                                  htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                  double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOEulerFluxZ(const htr_fluid_view *view, htr_rect3 my_fluid,
                                  htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                  double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOAEulerFluxX(const htr_fluid_view *view, htr_rect3 my_fluid,
                                   htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                   double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOAEulerFluxY(const htr_fluid_view *view, htr_rect3 my_fluid,
                                   htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                   double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOAEulerFluxZ(const htr_fluid_view *view, htr_rect3 my_fluid,
                                   htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                   double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOLADEulerFluxX(const htr_fluid_view *view, htr_rect3 my_fluid,
                                     htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                     double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOLADEulerFluxY(const htr_fluid_view *view, htr_rect3 my_fluid,
                                     htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                     double delta_time, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingTENOLADEulerFluxZ(const htr_fluid_view *view, htr_rect3 my_fluid,
                                     htr_rect3 fluid_bounds, const double rk_coeffs[2],
                                     double delta_time, htr_mixture_t mix, htr_stream_t stream);
/* Kennedy-Gruber skew-symmetric flux everywhere (src/prometeo_rhs.hpp:312-366). */
int htr_UpdateUsingSkewSymmetricEulerFluxX(const htr_fluid_view *view, htr_rect3 my_fluid,
                                           htr_rect3 fluid_bounds, htr_mixture_t mix,
                                           htr_stream_t stream);
int htr_UpdateUsingSkewSymmetricEulerFluxY(const htr_fluid_view *view, htr_rect3 my_fluid,
                                           htr_rect3 fluid_bounds, htr_mixture_t mix,
                                           htr_stream_t stream);
int htr_UpdateUsingSkewSymmetricEulerFluxZ(const htr_fluid_view *view, htr_rect3 my_fluid,
                                           htr_rect3 fluid_bounds, htr_mixture_t mix,
                                           htr_stream_t stream);

/* --- diffusion fluxes (src/prometeo_rhs.hpp:368-473, src/prometeo_rhs.cc:408-527) -- */
int htr_UpdateUsingDiffusionFluxX(const htr_fluid_view *view, htr_rect3 my_fluid,
                                  htr_rect3 fluid_bounds, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingDiffusionFluxY(const htr_fluid_view *view, htr_rect3 my_fluid,
                                  htr_rect3 fluid_bounds, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingDiffusionFluxZ(const htr_fluid_view *view, htr_rect3 my_fluid,
                                  htr_rect3 fluid_bounds, htr_mixture_t mix, htr_stream_t stream);

/* --- shock sensors (src/prometeo_sensor.hpp:49-131, src/prometeo_sensor.cc:33-128) -- */
int htr_UpdateDucrosSensor(const htr_fluid_view *view, htr_rect3 my_fluid,
                           htr_rect3 fluid_bounds, double vorticityScale, htr_stream_t stream);
int htr_UpdateShockSensorX(const htr_fluid_view *view, htr_rect3 my_fluid,
                           htr_rect3 fluid_bounds, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateShockSensorY(const htr_fluid_view *view, htr_rect3 my_fluid,
                           htr_rect3 fluid_bounds, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateShockSensorZ(const htr_fluid_view *view, htr_rect3 my_fluid,
                           htr_rect3 fluid_bounds, htr_mixture_t mix, htr_stream_t stream);

/* --- chemistry (src/prometeo_chem.hpp:96-150, src/prometeo_chem.cc:31-110) -- */
int htr_AddChemistrySources(const htr_fluid_view *view, htr_rect3 my_fluid, htr_mixture_t mix,
                            htr_stream_t stream);
/* Implicit Rosenbrock chemistry over Integrator_deltaTime.  `status` (device
 * int, may be null) receives HTR_ERR_ITERATION_CAP if any cell hit a cap. */
int htr_UpdateChemistry(const htr_fluid_view *view, htr_rect3 my_fluid,
                        double Integrator_deltaTime, htr_mixture_t mix, int *status,
                        htr_stream_t stream);

/* --- per-cell state refresh (src/prometeo_variables.hpp:52-210) ---------- */
int htr_UpdatePropertiesFromPrimitive(const htr_fluid_view *view, htr_rect3 my_fluid,
                                      htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateConservedFromPrimitive(const htr_fluid_view *view, htr_rect3 my_fluid,
                                     htr_mixture_t mix, htr_stream_t stream);
int htr_UpdatePrimitiveFromConserved(const htr_fluid_view *view, htr_rect3 my_fluid,
                                     htr_mixture_t mix, htr_stream_t stream);

/* --- time step (src/prometeo_cfl.hpp:55-190, src/prometeo.rg:1159-1166) --
 * Writes max over my_fluid of the spectral radius to *result_dev (device
 * double). */
int htr_CalculateMaxSpectralRadius(const htr_fluid_view *view, htr_rect3 my_fluid,
                                   htr_mixture_t mix, double *result_dev, htr_stream_t stream);

/* --- grid metrics (set-up of a stretched grid) -----------------------------
 * InitializeMetricTask (src/prometeo_metric.hpp:93-181,
 * src/prometeo_metric.cc:36-178): the Euler (dcsi_e, deta_e, dzet_e),
 * collocated diffusion (d*_d) and staggered (d*_s) metrics of every point of
 * my_fluid from the cell-centre coordinates (Vec3 per point) and the node
 * types; width[3] are the domain widths (bBox extents) used to unwarp
 * periodic stencils.  CorrectGhostMetricTask<dir> (src/prometeo_metric.hpp:
 * 183-268, src/prometeo_metric.cc:180-213): the Euler metric of direction
 * dir at the boundary nodes (L_S, L_C, R_S, R_C) of my_fluid from one-sided
 * coordinate differences.  Both write only metric fields. */
int htr_InitializeMetric(const htr_fluid_view *view, htr_field centerCoordinates, htr_rect3 my_fluid,
                         htr_rect3 fluid_bounds, const double width[3], htr_stream_t stream);
int htr_CorrectGhostMetricX(const htr_fluid_view *view, htr_field centerCoordinates, htr_rect3 my_fluid,
                            htr_stream_t stream);
int htr_CorrectGhostMetricY(const htr_fluid_view *view, htr_field centerCoordinates, htr_rect3 my_fluid,
                            htr_stream_t stream);
int htr_CorrectGhostMetricZ(const htr_fluid_view *view, htr_field centerCoordinates, htr_rect3 my_fluid,
                            htr_stream_t stream);

/* --- SSP-RK3 bookkeeping (Regent tasks of src/prometeo_rk.rg:47-112) ---- */
int htr_InitializeTemporaries(const htr_fluid_view *view, htr_rect3 my_fluid,
                              htr_mixture_t mix, htr_stream_t stream);
int htr_InitializeTimeDerivatives(const htr_fluid_view *view, htr_rect3 my_fluid,
                                  int implicitChemistry, htr_mixture_t mix, htr_stream_t stream);
/* stage in {1,2,3}: Conserved = C1*Conserved_old + C2*Conserved + C3*Conserved_t*dt. */
int htr_UpdateVars(const htr_fluid_view *view, htr_rect3 my_fluid, int stage, double deltaTime,
                   int implicitChemistry, htr_mixture_t mix, htr_stream_t stream);

/* --- NSCBC boundary terms (src/prometeo_rhs.hpp:476-719,
 * src/prometeo_rhs.inl:1284-1629, src/prometeo_rhs.cc:531-900) -------------
 * Add the LODI terms of a characteristic boundary to Conserved_t on the
 * boundary plane `bc` (the task's BC region).  Inflow: species terms of a
 * subsonic inlet whose velocity and temperature are imposed (dudtBoundary,
 * dTdtBoundary); the RHS is zeroed at a supersonic inlet.  Outflow: partially
 * non-reflecting outlet relaxed towards PInf with the maximum Mach number
 * MaxMach of the normal velocity (htr_CalculateMaxMachNumber) and
 * LengthScale; fluid_bounds bounds the tangential stencils. */
int htr_UpdateUsingFluxNSCBCInflowXNeg(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCInflowXPos(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCInflowYNeg(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCInflowYPos(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCInflowZNeg(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCInflowZPos(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCOutflowXNeg(const htr_fluid_view *view, htr_rect3 bc, htr_rect3 fluid_bounds,
                                        htr_mixture_t mix, double MaxMach, double LengthScale, double PInf,
                                        htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCOutflowXPos(const htr_fluid_view *view, htr_rect3 bc, htr_rect3 fluid_bounds,
                                        htr_mixture_t mix, double MaxMach, double LengthScale, double PInf,
                                        htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCOutflowYNeg(const htr_fluid_view *view, htr_rect3 bc, htr_rect3 fluid_bounds,
                                        htr_mixture_t mix, double MaxMach, double LengthScale, double PInf,
                                        htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCOutflowYPos(const htr_fluid_view *view, htr_rect3 bc, htr_rect3 fluid_bounds,
                                        htr_mixture_t mix, double MaxMach, double LengthScale, double PInf,
                                        htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCOutflowZNeg(const htr_fluid_view *view, htr_rect3 bc, htr_rect3 fluid_bounds,
                                        htr_mixture_t mix, double MaxMach, double LengthScale, double PInf,
                                        htr_stream_t stream);
int htr_UpdateUsingFluxNSCBCOutflowZPos(const htr_fluid_view *view, htr_rect3 bc, htr_rect3 fluid_bounds,
                                        htr_mixture_t mix, double MaxMach, double LengthScale, double PInf,
                                        htr_stream_t stream);
/* --- boundary-condition state updates --------------------------------------
 * Primitive variables of the boundary points after each RK stage
 * (UpdateGhostPrimitives, src/prometeo_bc.rg:1160-1279):
 *   NSCBC inflow   SetNSCBC_InflowBCTask<dir> (src/prometeo_bc.hpp:108-150,
 *                  src/prometeo_bc.cc:84-135): imposed profile; pressure from
 *                  the advanced density unless the inflow is supersonic (Pbc)
 *   NSCBC outflow  SetNSCBC_OutflowBCTask (src/prometeo_bc.cc:160-197):
 *                  primitive recovery of the advanced boundary point
 *   isothermal wall / adiabatic wall (src/prometeo_bc.rg:1207-1263): wall
 *                  ghost at rest with the first interior point's pressure and
 *                  composition, temperature from the wall profile / interior
 * and the NSCBC time derivatives of the imposed inflow after a time step
 * (UpdateNSCBCGhostCellTimeDerivatives, src/prometeo_bc.rg:1794-1810). */
int htr_SetNSCBC_InflowBCX(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, double Pbc, htr_stream_t stream);
int htr_SetNSCBC_InflowBCY(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, double Pbc, htr_stream_t stream);
int htr_SetNSCBC_InflowBCZ(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, double Pbc, htr_stream_t stream);
int htr_SetNSCBC_OutflowBC(const htr_fluid_view *view, htr_rect3 bc, htr_mixture_t mix, int *status_dev,
                           htr_stream_t stream);
/* side: 0 XNeg, 1 XPos, 2 YNeg, 3 YPos, 4 ZNeg, 5 ZPos */
int htr_SetIsothermalWallBC(const htr_fluid_view *view, htr_rect3 bc, int side, htr_mixture_t mix,
                            htr_stream_t stream);
int htr_SetAdiabaticWallBC(const htr_fluid_view *view, htr_rect3 bc, int side, htr_mixture_t mix,
                           htr_stream_t stream);
int htr_UpdateNSCBCGhostCellTimeDerivatives(const htr_fluid_view *view, htr_rect3 bc, double deltaTime,
                                            htr_stream_t stream);

/* max |velocity[dir]| / SoS over my_fluid (CalculateMaxMachNumber,
 * src/prometeo_stat.rg:223-234); the result is written to *result (device
 * pointer for the CUDA library, host pointer for the CPU oracle). */
int htr_CalculateMaxMachNumber(const htr_fluid_view *view, htr_rect3 my_fluid, int dir, double *result,
                               htr_stream_t stream);

/* --- fused time step (the driver of src/prometeo.rg:1153-1172, 1342-1486) --
 * Not a reference task: one whole SSP-RK3 step of a periodic grid
 * (sensors once per step, then per stage: RHS in the reference's order
 * chemistry -> Euler Z,Y,X -> diffusion Z,Y,X, RK update, primitive and
 * property refresh), asynchronous on `stream`.  With cfl > 0 the step size
 * is cfl / max spectral radius (one device-to-host read of the radius);
 * otherwise deltaTime is used and the call issues no synchronisation, so it
 * can be captured in a CUDA graph. */
typedef enum {
  HTR_SCHEME_HYBRID = 0,
  HTR_SCHEME_TENO = 1,
  HTR_SCHEME_TENOA = 2,
  HTR_SCHEME_TENOLAD = 3,
  HTR_SCHEME_SKEW = 4
} htr_scheme;

typedef struct {
  int scheme;               /* htr_scheme */
  double vorticityScale;    /* Ducros sensor scale of the hybrid scheme */
  double cfl;               /* > 0: CFL-based step size */
  double deltaTime;         /* used when cfl <= 0 */
  int explicitChemistry;    /* add chemistry sources to the RHS */
  /* Integrator.implicitChemistry (src/prometeo.rg:1360-1398): chemistry is
   * advanced by the implicit Rosenbrock solver instead of explicit sources.
   * After the sensors: the transport RHS of the step's start state
   * (RK_coeffs {0, 1}, deltaTime dt/2), UpdateChemistry over dt with that
   * RHS frozen, primitive and property refresh, then the three RK stages with
   * Conserved_t starting from -Conserved_t_old and dt halved
   * (src/prometeo_rk.rg:59-112).  explicitChemistry is ignored when set.
   * Supported by htr_rk3_step, htr_rk3_step_ws and htr_rk3_step_static;
   * htr_rk3_step_bc_ws returns HTR_ERR_UNSUPPORTED. */
  int implicitChemistry;
} htr_step_params;

int htr_rk3_step(const htr_fluid_view *view, htr_rect3 interior, htr_rect3 fluid_bounds,
                 const htr_step_params *params, htr_mixture_t mix, double *dt_used,
                 int *status_dev, htr_stream_t stream);

/* --- fused time step on a caller-provided workspace -------------------------
 * Not a reference task.  The same SSP-RK3 step as htr_rk3_step, computed by
 * the fused stage pipeline: per stage one per-cell prepass (velocity
 * gradients, molar weight, total enthalpy), Kennedy-Gruber faces of every
 * direction from shared-memory tiles with the sensor-rejected faces queued
 * for one load-balanced TENO kernel, diffusion faces, and one per-cell kernel
 * (chemistry sources, flux differences in the reference's order, RK update,
 * primitive recovery, property refresh).  Each face flux is computed once.
 * Grids periodic in every direction only (interior == fluid_bounds);
 * otherwise HTR_ERR_UNSUPPORTED.  `workspace` is device memory of at least
 * htr_rk3_workspace_bytes(interior, mix) bytes, 256-byte aligned, owned by
 * the caller; the call allocates nothing. */
size_t htr_rk3_workspace_bytes(htr_rect3 interior, htr_mixture_t mix);
int htr_rk3_step_ws(const htr_fluid_view *view, htr_rect3 interior, htr_rect3 fluid_bounds,
                    const htr_step_params *params, htr_mixture_t mix, void *workspace,
                    size_t workspace_bytes, double *dt_used, int *status_dev, htr_stream_t stream);

/* No reference counterpart: htr_rk3_step_ws with one step size per cell, for
 * many independent instances packed into one grid (the batched form: tubes
 * end to end in a strip, separated by their boundary ghost nodes).
 * `dt_cell` is device memory of one double per interior cell, dense with x
 * fastest; the cells of one instance share that instance's step size, so
 * each instance advances exactly as htr_rk3_step_ws would advance it alone
 * with its own deltaTime (RK update and positivity-limiter deltaTime per
 * cell).  params->cfl must be <= 0; params->deltaTime is not used. */
int htr_rk3_step_cells_ws(const htr_fluid_view *view, htr_rect3 interior, htr_rect3 fluid_bounds,
                          const htr_step_params *params, htr_mixture_t mix, const double *dt_cell,
                          void *workspace, size_t workspace_bytes, int *status_dev, htr_stream_t stream);

/* --- fused time step of a grid with boundary conditions --------------------
 * Not a reference task.  One SSP-RK3 step of the reference driver
 * (src/prometeo.rg:1342-1486, UpdateDerivatives :480-606,
 * UpdatePrimitivesAndBCsFromConserved :428-478) for a grid with NSCBC inflow
 * and outflow sides and isothermal or adiabatic walls, one ghost layer on
 * each non-periodic side (interior = fluid_bounds shrunk by one there), on
 * the fused stage pipeline run over the whole grid.  Per stage: the NSCBC
 * terms of every outflow plane (the interior's maximum Mach number stays on
 * the device) and inflow plane from the stage's state; prepass, Euler and
 * diffusion faces; one per-cell kernel in which a collocated boundary point
 * skips the flux divergence normal to its side, adds its NSCBC terms and
 * takes its side's state rule, and wall ghosts (never solved) are refreshed
 * from their first interior point after it (walls z, y, x).  After the step
 * the inflow time derivatives.  Zones as the reference's partitioner makes
 * them: bc->plane[s] is the side's p_xNeg[0]... (its face plus the edges and
 * corners it wins).  Schemes: all five; for the hybrid scheme the Ducros
 * sensor is computed everywhere and the shock sensors once per step over
 * bc->sensor[d] (UpdateShockSensors, src/prometeo_sensor.rg:96-125).
 * Workspace: htr_rk3_workspace_bytes(fluid_bounds, mix) bytes.  With cfl <= 0
 * the call issues no host synchronisation (CUDA-graph capturable). */
typedef enum {
  HTR_BC_PERIODIC = 0,
  HTR_BC_NSCBC_INFLOW = 1,
  HTR_BC_NSCBC_OUTFLOW = 2,
  HTR_BC_ISOTHERMAL_WALL = 3,
  HTR_BC_ADIABATIC_WALL = 4
} htr_bc_type;

typedef struct {
  int type[6];           /* htr_bc_type of xNeg, xPos, yNeg, yPos, zNeg, zPos */
  double P[6];           /* inflow: pressure of a supersonic inflow; outflow: PInf */
  double LengthScale[6]; /* outflow: relaxation length */
  htr_rect3 plane[6];    /* boundary points of each non-periodic side */
  htr_rect3 sensor[3];   /* hybrid scheme: the points whose shock sensor of
                            direction d is computed (p_x_faces ...); the others
                            keep their value (true after initialisation) */
} htr_bc_params;

int htr_rk3_step_bc_ws(const htr_fluid_view *view, htr_rect3 interior, htr_rect3 fluid_bounds,
                       const htr_step_params *params, const htr_bc_params *bc, htr_mixture_t mix,
                       void *workspace, size_t workspace_bytes, double *dt_used, int *status_dev,
                       htr_stream_t stream);

/* No counterpart in the reference.  The fused step of htr_rk3_step_ws on a
 * fixed scratch that the library owns: a module-scope device array of
 * htr_rk3_static_scratch_bytes() bytes, reserved on a device when the
 * module holding it loads there and kept until the process exits.
 * htr_load_mixture loads that module and resolves the array's address for
 * its current device, so once a mixture was loaded on the device the call
 * allocates no device or host memory; on a device where no mixture was
 * loaded, the first call does that set-up (make it before any stream
 * capture).  (Under CUDA's lazy module loading the first launch of each of
 * the library's kernels in a process loads that kernel's module, whichever
 * entry point launches it; CUDA_MODULE_LOADING=EAGER loads them all when the
 * library loads.)  After a cudaDeviceReset, load the mixture again.
 * Grids whose workspace (htr_rk3_workspace_bytes) exceeds the scratch are
 * rejected with HTR_ERR_UNSUPPORTED before any launch.  Calls share the
 * scratch of their device: run them on one stream (or serialise them),
 * never concurrently. */
int htr_rk3_step_static(const htr_fluid_view *view, htr_rect3 interior, htr_rect3 fluid_bounds,
                        const htr_step_params *params, htr_mixture_t mix, double *dt_used,
                        int *status_dev, htr_stream_t stream);
size_t htr_rk3_static_scratch_bytes(void);

/* Launch shapes of the fused stage, no counterpart in the reference
 * (process-wide; chosen by the autotuner of the batched form).  Allowed:
 * prepass_block 64/128/256, diffusion_block and update_block 32/64/128,
 * teno_blocks_per_sm 0..32 (0: the TENO queue kernel runs one queued face per
 * thread, its grid sized to the direction's face count; 1..32: that many
 * blocks per SM stride over the queue), kg_x_tile 64/128/256.  Defaults 256,
 * 128, 128, 0, 128.  Set it before launching (or capturing) the steps that use it. */
typedef struct {
  int prepass_block, diffusion_block, update_block, teno_blocks_per_sm, kg_x_tile;
} htr_stage_tuning;
int htr_rk3_set_tuning(const htr_stage_tuning *tuning);
int htr_rk3_get_tuning(htr_stage_tuning *tuning);

/* Profiling aid, no counterpart in the reference: copies Conserved to
 * Conserved_old, runs stage 1 of the fused pipeline once (deltaTime, no
 * sensor update) with CUDA events between its kernels, waits for it, and
 * writes the milliseconds of each kernel to ms_out[10]: prepass, KG faces Z,
 * Y, X, TENO faces, diffusion faces Z, Y, X, per-cell update, transport
 * properties (multi-species mixtures; 0 for a single species).  The state
 * advances by that forward-Euler stage. */
int htr_rk3_stage_profile(const htr_fluid_view *view, htr_rect3 interior, htr_rect3 fluid_bounds,
                          const htr_step_params *params, htr_mixture_t mix, void *workspace,
                          size_t workspace_bytes, float *ms_out, htr_stream_t stream);

/* Diagnostic, no counterpart in the reference: the numbers of faces of
 * directions X, Y, Z that the last fused hybrid stage run on `workspace`
 * (htr_rk3_step_ws, htr_rk3_stage_profile) reconstructed with TENO (the
 * shock-sensor-rejected faces of its TENO queues); waits for `stream`.
 * TENO-only schemes reconstruct every face and queue none. */
int htr_rk3_teno_face_counts(htr_rect3 interior, htr_mixture_t mix, const void *workspace, size_t workspace_bytes,
                             unsigned long long counts[3], htr_stream_t stream);

/* Diagnostic counters, no counterpart in the reference.  The kernels decide
 * TENO stencil selections and shock sensors first with single-precision
 * filters and fall back to the exact double-precision expression of the
 * reference when a value lies within the filter's safety margin; the
 * multi-species TENO flux may blend with the first-order flux (positivity
 * limiter).  htr_decision_counters waits for the device, adds the counts
 * gathered since the previous call to counts[0..6] (TENO selections filtered,
 * TENO selections exact, sensor nodes filtered, sensor nodes exact, sensor
 * cut-offs filtered, sensor cut-offs exact, limiter blends), clears them and
 * switches counting on (enable != 0) or off for later launches.  Counting
 * costs an atomic per decision: it is off by default. */
#define HTR_DECISION_COUNTERS 7
int htr_decision_counters(int enable, unsigned long long counts[HTR_DECISION_COUNTERS]);

#ifdef __cplusplus
}
#endif

#endif /* HTR_RHS_H */
