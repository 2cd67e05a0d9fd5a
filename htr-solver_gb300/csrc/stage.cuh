// Fused RK-stage pipeline: face-flux buffers and their launchers.
//
// htr_rk3_step evaluates one stage as
//   euler_kg_faces (Z, Y, X)  Kennedy-Gruber faces of every pencil tile from a
//                             shared-memory window; faces the hybrid sensor
//                             rejects go to one device-wide TENO queue
//   euler_teno_faces          the queued (or, for TENO schemes, all) faces,
//                             load-balanced over the whole GPU
//   diffusion_faces (Z, Y, X) viscous / heat / species faces
//   stage_update              per cell: chemistry + flux differences in the
//                             reference's order, RK update, primitive (Newton)
//                             and property refresh
// Face fluxes live in a caller-provided workspace (structure of arrays,
// component-major); each face is computed once.
#pragma once

#include "common.cuh"

namespace htr {

// Faces of direction D are indexed by the cell on their right, c in
// [lo_D, hi_D + 1] x the other two extents of the interior.
struct FaceGrid {
  long long lo[3];
  long long ext[3][3];  // ext[D][axis]
  long long nf[3];      // faces per direction
  HTR_HD long long index(int D, const long long *c) const {
    return (c[0] - lo[0]) + ext[D][0] * ((c[1] - lo[1]) + ext[D][1] * (c[2] - lo[2]));
  }
};

inline FaceGrid face_grid(const htr_rect3 &r) {
  FaceGrid g;
  long long n[3];
  for (int i = 0; i < 3; i++) {
    g.lo[i] = r.lo[i];
    n[i] = r.hi[i] - r.lo[i] + 1;
  }
  for (int D = 0; D < 3; D++) {
    for (int i = 0; i < 3; i++) g.ext[D][i] = n[i] + (i == D ? 1 : 0);
    g.nf[D] = g.ext[D][0] * g.ext[D][1] * g.ext[D][2];
  }
  return g;
}

// A queued TENO face: direction and right cell.
struct TenoEntry {
  int D, c0, c1, c2;
};

struct StageWorkspace {
  double *fe[3];    // Euler face fluxes, [NE][nf[D]]
  double *fd[3];    // diffusion face fluxes, [NE][nf[D]]
  TenoEntry *queue; // capacity nf[0]+nf[1]+nf[2]: the faces of direction D from offset nf[0]+..+nf[D-1]
  unsigned *count;  // queue lengths of the three directions
  double *prep;     // per-cell prepass values, [kPrepVals][ncell]
  double *tcache;   // per cell: T it was computed for, log(T TRef), 1/(T TRef), species h and c_p; [3 + 2 NS][ncell]
  double *scalars;  // 3 doubles in the counters' 256-byte block (maximum Mach number per direction)
};

// per-cell prepass values: velocity-gradient tensor (9), mixture molar
// weight (1), total enthalpy H (1)
constexpr int kPrepVals = 11;

size_t stage_workspace_bytes(const htr_rect3 &interior, int neq);
bool stage_workspace_carve(void *base, size_t bytes, const htr_rect3 &interior, int neq, StageWorkspace &w);

// What one launch_stage computes.
enum StageMode {
  kStageExplicit = 0,  // RHS from zero (+ chemistry sources), RK update, refresh
  kStageImplicit = 1,  // implicit chemistry: RHS from -Conserved_t_old, no sources,
                       // RK update with dt/2 (src/prometeo_rk.rg:59-112), refresh
  kStageRhsOnly = 2    // transport RHS of the current state into Conserved_t only
                       // (RK_coeffs {0, 1}, limiter deltaTime dt/2, src/prometeo.rg:1363-1376)
};

struct StageParams {
  int scheme;  // 0 hybrid, 1 skew, 2 TENO-only
  int kind;    // TENO flavour for scheme 2
  int chemistry;
  int stage;   // 1..3
  double dt;   // full step size
  int mode = kStageExplicit;
  // optional per-cell step sizes (dense over the interior, x fastest) of
  // independent instances packed into one grid; dt above is then unused.
  // dtc_c3 / dtc_h: the factors launch_stage derives from the stage and mode
  // (the limiter's deltaTime is (dt_cell * dtc_c3) * dtc_h)
  const double *dt_cell = nullptr;
  double dtc_c3 = 1.0, dtc_h = 1.0;
  // bit D set: direction D has more than one cell.  A one-cell periodic
  // direction contributes exactly zero to every flux difference (both faces
  // see the same cell), so its faces are not computed.
  unsigned active;
  // Boundary conditions (the boundary step only): kind of each side (BcKind,
  // xNeg, xPos, yNeg, yPos, zNeg, zPos) and the pressure of a supersonic
  // NSCBC inflow.  boundary = 0 keeps the periodic / Dirichlet-ghost update.
  int boundary = 0;
  int bc[6] = {0, 0, 0, 0, 0, 0};
  double Pbc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  htr_rect3 plane[6] = {};  // the sides' boundary points (NSCBC sides are refreshed plane by plane)
};

// Side kinds of the boundary step.  Walls have staggered ghost points (never
// solved); NSCBC sides have collocated boundary points, solved without the
// flux divergence normal to the side and refreshed by the side's rule.
enum BcKind { kBcPeriodic = 0, kBcWall = 1, kBcInflow = 2, kBcOutflow = 3 };

// Launch shapes of the fused stage (process-wide; set before launches or
// graph captures that should use them).
struct StageTuning {
  int prepass_block = 256;      // threads per block, per-cell prepass (64..256)
  int diffusion_block = 128;    // threads per block, diffusion faces (32..128)
  int update_block = 128;       // threads per block, per-cell update (32..128)
  int teno_blocks_per_sm = 0;   // grid of the TENO queue kernel: 0 one queued face per thread,
                                // 1..32 that many blocks per SM striding over the queue
  int kg_x_tile = 128;          // faces per x tile of the KG kernel (64, 128, 256)
};
StageTuning &stage_tuning();

struct ConstPropDev;
struct AirDev;

// Euler faces of one stage (Z, Y, X KG tiles, then the TENO faces); H is the
// dense per-cell total enthalpy written by the prepass.
template <class Mix>
cudaError_t launch_stage_euler(const htr_fluid_view &v, const htr_rect3 &interior, const htr_rect3 &fb,
                               const Mix &mix, const StageWorkspace &w, const Fd<double> &H,
                               const StageParams &p, double rk0, double rk1, double sdt, cudaStream_t s,
                               cudaEvent_t *ev = nullptr);

template <class Mix>
cudaError_t launch_stage(const htr_fluid_view &v, const htr_rect3 &interior, const htr_rect3 &fb,
                         const Mix &mix, const StageWorkspace &w, const StageParams &p, int *status,
                         cudaStream_t s, cudaEvent_t *ev = nullptr);

// Events of a profiled stage: start, then one after each kernel.
enum StageKernel { kPrepass, kKgZ, kKgY, kKgX, kTeno, kDiffZ, kDiffY, kDiffX, kUpdate, kTransport, kStageKernels };

}  // namespace htr
