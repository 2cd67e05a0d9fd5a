// Shared declarations of the Euler-face kernels of the fused stage.
#pragma once

#include "euler_face.cuh"
#include "stage.cuh"

namespace htr {

struct StageEulerArgs {
  EulerArgs e;       // fields, bounds, RK coefficients (e.my = interior)
  Fd<double> H;      // per-cell total enthalpy from the prepass (dense)
  FaceGrid g;
  double *fe;        // face buffer of this direction, [NE][nf]
  TenoEntry *queue;
  unsigned *count;
};

// Kennedy-Gruber faces of direction D (Z, Y or X tiles); the sensor-rejected
// faces of the hybrid scheme are appended to the TENO queue.
template <class Mix>
cudaError_t launch_kg_faces(const StageEulerArgs &A, const Mix &mix, int D, bool hybrid, cudaStream_t s);

}  // namespace htr
