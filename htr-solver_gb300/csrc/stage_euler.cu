// Characteristic TENO faces of the fused stage pipeline (compiled with
// -fmad=false) and the Euler orchestration of one stage.
//
// euler_teno_faces: the faces the hybrid sensor rejected (queued by the
// Kennedy-Gruber kernel, stage_kg.cu), one queued face per thread over the
// whole GPU, so the expensive reconstruction is load-balanced independently
// of where the shocks are.  euler_teno_faces_dir: every face of
// one direction for the TENO schemes, one face per thread.  The arithmetic
// per face is the one of the per-direction task kernels (euler_face.cuh), so
// selection flags and face fluxes are bit-identical to theirs.
#include "stage_euler.cuh"

namespace htr {

// --- characteristic TENO faces -------------------------------------------
struct StageTenoArgs {
  EulerArgs e[3];  // per direction (metric, node type, sensor fields differ)
  FaceGrid g;
  double *fe[3];
  const TenoEntry *queue;
  const unsigned *count;
  unsigned active; // directions whose faces are computed
};

template <class Mix, int D, int KIND>
HTR_D void teno_face_at(const StageTenoArgs &A, const Mix &mix, const long long *c) {
  constexpr int NE = Mix::NS + 4;
  const EulerArgs &a = A.e[D];
  EulerFace<Mix, D> ef{a, mix};
  long long p[3], q[3];
  int t;
  if (c[D] == a.my.lo[D]) {
    const int t0 = ld(a.nt.at(c));
    ef.shift(p, c, kNode[t0].off[1], false);
    q[0] = c[0];
    q[1] = c[1];
    q[2] = c[2];
    t = ld(a.nt.at(p));
  } else {
    p[0] = c[0];
    p[1] = c[1];
    p[2] = c[2];
    p[D] = c[D] - 1;
    t = ld(a.nt.at(p));
    ef.shift(q, p, kNode[t].off[2], true);
  }
  double F[NE];
  if (outside_face(t)) {
#pragma unroll
    for (int i = 0; i < NE; i++) F[i] = 0.0;
  } else {
    const double lim_f = a.face_dt(p) * (ld(a.me.at(p)) + ld(a.me.at(q)));
    ef.template teno_flux<KIND>(F, p, t, lim_f);
  }
  const long long nf = A.g.nf[D];
  const long long fi = A.g.index(D, c);
  double *out = A.fe[D];
#pragma unroll
  for (int i = 0; i < NE; i++) out[i * nf + fi] = F[i];
}

// The queued faces of direction D (one launch per direction: a launch holds
// one direction's code).
template <class Mix, int D, int KIND>
__global__ void __launch_bounds__(128) euler_teno_faces(const StageTenoArgs A, const __grid_constant__ Mix mix) {
  long long off = 0;
#pragma unroll
  for (int d = 0; d < D; d++) off += A.g.nf[d];
  const long long n = (long long)A.count[D];
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const TenoEntry e = A.queue[off + k];
    const long long c[3] = {e.c0, e.c1, e.c2};
    teno_face_at<Mix, D, KIND>(A, mix, c);
  }
}

// Every face of direction D (the TENO schemes): one face per thread,
// consecutive threads on consecutive x, one launch per direction, so a launch
// holds one direction's code and no queue.
template <class Mix, int D, int KIND>
__global__ void __launch_bounds__(128) euler_teno_faces_dir(const StageTenoArgs A, const __grid_constant__ Mix mix) {
  const long long nf = A.g.nf[D];
  const long long e0 = A.g.ext[D][0], e1 = A.g.ext[D][1];
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
    const long long c[3] = {A.g.lo[0] + f % e0, A.g.lo[1] + (f / e0) % e1, A.g.lo[2] + f / (e0 * e1)};
    teno_face_at<Mix, D, KIND>(A, mix, c);
  }
}

template <class Mix, int KIND>
static void launch_teno_dir(const StageTenoArgs &T, const Mix &mix, int D, dim3 grid, cudaStream_t s) {
  if (D == 0) euler_teno_faces_dir<Mix, 0, KIND><<<grid, 128, 0, s>>>(T, mix);
  else if (D == 1) euler_teno_faces_dir<Mix, 1, KIND><<<grid, 128, 0, s>>>(T, mix);
  else euler_teno_faces_dir<Mix, 2, KIND><<<grid, 128, 0, s>>>(T, mix);
}

// --- launchers --------------------------------------------------------------
static EulerArgs euler_args(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb, int dir,
                            double rk0, double rk1, double dt) {
  EulerArgs a;
  a.C = fd<double>(v.Conserved);
  a.Cold = fd<double>(v.Conserved_old);
  a.SoS = fd<double>(v.SoS);
  a.rho = fd<double>(v.rho);
  a.Y = fd<double>(v.MassFracs);
  a.u = fd<double>(v.velocity);
  a.P = fd<double>(v.pressure);
  a.Ct = fd<double>(v.Conserved_t);
  const htr_field *me[3] = {&v.dcsi_e, &v.deta_e, &v.dzet_e};
  const htr_field *nt[3] = {&v.nType_x, &v.nType_y, &v.nType_z};
  const htr_field *sn[3] = {&v.shockSensorX, &v.shockSensorY, &v.shockSensorZ};
  a.me = fd<double>(*me[dir]);
  a.nt = fd<int>(*nt[dir]);
  a.sen = fd<bool>(*sn[dir]);
  a.my = box(my);
  a.fb = box(fb);
  a.rk0 = rk0;
  a.rk1 = rk1;
  a.dt = dt;
  return a;
}

template <class Mix>
cudaError_t launch_stage_euler(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb, const Mix &mix,
                               const StageWorkspace &w, const Fd<double> &H, const StageParams &p,
                               double rk0, double rk1, double sdt, cudaStream_t s, cudaEvent_t *ev) {
  static const int order[3] = {2, 1, 0};  // Z, Y, X as the reference
  // ev (optional): recorded after KG Z, Y, X and after the TENO kernel
  auto mark = [&](int i) { return ev ? cudaEventRecord(ev[i], s) : cudaSuccess; };
  const FaceGrid g = face_grid(my);
  cudaError_t e = cudaSuccess;
  if (p.scheme != 2) {
    if ((e = cudaMemsetAsync(w.count, 0, 3 * sizeof(unsigned), s)) != cudaSuccess) return e;
    for (int k = 0; k < 3; k++) {
      const int D = order[k];
      if (!(p.active & (1u << D))) {
        if ((e = mark(k)) != cudaSuccess) return e;
        continue;
      }
      StageEulerArgs A;
      A.e = euler_args(v, my, fb, D, rk0, rk1, sdt);
      A.H = H;
      A.g = g;
      A.fe = w.fe[D];
      long long off = 0;
      for (int d = 0; d < D; d++) off += g.nf[d];
      A.queue = w.queue + off;
      A.count = w.count + D;
      e = launch_kg_faces(A, mix, D, p.scheme == 0, s);
      if (e != cudaSuccess || (e = mark(k)) != cudaSuccess) return e;
    }
    if (p.scheme == 1) return mark(3);  // skew-symmetric: KG everywhere
  } else {
    for (int k = 0; k < 3; k++)
      if ((e = mark(k)) != cudaSuccess) return e;
  }
  StageTenoArgs T;
  for (int D = 0; D < 3; D++) {
    T.e[D] = euler_args(v, my, fb, D, rk0, rk1, sdt);
    T.e[D].dtc = p.dt_cell;
    T.e[D].dtc_c3 = p.dtc_c3;
    T.e[D].dtc_h = p.dtc_h;
    T.fe[D] = w.fe[D];
  }
  T.g = g;
  T.queue = w.queue;
  T.count = w.count;
  T.active = p.active;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (p.scheme == 2) {
    for (int k = 0; k < 3; k++) {
      const int D = order[k];
      if (!(p.active & (1u << D))) continue;
      // one face per thread: a grid capped at 64 blocks per SM (each thread
      // then striding over ~10 faces) made the 512 x 192 x 128 boundary-layer
      // step 26 % slower (1642 ms against 1305 ms); the stride loop only
      // remains for grids beyond the launch limit
      const long long blocks = (g.nf[D] + 127) / 128, cap = 0x7fffffffLL;
      const dim3 gd((unsigned)(blocks < cap ? blocks : cap));
      if (p.kind == kTENO) launch_teno_dir<Mix, kTENO>(T, mix, D, gd, s);
      else if (p.kind == kTENOA) launch_teno_dir<Mix, kTENOA>(T, mix, D, gd, s);
      else launch_teno_dir<Mix, kTENOLAD>(T, mix, D, gd, s);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return mark(3);
  }
  // the hybrid scheme's sensor-rejected faces (plain TENO, rhs.inl:622-759),
  // one launch per direction over that direction's queue.  By default the
  // grid covers every face of the direction, one queued face per thread (the
  // blocks past the queue's length exit at once): on the 512 x 192 x 128
  // boundary layer a grid of 8 blocks per SM striding over the queue made the
  // hybrid step 8 % slower (1167 ms against 1083 ms), and the 256^3 air box
  // (a short queue) runs the same either way
  const int tb = stage_tuning().teno_blocks_per_sm;
  for (int k = 0; k < 3; k++) {
    const int D = order[k];
    if (!(p.active & (1u << D))) continue;
    const long long blocks = tb > 0 ? (long long)sms * tb : (g.nf[D] + 127) / 128;
    const dim3 grid((unsigned)(blocks < 1 ? 1 : (blocks > 0x7fffffffLL ? 0x7fffffffLL : blocks)));
    if (D == 0) euler_teno_faces<Mix, 0, kTENO><<<grid, 128, 0, s>>>(T, mix);
    else if (D == 1) euler_teno_faces<Mix, 1, kTENO><<<grid, 128, 0, s>>>(T, mix);
    else euler_teno_faces<Mix, 2, kTENO><<<grid, 128, 0, s>>>(T, mix);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return mark(3);
}

template cudaError_t launch_stage_euler<ConstPropDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                                      const ConstPropDev &, const StageWorkspace &, const Fd<double> &,
                                                      const StageParams &, double, double, double, cudaStream_t,
                                                      cudaEvent_t *);
template cudaError_t launch_stage_euler<AirDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                                const AirDev &, const StageWorkspace &, const Fd<double> &,
                                                const StageParams &, double, double, double, cudaStream_t,
                                                cudaEvent_t *);

// decision counters of this translation unit (htr_decision_counters)
HTR_DECISION_COUNTERS_ACCESS(decision_counters_stage_euler)

}  // namespace htr
