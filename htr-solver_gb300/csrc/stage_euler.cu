// Euler faces of the fused stage pipeline (compiled with -fmad=false).
//
// euler_kg_faces<D>: a block owns L pencils x S faces along D.  The cell data
// of its window (S + 6 points per pencil: the faces' 6-point stencils) is
// staged in shared memory once — rho, p, H = (rhoE + p)/rho (precomputed per
// cell by the stage prepass), mass fractions, velocity, sensor flag, node
// type — and each face is reconstructed from it.  Kennedy-Gruber faces are
// written to the face buffer directly; faces the hybrid sensor rejects are
// appended to a device-wide queue (warp-aggregated atomics).
//
// euler_teno_faces: characteristic TENO faces of the queue (hybrid) or of
// the whole grid (TENO schemes), spread over every SM with a grid-stride
// loop, so the expensive reconstruction is load-balanced independently of
// where the shocks are.
//
// The arithmetic per face is the one of the per-direction task kernels
// (euler_face.cuh), so the face fluxes are bit-identical to theirs.
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

template <int D> struct KGTile {
  static constexpr int L = (D == 0) ? 1 : 32;
  static constexpr int S = (D == 0) ? 128 : 8;
  static constexpr int WS = S + 6;
  static constexpr int THREADS = (D == 0) ? 128 : 256;
};

HTR_D long long wrap_in(long long v, long long lo, long long size) {
  return ((v - lo) % size + size) % size + lo;
}

template <class Mix, int D, bool HYBRID>
__global__ void __launch_bounds__(KGTile<D>::THREADS) euler_kg_faces(const StageEulerArgs A, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS, NE = NS + 4, iU = NS, iE = NS + 3;
  constexpr int L = KGTile<D>::L, S = KGTile<D>::S, WS = KGTile<D>::WS;
  extern __shared__ double win[];  // [NV][L*WS]
  __shared__ unsigned char sflag[L * WS];
  __shared__ signed char stype[L * WS];
  const EulerArgs &a = A.e;
  (void)iE;

  long long o[3];
  if (D == 0) {
    o[0] = a.my.lo[0] + (long long)blockIdx.x * S;
    o[1] = a.my.lo[1] + blockIdx.y;
    o[2] = a.my.lo[2] + blockIdx.z;
  } else if (D == 1) {
    o[0] = a.my.lo[0] + (long long)blockIdx.x * L;
    o[1] = a.my.lo[1] + (long long)blockIdx.y * S;
    o[2] = a.my.lo[2] + blockIdx.z;
  } else {
    o[0] = a.my.lo[0] + (long long)blockIdx.x * L;
    o[1] = a.my.lo[1] + blockIdx.y;
    o[2] = a.my.lo[2] + (long long)blockIdx.z * S;
  }
  const int nlines = (D == 0) ? 1 : (int)min((long long)L, a.my.hi[0] - o[0] + 1);
  const long long ncell = min((long long)S, a.my.hi[D] - o[D] + 1);
  // faces of this tile: right cells o..o+ncell-1, plus hi+1 on the last tile
  const int nfl = (int)ncell + ((o[D] + ncell - 1 == a.my.hi[D]) ? 1 : 0);
  const long long base_d = o[D] - 3;

  // --- stage the window ----------------------------------------------------
  const long long fbsz = a.fb.size(D);
  for (int idx = threadIdx.x; idx < L * WS; idx += blockDim.x) {
    const int l = idx % L, w = idx / L;
    if (l >= nlines) continue;
    long long p[3] = {o[0], o[1], o[2]};
    if (D != 0) p[0] += l;
    p[D] = wrap_in(base_d + w, a.fb.lo[D], fbsz);
    const int k = w * L + l;
    win[0 * L * WS + k] = ld(a.rho.at(p));
    win[1 * L * WS + k] = ld(a.P.at(p));
    win[2 * L * WS + k] = ld(A.H.at(p));
#pragma unroll
    for (int i = 0; i < NS; i++) win[(3 + i) * L * WS + k] = ld(&a.Y.at(p)[i]);
#pragma unroll
    for (int i = 0; i < 3; i++) win[(3 + NS + i) * L * WS + k] = ld(&a.u.at(p)[i]);
    sflag[k] = HYBRID ? (unsigned char)ld(a.sen.at(p)) : 1;
    stype[k] = (signed char)ld(a.nt.at(p));
  }
  __syncthreads();

  const long long nf = A.g.nf[D];
  const int lane = threadIdx.x & 31;
  const int nface = nlines * nfl;
  const int nround = (nface + blockDim.x - 1) / blockDim.x;
  for (int r = 0; r < nround; r++) {
    const int f = r * blockDim.x + threadIdx.x;
    bool active = f < nface;
    bool teno = false;
    long long c[3] = {o[0], o[1], o[2]};
    if (active) {
      const int l = (D == 0) ? 0 : f % nlines;
      const int j = (D == 0) ? f : f / nlines;
      if (D != 0) c[0] += l;
      c[D] += j;
      // left point p and right point q of the face, as window indices
      int wp, wq, t;
      if (c[D] == a.my.lo[D]) {
        const int w0 = (int)(c[D] - base_d);
        wp = w0 + kNode[stype[w0 * L + l]].off[1];
        wq = w0;
        t = stype[wp * L + l];
      } else {
        wp = (int)(c[D] - 1 - base_d);
        t = stype[wp * L + l];
        wq = wp + kNode[t].off[2];
      }
      const int wm = wp + kNode[t].off[1];
      const bool smooth = !HYBRID || (sflag[wm * L + l] && sflag[wp * L + l] && sflag[wq * L + l]);
      if (smooth) {
        double F[NE];
        const long long fi = A.g.index(D, c);
        auto V = [&](int q, int w) { return win[q * L * WS + w * L + l]; };
        if (t == L_S || t == Rm1_S) {
          // staggered boundary node: the flux is the physical flux at the face node
          const int wn = (t == L_S) ? wp : wp + kNode[t].off[2];
          long long pn[3] = {c[0], c[1], c[2]};
          pn[D] = wrap_in(base_d + wn, a.fb.lo[D], fbsz);
          const double un = V(3 + NS + D, wn), pq = V(1, wn);
          const double *Cq = a.C.at(pn);
#pragma unroll
          for (int i = 0; i < NE; i++) F[i] = -(ld(&Cq[i]) * un);
          F[iU + D] -= pq;
          F[NS + 3] -= pq * un;
        } else {
          int wk[6];
          wk[0] = wp + kNode[t].off[0];
          wk[1] = wm;
          wk[2] = wp;
          wk[3] = wp + kNode[t].off[2];
          wk[4] = wp + kNode[t].off[3];
          wk[5] = wp + kNode[t].off[4];
          double r_[6], v_[6], pr[6], h[6];
#pragma unroll
          for (int k = 0; k < 6; k++) {
            r_[k] = V(0, wk[k]);
            pr[k] = V(1, wk[k]);
            h[k] = V(2, wk[k]);
            v_[k] = -V(3 + NS + D, wk[k]);
          }
          const int order = kNode[t].kgOrder;
          const double kgc[3] = {kNode[t].kg[0], kNode[t].kg[1], kNode[t].kg[2]};
          double rv[3][3];
#pragma unroll
          for (int l2 = 0; l2 < 3; l2++)
#pragma unroll
            for (int m = 0; m < 3; m++)
              if (m <= l2 && l2 < order)
                rv[l2][m] = (r_[2 - m] + r_[2 - m + l2 + 1]) * (v_[2 - m] + v_[2 - m + l2 + 1]);
          auto triple = [&](int q) {
            double flux = 0.0;
#pragma unroll
            for (int l2 = 0; l2 < 3; l2++) {
              if (l2 < order) {
                double acc = 0.0;
#pragma unroll
                for (int m = 0; m <= l2; m++) acc += rv[l2][m] * (V(q, wk[2 - m]) + V(q, wk[2 - m + l2 + 1]));
                flux += kgc[l2] * acc;
              }
            }
            return flux * 0.25;
          };
#pragma unroll
          for (int i = 0; i < NS; i++) F[i] = triple(3 + i);
#pragma unroll
          for (int cc = 0; cc < 3; cc++) F[iU + cc] = triple(3 + NS + cc);
          double pflux = 0.0;
#pragma unroll
          for (int l2 = 0; l2 < 3; l2++) {
            if (l2 < order) {
              double acc = 0.0;
#pragma unroll
              for (int m = 0; m <= l2; m++) acc += (pr[2 - m] + pr[2 - m + l2 + 1]);
              pflux += kgc[l2] * acc;
            }
          }
          F[iU + D] -= pflux;
          // energy: the same triple product with phi = H
          {
            double flux = 0.0;
#pragma unroll
            for (int l2 = 0; l2 < 3; l2++) {
              if (l2 < order) {
                double acc = 0.0;
#pragma unroll
                for (int m = 0; m <= l2; m++) acc += rv[l2][m] * (h[2 - m] + h[2 - m + l2 + 1]);
                flux += kgc[l2] * acc;
              }
            }
            F[NS + 3] = flux * 0.25;
          }
        }
#pragma unroll
        for (int i = 0; i < NE; i++) A.fe[i * nf + fi] = F[i];
      } else {
        teno = true;
      }
    }
    // warp-aggregated append of the rejected faces to the TENO queue
    const unsigned m = __ballot_sync(0xffffffffu, teno);
    if (m) {
      unsigned base = 0;
      const int leader = __ffs(m) - 1;
      if (lane == leader) base = atomicAdd(A.count, (unsigned)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (teno) {
        const unsigned slot = base + __popc(m & ((1u << lane) - 1u));
        A.queue[slot] = TenoEntry{D, (int)c[0], (int)c[1], (int)c[2]};
      }
    }
  }
}

// --- characteristic TENO faces -------------------------------------------
struct StageTenoArgs {
  EulerArgs e[3];  // per direction (metric, node type, sensor fields differ)
  FaceGrid g;
  double *fe[3];
  const TenoEntry *queue;
  const unsigned *count;
  long long nall;  // > 0: every face of the three directions (no queue)
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
  const double lim_f = a.dt * (ld(a.me.at(p)) + ld(a.me.at(q)));
  ef.template teno_flux<KIND>(F, p, t, lim_f);
  const long long nf = A.g.nf[D];
  const long long fi = A.g.index(D, c);
  double *out = A.fe[D];
#pragma unroll
  for (int i = 0; i < NE; i++) out[i * nf + fi] = F[i];
}

template <class Mix, int KIND>
__global__ void __launch_bounds__(128) euler_teno_faces(const StageTenoArgs A, const __grid_constant__ Mix mix) {
  const long long n = A.nall > 0 ? A.nall : (long long)*A.count;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    int D;
    long long c[3];
    if (A.nall > 0) {
      long long f = k;
      D = 0;
      while (D < 2 && f >= A.g.nf[D]) f -= A.g.nf[D++];
      const long long e0 = A.g.ext[D][0], e1 = A.g.ext[D][1];
      c[0] = A.g.lo[0] + f % e0;
      c[1] = A.g.lo[1] + (f / e0) % e1;
      c[2] = A.g.lo[2] + f / (e0 * e1);
    } else {
      const TenoEntry e = A.queue[k];
      D = e.D;
      c[0] = e.c0;
      c[1] = e.c1;
      c[2] = e.c2;
    }
    if (D == 0)
      teno_face_at<Mix, 0, KIND>(A, mix, c);
    else if (D == 1)
      teno_face_at<Mix, 1, KIND>(A, mix, c);
    else
      teno_face_at<Mix, 2, KIND>(A, mix, c);
  }
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

template <class Mix, int D, bool HYBRID>
static cudaError_t kg_dir(const StageEulerArgs &A, const Mix &mix, cudaStream_t s) {
  using TL = KGTile<D>;
  const long long n[3] = {A.e.my.size(0), A.e.my.size(1), A.e.my.size(2)};
  dim3 grid;
  if (D == 0) grid = dim3((unsigned)((n[0] + TL::S - 1) / TL::S), (unsigned)n[1], (unsigned)n[2]);
  else if (D == 1) grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)((n[1] + TL::S - 1) / TL::S), (unsigned)n[2]);
  else grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)n[1], (unsigned)((n[2] + TL::S - 1) / TL::S));
  const size_t sm = sizeof(double) * (Mix::NS + 6) * TL::L * TL::WS;
  auto k = euler_kg_faces<Mix, D, HYBRID>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, TL::THREADS, sm, s>>>(A, mix);
  return cudaGetLastError();
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
    if ((e = cudaMemsetAsync(w.count, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
    for (int k = 0; k < 3; k++) {
      const int D = order[k];
      StageEulerArgs A;
      A.e = euler_args(v, my, fb, D, rk0, rk1, sdt);
      A.H = H;
      A.g = g;
      A.fe = w.fe[D];
      A.queue = w.queue;
      A.count = w.count;
      const bool hyb = p.scheme == 0;
      if (D == 0) e = hyb ? kg_dir<Mix, 0, true>(A, mix, s) : kg_dir<Mix, 0, false>(A, mix, s);
      else if (D == 1) e = hyb ? kg_dir<Mix, 1, true>(A, mix, s) : kg_dir<Mix, 1, false>(A, mix, s);
      else e = hyb ? kg_dir<Mix, 2, true>(A, mix, s) : kg_dir<Mix, 2, false>(A, mix, s);
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
    T.fe[D] = w.fe[D];
  }
  T.g = g;
  T.queue = w.queue;
  T.count = w.count;
  T.nall = (p.scheme == 2) ? (g.nf[0] + g.nf[1] + g.nf[2]) : 0;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  dim3 grid((unsigned)(sms * 8));
  const int kind = (p.scheme == 2) ? p.kind : 0;
  if (kind == kTENO) euler_teno_faces<Mix, kTENO><<<grid, 128, 0, s>>>(T, mix);
  else if (kind == kTENOA) euler_teno_faces<Mix, kTENOA><<<grid, 128, 0, s>>>(T, mix);
  else euler_teno_faces<Mix, kTENOLAD><<<grid, 128, 0, s>>>(T, mix);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
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

}  // namespace htr
