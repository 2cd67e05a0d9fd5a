// Euler fluxes: hybrid TENO / Kennedy-Gruber, TENO-only and skew-symmetric.
//
// Replaces UpdateUsingHybridEulerFluxTask, UpdateUsingTENOEulerFluxTask and
// UpdateUsingSkewSymmetricEulerFluxTask (src/prometeo_rhs.hpp:54-366,
// src/prometeo_rhs.inl:37-1052, GPU variants src/prometeo_rhs.cu:37-480).
//
// Kernel design (one launch per direction):
//   * a block owns a tile of cells: L pencils x S cells along the flux
//     direction (x: 1 x 256, y/z: 32 x 8 with the 32 pencils consecutive in
//     x, so neighbouring lanes read neighbouring addresses);
//   * every face of the tile (S+1 per pencil) is computed exactly once, into
//     shared memory (structure of arrays, conflict-free);
//   * hybrid: faces whose sensor says smooth are reconstructed with the
//     Kennedy-Gruber split form right away; the others are appended to a
//     shared queue and processed by all threads of the block together, so
//     the expensive characteristic TENO path is never diverged against the
//     cheap KG path inside a warp;
//   * then each cell adds m_e * (F(i+1/2) - F(i-1/2)) to Conserved_t.
//
// This translation unit is compiled with -fmad=false: the characteristic
// projections, Roe average and TENO weights are rounded exactly as the
// reference's CPU code rounds them, so stencil selections and sensor
// decisions agree bit for bit.
#include "euler_face.cuh"
#include "kernels.cuh"

namespace htr {

// Tile geometry.  The TENO schemes reconstruct every face with the same
// cost, so their tiles hold exactly one face per thread (255 x 1 or 7 x 32
// cells: 256 faces); the others keep the 256 x 1 / 8 x 32 cell tiles.
template <int D, int SCHEME> struct Tile {
  static constexpr bool EQ = SCHEME == kSchemeTeno;
  static constexpr int L = (D == 0) ? 1 : 32;                          // pencils per block (consecutive x)
  static constexpr int S = (D == 0) ? (EQ ? 255 : 256) : (EQ ? 7 : 8);  // cells per pencil
  static constexpr int NF = L * (S + 1);                               // faces per block
  static constexpr int THREADS = 256;
};

// Two blocks per SM (128 registers): the occupancy gain outweighs the spills
// for every scheme.
template <class Mix, int D, int SCHEME, int KIND>
__global__ void __launch_bounds__(256, 2) euler_kernel(const EulerArgs a, const __grid_constant__ Mix mix) {
  using TL = Tile<D, SCHEME>;
  using EF = EulerFace<Mix, D>;
  constexpr int NE = Mix::NS + 4;
  extern __shared__ double smem[];
  double *Fs = smem;  // [NE][NF]
  __shared__ int qn;
  __shared__ short qlist[TL::NF];

  // tile origin
  long long o[3];
  const int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
  if (D == 0) {
    o[0] = a.my.lo[0] + (long long)bx * TL::S;
    o[1] = a.my.lo[1] + by;
    o[2] = a.my.lo[2] + bz;
  } else if (D == 1) {
    o[0] = a.my.lo[0] + (long long)bx * TL::L;
    o[1] = a.my.lo[1] + (long long)by * TL::S;
    o[2] = a.my.lo[2] + bz;
  } else {
    o[0] = a.my.lo[0] + (long long)bx * TL::L;
    o[1] = a.my.lo[1] + by;
    o[2] = a.my.lo[2] + (long long)bz * TL::S;
  }
  const long long nseg = min((long long)TL::S, a.my.hi[D] - o[D] + 1);  // cells in this tile
  const int nlines = (D == 0) ? 1 : (int)min((long long)TL::L, a.my.hi[0] - o[0] + 1);
  if (threadIdx.x == 0) qn = 0;
  __syncthreads();

  EF ef{a, mix};
  const int nface = nlines * (int)(nseg + 1);
  // face f -> (line l, index j): face j lies between cells o+j-1 and o+j
  auto face_point = [&](int f, long long *p, long long *q, int &t) {
    const int l = (D == 0) ? 0 : f % nlines;
    const int j = (D == 0) ? f : f / nlines;
    long long c[3] = {o[0], o[1], o[2]};
    if (D != 0) c[0] += l;
    c[D] += j;  // the cell right of the face
    if (j == 0 && c[D] == a.my.lo[D]) {
      // first face of the task's span: left point from the node type of the
      // first cell, right point is that cell (rhs.inl:782-800)
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
  };

  for (int f = threadIdx.x; f < nface; f += blockDim.x) {
    long long p[3], q[3];
    int t;
    face_point(f, p, q, t);
    if (SCHEME == kSchemeTeno) {
      // every face reconstructed here, one per thread: no queue
      double F[NE];
      const double lim_f = a.dt * (ld(a.me.at(p)) + ld(a.me.at(q)));
      ef.template teno_flux<KIND>(F, p, t, lim_f);
#pragma unroll
      for (int i = 0; i < NE; i++) Fs[i * TL::NF + f] = F[i];
      continue;
    }
    bool smooth;
    if (SCHEME == kSchemeSkew) {
      smooth = true;
    } else {
      long long pm[3];
      ef.shift(pm, p, kNode[t].off[1], false);
      smooth = ld(a.sen.at(pm)) && ld(a.sen.at(p)) && ld(a.sen.at(q));
    }
    if (smooth) {
      double F[NE];
      ef.kg(F, p, t);
#pragma unroll
      for (int i = 0; i < NE; i++) Fs[i * TL::NF + f] = F[i];
    } else {
      const int slot = atomicAdd(&qn, 1);
      qlist[slot] = (short)f;
    }
  }
  __syncthreads();
  const int nq = qn;
  for (int k = threadIdx.x; k < nq; k += blockDim.x) {
    const int f = qlist[k];
    long long p[3], q[3];
    int t;
    face_point(f, p, q, t);
    double F[NE];
    const double lim_f = a.dt * (ld(a.me.at(p)) + ld(a.me.at(q)));
    ef.template teno_flux<KIND>(F, p, t, lim_f);
#pragma unroll
    for (int i = 0; i < NE; i++) Fs[i * TL::NF + f] = F[i];
  }
  __syncthreads();
  const int ncell = nlines * (int)nseg;
  for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
    const int l = (D == 0) ? 0 : c % nlines;
    const int j = (D == 0) ? c : c / nlines;
    long long p[3] = {o[0], o[1], o[2]};
    if (D != 0) p[0] += l;
    p[D] += j;
    const int fm = (D == 0) ? j : j * nlines + l;
    const int fp = (D == 0) ? j + 1 : (j + 1) * nlines + l;
    double *ct = a.Ct.at(p);
    const double m = ld(a.me.at(p));
#pragma unroll
    for (int i = 0; i < NE; i++) ct[i] += m * (Fs[i * TL::NF + fp] - Fs[i * TL::NF + fm]);
  }
}

template <class Mix, int D, int SCHEME, int KIND>
static cudaError_t launch_euler_dir(const EulerArgs &a, const Mix &mix, cudaStream_t s) {
  using TL = Tile<D, SCHEME>;
  const long long n[3] = {a.my.size(0), a.my.size(1), a.my.size(2)};
  dim3 grid;
  if (D == 0) grid = dim3((unsigned)((n[0] + TL::S - 1) / TL::S), (unsigned)n[1], (unsigned)n[2]);
  else if (D == 1) grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)((n[1] + TL::S - 1) / TL::S), (unsigned)n[2]);
  else grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)n[1], (unsigned)((n[2] + TL::S - 1) / TL::S));
  const size_t sm = sizeof(double) * (Mix::NS + 4) * TL::NF;
  auto k = euler_kernel<Mix, D, SCHEME, KIND>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, TL::THREADS, sm, s>>>(a, mix);
  return cudaGetLastError();
}

template <class Mix>
cudaError_t launch_euler(const htr_fluid_view &v, const htr_rect3 &my, const htr_rect3 &fb,
                         const double *rk, double dt, const Mix &mix, int dir, int scheme, int kind,
                         cudaStream_t s) {
  EulerArgs a;
  a.C = fd<double>(v.Conserved);
  a.Cold = fd<double>(v.Conserved_old);
  a.SoS = fd<double>(v.SoS);
  a.rho = fd<double>(v.rho);
  a.Y = fd<double>(v.MassFracs);
  a.u = fd<double>(v.velocity);
  a.P = fd<double>(v.pressure);
  a.Ct = fd<double>(v.Conserved_t);
  const htr_field &me = dir == 0 ? v.dcsi_e : (dir == 1 ? v.deta_e : v.dzet_e);
  const htr_field &nt = dir == 0 ? v.nType_x : (dir == 1 ? v.nType_y : v.nType_z);
  const htr_field &sn = dir == 0 ? v.shockSensorX : (dir == 1 ? v.shockSensorY : v.shockSensorZ);
  a.me = fd<double>(me);
  a.nt = fd<int>(nt);
  a.sen = fd<bool>(sn);
  a.my = box(my);
  a.fb = box(fb);
  a.rk0 = rk ? rk[0] : 0.0;
  a.rk1 = rk ? rk[1] : 1.0;
  a.dt = dt;
#define HTR_EULER_CASE(DIR)                                                                   \
  if (dir == DIR) {                                                                           \
    if (scheme == kSchemeHybrid) return launch_euler_dir<Mix, DIR, kSchemeHybrid, kTENO>(a, mix, s); \
    if (scheme == kSchemeSkew) return launch_euler_dir<Mix, DIR, kSchemeSkew, kTENO>(a, mix, s);     \
    if (kind == kTENO) return launch_euler_dir<Mix, DIR, kSchemeTeno, kTENO>(a, mix, s);      \
    if (kind == kTENOA) return launch_euler_dir<Mix, DIR, kSchemeTeno, kTENOA>(a, mix, s);    \
    return launch_euler_dir<Mix, DIR, kSchemeTeno, kTENOLAD>(a, mix, s);                      \
  }
  HTR_EULER_CASE(0)
  HTR_EULER_CASE(1)
  HTR_EULER_CASE(2)
#undef HTR_EULER_CASE
  return cudaErrorInvalidValue;
}

template cudaError_t launch_euler<ConstPropDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                                const double *, double, const ConstPropDev &, int, int, int,
                                                cudaStream_t);
template cudaError_t launch_euler<AirDev>(const htr_fluid_view &, const htr_rect3 &, const htr_rect3 &,
                                          const double *, double, const AirDev &, int, int, int, cudaStream_t);

// decision counters of this translation unit (htr_decision_counters)
HTR_DECISION_COUNTERS_ACCESS(decision_counters_euler)

}  // namespace htr
