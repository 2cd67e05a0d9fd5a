// Kennedy-Gruber faces of the fused stage pipeline.
//
// A block owns L pencils x S faces along D.  The cell data of its window
// (S + 6 points per pencil: the faces' 6-point stencils) is staged in shared
// memory once -- rho, p, H = (rhoE + p)/rho (precomputed per cell by the
// stage prepass), mass fractions, velocity, sensor flag, node type -- and
// each face is reconstructed from it.  Kennedy-Gruber faces are written to
// the face buffer directly; faces the hybrid sensor rejects are appended to a
// device-wide queue (warp-aggregated atomics) for the TENO kernel.
//
// The split form is the one of src/prometeo_rhs.inl:137-196 (direct
// variant); this translation unit keeps FMA contraction (no selection flag
// depends on these fluxes), so the face values agree with the task kernels
// to rounding.
#include "stage_euler.cuh"

namespace htr {

template <int D, int SX = 128> struct KGTile {
  static constexpr int L = (D == 0) ? 1 : 32;
  static constexpr int S = (D == 0) ? SX : 8;
  static constexpr int WS = S + 6;
  static constexpr int THREADS = (D == 0) ? SX : 256;
};

HTR_D long long wrap_in(long long v, long long lo, long long size) {
  return ((v - lo) % size + size) % size + lo;
}

template <class Mix, int D, bool HYBRID, int SX>
__global__ void __launch_bounds__(KGTile<D, SX>::THREADS) euler_kg_faces(const StageEulerArgs A, const __grid_constant__ Mix mix) {
  constexpr int NS = Mix::NS, NE = NS + 4, iU = NS, iE = NS + 3;
  constexpr int L = KGTile<D, SX>::L, S = KGTile<D, SX>::S, WS = KGTile<D, SX>::WS;
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
      const bool outside = outside_face(t);
      const bool smooth = outside || !HYBRID || (sflag[wm * L + l] && sflag[wp * L + l] && sflag[wq * L + l]);
      if (outside) {
        const long long fi = A.g.index(D, c);
#pragma unroll
        for (int i = 0; i < NE; i++) A.fe[i * nf + fi] = 0.0;
      } else if (smooth) {
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
          // The split form sums, over the stencil pairs (a, b) of each order
          // l, kg_l (rho_a + rho_b)(v_a + v_b)(phi_a + phi_b) / 4.  Collected
          // per stencil point, every transported scalar's flux is one dot
          // product sum_k cw[k] phi_k, with cw[k] the pair weights
          // kg_l (rho_a + rho_b)(v_a + v_b) / 4 of the pairs holding point k,
          // computed once per face (the pressure term likewise with cp[k] =
          // sum of kg_l).  Same value, regrouped: rounding only.
          double cw[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, cp[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
          for (int l2 = 0; l2 < 3; l2++)
#pragma unroll
            for (int m = 0; m < 3; m++)
              if (m <= l2 && l2 < order) {
                const int a0 = 2 - m, b0 = 2 - m + l2 + 1;
                const double w = (0.25 * kgc[l2]) * ((r_[a0] + r_[b0]) * (v_[a0] + v_[b0]));
                cw[a0] += w;
                cw[b0] += w;
                cp[a0] += kgc[l2];
                cp[b0] += kgc[l2];
              }
          auto dot = [&](int q) {
            double flux = 0.0;
#pragma unroll
            for (int k = 0; k < 6; k++) flux += cw[k] * V(q, wk[k]);
            return flux;
          };
#pragma unroll
          for (int i = 0; i < NS; i++) F[i] = dot(3 + i);
#pragma unroll
          for (int cc = 0; cc < 3; cc++) F[iU + cc] = dot(3 + NS + cc);
          double pflux = 0.0;
#pragma unroll
          for (int k = 0; k < 6; k++) pflux += cp[k] * pr[k];
          F[iU + D] -= pflux;
          // energy: the same dot product with phi = H
          {
            double flux = 0.0;
#pragma unroll
            for (int k = 0; k < 6; k++) flux += cw[k] * h[k];
            F[NS + 3] = flux;
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

template <class Mix, int D, bool HYBRID, int SX = 128>
static cudaError_t kg_dir(const StageEulerArgs &A, const Mix &mix, cudaStream_t s) {
  using TL = KGTile<D, SX>;
  const long long n[3] = {A.e.my.size(0), A.e.my.size(1), A.e.my.size(2)};
  dim3 grid;
  if (D == 0) grid = dim3((unsigned)((n[0] + TL::S - 1) / TL::S), (unsigned)n[1], (unsigned)n[2]);
  else if (D == 1) grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)((n[1] + TL::S - 1) / TL::S), (unsigned)n[2]);
  else grid = dim3((unsigned)((n[0] + TL::L - 1) / TL::L), (unsigned)n[1], (unsigned)((n[2] + TL::S - 1) / TL::S));
  const size_t sm = sizeof(double) * (Mix::NS + 6) * TL::L * TL::WS;
  auto k = euler_kg_faces<Mix, D, HYBRID, SX>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<grid, TL::THREADS, sm, s>>>(A, mix);
  return cudaGetLastError();
}

template <class Mix>
cudaError_t launch_kg_faces(const StageEulerArgs &A, const Mix &mix, int D, bool hybrid, cudaStream_t s) {
  if (D == 0) {
    const int sx = stage_tuning().kg_x_tile;
    if (sx == 64) return hybrid ? kg_dir<Mix, 0, true, 64>(A, mix, s) : kg_dir<Mix, 0, false, 64>(A, mix, s);
    if (sx == 256) return hybrid ? kg_dir<Mix, 0, true, 256>(A, mix, s) : kg_dir<Mix, 0, false, 256>(A, mix, s);
    return hybrid ? kg_dir<Mix, 0, true>(A, mix, s) : kg_dir<Mix, 0, false>(A, mix, s);
  }
  if (D == 1) return hybrid ? kg_dir<Mix, 1, true>(A, mix, s) : kg_dir<Mix, 1, false>(A, mix, s);
  return hybrid ? kg_dir<Mix, 2, true>(A, mix, s) : kg_dir<Mix, 2, false>(A, mix, s);
}

template cudaError_t launch_kg_faces<ConstPropDev>(const StageEulerArgs &, const ConstPropDev &, int, bool, cudaStream_t);
template cudaError_t launch_kg_faces<AirDev>(const StageEulerArgs &, const AirDev &, int, bool, cudaStream_t);

}  // namespace htr
