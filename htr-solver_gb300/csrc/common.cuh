// Common device-side definitions of the htr_gb300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "htr_rhs.h"

#define HTR_HD __host__ __device__ __forceinline__
#define HTR_D __device__ __forceinline__

namespace htr {

// One field as the kernels see it: address of point (0,0,0) + byte strides.
template <class T> struct Fd {
  char *b;
  long long s0, s1, s2;
  HTR_HD T *at(long long x, long long y, long long z) const {
    return reinterpret_cast<T *>(b + x * s0 + y * s1 + z * s2);
  }
  HTR_HD T *at(const long long *p) const { return at(p[0], p[1], p[2]); }
};

template <class T> inline Fd<T> fd(const htr_field &f) {
  Fd<T> r;
  r.b = static_cast<char *>(f.base);
  r.s0 = f.stride[0];
  r.s1 = f.stride[1];
  r.s2 = f.stride[2];
  return r;
}

// Read-only load through the non-coherent cache.
template <class T> HTR_D T ld(const T *p) { return __ldg(p); }
template <> HTR_D bool ld<bool>(const bool *p) {
  return __ldg(reinterpret_cast<const unsigned char *>(p)) != 0;
}

struct Box {
  long long lo[3], hi[3];
  HTR_HD long long size(int d) const { return hi[d] - lo[d] + 1; }
  // dense index of p in the box, x fastest
  HTR_HD long long dense(const long long *p) const {
    return (p[0] - lo[0]) + size(0) * ((p[1] - lo[1]) + size(1) * (p[2] - lo[2]));
  }
};
inline Box box(const htr_rect3 &r) {
  Box b;
  for (int i = 0; i < 3; i++) {
    b.lo[i] = r.lo[i];
    b.hi[i] = r.hi[i];
  }
  return b;
}

// Periodic wrap of a stencil point inside the grid bounds; same formula as
// the reference's warpPeriodic (src/Utils/PointDomain_helper.hpp:160-190).
HTR_HD long long wrap_minus(long long p, long long lo, long long size, int off) {
  return ((p + off - lo) % size + size) % size + lo;
}
HTR_HD long long wrap_plus(long long p, long long lo, long long size, int off) {
  return (p + off - lo) % size + lo;
}

// TENO flavours: standard, adaptive-cutoff TENO-A, TENO-LAD
enum TenoKind { kTENO = 0, kTENOA = 1, kTENOLAD = 2 };

// min / max with the operand semantics of std::min / std::max.
HTR_HD double smin(double a, double b) { return (b < a) ? b : a; }
HTR_HD double smax(double a, double b) { return (a < b) ? b : a; }

// Montgomery's simultaneous inversion: v[k] <- 1 / v[k] for N values with
// one division and 3 (N - 1) multiplications.  The running products must
// stay inside the double range (true for the bounded physical quantities it
// is used on); the relative error is a few ulp.
template <int N> HTR_D void batch_inverse(double *v) {
  double pre[N];
  pre[0] = v[0];
#pragma unroll
  for (int k = 1; k < N; k++) pre[k] = pre[k - 1] * v[k];
  double inv = 1.0 / pre[N - 1];
#pragma unroll
  for (int k = N - 1; k > 0; k--) {
    const double vk = v[k];
    v[k] = inv * pre[k - 1];
    inv *= vk;
  }
  v[0] = inv;
}

HTR_HD double mod2(const double *v) {
  double r = 0.0;
  r += v[0] * v[0];
  r += v[1] * v[1];
  r += v[2] * v[2];
  return r;
}

}  // namespace htr
