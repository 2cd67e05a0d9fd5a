// Shared glue for the reference-build harness (test infrastructure only).
//
// Each harness translation unit #includes ONE of the reference's task
// sources (src/prometeo_*.cc) unmodified — the reference's own
// src/prometeo_metric.inl has no include guard, so the tasks cannot share a
// TU — and exposes the htr_rhs.h entry points on host buffers by building
// shim "regions" over the caller's fields and calling the reference's
// `cpu_base_impl` directly.
#ifndef HTR_ORACLE_REF_COMMON_H
#define HTR_ORACLE_REF_COMMON_H

#include <cstring>
#include <string>
#include <vector>

#include "htr_rhs.h"

struct htr_mixture_s {
  int eos;
  std::vector<unsigned char> bytes;  // a copy of the reference struct Mix
};

namespace htr_ref {

inline Legion::Rect<3> to_rect(const htr_rect3 &r) {
  return Legion::Rect<3>(Legion::Point<3>(r.lo[0], r.lo[1], r.lo[2]),
                         Legion::Point<3>(r.hi[0], r.hi[1], r.hi[2]));
}

inline void bind(Legion::PhysicalRegion &reg, Legion::FieldID fid, const htr_field &f) {
  if (f.base == nullptr) return;
  Legion::FieldBinding b;
  b.base = static_cast<char *>(f.base);
  b.stride[0] = f.stride[0];
  b.stride[1] = f.stride[1];
  b.stride[2] = f.stride[2];
  reg.fields[fid] = b;
}

// One region exposing every field of the view; its index space is `rect`.
inline Legion::PhysicalRegion make_region(const htr_fluid_view *v, const Legion::Rect<3> *rect) {
  Legion::PhysicalRegion r;
  r.lr.is.rect = rect;
  bind(r, FID_nType_x, v->nType_x);
  bind(r, FID_nType_y, v->nType_y);
  bind(r, FID_nType_z, v->nType_z);
  bind(r, FID_dcsi_e, v->dcsi_e);
  bind(r, FID_deta_e, v->deta_e);
  bind(r, FID_dzet_e, v->dzet_e);
  bind(r, FID_dcsi_d, v->dcsi_d);
  bind(r, FID_deta_d, v->deta_d);
  bind(r, FID_dzet_d, v->dzet_d);
  bind(r, FID_dcsi_s, v->dcsi_s);
  bind(r, FID_deta_s, v->deta_s);
  bind(r, FID_dzet_s, v->dzet_s);
  bind(r, FID_rho, v->rho);
  bind(r, FID_mu, v->mu);
  bind(r, FID_lam, v->lam);
  bind(r, FID_Di, v->Di);
  bind(r, FID_SoS, v->SoS);
  bind(r, FID_pressure, v->pressure);
  bind(r, FID_temperature, v->temperature);
  bind(r, FID_MassFracs, v->MassFracs);
  bind(r, FID_MolarFracs, v->MolarFracs);
  bind(r, FID_velocity, v->velocity);
  bind(r, FID_Conserved, v->Conserved);
  bind(r, FID_Conserved_old, v->Conserved_old);
  bind(r, FID_Conserved_t, v->Conserved_t);
  bind(r, FID_Conserved_t_old, v->Conserved_t_old);
  bind(r, FID_shockSensorX, v->shockSensorX);
  bind(r, FID_shockSensorY, v->shockSensorY);
  bind(r, FID_shockSensorZ, v->shockSensorZ);
  bind(r, FID_DucrosSensor, v->DucrosSensor);
  bind(r, FID_dudtBoundary, v->dudtBoundary);
  bind(r, FID_dTdtBoundary, v->dTdtBoundary);
  bind(r, FID_velocity_old_NSCBC, v->velocity_old_NSCBC);
  bind(r, FID_temperature_old_NSCBC, v->temperature_old_NSCBC);
  bind(r, FID_MolarFracs_profile, v->MolarFracs_profile);
  bind(r, FID_velocity_profile, v->velocity_profile);
  bind(r, FID_temperature_profile, v->temperature_profile);
  return r;
}

inline std::vector<Legion::PhysicalRegion> regions(const htr_fluid_view *v,
                                                   const Legion::Rect<3> *rect, int n) {
  std::vector<Legion::PhysicalRegion> out;
  for (int i = 0; i < n; i++) out.push_back(make_region(v, rect));
  return out;
}

// Task arguments hold a `Mix`, which has no default constructor: build them
// in zeroed storage and copy the mixture bytes in.
template <typename Args> struct ArgsBuf {
  alignas(Args) unsigned char storage[sizeof(Args)];
  ArgsBuf(const htr_mixture_s *m) {
    std::memset(storage, 0, sizeof(storage));
    std::memcpy(&get().mix, m->bytes.data(), sizeof(get().mix));
  }
  Args &get() { return *reinterpret_cast<Args *>(storage); }
};

inline bool valid(const htr_fluid_view *v, const htr_mixture_s *m, int eos) {
  return v != nullptr && m != nullptr && m->eos == eos;
}

}  // namespace htr_ref

#endif
