// Reference-build harness: mixture construction and the Regent-side RK
// bookkeeping (test infrastructure only).
//
// Mixtures are built with the reference's own constructors
// (src/Mixtures/ConstPropMix.inl:31-51, src/Mixtures/AirMix.hpp:319-332).
// The SSP-RK3 helpers are Regent tasks in the reference
// (src/prometeo_rk.rg:47-112); they are restated here in C++.
#include <cstdio>

#include "legion.h"
#include "prometeo_types.h"
#include "ref_common.h"

namespace {
thread_local std::string g_err;
constexpr double RK_C[3][3] = {
    {1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};

inline double *at(const htr_field &f, long long x, long long y, long long z) {
  return reinterpret_cast<double *>(static_cast<char *>(f.base) + x * f.stride[0] +
                                    y * f.stride[1] + z * f.stride[2]);
}
}  // namespace

extern "C" const char *htr_last_error(void) { return g_err.c_str(); }

extern "C" int htr_load_mixture(int eos, const void *mix, size_t bytes, htr_mixture_t *out) {
  if (mix == nullptr || out == nullptr || eos != HTR_REF_EOS_ID || bytes != sizeof(Mix)) {
    g_err = "htr_load_mixture: wrong EOS or size for this reference build";
    return HTR_ERR_ARGUMENT;
  }
  htr_mixture_s *m = new htr_mixture_s;
  m->eos = eos;
  m->bytes.assign(static_cast<const unsigned char *>(mix),
                  static_cast<const unsigned char *>(mix) + bytes);
  *out = m;
  return HTR_OK;
}

extern "C" int htr_free_mixture(htr_mixture_t m) {
  delete m;
  return HTR_OK;
}

extern "C" int htr_mixture_eos(htr_mixture_t m) { return m ? m->eos : 0; }

extern "C" size_t htr_ref_mix_sizeof(void) { return sizeof(Mix); }

extern "C" int htr_constpropmix_init(double gasConstant, double gamma, double prandtl,
                                     int viscosityModel, double p0, double p1, double p2,
                                     htr_constpropmix_t *out) {
#if HTR_REF_EOS_ID == 1
  Config c;
  std::memset(&c, 0, sizeof(c));
  c.Flow.mixture.type = MixtureModel_ConstPropMix;
  c.Flow.mixture.u.ConstPropMix.gasConstant = gasConstant;
  c.Flow.mixture.u.ConstPropMix.gamma = gamma;
  c.Flow.mixture.u.ConstPropMix.prandtl = prandtl;
  c.Flow.mixture.u.ConstPropMix.viscosityModel.type = viscosityModel;
  c.Flow.mixture.u.ConstPropMix.viscosityModel.u.Constant.Visc = p0;
  c.Flow.mixture.u.ConstPropMix.viscosityModel.u.PowerLaw.TempRef = p0;
  c.Flow.mixture.u.ConstPropMix.viscosityModel.u.PowerLaw.ViscRef = p1;
  c.Flow.mixture.u.ConstPropMix.viscosityModel.u.Sutherland.SRef = p0;
  c.Flow.mixture.u.ConstPropMix.viscosityModel.u.Sutherland.TempRef = p1;
  c.Flow.mixture.u.ConstPropMix.viscosityModel.u.Sutherland.ViscRef = p2;
  std::memset(out, 0, sizeof(*out));
  Mix m(c);
  static_assert(sizeof(Mix) == sizeof(htr_constpropmix_t), "layout");
  std::memcpy(out, &m, sizeof(Mix));
  return HTR_OK;
#else
  (void)gasConstant; (void)gamma; (void)prandtl; (void)viscosityModel;
  (void)p0; (void)p1; (void)p2; (void)out;
  return HTR_ERR_UNSUPPORTED;
#endif
}

extern "C" int htr_airmix_init(double PRef, double TRef, double LRef, const double XiRef[5],
                               htr_airmix_t *out) {
#if HTR_REF_EOS_ID == 2
  static const char *names[5] = {"N2", "O2", "NO", "N", "O"};
  Config c;
  std::memset(&c, 0, sizeof(c));
  c.Flow.mixture.type = MixtureModel_AirMix;
  c.Flow.mixture.u.AirMix.PRef = PRef;
  c.Flow.mixture.u.AirMix.TRef = TRef;
  c.Flow.mixture.u.AirMix.LRef = LRef;
  unsigned n = 0;
  for (int i = 0; i < 5; i++)
    if (XiRef[i] > 0.0) {
      std::strncpy(c.Flow.mixture.u.AirMix.XiRef.Species.values[n].Name, names[i], 9);
      c.Flow.mixture.u.AirMix.XiRef.Species.values[n].MolarFrac = XiRef[i];
      n++;
    }
  c.Flow.mixture.u.AirMix.XiRef.Species.length = n;
  std::memset(out, 0, sizeof(*out));
  Mix m(c);
  static_assert(sizeof(Mix) == sizeof(htr_airmix_t), "layout");
  std::memcpy(out, &m, sizeof(Mix));
  return HTR_OK;
#else
  (void)PRef; (void)TRef; (void)LRef; (void)XiRef; (void)out;
  return HTR_ERR_UNSUPPORTED;
#endif
}

// Offsets of selected members of the reference struct Mix, used to check
// that htr_mix.h is byte-compatible.
extern "C" int htr_ref_mix_offsets(long long *out, int n) {
#if HTR_REF_EOS_ID == 1
  const long long v[] = {(long long)offsetof(Mix, R), (long long)offsetof(Mix, gamma),
                         (long long)offsetof(Mix, viscosityModel),
                         (long long)offsetof(Mix, constantVisc),
                         (long long)offsetof(Mix, powerlawViscRef),
                         (long long)offsetof(Mix, Prandtl)};
#else
  const long long v[] = {(long long)offsetof(Mix, species[1]),
                         (long long)offsetof(Mix, species[0].W),
                         (long long)offsetof(Mix, species[0].cpCoeff.cpL),
                         (long long)offsetof(Mix, species[0].DiffCoeff.Z298),
                         (long long)offsetof(Mix, reactions[0]),
                         (long long)offsetof(Mix, reactions[1].pducts[1].nu),
                         (long long)offsetof(Mix, ThirdbodyReactions[0]),
                         (long long)offsetof(Mix, ThirdbodyReactions[2].thirdb[4].eff),
                         (long long)offsetof(Mix, PRef),
                         (long long)offsetof(Mix, TMin)};
#endif
  const int m = int(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < n && i < m; i++) out[i] = v[i];
  return m;
}

// --- Regent RK bookkeeping restated (src/prometeo_rk.rg:47-112) ----------

extern "C" int htr_InitializeTemporaries(const htr_fluid_view *v, htr_rect3 r, htr_mixture_t,
                                         htr_stream_t) {
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        const double *c = at(v->Conserved, i, j, k);
        double *o = at(v->Conserved_old, i, j, k);
        for (int e = 0; e < nEq; e++) o[e] = c[e];
      }
  return HTR_OK;
}

extern "C" int htr_InitializeTimeDerivatives(const htr_fluid_view *v, htr_rect3 r, int implicit,
                                             htr_mixture_t, htr_stream_t) {
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        double *t = at(v->Conserved_t, i, j, k);
        if (implicit) {
          const double *o = at(v->Conserved_t_old, i, j, k);
          for (int e = 0; e < nEq; e++) t[e] = -o[e];
        } else {
          for (int e = 0; e < nEq; e++) t[e] = 0.0;
        }
      }
  return HTR_OK;
}

extern "C" int htr_UpdateVars(const htr_fluid_view *v, htr_rect3 r, int stage, double deltaTime,
                              int implicit, htr_mixture_t, htr_stream_t) {
  if (stage < 1 || stage > 3) return HTR_ERR_ARGUMENT;
  double dt = deltaTime;
  if (implicit) dt *= 0.5;
  const double c1 = RK_C[stage - 1][0], c2 = RK_C[stage - 1][1], c3 = RK_C[stage - 1][2];
  for (long long k = r.lo[2]; k <= r.hi[2]; k++)
    for (long long j = r.lo[1]; j <= r.hi[1]; j++)
      for (long long i = r.lo[0]; i <= r.hi[0]; i++) {
        double *c = at(v->Conserved, i, j, k);
        const double *o = at(v->Conserved_old, i, j, k);
        const double *t = at(v->Conserved_t, i, j, k);
        for (int e = 0; e < nEq; e++) c[e] = c1 * o[e] + c2 * c[e] + c3 * t[e] * dt;
      }
  return HTR_OK;
}
