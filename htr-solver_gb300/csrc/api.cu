// extern "C" entry points of libhtr_gb300 (declared in include/htr_rhs.h).
//
// Each entry point validates its arguments on the host (null fields,
// rectangles, element alignment of bases and strides, mixture kind),
// dispatches on the loaded mixture and enqueues the kernel(s) on the
// caller's stream.  Nothing is allocated after htr_load_mixture.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "kernels.cuh"
#include "mixture_host.h"
#include "stage.cuh"

struct htr_mixture_s {
  int eos;
  htr::ConstPropDev cp;
  htr::AirDev air;
};

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, const char *what = "") {
  char buf[512];
  std::snprintf(buf, sizeof(buf), fmt, what);
  g_err = buf;
  return code;
}

int cuda_status(cudaError_t e, const char *where) {
  if (e == cudaSuccess) return HTR_OK;
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return HTR_ERR_CUDA;
}

bool rect_ok(const htr_rect3 &r) {
  for (int i = 0; i < 3; i++)
    if (r.lo[i] > r.hi[i]) return false;
  return true;
}
bool inside(const htr_rect3 &a, const htr_rect3 &b) {
  for (int i = 0; i < 3; i++)
    if (a.lo[i] < b.lo[i] || a.hi[i] > b.hi[i]) return false;
  return true;
}

// field present, base and strides aligned to the element's alignment
int check_field(const htr_field &f, size_t align, const char *name) {
  if (f.base == nullptr) return fail(HTR_ERR_ARGUMENT, "field %s is null", name);
  if (reinterpret_cast<uintptr_t>(f.base) % align != 0)
    return fail(HTR_ERR_LAYOUT, "field %s: misaligned base", name);
  for (int i = 0; i < 3; i++)
    if (f.stride[i] % (int64_t)align != 0) return fail(HTR_ERR_LAYOUT, "field %s: stride not a multiple of the element alignment", name);
  return HTR_OK;
}

#define HTR_REQ_D(V, F) \
  if (int st_ = check_field((V).F, 8, #F)) return st_;
#define HTR_REQ_I(V, F) \
  if (int st_ = check_field((V).F, 4, #F)) return st_;
#define HTR_REQ_B(V, F) \
  if (int st_ = check_field((V).F, 1, #F)) return st_;

int check_common(const htr_fluid_view *v, htr_mixture_t m, const htr_rect3 &my) {
  if (v == nullptr) return fail(HTR_ERR_ARGUMENT, "null view%s");
  if (m == nullptr) return fail(HTR_ERR_ARGUMENT, "null mixture%s");
  if (!rect_ok(my)) return fail(HTR_ERR_ARGUMENT, "inverted execution rectangle%s");
  return HTR_OK;
}

const htr_field &dirf(const htr_fluid_view &v, int d, int which) {
  // which: 0 nType, 1 m_e, 2 m_d, 3 m_s, 4 sensor
  const htr_field *t[5][3] = {{&v.nType_x, &v.nType_y, &v.nType_z},
                              {&v.dcsi_e, &v.deta_e, &v.dzet_e},
                              {&v.dcsi_d, &v.deta_d, &v.dzet_d},
                              {&v.dcsi_s, &v.deta_s, &v.dzet_s},
                              {&v.shockSensorX, &v.shockSensorY, &v.shockSensorZ}};
  return *t[which][d];
}

template <class F> int with_mix(htr_mixture_t m, F &&f) {
  if (m->eos == HTR_EOS_CONSTPROPMIX) return f(m->cp);
  if (m->eos == HTR_EOS_AIRMIX) return f(m->air);
  return fail(HTR_ERR_UNSUPPORTED, "unknown mixture kind%s");
}

int euler(const htr_fluid_view *v, htr_rect3 my, htr_rect3 fb, const double *rk, double dt,
          htr_mixture_t m, int d, int scheme, int kind, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  if (!rect_ok(fb) || !inside(my, fb)) return fail(HTR_ERR_ARGUMENT, "execution rectangle outside the grid bounds%s");
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, MassFracs);
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, Conserved_t);
  if (int st = check_field(dirf(*v, d, 0), 4, "nType")) return st;
  if (int st = check_field(dirf(*v, d, 1), 8, "m_e")) return st;
  if (scheme != 1) {
    HTR_REQ_D(*v, SoS);
    if (m->eos == HTR_EOS_AIRMIX) HTR_REQ_D(*v, Conserved_old);
  }
  if (scheme == 0)
    if (int st = check_field(dirf(*v, d, 4), 1, "shockSensor")) return st;
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_euler(*v, my, fb, rk, dt, mix, d, scheme, kind, (cudaStream_t)s), "euler");
  });
}

int diffusion(const htr_fluid_view *v, htr_rect3 my, htr_rect3 fb, htr_mixture_t m, int d, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  if (!rect_ok(fb) || !inside(my, fb)) return fail(HTR_ERR_ARGUMENT, "execution rectangle outside the grid bounds%s");
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, MolarFracs);
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, mu);
  HTR_REQ_D(*v, lam);
  HTR_REQ_D(*v, Di);
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, Conserved_t);
  for (int e = 0; e < 3; e++) {
    if (int st = check_field(dirf(*v, e, 0), 4, "nType")) return st;
    if (int st = check_field(dirf(*v, e, 2), 8, "m_d")) return st;
  }
  if (int st = check_field(dirf(*v, d, 3), 8, "m_s")) return st;
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_diffusion(*v, my, fb, mix, d, (cudaStream_t)s), "diffusion");
  });
}

int neq_of(htr_mixture_t m) { return m->eos == HTR_EOS_AIRMIX ? 9 : 5; }
int nspec_of(htr_mixture_t m) { return m->eos == HTR_EOS_AIRMIX ? 5 : 1; }


// Fixed device scratch of htr_rk3_step_static: module-scope, reserved on a
// device when this translation unit's module loads there.  The module has no
// kernels, so under CUDA's lazy module loading it loads at the first lookup
// of the array's address; htr_load_mixture does that lookup (set-up time)
// and refreshes the cached address of the current device, so the step
// itself neither loads a module nor reserves memory.  A step on a device
// where no mixture was loaded does the lookup on its first call.
constexpr size_t kStaticScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
std::mutex g_static_scratch_mu;
constexpr int kMaxDevices = 64;
void *g_static_scratch_ptr[kMaxDevices] = {};

// refresh = true: look the address up again (after a cudaDeviceReset the
// module, and the array with it, is loaded anew)
int static_scratch(void **out, bool refresh = false) {
  int dev = 0;
  if (int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice")) return st;
  if (dev < 0 || dev >= kMaxDevices) return fail(HTR_ERR_UNSUPPORTED, "device ordinal out of range%s");
  std::lock_guard<std::mutex> lock(g_static_scratch_mu);
  if (refresh || g_static_scratch_ptr[dev] == nullptr) {
    void *p = nullptr;
    if (int st = cuda_status(cudaGetSymbolAddress(&p, g_static_scratch), "scratch symbol")) return st;
    g_static_scratch_ptr[dev] = p;
  }
  if (out) *out = g_static_scratch_ptr[dev];
  return HTR_OK;
}

long long ncells_of(const htr_rect3 &r) {
  return (r.hi[0] - r.lo[0] + 1) * (r.hi[1] - r.lo[1] + 1) * (r.hi[2] - r.lo[2] + 1);
}

// Directions with more than one cell (a one-cell direction is periodic and
// contributes nothing to the RHS).
unsigned active_dirs(const htr_rect3 &r) {
  unsigned a = 0;
  for (int d = 0; d < 3; d++)
    if (r.hi[d] > r.lo[d]) a |= 1u << d;
  return a;
}

int check_step_fields(const htr_fluid_view *v, htr_mixture_t m) {
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, mu);
  HTR_REQ_D(*v, lam);
  HTR_REQ_D(*v, Di);
  HTR_REQ_D(*v, SoS);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, MassFracs);
  HTR_REQ_D(*v, MolarFracs);
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, Conserved_old);
  HTR_REQ_D(*v, Conserved_t);
  for (int d = 0; d < 3; d++) {
    if (int st = check_field(dirf(*v, d, 0), 4, "nType")) return st;
    for (int k = 1; k <= 3; k++)
      if (int st = check_field(dirf(*v, d, k), 8, "metric")) return st;
    if (int st = check_field(dirf(*v, d, 4), 1, "shockSensor")) return st;
  }
  (void)m;
  return HTR_OK;
}

}  // namespace

extern "C" int htr_InitializeTemporaries(const htr_fluid_view *, htr_rect3, htr_mixture_t, htr_stream_t);
extern "C" int htr_UpdateDucrosSensor(const htr_fluid_view *, htr_rect3, htr_rect3, double, htr_stream_t);
extern "C" int htr_CalculateMaxSpectralRadius(const htr_fluid_view *, htr_rect3, htr_mixture_t, double *, htr_stream_t);

namespace {

// Step size, sensors (once per step) and Conserved_old (src/prometeo.rg:1342-1380).
// dt, sensors and (unless the step starts with implicit chemistry, which
// moves it after the chemistry solve) InitializeTemporaries of one step.
int step_prologue(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
                  htr_mixture_t m, double *dt_out, htr_stream_t s, unsigned sensor_dirs = 7u) {
  if (p == nullptr) return fail(HTR_ERR_ARGUMENT, "null step parameters%s");
  if (int st = check_common(v, m, inner)) return st;
  if (p->scheme < HTR_SCHEME_HYBRID || p->scheme > HTR_SCHEME_SKEW) return fail(HTR_ERR_ARGUMENT, "unknown scheme%s");
  const cudaStream_t cs = (cudaStream_t)s;
  double dt = p->deltaTime;
  if (p->cfl > 0.0) {
    // the radius lands in Conserved_t[first cell][0], which the stage overwrites anyway
    double *scratch = reinterpret_cast<double *>(static_cast<char *>(v->Conserved_t.base) +
                                                 inner.lo[0] * v->Conserved_t.stride[0] +
                                                 inner.lo[1] * v->Conserved_t.stride[1] +
                                                 inner.lo[2] * v->Conserved_t.stride[2]);
    if (int st = htr_CalculateMaxSpectralRadius(v, inner, m, scratch, s)) return st;
    double r = 0.0;
    if (int st = cuda_status(cudaMemcpyAsync(&r, scratch, sizeof(double), cudaMemcpyDeviceToHost, cs), "dt read")) return st;
    if (int st = cuda_status(cudaStreamSynchronize(cs), "dt sync")) return st;
    if (!(r > 0.0)) return fail(HTR_ERR_ARGUMENT, "non-positive spectral radius%s");
    dt = p->cfl / r;
  }
  if (!(dt > 0.0)) return fail(HTR_ERR_ARGUMENT, "non-positive time step%s");
  *dt_out = dt;
  int st;
  if (p->scheme == HTR_SCHEME_HYBRID) {
    if ((st = htr_UpdateDucrosSensor(v, fb, fb, p->vorticityScale, s))) return st;
    if ((st = check_field(v->shockSensorX, 1, "shockSensorX")) || (st = check_field(v->shockSensorY, 1, "shockSensorY")) ||
        (st = check_field(v->shockSensorZ, 1, "shockSensorZ")))
      return st;
    if ((st = cuda_status(htr::launch_shock_sensor(*v, fb, fb, nspec_of(m), (int)sensor_dirs, cs),
                          "shock sensors")))
      return st;
  }
  if (p->implicitChemistry) return check_field(v->Conserved_t_old, 8, "Conserved_t_old");
  return htr_InitializeTemporaries(v, fb, m, s);
}

// The implicit chemistry block at the start of a step (src/prometeo.rg:1360-1398)
// after the transport RHS of the start state is in Conserved_t: UpdateChemistry
// over dt, then UpdatePrimitivesAndBCsFromConserved (primitives of the
// interior, properties everywhere) and InitializeTemporaries.
// skip_ghosts (the fused path, where `inner` is the whole grid): the
// boundary ghost nodes of packed instances keep their imposed state.
// dt_cell (the per-cell step sizes of packed instances, dense over `inner`)
// replaces dt where given.
int implicit_chemistry_block(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, htr_mixture_t m, double dt,
                             int *status_dev, htr_stream_t s, unsigned skip_ghosts = 0,
                             const double *dt_cell = nullptr) {
  const cudaStream_t cs = (cudaStream_t)s;
  int st;
  if ((st = check_common(v, m, inner))) return st;
  if ((st = with_mix(m, [&](const auto &mix) {
         return cuda_status(
             htr::launch_update_chemistry(*v, inner, dt, mix, status_dev, cs, skip_ghosts, dt_cell),
             "UpdateChemistry");
       })))
    return st;
  if ((st = with_mix(m, [&](const auto &mix) {
         return cuda_status(htr::launch_primitive(*v, inner, mix, status_dev, cs, skip_ghosts), "primitive");
       })))
    return st;
  if ((st = htr_UpdatePropertiesFromPrimitive(v, fb, m, s))) return st;
  return htr_InitializeTemporaries(v, fb, m, s);
}

// Three stages of the fused pipeline (one prepass, Euler KG + TENO faces,
// diffusion faces and one per-cell update kernel per stage).
int fused_step(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
               htr_mixture_t m, const htr::StageWorkspace &w, double *dt_used, int *status_dev, htr_stream_t s,
               const double *dt_cell = nullptr) {
  double dt = 0.0;
  // the fused stages read the sensors of the active directions only
  if (int st = step_prologue(v, inner, fb, p, m, &dt, s, active_dirs(inner))) return st;
  if (dt_used) *dt_used = dt;
  htr::StageParams sp;
  sp.dt_cell = dt_cell;
  sp.scheme = p->scheme == HTR_SCHEME_HYBRID ? 0 : (p->scheme == HTR_SCHEME_SKEW ? 1 : 2);
  sp.kind = p->scheme == HTR_SCHEME_TENOA ? htr::kTENOA : (p->scheme == HTR_SCHEME_TENOLAD ? htr::kTENOLAD : htr::kTENO);
  sp.chemistry = p->explicitChemistry ? 1 : 0;
  sp.dt = dt;
  sp.active = active_dirs(inner);
  // the temperature cache of the update kernel starts empty every step
  if (int st = cuda_status(cudaMemsetAsync(w.tcache, 0, sizeof(double) * 3 * ncells_of(inner), (cudaStream_t)s),
                           "cache reset"))
    return st;
  if (p->implicitChemistry) {
    // transport RHS of the start state, then the chemistry solve
    sp.mode = htr::kStageRhsOnly;
    sp.stage = 1;
    if (int st = with_mix(m, [&](const auto &mix) {
          return cuda_status(htr::launch_stage(*v, inner, fb, mix, w, sp, status_dev, (cudaStream_t)s), "stage");
        }))
      return st;
    if (int st = implicit_chemistry_block(v, inner, fb, m, dt, status_dev, s, active_dirs(inner), dt_cell))
      return st;
    sp.mode = htr::kStageImplicit;
  }
  for (int stage = 1; stage <= 3; stage++) {
    sp.stage = stage;
    if (int st = with_mix(m, [&](const auto &mix) {
          return cuda_status(htr::launch_stage(*v, inner, fb, mix, w, sp, status_dev, (cudaStream_t)s), "stage");
        }))
      return st;
  }
  return HTR_OK;
}

}  // namespace

namespace htr {
// the message htr_last_error() returns, for entry points in other files
int set_last_error(int code, const std::string &msg) {
  g_err = msg;
  return code;
}
}  // namespace htr

extern "C" {


const char *htr_last_error(void) { return g_err.c_str(); }

int htr_load_mixture(int eos, const void *mix, size_t bytes, htr_mixture_t *out) {
  if (mix == nullptr || out == nullptr) return fail(HTR_ERR_ARGUMENT, "null argument%s");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(HTR_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return fail(HTR_ERR_NO_DEVICE, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
  if (prop.major != 10 || prop.minor != 3)
    return fail(HTR_ERR_NO_DEVICE, "the library targets sm_103 (GB300); device is %s", prop.name);
  // set-up of htr_rk3_step_static on this device (loads its module)
  if (int st = static_scratch(nullptr, true)) return st;
  htr_mixture_s *m = new (std::nothrow) htr_mixture_s();
  if (m == nullptr) return fail(HTR_ERR_ARGUMENT, "out of host memory%s");
  m->eos = eos;
  bool ok = false;
  if (eos == HTR_EOS_CONSTPROPMIX && bytes == sizeof(htr_constpropmix_t))
    ok = htr::derive(*static_cast<const htr_constpropmix_t *>(mix), m->cp);
  else if (eos == HTR_EOS_AIRMIX && bytes == sizeof(htr_airmix_t))
    ok = htr::derive(*static_cast<const htr_airmix_t *>(mix), m->air);
  if (!ok) {
    delete m;
    return fail(HTR_ERR_ARGUMENT, "htr_load_mixture: unknown EOS, wrong struct size or unusable data%s");
  }
  *out = m;
  return HTR_OK;
}

int htr_free_mixture(htr_mixture_t m) {
  delete m;
  return HTR_OK;
}

int htr_mixture_eos(htr_mixture_t m) { return m ? m->eos : 0; }

#define HTR_EULER_EP(NAME, D, SCHEME, KIND)                                                         \
  int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, const double rk[2], double dt,       \
           htr_mixture_t mix, htr_stream_t s) {                                                     \
    return euler(v, m, b, rk, dt, mix, D, SCHEME, KIND, s);                                         \
  }
HTR_EULER_EP(htr_UpdateUsingHybridEulerFluxX, 0, 0, 0)
HTR_EULER_EP(htr_UpdateUsingHybridEulerFluxY, 1, 0, 0)
HTR_EULER_EP(htr_UpdateUsingHybridEulerFluxZ, 2, 0, 0)
HTR_EULER_EP(htr_UpdateUsingTENOEulerFluxX, 0, 2, 0)
HTR_EULER_EP(htr_UpdateUsingTENOEulerFluxY, 1, 2, 0)
HTR_EULER_EP(htr_UpdateUsingTENOEulerFluxZ, 2, 2, 0)
HTR_EULER_EP(htr_UpdateUsingTENOAEulerFluxX, 0, 2, 1)
HTR_EULER_EP(htr_UpdateUsingTENOAEulerFluxY, 1, 2, 1)
HTR_EULER_EP(htr_UpdateUsingTENOAEulerFluxZ, 2, 2, 1)
HTR_EULER_EP(htr_UpdateUsingTENOLADEulerFluxX, 0, 2, 2)
HTR_EULER_EP(htr_UpdateUsingTENOLADEulerFluxY, 1, 2, 2)
HTR_EULER_EP(htr_UpdateUsingTENOLADEulerFluxZ, 2, 2, 2)
#undef HTR_EULER_EP

#define HTR_SKEW_EP(NAME, D)                                                                        \
  int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t mix, htr_stream_t s) { \
    return euler(v, m, b, nullptr, 0.0, mix, D, 1, 0, s);                                           \
  }
HTR_SKEW_EP(htr_UpdateUsingSkewSymmetricEulerFluxX, 0)
HTR_SKEW_EP(htr_UpdateUsingSkewSymmetricEulerFluxY, 1)
HTR_SKEW_EP(htr_UpdateUsingSkewSymmetricEulerFluxZ, 2)
#undef HTR_SKEW_EP

#define HTR_DIFF_EP(NAME, D)                                                                        \
  int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t mix, htr_stream_t s) { \
    return diffusion(v, m, b, mix, D, s);                                                           \
  }
HTR_DIFF_EP(htr_UpdateUsingDiffusionFluxX, 0)
HTR_DIFF_EP(htr_UpdateUsingDiffusionFluxY, 1)
HTR_DIFF_EP(htr_UpdateUsingDiffusionFluxZ, 2)
#undef HTR_DIFF_EP

int htr_UpdateDucrosSensor(const htr_fluid_view *v, htr_rect3 my, htr_rect3 fb, double vorticityScale,
                           htr_stream_t s) {
  if (v == nullptr || !rect_ok(my) || !rect_ok(fb) || !inside(my, fb))
    return fail(HTR_ERR_ARGUMENT, "bad view or rectangle%s");
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, DucrosSensor);
  for (int e = 0; e < 3; e++) {
    if (int st = check_field(dirf(*v, e, 0), 4, "nType")) return st;
    if (int st = check_field(dirf(*v, e, 2), 8, "m_d")) return st;
  }
  return cuda_status(htr::launch_ducros(*v, my, fb, vorticityScale, (cudaStream_t)s), "ducros");
}

static int shock(const htr_fluid_view *v, htr_rect3 my, htr_rect3 fb, htr_mixture_t m, int d, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  if (!rect_ok(fb) || !inside(my, fb)) return fail(HTR_ERR_ARGUMENT, "execution rectangle outside the grid bounds%s");
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, DucrosSensor);
  if (int st = check_field(dirf(*v, d, 0), 4, "nType")) return st;
  if (int st = check_field(dirf(*v, d, 4), 1, "shockSensor")) return st;
  return cuda_status(htr::launch_shock_sensor(*v, my, fb, nspec_of(m), 1 << d, (cudaStream_t)s), "shock sensor");
}
int htr_UpdateShockSensorX(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t x, htr_stream_t s) {
  return shock(v, m, b, x, 0, s);
}
int htr_UpdateShockSensorY(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t x, htr_stream_t s) {
  return shock(v, m, b, x, 1, s);
}
int htr_UpdateShockSensorZ(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t x, htr_stream_t s) {
  return shock(v, m, b, x, 2, s);
}

int htr_AddChemistrySources(const htr_fluid_view *v, htr_rect3 my, htr_mixture_t m, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, MassFracs);
  HTR_REQ_D(*v, Conserved_t);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_chem_sources(*v, my, mix, (cudaStream_t)s), "chemistry sources");
  });
}

int htr_UpdateChemistry(const htr_fluid_view *v, htr_rect3 my, double dt, htr_mixture_t m, int *status,
                        htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, Conserved_t);
  HTR_REQ_D(*v, Conserved_t_old);
  HTR_REQ_D(*v, temperature);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_update_chemistry(*v, my, dt, mix, status, (cudaStream_t)s), "UpdateChemistry");
  });
}

int htr_UpdatePropertiesFromPrimitive(const htr_fluid_view *v, htr_rect3 my, htr_mixture_t m, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, MolarFracs);
  HTR_REQ_D(*v, MassFracs);
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, mu);
  HTR_REQ_D(*v, lam);
  HTR_REQ_D(*v, Di);
  HTR_REQ_D(*v, SoS);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_properties(*v, my, mix, (cudaStream_t)s), "properties");
  });
}

int htr_UpdateConservedFromPrimitive(const htr_fluid_view *v, htr_rect3 my, htr_mixture_t m, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  HTR_REQ_D(*v, MassFracs);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, Conserved);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_conserved(*v, my, mix, (cudaStream_t)s), "conserved");
  });
}

int htr_UpdatePrimitiveFromConserved(const htr_fluid_view *v, htr_rect3 my, htr_mixture_t m, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, MolarFracs);
  HTR_REQ_D(*v, velocity);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_primitive(*v, my, mix, nullptr, (cudaStream_t)s), "primitive");
  });
}

int htr_CalculateMaxSpectralRadius(const htr_fluid_view *v, htr_rect3 my, htr_mixture_t m, double *result,
                                   htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  if (result == nullptr) return fail(HTR_ERR_ARGUMENT, "null result%s");
  HTR_REQ_D(*v, dcsi_d);
  HTR_REQ_D(*v, deta_d);
  HTR_REQ_D(*v, dzet_d);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, MassFracs);
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, mu);
  HTR_REQ_D(*v, lam);
  HTR_REQ_D(*v, Di);
  HTR_REQ_D(*v, SoS);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_spectral_radius(*v, my, mix, result, (cudaStream_t)s), "spectral radius");
  });
}

int htr_InitializeTemporaries(const htr_fluid_view *v, htr_rect3 my, htr_mixture_t m, htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, Conserved_old);
  return cuda_status(htr::launch_copy_conserved(*v, my, neq_of(m), (cudaStream_t)s), "InitializeTemporaries");
}

int htr_InitializeTimeDerivatives(const htr_fluid_view *v, htr_rect3 my, int implicit, htr_mixture_t m,
                                  htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  HTR_REQ_D(*v, Conserved_t);
  if (implicit) HTR_REQ_D(*v, Conserved_t_old);
  return cuda_status(htr::launch_init_rhs(*v, my, neq_of(m), implicit, (cudaStream_t)s), "InitializeTimeDerivatives");
}

int htr_UpdateVars(const htr_fluid_view *v, htr_rect3 my, int stage, double dt, int implicit, htr_mixture_t m,
                   htr_stream_t s) {
  if (int st = check_common(v, m, my)) return st;
  if (stage < 1 || stage > 3) return fail(HTR_ERR_ARGUMENT, "stage must be 1, 2 or 3%s");
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, Conserved_old);
  HTR_REQ_D(*v, Conserved_t);
  return cuda_status(htr::launch_rk_update(*v, my, neq_of(m), stage, dt, implicit, (cudaStream_t)s), "UpdateVars");
}

// One SSP-RK3 time step of a periodic grid in the reference's driver order.
}  // extern "C"

namespace {

int nscbc_common(const htr_fluid_view *v, htr_mixture_t m, const htr_rect3 &bc, int dir) {
  if (int st = check_common(v, m, bc)) return st;
  if (bc.lo[dir] != bc.hi[dir]) return fail(HTR_ERR_ARGUMENT, "the boundary region must be one plane thick%s");
  HTR_REQ_D(*v, MassFracs);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, rho);
  HTR_REQ_D(*v, SoS);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, Conserved_t);
  if (int st = check_field(dirf(*v, dir, 0), 4, "nType")) return st;
  if (int st = check_field(dirf(*v, dir, 2), 8, "m_d")) return st;
  return HTR_OK;
}

int nscbc_inflow(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, int dir, bool minus, htr_stream_t s) {
  if (int st = nscbc_common(v, m, bc, dir)) return st;
  HTR_REQ_D(*v, dudtBoundary);
  HTR_REQ_D(*v, dTdtBoundary);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_nscbc_inflow(*v, bc, mix, dir, minus, (cudaStream_t)s), "nscbc inflow");
  });
}

int nscbc_outflow(const htr_fluid_view *v, htr_rect3 bc, htr_rect3 fb, htr_mixture_t m, int dir, bool minus,
                  double MaxMach, double LengthScale, double PInf, htr_stream_t s) {
  if (int st = nscbc_common(v, m, bc, dir)) return st;
  if (!rect_ok(fb) || !inside(bc, fb)) return fail(HTR_ERR_ARGUMENT, "boundary plane outside the grid bounds%s");
  HTR_REQ_D(*v, mu);
  HTR_REQ_D(*v, Conserved);
  for (int e = 0; e < 3; e++) {
    if (int st = check_field(dirf(*v, e, 0), 4, "nType")) return st;
    if (int st = check_field(dirf(*v, e, 2), 8, "m_d")) return st;
  }
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_nscbc_outflow(*v, bc, fb, mix, dir, minus, MaxMach, LengthScale, PInf,
                                                 (cudaStream_t)s),
                       "nscbc outflow");
  });
}

}  // namespace

extern "C" {

#define HTR_NSCBC(SIDE, DIR, MINUS)                                                                           \
  int htr_UpdateUsingFluxNSCBCInflow##SIDE(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m,            \
                                           htr_stream_t s) {                                                  \
    return nscbc_inflow(v, bc, m, DIR, MINUS, s);                                                             \
  }                                                                                                           \
  int htr_UpdateUsingFluxNSCBCOutflow##SIDE(const htr_fluid_view *v, htr_rect3 bc, htr_rect3 fb, htr_mixture_t m, \
                                            double MaxMach, double LengthScale, double PInf, htr_stream_t s) {  \
    return nscbc_outflow(v, bc, fb, m, DIR, MINUS, MaxMach, LengthScale, PInf, s);                          \
  }
HTR_NSCBC(XNeg, 0, true)
HTR_NSCBC(XPos, 0, false)
HTR_NSCBC(YNeg, 1, true)
HTR_NSCBC(YPos, 1, false)
HTR_NSCBC(ZNeg, 2, true)
HTR_NSCBC(ZPos, 2, false)
#undef HTR_NSCBC

static int inflow_state(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, int dir,
                        htr_stream_t s) {
  if (int st = check_common(v, m, bc)) return st;
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, SoS);
  HTR_REQ_D(*v, MolarFracs_profile);
  HTR_REQ_D(*v, temperature_profile);
  HTR_REQ_D(*v, velocity_profile);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, MolarFracs);
  HTR_REQ_D(*v, velocity);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_inflow_state(*v, bc, mix, Pbc, dir, (cudaStream_t)s), "nscbc inflow state");
  });
}
int htr_SetNSCBC_InflowBCX(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t s) {
  return inflow_state(v, bc, m, Pbc, 0, s);
}
int htr_SetNSCBC_InflowBCY(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t s) {
  return inflow_state(v, bc, m, Pbc, 1, s);
}
int htr_SetNSCBC_InflowBCZ(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t s) {
  return inflow_state(v, bc, m, Pbc, 2, s);
}
int htr_SetNSCBC_OutflowBC(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, int *status_dev, htr_stream_t s) {
  if (int st = check_common(v, m, bc)) return st;
  HTR_REQ_D(*v, Conserved);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, MolarFracs);
  HTR_REQ_D(*v, velocity);
  return with_mix(m, [&](const auto &mix) {
    return cuda_status(htr::launch_primitive(*v, bc, mix, status_dev, (cudaStream_t)s), "nscbc outflow state");
  });
}
static int wall_state(const htr_fluid_view *v, htr_rect3 bc, int side, htr_mixture_t m, bool iso, htr_stream_t s) {
  if (int st = check_common(v, m, bc)) return st;
  if (side < 0 || side > 5) return fail(HTR_ERR_ARGUMENT, "side must be 0..5%s");
  if (bc.lo[side / 2] != bc.hi[side / 2]) return fail(HTR_ERR_ARGUMENT, "the boundary region must be one plane thick%s");
  HTR_REQ_D(*v, MolarFracs);
  HTR_REQ_D(*v, pressure);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, velocity);
  if (iso) HTR_REQ_D(*v, temperature_profile);
  return cuda_status(htr::launch_wall_state(*v, bc, nspec_of(m), side, iso, (cudaStream_t)s), "wall state");
}
int htr_SetIsothermalWallBC(const htr_fluid_view *v, htr_rect3 bc, int side, htr_mixture_t m, htr_stream_t s) {
  return wall_state(v, bc, side, m, true, s);
}
int htr_SetAdiabaticWallBC(const htr_fluid_view *v, htr_rect3 bc, int side, htr_mixture_t m, htr_stream_t s) {
  return wall_state(v, bc, side, m, false, s);
}
int htr_UpdateNSCBCGhostCellTimeDerivatives(const htr_fluid_view *v, htr_rect3 bc, double dt, htr_stream_t s) {
  if (v == nullptr || !rect_ok(bc)) return fail(HTR_ERR_ARGUMENT, "null view or inverted rectangle%s");
  if (!(dt > 0.0)) return fail(HTR_ERR_ARGUMENT, "non-positive time step%s");
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, temperature);
  HTR_REQ_D(*v, dudtBoundary);
  HTR_REQ_D(*v, dTdtBoundary);
  HTR_REQ_D(*v, velocity_old_NSCBC);
  HTR_REQ_D(*v, temperature_old_NSCBC);
  return cuda_status(htr::launch_nscbc_time_derivatives(*v, bc, dt, (cudaStream_t)s), "nscbc time derivatives");
}

int htr_rk3_teno_face_counts(htr_rect3 inner, htr_mixture_t m, const void *workspace, size_t workspace_bytes,
                             unsigned long long counts[3], htr_stream_t s) {
  if (m == nullptr || counts == nullptr || !rect_ok(inner)) return fail(HTR_ERR_ARGUMENT, "null or bad argument%s");
  htr::StageWorkspace w;
  if (!htr::stage_workspace_carve(const_cast<void *>(workspace), workspace_bytes, inner, neq_of(m), w))
    return fail(HTR_ERR_ARGUMENT, "workspace null or smaller than htr_rk3_workspace_bytes%s");
  unsigned c[3] = {0u, 0u, 0u};
  const cudaStream_t cs = (cudaStream_t)s;
  int st;
  if ((st = cuda_status(cudaMemcpyAsync(c, w.count, sizeof(c), cudaMemcpyDeviceToHost, cs), "teno counts")) ||
      (st = cuda_status(cudaStreamSynchronize(cs), "teno counts sync")))
    return st;
  for (int d = 0; d < 3; d++) counts[d] = c[d];
  return HTR_OK;
}

int htr_decision_counters(int enable, unsigned long long counts[HTR_DECISION_COUNTERS]) {
  if (counts == nullptr) return fail(HTR_ERR_ARGUMENT, "null counts%s");
  for (int k = 0; k < HTR_DECISION_COUNTERS; k++) counts[k] = 0ull;
  int st;
  if ((st = cuda_status(cudaDeviceSynchronize(), "decision counters sync"))) return st;
  if ((st = cuda_status(htr::decision_counters_euler(enable, counts), "decision counters")) ||
      (st = cuda_status(htr::decision_counters_stage_euler(enable, counts), "decision counters")) ||
      (st = cuda_status(htr::decision_counters_sensor(enable, counts), "decision counters")))
    return st;
  return HTR_OK;
}

int htr_rk3_set_tuning(const htr_stage_tuning *t) {
  if (t == nullptr) return fail(HTR_ERR_ARGUMENT, "null tuning%s");
  auto pow2_in = [](int v, int lo, int hi) { return v >= lo && v <= hi && (v & (v - 1)) == 0; };
  if (!pow2_in(t->prepass_block, 64, 256) || !pow2_in(t->diffusion_block, 32, 128) ||
      !pow2_in(t->update_block, 32, 128) || t->teno_blocks_per_sm < 0 || t->teno_blocks_per_sm > 32 ||
      !(t->kg_x_tile == 64 || t->kg_x_tile == 128 || t->kg_x_tile == 256))
    return fail(HTR_ERR_ARGUMENT, "tuning value outside the supported set%s");
  htr::StageTuning &g = htr::stage_tuning();
  g.prepass_block = t->prepass_block;
  g.diffusion_block = t->diffusion_block;
  g.update_block = t->update_block;
  g.teno_blocks_per_sm = t->teno_blocks_per_sm;
  g.kg_x_tile = t->kg_x_tile;
  return HTR_OK;
}

int htr_rk3_get_tuning(htr_stage_tuning *t) {
  if (t == nullptr) return fail(HTR_ERR_ARGUMENT, "null tuning%s");
  const htr::StageTuning &g = htr::stage_tuning();
  t->prepass_block = g.prepass_block;
  t->diffusion_block = g.diffusion_block;
  t->update_block = g.update_block;
  t->teno_blocks_per_sm = g.teno_blocks_per_sm;
  t->kg_x_tile = g.kg_x_tile;
  return HTR_OK;
}

static int check_metric_fields(const htr_fluid_view *v, const htr_field &cc) {
  if (v == nullptr) return fail(HTR_ERR_ARGUMENT, "null view%s");
  if (int st = check_field(cc, 8, "centerCoordinates")) return st;
  HTR_REQ_I(*v, nType_x);
  HTR_REQ_I(*v, nType_y);
  HTR_REQ_I(*v, nType_z);
  HTR_REQ_D(*v, dcsi_e);
  HTR_REQ_D(*v, deta_e);
  HTR_REQ_D(*v, dzet_e);
  return HTR_OK;
}

int htr_InitializeMetric(const htr_fluid_view *v, htr_field cc, htr_rect3 my, htr_rect3 fb, const double width[3],
                         htr_stream_t s) {
  if (int st = check_metric_fields(v, cc)) return st;
  if (width == nullptr) return fail(HTR_ERR_ARGUMENT, "null width%s");
  if (!rect_ok(my) || !rect_ok(fb) || !inside(my, fb))
    return fail(HTR_ERR_ARGUMENT, "execution rectangle outside the grid bounds%s");
  HTR_REQ_D(*v, dcsi_d);
  HTR_REQ_D(*v, deta_d);
  HTR_REQ_D(*v, dzet_d);
  HTR_REQ_D(*v, dcsi_s);
  HTR_REQ_D(*v, deta_s);
  HTR_REQ_D(*v, dzet_s);
  return cuda_status(htr::launch_init_metric(*v, cc, my, fb, width, (cudaStream_t)s), "initialize metric");
}

static int correct_metric(const htr_fluid_view *v, const htr_field &cc, const htr_rect3 &my, int dir, htr_stream_t s) {
  if (int st = check_metric_fields(v, cc)) return st;
  if (!rect_ok(my)) return fail(HTR_ERR_ARGUMENT, "inverted execution rectangle%s");
  return cuda_status(htr::launch_correct_metric(*v, cc, my, dir, (cudaStream_t)s), "correct ghost metric");
}
int htr_CorrectGhostMetricX(const htr_fluid_view *v, htr_field cc, htr_rect3 my, htr_stream_t s) {
  return correct_metric(v, cc, my, 0, s);
}
int htr_CorrectGhostMetricY(const htr_fluid_view *v, htr_field cc, htr_rect3 my, htr_stream_t s) {
  return correct_metric(v, cc, my, 1, s);
}
int htr_CorrectGhostMetricZ(const htr_fluid_view *v, htr_field cc, htr_rect3 my, htr_stream_t s) {
  return correct_metric(v, cc, my, 2, s);
}

int htr_CalculateMaxMachNumber(const htr_fluid_view *v, htr_rect3 my, int dir, double *result, htr_stream_t s) {
  if (v == nullptr || result == nullptr || dir < 0 || dir > 2) return fail(HTR_ERR_ARGUMENT, "null argument or bad direction%s");
  if (!rect_ok(my)) return fail(HTR_ERR_ARGUMENT, "inverted rectangle%s");
  HTR_REQ_D(*v, velocity);
  HTR_REQ_D(*v, SoS);
  return cuda_status(htr::launch_max_mach(*v, my, dir, result, (cudaStream_t)s), "max mach");
}

int htr_rk3_step(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
                 htr_mixture_t m, double *dt_used, int *status_dev, htr_stream_t s) {
  static const double RK[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
  const cudaStream_t cs = (cudaStream_t)s;
  double dt = 0.0;
  int st;
  if ((st = step_prologue(v, inner, fb, p, m, &dt, s))) return st;
  if (dt_used) *dt_used = dt;
  const int implicit = p->implicitChemistry ? 1 : 0;
  // UpdateDerivatives (src/prometeo.rg:480-606) with the given limiter
  // arguments: time derivatives from zero or from -Conserved_t_old,
  // explicit chemistry sources, Euler Z, Y, X, diffusion Z, Y, X
  auto derivatives = [&](const double rk[2], double sdt, int old) -> int {
    int e;
    if ((e = htr_InitializeTimeDerivatives(v, fb, old, m, s))) return e;
    if (p->explicitChemistry && !implicit)
      if ((e = htr_AddChemistrySources(v, inner, m, s))) return e;
    for (int d = 2; d >= 0; d--) {
      if (p->scheme == HTR_SCHEME_SKEW)
        e = euler(v, inner, fb, nullptr, 0.0, m, d, 1, 0, s);
      else if (p->scheme == HTR_SCHEME_HYBRID)
        e = euler(v, inner, fb, rk, sdt, m, d, 0, 0, s);
      else
        e = euler(v, inner, fb, rk, sdt, m, d, 2, p->scheme - 1, s);
      if (e) return e;
    }
    for (int d = 2; d >= 0; d--)
      if ((e = diffusion(v, inner, fb, m, d, s))) return e;
    return (int)HTR_OK;
  };
  if (implicit) {
    const double rk0[2] = {0.0, 1.0};
    if ((st = derivatives(rk0, dt * 0.5, 0))) return st;
    if ((st = implicit_chemistry_block(v, inner, fb, m, dt, status_dev, s))) return st;
  }
  for (int stage = 1; stage <= 3; stage++) {
    const double rk[2] = {RK[stage - 1][0], RK[stage - 1][1]};
    double sdt = dt * RK[stage - 1][2];
    if (implicit) sdt *= 0.5;
    if ((st = derivatives(rk, sdt, implicit))) return st;
    // ghost cells keep their imposed state (the reference restores them
    // from their primitives after the update)
    if ((st = htr_UpdateVars(v, inner, stage, dt, implicit, m, s))) return st;
    if ((st = check_common(v, m, inner))) return st;
    if ((st = with_mix(m, [&](const auto &mix) {
           return cuda_status(htr::launch_primitive(*v, inner, mix, status_dev, cs), "primitive");
         })))
      return st;
    if ((st = htr_UpdatePropertiesFromPrimitive(v, fb, m, s))) return st;
  }
  return HTR_OK;
}

size_t htr_rk3_workspace_bytes(htr_rect3 interior, htr_mixture_t m) {
  if (m == nullptr || !rect_ok(interior)) return 0;
  return htr::stage_workspace_bytes(interior, neq_of(m));
}

int htr_rk3_step_ws(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
                    htr_mixture_t m, void *workspace, size_t workspace_bytes, double *dt_used,
                    int *status_dev, htr_stream_t s) {
  int st;
  if ((st = check_common(v, m, inner))) return st;
  if ((st = check_step_fields(v, m))) return st;
  for (int i = 0; i < 3; i++)
    if (inner.lo[i] != fb.lo[i] || inner.hi[i] != fb.hi[i])
      return fail(HTR_ERR_UNSUPPORTED, "the fused step needs a grid periodic in every direction (interior == bounds)%s");
  htr::StageWorkspace w;
  if (!htr::stage_workspace_carve(workspace, workspace_bytes, inner, neq_of(m), w))
    return fail(HTR_ERR_ARGUMENT, "workspace null or smaller than htr_rk3_workspace_bytes%s");
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return fail(HTR_ERR_LAYOUT, "workspace not 256-byte aligned%s");
  return fused_step(v, inner, fb, p, m, w, dt_used, status_dev, s);
}

int htr_rk3_step_cells_ws(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
                          htr_mixture_t m, const double *dt_cell, void *workspace, size_t workspace_bytes,
                          int *status_dev, htr_stream_t s) {
  int st;
  if (p == nullptr || dt_cell == nullptr) return fail(HTR_ERR_ARGUMENT, "null step parameters or step sizes%s");
  if (p->cfl > 0.0) return fail(HTR_ERR_ARGUMENT, "per-cell step sizes take no CFL step size%s");
  if (reinterpret_cast<uintptr_t>(dt_cell) % 8 != 0) return fail(HTR_ERR_LAYOUT, "dt_cell not 8-byte aligned%s");
  if ((st = check_common(v, m, inner))) return st;
  if ((st = check_step_fields(v, m))) return st;
  for (int i = 0; i < 3; i++)
    if (inner.lo[i] != fb.lo[i] || inner.hi[i] != fb.hi[i])
      return fail(HTR_ERR_UNSUPPORTED, "the fused step needs a grid periodic in every direction (interior == bounds)%s");
  htr::StageWorkspace w;
  if (!htr::stage_workspace_carve(workspace, workspace_bytes, inner, neq_of(m), w))
    return fail(HTR_ERR_ARGUMENT, "workspace null or smaller than htr_rk3_workspace_bytes%s");
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return fail(HTR_ERR_LAYOUT, "workspace not 256-byte aligned%s");
  htr_step_params q = *p;
  q.deltaTime = 1.0;  // unused: every cell takes its own step size
  return fused_step(v, inner, fb, &q, m, w, nullptr, status_dev, s, dt_cell);
}

static int check_bc_params(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_bc_params *bc) {
  if (bc == nullptr) return fail(HTR_ERR_ARGUMENT, "null boundary parameters%s");
  for (int d = 0; d < 3; d++) {
    const int a = bc->type[2 * d], b = bc->type[2 * d + 1];
    for (int t : {a, b})
      if (t < HTR_BC_PERIODIC || t > HTR_BC_ADIABATIC_WALL) return fail(HTR_ERR_ARGUMENT, "unknown boundary type%s");
    if ((a == HTR_BC_PERIODIC) != (b == HTR_BC_PERIODIC))
      return fail(HTR_ERR_ARGUMENT, "a periodic direction is periodic on both sides%s");
    const int g = (a == HTR_BC_PERIODIC) ? 0 : 1;
    if (inner.lo[d] != fb.lo[d] + g || inner.hi[d] != fb.hi[d] - g || fb.hi[d] - fb.lo[d] < 4 * g)
      return fail(HTR_ERR_ARGUMENT, "interior must be the bounds less one ghost layer on each non-periodic side%s");
    for (int side = 2 * d; side < 2 * d + 2; side++) {
      if (bc->type[side] == HTR_BC_PERIODIC) continue;
      const htr_rect3 &r = bc->plane[side];
      const int64_t at = (side % 2 == 0) ? fb.lo[d] : fb.hi[d];
      if (!rect_ok(r) || !inside(r, fb) || r.lo[d] != at || r.hi[d] != at)
        return fail(HTR_ERR_ARGUMENT, "a boundary plane is not the side's ghost layer%s");
      if (bc->type[side] == HTR_BC_NSCBC_OUTFLOW && !(bc->LengthScale[side] > 0.0))
        return fail(HTR_ERR_ARGUMENT, "outflow LengthScale must be positive%s");
    }
  }
  bool inflow = false, iso = false;
  for (int k = 0; k < 6; k++) {
    inflow = inflow || bc->type[k] == HTR_BC_NSCBC_INFLOW;
    iso = iso || bc->type[k] == HTR_BC_ISOTHERMAL_WALL;
  }
  if (inflow) {
    HTR_REQ_D(*v, MolarFracs_profile);
    HTR_REQ_D(*v, velocity_profile);
    HTR_REQ_D(*v, temperature_profile);
    HTR_REQ_D(*v, dudtBoundary);
    HTR_REQ_D(*v, dTdtBoundary);
    HTR_REQ_D(*v, velocity_old_NSCBC);
    HTR_REQ_D(*v, temperature_old_NSCBC);
  }
  if (iso) HTR_REQ_D(*v, temperature_profile);
  return HTR_OK;
}

int htr_rk3_step_bc_ws(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
                       const htr_bc_params *bc, htr_mixture_t m, void *workspace, size_t workspace_bytes,
                       double *dt_used, int *status_dev, htr_stream_t s) {
  int st;
  if ((st = check_common(v, m, inner))) return st;
  if ((st = check_step_fields(v, m))) return st;
  if (p == nullptr) return fail(HTR_ERR_ARGUMENT, "null step parameters%s");
  if (p->scheme < HTR_SCHEME_HYBRID || p->scheme > HTR_SCHEME_SKEW) return fail(HTR_ERR_ARGUMENT, "unknown scheme%s");
  if (p->implicitChemistry)
    return fail(HTR_ERR_UNSUPPORTED, "implicit chemistry is not supported by the boundary step%s");
  if ((st = check_bc_params(v, inner, fb, bc))) return st;
  const bool hybrid = p->scheme == HTR_SCHEME_HYBRID;
  if (hybrid) {
    for (int d = 0; d < 3; d++)
      if (!rect_ok(bc->sensor[d]) || !inside(bc->sensor[d], fb))
        return fail(HTR_ERR_ARGUMENT, "a sensor zone lies outside the grid%s");
    if ((st = check_field(v->DucrosSensor, 8, "DucrosSensor")) || (st = check_field(v->shockSensorX, 1, "shockSensorX")) ||
        (st = check_field(v->shockSensorY, 1, "shockSensorY")) || (st = check_field(v->shockSensorZ, 1, "shockSensorZ")))
      return st;
  }
  htr::StageWorkspace w;
  if (!htr::stage_workspace_carve(workspace, workspace_bytes, fb, neq_of(m), w))
    return fail(HTR_ERR_ARGUMENT, "workspace null or smaller than htr_rk3_workspace_bytes(fluid_bounds)%s");
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return fail(HTR_ERR_LAYOUT, "workspace not 256-byte aligned%s");
  const cudaStream_t cs = (cudaStream_t)s;
  double dt = p->deltaTime;
  if (p->cfl > 0.0) {
    if ((st = htr_CalculateMaxSpectralRadius(v, inner, m, w.scalars, s))) return st;
    double r = 0.0;
    if ((st = cuda_status(cudaMemcpyAsync(&r, w.scalars, sizeof(double), cudaMemcpyDeviceToHost, cs), "dt read"))) return st;
    if ((st = cuda_status(cudaStreamSynchronize(cs), "dt sync"))) return st;
    if (!(r > 0.0)) return fail(HTR_ERR_ARGUMENT, "non-positive spectral radius%s");
    dt = p->cfl / r;
  }
  if (!(dt > 0.0)) return fail(HTR_ERR_ARGUMENT, "non-positive time step%s");
  if (dt_used) *dt_used = dt;
  if (hybrid) {
    // UpdateShockSensors (src/prometeo_sensor.rg:96-125): Ducros over p_All,
    // the shock sensor of each direction over its faces zone
    if ((st = htr_UpdateDucrosSensor(v, fb, fb, p->vorticityScale, s))) return st;
    for (int d = 0; d < 3; d++)
      if ((st = cuda_status(htr::launch_shock_sensor(*v, bc->sensor[d], fb, nspec_of(m), 1 << d, cs), "shock sensor")))
        return st;
  }
  if ((st = htr_InitializeTemporaries(v, fb, m, s))) return st;
  htr::StageParams sp;
  sp.scheme = hybrid ? 0 : (p->scheme == HTR_SCHEME_SKEW ? 1 : 2);
  sp.kind = p->scheme == HTR_SCHEME_TENOA ? htr::kTENOA : (p->scheme == HTR_SCHEME_TENOLAD ? htr::kTENOLAD : htr::kTENO);
  sp.chemistry = p->explicitChemistry ? 1 : 0;
  sp.dt = dt;
  sp.active = active_dirs(fb);
  sp.boundary = 1;
  for (int k = 0; k < 6; k++) {
    const int t = bc->type[k];
    sp.bc[k] = t == HTR_BC_NSCBC_INFLOW ? htr::kBcInflow
             : t == HTR_BC_NSCBC_OUTFLOW ? htr::kBcOutflow
             : (t == HTR_BC_ISOTHERMAL_WALL || t == HTR_BC_ADIABATIC_WALL) ? htr::kBcWall : htr::kBcPeriodic;
    sp.Pbc[k] = bc->P[k];
    sp.plane[k] = bc->plane[k];
  }
  if ((st = cuda_status(cudaMemsetAsync(w.tcache, 0, sizeof(double) * 3 * ncells_of(fb), cs), "cache reset"))) return st;
  const int neq = neq_of(m), ns = nspec_of(m);
  return with_mix(m, [&](const auto &mix) -> int {
    cudaError_t e;
    for (int stage = 1; stage <= 3; stage++) {
      // NSCBC terms of the stage's state, left in Conserved_t of the planes
      for (int k = 0; k < 6; k++)
        if (sp.bc[k] == htr::kBcInflow || sp.bc[k] == htr::kBcOutflow)
          if ((e = htr::launch_init_rhs(*v, bc->plane[k], neq, 0, cs)) != cudaSuccess) return cuda_status(e, "plane rhs");
      for (int d = 0; d < 3; d++) {
        if (sp.bc[2 * d] != htr::kBcOutflow && sp.bc[2 * d + 1] != htr::kBcOutflow) continue;
        if ((e = htr::launch_max_mach(*v, inner, d, w.scalars + d, cs)) != cudaSuccess) return cuda_status(e, "max mach");
        for (int k = 2 * d; k < 2 * d + 2; k++)
          if (sp.bc[k] == htr::kBcOutflow &&
              (e = htr::launch_nscbc_outflow(*v, bc->plane[k], fb, mix, d, k % 2 == 0, 0.0, bc->LengthScale[k],
                                             bc->P[k], cs, w.scalars + d)) != cudaSuccess)
            return cuda_status(e, "nscbc outflow");
      }
      for (int k = 0; k < 6; k++)
        if (sp.bc[k] == htr::kBcInflow &&
            (e = htr::launch_nscbc_inflow(*v, bc->plane[k], mix, k / 2, k % 2 == 0, cs)) != cudaSuccess)
          return cuda_status(e, "nscbc inflow");
      sp.stage = stage;
      if ((e = htr::launch_stage(*v, fb, fb, mix, w, sp, status_dev, cs)) != cudaSuccess) return cuda_status(e, "stage");
      // wall ghosts from their first interior point, walls z, y, x
      for (int k : {4, 5, 2, 3, 0, 1}) {
        if (sp.bc[k] != htr::kBcWall) continue;
        const bool iso = bc->type[k] == HTR_BC_ISOTHERMAL_WALL;
        if ((e = htr::launch_wall_state(*v, bc->plane[k], ns, k, iso, cs)) != cudaSuccess ||
            (e = htr::launch_properties(*v, bc->plane[k], mix, cs)) != cudaSuccess ||
            (e = htr::launch_conserved(*v, bc->plane[k], mix, cs)) != cudaSuccess)
          return cuda_status(e, "wall");
      }
    }
    for (int k = 0; k < 6; k++)
      if (sp.bc[k] == htr::kBcInflow &&
          (e = htr::launch_nscbc_time_derivatives(*v, bc->plane[k], dt, cs)) != cudaSuccess)
        return cuda_status(e, "inflow time derivatives");
    return (int)HTR_OK;
  });
}

int htr_rk3_step_static(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
                        htr_mixture_t m, double *dt_used, int *status_dev, htr_stream_t s) {
  int st;
  if ((st = check_common(v, m, inner))) return st;
  if ((st = check_step_fields(v, m))) return st;
  for (int i = 0; i < 3; i++)
    if (inner.lo[i] != fb.lo[i] || inner.hi[i] != fb.hi[i])
      return fail(HTR_ERR_UNSUPPORTED, "the fused step needs a grid periodic in every direction (interior == bounds)%s");
  const size_t need = htr::stage_workspace_bytes(inner, neq_of(m));
  if (need > kStaticScratchBytes) return fail(HTR_ERR_UNSUPPORTED, "grid too large for the static scratch%s");
  void *scratch = nullptr;
  if ((st = static_scratch(&scratch))) return st;
  htr::StageWorkspace w;
  if (!htr::stage_workspace_carve(scratch, kStaticScratchBytes, inner, neq_of(m), w))
    return fail(HTR_ERR_ARGUMENT, "static scratch carve failed%s");
  return fused_step(v, inner, fb, p, m, w, dt_used, status_dev, s);
}

size_t htr_rk3_static_scratch_bytes(void) { return kStaticScratchBytes; }

int htr_rk3_stage_profile(const htr_fluid_view *v, htr_rect3 inner, htr_rect3 fb, const htr_step_params *p,
                          htr_mixture_t m, void *workspace, size_t workspace_bytes, float *ms_out,
                          htr_stream_t s) {
  int st;
  if (p == nullptr || ms_out == nullptr) return fail(HTR_ERR_ARGUMENT, "null argument%s");
  if ((st = check_common(v, m, inner))) return st;
  if ((st = check_step_fields(v, m))) return st;
  for (int i = 0; i < 3; i++)
    if (inner.lo[i] != fb.lo[i] || inner.hi[i] != fb.hi[i])
      return fail(HTR_ERR_UNSUPPORTED, "the fused step needs a grid periodic in every direction (interior == bounds)%s");
  htr::StageWorkspace w;
  if (!htr::stage_workspace_carve(workspace, workspace_bytes, inner, neq_of(m), w))
    return fail(HTR_ERR_ARGUMENT, "workspace null or smaller than htr_rk3_workspace_bytes%s");
  if (!(p->deltaTime > 0.0)) return fail(HTR_ERR_ARGUMENT, "non-positive time step%s");
  htr::StageParams sp;
  sp.scheme = p->scheme == HTR_SCHEME_HYBRID ? 0 : (p->scheme == HTR_SCHEME_SKEW ? 1 : 2);
  sp.kind = p->scheme == HTR_SCHEME_TENOA ? htr::kTENOA : (p->scheme == HTR_SCHEME_TENOLAD ? htr::kTENOLAD : htr::kTENO);
  sp.chemistry = p->explicitChemistry ? 1 : 0;
  sp.dt = p->deltaTime;
  sp.stage = 1;
  sp.active = active_dirs(inner);
  // the profiled stage starts from the current state (Conserved_old =
  // Conserved), so repeated profiles advance the state by forward-Euler
  // stages instead of iterating stage 1 from an old step start
  if (int st = cuda_status(htr::launch_copy_conserved(*v, fb, neq_of(m), (cudaStream_t)s), "profile start")) return st;
  if (int st = cuda_status(cudaMemsetAsync(w.tcache, 0, sizeof(double) * 3 * ncells_of(inner), (cudaStream_t)s),
                           "cache reset"))
    return st;
  cudaEvent_t ev[htr::kStageKernels + 1];
  int made = 0;
  cudaError_t e = cudaSuccess;
  for (; made <= htr::kStageKernels && e == cudaSuccess; made++) e = cudaEventCreate(&ev[made]);
  if (e == cudaSuccess)
    st = with_mix(m, [&](const auto &mix) {
      return cuda_status(htr::launch_stage(*v, inner, fb, mix, w, sp, nullptr, (cudaStream_t)s, ev), "stage");
    });
  else
    st = cuda_status(e, "event create");
  if (st == HTR_OK) st = cuda_status(cudaEventSynchronize(ev[htr::kStageKernels]), "stage sync");
  for (int k = 0; st == HTR_OK && k < htr::kStageKernels; k++)
    st = cuda_status(cudaEventElapsedTime(&ms_out[k], ev[k], ev[k + 1]), "event time");
  for (int k = 0; k < made; k++) cudaEventDestroy(ev[k]);
  return st;
}

}  // extern "C"
