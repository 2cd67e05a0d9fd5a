// Reference-build harness: Euler and diffusion flux tasks.
// Compiles the reference's src/prometeo_rhs.cc unmodified (test infrastructure only).
#include "prometeo_rhs.cc"

#include "ref_common.h"

using namespace htr_ref;

namespace {

template <class Task>
int run_flux(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fb, const double rk[2], double dt,
             htr_mixture_t mix) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  ArgsBuf<typename Task::Args> a(mix);
  a.get().Fluid_bounds = to_rect(fb);
  a.get().RK_coeffs[0] = rk ? rk[0] : 0.0;
  a.get().RK_coeffs[1] = rk ? rk[1] : 1.0;
  a.get().deltaTime = dt;
  std::vector<Future> fut{Future(dt)};
  Runtime rt;
  Task::cpu_base_impl(a.get(), regions(v, &exec, 4), fut, nullptr, &rt);
  return HTR_OK;
}

template <class Task>
int run_skew(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fb, htr_mixture_t mix) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  ArgsBuf<typename Task::Args> a(mix);
  a.get().Fluid_bounds = to_rect(fb);
  std::vector<Future> fut;
  Runtime rt;
  Task::cpu_base_impl(a.get(), regions(v, &exec, 4), fut, nullptr, &rt);
  return HTR_OK;
}

template <class Task>
int run_diff(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fb, htr_mixture_t mix) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  ArgsBuf<typename Task::Args> a(mix);
  a.get().Fluid_bounds = to_rect(fb);
  std::vector<Future> fut;
  Runtime rt;
  Task::cpu_base_impl(a.get(), regions(v, &exec, 5), fut, nullptr, &rt);
  return HTR_OK;
}

}  // namespace

#define HTR_REF_FLUX(NAME, TASK)                                                              \
  extern "C" int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, const double rk[2], \
                      double dt, htr_mixture_t mix, htr_stream_t) {                           \
    return run_flux<TASK>(v, m, b, rk, dt, mix);                                               \
  }

HTR_REF_FLUX(htr_UpdateUsingHybridEulerFluxX, UpdateUsingHybridEulerFluxTask<Xdir>)
HTR_REF_FLUX(htr_UpdateUsingHybridEulerFluxY, UpdateUsingHybridEulerFluxTask<Ydir>)
HTR_REF_FLUX(htr_UpdateUsingHybridEulerFluxZ, UpdateUsingHybridEulerFluxTask<Zdir>)
typedef UpdateUsingTENOEulerFluxTask<Xdir, TENO_Op<>> TenoX;
typedef UpdateUsingTENOEulerFluxTask<Ydir, TENO_Op<>> TenoY;
typedef UpdateUsingTENOEulerFluxTask<Zdir, TENO_Op<>> TenoZ;
typedef UpdateUsingTENOEulerFluxTask<Xdir, TENOA_Op<>> TenoAX;
typedef UpdateUsingTENOEulerFluxTask<Ydir, TENOA_Op<>> TenoAY;
typedef UpdateUsingTENOEulerFluxTask<Zdir, TENOA_Op<>> TenoAZ;
typedef UpdateUsingTENOEulerFluxTask<Xdir, TENOLAD_Op<>> TenoLadX;
typedef UpdateUsingTENOEulerFluxTask<Ydir, TENOLAD_Op<>> TenoLadY;
typedef UpdateUsingTENOEulerFluxTask<Zdir, TENOLAD_Op<>> TenoLadZ;
HTR_REF_FLUX(htr_UpdateUsingTENOEulerFluxX, TenoX)
HTR_REF_FLUX(htr_UpdateUsingTENOEulerFluxY, TenoY)
HTR_REF_FLUX(htr_UpdateUsingTENOEulerFluxZ, TenoZ)
HTR_REF_FLUX(htr_UpdateUsingTENOAEulerFluxX, TenoAX)
HTR_REF_FLUX(htr_UpdateUsingTENOAEulerFluxY, TenoAY)
HTR_REF_FLUX(htr_UpdateUsingTENOAEulerFluxZ, TenoAZ)
HTR_REF_FLUX(htr_UpdateUsingTENOLADEulerFluxX, TenoLadX)
HTR_REF_FLUX(htr_UpdateUsingTENOLADEulerFluxY, TenoLadY)
HTR_REF_FLUX(htr_UpdateUsingTENOLADEulerFluxZ, TenoLadZ)

#define HTR_REF_SKEW(NAME, DIR)                                                              \
  extern "C" int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t mix, \
                      htr_stream_t) {                                                        \
    return run_skew<UpdateUsingSkewSymmetricEulerFluxTask<DIR>>(v, m, b, mix);              \
  }
HTR_REF_SKEW(htr_UpdateUsingSkewSymmetricEulerFluxX, Xdir)
HTR_REF_SKEW(htr_UpdateUsingSkewSymmetricEulerFluxY, Ydir)
HTR_REF_SKEW(htr_UpdateUsingSkewSymmetricEulerFluxZ, Zdir)

#define HTR_REF_DIFF(NAME, DIR)                                                              \
  extern "C" int NAME(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b, htr_mixture_t mix, \
                      htr_stream_t) {                                                        \
    return run_diff<UpdateUsingDiffusionFluxTask<DIR>>(v, m, b, mix);                       \
  }
HTR_REF_DIFF(htr_UpdateUsingDiffusionFluxX, Xdir)
HTR_REF_DIFF(htr_UpdateUsingDiffusionFluxY, Ydir)
HTR_REF_DIFF(htr_UpdateUsingDiffusionFluxZ, Zdir)

// NSCBC boundary terms: the BC region (the boundary plane) is the index
// space every region of the task is built on (the tasks iterate over it).
namespace {
template <class Task> int run_inflow(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t mix) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(bc);
  ArgsBuf<typename Task::Args> a(mix);
  std::vector<Future> fut;
  Runtime rt;
  Task::cpu_base_impl(a.get(), regions(v, &exec, 3), fut, nullptr, &rt);
  return HTR_OK;
}
template <class Task>
int run_outflow(const htr_fluid_view *v, htr_rect3 bc, htr_rect3 fb, htr_mixture_t mix, double MaxMach,
                double LengthScale, double PInf) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(bc);
  ArgsBuf<typename Task::Args> a(mix);
  a.get().Fluid_bounds = to_rect(fb);
  a.get().MaxMach = MaxMach;
  a.get().LengthScale = LengthScale;
  a.get().PInf = PInf;
  std::vector<Future> fut{Future(MaxMach)};
  Runtime rt;
  Task::cpu_base_impl(a.get(), regions(v, &exec, 4), fut, nullptr, &rt);
  return HTR_OK;
}
}  // namespace

#define HTR_REF_NSCBC(SIDE, DIR, PM)                                                                      \
  extern "C" int htr_UpdateUsingFluxNSCBCInflow##SIDE(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, \
                                                      htr_stream_t) {                                     \
    return run_inflow<UpdateUsingFluxNSCBCInflow##PM##SideTask<DIR>>(v, bc, m);                          \
  }                                                                                                       \
  extern "C" int htr_UpdateUsingFluxNSCBCOutflow##SIDE(const htr_fluid_view *v, htr_rect3 bc, htr_rect3 fb, \
                                                       htr_mixture_t m, double MaxMach, double LS, double PInf, \
                                                       htr_stream_t) {                                     \
    return run_outflow<UpdateUsingFluxNSCBCOutflow##PM##SideTask<DIR>>(v, bc, fb, m, MaxMach, LS, PInf);  \
  }
HTR_REF_NSCBC(XNeg, Xdir, Minus)
HTR_REF_NSCBC(XPos, Xdir, Plus)
HTR_REF_NSCBC(YNeg, Ydir, Minus)
HTR_REF_NSCBC(YPos, Ydir, Plus)
HTR_REF_NSCBC(ZNeg, Zdir, Minus)
HTR_REF_NSCBC(ZPos, Zdir, Plus)
#undef HTR_REF_NSCBC
