// Reference-build harness: shock-sensor tasks.
// Compiles the reference's src/prometeo_sensor.cc unmodified (test infrastructure only).
#include "prometeo_sensor.cc"

#include "ref_common.h"

using namespace htr_ref;

extern "C" int htr_UpdateDucrosSensor(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fb,
                                      double vorticityScale, htr_stream_t) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  UpdateDucrosSensorTask::Args a;
  std::memset(&a, 0, sizeof(a));
  a.Fluid_bounds = to_rect(fb);
  a.vorticityScale = vorticityScale;
  std::vector<Future> fut;
  Runtime rt;
  UpdateDucrosSensorTask::cpu_base_impl(a, regions(v, &exec, 3), fut, nullptr, &rt);
  return HTR_OK;
}

template <direction dir>
static int shock(const htr_fluid_view *v, htr_rect3 myf, htr_rect3 fb) {
  if (v == nullptr) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  typename UpdateShockSensorTask<dir>::Args a;
  std::memset(&a, 0, sizeof(a));
  a.Fluid_bounds = to_rect(fb);
  std::vector<Future> fut;
  Runtime rt;
  UpdateShockSensorTask<dir>::cpu_base_impl(a, regions(v, &exec, 3), fut, nullptr, &rt);
  return HTR_OK;
}

extern "C" int htr_UpdateShockSensorX(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b,
                                      htr_mixture_t, htr_stream_t) { return shock<Xdir>(v, m, b); }
extern "C" int htr_UpdateShockSensorY(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b,
                                      htr_mixture_t, htr_stream_t) { return shock<Ydir>(v, m, b); }
extern "C" int htr_UpdateShockSensorZ(const htr_fluid_view *v, htr_rect3 m, htr_rect3 b,
                                      htr_mixture_t, htr_stream_t) { return shock<Zdir>(v, m, b); }
