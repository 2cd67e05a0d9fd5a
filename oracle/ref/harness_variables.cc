// Reference-build harness: per-cell state refresh tasks.
// Compiles the reference's src/prometeo_variables.cc unmodified (test infrastructure only).
#include "prometeo_variables.cc"

#include "ref_common.h"

using namespace htr_ref;

template <class Task>
static int run(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  ArgsBuf<typename Task::Args> a(mix);
  std::vector<Future> fut;
  Runtime rt;
  Task::cpu_base_impl(a.get(), regions(v, &exec, 2), fut, nullptr, &rt);
  return HTR_OK;
}

extern "C" int htr_UpdatePropertiesFromPrimitive(const htr_fluid_view *v, htr_rect3 m,
                                                 htr_mixture_t mix, htr_stream_t) {
  return run<UpdatePropertiesFromPrimitiveTask>(v, m, mix);
}
extern "C" int htr_UpdateConservedFromPrimitive(const htr_fluid_view *v, htr_rect3 m,
                                                htr_mixture_t mix, htr_stream_t) {
  return run<UpdateConservedFromPrimitiveTask>(v, m, mix);
}
extern "C" int htr_UpdatePrimitiveFromConserved(const htr_fluid_view *v, htr_rect3 m,
                                                htr_mixture_t mix, htr_stream_t) {
  return run<UpdatePrimitiveFromConservedTask>(v, m, mix);
}
