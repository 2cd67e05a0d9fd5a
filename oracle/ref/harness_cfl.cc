// Reference-build harness: spectral-radius task.
// Compiles the reference's src/prometeo_cfl.cc unmodified (test infrastructure only).
#include "prometeo_cfl.cc"

#include "ref_common.h"

using namespace htr_ref;

extern "C" int htr_CalculateMaxSpectralRadius(const htr_fluid_view *v, htr_rect3 myf,
                                              htr_mixture_t mix, double *result, htr_stream_t) {
  if (!valid(v, mix, HTR_REF_EOS_ID) || result == nullptr) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  ArgsBuf<CalculateMaxSpectralRadiusTask::Args> a(mix);
  std::vector<Future> fut;
  Runtime rt;
  *result = CalculateMaxSpectralRadiusTask::cpu_base_impl(a.get(), regions(v, &exec, 1), fut,
                                                          nullptr, &rt);
  return HTR_OK;
}
