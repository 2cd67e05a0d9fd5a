// Reference-build harness: chemistry tasks.
// Compiles the reference's src/prometeo_chem.cc unmodified (test infrastructure only).
#include "prometeo_chem.cc"

#include "ref_common.h"

using namespace htr_ref;

extern "C" int htr_AddChemistrySources(const htr_fluid_view *v, htr_rect3 myf, htr_mixture_t mix,
                                       htr_stream_t) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  ArgsBuf<AddChemistrySourcesTask::Args> a(mix);
  std::vector<Future> fut;
  Runtime rt;
  AddChemistrySourcesTask::cpu_base_impl(a.get(), regions(v, &exec, 2), fut, nullptr, &rt);
  return HTR_OK;
}

extern "C" int htr_UpdateChemistry(const htr_fluid_view *v, htr_rect3 myf, double dt,
                                   htr_mixture_t mix, int *status, htr_stream_t) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  ArgsBuf<UpdateChemistryTask::Args> a(mix);
  a.get().Integrator_deltaTime = dt;
  std::vector<Future> fut{Future(dt)};
  Runtime rt;
  UpdateChemistryTask::cpu_base_impl(a.get(), regions(v, &exec, 2), fut, nullptr, &rt);
  if (status) *status = HTR_OK;
  return HTR_OK;
}
