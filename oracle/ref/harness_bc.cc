// Reference-build harness: boundary-condition state updates.
// Compiles the reference's src/prometeo_bc.cc unmodified (test infrastructure only).
#include "prometeo_bc.cc"

#include "ref_common.h"

using namespace htr_ref;

namespace {
template <class Task> int run_bc(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t mix, double Pbc, bool pbc) {
  if (!valid(v, mix, HTR_REF_EOS_ID)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(bc);
  ArgsBuf<typename Task::Args> a(mix);
  if constexpr (std::is_same_v<Task, SetNSCBC_InflowBCTask<Xdir>> || std::is_same_v<Task, SetNSCBC_InflowBCTask<Ydir>> ||
                std::is_same_v<Task, SetNSCBC_InflowBCTask<Zdir>>)
    a.get().Pbc = Pbc;
  (void)pbc;
  std::vector<Future> fut;
  Runtime rt;
  Task::cpu_base_impl(a.get(), regions(v, &exec, 2), fut, nullptr, &rt);
  return HTR_OK;
}
}  // namespace

extern "C" int htr_SetNSCBC_InflowBCX(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t) {
  return run_bc<SetNSCBC_InflowBCTask<Xdir>>(v, bc, m, Pbc, true);
}
extern "C" int htr_SetNSCBC_InflowBCY(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t) {
  return run_bc<SetNSCBC_InflowBCTask<Ydir>>(v, bc, m, Pbc, true);
}
extern "C" int htr_SetNSCBC_InflowBCZ(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, double Pbc, htr_stream_t) {
  return run_bc<SetNSCBC_InflowBCTask<Zdir>>(v, bc, m, Pbc, true);
}
extern "C" int htr_SetNSCBC_OutflowBC(const htr_fluid_view *v, htr_rect3 bc, htr_mixture_t m, int *status, htr_stream_t) {
  if (status) *status = 0;
  return run_bc<SetNSCBC_OutflowBCTask>(v, bc, m, 0.0, false);
}
