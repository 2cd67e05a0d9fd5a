// Reference-build harness: grid metrics.
// Compiles the reference's src/prometeo_metric.cc unmodified (test infrastructure only).
#include "prometeo_metric.cc"

#include "ref_common.h"

using namespace htr_ref;

namespace {
std::vector<PhysicalRegion> metric_regions(const htr_fluid_view *v, htr_field cc, const Rect<3> *rect) {
  std::vector<PhysicalRegion> r = regions(v, rect, 2);
  for (auto &reg : r) bind(reg, FID_centerCoordinates, cc);
  return r;
}

bool bad(const htr_fluid_view *v, htr_field cc) { return v == nullptr || cc.base == nullptr; }

template <direction dir> int correct(const htr_fluid_view *v, htr_field cc, htr_rect3 myf) {
  if (bad(v, cc)) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  typename CorrectGhostMetricTask<dir>::Args a;
  std::memset(&a, 0, sizeof(a));
  std::vector<Future> fut;
  Runtime rt;
  CorrectGhostMetricTask<dir>::cpu_base_impl(a, metric_regions(v, cc, &exec), fut, nullptr, &rt);
  return HTR_OK;
}
}  // namespace

extern "C" int htr_InitializeMetric(const htr_fluid_view *v, htr_field cc, htr_rect3 myf, htr_rect3 fb,
                                    const double width[3], htr_stream_t) {
  if (bad(v, cc) || width == nullptr) return HTR_ERR_ARGUMENT;
  const Rect<3> exec = to_rect(myf);
  InitializeMetricTask::Args a;
  std::memset(&a, 0, sizeof(a));
  a.Fluid_bounds = to_rect(fb);
  // a box whose extents are the widths (only the extents are read)
  a.bBox.v1[0] = width[0];
  a.bBox.v3[1] = width[1];
  a.bBox.v4[2] = width[2];
  std::vector<Future> fut;
  Runtime rt;
  InitializeMetricTask::cpu_base_impl(a, metric_regions(v, cc, &exec), fut, nullptr, &rt);
  return HTR_OK;
}
extern "C" int htr_CorrectGhostMetricX(const htr_fluid_view *v, htr_field cc, htr_rect3 m, htr_stream_t) {
  return correct<Xdir>(v, cc, m);
}
extern "C" int htr_CorrectGhostMetricY(const htr_fluid_view *v, htr_field cc, htr_rect3 m, htr_stream_t) {
  return correct<Ydir>(v, cc, m);
}
extern "C" int htr_CorrectGhostMetricZ(const htr_fluid_view *v, htr_field cc, htr_rect3 m, htr_stream_t) {
  return correct<Zdir>(v, cc, m);
}
