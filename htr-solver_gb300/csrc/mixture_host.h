// Host-side derivation of the device mixture constants.
#pragma once

#include "htr_rhs.h"
#include "mixture.cuh"

namespace htr {
// Fill the device-side constants from a reference-compatible mixture struct;
// false if the struct is not usable.
bool derive(const htr_constpropmix_t &s, ConstPropDev &d);
bool derive(const htr_airmix_t &s, AirDev &d);
}  // namespace htr
