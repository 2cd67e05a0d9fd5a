// CPU oracle port: the mixture handle shared by the port's translation units.
// TEST INFRASTRUCTURE ONLY.
#ifndef HTR_ORACLE_PORT_PORT_HPP
#define HTR_ORACLE_PORT_PORT_HPP

#include "htr_rhs.h"
#include "mixtures.hpp"

struct htr_mixture_s {
  int eos;
  oport::ConstProp cp;
  oport::Air air;
};

#endif
