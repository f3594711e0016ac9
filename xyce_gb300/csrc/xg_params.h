// xg_params.h — host parameter processing for the device model tables.
#pragma once
#include "xg_internal.h"

namespace xg {

struct Mos1Instance {
  Mos1Model model;  // model-level part (shared by instances with equal values)
  double beta;      // tTransconductance * W / Leff
  double tVbi;
  bool valid;
};

DiodeModel diode_model(const double *params);
Mos1Instance mos1_instance(const double *params);

}  // namespace xg
