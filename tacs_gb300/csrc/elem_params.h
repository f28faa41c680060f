// Element constants and KS statistics shared by the kernels, the host
// runtime and the host-compiled element checks (no CUDA headers).
#pragma once

namespace tg {

// Material and element constants shared by every element of one assembler.
struct ElemParams {
  int elem_type;  // TG_ELEM_MITC4 / TG_ELEM_HEX8
  double rho, E, nu, ys;
  int transform;       // shells: 0 natural, 1 reference axis
  double ref_axis[3];  // normalised reference axis
};

// KS aggregate statistics: max over the points and sum of w detXd
// exp(weight (f - max)) (TACSKSFailure, src/functions/TACSKSFailure.cpp).
struct KsStats {
  double max, sum, weight;
};

}  // namespace tg
