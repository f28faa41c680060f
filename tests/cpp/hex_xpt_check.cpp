// CPU check of the hex8 node-coordinate derivative
// (tacs_gb300/csrc/hex_xpt.cuh): the same device functions compiled for the
// host, the reverse sweep against the dual-number forward derivative of
// every coordinate.  Built by tests/test_xpt_sens.py with g++ and called
// through ctypes; test infrastructure only.
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__
#include <cmath>

#include "../../include/tacs_gb300.h"
#include "dual.cuh"
#include "elem_params.h"

namespace tg {
namespace {
#include "hex_common.cuh"
#include "hex_xpt.cuh"
}  // namespace
}  // namespace tg

extern "C" {

// p: E, nu, ys; ks: max, sum, weight; s: coef, scale, lambda; faces /
// tvals: ntrac face tractions.  has_psi: the adjoint term is present.
// fwd[24]: forward derivative per coordinate; rev[24]: the reverse sweep.
void hx_derivatives(const double *p, const double *X, const double *u,
                    const double *w, double t, int has_psi, int ntrac,
                    const int *faces, const double *tvals, int func,
                    const double *ks, const double *s, double *fwd,
                    double *rev) {
  tg::ElemParams ep;
  ep.elem_type = TG_ELEM_HEX8;
  ep.rho = 2700.0;
  ep.E = p[0];
  ep.nu = p[1];
  ep.ys = p[2];
  ep.transform = 0;
  ep.ref_axis[0] = 1.0;
  ep.ref_axis[1] = ep.ref_axis[2] = 0.0;
  tg::HexXptData dt;
  for (int i = 0; i < 24; i++) {
    dt.X[i] = X[i];
    dt.u[i] = u[i];
    dt.w[i] = w[i];
  }
  dt.t = t;
  dt.has_psi = has_psi != 0;
  dt.ntrac = ntrac;
  dt.trac_face = faces;
  dt.trac_val = tvals;
  const tg::KsStats kk{ks[0], ks[1], ks[2]};
  for (int kc = 0; kc < 24; kc++)
    fwd[kc] = tg::hex_xpt_forward(ep, dt, kc, func, kk, s[0], s[1], s[2]);
  for (int i = 0; i < 24; i++) rev[i] = 0.0;
  tg::hex_xpt_reverse(ep, dt, func, kk, s[0], s[1], s[2], rev);
}

}  // extern "C"

extern "C" {

// The whole-mesh sum of the element derivatives (see sx_mesh): face
// tractions as a CSR list per element (trac_ptr[nelem + 1], nullptr: none),
// 3 entries per node for the state and adjoint.
void hx_mesh(int nelem, const int *conn, const double *xpts,
             const double *thick, const int *trac_ptr, const int *trac_face,
             const double *trac_val, const double *vars, const double *psi,
             const double *p, int func, const double *ks, const double *s,
             int reverse, double *dfdX) {
  tg::ElemParams ep;
  ep.elem_type = TG_ELEM_HEX8;
  ep.rho = 2700.0;
  ep.E = p[0];
  ep.nu = p[1];
  ep.ys = p[2];
  ep.transform = 0;
  ep.ref_axis[0] = 1.0;
  ep.ref_axis[1] = ep.ref_axis[2] = 0.0;
  const tg::KsStats kk{ks[0], ks[1], ks[2]};
  for (int e = 0; e < nelem; e++) {
    tg::HexXptData dt;
    const int *nd = conn + 8 * e;
    for (int i = 0; i < 24; i++) {
      const int g = 3 * nd[i / 3] + i % 3;
      dt.X[i] = xpts[g];
      dt.u[i] = vars[g];
      dt.w[i] = psi ? psi[g] : 0.0;
    }
    dt.t = thick[e];
    dt.has_psi = psi != nullptr;
    dt.ntrac = trac_ptr ? trac_ptr[e + 1] - trac_ptr[e] : 0;
    dt.trac_face = trac_ptr ? trac_face + trac_ptr[e] : nullptr;
    dt.trac_val = trac_ptr ? trac_val + 3 * trac_ptr[e] : nullptr;
    double dX[24] = {0.0};
    if (reverse) {
      tg::hex_xpt_reverse(ep, dt, func, kk, s[0], s[1], s[2], dX);
    } else {
      for (int kc = 0; kc < 24; kc++)
        dX[kc] = tg::hex_xpt_forward(ep, dt, kc, func, kk, s[0], s[1], s[2]);
    }
    for (int i = 0; i < 24; i++) dfdX[3 * nd[i / 3] + i % 3] += dX[i];
  }
}

}  // extern "C"
