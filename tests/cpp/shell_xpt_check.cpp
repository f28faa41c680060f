// CPU check of the shell node-coordinate derivative
// (tacs_gb300/csrc/shell_xpt.cuh): the same device functions compiled for
// the host, the reverse sweep against the dual-number forward derivative of
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
#include "shell_common.cuh"
#include "shell_xpt.cuh"
}  // namespace
}  // namespace tg

extern "C" {

// p: E, nu, ys, transform, ref_axis[3]; ks: max, sum, weight;
// s: coef, scale, lambda.  flags: bit 0 psi present, bit 1 pressure.
// fwd[12]: forward derivative per coordinate; rev[12]: the reverse sweep.
void sx_derivatives(const double *p, const double *X, const double *u,
                    const double *w, double t, const double *pres, int flags,
                    int func, const double *ks, const double *s, double *fwd,
                    double *rev) {
  tg::ElemParams ep;
  ep.elem_type = TG_ELEM_MITC4;
  ep.rho = 2700.0;
  ep.E = p[0];
  ep.nu = p[1];
  ep.ys = p[2];
  ep.transform = (int)p[3];
  for (int i = 0; i < 3; i++) ep.ref_axis[i] = p[4 + i];
  tg::ShellXptData dt;
  for (int i = 0; i < 12; i++) dt.X[i] = X[i];
  for (int i = 0; i < 24; i++) {
    dt.u[i] = u[i];
    dt.w[i] = w[i];
  }
  dt.t = t;
  for (int k = 0; k < 4; k++) dt.pres[k] = pres[k];
  dt.has_psi = (flags & 1) != 0;
  dt.has_pres = (flags & 2) != 0;
  const tg::KsStats kk{ks[0], ks[1], ks[2]};
  for (int kc = 0; kc < 12; kc++)
    fwd[kc] = tg::shell_xpt_forward(ep, dt, kc, func, kk, s[0], s[1], s[2]);
  for (int i = 0; i < 12; i++) rev[i] = 0.0;
  tg::shell_xpt_reverse(ep, dt, func, kk, s[0], s[1], s[2], rev);
}

}  // extern "C"

extern "C" {

// The whole-mesh sum of the element derivatives, as the kernels scatter
// it: dfdX[3 nnodes] += d/dX (scale psi^T R + coef f) with the element
// pressures pres[4 nelem] (nullptr: none) and the state / adjoint with 6
// entries per node (psi nullptr: no adjoint term).  reverse: the reverse
// sweep, else the dual form per coordinate.
void sx_mesh(int nelem, const int *conn, const double *xpts,
             const double *thick, const double *pres, const double *vars,
             const double *psi, const double *p, int func, const double *ks,
             const double *s, int reverse, double *dfdX) {
  tg::ElemParams ep;
  ep.elem_type = TG_ELEM_MITC4;
  ep.rho = 2700.0;
  ep.E = p[0];
  ep.nu = p[1];
  ep.ys = p[2];
  ep.transform = (int)p[3];
  for (int i = 0; i < 3; i++) ep.ref_axis[i] = p[4 + i];
  const tg::KsStats kk{ks[0], ks[1], ks[2]};
  for (int e = 0; e < nelem; e++) {
    tg::ShellXptData dt;
    const int *nd = conn + 4 * e;
    for (int i = 0; i < 12; i++) dt.X[i] = xpts[3 * nd[i / 3] + i % 3];
    for (int i = 0; i < 24; i++) {
      dt.u[i] = vars[6 * nd[i / 6] + i % 6];
      dt.w[i] = psi ? psi[6 * nd[i / 6] + i % 6] : 0.0;
    }
    dt.t = thick[e];
    dt.has_psi = psi != nullptr;
    dt.has_pres = pres != nullptr;
    for (int k = 0; k < 4; k++) dt.pres[k] = pres ? pres[4 * e + k] : 0.0;
    double dX[12] = {0.0};
    if (reverse) {
      tg::shell_xpt_reverse(ep, dt, func, kk, s[0], s[1], s[2], dX);
    } else {
      for (int kc = 0; kc < 12; kc++)
        dX[kc] = tg::shell_xpt_forward(ep, dt, kc, func, kk, s[0], s[1], s[2]);
    }
    for (int i = 0; i < 12; i++) dfdX[3 * nd[i / 3] + i % 3] += dX[i];
  }
}

}  // extern "C"
