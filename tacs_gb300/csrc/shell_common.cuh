// Device helpers of the MITC4 shell kernels (TACSQuad4Shell kinematics,
// TACSIsoShellConstitutive, point quantities).  Included by the shell
// kernel translation units inside namespace tg::<anonymous>.  The helpers
// that depend on the node coordinates are templates over the scalar type:
// double for assembly and the point quantities, ad::Dual for the
// node-coordinate sensitivities.
#pragma once

#include "elem_math.cuh"

template <class RA, class RB, class RC>
__device__ __forceinline__ void mm3(const RA *A, const RB *B, RC *C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] +
                     A[3 * i + 2] * B[6 + j];
}
template <class RA, class RB, class RC>
__device__ __forceinline__ void mmT3(const RA *A, const RB *B, RC *C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[3 * j] + A[3 * i + 1] * B[3 * j + 1] +
                     A[3 * i + 2] * B[3 * j + 2];
}
// TACSShellQuadBasis<2> shape functions
__device__ __forceinline__ void shape2(double xi, double eta, double *N,
                                       double *Na, double *Nb) {
  double na0 = 0.5 * (1.0 - xi), na1 = 0.5 * (1.0 + xi);
  double nb0 = 0.5 * (1.0 - eta), nb1 = 0.5 * (1.0 + eta);
  N[0] = na0 * nb0; N[1] = na1 * nb0; N[2] = na0 * nb1; N[3] = na1 * nb1;
  Na[0] = -0.5 * nb0; Na[1] = 0.5 * nb0; Na[2] = -0.5 * nb1; Na[3] = 0.5 * nb1;
  Nb[0] = na0 * -0.5; Nb[1] = na1 * -0.5; Nb[2] = na0 * 0.5; Nb[3] = na1 * 0.5;
}
template <class R>
__device__ __forceinline__ void grad3(const double *Na, const double *Nb,
                                      const R *X, R *Xxi) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    R a = 0.0, b = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++) {
      a += Na[m] * X[3 * m + k];
      b += Nb[m] * X[3 * m + k];
    }
    Xxi[2 * k] = a;
    Xxi[2 * k + 1] = b;
  }
}
template <class R>
__device__ __forceinline__ void interp3(const double *N, const R *X, R *o) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    R a = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++) a += N[m] * X[3 * m + k];
    o[k] = a;
  }
}
template <class R>
__device__ __forceinline__ void frame(const R *Xxi, const R *n, R *Xd) {
  Xd[0] = Xxi[0]; Xd[1] = Xxi[1]; Xd[2] = n[0];
  Xd[3] = Xxi[2]; Xd[4] = Xxi[3]; Xd[5] = n[1];
  Xd[6] = Xxi[4]; Xd[7] = Xxi[5]; Xd[8] = n[2];
}
// TACSShellNaturalTransform / TACSShellRefAxisTransform::computeTransform
// (src/elements/shell/TACSShellElementTransform.h:24-93, 95-160), including
// the natural transform's three-fold subtraction of d*n[0] from t1[0].
template <class R>
__device__ void shell_transform(const ElemParams &ep, const R *Xxi,
                                const R *n0, R *T) {
  R n[3] = {n0[0], n0[1], n0[2]};
  R inv = 1.0 / sqrt(dot3(n, n));
  n[0] *= inv; n[1] *= inv; n[2] *= inv;
  R t1[3];
  if (ep.transform == 0) {
    t1[0] = Xxi[0]; t1[1] = Xxi[2]; t1[2] = Xxi[4];
    R d = dot3(n, t1);
    t1[0] = t1[0] - d * n[0];
    t1[0] = t1[0] - d * n[0];
    t1[0] = t1[0] - d * n[0];
  } else {
    R an = dot3(ep.ref_axis, n);
    t1[0] = ep.ref_axis[0] - an * n[0];
    t1[1] = ep.ref_axis[1] - an * n[1];
    t1[2] = ep.ref_axis[2] - an * n[2];
  }
  inv = 1.0 / sqrt(dot3(t1, t1));
  t1[0] *= inv; t1[1] *= inv; t1[2] *= inv;
  R t2[3];
  cross3(n, t1, t2);
  T[0] = t1[0]; T[3] = t1[1]; T[6] = t1[2];
  T[1] = t2[0]; T[4] = t2[1]; T[7] = t2[2];
  T[2] = n[0];  T[5] = n[1];  T[8] = n[2];
}
// director map d = q x fn: entry (i, b) of the 3x3 map for node m
template <class R>
__device__ __forceinline__ R dmap(const R *f, int i, int b) {
  // rows: [0, f2, -f1], [-f2, 0, f0], [f1, -f0, 0]
  if (i == b) return 0.0;
  if (i == 0) return b == 1 ? f[2] : -f[1];
  if (i == 1) return b == 0 ? -f[2] : f[0];
  return b == 0 ? f[1] : -f[0];
}

// Tying points of TACSShellQuadBasis<2> (TACSShellElementQuadBasis.h:500-
// 540) and the symmetric-tensor position of each tying field.
__device__ __constant__ double c_ty_pt[9][2] = {
    {0, -1}, {0, 1}, {-1, 0}, {1, 0}, {0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}};
__device__ __constant__ int c_ty_field[9] = {0, 0, 1, 1, 2, 3, 3, 4, 4};
__device__ __constant__ int c_ty_ij[5][2] = {
    {0, 0}, {1, 1}, {0, 1}, {1, 2}, {0, 2}};
// strain rows fed by the tying strain: e0, e1, e2, e6, e7
__device__ __constant__ int c_erc[5][2] = {
    {0, 0}, {1, 1}, {0, 1}, {1, 2}, {0, 2}};
__device__ __constant__ double c_efac[5] = {1.0, 1.0, 2.0, 2.0, 2.0};
__device__ __constant__ int c_ri_of_row[9] = {0, 1, 2, -1, -1, -1, 3, 4, -1};

// TACSIsoShellConstitutive tangent (tOffset = 0, kcorr = 5/6, drilling
// regularisation 0.1; TACSIsoShellConstitutive.cpp:181-217)
struct ShellStiff {
  double A[6], D[6], As[3], drill;
};
__device__ __forceinline__ ShellStiff shell_stiff(const ElemParams &ep,
                                                  double t) {
  ShellStiff c;
  double Dm = ep.E / (1.0 - ep.nu * ep.nu);
  double G = 0.5 * ep.E / (1.0 + ep.nu);
  double A0[6] = {Dm, ep.nu * Dm, 0.0, Dm, 0.0, G};
  double I = t * t * t / 12.0;
#pragma unroll
  for (int i = 0; i < 6; i++) {
    c.D[i] = I * A0[i];
    c.A[i] = A0[i] * t;
  }
  c.As[0] = c.As[2] = (5.0 / 6.0) * c.A[5];
  c.As[1] = 0.0;
  c.drill = 0.5 * 0.1 * (c.As[0] + c.As[2]);
  return c;
}
// TACSShellConstitutive::computeStress (TACSShellConstitutive.h:133-155)
template <class R>
__device__ __forceinline__ R shell_stress_row(const ShellStiff &c, const R *e,
                                              int r) {
  switch (r) {
    case 0: return c.A[0] * e[0] + c.A[1] * e[1] + c.A[2] * e[2];
    case 1: return c.A[1] * e[0] + c.A[3] * e[1] + c.A[4] * e[2];
    case 2: return c.A[2] * e[0] + c.A[4] * e[1] + c.A[5] * e[2];
    case 3: return c.D[0] * e[3] + c.D[1] * e[4] + c.D[2] * e[5];
    case 4: return c.D[1] * e[3] + c.D[3] * e[4] + c.D[4] * e[5];
    case 5: return c.D[2] * e[3] + c.D[4] * e[4] + c.D[5] * e[5];
    case 6: return c.As[0] * e[6] + c.As[1] * e[7];
    case 7: return c.As[1] * e[6] + c.As[2] * e[7];
    default: return c.drill * e[8];
  }
}

// Point quantities at the 4 Gauss points with the drilling strain excluded
// (TACSShellElement::evalPointQuantity, TACSShellElement.h:1015-1072):
// failure value (TACSIsoShellConstitutive::evalFailure, .cpp:254-300),
// detXd, and sum_q detXd_q e.s (strain energy, TACSCompliance).
template <class R>
struct FailOutT {
  R f, dfde[6], dfdt;
};
using FailOut = FailOutT<double>;
template <class R>
__device__ FailOutT<R> shell_failure(const ElemParams &ep, double t,
                                     const R *e) {
  FailOutT<R> o;
  double Dm = ep.E / (1.0 - ep.nu * ep.nu);
  double A0[6] = {Dm, ep.nu * Dm, 0.0, Dm, 0.0, 0.5 * ep.E / (1.0 + ep.nu)};
  double ht = 0.5 * t, hb = -(0.5) * t;
  R et[3], eb[3], st[3], sb[3];
  for (int i = 0; i < 3; i++) {
    et[i] = e[i] + ht * e[3 + i];
    eb[i] = e[i] + hb * e[3 + i];
  }
  st[0] = A0[0] * et[0] + A0[1] * et[1] + A0[2] * et[2];
  st[1] = A0[1] * et[0] + A0[3] * et[1] + A0[4] * et[2];
  st[2] = A0[2] * et[0] + A0[4] * et[1] + A0[5] * et[2];
  sb[0] = A0[0] * eb[0] + A0[1] * eb[1] + A0[2] * eb[2];
  sb[1] = A0[1] * eb[0] + A0[3] * eb[1] + A0[4] * eb[2];
  sb[2] = A0[2] * eb[0] + A0[4] * eb[1] + A0[5] * eb[2];
  // vonMisesFailure2D / StressSens (TACSMaterialProperties.cpp:481-500)
  R ftop = sqrt(st[0] * st[0] + st[1] * st[1] - st[0] * st[1] +
                     3.0 * st[2] * st[2]);
  R fbot = sqrt(sb[0] * sb[0] + sb[1] * sb[1] - sb[0] * sb[1] +
                     3.0 * sb[2] * sb[2]);
  R pt[3] = {0.0, 0.0, 0.0}, pb[3] = {0.0, 0.0, 0.0};
  if (ftop != 0.0) {
    pt[0] = (st[0] - 0.5 * st[1]) / (ftop * ep.ys);
    pt[1] = (st[1] - 0.5 * st[0]) / (ftop * ep.ys);
    pt[2] = (3.0 * st[2]) / (ftop * ep.ys);
  }
  if (fbot != 0.0) {
    pb[0] = (sb[0] - 0.5 * sb[1]) / (fbot * ep.ys);
    pb[1] = (sb[1] - 0.5 * sb[0]) / (fbot * ep.ys);
    pb[2] = (3.0 * sb[2]) / (fbot * ep.ys);
  }
  R top = ftop / ep.ys, bot = fbot / ep.ys;
  R mx = (top > bot) ? top : bot;
  const double ksw = 100.0;  // TACSIsoShellConstitutive.cpp:42
  R ksum = exp(ksw * (top - mx)) + exp(ksw * (bot - mx));
  o.f = mx + log(ksum) / ksw;
  R ft = exp(ksw * (top - mx)) / ksum, fb = exp(ksw * (bot - mx)) / ksum;
  R phit[3], phib[3];
  phit[0] = A0[0] * pt[0] + A0[1] * pt[1] + A0[2] * pt[2];
  phit[1] = A0[1] * pt[0] + A0[3] * pt[1] + A0[4] * pt[2];
  phit[2] = A0[2] * pt[0] + A0[4] * pt[1] + A0[5] * pt[2];
  phib[0] = A0[0] * pb[0] + A0[1] * pb[1] + A0[2] * pb[2];
  phib[1] = A0[1] * pb[0] + A0[3] * pb[1] + A0[4] * pb[2];
  phib[2] = A0[2] * pb[0] + A0[4] * pb[1] + A0[5] * pb[2];
  for (int i = 0; i < 3; i++) {
    o.dfde[i] = ft * phit[i] + fb * phib[i];
    o.dfde[3 + i] = ft * ht * phit[i] + fb * hb * phib[i];
  }
  o.dfdt = ft * 0.5 * (phit[0] * e[3] + phit[1] * e[4] + phit[2] * e[5]) +
           fb * -(0.5) * (phib[0] * e[3] + phib[1] * e[4] + phib[2] * e[5]);
  return o;
}

// d(stress . psi)/dt: TACSIsoShellConstitutive::addStressDVSens
// (.cpp:229-252) with tOffset = 0
__device__ __forceinline__ double shell_stress_dv(const ElemParams &ep,
                                                  double t, const double *e,
                                                  const double *psi) {
  double Dm = ep.E / (1.0 - ep.nu * ep.nu), G = 0.5 * ep.E / (1.0 + ep.nu);
  double A[6] = {Dm, ep.nu * Dm, 0.0, Dm, 0.0, G};
  auto symin = [&](const double *x, const double *y) {
    return x[0] * (A[0] * y[0] + A[1] * y[1] + A[2] * y[2]) +
           x[1] * (A[1] * y[0] + A[3] * y[1] + A[4] * y[2]) +
           x[2] * (A[2] * y[0] + A[4] * y[1] + A[5] * y[2]);
  };
  double dI = 0.25 * t * t;
  return symin(psi, e) + dI * symin(psi + 3, e + 3) +
         (5.0 / 6.0) * A[5] *
             (psi[6] * e[6] + psi[7] * e[7] + 0.1 * psi[8] * e[8]);
}

