// Device helpers of the hex8 kernels (TACSLinearHexaBasis,
// TACSLinearElasticity3D with the isotropic TACSSolidConstitutive): shape
// functions, the isotropic stiffness, face quadrature and the von Mises
// value (the shared dense helpers are in elem_math.cuh).  Included by the
// hex kernel translation unit inside namespace tg::<anonymous> (and
// compiled for the host by the CPU check of the node-coordinate
// derivative).  The helpers that depend on the node coordinates are
// templates over the scalar type.
#pragma once

#include "elem_math.cuh"

// TACSLinearHexaBasis::computeBasis / computeBasisGradient
// (src/elements/basis/TACSHexaBasis.cpp:137-170), node m = i + 2j + 4k
__device__ __forceinline__ void hex_shape(const double *pt, double *N,
                                          double *Nxi) {
  double x[2] = {1.0 - pt[0], 1.0 + pt[0]};
  double y[2] = {1.0 - pt[1], 1.0 + pt[1]};
  double z[2] = {1.0 - pt[2], 1.0 + pt[2]};
#pragma unroll
  for (int m = 0; m < 8; m++) {
    const int i = m & 1, j = (m >> 1) & 1, k = m >> 2;
    const double si = i ? 1.0 : -1.0, sj = j ? 1.0 : -1.0, sk = k ? 1.0 : -1.0;
    if (N) N[m] = 0.125 * x[i] * y[j] * z[k];
    Nxi[3 * m] = 0.125 * si * y[j] * z[k];
    Nxi[3 * m + 1] = 0.125 * x[i] * sj * z[k];
    Nxi[3 * m + 2] = 0.125 * x[i] * y[j] * sk;
  }
}

struct HexC {
  double c0, c1, G;
};
// TACSMaterialProperties::evalTangentStiffness3D, isotropic branch
__device__ __forceinline__ HexC hex_c(const ElemParams &ep) {
  HexC c;
  double D = ep.E / ((1.0 + ep.nu) * (1.0 - 2.0 * ep.nu));
  c.c0 = (1.0 - ep.nu) * D;
  c.c1 = ep.nu * D;
  c.G = 0.5 * ep.E / (1.0 + ep.nu);
  return c;
}
template <class R>
__device__ __forceinline__ void hex_Ce(const HexC &c, const R *e, R *s) {
  s[0] = c.c0 * e[0] + c.c1 * e[1] + c.c1 * e[2];
  s[1] = c.c1 * e[0] + c.c0 * e[1] + c.c1 * e[2];
  s[2] = c.c1 * e[0] + c.c1 * e[1] + c.c0 * e[2];
  s[3] = c.G * e[3];
  s[4] = c.G * e[4];
  s[5] = c.G * e[5];
}

// Face quadrature point n of face `face`: shape functions N and the area
// element |t1 x t2| (TACSElementBasis::getFaceNormal,
// TACSElementBasis.cpp:37-63; face tangents TACSHexaBasis.cpp:21-70).
template <class R>
__device__ R hex_face_point(const R *X, int face, int n, double *N) {
  const int f2 = face >> 1;
  const double u = gauss2(n & 1), v = gauss2(n >> 1);
  const double cc = -1.0 + 2.0 * (face & 1);
  double pt[3];
  if (f2 == 0) { pt[0] = cc; pt[1] = u; pt[2] = v; }
  else if (f2 == 1) { pt[0] = u; pt[1] = cc; pt[2] = v; }
  else { pt[0] = u; pt[1] = v; pt[2] = cc; }
  double Nxi[24];
  R Xd[9];
  hex_shape(pt, N, Nxi);
  for (int ii = 0; ii < 3; ii++)
    for (int jj = 0; jj < 3; jj++) {
      R s = 0.0;
      for (int q = 0; q < 8; q++) s += Nxi[3 * q + jj] * X[3 * q + ii];
      Xd[3 * ii + jj] = s;
    }
  int ta, tb;
  if (f2 == 0) { ta = 2; tb = 1; }
  else if (f2 == 1) { ta = 0; tb = 2; }
  else { ta = 1; tb = 0; }
  if (face == 1) { ta = 1; tb = 2; }
  if (face == 3) { ta = 2; tb = 0; }
  if (face == 5) { ta = 0; tb = 1; }
  R t1[3], t2[3];
  for (int ii = 0; ii < 3; ii++) {
    t1[ii] = Xd[3 * ii + ta];
    t2[ii] = Xd[3 * ii + tb];
  }
  const R nr[3] = {t1[1] * t2[2] - t1[2] * t2[1],
                   t1[2] * t2[0] - t1[0] * t2[2],
                   t1[0] * t2[1] - t1[1] * t2[0]};
  return sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
}

template <class R>
__device__ R hex_vm(const ElemParams &ep, const R *s) {
  return sqrt(0.5 * ((s[0] - s[1]) * (s[0] - s[1]) +
                     (s[0] - s[2]) * (s[0] - s[2]) +
                     (s[1] - s[2]) * (s[1] - s[2]) +
                     6.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]))) /
         ep.ys;
}

