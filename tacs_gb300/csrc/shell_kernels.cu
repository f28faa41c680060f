// MITC4 shell (TACSQuad4Shell) element kernels for sm_103a.
//
// One warp owns one element at a time.  The element's strain-displacement
// operators B_q (9 x 24 at each of the 4 Gauss points) are built
// cooperatively in shared memory from exactly the reference kinematics
// (node normals, nodal drilling strains, the 9 MITC tying strains, the
// transform T, Xd^-1 T and the through-thickness term), then:
//   residual  r = sum_q detXd_q B_q^T C e_q + loads   (TACSShellElement::
//             addResidual, src/elements/shell/TACSShellElement.h:295-433)
//   Jacobian  K = sum_q detXd_q B_q^T C B_q           (addJacobian,
//             TACSShellElement.h:436-641, alpha = 1, beta = gamma = 0)
// and K is added into the 6x6 BCSR blocks of the element's 16 node pairs.
// Elements of one launch share no node (graph colouring), so the block
// read-modify-writes and residual scatters need no atomics and the result
// is bitwise deterministic.
#include <cmath>

#include "tg_internal.h"

namespace tg {
namespace {

// TacsGaussQuadPts2 (src/elements/basis/TACSGaussQuadrature.h:26)
#define TG_GPT 0.577350269189626

struct ShellSmem {
  double X[12];
  double u[24];
  double w[24];
  double fn[12];
  double Bd[4][24];
  double Bty[9][24];
  double T[4][9], P[4][9], Q[4][9];
  double det[4];
  double n0[4][3];
  double M[4][5][9];
  double B[4][9][24];
  double CB[4][9][24];
  double e[4][9];
  double g[4][9];
  double coef[4];
  double t;
  int nodes[4];
  int slot[16];
};

__device__ __forceinline__ double gauss2(int i) {
  return i ? TG_GPT : -TG_GPT;
}

__device__ __forceinline__ double dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ void cross3(const double *x, const double *y,
                                       double *o) {
  o[0] = x[1] * y[2] - x[2] * y[1];
  o[1] = x[2] * y[0] - x[0] * y[2];
  o[2] = x[0] * y[1] - x[1] * y[0];
}
// inv3x3 (src/elements/TACSElementAlgebra.h:1980)
__device__ double inv3(const double *A, double *Ai) {
  double det = (A[8] * (A[0] * A[4] - A[3] * A[1]) -
                A[7] * (A[0] * A[5] - A[3] * A[2]) +
                A[6] * (A[1] * A[5] - A[2] * A[4]));
  double di = 1.0 / det;
  Ai[0] = (A[4] * A[8] - A[5] * A[7]) * di;
  Ai[1] = -(A[1] * A[8] - A[2] * A[7]) * di;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * di;
  Ai[3] = -(A[3] * A[8] - A[5] * A[6]) * di;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * di;
  Ai[5] = -(A[0] * A[5] - A[2] * A[3]) * di;
  Ai[6] = (A[3] * A[7] - A[4] * A[6]) * di;
  Ai[7] = -(A[0] * A[7] - A[1] * A[6]) * di;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * di;
  return det;
}
__device__ __forceinline__ void mm3(const double *A, const double *B,
                                    double *C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] +
                     A[3 * i + 2] * B[6 + j];
}
__device__ __forceinline__ void mmT3(const double *A, const double *B,
                                     double *C) {
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
__device__ __forceinline__ void grad3(const double *Na, const double *Nb,
                                      const double *X, double *Xxi) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++) {
      a += Na[m] * X[3 * m + k];
      b += Nb[m] * X[3 * m + k];
    }
    Xxi[2 * k] = a;
    Xxi[2 * k + 1] = b;
  }
}
__device__ __forceinline__ void interp3(const double *N, const double *X,
                                        double *o) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double a = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++) a += N[m] * X[3 * m + k];
    o[k] = a;
  }
}
__device__ __forceinline__ void frame(const double *Xxi, const double *n,
                                      double *Xd) {
  Xd[0] = Xxi[0]; Xd[1] = Xxi[1]; Xd[2] = n[0];
  Xd[3] = Xxi[2]; Xd[4] = Xxi[3]; Xd[5] = n[1];
  Xd[6] = Xxi[4]; Xd[7] = Xxi[5]; Xd[8] = n[2];
}
// TACSShellNaturalTransform / TACSShellRefAxisTransform::computeTransform
// (src/elements/shell/TACSShellElementTransform.h:24-93, 95-160), including
// the natural transform's three-fold subtraction of d*n[0] from t1[0].
__device__ void shell_transform(const ElemParams &ep, const double *Xxi,
                                const double *n0, double *T) {
  double n[3] = {n0[0], n0[1], n0[2]};
  double inv = 1.0 / sqrt(dot3(n, n));
  n[0] *= inv; n[1] *= inv; n[2] *= inv;
  double t1[3];
  if (ep.transform == 0) {
    t1[0] = Xxi[0]; t1[1] = Xxi[2]; t1[2] = Xxi[4];
    double d = dot3(n, t1);
    t1[0] = t1[0] - d * n[0];
    t1[0] = t1[0] - d * n[0];
    t1[0] = t1[0] - d * n[0];
  } else {
    double an = dot3(ep.ref_axis, n);
    t1[0] = ep.ref_axis[0] - an * n[0];
    t1[1] = ep.ref_axis[1] - an * n[1];
    t1[2] = ep.ref_axis[2] - an * n[2];
  }
  inv = 1.0 / sqrt(dot3(t1, t1));
  t1[0] *= inv; t1[1] *= inv; t1[2] *= inv;
  double t2[3];
  cross3(n, t1, t2);
  T[0] = t1[0]; T[3] = t1[1]; T[6] = t1[2];
  T[1] = t2[0]; T[4] = t2[1]; T[7] = t2[2];
  T[2] = n[0];  T[5] = n[1];  T[8] = n[2];
}
// director map d = q x fn: entry (i, b) of the 3x3 map for node m
__device__ __forceinline__ double dmap(const double *f, int i, int b) {
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

// Build fn, Bd, Bty and the Gauss-point geometry, then B_q, for the element
// whose coordinates are in S.X.  All lanes participate.
__device__ void shell_build_B(ShellSmem &S, const ElemParams &ep, int lane) {
  double N[4], Na[4], Nb[4], Xxi[6];
  // node normals (TacsShellComputeNodeNormals, TACSShellUtilities.h:301)
  if (lane < 4) {
    shape2(-1.0 + 2.0 * (lane % 2), -1.0 + 2.0 * (lane / 2), N, Na, Nb);
    grad3(Na, Nb, S.X, Xxi);
    double a[3] = {Xxi[0], Xxi[2], Xxi[4]}, b[3] = {Xxi[1], Xxi[3], Xxi[5]};
    double f[3];
    cross3(a, b, f);
    double nrm = sqrt(dot3(f, f));
    if (nrm != 0.0) {
      double s = 1.0 / nrm;
      f[0] *= s; f[1] *= s; f[2] *= s;
    }
    S.fn[3 * lane] = f[0];
    S.fn[3 * lane + 1] = f[1];
    S.fn[3 * lane + 2] = f[2];
  }
  __syncwarp();
  if (lane < 4) {
    // nodal drilling-strain row (TacsShellComputeDrillStrain +
    // TacsShellAddDrillStrainSens, TACSShellUtilities.h:651-790)
    const int k = lane;
    const double *f = &S.fn[3 * k];
    double Xdn[9], Tn[9], Xdinv[9], XdinvT[9], tmp[9], du0d[9], dCpt[9];
    frame(Xxi, f, Xdn);
    shell_transform(ep, Xxi, f, Tn);
    inv3(Xdn, Xdinv);
    mm3(Xdinv, Tn, XdinvT);
    const double du0x[9] = {0.0, -0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0};
    mmT3(du0x, XdinvT, tmp);
    mm3(Tn, tmp, du0d);
    mm3(Tn, du0x, tmp);
    mmT3(tmp, Tn, dCpt);
    shape2(-1.0 + 2.0 * (k % 2), -1.0 + 2.0 * (k / 2), N, Na, Nb);
    for (int m = 0; m < 4; m++) {
      for (int a = 0; a < 3; a++)
        S.Bd[k][6 * m + a] = Na[m] * du0d[3 * a] + Nb[m] * du0d[3 * a + 1];
      S.Bd[k][6 * m + 3] = 0.0;
      S.Bd[k][6 * m + 4] = 0.0;
      S.Bd[k][6 * m + 5] = 0.0;
    }
    S.Bd[k][6 * k + 3] = 0.0 + -(dCpt[7] - dCpt[5]);
    S.Bd[k][6 * k + 4] = 0.0 + -(dCpt[2] - dCpt[6]);
    S.Bd[k][6 * k + 5] = 0.0 + -(dCpt[3] - dCpt[1]);
  } else if (lane < 8) {
    // Gauss-point geometry (TacsShellComputeDispGrad,
    // TACSShellUtilities.h:361-420) and the tying-to-strain map M_q
    const int q = lane - 4;
    const double xi = gauss2(q % 2), eta = gauss2(q / 2);
    double n0[3], T[9], nxi[6], Xd[9], Xdz[9], Xdinv[9], nXX[9], P[9], Qm[9];
    shape2(xi, eta, N, Na, Nb);
    grad3(Na, Nb, S.X, Xxi);
    interp3(N, S.fn, n0);
    shell_transform(ep, Xxi, n0, T);
    grad3(Na, Nb, S.fn, nxi);
    frame(Xxi, n0, Xd);
    Xdz[0] = nxi[0]; Xdz[1] = nxi[1]; Xdz[2] = 0.0;
    Xdz[3] = nxi[2]; Xdz[4] = nxi[3]; Xdz[5] = 0.0;
    Xdz[6] = nxi[4]; Xdz[7] = nxi[5]; Xdz[8] = 0.0;
    S.det[q] = inv3(Xd, Xdinv);
    mm3(Xdinv, Xdz, nXX);
    for (int i = 0; i < 9; i++) nXX[i] = -nXX[i];
    mm3(Xdinv, T, P);
    mm3(nXX, P, Qm);
    for (int i = 0; i < 9; i++) {
      S.T[q][i] = T[i];
      S.P[q][i] = P[i];
      S.Q[q][i] = Qm[i];
    }
    S.n0[q][0] = n0[0]; S.n0[q][1] = n0[1]; S.n0[q][2] = n0[2];
    // tying interpolation (evalTyingInterp, TACSShellElementQuadBasis.h:552)
    double la0 = (xi - 1.0) * -0.5, la1 = (xi + 1.0) * 0.5;
    double lb0 = (eta - 1.0) * -0.5, lb1 = (eta + 1.0) * 0.5;
    double Nty[9] = {lb0, lb1, la0, la1, 1.0, la0, la1, lb0, lb1};
    for (int t = 0; t < 9; t++) {
      int i = c_ty_ij[c_ty_field[t]][0], j = c_ty_ij[c_ty_field[t]][1];
      for (int r = 0; r < 5; r++) {
        int a = c_erc[r][0], c = c_erc[r][1];
        double s = P[3 * i + a] * P[3 * j + c];
        if (i != j) s += P[3 * j + a] * P[3 * i + c];
        S.M[q][r][t] = c_efac[r] * Nty[t] * s;
      }
    }
  } else if (lane < 17) {
    // tying-strain rows (TACSShellLinearModel::computeTyingStrain,
    // TACSShellElementModel.h:28-73)
    const int t = lane - 8;
    double n0[3];
    shape2(c_ty_pt[t][0], c_ty_pt[t][1], N, Na, Nb);
    grad3(Na, Nb, S.X, Xxi);
    interp3(N, S.fn, n0);
    const int f = c_ty_field[t];
    for (int m = 0; m < 4; m++) {
      for (int a = 0; a < 3; a++) {
        double v;
        if (f == 0) v = Na[m] * Xxi[2 * a];
        else if (f == 1) v = Nb[m] * Xxi[2 * a + 1];
        else if (f == 2)
          v = 0.5 * (Na[m] * Xxi[2 * a + 1] + Nb[m] * Xxi[2 * a]);
        else if (f == 3) v = 0.5 * n0[a] * Nb[m];
        else v = 0.5 * n0[a] * Na[m];
        S.Bty[t][6 * m + a] = v;
      }
      for (int b = 0; b < 3; b++) {
        double v = 0.0;
        if (f >= 3) {
          const int c = (f == 3) ? 1 : 0;
          double acc = 0.0;
          for (int i = 0; i < 3; i++)
            acc += Xxi[2 * i + c] * dmap(&S.fn[3 * m], i, b);
          v = 0.5 * N[m] * acc;
        }
        S.Bty[t][6 * m + 3 + b] = v;
      }
    }
  }
  __syncwarp();

  // B_q entries: rows 0,1,2,6,7 from the tying strains, 3,4,5 bending,
  // 8 drilling (TACSShellLinearModel::evalStrain, .h:717-732)
  for (int idx = lane; idx < 4 * 9 * 24; idx += 32) {
    const int q = idx / 216, rem = idx - 216 * q;
    const int r = rem / 24, c = rem - 24 * r;
    double v = 0.0;
    const int ri = c_ri_of_row[r];
    if (ri >= 0) {
      for (int t = 0; t < 9; t++) {
        double w = S.M[q][ri][t];
        if (w != 0.0) v += w * S.Bty[t][c];
      }
    } else if (r == 8) {
      shape2(gauss2(q % 2), gauss2(q / 2), N, Na, Nb);
      for (int k = 0; k < 4; k++) v += N[k] * S.Bd[k][c];
    } else {
      shape2(gauss2(q % 2), gauss2(q / 2), N, Na, Nb);
      const int m = c / 6, a = c - 6 * m;
      const double *T = S.T[q], *P = S.P[q], *Qm = S.Q[q];
      double cu0 = Na[m] * Qm[0] + Nb[m] * Qm[3];
      double cu1 = Na[m] * Qm[1] + Nb[m] * Qm[4];
      if (a < 3) {
        if (r == 3) v = T[3 * a] * cu0;
        else if (r == 4) v = T[3 * a + 1] * cu1;
        else v = T[3 * a] * cu1 + T[3 * a + 1] * cu0;
      } else {
        const int b = a - 3;
        double cd0 = Na[m] * P[0] + Nb[m] * P[3] + N[m] * Qm[6];
        double cd1 = Na[m] * P[1] + Nb[m] * P[4] + N[m] * Qm[7];
        const double *f = &S.fn[3 * m];
        for (int aa = 0; aa < 3; aa++) {
          double bd;
          if (r == 3) bd = T[3 * aa] * cd0;
          else if (r == 4) bd = T[3 * aa + 1] * cd1;
          else bd = T[3 * aa] * cd1 + T[3 * aa + 1] * cd0;
          v += bd * dmap(f, aa, b);
        }
      }
    }
    S.B[q][r][c] = v;
  }
  __syncwarp();
}

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
__device__ __forceinline__ double shell_stress_row(const ShellStiff &c,
                                                   const double *e, int r) {
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

// strains e_q = B_q v for the 4 points (36 outputs), v in shared memory
__device__ __forceinline__ void shell_strains(ShellSmem &S, const double *v,
                                             double (*e)[9], int lane) {
  for (int idx = lane; idx < 36; idx += 32) {
    const int q = idx / 9, r = idx - 9 * q;
    double acc = 0.0;
    for (int k = 0; k < 24; k++) acc += S.B[q][r][k] * v[k];
    e[q][r] = acc;
  }
  __syncwarp();
}

__device__ __forceinline__ void load_element(ShellSmem &S, const MeshView &m,
                                             int e, const double *vars,
                                             const double *vars2, int lane) {
  if (lane < 4) S.nodes[lane] = m.conn[4 * e + lane];
  if (lane == 0) S.t = m.thick[e];
  __syncwarp();
  if (lane < 12) S.X[lane] = m.xpts[3 * S.nodes[lane / 3] + lane % 3];
  if (lane < 24) {
    S.u[lane] = vars ? vars[6 * S.nodes[lane / 6] + lane % 6] : 0.0;
    if (vars2) S.w[lane] = vars2[6 * S.nodes[lane / 6] + lane % 6];
  }
  __syncwarp();
}

// binary search of col in the sorted column list of row
__device__ __forceinline__ int find_slot(const int *rowp, const int *cols,
                                         int row, int col) {
  int lo = rowp[row], hi = rowp[row + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    int c = cols[mid];
    if (c == col) return mid;
    if (c < col) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    shell_assembly_kernel(ElemParams ep, MeshView m, ColorRange cr,
                          const double *__restrict__ vars, double lambda,
                          double *__restrict__ res, double *__restrict__ mat,
                          int transpose) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ShellSmem &S = reinterpret_cast<ShellSmem *>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;

  for (int idx = gw; idx < cr.count; idx += nw) {
    const int e = cr.elem_list[idx];
    load_element(S, m, e, vars, nullptr, lane);
    if (mat && lane < 16)
      S.slot[lane] = find_slot(m.rowp, m.cols, S.nodes[lane >> 2],
                               S.nodes[lane & 3]);
    shell_build_B(S, ep, lane);
    const ShellStiff c = shell_stiff(ep, S.t);

    if (res) {
      shell_strains(S, S.u, S.e, lane);
      for (int idx2 = lane; idx2 < 36; idx2 += 32) {
        const int q = idx2 / 9, r = idx2 - 9 * q;
        S.g[q][r] = shell_stress_row(c, S.e[q], r);
      }
      __syncwarp();
      if (lane < 24) {
        double rk = 0.0;
        for (int q = 0; q < 4; q++) {
          double v = 0.0;
          for (int r = 0; r < 9; r++) v += S.B[q][r][lane] * S.g[q][r];
          rk += S.det[q] * v;
        }
        // TACSShellPressure::addResidual (TACSShellPressure.h:56-90)
        if (m.pres) {
          const int mm = lane / 6, a = lane - 6 * mm;
          double aux = 0.0;
          if (a < 3) {
            const double *pn = &m.pres[4 * e];
            for (int q = 0; q < 4; q++) {
              double N[4], Na[4], Nb[4];
              shape2(gauss2(q % 2), gauss2(q / 2), N, Na, Nb);
              double pr = N[0] * pn[0] + N[1] * pn[1] + N[2] * pn[2] +
                          N[3] * pn[3];
              aux += N[mm] * (pr * -S.det[q] * S.n0[q][a]);
            }
          }
          rk += lambda * aux;
        }
        res[6 * S.nodes[lane / 6] + lane % 6] += rk;
      }
    }

    if (mat) {
      for (int idx2 = lane; idx2 < 864; idx2 += 32) {
        const int q = idx2 / 216, rem = idx2 - 216 * q;
        const int r = rem / 24, col = rem - 24 * r;
        double ecol[9];
#pragma unroll
        for (int k = 0; k < 9; k++) ecol[k] = S.B[q][k][col];
        S.CB[q][r][col] = shell_stress_row(c, ecol, r);
      }
      __syncwarp();
      // upper blocks (a <= b): 10 blocks x 36 entries
      for (int idx2 = lane; idx2 < 360; idx2 += 32) {
        const int blk = idx2 / 36, w = idx2 - 36 * blk;
        // blk -> (a, b) with a <= b
        const int a = blk < 4 ? 0 : (blk < 7 ? 1 : (blk < 9 ? 2 : 3));
        const int b = a + blk - (a == 0 ? 0 : (a == 1 ? 4 : (a == 2 ? 7 : 9)));
        const int ii = w / 6, jj = w - 6 * ii;
        const int i = 6 * a + ii, j = 6 * b + jj;
        double kij = 0.0;
        for (int q = 0; q < 4; q++) {
          double v = 0.0;
#pragma unroll
          for (int r = 0; r < 9; r++) v += S.B[q][r][i] * S.CB[q][r][j];
          kij += S.det[q] * v;
        }
        kij *= 1.0;
        // TACS_MAT_TRANSPOSE writes K^T; K is symmetric by construction
        // (upper blocks mirrored), so both orientations store the same.
        (void)transpose;
        const int s_ab = S.slot[4 * a + b], s_ba = S.slot[4 * b + a];
        if (s_ab >= 0) mat[36 * (size_t)s_ab + w] += kij;
        if (a != b && s_ba >= 0) mat[36 * (size_t)s_ba + 6 * jj + ii] += kij;
      }
    }
    __syncwarp();
  }
}

// Point quantities at the 4 Gauss points with the drilling strain excluded
// (TACSShellElement::evalPointQuantity, TACSShellElement.h:1015-1072):
// failure value (TACSIsoShellConstitutive::evalFailure, .cpp:254-300),
// detXd, and sum_q detXd_q e.s (strain energy, TACSCompliance).
struct FailOut {
  double f, dfde[6], dfdt;
};
__device__ FailOut shell_failure(const ElemParams &ep, double t,
                                 const double *e) {
  FailOut o;
  double Dm = ep.E / (1.0 - ep.nu * ep.nu);
  double A0[6] = {Dm, ep.nu * Dm, 0.0, Dm, 0.0, 0.5 * ep.E / (1.0 + ep.nu)};
  double ht = 0.5 * t, hb = -(0.5) * t;
  double et[3], eb[3], st[3], sb[3];
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
  double ftop = sqrt(st[0] * st[0] + st[1] * st[1] - st[0] * st[1] +
                     3.0 * st[2] * st[2]);
  double fbot = sqrt(sb[0] * sb[0] + sb[1] * sb[1] - sb[0] * sb[1] +
                     3.0 * sb[2] * sb[2]);
  double pt[3] = {0, 0, 0}, pb[3] = {0, 0, 0};
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
  double top = ftop / ep.ys, bot = fbot / ep.ys;
  double mx = (top > bot) ? top : bot;
  const double ksw = 100.0;  // TACSIsoShellConstitutive.cpp:42
  double ksum = exp(ksw * (top - mx)) + exp(ksw * (bot - mx));
  o.f = mx + log(ksum) / ksw;
  double ft = exp(ksw * (top - mx)) / ksum, fb = exp(ksw * (bot - mx)) / ksum;
  double phit[3], phib[3];
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

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    shell_points_kernel(ElemParams ep, MeshView m,
                        const double *__restrict__ vars,
                        double *__restrict__ elem_fail,
                        double *__restrict__ elem_wdet,
                        double *__restrict__ elem_sed) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ShellSmem &S = reinterpret_cast<ShellSmem *>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  for (int e = gw; e < m.nelem; e += nw) {
    load_element(S, m, e, vars, nullptr, lane);
    shell_build_B(S, ep, lane);
    shell_strains(S, S.u, S.e, lane);
    if (lane < 4) {
      const int q = lane;
      double ev[9];
      for (int r = 0; r < 9; r++) ev[r] = S.e[q][r];
      ev[8] = 0.0;
      const ShellStiff c = shell_stiff(ep, S.t);
      double sed = 0.0;
      for (int r = 0; r < 9; r++) sed += ev[r] * shell_stress_row(c, ev, r);
      FailOut fo = shell_failure(ep, S.t, ev);
      elem_fail[4 * (size_t)e + q] = fo.f;
      elem_wdet[4 * (size_t)e + q] = S.det[q];
      S.coef[q] = S.det[q] * sed;
    }
    __syncwarp();
    if (lane == 0)
      elem_sed[e] = ((S.coef[0] + S.coef[1]) + S.coef[2]) + S.coef[3];
    __syncwarp();
  }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    shell_sv_kernel(ElemParams ep, MeshView m, ColorRange cr,
                    const double *__restrict__ vars, int func, KsStats ks,
                    double alpha, double *__restrict__ dfdu) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ShellSmem &S = reinterpret_cast<ShellSmem *>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  for (int idx = gw; idx < cr.count; idx += nw) {
    const int e = cr.elem_list[idx];
    load_element(S, m, e, vars, nullptr, lane);
    shell_build_B(S, ep, lane);
    shell_strains(S, S.u, S.e, lane);
    if (lane < 4) {
      const int q = lane;
      double ev[9];
      for (int r = 0; r < 9; r++) ev[r] = S.e[q][r];
      ev[8] = 0.0;
      if (func == TG_FUNC_COMPLIANCE) {
        // TACSCompliance::getElementSVSens: dfdq = detXd, sens = 2 s
        const ShellStiff c = shell_stiff(ep, S.t);
        for (int r = 0; r < 9; r++) S.g[q][r] = 2.0 * shell_stress_row(c, ev, r);
        S.coef[q] = S.det[q];
      } else {
        // TACSKSFailure::getElementSVSens (KS_CONTINUOUS)
        FailOut fo = shell_failure(ep, S.t, ev);
        for (int r = 0; r < 6; r++) S.g[q][r] = fo.dfde[r];
        S.g[q][6] = S.g[q][7] = S.g[q][8] = 0.0;
        S.coef[q] = exp(ks.weight * (fo.f - ks.max)) / ks.sum * S.det[q];
      }
    }
    __syncwarp();
    if (lane < 24) {
      double acc = 0.0;
      for (int q = 0; q < 4; q++) {
        double v = 0.0;
        for (int r = 0; r < 8; r++) v += S.B[q][r][lane] * S.g[q][r];
        acc += S.coef[q] * v;
      }
      dfdu[6 * S.nodes[lane / 6] + lane % 6] += alpha * acc;
    }
    __syncwarp();
  }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    shell_dv_kernel(ElemParams ep, MeshView m, const double *__restrict__ vars,
                    int func, KsStats ks, double coef,
                    const double *__restrict__ psi, double scale,
                    double *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ShellSmem &S = reinterpret_cast<ShellSmem *>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  for (int e = gw; e < m.nelem; e += nw) {
    load_element(S, m, e, vars, psi, lane);
    shell_build_B(S, ep, lane);
    shell_strains(S, S.u, S.e, lane);
    if (psi) shell_strains(S, S.w, S.g, lane);
    if (lane < 4) {
      const int q = lane;
      double acc = 0.0;
      if (func >= 0) {
        double ev[9];
        for (int r = 0; r < 9; r++) ev[r] = S.e[q][r];
        ev[8] = 0.0;
        if (func == TG_FUNC_COMPLIANCE) {
          // TACSCompliance::addElementDVSens -> addStressDVSens(e, e)
          acc += coef * S.det[q] * shell_stress_dv(ep, S.t, ev, ev);
        } else {
          FailOut fo = shell_failure(ep, S.t, ev);
          double dfdq = S.det[q] * exp(ks.weight * (fo.f - ks.max)) / ks.sum;
          acc += coef * dfdq * fo.dfdt;
        }
      }
      if (psi) {
        // TACSShellElement::addAdjResProduct (TACSShellElement.h:918-1012)
        acc += scale * S.det[q] * shell_stress_dv(ep, S.t, S.e[q], S.g[q]);
      }
      S.coef[q] = acc;
    }
    __syncwarp();
    if (lane == 0) out[e] = ((S.coef[0] + S.coef[1]) + S.coef[2]) + S.coef[3];
    __syncwarp();
  }
}

constexpr int kWarps = 4;

int grid_for(int count, int ctas_per_sm) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int need = (count + kWarps - 1) / kWarps;
  int cap = sms * ctas_per_sm;
  if (need < 1) need = 1;
  return need < cap ? need : cap;
}

template <typename K>
void prep(K kernel) {
  static bool done = false;
  if (!done) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(ShellSmem) * kWarps));
    done = true;
  }
}

}  // namespace

void launch_shell_assembly(const ElemParams &ep, const MeshView &m,
                           ColorRange cr, const double *vars, double lambda,
                           double *res, double *mat, int transpose,
                           cudaStream_t s) {
  if (cr.count <= 0) return;
  auto k = shell_assembly_kernel<kWarps>;
  prep(k);
  k<<<grid_for(cr.count, 2), kWarps * 32, sizeof(ShellSmem) * kWarps, s>>>(
      ep, m, cr, vars, lambda, res, mat, transpose);
}

void launch_shell_points(const ElemParams &ep, const MeshView &m,
                         const double *vars, double *elem_fail,
                         double *elem_wdet, double *elem_sed,
                         cudaStream_t s) {
  if (m.nelem <= 0) return;
  auto k = shell_points_kernel<kWarps>;
  prep(k);
  k<<<grid_for(m.nelem, 2), kWarps * 32, sizeof(ShellSmem) * kWarps, s>>>(
      ep, m, vars, elem_fail, elem_wdet, elem_sed);
}

void launch_shell_sv_sens(const ElemParams &ep, const MeshView &m,
                          ColorRange cr, const double *vars, int func,
                          KsStats ks, double alpha, double *dfdu,
                          cudaStream_t s) {
  if (cr.count <= 0) return;
  auto k = shell_sv_kernel<kWarps>;
  prep(k);
  k<<<grid_for(cr.count, 2), kWarps * 32, sizeof(ShellSmem) * kWarps, s>>>(
      ep, m, cr, vars, func, ks, alpha, dfdu);
}

void launch_shell_dv(const ElemParams &ep, const MeshView &m,
                     const double *vars, int func, KsStats ks, double coef,
                     const double *psi, double scale, double *out,
                     cudaStream_t s) {
  if (m.nelem <= 0) return;
  auto k = shell_dv_kernel<kWarps>;
  prep(k);
  k<<<grid_for(m.nelem, 2), kWarps * 32, sizeof(ShellSmem) * kWarps, s>>>(
      ep, m, vars, func, ks, coef, psi, scale, out);
}

}  // namespace tg
