/*
  CPU oracle for the TACS finite-element hot path -- TEST INFRASTRUCTURE.
  See tacs_oracle.h for scope.  Every routine cites the reference function it
  restates (paths relative to the TACS source tree).

  Element formulation.  TACSQuad4Shell with TACSShellLinearModel and
  TACSLinearizedRotation is linear in the element variables: every strain
  component at a quadrature point (membrane and transverse shear through the
  MITC tying strains, bending through u1x, drilling through the nodal drill
  strains) is e = B u for a 9 x 24 matrix B that depends only on geometry.
  The reference forms the residual as B^T s and the Jacobian through the
  chain of strain/tying/director Hessians
  (src/elements/shell/TACSShellElement.h:295-641); both equal
  sum_q detXd_q B_q^T C B_q (+ load terms), which is what is computed here.
  B is built from exactly the reference kinematics, including the natural
  transform's repeated projection of t1[0] (TACSShellElementTransform.h:40-42).
*/
#include "tacs_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* TacsGaussQuadPts2 (src/elements/basis/TACSGaussQuadrature.h:26): the
   reference uses this 15-digit value, not 1/sqrt(3). */
#define GPT 0.577350269189626
static const double gauss2[2] = {-GPT, GPT};

/* ----------------------------- 3x3 algebra ----------------------------- */
/* inv3x3 (src/elements/TACSElementAlgebra.h:1980) */
static double inv3(const double A[9], double Ai[9]) {
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
static void mm3(const double A[9], const double B[9], double C[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] +
                     A[3 * i + 2] * B[6 + j];
}
/* C = A * B^T */
static void mmT3(const double A[9], const double B[9], double C[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[3 * j] + A[3 * i + 1] * B[3 * j + 1] +
                     A[3 * i + 2] * B[3 * j + 2];
}
static double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static void cross3(const double x[3], const double y[3], double o[3]) {
  o[0] = x[1] * y[2] - x[2] * y[1];
  o[1] = x[2] * y[0] - x[0] * y[2];
  o[2] = x[0] * y[1] - x[1] * y[0];
}

/* --------------------------- shell kinematics -------------------------- */
/* TACSShellQuadBasis<2> shape functions (TACSShellElementQuadBasis.h:86-99) */
static void shape2(double xi, double eta, double N[4], double Na[4],
                   double Nb[4]) {
  double na[2] = {0.5 * (1.0 - xi), 0.5 * (1.0 + xi)};
  double nb[2] = {0.5 * (1.0 - eta), 0.5 * (1.0 + eta)};
  double dn[2] = {-0.5, 0.5};
  for (int j = 0; j < 2; j++)
    for (int i = 0; i < 2; i++) {
      N[i + 2 * j] = na[i] * nb[j];
      Na[i + 2 * j] = dn[i] * nb[j];
      Nb[i + 2 * j] = na[i] * dn[j];
    }
}
/* interpFieldsGrad<3,3> (TACSShellElementQuadBasis.h:200-222) */
static void grad3(const double Na[4], const double Nb[4], const double *X,
                  double Xxi[6]) {
  for (int k = 0; k < 3; k++) {
    double a = 0.0, b = 0.0;
    for (int m = 0; m < 4; m++) {
      a += Na[m] * X[3 * m + k];
      b += Nb[m] * X[3 * m + k];
    }
    Xxi[2 * k] = a;
    Xxi[2 * k + 1] = b;
  }
}
static void interp3(const double N[4], const double *X, double out[3]) {
  for (int k = 0; k < 3; k++) {
    double a = 0.0;
    for (int m = 0; m < 4; m++) a += N[m] * X[3 * m + k];
    out[k] = a;
  }
}
/* TacsShellAssembleFrame(Xxi, n, Xd) (TACSShellUtilities.h:8-21) */
static void frame(const double Xxi[6], const double n[3], double Xd[9]) {
  Xd[0] = Xxi[0]; Xd[1] = Xxi[1]; Xd[2] = n[0];
  Xd[3] = Xxi[2]; Xd[4] = Xxi[3]; Xd[5] = n[1];
  Xd[6] = Xxi[4]; Xd[7] = Xxi[5]; Xd[8] = n[2];
}
/* TACSShellNaturalTransform / TACSShellRefAxisTransform::computeTransform
   (TACSShellElementTransform.h:24-93, 95-160) */
static void shell_transform(const or_problem *p, const double Xxi[6],
                            const double n0[3], double T[9]) {
  double n[3] = {n0[0], n0[1], n0[2]};
  double inv = 1.0 / sqrt(dot3(n, n));
  n[0] *= inv; n[1] *= inv; n[2] *= inv;
  double t1[3];
  if (p->transform == 0) {
    t1[0] = Xxi[0]; t1[1] = Xxi[2]; t1[2] = Xxi[4];
    double d = dot3(n, t1);
    /* the reference subtracts d*n[0] from t1[0] three times */
    t1[0] = t1[0] - d * n[0];
    t1[0] = t1[0] - d * n[0];
    t1[0] = t1[0] - d * n[0];
  } else {
    double ax[3] = {p->ref_axis[0], p->ref_axis[1], p->ref_axis[2]};
    double nrm = sqrt(dot3(ax, ax));
    double ivn = (nrm != 0.0) ? 1.0 / nrm : 0.0;
    ax[0] *= ivn; ax[1] *= ivn; ax[2] *= ivn;
    double an = dot3(ax, n);
    t1[0] = ax[0] - an * n[0];
    t1[1] = ax[1] - an * n[1];
    t1[2] = ax[2] - an * n[2];
  }
  inv = 1.0 / sqrt(dot3(t1, t1));
  t1[0] *= inv; t1[1] *= inv; t1[2] *= inv;
  double t2[3];
  cross3(n, t1, t2);
  T[0] = t1[0]; T[3] = t1[1]; T[6] = t1[2];
  T[1] = t2[0]; T[4] = t2[1]; T[7] = t2[2];
  T[2] = n[0];  T[5] = n[1];  T[8] = n[2];
}

/* Strain-displacement operators of one shell element. */
typedef struct {
  double B[4][9][24]; /* e_q = B[q] u (q = quadrature point) */
  double detXd[4];    /* det(Xd) at the quadrature points (weights are 1) */
  double N[4][4];     /* shape functions at the quadrature points */
  double n0[4][3];    /* interpolated (unnormalised) node normal */
} shell_geo;

/* Tying-point locations for order 2 (TACSShellElementQuadBasis.h:500-540):
   g11 (0,-1),(0,1); g22 (-1,0),(1,0); g12 (0,0); g23 (-1,0),(1,0);
   g13 (0,-1),(0,1). */
static const double ty_pt[9][2] = {{0, -1}, {0, 1}, {-1, 0}, {1, 0}, {0, 0},
                                   {-1, 0}, {1, 0}, {0, -1}, {0, 1}};
/* field of each tying point: 0 g11, 1 g22, 2 g12, 3 g23, 4 g13 */
static const int ty_field[9] = {0, 0, 1, 1, 2, 3, 3, 4, 4};
/* (i,j) position of each field in the symmetric 3x3 tying tensor */
static const int ty_ij[5][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 2}, {0, 2}};

static void shell_geometry(const double X[12], const or_problem *p,
                           shell_geo *g) {
  double fn[12], Xdn[36];
  double N[4], Na[4], Nb[4], Xxi[6];

  /* TacsShellComputeNodeNormals (TACSShellUtilities.h:301-340) */
  for (int k = 0; k < 4; k++) {
    shape2(-1.0 + 2.0 * (k % 2), -1.0 + 2.0 * (k / 2), N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    double a[3] = {Xxi[0], Xxi[2], Xxi[4]}, b[3] = {Xxi[1], Xxi[3], Xxi[5]};
    cross3(a, b, &fn[3 * k]);
    double nrm = sqrt(dot3(&fn[3 * k], &fn[3 * k]));
    if (nrm != 0.0) {
      double s = 1.0 / nrm;
      fn[3 * k] *= s; fn[3 * k + 1] *= s; fn[3 * k + 2] *= s;
    }
    frame(Xxi, &fn[3 * k], &Xdn[9 * k]);
  }

  /* Director d_k = q_k x fn_k = Dm[k] q_k  (TACSDirector.h:210-245) */
  double Dm[4][9];
  for (int k = 0; k < 4; k++) {
    const double *f = &fn[3 * k];
    Dm[k][0] = 0.0;   Dm[k][1] = f[2];  Dm[k][2] = -f[1];
    Dm[k][3] = -f[2]; Dm[k][4] = 0.0;   Dm[k][5] = f[0];
    Dm[k][6] = f[1];  Dm[k][7] = -f[0]; Dm[k][8] = 0.0;
  }

  /* Nodal drill strain gradients: TacsShellComputeDrillStrain and
     TacsShellAddDrillStrainSens with unit seed (TACSShellUtilities.h:651-790,
     TACSDirector.h:562-590). */
  double Bd[4][24];
  memset(Bd, 0, sizeof(Bd));
  for (int k = 0; k < 4; k++) {
    double Tn[9], Xdinv[9], XdinvT[9], tmp[9], du0d[9], dCpt[9];
    double xk[6] = {Xdn[9 * k], Xdn[9 * k + 1], Xdn[9 * k + 3],
                    Xdn[9 * k + 4], Xdn[9 * k + 6], Xdn[9 * k + 7]};
    shell_transform(p, xk, &fn[3 * k], Tn);
    inv3(&Xdn[9 * k], Xdinv);
    mm3(Xdinv, Tn, XdinvT);
    const double du0x[9] = {0.0, -0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0};
    mmT3(du0x, XdinvT, tmp);
    mm3(Tn, tmp, du0d);
    mm3(Tn, du0x, tmp);
    mmT3(tmp, Tn, dCpt);
    shape2(-1.0 + 2.0 * (k % 2), -1.0 + 2.0 * (k / 2), N, Na, Nb);
    for (int m = 0; m < 4; m++)
      for (int a = 0; a < 3; a++)
        Bd[k][6 * m + a] += Na[m] * du0d[3 * a] + Nb[m] * du0d[3 * a + 1];
    Bd[k][6 * k + 3] += -(dCpt[7] - dCpt[5]);
    Bd[k][6 * k + 4] += -(dCpt[2] - dCpt[6]);
    Bd[k][6 * k + 5] += -(dCpt[3] - dCpt[1]);
  }

  /* Tying strains at the 9 tying points as rows of Bty
     (TACSShellLinearModel::computeTyingStrain,
     TACSShellElementModel.h:28-73) */
  double Bty[9][24];
  memset(Bty, 0, sizeof(Bty));
  for (int t = 0; t < 9; t++) {
    double n0[3];
    shape2(ty_pt[t][0], ty_pt[t][1], N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    interp3(N, fn, n0);
    int f = ty_field[t];
    for (int m = 0; m < 4; m++) {
      for (int a = 0; a < 3; a++) {
        double v = 0.0;
        if (f == 0) v = Na[m] * Xxi[2 * a];
        else if (f == 1) v = Nb[m] * Xxi[2 * a + 1];
        else if (f == 2)
          v = 0.5 * (Na[m] * Xxi[2 * a + 1] + Nb[m] * Xxi[2 * a]);
        else if (f == 3) v = 0.5 * n0[a] * Nb[m];
        else v = 0.5 * n0[a] * Na[m];
        Bty[t][6 * m + a] = v;
      }
      if (f >= 3) {
        int c = (f == 3) ? 1 : 0; /* g23 uses X,eta ; g13 uses X,xi */
        for (int b = 0; b < 3; b++) {
          double v = 0.0;
          for (int i = 0; i < 3; i++) v += Xxi[2 * i + c] * Dm[m][3 * i + b];
          Bty[t][6 * m + 3 + b] = 0.5 * N[m] * v;
        }
      }
    }
  }

  /* Quadrature points (TACSQuadLinearQuadrature, .h:13-30) */
  for (int q = 0; q < 4; q++) {
    double xi = gauss2[q % 2], eta = gauss2[q / 2];
    double T[9], nxi[6], Xd[9], Xdz[9], Xdinv[9], nXX[9], P[9], Q[9], n0[3];
    shape2(xi, eta, N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    interp3(N, fn, n0);
    shell_transform(p, Xxi, n0, T);
    /* TacsShellComputeDispGrad (TACSShellUtilities.h:361-420) */
    grad3(Na, Nb, fn, nxi);
    frame(Xxi, n0, Xd);
    Xdz[0] = nxi[0]; Xdz[1] = nxi[1]; Xdz[2] = 0.0;
    Xdz[3] = nxi[2]; Xdz[4] = nxi[3]; Xdz[5] = 0.0;
    Xdz[6] = nxi[4]; Xdz[7] = nxi[5]; Xdz[8] = 0.0;
    g->detXd[q] = inv3(Xd, Xdinv);
    mm3(Xdinv, Xdz, nXX);
    for (int i = 0; i < 9; i++) nXX[i] = -nXX[i];
    mm3(Xdinv, T, P);  /* XdinvT */
    mm3(nXX, P, Q);    /* XdinvzT */
    memcpy(g->N[q], N, sizeof(N));
    memcpy(g->n0[q], n0, sizeof(n0));

    double (*B)[24] = g->B[q];
    memset(B, 0, sizeof(g->B[q]));

    /* bending: u1x = T^T (u1d P + u0d Q), e3 = u1x00, e4 = u1x11,
       e5 = u1x01 + u1x10 (TACSShellLinearModel::evalStrain, .h:717-732) */
    for (int m = 0; m < 4; m++) {
      double cu[2], cd[2];
      for (int c = 0; c < 2; c++) {
        cu[c] = Na[m] * Q[c] + Nb[m] * Q[3 + c];
        cd[c] = Na[m] * P[c] + Nb[m] * P[3 + c] + N[m] * Q[6 + c];
      }
      double bd[3][3]; /* coefficient of d_m,a in e3..e5 */
      for (int a = 0; a < 3; a++) {
        B[3][6 * m + a] = T[3 * a] * cu[0];
        B[4][6 * m + a] = T[3 * a + 1] * cu[1];
        B[5][6 * m + a] = T[3 * a] * cu[1] + T[3 * a + 1] * cu[0];
        bd[0][a] = T[3 * a] * cd[0];
        bd[1][a] = T[3 * a + 1] * cd[1];
        bd[2][a] = T[3 * a] * cd[1] + T[3 * a + 1] * cd[0];
      }
      for (int r = 0; r < 3; r++)
        for (int b = 0; b < 3; b++) {
          double v = 0.0;
          for (int a = 0; a < 3; a++) v += bd[r][a] * Dm[m][3 * a + b];
          B[3 + r][6 * m + 3 + b] = v;
        }
    }

    /* membrane + transverse shear from the interpolated tying strain:
       e0ty = P^T gty P (mat3x3SymmTransformTranspose) and
       e0 = e0ty00, e1 = e0ty11, e2 = 2 e0ty01, e6 = 2 e0ty12,
       e7 = 2 e0ty02.  Tying interpolation: evalTyingInterp
       (TACSShellElementQuadBasis.h:552-600). */
    double la[2] = {(xi - 1.0) * -0.5, (xi + 1.0) * 0.5};
    double lb[2] = {(eta - 1.0) * -0.5, (eta + 1.0) * 0.5};
    double Nty[9] = {lb[0], lb[1], la[0], la[1], 1.0, la[0], la[1], lb[0],
                     lb[1]};
    static const int erow[5] = {0, 1, 2, 6, 7};
    static const int erc[5][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 2}, {0, 2}};
    static const double efac[5] = {1.0, 1.0, 2.0, 2.0, 2.0};
    for (int t = 0; t < 9; t++) {
      int i = ty_ij[ty_field[t]][0], j = ty_ij[ty_field[t]][1];
      for (int r = 0; r < 5; r++) {
        int a = erc[r][0], c = erc[r][1];
        double s = P[3 * i + a] * P[3 * j + c];
        if (i != j) s += P[3 * j + a] * P[3 * i + c];
        double w = efac[r] * Nty[t] * s;
        if (w != 0.0)
          for (int k = 0; k < 24; k++) B[erow[r]][k] += w * Bty[t][k];
      }
    }
    /* drilling: e8 = sum_k N_k etn_k */
    for (int k = 0; k < 4; k++)
      for (int c = 0; c < 24; c++) B[8][c] += N[k] * Bd[k][c];
  }
}

/* TACSIsoShellConstitutive::evalTangentStiffness with tOffset = 0,
   kcorr = 5/6 and DRILLING_REGULARIZATION = 0.1
   (TACSIsoShellConstitutive.cpp:181-217, TACSShellConstitutive.cpp:61) */
typedef struct {
  double A0[6], A[6], D[6], As[3], drill;
} shell_stiff;
static void shell_constitutive(const or_problem *p, double t, shell_stiff *c) {
  double Dm = p->E / (1.0 - p->nu * p->nu);
  double G = 0.5 * p->E / (1.0 + p->nu);
  c->A0[0] = Dm; c->A0[1] = p->nu * Dm; c->A0[2] = 0.0;
  c->A0[3] = Dm; c->A0[4] = 0.0; c->A0[5] = G;
  double I = t * t * t / 12.0;
  for (int i = 0; i < 6; i++) {
    c->D[i] = I * c->A0[i];
    c->A[i] = c->A0[i] * t;
  }
  double kcorr = 5.0 / 6.0;
  c->As[0] = c->As[2] = kcorr * c->A[5];
  c->As[1] = 0.0;
  c->drill = 0.5 * 0.1 * (c->As[0] + c->As[2]);
}
/* TACSShellConstitutive::computeStress (TACSShellConstitutive.h:133-155) */
static void shell_stress(const shell_stiff *c, const double e[9],
                         double s[9]) {
  const double *A = c->A, *D = c->D, *As = c->As;
  s[0] = A[0] * e[0] + A[1] * e[1] + A[2] * e[2];
  s[1] = A[1] * e[0] + A[3] * e[1] + A[4] * e[2];
  s[2] = A[2] * e[0] + A[4] * e[1] + A[5] * e[2];
  s[3] = D[0] * e[3] + D[1] * e[4] + D[2] * e[5];
  s[4] = D[1] * e[3] + D[3] * e[4] + D[4] * e[5];
  s[5] = D[2] * e[3] + D[4] * e[4] + D[5] * e[5];
  s[6] = As[0] * e[6] + As[1] * e[7];
  s[7] = As[1] * e[6] + As[2] * e[7];
  s[8] = c->drill * e[8];
}
static void shell_strain(const double B[9][24], const double *u,
                         double e[9]) {
  for (int r = 0; r < 9; r++) {
    double v = 0.0;
    for (int k = 0; k < 24; k++) v += B[r][k] * u[k];
    e[r] = v;
  }
}

/* TACSShellPressure::addResidual (TACSShellPressure.h:56-90) */
static void shell_pressure(const shell_geo *g, const double pres[4],
                           double res[24]) {
  for (int q = 0; q < 4; q++) {
    double pr = 0.0;
    for (int m = 0; m < 4; m++) pr += g->N[q][m] * pres[m];
    double f[3];
    for (int a = 0; a < 3; a++) f[a] = pr * -g->detXd[q] * g->n0[q][a];
    for (int m = 0; m < 4; m++)
      for (int a = 0; a < 3; a++) res[6 * m + a] += g->N[q][m] * f[a];
  }
}

/* TACSShellElement::addResidual (TACSShellElement.h:295-433), static case */
void or_shell_res(const double X[12], double t, const or_problem *p,
                  const double vars[24], const double pres[4],
                  double res[24]) {
  shell_geo g;
  shell_stiff c;
  shell_geometry(X, p, &g);
  shell_constitutive(p, t, &c);
  for (int q = 0; q < 4; q++) {
    double e[9], s[9];
    shell_strain(g.B[q], vars, e);
    shell_stress(&c, e, s);
    for (int k = 0; k < 24; k++) {
      double v = 0.0;
      for (int r = 0; r < 9; r++) v += g.B[q][r][k] * s[r];
      res[k] += g.detXd[q] * v;
    }
  }
  if (pres) shell_pressure(&g, pres, res);
}

/* TACSShellElement::addJacobian (TACSShellElement.h:436-641), alpha = 1,
   beta = gamma = 0: mat += sum_q detXd B^T C B; res += B^T s. */
void or_shell_jac(const double X[12], double t, const or_problem *p,
                  double res[24], const double vars[24], double mat[576]) {
  shell_geo g;
  shell_stiff c;
  shell_geometry(X, p, &g);
  shell_constitutive(p, t, &c);
  for (int q = 0; q < 4; q++) {
    double CB[9][24];
    for (int k = 0; k < 24; k++) {
      double e[9], s[9];
      for (int r = 0; r < 9; r++) e[r] = g.B[q][r][k];
      shell_stress(&c, e, s);
      for (int r = 0; r < 9; r++) CB[r][k] = s[r];
    }
    for (int i = 0; i < 24; i++)
      for (int j = 0; j < 24; j++) {
        double v = 0.0;
        for (int r = 0; r < 9; r++) v += g.B[q][r][i] * CB[r][j];
        mat[24 * i + j] += g.detXd[q] * v;
      }
    if (res && vars) {
      double e[9], s[9];
      shell_strain(g.B[q], vars, e);
      shell_stress(&c, e, s);
      for (int k = 0; k < 24; k++) {
        double v = 0.0;
        for (int r = 0; r < 9; r++) v += g.B[q][r][k] * s[r];
        res[k] += g.detXd[q] * v;
      }
    }
  }
}

/* ------------------------------ hex8 ----------------------------------- */
/* TACSLinearHexaBasis::computeBasis / computeBasisGradient
   (src/elements/basis/TACSHexaBasis.cpp:137-170) */
static void hex_shape(const double pt[3], double N[8], double Nxi[24]) {
  double x[2] = {1.0 - pt[0], 1.0 + pt[0]};
  double y[2] = {1.0 - pt[1], 1.0 + pt[1]};
  double z[2] = {1.0 - pt[2], 1.0 + pt[2]};
  double s[2] = {-1.0, 1.0};
  for (int k = 0; k < 2; k++)
    for (int j = 0; j < 2; j++)
      for (int i = 0; i < 2; i++) {
        int m = i + 2 * j + 4 * k;
        N[m] = 0.125 * x[i] * y[j] * z[k];
        Nxi[3 * m] = 0.125 * s[i] * y[j] * z[k];
        Nxi[3 * m + 1] = 0.125 * x[i] * s[j] * z[k];
        Nxi[3 * m + 2] = 0.125 * x[i] * y[j] * s[k];
      }
}

typedef struct {
  double Nx[8][24]; /* physical shape gradients dN_m/dx_j at each point */
  double detXd[8];
} hex_geo;

/* TACSElementBasis::getFieldGradient (TACSElementBasis.cpp:266-330) */
static void hex_geometry(const double X[24], hex_geo *g) {
  for (int q = 0; q < 8; q++) {
    double pt[3] = {gauss2[q % 2], gauss2[(q % 4) / 2], gauss2[q / 4]};
    double N[8], Nxi[24], Xd[9], J[9];
    hex_shape(pt, N, Nxi);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double v = 0.0;
        for (int m = 0; m < 8; m++) v += Nxi[3 * m + j] * X[3 * m + i];
        Xd[3 * i + j] = v;
      }
    g->detXd[q] = inv3(Xd, J);
    for (int m = 0; m < 8; m++)
      for (int j = 0; j < 3; j++)
        g->Nx[q][3 * m + j] = Nxi[3 * m] * J[j] + Nxi[3 * m + 1] * J[3 + j] +
                              Nxi[3 * m + 2] * J[6 + j];
  }
}
/* strain (TACSLinearElasticity3D::evalWeakIntegrand, linear branch,
   TACSLinearElasticity.cpp:890-900) */
static void hex_strain(const double Nx[24], const double *u, double e[6]) {
  double Ux[9] = {0};
  for (int m = 0; m < 8; m++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Ux[3 * i + j] += u[3 * m + i] * Nx[3 * m + j];
  e[0] = Ux[0];
  e[1] = Ux[4];
  e[2] = Ux[8];
  e[3] = Ux[5] + Ux[7];
  e[4] = Ux[2] + Ux[6];
  e[5] = Ux[1] + Ux[3];
}
/* C*e for the isotropic TACSMaterialProperties::evalTangentStiffness3D
   (TACSMaterialProperties.cpp:270-293) */
static void hex_Ce(const or_problem *p, const double e[6], double s[6]) {
  double D = p->E / ((1.0 + p->nu) * (1.0 - 2.0 * p->nu));
  double c0 = (1.0 - p->nu) * D, c1 = p->nu * D;
  double G = 0.5 * p->E / (1.0 + p->nu);
  s[0] = c0 * e[0] + c1 * e[1] + c1 * e[2];
  s[1] = c1 * e[0] + c0 * e[1] + c1 * e[2];
  s[2] = c1 * e[0] + c1 * e[1] + c0 * e[2];
  s[3] = G * e[3];
  s[4] = G * e[4];
  s[5] = G * e[5];
}
/* B^T s for one point, added with weight w */
static void hex_addBts(const double Nx[24], double w, const double s[6],
                       double *r) {
  for (int m = 0; m < 8; m++) {
    const double *g = &Nx[3 * m];
    r[3 * m + 0] += w * (g[0] * s[0] + g[1] * s[5] + g[2] * s[4]);
    r[3 * m + 1] += w * (g[1] * s[1] + g[0] * s[5] + g[2] * s[3]);
    r[3 * m + 2] += w * (g[2] * s[2] + g[1] * s[3] + g[0] * s[4]);
  }
}

/* TACSElement3D::addResidual (TACSElement3D.cpp:139-174) */
void or_hex_res(const double X[24], double t, const or_problem *p,
                const double vars[24], double res[24]) {
  hex_geo g;
  hex_geometry(X, &g);
  for (int q = 0; q < 8; q++) {
    double e[6], s[6];
    hex_strain(g.Nx[q], vars, e);
    hex_Ce(p, e, s);
    for (int i = 0; i < 6; i++) s[i] *= t;
    hex_addBts(g.Nx[q], g.detXd[q], s, res);
  }
}

/* TACSElement3D::addJacobian (TACSElement3D.cpp:176-225), alpha = 1 */
void or_hex_jac(const double X[24], double t, const or_problem *p,
                double mat[576]) {
  hex_geo g;
  hex_geometry(X, &g);
  for (int q = 0; q < 8; q++) {
    for (int j = 0; j < 24; j++) {
      double u[24] = {0}, e[6], s[6], col[24] = {0};
      u[j] = 1.0;
      hex_strain(g.Nx[q], u, e);
      hex_Ce(p, e, s);
      for (int i = 0; i < 6; i++) s[i] *= t;
      hex_addBts(g.Nx[q], g.detXd[q], s, col);
      for (int i = 0; i < 24; i++) mat[24 * i + j] += col[i];
    }
  }
}

/* TACSTraction3D::addResidual with tractionCoordinateComponent = 1
   (TACSTraction3D.cpp:87-125) and TACSElementBasis::getFaceNormal
   (TACSElementBasis.cpp:37-63) */
static void hex_traction(const double X[24], int face, const double tr[3],
                         double res[24]) {
  static const double tang[6][6] = {
      {0, 0, 1, 0, 1, 0}, {0, 1, 0, 0, 0, 1}, {1, 0, 0, 0, 0, 1},
      {0, 0, 1, 1, 0, 0}, {0, 1, 0, 1, 0, 0}, {1, 0, 0, 0, 1, 0}};
  for (int n = 0; n < 4; n++) {
    double pt[3];
    double a = gauss2[n % 2], b = gauss2[n / 2], c = -1.0 + 2.0 * (face % 2);
    if (face / 2 == 0) { pt[0] = c; pt[1] = a; pt[2] = b; }
    else if (face / 2 == 1) { pt[0] = a; pt[1] = c; pt[2] = b; }
    else { pt[0] = a; pt[1] = b; pt[2] = c; }
    double N[8], Nxi[24], Xd[9], t1[3], t2[3], nrm[3];
    hex_shape(pt, N, Nxi);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double v = 0.0;
        for (int m = 0; m < 8; m++) v += Nxi[3 * m + j] * X[3 * m + i];
        Xd[3 * i + j] = v;
      }
    for (int i = 0; i < 3; i++) {
      t1[i] = Xd[3 * i] * tang[face][0] + Xd[3 * i + 1] * tang[face][1] +
              Xd[3 * i + 2] * tang[face][2];
      t2[i] = Xd[3 * i] * tang[face][3] + Xd[3 * i + 1] * tang[face][4] +
              Xd[3 * i + 2] * tang[face][5];
    }
    cross3(t1, t2, nrm);
    double area = sqrt(dot3(nrm, nrm));
    for (int m = 0; m < 8; m++)
      for (int k = 0; k < 3; k++) res[3 * m + k] += area * N[m] * -tr[k];
  }
}

/* ----------------------------- gather helpers --------------------------- */
static int npe_of(const or_problem *p) { return p->elem_type == 0 ? 4 : 8; }
static int vpn_of(const or_problem *p) { return p->elem_type == 0 ? 6 : 3; }

static void gather(const or_problem *p, int e, const double *vec, int bs,
                   double *out) {
  int npe = npe_of(p);
  for (int m = 0; m < npe; m++) {
    int n = p->conn[npe * e + m];
    for (int k = 0; k < bs; k++) out[bs * m + k] = vec[(size_t)bs * n + k];
  }
}

/* Per-element load lookups (the reference keeps aux elements sorted by
   element number, TACSAuxElements::sort, TACSAuxElements.cpp:58). */
typedef struct {
  int *pres_of;  /* element -> index into pres arrays or -1 */
  int *trac_ptr; /* CSR over elements of traction entries */
  int *trac_idx;
} load_index;

static void build_load_index(const or_problem *p, load_index *L) {
  L->pres_of = (int *)malloc(sizeof(int) * (p->nelem ? p->nelem : 1));
  for (int e = 0; e < p->nelem; e++) L->pres_of[e] = -1;
  for (int k = 0; k < p->npres; k++) L->pres_of[p->pres_elems[k]] = k;
  L->trac_ptr = (int *)calloc(p->nelem + 1, sizeof(int));
  for (int k = 0; k < p->ntrac; k++) L->trac_ptr[p->trac_elems[k] + 1]++;
  for (int e = 0; e < p->nelem; e++) L->trac_ptr[e + 1] += L->trac_ptr[e];
  L->trac_idx = (int *)malloc(sizeof(int) * (p->ntrac ? p->ntrac : 1));
  int *fill = (int *)calloc(p->nelem + 1, sizeof(int));
  for (int k = 0; k < p->ntrac; k++) {
    int e = p->trac_elems[k];
    L->trac_idx[L->trac_ptr[e] + fill[e]++] = k;
  }
  free(fill);
}
static void free_load_index(load_index *L) {
  free(L->pres_of);
  free(L->trac_ptr);
  free(L->trac_idx);
}

/* Element residual including its aux loads scaled by lambda
   (TACSAssembler::assembleRes, TACSAssembler.cpp:4176-4225), at element
   coordinates X and element variables u. */
static void elem_residual_at(const or_problem *p, const load_index *L, int e,
                             const double *X, const double *u, double lambda,
                             double *res) {
  memset(res, 0, 24 * sizeof(double));
  double t = p->thick[e];
  double aux[24];
  memset(aux, 0, sizeof(aux));
  if (p->elem_type == 0) {
    or_shell_res(X, t, p, u, NULL, res);
    if (L->pres_of[e] >= 0) {
      shell_geo g;
      shell_geometry(X, p, &g);
      shell_pressure(&g, &p->pres_vals[4 * L->pres_of[e]], aux);
    }
  } else {
    or_hex_res(X, t, p, u, res);
    for (int k = L->trac_ptr[e]; k < L->trac_ptr[e + 1]; k++) {
      int j = L->trac_idx[k];
      hex_traction(X, p->trac_faces[j], &p->trac_vals[3 * j], aux);
    }
  }
  for (int k = 0; k < 24; k++) res[k] += lambda * aux[k];
}
static void elem_residual(const or_problem *p, const load_index *L, int e,
                          const double *vars, double lambda, double *res) {
  double X[24], u[24];
  gather(p, e, p->xpts, 3, X);
  gather(p, e, vars, vpn_of(p), u);
  elem_residual_at(p, L, e, X, u, lambda, res);
}

/* ------------------------------ threading ------------------------------ */
typedef void (*range_fn)(void *ctx, int begin, int end, int tid);
typedef struct {
  range_fn fn;
  void *ctx;
  int begin, end, tid;
} range_job;
static void *range_run(void *arg) {
  range_job *j = (range_job *)arg;
  j->fn(j->ctx, j->begin, j->end, j->tid);
  return NULL;
}
static void parallel_for(int n, int nthreads, range_fn fn, void *ctx) {
  if (nthreads <= 1 || n < 2 * nthreads) {
    fn(ctx, 0, n, 0);
    return;
  }
  pthread_t th[64];
  range_job jobs[64];
  if (nthreads > 64) nthreads = 64;
  for (int i = 0; i < nthreads; i++) {
    jobs[i].fn = fn;
    jobs[i].ctx = ctx;
    jobs[i].begin = (int)((long long)n * i / nthreads);
    jobs[i].end = (int)((long long)n * (i + 1) / nthreads);
    jobs[i].tid = i;
    pthread_create(&th[i], NULL, range_run, &jobs[i]);
  }
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
}

/* ------------------------------ assembly ------------------------------- */
typedef struct {
  const or_problem *p;
  const load_index *L;
  const double *vars;
  double lambda;
  double *res;
  or_bcsr *A;
  int transpose;
  pthread_mutex_t *lock;
} asm_ctx;

static void res_range(void *vctx, int b, int e_end, int tid) {
  asm_ctx *c = (asm_ctx *)vctx;
  const or_problem *p = c->p;
  int npe = npe_of(p), vpn = vpn_of(p);
  double r[24];
  (void)tid;
  for (int e = b; e < e_end; e++) {
    elem_residual(p, c->L, e, c->vars, c->lambda, r);
    /* scatter under one lock, as TACSAssembler_thread.cpp:134-136 */
    if (c->lock) pthread_mutex_lock(c->lock);
    for (int m = 0; m < npe; m++) {
      int n = p->conn[npe * e + m];
      for (int k = 0; k < vpn; k++) c->res[(size_t)vpn * n + k] += r[vpn * m + k];
    }
    if (c->lock) pthread_mutex_unlock(c->lock);
  }
}

void or_apply_bcs_vec(const or_problem *p, double *x) {
  int vpn = vpn_of(p);
  for (int i = 0; i < p->nbcs; i++)
    for (int k = 0; k < vpn; k++)
      if (p->bc_masks[i] & (1 << k)) x[(size_t)vpn * p->bc_nodes[i] + k] = 0.0;
}

/* TACSBVec::applyBCs with the state vector (TACSBVec.cpp:546-600):
   res = u - lambda * 0 on constrained dofs */
static void apply_bcs_res(const or_problem *p, const double *vars,
                          double *res) {
  int vpn = vpn_of(p);
  for (int i = 0; i < p->nbcs; i++)
    for (int k = 0; k < vpn; k++)
      if (p->bc_masks[i] & (1 << k)) {
        size_t d = (size_t)vpn * p->bc_nodes[i] + k;
        res[d] = vars ? vars[d] : 0.0;
      }
}

/* TACSAssembler::assembleRes (TACSAssembler.cpp:4133-4256) */
void or_assemble_res(const or_problem *p, const double *vars, double lambda,
                     int apply_bcs, double *res) {
  load_index L;
  build_load_index(p, &L);
  memset(res, 0, sizeof(double) * (size_t)p->nnodes * vpn_of(p));
  pthread_mutex_t lock = PTHREAD_MUTEX_INITIALIZER;
  asm_ctx c = {p, &L, vars, lambda, res, NULL, 0,
               p->nthreads > 1 ? &lock : NULL};
  parallel_for(p->nelem, p->nthreads, res_range, &c);
  if (apply_bcs) apply_bcs_res(p, vars, res);
  free_load_index(&L);
}

/* BCSR non-zero pattern: the node-to-node graph of the connectivity with
   the diagonal, columns sorted (TACSAssembler::createMat ->
   computeLocalNodeToNodeCSR, TACSAssembler.cpp:3384) */
static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}
int or_bcsr_create(const or_problem *p, or_bcsr *A) {
  int nn = p->nnodes, npe = npe_of(p);
  int *cnt = (int *)calloc(nn + 1, sizeof(int));
  for (int e = 0; e < p->nelem; e++)
    for (int m = 0; m < npe; m++) cnt[p->conn[npe * e + m] + 1] += npe;
  for (int i = 0; i < nn; i++) cnt[i + 1] += cnt[i] + 1;
  int *tmp = (int *)malloc(sizeof(int) * cnt[nn]);
  int *fill = (int *)calloc(nn, sizeof(int));
  for (int i = 0; i < nn; i++) tmp[cnt[i] + fill[i]++] = i;
  for (int e = 0; e < p->nelem; e++)
    for (int m = 0; m < npe; m++) {
      int r = p->conn[npe * e + m];
      for (int k = 0; k < npe; k++) tmp[cnt[r] + fill[r]++] = p->conn[npe * e + k];
    }
  A->bsize = vpn_of(p);
  A->nrows = nn;
  A->rowp = (int *)malloc(sizeof(int) * (nn + 1));
  A->rowp[0] = 0;
  int nnz = 0;
  for (int i = 0; i < nn; i++) {
    int *r = &tmp[cnt[i]];
    int len = fill[i];
    qsort(r, len, sizeof(int), cmp_int);
    int u = 0;
    for (int k = 0; k < len; k++)
      if (u == 0 || r[k] != r[u - 1]) r[u++] = r[k];
    fill[i] = u;
    nnz += u;
    A->rowp[i + 1] = nnz;
  }
  A->cols = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
  A->diag = (int *)malloc(sizeof(int) * (nn ? nn : 1));
  for (int i = 0; i < nn; i++) {
    memcpy(&A->cols[A->rowp[i]], &tmp[cnt[i]], sizeof(int) * fill[i]);
    for (int j = A->rowp[i]; j < A->rowp[i + 1]; j++)
      if (A->cols[j] == i) A->diag[i] = j;
  }
  size_t b2 = (size_t)A->bsize * A->bsize;
  A->vals = (double *)calloc((size_t)nnz * b2 + 1, sizeof(double));
  free(tmp);
  free(fill);
  free(cnt);
  return 0;
}
void or_bcsr_free(or_bcsr *A) {
  free(A->rowp);
  free(A->cols);
  free(A->diag);
  free(A->vals);
  memset(A, 0, sizeof(*A));
}
static int find_col(const or_bcsr *A, int row, int col) {
  int lo = A->rowp[row], hi = A->rowp[row + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) / 2;
    if (A->cols[mid] == col) return mid;
    if (A->cols[mid] < col) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

static void jac_range(void *vctx, int b, int e_end, int tid) {
  asm_ctx *c = (asm_ctx *)vctx;
  const or_problem *p = c->p;
  int npe = npe_of(p), vpn = vpn_of(p), nv = npe * vpn;
  double mat[576], r[24], X[24], u[24];
  (void)tid;
  for (int e = b; e < e_end; e++) {
    gather(p, e, p->xpts, 3, X);
    gather(p, e, c->vars, vpn, u);
    memset(mat, 0, sizeof(mat));
    if (p->elem_type == 0) {
      or_shell_jac(X, p->thick[e], p, NULL, NULL, mat);
    } else {
      or_hex_jac(X, p->thick[e], p, mat);
    }
    if (c->res) elem_residual(p, c->L, e, c->vars, 1.0, r);
    if (c->lock) pthread_mutex_lock(c->lock);
    if (c->res)
      for (int m = 0; m < npe; m++) {
        int n = p->conn[npe * e + m];
        for (int k = 0; k < vpn; k++)
          c->res[(size_t)vpn * n + k] += r[vpn * m + k];
      }
    /* BCSRMat::addRowValues / addRowWeightValues (BCSRMat.cpp:1800,1879) */
    for (int i = 0; i < npe; i++) {
      int row = p->conn[npe * e + i];
      for (int j = 0; j < npe; j++) {
        int col = p->conn[npe * e + j];
        int slot = find_col(c->A, row, col);
        double *a = &c->A->vals[(size_t)slot * vpn * vpn];
        for (int ii = 0; ii < vpn; ii++)
          for (int jj = 0; jj < vpn; jj++) {
            double v = c->transpose ? mat[nv * (vpn * j + jj) + vpn * i + ii]
                                    : mat[nv * (vpn * i + ii) + vpn * j + jj];
            a[vpn * ii + jj] += v;
          }
      }
    }
    if (c->lock) pthread_mutex_unlock(c->lock);
  }
}

/* BCSRMat::zeroRow with ident = 1 (BCSRMat.cpp:2027-2050) */
static void bcsr_apply_bcs(const or_problem *p, or_bcsr *A) {
  int bs = A->bsize;
  for (int i = 0; i < p->nbcs; i++) {
    int row = p->bc_nodes[i], vars = p->bc_masks[i];
    for (int j = A->rowp[row]; j < A->rowp[row + 1]; j++) {
      double *a = &A->vals[(size_t)bs * bs * j];
      for (int ii = 0; ii < bs; ii++)
        if (vars & (1 << ii))
          for (int jj = 0; jj < bs; jj++) a[bs * ii + jj] = 0.0;
      if (A->cols[j] == row)
        for (int ii = 0; ii < bs; ii++)
          if (vars & (1 << ii)) a[(bs + 1) * ii] = 1.0;
    }
  }
}

/* TACSAssembler::assembleJacobian (TACSAssembler.cpp:4291-4405) */
void or_assemble_jac(const or_problem *p, const double *vars, double *res,
                     or_bcsr *A, int transpose, int apply_bcs) {
  load_index L;
  build_load_index(p, &L);
  size_t n = (size_t)p->nnodes * vpn_of(p);
  if (res) memset(res, 0, sizeof(double) * n);
  memset(A->vals, 0,
         sizeof(double) * (size_t)A->rowp[A->nrows] * A->bsize * A->bsize);
  pthread_mutex_t lock = PTHREAD_MUTEX_INITIALIZER;
  asm_ctx c = {p, &L, vars, 1.0, res, A, transpose,
               p->nthreads > 1 ? &lock : NULL};
  parallel_for(p->nelem, p->nthreads, jac_range, &c);
  if (apply_bcs) {
    if (res) apply_bcs_res(p, vars, res);
    bcsr_apply_bcs(p, A);
  }
  free_load_index(&L);
}

/* --------------------------- linear algebra ---------------------------- */
typedef struct {
  const or_bcsr *A;
  const double *x;
  double *y;
} mult_ctx;
static void mult_range(void *vctx, int b, int e, int tid) {
  mult_ctx *c = (mult_ctx *)vctx;
  const or_bcsr *A = c->A;
  int bs = A->bsize;
  (void)tid;
  for (int i = b; i < e; i++) {
    double acc[8] = {0};
    for (int j = A->rowp[i]; j < A->rowp[i + 1]; j++) {
      const double *a = &A->vals[(size_t)bs * bs * j];
      const double *xx = &c->x[(size_t)bs * A->cols[j]];
      for (int ii = 0; ii < bs; ii++) {
        double s = 0.0;
        for (int jj = 0; jj < bs; jj++) s += a[bs * ii + jj] * xx[jj];
        acc[ii] += s;
      }
    }
    for (int ii = 0; ii < bs; ii++) c->y[(size_t)bs * i + ii] = acc[ii];
  }
}
/* BCSRMatVecMult6 / BCSRMatVecMult3 (BCSRMatMult6.cpp:82, Mult3.cpp:28) */
void or_bcsr_mult(const or_bcsr *A, const double *x, double *y, int nthreads) {
  mult_ctx c = {A, x, y};
  parallel_for(A->nrows, nthreads, mult_range, &c);
}

/* BMatComputeInverse (BCSRMatMult.cpp:308-390): partial-pivot LU of the
   row-major block then explicit inverse. */
static int block_inverse(double *Ainv, double *A, int n) {
  int ipiv[8];
  for (int k = 0; k < n - 1; k++) {
    int nk = n * k, r = k;
    double maxv = fabs(A[nk + k]);
    for (int j = k + 1; j < n; j++) {
      double t = fabs(A[n * j + k]);
      if (t > maxv) {
        maxv = t;
        r = j;
      }
    }
    ipiv[k] = r;
    if (r != k)
      for (int j = 0; j < n; j++) {
        double t = A[nk + j];
        A[nk + j] = A[n * r + j];
        A[n * r + j] = t;
      }
    if (A[nk + k] == 0.0) return k + 1;
    for (int i = k + 1; i < n; i++) A[n * i + k] = A[n * i + k] / A[nk + k];
    for (int i = k + 1; i < n; i++)
      for (int j = k + 1; j < n; j++) A[n * i + j] -= A[n * i + k] * A[nk + j];
  }
  /* Column k of the inverse: locate the permuted unit entry, then forward
     (unit lower) and backward substitution (BCSRMatMult.cpp:353-386). */
  for (int k = 0; k < n; k++) {
    int ip = k;
    for (int i = 0; i < n - 1; i++) {
      if (ip == ipiv[i]) ip = i;
      else if (ip == i) ip = ipiv[i];
    }
    for (int i = 0; i < ip; i++) Ainv[n * i + k] = 0.0;
    Ainv[n * ip + k] = 1.0;
    for (int i = ip + 1; i < n; i++) {
      Ainv[n * i + k] = 0.0;
      for (int j = ip; j < i; j++) Ainv[n * i + k] -= A[n * i + j] * Ainv[n * j + k];
    }
    for (int i = n - 1; i >= 0; i--) {
      for (int j = i + 1; j < n; j++) Ainv[n * i + k] -= A[n * i + j] * Ainv[n * j + k];
      Ainv[n * i + k] = Ainv[n * i + k] / A[n * i + i];
    }
  }
  return 0;
}

/* Block ILU(0) in place on a copy of A: BCSRMatFactor6/3
   (BCSRMatFact6.cpp:946-1330, BCSRMatFact3.cpp:30-146).  Off-diagonal
   lower blocks become L_ij = A_ij D_j^{-1}, the stored diagonal blocks are
   the inverses D_i^{-1}. */
static int ilu_numeric(or_bcsr *F);

int or_ilu0_factor(const or_bcsr *A, or_bcsr *F) {
  int bs = A->bsize, n = A->nrows;
  size_t b2 = (size_t)bs * bs, nnz = A->rowp[n];
  if (!F->rowp) {
    F->bsize = bs;
    F->nrows = n;
    F->rowp = (int *)malloc(sizeof(int) * (n + 1));
    F->cols = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
    F->diag = (int *)malloc(sizeof(int) * (n ? n : 1));
    F->vals = (double *)malloc(sizeof(double) * (nnz * b2 + 1));
    memcpy(F->rowp, A->rowp, sizeof(int) * (n + 1));
    memcpy(F->cols, A->cols, sizeof(int) * nnz);
    memcpy(F->diag, A->diag, sizeof(int) * n);
  }
  memcpy(F->vals, A->vals, sizeof(double) * nnz * b2);
  return ilu_numeric(F);
}

/* Numeric block ILU in F's own pattern (IKJ: row i's lower blocks become
   L_ij = A_ij D_j^{-1} and update the blocks of row i that row j's upper
   part reaches; the diagonal blocks end as D_i^{-1}), BCSRMatFactor6 /
   BCSRMatFactor3 (BCSRMatFact6.cpp:946-1330, BCSRMatFact3.cpp:30-146). */
static int ilu_numeric(or_bcsr *F) {
  const int bs = F->bsize, n = F->nrows;
  const size_t b2 = (size_t)bs * bs;
  const int *rowp = F->rowp, *cols = F->cols, *diag = F->diag;
  double *V = F->vals;
  double d[64], D[64];
  int fail = 0;
  for (int i = 0; i < n; i++) {
    int row_end = rowp[i + 1];
    for (int j = rowp[i]; cols[j] < i; j++) {
      int cj = cols[j];
      double *a = &V[b2 * j];
      const double *b = &V[b2 * diag[cj]];
      for (int r = 0; r < bs; r++)
        for (int c = 0; c < bs; c++) {
          double s = 0.0;
          for (int k = 0; k < bs; k++) s += a[bs * r + k] * b[bs * k + c];
          d[bs * r + c] = s;
        }
      int k = j + 1, pp = diag[cj] + 1, end = rowp[cj + 1];
      for (; pp < end && k < row_end; pp++) {
        while (k < row_end && cols[k] < cols[pp]) k++;
        if (k < row_end && cols[k] == cols[pp]) {
          double *ak = &V[b2 * k];
          const double *bp = &V[b2 * pp];
          for (int r = 0; r < bs; r++)
            for (int c = 0; c < bs; c++) {
              double s = 0.0;
              for (int q = 0; q < bs; q++) s += d[bs * r + q] * bp[bs * q + c];
              ak[bs * r + c] -= s;
            }
        }
      }
      memcpy(a, d, sizeof(double) * b2);
    }
    double *a = &V[b2 * diag[i]];
    memcpy(D, a, sizeof(double) * b2);
    int info = block_inverse(a, D, bs);
    if (info > 0 && !fail) fail = i + 1;
  }
  return fail;
}

/* ILU(k) pattern (BCSRMat::computeILUk, BCSRMat.cpp:625-730): within row
   i, every entry (i, c) left of the diagonal, taken in increasing c, meets
   the upper entries (c, j) of the finished row c; (i, j) gets level
   lev(i, c) + lev(c, j) + 1 if smaller than its current level, or is
   inserted (row kept sorted) if new and at most lev_fill.  A's entries
   have level 0 and the diagonal is always present. */
static void iluk_symbolic(const or_bcsr *A, int lev_fill, or_bcsr *F,
                          int **levs_out) {
  const int n = A->nrows;
  size_t cap = (size_t)A->rowp[n] * 2 + n + 16, size = 0;
  int *cols = (int *)malloc(sizeof(int) * cap);
  int *levs = (int *)malloc(sizeof(int) * cap);
  int *rowp = (int *)malloc(sizeof(int) * (n + 1));
  int *diag = (int *)malloc(sizeof(int) * (n ? n : 1));
  int *rc = (int *)malloc(sizeof(int) * (n + 1));
  int *rl = (int *)malloc(sizeof(int) * (n + 1));
  rowp[0] = 0;
  for (int i = 0; i < n; i++) {
    int nr = 0, has_diag = 0;
    for (int j = A->rowp[i]; j < A->rowp[i + 1]; j++) {
      if (A->cols[j] == i) has_diag = 1;
      rc[nr] = A->cols[j];
      rl[nr++] = 0;
    }
    if (!has_diag) {
      int p = 0;
      while (p < nr && rc[p] < i) p++;
      for (int m = nr; m > p; m--) {
        rc[m] = rc[m - 1];
        rl[m] = rl[m - 1];
      }
      rc[p] = i;
      rl[p] = 0;
      nr++;
    }
    for (int j = 0; j < nr && rc[j] < i; j++) {
      const int c = rc[j], lc = rl[j];
      int p = j + 1;
      for (int q = diag[c] + 1; q < rowp[c + 1]; q++) {
        const int col = cols[q], lev = lc + levs[q] + 1;
        while (p < nr && rc[p] < col) p++;
        if (p < nr && rc[p] == col) {
          if (lev < rl[p]) rl[p] = lev;
        } else if (lev <= lev_fill) {
          for (int m = nr; m > p; m--) {
            rc[m] = rc[m - 1];
            rl[m] = rl[m - 1];
          }
          rc[p] = col;
          rl[p] = lev;
          nr++;
        }
      }
    }
    if (size + nr > cap) {
      cap = 2 * (size + nr);
      cols = (int *)realloc(cols, sizeof(int) * cap);
      levs = (int *)realloc(levs, sizeof(int) * cap);
    }
    for (int k = 0; k < nr; k++) {
      if (rc[k] == i) diag[i] = (int)size;
      cols[size] = rc[k];
      levs[size++] = rl[k];
    }
    rowp[i + 1] = (int)size;
  }
  free(rc);
  free(rl);
  F->bsize = A->bsize;
  F->nrows = n;
  F->rowp = rowp;
  F->cols = cols;
  F->diag = diag;
  F->vals = (double *)malloc(sizeof(double) *
                             (size * (size_t)A->bsize * A->bsize + 1));
  if (levs_out) *levs_out = levs;
  else free(levs);
}

/* TACSAdditiveSchwarz(mat, levFill, fill) + factor: ILU(lev_fill) of A.
   F is built on the first call (F->rowp == NULL) and refactored after. */
int or_iluk_factor(const or_bcsr *A, int lev_fill, or_bcsr *F) {
  if (!F->rowp) iluk_symbolic(A, lev_fill, F, NULL);
  const int n = A->nrows;
  const size_t b2 = (size_t)A->bsize * A->bsize;
  memset(F->vals, 0, sizeof(double) * F->rowp[n] * b2);
  for (int i = 0; i < n; i++) {
    int f = F->rowp[i];
    for (int j = A->rowp[i]; j < A->rowp[i + 1]; j++) {
      while (F->cols[f] < A->cols[j]) f++;
      memcpy(&F->vals[b2 * f], &A->vals[b2 * j], sizeof(double) * b2);
    }
  }
  return ilu_numeric(F);
}

/* BCSRMatApplyLower / BCSRMatApplyUpper (BCSRMatMult6.cpp:319-415) */
void or_ilu0_apply(const or_bcsr *F, const double *x, double *y) {
  int bs = F->bsize, n = F->nrows;
  size_t b2 = (size_t)bs * bs;
  double z[8];
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < bs; k++) z[k] = x[(size_t)bs * i + k];
    for (int j = F->rowp[i]; F->cols[j] < i; j++) {
      const double *a = &F->vals[b2 * j];
      const double *yy = &y[(size_t)bs * F->cols[j]];
      for (int r = 0; r < bs; r++) {
        double s = 0.0;
        for (int c = 0; c < bs; c++) s += a[bs * r + c] * yy[c];
        z[r] -= s;
      }
    }
    for (int k = 0; k < bs; k++) y[(size_t)bs * i + k] = z[k];
  }
  for (int i = n - 1; i >= 0; i--) {
    for (int k = 0; k < bs; k++) z[k] = y[(size_t)bs * i + k];
    for (int j = F->diag[i] + 1; j < F->rowp[i + 1]; j++) {
      const double *a = &F->vals[b2 * j];
      const double *yy = &y[(size_t)bs * F->cols[j]];
      for (int r = 0; r < bs; r++) {
        double s = 0.0;
        for (int c = 0; c < bs; c++) s += a[bs * r + c] * yy[c];
        z[r] -= s;
      }
    }
    const double *dinv = &F->vals[b2 * F->diag[i]];
    for (int r = 0; r < bs; r++) {
      double s = 0.0;
      for (int c = 0; c < bs; c++) s += dinv[bs * r + c] * z[c];
      y[(size_t)bs * i + r] = s;
    }
  }
}

static double vdot(const double *a, const double *b, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* GMRES::solve, right preconditioned, MGS, Givens rotations, convergence
   on the estimated residual relative to the first cycle's initial residual
   (src/bpmat/KSM.cpp:785-970). */
int or_gmres(const or_bcsr *A, const or_bcsr *F, const double *b, double *x,
             int m, int nrestart, double rtol, double atol, int *iters,
             int nthreads) {
  size_t n = (size_t)A->nrows * A->bsize;
  double *W = (double *)malloc(sizeof(double) * n * (m + 1));
  double *work = (double *)malloc(sizeof(double) * n);
  double *H = (double *)calloc((size_t)(m + 1) * m, sizeof(double));
  double *res = (double *)calloc(m + 1, sizeof(double));
  double *Qc = (double *)calloc(m, sizeof(double));
  double *Qs = (double *)calloc(m, sizeof(double));
  double rhs_norm = 0.0;
  int flag = 0, total = 0;
  for (int count = 0; count < nrestart + 1; count++) {
    if (count == 0) {
      memset(x, 0, sizeof(double) * n);
      memcpy(W, b, sizeof(double) * n);
      res[0] = sqrt(vdot(W, W, n));
      double s = 1.0 / res[0];
      for (size_t i = 0; i < n; i++) W[i] *= s;
    } else {
      or_bcsr_mult(A, x, W, nthreads);
      for (size_t i = 0; i < n; i++) W[i] -= b[i];
      res[0] = sqrt(vdot(W, W, n));
      double s = -1.0 / res[0];
      for (size_t i = 0; i < n; i++) W[i] *= s;
    }
    if (count == 0) rhs_norm = res[0];
    int niters = 0;
    if (res[0] < atol) {
      flag = 1;
      break;
    }
    for (int i = 0; i < m; i++) {
      double *Wi = &W[n * i], *Wn = &W[n * (i + 1)];
      or_ilu0_apply(F, Wi, work);
      or_bcsr_mult(A, work, Wn, nthreads);
      /* ModifiedGramSchmidt (KSM.cpp:526-533) */
      for (int k = 0; k <= i; k++) {
        double h = vdot(Wn, &W[n * k], n);
        H[(size_t)(m + 1) * i + k] = h;
        for (size_t r = 0; r < n; r++) Wn[r] -= h * W[n * k + r];
      }
      double *Hc = &H[(size_t)(m + 1) * i];
      Hc[i + 1] = sqrt(vdot(Wn, Wn, n));
      double s = 1.0 / Hc[i + 1];
      for (size_t r = 0; r < n; r++) Wn[r] *= s;
      for (int k = 0; k < i; k++) {
        double h1 = Hc[k], h2 = Hc[k + 1];
        Hc[k] = h1 * Qc[k] + h2 * Qs[k];
        Hc[k + 1] = -h1 * Qs[k] + h2 * Qc[k];
      }
      double h1 = Hc[i], h2 = Hc[i + 1];
      double sq = sqrt(h1 * h1 + h2 * h2);
      Qc[i] = h1 / sq;
      Qs[i] = h2 / sq;
      Hc[i] = h1 * Qc[i] + h2 * Qs[i];
      Hc[i + 1] = -h1 * Qs[i] + h2 * Qc[i];
      h1 = res[i];
      res[i] = h1 * Qc[i];
      res[i + 1] = -h1 * Qs[i];
      niters++;
      double rn = fabs(res[i + 1]);
      if (rn < atol || rn < rtol * rhs_norm) {
        flag = 1;
        break;
      }
    }
    total += niters;
    for (int i = niters - 1; i >= 0; i--) {
      for (int j = i + 1; j < niters; j++)
        res[i] = res[i] - H[(size_t)(m + 1) * j + i] * res[j];
      res[i] = res[i] / H[(size_t)(m + 1) * i + i];
    }
    memset(work, 0, sizeof(double) * n);
    for (int i = 0; i < niters; i++)
      for (size_t r = 0; r < n; r++) work[r] += res[i] * W[n * i + r];
    or_ilu0_apply(F, work, W);
    for (size_t r = 0; r < n; r++) x[r] += W[r];
    if (flag) break;
  }
  if (iters) *iters = total;
  free(W);
  free(work);
  free(H);
  free(res);
  free(Qc);
  free(Qs);
  return flag;
}

/* ----------------------------- functions ------------------------------- */
/* Per-point strain with the drilling strain excluded (evalPointQuantity
   sets e[8] = 0, TACSShellElement.h:1063). */
typedef struct {
  int nq;
  double e[8][9];
  double detXd[8];
  double B[8][9][24]; /* shells only (hex uses Nx) */
  double Nx[8][24];
} elem_points;

static void elem_points_eval(const or_problem *p, int el, const double *vars,
                             elem_points *ep) {
  double X[24], u[24];
  gather(p, el, p->xpts, 3, X);
  gather(p, el, vars, vpn_of(p), u);
  if (p->elem_type == 0) {
    shell_geo g;
    shell_geometry(X, p, &g);
    ep->nq = 4;
    for (int q = 0; q < 4; q++) {
      shell_strain(g.B[q], u, ep->e[q]);
      ep->e[q][8] = 0.0;
      ep->detXd[q] = g.detXd[q];
      memcpy(ep->B[q], g.B[q], sizeof(g.B[q]));
    }
  } else {
    hex_geo g;
    hex_geometry(X, &g);
    ep->nq = 8;
    for (int q = 0; q < 8; q++) {
      hex_strain(g.Nx[q], u, ep->e[q]);
      ep->detXd[q] = g.detXd[q];
      memcpy(ep->Nx[q], g.Nx[q], sizeof(g.Nx[q]));
    }
  }
}

/* TACSMaterialProperties::vonMisesFailure2D / 2DStressSens
   (TACSMaterialProperties.cpp:481-500) */
static double vm2(const or_problem *p, const double s[3], double sens[3]) {
  double f = sqrt(s[0] * s[0] + s[1] * s[1] - s[0] * s[1] + 3.0 * s[2] * s[2]);
  if (sens) {
    if (f != 0.0) {
      sens[0] = (s[0] - 0.5 * s[1]) / (f * p->ys);
      sens[1] = (s[1] - 0.5 * s[0]) / (f * p->ys);
      sens[2] = (3.0 * s[2]) / (f * p->ys);
    } else {
      sens[0] = sens[1] = sens[2] = 0.0;
    }
  }
  return f / p->ys;
}
/* TACSMaterialProperties::vonMisesFailure3D / 3DStressSens (.cpp:439-470) */
static double vm3(const or_problem *p, const double s[6], double sens[6]) {
  double f = sqrt(0.5 * ((s[0] - s[1]) * (s[0] - s[1]) +
                         (s[0] - s[2]) * (s[0] - s[2]) +
                         (s[1] - s[2]) * (s[1] - s[2]) +
                         6.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5])));
  if (sens) {
    if (f != 0.0) {
      double fact = 0.5 / (p->ys * f);
      sens[0] = fact * (2.0 * s[0] - s[1] - s[2]);
      sens[1] = fact * (2.0 * s[1] - s[0] - s[2]);
      sens[2] = fact * (2.0 * s[2] - s[0] - s[1]);
      sens[3] = 6.0 * fact * s[3];
      sens[4] = 6.0 * fact * s[4];
      sens[5] = 6.0 * fact * s[5];
    } else {
      for (int i = 0; i < 6; i++) sens[i] = 0.0;
    }
  }
  return f / p->ys;
}

/* Failure index at a point and its strain gradient dfde (shell:
   TACSIsoShellConstitutive::evalFailure / evalFailureStrainSens with the
   internal top/bottom KS weight 100, TACSIsoShellConstitutive.cpp:254-395;
   solid: TACSSolidConstitutive::evalFailure, .cpp:274-330).  For shells,
   dfdt_e (the design sensitivity at fixed strain, addFailureDVSens
   .cpp:397-436) is returned through dfdt. */
static double point_failure(const or_problem *p, double t, const double *e,
                            double *dfde, double *dfdt) {
  if (p->elem_type == 0) {
    double A0[6];
    double Dm = p->E / (1.0 - p->nu * p->nu);
    A0[0] = Dm; A0[1] = p->nu * Dm; A0[2] = 0.0; A0[3] = Dm; A0[4] = 0.0;
    A0[5] = 0.5 * p->E / (1.0 + p->nu);
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
    double pt[3], pb[3];
    double top = vm2(p, st, pt), bot = vm2(p, sb, pb);
    double mx = (top > bot) ? top : bot;
    const double ksw = 100.0;
    double ksum = exp(ksw * (top - mx)) + exp(ksw * (bot - mx));
    double val = mx + log(ksum) / ksw;
    double ft = exp(ksw * (top - mx)) / ksum;
    double fb = exp(ksw * (bot - mx)) / ksum;
    double phit[3], phib[3];
    phit[0] = A0[0] * pt[0] + A0[1] * pt[1] + A0[2] * pt[2];
    phit[1] = A0[1] * pt[0] + A0[3] * pt[1] + A0[4] * pt[2];
    phit[2] = A0[2] * pt[0] + A0[4] * pt[1] + A0[5] * pt[2];
    phib[0] = A0[0] * pb[0] + A0[1] * pb[1] + A0[2] * pb[2];
    phib[1] = A0[1] * pb[0] + A0[3] * pb[1] + A0[4] * pb[2];
    phib[2] = A0[2] * pb[0] + A0[4] * pb[1] + A0[5] * pb[2];
    if (dfde) {
      for (int i = 0; i < 3; i++) {
        dfde[i] = ft * phit[i] + fb * phib[i];
        dfde[3 + i] = ft * ht * phit[i] + fb * hb * phib[i];
      }
      dfde[6] = dfde[7] = dfde[8] = 0.0;
    }
    if (dfdt) {
      *dfdt = ft * 0.5 * (phit[0] * e[3] + phit[1] * e[4] + phit[2] * e[5]) +
              fb * -(0.5) * (phib[0] * e[3] + phib[1] * e[4] + phib[2] * e[5]);
    }
    return val;
  } else {
    double s[6], sens[6];
    hex_Ce(p, e, s);
    double f = vm3(p, s, sens);
    if (dfde) hex_Ce(p, sens, dfde);
    if (dfdt) *dfdt = 0.0;
    return f;
  }
}

/* Strain energy density e.s (TACSShellElement::evalPointQuantity,
   .h:1065-1072; TACSLinearElasticity3D::evalPointQuantity, .cpp:1975) and
   s = C e (the stress, whose double is d(e.s)/de). */
static double point_sed(const or_problem *p, double t, const double *e,
                        double *s) {
  double sl[9];
  if (!s) s = sl;
  if (p->elem_type == 0) {
    shell_stiff c;
    shell_constitutive(p, t, &c);
    shell_stress(&c, e, s);
    double v = 0.0;
    for (int i = 0; i < 9; i++) v += e[i] * s[i];
    return v;
  }
  hex_Ce(p, e, s);
  for (int i = 0; i < 6; i++) s[i] *= t;
  double v = 0.0;
  for (int i = 0; i < 6; i++) v += e[i] * s[i];
  return v;
}

/* d(stress . psi)/dt at strain e: TACSIsoShellConstitutive::addStressDVSens
   (.cpp:229-252) with tOffset = 0 / TACSSolidConstitutive::addStressDVSens
   (.cpp:181-209). */
static double stress_dv(const or_problem *p, double t, const double *e,
                        const double *psi) {
  if (p->elem_type == 0) {
    double Dm = p->E / (1.0 - p->nu * p->nu), G = 0.5 * p->E / (1.0 + p->nu);
    double A[6] = {Dm, p->nu * Dm, 0.0, Dm, 0.0, G};
#define SYMIN(x, y)                                                     \
  ((x)[0] * (A[0] * (y)[0] + A[1] * (y)[1] + A[2] * (y)[2]) +          \
   (x)[1] * (A[1] * (y)[0] + A[3] * (y)[1] + A[4] * (y)[2]) +          \
   (x)[2] * (A[2] * (y)[0] + A[4] * (y)[1] + A[5] * (y)[2]))
    double dI = 0.25 * t * t;
    double kcorr = 5.0 / 6.0;
    return SYMIN(psi, e) + dI * SYMIN(psi + 3, e + 3) +
           kcorr * A[5] * (psi[6] * e[6] + psi[7] * e[7] + 0.1 * psi[8] * e[8]);
#undef SYMIN
  }
  double s[6];
  hex_Ce(p, e, s);
  return s[0] * psi[0] + s[1] * psi[1] + s[2] * psi[2] + s[3] * psi[3] +
         s[4] * psi[4] + s[5] * psi[5];
}

/* dfdu += scale * B_q^T g for the 8 (shell) / 6 (hex) strain components */
static void add_BT(const or_problem *p, const elem_points *ep, int q,
                   double scale, const double *g, double *out24) {
  if (p->elem_type == 0) {
    for (int k = 0; k < 24; k++) {
      double v = 0.0;
      for (int r = 0; r < 8; r++) v += ep->B[q][r][k] * g[r];
      out24[k] += scale * v;
    }
  } else {
    hex_addBts(ep->Nx[q], scale, g, out24);
  }
}

static double gauss_weight(void) { return 1.0; }

/* KS state: two-stage max then sum (TACSKSFailure.cpp:100-195, KS_CONTINUOUS) */
static void ks_stats(const or_problem *p, const double *vars, double *maxf,
                     double *ksum) {
  double mx = -1e20, sum = 0.0;
  elem_points ep;
  for (int el = 0; el < p->nelem; el++) {
    elem_points_eval(p, el, vars, &ep);
    for (int q = 0; q < ep.nq; q++) {
      double f = point_failure(p, p->thick[el], ep.e[q], NULL, NULL);
      if (f > mx) mx = f;
    }
  }
  for (int el = 0; el < p->nelem; el++) {
    elem_points_eval(p, el, vars, &ep);
    for (int q = 0; q < ep.nq; q++) {
      double f = point_failure(p, p->thick[el], ep.e[q], NULL, NULL);
      sum += gauss_weight() * ep.detXd[q] * exp(p->ks_weight * (f - mx));
    }
  }
  *maxf = mx;
  *ksum = sum;
}

/* TACSAssembler::evalFunctions (TACSAssembler.cpp:4617-4668) */
void or_eval_funcs(const or_problem *p, const double *vars, double f[2]) {
  double comp = 0.0;
  elem_points ep;
  for (int el = 0; el < p->nelem; el++) {
    elem_points_eval(p, el, vars, &ep);
    for (int q = 0; q < ep.nq; q++)
      comp += ep.detXd[q] * gauss_weight() *
              point_sed(p, p->thick[el], ep.e[q], NULL);
  }
  double mx, ksum;
  ks_stats(p, vars, &mx, &ksum);
  f[0] = comp;
  f[1] = mx + log(ksum / 1.0) / p->ks_weight;
}

/* TACSAssembler::addSVSens (TACSAssembler.cpp:4941-5031) for compliance
   (which = 0, TACSCompliance.cpp:95-120) or KS failure (which = 1,
   TACSKSFailure.cpp:221-300). */
void or_add_sv_sens(const or_problem *p, const double *vars, int which,
                    double *dfdu) {
  double mx = 0.0, ksum = 1.0;
  if (which == 1) ks_stats(p, vars, &mx, &ksum);
  int npe = npe_of(p), vpn = vpn_of(p);
  elem_points ep;
  for (int el = 0; el < p->nelem; el++) {
    elem_points_eval(p, el, vars, &ep);
    double r[24] = {0};
    for (int q = 0; q < ep.nq; q++) {
      double g[9];
      if (which == 0) {
        double s[9];
        point_sed(p, p->thick[el], ep.e[q], s);
        for (int i = 0; i < 9; i++) g[i] = 2.0 * s[i];
        add_BT(p, &ep, q, ep.detXd[q] * gauss_weight(), g, r);
      } else {
        double f = point_failure(p, p->thick[el], ep.e[q], g, NULL);
        double dfdq = exp(p->ks_weight * (f - mx)) / ksum;
        dfdq *= gauss_weight() * ep.detXd[q];
        add_BT(p, &ep, q, dfdq, g, r);
      }
    }
    for (int m = 0; m < npe; m++) {
      int n = p->conn[npe * el + m];
      for (int k = 0; k < vpn; k++) dfdu[(size_t)vpn * n + k] += r[vpn * m + k];
    }
  }
}

/* TACSAssembler::addDVSens (TACSAssembler.cpp:4767-4856) */
void or_add_dv_sens(const or_problem *p, const double *vars, int which,
                    double scale, double *dfdx) {
  double mx = 0.0, ksum = 1.0;
  if (which == 1) ks_stats(p, vars, &mx, &ksum);
  elem_points ep;
  for (int el = 0; el < p->nelem; el++) {
    if (p->dvnum[el] < 0) continue;
    elem_points_eval(p, el, vars, &ep);
    double acc = 0.0;
    for (int q = 0; q < ep.nq; q++) {
      if (which == 0) {
        acc += scale * ep.detXd[q] * gauss_weight() *
               stress_dv(p, p->thick[el], ep.e[q], ep.e[q]);
      } else {
        double dfdt;
        double f = point_failure(p, p->thick[el], ep.e[q], NULL, &dfdt);
        double dfdq = gauss_weight() * ep.detXd[q] *
                      exp(p->ks_weight * (f - mx)) / ksum;
        acc += scale * dfdq * dfdt;
      }
    }
    dfdx[p->dvnum[el]] += acc;
  }
}

/* TACSAssembler::addAdjointResProducts (TACSAssembler.cpp:5033-5134) ->
   TACSShellElement::addAdjResProduct (TACSShellElement.h:918-1012) /
   TACSElement3D::addAdjResProduct -> addWeakAdjProduct
   (TACSLinearElasticity.cpp:953-1000).  Loads carry no design dependence. */
void or_add_adj_res_product(const or_problem *p, const double *vars,
                            const double *psi, double scale, double *dfdx) {
  int vpn = vpn_of(p);
  for (int el = 0; el < p->nelem; el++) {
    if (p->dvnum[el] < 0) continue;
    double X[24], u[24], ps[24];
    gather(p, el, p->xpts, 3, X);
    gather(p, el, vars, vpn, u);
    gather(p, el, psi, vpn, ps);
    double acc = 0.0;
    if (p->elem_type == 0) {
      shell_geo g;
      shell_geometry(X, p, &g);
      for (int q = 0; q < 4; q++) {
        double e[9], ed[9];
        shell_strain(g.B[q], u, e);
        shell_strain(g.B[q], ps, ed);
        acc += scale * g.detXd[q] * stress_dv(p, p->thick[el], e, ed);
      }
    } else {
      hex_geo g;
      hex_geometry(X, &g);
      for (int q = 0; q < 8; q++) {
        double e[6], ed[6];
        hex_strain(g.Nx[q], u, e);
        hex_strain(g.Nx[q], ps, ed);
        acc += scale * g.detXd[q] * stress_dv(p, p->thick[el], e, ed);
      }
    }
    dfdx[p->dvnum[el]] += acc;
  }
}

/* ------------------- node-coordinate sensitivities -------------------
   Central differences of the element terms in each element coordinate,
   step h = 1e-6 times the element's largest coordinate extent.  The
   reference's own default for the shell and load elements is the same
   difference taken forward (TACSElement::addAdjResXptProduct,
   TACSElement.cpp:270; addPointQuantityXptSens, :746) or by complex step
   in its complex build. */
static double elem_extent(const double *X, int npe) {
  double ext = 0.0;
  for (int d = 0; d < 3; d++) {
    double lo = X[d], hi = X[d];
    for (int m = 1; m < npe; m++) {
      if (X[3 * m + d] < lo) lo = X[3 * m + d];
      if (X[3 * m + d] > hi) hi = X[3 * m + d];
    }
    if (hi - lo > ext) ext = hi - lo;
  }
  return ext;
}

/* Function terms of one element at coordinates X: which = 0 compliance
   sum_q detXd e.s; which = 1 the KS sum sum_q detXd e^{rho (f - mx)} / (rho
   ksum), whose derivative is TACSKSFailure::getElementXptSens
   (TACSKSFailure.cpp:289-340) with dfdq, dfddetXd at their values. */
static double elem_func_at(const or_problem *p, int el, const double *X,
                           const double *u, int which, double mx,
                           double ksum) {
  double acc = 0.0;
  double e[9];
  if (p->elem_type == 0) {
    shell_geo g;
    shell_geometry(X, p, &g);
    for (int q = 0; q < 4; q++) {
      shell_strain(g.B[q], u, e);
      e[8] = 0.0;
      if (which == 0)
        acc += g.detXd[q] * point_sed(p, p->thick[el], e, NULL);
      else
        acc += g.detXd[q] *
               exp(p->ks_weight *
                   (point_failure(p, p->thick[el], e, NULL, NULL) - mx));
    }
  } else {
    hex_geo g;
    hex_geometry(X, &g);
    for (int q = 0; q < 8; q++) {
      hex_strain(g.Nx[q], u, e);
      if (which == 0)
        acc += g.detXd[q] * point_sed(p, p->thick[el], e, NULL);
      else
        acc += g.detXd[q] *
               exp(p->ks_weight *
                   (point_failure(p, p->thick[el], e, NULL, NULL) - mx));
    }
  }
  return which == 0 ? acc : acc / (p->ks_weight * ksum);
}

/* TACSAssembler::addXptSens (TACSAssembler.cpp:4858-4920) */
void or_add_xpt_sens(const or_problem *p, const double *vars, int which,
                     double coef, double *dfdX) {
  double mx = 0.0, ksum = 1.0;
  if (which == 1) ks_stats(p, vars, &mx, &ksum);
  const int npe = npe_of(p);
  for (int el = 0; el < p->nelem; el++) {
    double X[24], u[24];
    gather(p, el, p->xpts, 3, X);
    gather(p, el, vars, vpn_of(p), u);
    const double h = 1e-6 * elem_extent(X, npe);
    for (int k = 0; k < 3 * npe; k++) {
      const double x0 = X[k];
      X[k] = x0 + h;
      const double fp = elem_func_at(p, el, X, u, which, mx, ksum);
      X[k] = x0 - h;
      const double fm = elem_func_at(p, el, X, u, which, mx, ksum);
      X[k] = x0;
      dfdX[3 * (size_t)p->conn[npe * el + k / 3] + k % 3] +=
          coef * (fp - fm) / (2.0 * h);
    }
  }
}

/* TACSAssembler::addAdjointResXptSensProducts (TACSAssembler.cpp:
   5136-5205): element residual and its loads (scaled by lambda) */
void or_add_adj_res_xpt_product(const or_problem *p, const double *vars,
                                const double *psi, double scale,
                                double lambda, double *dfdX) {
  load_index L;
  build_load_index(p, &L);
  const int npe = npe_of(p), vpn = vpn_of(p), nv = npe * vpn;
  for (int el = 0; el < p->nelem; el++) {
    double X[24], u[24], ps[24], rp[24], rm[24];
    gather(p, el, p->xpts, 3, X);
    gather(p, el, vars, vpn, u);
    gather(p, el, psi, vpn, ps);
    const double h = 1e-6 * elem_extent(X, npe);
    for (int k = 0; k < 3 * npe; k++) {
      const double x0 = X[k];
      X[k] = x0 + h;
      elem_residual_at(p, &L, el, X, u, lambda, rp);
      X[k] = x0 - h;
      elem_residual_at(p, &L, el, X, u, lambda, rm);
      X[k] = x0;
      double d = 0.0;
      for (int i = 0; i < nv; i++) d += ps[i] * (rp[i] - rm[i]);
      dfdX[3 * (size_t)p->conn[npe * el + k / 3] + k % 3] +=
          scale * d / (2.0 * h);
    }
  }
  free_load_index(&L);
}

/* The full static-solve + adjoint-gradient step, following
   tests/integration_tests/static_analysis_base_test.py:359-427. */
int or_static_adjoint(const or_problem *p, int m, int nrestart, double rtol,
                      double atol, const double *force, double *u,
                      double funcs[2], double *grad_comp, double *grad_ks,
                      int *iters) {
  size_t n = (size_t)p->nnodes * vpn_of(p);
  int ndv = 0;
  for (int e = 0; e < p->nelem; e++)
    if (p->dvnum[e] + 1 > ndv) ndv = p->dvnum[e] + 1;
  or_bcsr A, F;
  memset(&F, 0, sizeof(F));
  or_bcsr_create(p, &A);
  double *res = (double *)calloc(n, sizeof(double));
  double *f = (double *)malloc(sizeof(double) * n);
  double *zero = (double *)calloc(n, sizeof(double));
  double *dfdu = (double *)malloc(sizeof(double) * n);
  double *psi = (double *)malloc(sizeof(double) * n);
  int it = 0, flag;
  or_assemble_jac(p, zero, res, &A, 0, 1);
  or_ilu0_factor(&A, &F);
  memcpy(f, force, sizeof(double) * n);
  or_apply_bcs_vec(p, f);
  for (size_t i = 0; i < n; i++) res[i] -= f[i];
  flag = or_gmres(&A, &F, res, u, m, nrestart, rtol, atol, &it, p->nthreads);
  for (size_t i = 0; i < n; i++) u[i] = -u[i];
  if (iters) iters[0] = it;
  or_eval_funcs(p, u, funcs);
  /* The element matrices are symmetric, so the transpose assembly with
     row BCs equals the forward matrix with row BCs. */
  double *grads[2] = {grad_comp, grad_ks};
  for (int w = 0; w < 2; w++) {
    if (!grads[w]) continue;
    memset(dfdu, 0, sizeof(double) * n);
    or_add_sv_sens(p, u, w, dfdu);
    or_apply_bcs_vec(p, dfdu);
    or_gmres(&A, &F, dfdu, psi, m, nrestart, rtol, atol, &it, p->nthreads);
    if (iters) iters[1 + w] = it;
    memset(grads[w], 0, sizeof(double) * ndv);
    or_add_dv_sens(p, u, w, 1.0, grads[w]);
    or_add_adj_res_product(p, u, psi, -1.0, grads[w]);
  }
  or_bcsr_free(&A);
  or_bcsr_free(&F);
  free(res);
  free(f);
  free(zero);
  free(dfdu);
  free(psi);
  return flag;
}
