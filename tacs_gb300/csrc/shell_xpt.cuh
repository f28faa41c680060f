// Node-coordinate derivative of one MITC4 shell element (TACSQuad4Shell):
//   d/dX [ scale psi^T R_e(X) + coef f_e(X) ]
// where R_e is the shell residual sum_q detXd_q e_q(psi) . s(e_q(u))
// (TACSShellElement::addResidual, TACSShellElement.h:295-433) plus the
// pressure load scaled by lambda (TACSShellPressure::addResidual,
// TACSShellPressure.h:51-90), and f_e the element's compliance
// sum_q detXd_q e_q . s_q (TACSCompliance::getElementXptSens,
// TACSCompliance.cpp:129-156) or its KS_CONTINUOUS failure terms with
// dfdq = detXd e^{rho (f - max)} / sum and dfddetXd = e^{rho (f - max)} /
// (rho sum) held at their values (TACSKSFailure::getElementXptSens,
// TACSKSFailure.cpp:289-340).  These are the products the reference forms
// by complex step in its complex build (TACSElement::addAdjResXptProduct /
// addPointQuantityXptSens, src/elements/TACSElement.cpp:270, 746).
//
// Two exact forms of the same derivative:
//  - shell_xpt_forward: one coordinate per call, the element kinematics of
//    shell_common.cuh evaluated in dual numbers (value + one tangent);
//  - shell_xpt_reverse: all 12 coordinates in one call, a hand-written
//    reverse (adjoint) sweep: the forward values of the node normals, the
//    nodal drilling strains and the tying strains are kept, every Gauss
//    point is recomputed and differentiated backwards into the adjoints of
//    those, and the tying, drilling and normal stages are then reversed in
//    turn.  About 4x the value arithmetic instead of 12 x (value + tangent).
//
// Included inside namespace tg::<anonymous> after shell_common.cuh and
// dual.cuh; device functions, also compiled for the host by the CPU check
// (tests/cpp/shell_xpt_check.cpp).
#pragma once

// stage functions of the reverse sweep keep their own register frames
#ifdef __CUDACC__
#define TG_XPT_STAGE __device__ __noinline__
#else
#define TG_XPT_STAGE inline
#endif

// The inputs of one element: coordinates, state and adjoint, thickness and
// nodal pressures.
struct ShellXptData {
  double X[12], u[24], w[24], t, pres[4];
  bool has_psi, has_pres;
};

__device__ __forceinline__ void shell_corner(int k, double *N, double *Na,
                                             double *Nb) {
  shape2(-1.0 + 2.0 * (k % 2), -1.0 + 2.0 * (k / 2), N, Na, Nb);
}

// ---------------------------------------------------------------- forward
// d/dX_kc of the quantity above (kc = 3 node + direction).
__device__ double shell_xpt_forward(const ElemParams &ep,
                                    const ShellXptData &dt, int kc, int func,
                                    KsStats kk, double coef, double scale,
                                    double lambda) {
  using ad::Dual;
  Dual X[12];
  for (int i = 0; i < 12; i++) X[i] = Dual(dt.X[i], i == kc ? 1.0 : 0.0);
  const double *u = dt.u, *w = dt.w;
  const double t = dt.t;
  double N[4], Na[4], Nb[4];
  Dual Xxi[6];

  // node normals (TacsShellComputeNodeNormals, TACSShellUtilities.h:301)
  Dual fn[12];
  for (int k = 0; k < 4; k++) {
    shell_corner(k, N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    Dual a[3] = {Xxi[0], Xxi[2], Xxi[4]}, b[3] = {Xxi[1], Xxi[3], Xxi[5]};
    Dual f[3];
    cross3(a, b, f);
    Dual nrm = sqrt(dot3(f, f));
    if (nrm != 0.0) {
      Dual sc = 1.0 / nrm;
      f[0] *= sc; f[1] *= sc; f[2] *= sc;
    }
    fn[3 * k] = f[0]; fn[3 * k + 1] = f[1]; fn[3 * k + 2] = f[2];
  }

  // nodal drilling strains of u and psi (TacsShellComputeDrillStrain,
  // TACSShellUtilities.h:651-790)
  Dual ed_u[4], ed_w[4];
  for (int k = 0; k < 4; k++) {
    shell_corner(k, N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    const Dual *f = &fn[3 * k];
    Dual Xdn[9], Tn[9], Xdinv[9], XdinvT[9], tmp[9], du0d[9], dCpt[9];
    frame(Xxi, f, Xdn);
    shell_transform(ep, Xxi, f, Tn);
    inv3(Xdn, Xdinv);
    mm3(Xdinv, Tn, XdinvT);
    const double du0x[9] = {0.0, -0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0};
    mmT3(du0x, XdinvT, tmp);
    mm3(Tn, tmp, du0d);
    mm3(Tn, du0x, tmp);
    mmT3(tmp, Tn, dCpt);
    Dual su = 0.0, sw = 0.0;
    for (int mm = 0; mm < 4; mm++)
      for (int a = 0; a < 3; a++) {
        const Dual v = Na[mm] * du0d[3 * a] + Nb[mm] * du0d[3 * a + 1];
        su += v * u[6 * mm + a];
        sw += v * w[6 * mm + a];
      }
    const Dual r3 = -(dCpt[7] - dCpt[5]), r4 = -(dCpt[2] - dCpt[6]),
               r5 = -(dCpt[3] - dCpt[1]);
    su += r3 * u[6 * k + 3] + r4 * u[6 * k + 4] + r5 * u[6 * k + 5];
    sw += r3 * w[6 * k + 3] + r4 * w[6 * k + 4] + r5 * w[6 * k + 5];
    ed_u[k] = su;
    ed_w[k] = sw;
  }

  // tying strains of u and psi (TACSShellLinearModel::computeTyingStrain,
  // TACSShellElementModel.h:28-73)
  Dual ety_u[9], ety_w[9];
  for (int ty = 0; ty < 9; ty++) {
    Dual n0[3];
    shape2(c_ty_pt[ty][0], c_ty_pt[ty][1], N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    interp3(N, fn, n0);
    const int f = c_ty_field[ty];
    Dual su = 0.0, sw = 0.0;
    for (int mm = 0; mm < 4; mm++) {
      for (int a = 0; a < 3; a++) {
        Dual v;
        if (f == 0) v = Na[mm] * Xxi[2 * a];
        else if (f == 1) v = Nb[mm] * Xxi[2 * a + 1];
        else if (f == 2)
          v = 0.5 * (Na[mm] * Xxi[2 * a + 1] + Nb[mm] * Xxi[2 * a]);
        else if (f == 3) v = 0.5 * n0[a] * Nb[mm];
        else v = 0.5 * n0[a] * Na[mm];
        su += v * u[6 * mm + a];
        sw += v * w[6 * mm + a];
      }
      if (f >= 3) {
        const int c = (f == 3) ? 1 : 0;
        for (int b = 0; b < 3; b++) {
          Dual acc = 0.0;
          for (int i = 0; i < 3; i++)
            acc += Xxi[2 * i + c] * dmap(&fn[3 * mm], i, b);
          const Dual v = 0.5 * N[mm] * acc;
          su += v * u[6 * mm + 3 + b];
          sw += v * w[6 * mm + 3 + b];
        }
      }
    }
    ety_u[ty] = su;
    ety_w[ty] = sw;
  }

  const ShellStiff cs = shell_stiff(ep, t);
  Dual adj = 0.0, comp = 0.0;
  double ks_d = 0.0;
  for (int q = 0; q < 4; q++) {
    const double xi = gauss2(q % 2), eta = gauss2(q / 2);
    Dual n0[3], T[9], nxi[6], Xd[9], Xdz[9], Xdinv[9], nXX[9], P[9], Qm[9];
    shape2(xi, eta, N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    interp3(N, fn, n0);
    shell_transform(ep, Xxi, n0, T);
    grad3(Na, Nb, fn, nxi);
    frame(Xxi, n0, Xd);
    Xdz[0] = nxi[0]; Xdz[1] = nxi[1]; Xdz[2] = 0.0;
    Xdz[3] = nxi[2]; Xdz[4] = nxi[3]; Xdz[5] = 0.0;
    Xdz[6] = nxi[4]; Xdz[7] = nxi[5]; Xdz[8] = 0.0;
    const Dual det = inv3(Xd, Xdinv);
    mm3(Xdinv, Xdz, nXX);
    for (int i = 0; i < 9; i++) nXX[i] = -nXX[i];
    mm3(Xdinv, T, P);
    mm3(nXX, P, Qm);

    Dual eu[9], ew[9];
    // rows 0, 1, 2, 6, 7 from the tying strains (evalTyingInterp,
    // TACSShellElementQuadBasis.h:552)
    const double la0 = (xi - 1.0) * -0.5, la1 = (xi + 1.0) * 0.5;
    const double lb0 = (eta - 1.0) * -0.5, lb1 = (eta + 1.0) * 0.5;
    const double Nty[9] = {lb0, lb1, la0, la1, 1.0, la0, la1, lb0, lb1};
    const int row_of[5] = {0, 1, 2, 6, 7};
    for (int ri = 0; ri < 5; ri++) {
      const int a = c_erc[ri][0], c = c_erc[ri][1];
      Dual su = 0.0, sw = 0.0;
      for (int ty = 0; ty < 9; ty++) {
        const int i = c_ty_ij[c_ty_field[ty]][0], j = c_ty_ij[c_ty_field[ty]][1];
        Dual pp = P[3 * i + a] * P[3 * j + c];
        if (i != j) pp += P[3 * j + a] * P[3 * i + c];
        const Dual mrt = c_efac[ri] * Nty[ty] * pp;
        su += mrt * ety_u[ty];
        sw += mrt * ety_w[ty];
      }
      eu[row_of[ri]] = su;
      ew[row_of[ri]] = sw;
    }
    // row 8: drilling strain interpolated from the nodes
    {
      Dual su = 0.0, sw = 0.0;
      for (int k = 0; k < 4; k++) {
        su += N[k] * ed_u[k];
        sw += N[k] * ed_w[k];
      }
      eu[8] = su;
      ew[8] = sw;
    }
    // rows 3, 4, 5: bending (TACSShellLinearModel::evalStrain, .h:717-732)
    {
      Dual bu[3] = {0.0, 0.0, 0.0}, bw[3] = {0.0, 0.0, 0.0};
      for (int mm = 0; mm < 4; mm++) {
        const Dual cu0 = Na[mm] * Qm[0] + Nb[mm] * Qm[3];
        const Dual cu1 = Na[mm] * Qm[1] + Nb[mm] * Qm[4];
        const Dual cd0 = Na[mm] * P[0] + Nb[mm] * P[3] + N[mm] * Qm[6];
        const Dual cd1 = Na[mm] * P[1] + Nb[mm] * P[4] + N[mm] * Qm[7];
        for (int a = 0; a < 3; a++) {
          const Dual v3 = T[3 * a] * cu0, v4 = T[3 * a + 1] * cu1;
          const Dual v5 = T[3 * a] * cu1 + T[3 * a + 1] * cu0;
          const double uu = u[6 * mm + a], ww = w[6 * mm + a];
          bu[0] += v3 * uu; bu[1] += v4 * uu; bu[2] += v5 * uu;
          bw[0] += v3 * ww; bw[1] += v4 * ww; bw[2] += v5 * ww;
        }
        for (int b = 0; b < 3; b++) {
          Dual v3 = 0.0, v4 = 0.0, v5 = 0.0;
          for (int aa = 0; aa < 3; aa++) {
            const Dual dm = dmap(&fn[3 * mm], aa, b);
            v3 += T[3 * aa] * cd0 * dm;
            v4 += T[3 * aa + 1] * cd1 * dm;
            v5 += (T[3 * aa] * cd1 + T[3 * aa + 1] * cd0) * dm;
          }
          const double uu = u[6 * mm + 3 + b], ww = w[6 * mm + 3 + b];
          bu[0] += v3 * uu; bu[1] += v4 * uu; bu[2] += v5 * uu;
          bw[0] += v3 * ww; bw[1] += v4 * ww; bw[2] += v5 * ww;
        }
      }
      for (int r = 0; r < 3; r++) {
        eu[3 + r] = bu[r];
        ew[3 + r] = bw[r];
      }
    }

    if (dt.has_psi) {
      Dual v = 0.0;
      for (int r = 0; r < 9; r++) v += ew[r] * shell_stress_row(cs, eu, r);
      adj += det * v;
      if (dt.has_pres) {
        // TACSShellPressure: r_(mm,a) = -N_mm p detXd n0_a
        double pr = 0.0;
        for (int k = 0; k < 4; k++) pr += N[k] * dt.pres[k];
        Dual wn = 0.0;
        for (int mm = 0; mm < 4; mm++)
          for (int a = 0; a < 3; a++) wn += (N[mm] * w[6 * mm + a]) * n0[a];
        adj += lambda * (pr * -det * wn);
      }
    }
    if (func >= 0) {
      eu[8] = 0.0;  // point quantities exclude the drilling strain
      if (func == TG_FUNC_COMPLIANCE) {
        Dual sed = 0.0;
        for (int r = 0; r < 9; r++) sed += eu[r] * shell_stress_row(cs, eu, r);
        comp += det * sed;
      } else {
        const FailOutT<Dual> fo = shell_failure(ep, t, eu);
        const double ex = ::exp(kk.weight * (fo.f.v - kk.max)) / kk.sum;
        ks_d += ex / kk.weight * det.d + det.v * ex * fo.f.d;
      }
    }
  }
  double val = dt.has_psi ? scale * adj.d : 0.0;
  if (func == TG_FUNC_COMPLIANCE) val += coef * comp.d;
  else if (func == TG_FUNC_KS_FAILURE) val += coef * ks_d;
  return val;
}

// ---------------------------------------------------------------- reverse
// Adjoints of the value-level building blocks (b* += d(out)/d(in)^T b_out).

// C = A B
__device__ __forceinline__ void mm3_rev(const double *A, const double *B,
                                        const double *bC, double *bA,
                                        double *bB) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      if (bA)
        bA[3 * i + j] += bC[3 * i] * B[3 * j] + bC[3 * i + 1] * B[3 * j + 1] +
                         bC[3 * i + 2] * B[3 * j + 2];
      if (bB)
        bB[3 * i + j] += A[i] * bC[j] + A[3 + i] * bC[3 + j] +
                         A[6 + i] * bC[6 + j];
    }
}
// Ai = A^-1, det = det A: bA += -Ai^T bAi Ai^T + bdet det Ai^T
__device__ __forceinline__ void inv3_rev(const double *Ai, double det,
                                         const double *bAi, double bdet,
                                         double *bA) {
  double M[9];  // Ai^T bAi
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      M[3 * i + j] = Ai[i] * bAi[j] + Ai[3 + i] * bAi[3 + j] +
                     Ai[6 + i] * bAi[6 + j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      bA[3 * i + j] += -(M[3 * i] * Ai[3 * j] + M[3 * i + 1] * Ai[3 * j + 1] +
                         M[3 * i + 2] * Ai[3 * j + 2]) +
                       bdet * det * Ai[3 * j + i];
}
__device__ __forceinline__ void grad3_rev(const double *Na, const double *Nb,
                                          const double *bXxi, double *bX) {
  for (int m = 0; m < 4; m++)
    for (int k = 0; k < 3; k++)
      bX[3 * m + k] += Na[m] * bXxi[2 * k] + Nb[m] * bXxi[2 * k + 1];
}
__device__ __forceinline__ void interp3_rev(const double *N, const double *bo,
                                            double *bX) {
  for (int m = 0; m < 4; m++)
    for (int k = 0; k < 3; k++) bX[3 * m + k] += N[m] * bo[k];
}
// Xd = frame(Xxi, n)
__device__ __forceinline__ void frame_rev(const double *bXd, double *bXxi,
                                          double *bn) {
  bXxi[0] += bXd[0]; bXxi[1] += bXd[1]; bn[0] += bXd[2];
  bXxi[2] += bXd[3]; bXxi[3] += bXd[4]; bn[1] += bXd[5];
  bXxi[4] += bXd[6]; bXxi[5] += bXd[7]; bn[2] += bXd[8];
}
// entry (i, b) of dmap is sign * f[idx] (0 on the diagonal)
__device__ __forceinline__ int dmap_entry(int i, int b, double *sign) {
  if (i == b) {
    *sign = 0.0;
    return 0;
  }
  if (i == 0) { *sign = b == 1 ? 1.0 : -1.0; return b == 1 ? 2 : 1; }
  if (i == 1) { *sign = b == 0 ? -1.0 : 1.0; return b == 0 ? 2 : 0; }
  *sign = b == 0 ? 1.0 : -1.0;
  return b == 0 ? 1 : 0;
}
// T = shell_transform(ep, Xxi, n0): adjoints of Xxi and n0
__device__ void transform_rev(const ElemParams &ep, const double *Xxi,
                              const double *n0, const double *bT,
                              double *bXxi, double *bn0) {
  const double nl = sqrt(dot3(n0, n0));
  const double n[3] = {n0[0] / nl, n0[1] / nl, n0[2] / nl};
  const double x[3] = {Xxi[0], Xxi[2], Xxi[4]};
  double t1u[3], d = 0.0, an = 0.0;
  if (ep.transform == 0) {
    d = dot3(n, x);
    t1u[0] = x[0] - 3.0 * d * n[0];
    t1u[1] = x[1];
    t1u[2] = x[2];
  } else {
    an = dot3(ep.ref_axis, n);
    for (int i = 0; i < 3; i++) t1u[i] = ep.ref_axis[i] - an * n[i];
  }
  const double tl = sqrt(dot3(t1u, t1u));
  const double t1[3] = {t1u[0] / tl, t1u[1] / tl, t1u[2] / tl};
  double bt1[3] = {bT[0], bT[3], bT[6]};
  const double bt2[3] = {bT[1], bT[4], bT[7]};
  double bn[3] = {bT[2], bT[5], bT[8]};
  double c[3];
  cross3(t1, bt2, c);  // t2 = n x t1
  bn[0] += c[0]; bn[1] += c[1]; bn[2] += c[2];
  cross3(bt2, n, c);
  bt1[0] += c[0]; bt1[1] += c[1]; bt1[2] += c[2];
  const double s1 = dot3(t1, bt1);
  double bt1u[3];
  for (int i = 0; i < 3; i++) bt1u[i] = (bt1[i] - t1[i] * s1) / tl;
  if (ep.transform == 0) {
    double bx[3] = {bt1u[0], bt1u[1], bt1u[2]};
    const double bd = -3.0 * n[0] * bt1u[0];
    bn[0] += -3.0 * d * bt1u[0];
    for (int i = 0; i < 3; i++) {
      bn[i] += bd * x[i];
      bx[i] += bd * n[i];
    }
    bXxi[0] += bx[0]; bXxi[2] += bx[1]; bXxi[4] += bx[2];
  } else {
    const double ban = -dot3(n, bt1u);
    for (int i = 0; i < 3; i++) bn[i] += -an * bt1u[i] + ban * ep.ref_axis[i];
  }
  const double sn = dot3(n, bn);
  for (int i = 0; i < 3; i++) bn0[i] += (bn[i] - n[i] * sn) / nl;
}

// Values shared by the reverse stages of one element.
struct ShellXptFwd {
  double fn[12], ed_u[4], ed_w[4], ety_u[9], ety_w[9];
};

// The node normals, nodal drilling strains and tying strains (values).
TG_XPT_STAGE void shell_xpt_values(const ElemParams &ep, const ShellXptData &dt,
                                 ShellXptFwd &fw) {
  const double *X = dt.X, *u = dt.u, *w = dt.w;
  double N[4], Na[4], Nb[4], Xxi[6];
  for (int k = 0; k < 4; k++) {
    shell_corner(k, N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    const double a[3] = {Xxi[0], Xxi[2], Xxi[4]},
                 b[3] = {Xxi[1], Xxi[3], Xxi[5]};
    double f[3];
    cross3(a, b, f);
    const double nrm = sqrt(dot3(f, f));
    if (nrm != 0.0) {
      const double sc = 1.0 / nrm;
      f[0] *= sc; f[1] *= sc; f[2] *= sc;
    }
    fw.fn[3 * k] = f[0]; fw.fn[3 * k + 1] = f[1]; fw.fn[3 * k + 2] = f[2];
  }
  const double du0x[9] = {0.0, -0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = 0; k < 4; k++) {
    shell_corner(k, N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    const double *f = &fw.fn[3 * k];
    double Xdn[9], Tn[9], Xdinv[9], XdinvT[9], tmp[9], du0d[9], dCpt[9];
    frame(Xxi, f, Xdn);
    shell_transform(ep, Xxi, f, Tn);
    inv3(Xdn, Xdinv);
    mm3(Xdinv, Tn, XdinvT);
    mmT3(du0x, XdinvT, tmp);
    mm3(Tn, tmp, du0d);
    mm3(Tn, du0x, tmp);
    mmT3(tmp, Tn, dCpt);
    double su = 0.0, sw = 0.0;
    for (int mm = 0; mm < 4; mm++)
      for (int a = 0; a < 3; a++) {
        const double v = Na[mm] * du0d[3 * a] + Nb[mm] * du0d[3 * a + 1];
        su += v * u[6 * mm + a];
        sw += v * w[6 * mm + a];
      }
    const double r3 = -(dCpt[7] - dCpt[5]), r4 = -(dCpt[2] - dCpt[6]),
                 r5 = -(dCpt[3] - dCpt[1]);
    su += r3 * u[6 * k + 3] + r4 * u[6 * k + 4] + r5 * u[6 * k + 5];
    sw += r3 * w[6 * k + 3] + r4 * w[6 * k + 4] + r5 * w[6 * k + 5];
    fw.ed_u[k] = su;
    fw.ed_w[k] = sw;
  }
  for (int ty = 0; ty < 9; ty++) {
    double n0[3];
    shape2(c_ty_pt[ty][0], c_ty_pt[ty][1], N, Na, Nb);
    grad3(Na, Nb, X, Xxi);
    interp3(N, fw.fn, n0);
    const int f = c_ty_field[ty];
    double su = 0.0, sw = 0.0;
    for (int mm = 0; mm < 4; mm++) {
      for (int a = 0; a < 3; a++) {
        double v;
        if (f == 0) v = Na[mm] * Xxi[2 * a];
        else if (f == 1) v = Nb[mm] * Xxi[2 * a + 1];
        else if (f == 2)
          v = 0.5 * (Na[mm] * Xxi[2 * a + 1] + Nb[mm] * Xxi[2 * a]);
        else if (f == 3) v = 0.5 * n0[a] * Nb[mm];
        else v = 0.5 * n0[a] * Na[mm];
        su += v * u[6 * mm + a];
        sw += v * w[6 * mm + a];
      }
      if (f >= 3) {
        const int c = (f == 3) ? 1 : 0;
        for (int b = 0; b < 3; b++) {
          double acc = 0.0;
          for (int i = 0; i < 3; i++)
            acc += Xxi[2 * i + c] * dmap(&fw.fn[3 * mm], i, b);
          const double v = 0.5 * N[mm] * acc;
          su += v * u[6 * mm + 3 + b];
          sw += v * w[6 * mm + 3 + b];
        }
      }
    }
    fw.ety_u[ty] = su;
    fw.ety_w[ty] = sw;
  }
}

// One Gauss point q, recomputed from the shared values and differentiated
// backwards: accumulates the adjoints of X, the node normals, the drilling
// and the tying strains.
TG_XPT_STAGE void shell_xpt_point_rev(const ElemParams &ep,
                                    const ShellXptData &dt,
                                    const ShellXptFwd &fw, int q, int func,
                                    KsStats kk, double coef, double scale,
                                    double lambda, const ShellStiff &cs,
                                    double *bX, double *bfn, double *bed_u,
                                    double *bed_w, double *bety_u,
                                    double *bety_w) {
  const double *X = dt.X, *u = dt.u, *w = dt.w;
  const double *fn = fw.fn;
  const double xi = gauss2(q % 2), eta = gauss2(q / 2);
  double N[4], Na[4], Nb[4], Xxi[6];
  double n0[3], T[9], nxi[6], Xd[9], Xdz[9], Xdinv[9], nXX[9], P[9], Qm[9];
  shape2(xi, eta, N, Na, Nb);
  grad3(Na, Nb, X, Xxi);
  interp3(N, fn, n0);
  shell_transform(ep, Xxi, n0, T);
  grad3(Na, Nb, fn, nxi);
  frame(Xxi, n0, Xd);
  Xdz[0] = nxi[0]; Xdz[1] = nxi[1]; Xdz[2] = 0.0;
  Xdz[3] = nxi[2]; Xdz[4] = nxi[3]; Xdz[5] = 0.0;
  Xdz[6] = nxi[4]; Xdz[7] = nxi[5]; Xdz[8] = 0.0;
  const double det = inv3(Xd, Xdinv);
  mm3(Xdinv, Xdz, nXX);
  for (int i = 0; i < 9; i++) nXX[i] = -nXX[i];
  mm3(Xdinv, T, P);
  mm3(nXX, P, Qm);

  const double la0 = (xi - 1.0) * -0.5, la1 = (xi + 1.0) * 0.5;
  const double lb0 = (eta - 1.0) * -0.5, lb1 = (eta + 1.0) * 0.5;
  const double Nty[9] = {lb0, lb1, la0, la1, 1.0, la0, la1, lb0, lb1};
  const int row_of[5] = {0, 1, 2, 6, 7};

  // forward values of the strains of u and psi at this point
  double eu[9], ew[9];
  for (int ri = 0; ri < 5; ri++) {
    const int a = c_erc[ri][0], c = c_erc[ri][1];
    double su = 0.0, sw = 0.0;
    for (int ty = 0; ty < 9; ty++) {
      const int i = c_ty_ij[c_ty_field[ty]][0], j = c_ty_ij[c_ty_field[ty]][1];
      double pp = P[3 * i + a] * P[3 * j + c];
      if (i != j) pp += P[3 * j + a] * P[3 * i + c];
      const double mrt = c_efac[ri] * Nty[ty] * pp;
      su += mrt * fw.ety_u[ty];
      sw += mrt * fw.ety_w[ty];
    }
    eu[row_of[ri]] = su;
    ew[row_of[ri]] = sw;
  }
  {
    double su = 0.0, sw = 0.0;
    for (int k = 0; k < 4; k++) {
      su += N[k] * fw.ed_u[k];
      sw += N[k] * fw.ed_w[k];
    }
    eu[8] = su;
    ew[8] = sw;
  }
  {
    double bu[3] = {0.0, 0.0, 0.0}, bw[3] = {0.0, 0.0, 0.0};
    for (int mm = 0; mm < 4; mm++) {
      const double cu0 = Na[mm] * Qm[0] + Nb[mm] * Qm[3];
      const double cu1 = Na[mm] * Qm[1] + Nb[mm] * Qm[4];
      const double cd0 = Na[mm] * P[0] + Nb[mm] * P[3] + N[mm] * Qm[6];
      const double cd1 = Na[mm] * P[1] + Nb[mm] * P[4] + N[mm] * Qm[7];
      for (int a = 0; a < 3; a++) {
        const double v3 = T[3 * a] * cu0, v4 = T[3 * a + 1] * cu1;
        const double v5 = T[3 * a] * cu1 + T[3 * a + 1] * cu0;
        const double uu = u[6 * mm + a], ww = w[6 * mm + a];
        bu[0] += v3 * uu; bu[1] += v4 * uu; bu[2] += v5 * uu;
        bw[0] += v3 * ww; bw[1] += v4 * ww; bw[2] += v5 * ww;
      }
      for (int b = 0; b < 3; b++) {
        double v3 = 0.0, v4 = 0.0, v5 = 0.0;
        for (int aa = 0; aa < 3; aa++) {
          const double dm = dmap(&fn[3 * mm], aa, b);
          v3 += T[3 * aa] * cd0 * dm;
          v4 += T[3 * aa + 1] * cd1 * dm;
          v5 += (T[3 * aa] * cd1 + T[3 * aa + 1] * cd0) * dm;
        }
        const double uu = u[6 * mm + 3 + b], ww = w[6 * mm + 3 + b];
        bu[0] += v3 * uu; bu[1] += v4 * uu; bu[2] += v5 * uu;
        bw[0] += v3 * ww; bw[1] += v4 * ww; bw[2] += v5 * ww;
      }
    }
    for (int r = 0; r < 3; r++) {
      eu[3 + r] = bu[r];
      ew[3 + r] = bw[r];
    }
  }

  // adjoints of the point's outputs
  double bdet = 0.0, beu[9], bew[9], bn0[3] = {0.0, 0.0, 0.0};
  for (int r = 0; r < 9; r++) beu[r] = bew[r] = 0.0;
  if (dt.has_psi) {
    double v = 0.0;
    for (int r = 0; r < 9; r++) {
      const double su = shell_stress_row(cs, eu, r);
      const double sw = shell_stress_row(cs, ew, r);
      v += ew[r] * su;
      bew[r] += scale * det * su;
      beu[r] += scale * det * sw;  // the stiffness is symmetric
    }
    bdet += scale * v;
    if (dt.has_pres) {
      double pr = 0.0;
      for (int k = 0; k < 4; k++) pr += N[k] * dt.pres[k];
      double Wa[3] = {0.0, 0.0, 0.0};
      for (int mm = 0; mm < 4; mm++)
        for (int a = 0; a < 3; a++) Wa[a] += N[mm] * w[6 * mm + a];
      const double wn = dot3(Wa, n0);
      bdet += scale * lambda * pr * -wn;
      for (int a = 0; a < 3; a++) bn0[a] += scale * lambda * pr * -det * Wa[a];
    }
  }
  if (func >= 0) {
    double ep8[9];
    for (int r = 0; r < 9; r++) ep8[r] = eu[r];
    ep8[8] = 0.0;  // point quantities exclude the drilling strain
    if (func == TG_FUNC_COMPLIANCE) {
      double sed = 0.0;
      for (int r = 0; r < 8; r++) {
        const double s = shell_stress_row(cs, ep8, r);
        sed += ep8[r] * s;
        beu[r] += coef * det * 2.0 * s;
      }
      bdet += coef * sed;
    } else {
      const FailOutT<double> fo = shell_failure(ep, dt.t, ep8);
      const double ex = ::exp(kk.weight * (fo.f - kk.max)) / kk.sum;
      bdet += coef * ex / kk.weight;
      for (int r = 0; r < 6; r++) beu[r] += coef * det * ex * fo.dfde[r];
    }
  }

  // strains -> tying strains, drilling strains, P, T, Qm, normals
  double bP[9], bT[9], bQm[9];
  for (int i = 0; i < 9; i++) bP[i] = bT[i] = bQm[i] = 0.0;
  for (int ri = 0; ri < 5; ri++) {
    const int a = c_erc[ri][0], c = c_erc[ri][1], row = row_of[ri];
    for (int ty = 0; ty < 9; ty++) {
      const int i = c_ty_ij[c_ty_field[ty]][0], j = c_ty_ij[c_ty_field[ty]][1];
      double pp = P[3 * i + a] * P[3 * j + c];
      if (i != j) pp += P[3 * j + a] * P[3 * i + c];
      const double f = c_efac[ri] * Nty[ty];
      bety_u[ty] += beu[row] * f * pp;
      bety_w[ty] += bew[row] * f * pp;
      const double bpp = f * (beu[row] * fw.ety_u[ty] + bew[row] * fw.ety_w[ty]);
      bP[3 * i + a] += bpp * P[3 * j + c];
      bP[3 * j + c] += bpp * P[3 * i + a];
      if (i != j) {
        bP[3 * j + a] += bpp * P[3 * i + c];
        bP[3 * i + c] += bpp * P[3 * j + a];
      }
    }
  }
  for (int k = 0; k < 4; k++) {
    bed_u[k] += N[k] * beu[8];
    bed_w[k] += N[k] * bew[8];
  }
  for (int mm = 0; mm < 4; mm++) {
    const double cu0 = Na[mm] * Qm[0] + Nb[mm] * Qm[3];
    const double cu1 = Na[mm] * Qm[1] + Nb[mm] * Qm[4];
    const double cd0 = Na[mm] * P[0] + Nb[mm] * P[3] + N[mm] * Qm[6];
    const double cd1 = Na[mm] * P[1] + Nb[mm] * P[4] + N[mm] * Qm[7];
    double bcu0 = 0.0, bcu1 = 0.0, bcd0 = 0.0, bcd1 = 0.0;
    for (int a = 0; a < 3; a++) {
      const double uu = u[6 * mm + a], ww = w[6 * mm + a];
      const double b3 = beu[3] * uu + bew[3] * ww;
      const double b4 = beu[4] * uu + bew[4] * ww;
      const double b5 = beu[5] * uu + bew[5] * ww;
      bT[3 * a] += b3 * cu0 + b5 * cu1;
      bT[3 * a + 1] += b4 * cu1 + b5 * cu0;
      bcu0 += b3 * T[3 * a] + b5 * T[3 * a + 1];
      bcu1 += b4 * T[3 * a + 1] + b5 * T[3 * a];
    }
    for (int b = 0; b < 3; b++) {
      const double uu = u[6 * mm + 3 + b], ww = w[6 * mm + 3 + b];
      const double b3 = beu[3] * uu + bew[3] * ww;
      const double b4 = beu[4] * uu + bew[4] * ww;
      const double b5 = beu[5] * uu + bew[5] * ww;
      for (int aa = 0; aa < 3; aa++) {
        double sg;
        const int fi = dmap_entry(aa, b, &sg);
        if (sg == 0.0) continue;
        const double dm = sg * fn[3 * mm + fi];
        bT[3 * aa] += (b3 * cd0 + b5 * cd1) * dm;
        bT[3 * aa + 1] += (b4 * cd1 + b5 * cd0) * dm;
        bcd0 += (b3 * T[3 * aa] + b5 * T[3 * aa + 1]) * dm;
        bcd1 += (b4 * T[3 * aa + 1] + b5 * T[3 * aa]) * dm;
        const double bdm = b3 * T[3 * aa] * cd0 + b4 * T[3 * aa + 1] * cd1 +
                           b5 * (T[3 * aa] * cd1 + T[3 * aa + 1] * cd0);
        bfn[3 * mm + fi] += sg * bdm;
      }
    }
    bQm[0] += Na[mm] * bcu0; bQm[3] += Nb[mm] * bcu0;
    bQm[1] += Na[mm] * bcu1; bQm[4] += Nb[mm] * bcu1;
    bP[0] += Na[mm] * bcd0; bP[3] += Nb[mm] * bcd0; bQm[6] += N[mm] * bcd0;
    bP[1] += Na[mm] * bcd1; bP[4] += Nb[mm] * bcd1; bQm[7] += N[mm] * bcd1;
  }

  // Qm = nXX P, nXX = -Xdinv Xdz, P = Xdinv T, (Xdinv, det) = inv(Xd)
  double bnXX[9], bXdinv[9], bXdz[9], bXd[9], bXxi[6], bnxi[6];
  for (int i = 0; i < 9; i++) bnXX[i] = bXdinv[i] = bXdz[i] = bXd[i] = 0.0;
  for (int i = 0; i < 6; i++) bXxi[i] = bnxi[i] = 0.0;
  mm3_rev(nXX, P, bQm, bnXX, bP);
  for (int i = 0; i < 9; i++) bnXX[i] = -bnXX[i];
  mm3_rev(Xdinv, Xdz, bnXX, bXdinv, bXdz);
  mm3_rev(Xdinv, T, bP, bXdinv, bT);
  inv3_rev(Xdinv, det, bXdinv, bdet, bXd);
  bnxi[0] += bXdz[0]; bnxi[1] += bXdz[1];
  bnxi[2] += bXdz[3]; bnxi[3] += bXdz[4];
  bnxi[4] += bXdz[6]; bnxi[5] += bXdz[7];
  frame_rev(bXd, bXxi, bn0);
  transform_rev(ep, Xxi, n0, bT, bXxi, bn0);
  grad3_rev(Na, Nb, bnxi, bfn);
  interp3_rev(N, bn0, bfn);
  grad3_rev(Na, Nb, bXxi, bX);
}

// One tying point backwards: adjoints of X and the node normals.
TG_XPT_STAGE void shell_xpt_tying_rev(const ShellXptData &dt,
                                    const ShellXptFwd &fw, int ty,
                                    double bsu, double bsw, double *bX,
                                    double *bfn) {
  const double *u = dt.u, *w = dt.w;
  double N[4], Na[4], Nb[4], Xxi[6], n0[3];
  shape2(c_ty_pt[ty][0], c_ty_pt[ty][1], N, Na, Nb);
  grad3(Na, Nb, dt.X, Xxi);
  interp3(N, fw.fn, n0);
  const int f = c_ty_field[ty];
  double bXxi[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, bn0[3] = {0.0, 0.0, 0.0};
  for (int mm = 0; mm < 4; mm++) {
    for (int a = 0; a < 3; a++) {
      const double bv = bsu * u[6 * mm + a] + bsw * w[6 * mm + a];
      if (f == 0) bXxi[2 * a] += Na[mm] * bv;
      else if (f == 1) bXxi[2 * a + 1] += Nb[mm] * bv;
      else if (f == 2) {
        bXxi[2 * a + 1] += 0.5 * Na[mm] * bv;
        bXxi[2 * a] += 0.5 * Nb[mm] * bv;
      } else if (f == 3) bn0[a] += 0.5 * Nb[mm] * bv;
      else bn0[a] += 0.5 * Na[mm] * bv;
    }
    if (f >= 3) {
      const int c = (f == 3) ? 1 : 0;
      for (int b = 0; b < 3; b++) {
        const double bv = 0.5 * N[mm] *
                          (bsu * u[6 * mm + 3 + b] + bsw * w[6 * mm + 3 + b]);
        for (int i = 0; i < 3; i++) {
          double sg;
          const int fi = dmap_entry(i, b, &sg);
          if (sg == 0.0) continue;
          bXxi[2 * i + c] += bv * sg * fw.fn[3 * mm + fi];
          bfn[3 * mm + fi] += bv * sg * Xxi[2 * i + c];
        }
      }
    }
  }
  interp3_rev(N, bn0, bfn);
  grad3_rev(Na, Nb, bXxi, bX);
}

// One corner's drilling strain backwards: adjoints of X and that node's
// normal.
TG_XPT_STAGE void shell_xpt_drill_rev(const ElemParams &ep,
                                    const ShellXptData &dt,
                                    const ShellXptFwd &fw, int k, double bsu,
                                    double bsw, double *bX, double *bfn) {
  const double *u = dt.u, *w = dt.w;
  double N[4], Na[4], Nb[4], Xxi[6];
  shell_corner(k, N, Na, Nb);
  grad3(Na, Nb, dt.X, Xxi);
  const double *f = &fw.fn[3 * k];
  double Xdn[9], Tn[9], Xdinv[9], XdinvT[9], tmp[9], Mx[9];
  frame(Xxi, f, Xdn);
  shell_transform(ep, Xxi, f, Tn);
  const double det = inv3(Xdn, Xdinv);
  mm3(Xdinv, Tn, XdinvT);
  const double du0x[9] = {0.0, -0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0};
  mmT3(du0x, XdinvT, Mx);  // du0d = Tn Mx
  mm3(Tn, du0x, tmp);      // dCpt = tmp Tn^T
  double bdu0d[9], bdCpt[9];
  for (int i = 0; i < 9; i++) bdu0d[i] = bdCpt[i] = 0.0;
  for (int mm = 0; mm < 4; mm++)
    for (int a = 0; a < 3; a++) {
      const double bv = bsu * u[6 * mm + a] + bsw * w[6 * mm + a];
      bdu0d[3 * a] += Na[mm] * bv;
      bdu0d[3 * a + 1] += Nb[mm] * bv;
    }
  const double br3 = bsu * u[6 * k + 3] + bsw * w[6 * k + 3];
  const double br4 = bsu * u[6 * k + 4] + bsw * w[6 * k + 4];
  const double br5 = bsu * u[6 * k + 5] + bsw * w[6 * k + 5];
  bdCpt[7] -= br3; bdCpt[5] += br3;
  bdCpt[2] -= br4; bdCpt[6] += br4;
  bdCpt[3] -= br5; bdCpt[1] += br5;
  double bTn[9], bMx[9], bXdinvT[9], bXdinv[9], btmp[9], bXdn[9];
  for (int i = 0; i < 9; i++)
    bTn[i] = bMx[i] = bXdinvT[i] = bXdinv[i] = btmp[i] = bXdn[i] = 0.0;
  // dCpt = tmp Tn^T: btmp += bdCpt Tn, bTn += bdCpt^T tmp
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int l = 0; l < 3; l++) {
        btmp[3 * i + l] += bdCpt[3 * i + j] * Tn[3 * j + l];
        bTn[3 * j + l] += bdCpt[3 * i + j] * tmp[3 * i + l];
      }
  mm3_rev(Tn, du0x, btmp, bTn, nullptr);  // tmp = Tn du0x
  mm3_rev(Tn, Mx, bdu0d, bTn, bMx);       // du0d = Tn Mx
  // Mx = du0x XdinvT^T: bXdinvT += bMx^T du0x
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      bXdinvT[3 * i + j] += bMx[i] * du0x[j] + bMx[3 + i] * du0x[3 + j] +
                            bMx[6 + i] * du0x[6 + j];
  mm3_rev(Xdinv, Tn, bXdinvT, bXdinv, bTn);  // XdinvT = Xdinv Tn
  inv3_rev(Xdinv, det, bXdinv, 0.0, bXdn);
  double bXxi[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double bf[3] = {0.0, 0.0, 0.0};
  frame_rev(bXdn, bXxi, bf);
  transform_rev(ep, Xxi, f, bTn, bXxi, bf);
  bfn[3 * k] += bf[0]; bfn[3 * k + 1] += bf[1]; bfn[3 * k + 2] += bf[2];
  grad3_rev(Na, Nb, bXxi, bX);
}

// All 12 coordinate derivatives of the quantity above, added into dX.
__device__ void shell_xpt_reverse(const ElemParams &ep, const ShellXptData &dt,
                                  int func, KsStats kk, double coef,
                                  double scale, double lambda, double *dX) {
  ShellXptFwd fw;
  shell_xpt_values(ep, dt, fw);
  const ShellStiff cs = shell_stiff(ep, dt.t);
  double bX[12], bfn[12], bed_u[4], bed_w[4], bety_u[9], bety_w[9];
  for (int i = 0; i < 12; i++) bX[i] = bfn[i] = 0.0;
  for (int i = 0; i < 4; i++) bed_u[i] = bed_w[i] = 0.0;
  for (int i = 0; i < 9; i++) bety_u[i] = bety_w[i] = 0.0;
  const double sc = dt.has_psi ? scale : 0.0;
  for (int q = 0; q < 4; q++)
    shell_xpt_point_rev(ep, dt, fw, q, func, kk, coef, sc, lambda, cs, bX,
                        bfn, bed_u, bed_w, bety_u, bety_w);
  for (int ty = 0; ty < 9; ty++)
    shell_xpt_tying_rev(dt, fw, ty, bety_u[ty], bety_w[ty], bX, bfn);
  for (int k = 0; k < 4; k++)
    shell_xpt_drill_rev(ep, dt, fw, k, bed_u[k], bed_w[k], bX, bfn);
  // node normals fn_k = f / |f|, f = a x b with a, b the corner's
  // coordinate derivatives
  for (int k = 0; k < 4; k++) {
    double N[4], Na[4], Nb[4], Xxi[6];
    shell_corner(k, N, Na, Nb);
    grad3(Na, Nb, dt.X, Xxi);
    const double a[3] = {Xxi[0], Xxi[2], Xxi[4]},
                 b[3] = {Xxi[1], Xxi[3], Xxi[5]};
    double f[3];
    cross3(a, b, f);
    const double nrm = sqrt(dot3(f, f));
    double bf[3] = {bfn[3 * k], bfn[3 * k + 1], bfn[3 * k + 2]};
    if (nrm != 0.0) {
      const double *fk = &fw.fn[3 * k];
      const double s = dot3(fk, bf);
      for (int i = 0; i < 3; i++) bf[i] = (bf[i] - fk[i] * s) / nrm;
    }
    double ba[3], bb[3];
    cross3(b, bf, ba);
    cross3(bf, a, bb);
    const double bXxi[6] = {ba[0], bb[0], ba[1], bb[1], ba[2], bb[2]};
    grad3_rev(Na, Nb, bXxi, bX);
  }
  for (int i = 0; i < 12; i++) dX[i] += bX[i];
}
