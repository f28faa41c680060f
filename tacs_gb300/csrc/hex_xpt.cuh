// Node-coordinate derivative of one hex8 element (TACSElement3D with
// TACSLinearElasticity3D and TACSLinearHexaBasis; TACSElement3D::
// addAdjResXptProduct and addPointQuantityXptSens, TACSElement3D.cpp:
// 260-300, 618-660; the traction load through
// TACSElement::addAdjResXptProduct, TACSElement.cpp:270):
//   d/dX [ scale psi^T R_e(X) + coef f_e(X) ]
//   psi^T R_e = sum_q detXd_q t e_q(psi) . C e_q(u)
//               + lambda sum_faces sum_n area_n N_n . (-traction) . psi
//   compliance = sum_q detXd_q e_q . t C e_q;  KS as for the shell, with
//   the failure value vonMises(C e)/ys.
// Two exact forms: hex_xpt_forward (dual numbers, one coordinate per call)
// and hex_xpt_reverse (a hand-written reverse sweep, all 24 coordinates in
// one call).  Included inside namespace tg::<anonymous> after
// hex_common.cuh and dual.cuh; also compiled for the host by the CPU check
// (tests/cpp/hex_xpt_check.cpp).
#pragma once

// stage functions of the reverse sweep keep their own register frames
#ifdef __CUDACC__
#define TG_HEX_STAGE __device__ __noinline__
#else
#define TG_HEX_STAGE inline
#endif

// The inputs of one element; the face tractions are ntrac (face, value[3])
// entries.
struct HexXptData {
  double X[24], u[24], w[24], t;
  bool has_psi;
  int ntrac;
  const int *trac_face;
  const double *trac_val;
};

__device__ double hex_xpt_forward(const ElemParams &ep, const HexXptData &dt,
                                  int kc, int func, KsStats kk, double coef,
                                  double scale, double lambda) {
  using ad::Dual;
  Dual X[24];
  for (int i = 0; i < 24; i++) X[i] = Dual(dt.X[i], i == kc ? 1.0 : 0.0);
  const double *u = dt.u, *w = dt.w;
  const double t = dt.t;
  const HexC c = hex_c(ep);
  Dual adj = 0.0, comp = 0.0;
  double ks_d = 0.0;
  for (int q = 0; q < 8; q++) {
    const double pt[3] = {gauss2(q & 1), gauss2((q >> 1) & 1), gauss2(q >> 2)};
    double Nxi[24];
    hex_shape(pt, nullptr, Nxi);
    Dual Xd[9], J[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        Dual v = 0.0;
        for (int mm = 0; mm < 8; mm++) v += Nxi[3 * mm + j] * X[3 * mm + i];
        Xd[3 * i + j] = v;
      }
    const Dual det = inv3(Xd, J);
    Dual Uu[9], Uw[9];
    for (int i = 0; i < 9; i++) Uu[i] = Uw[i] = 0.0;
    for (int mm = 0; mm < 8; mm++) {
      const double n0 = Nxi[3 * mm], n1 = Nxi[3 * mm + 1], n2 = Nxi[3 * mm + 2];
      Dual g[3];
      for (int cc = 0; cc < 3; cc++)
        g[cc] = n0 * J[cc] + n1 * J[3 + cc] + n2 * J[6 + cc];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          Uu[3 * i + j] += u[3 * mm + i] * g[j];
          Uw[3 * i + j] += w[3 * mm + i] * g[j];
        }
    }
    const Dual eu[6] = {Uu[0], Uu[4], Uu[8], Uu[5] + Uu[7], Uu[2] + Uu[6],
                        Uu[1] + Uu[3]};
    Dual s[6];
    hex_Ce(c, eu, s);
    if (dt.has_psi) {
      const Dual ew[6] = {Uw[0], Uw[4], Uw[8], Uw[5] + Uw[7], Uw[2] + Uw[6],
                          Uw[1] + Uw[3]};
      Dual v = 0.0;
      for (int k = 0; k < 6; k++) v += ew[k] * s[k];
      adj += det * t * v;
    }
    if (func == TG_FUNC_COMPLIANCE) {
      Dual v = 0.0;
      for (int k = 0; k < 6; k++) v += eu[k] * (s[k] * t);
      comp += det * v;
    } else if (func == TG_FUNC_KS_FAILURE) {
      const Dual f = hex_vm(ep, s);
      const double ex = ::exp(kk.weight * (f.v - kk.max)) / kk.sum;
      ks_d += ex / kk.weight * det.d + det.v * ex * f.d;
    }
  }
  if (dt.has_psi && lambda != 0.0) {
    for (int tk = 0; tk < dt.ntrac; tk++) {
      const int face = dt.trac_face[tk];
      const double *tr = &dt.trac_val[3 * tk];
      for (int n = 0; n < 4; n++) {
        double N[8];
        const Dual area = hex_face_point(X, face, n, N);
        double pw = 0.0;
        for (int a = 0; a < 8; a++)
          pw += N[a] * (-tr[0] * w[3 * a] - tr[1] * w[3 * a + 1] -
                        tr[2] * w[3 * a + 2]);
        adj += lambda * (area * pw);
      }
    }
  }
  double val = dt.has_psi ? scale * adj.d : 0.0;
  if (func == TG_FUNC_COMPLIANCE) val += coef * comp.d;
  else if (func == TG_FUNC_KS_FAILURE) val += coef * ks_d;
  return val;
}

// Ai = A^-1, det = det A: bA += -Ai^T bAi Ai^T + bdet det Ai^T
__device__ __forceinline__ void hex_inv3_rev(const double *Ai, double det,
                                             const double *bAi, double bdet,
                                             double *bA) {
  double M[9];
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

// One Gauss point of the reverse sweep: adds d/dX of that point's terms
// into bX.
TG_HEX_STAGE void hex_xpt_point_rev(const ElemParams &ep,
                                    const HexXptData &dt, const HexC &c,
                                    int q, int func, KsStats kk, double coef,
                                    double sc, double *bX) {
  const double *X = dt.X, *u = dt.u, *w = dt.w;
  const double t = dt.t;
  const double pt[3] = {gauss2(q & 1), gauss2((q >> 1) & 1), gauss2(q >> 2)};
  double Nxi[24];
  hex_shape(pt, nullptr, Nxi);
  double Xd[9], J[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double v = 0.0;
      for (int mm = 0; mm < 8; mm++) v += Nxi[3 * mm + j] * X[3 * mm + i];
      Xd[3 * i + j] = v;
    }
  const double det = inv3(Xd, J);
  double Uu[9], Uw[9];
  for (int i = 0; i < 9; i++) Uu[i] = Uw[i] = 0.0;
  for (int mm = 0; mm < 8; mm++)
    for (int j = 0; j < 3; j++) {
      const double g = Nxi[3 * mm] * J[j] + Nxi[3 * mm + 1] * J[3 + j] +
                       Nxi[3 * mm + 2] * J[6 + j];
      for (int i = 0; i < 3; i++) {
        Uu[3 * i + j] += u[3 * mm + i] * g;
        Uw[3 * i + j] += w[3 * mm + i] * g;
      }
    }
  const double eu[6] = {Uu[0], Uu[4], Uu[8], Uu[5] + Uu[7], Uu[2] + Uu[6],
                        Uu[1] + Uu[3]};
  const double ew[6] = {Uw[0], Uw[4], Uw[8], Uw[5] + Uw[7], Uw[2] + Uw[6],
                        Uw[1] + Uw[3]};
  double s[6], sw[6];
  hex_Ce(c, eu, s);
  hex_Ce(c, ew, sw);
  // adjoints of det and of the strains (the stiffness is symmetric)
  double bdet = 0.0, beu[6] = {0, 0, 0, 0, 0, 0}, bew[6] = {0, 0, 0, 0, 0, 0};
  if (dt.has_psi) {
    double v = 0.0;
    for (int k = 0; k < 6; k++) {
      v += ew[k] * s[k];
      bew[k] += sc * det * t * s[k];
      beu[k] += sc * det * t * sw[k];
    }
    bdet += sc * t * v;
  }
  if (func == TG_FUNC_COMPLIANCE) {
    double v = 0.0;
    for (int k = 0; k < 6; k++) {
      v += eu[k] * (s[k] * t);
      beu[k] += coef * det * t * 2.0 * s[k];
    }
    bdet += coef * v;
  } else if (func == TG_FUNC_KS_FAILURE) {
    const double f = hex_vm(ep, s);
    const double ex = ::exp(kk.weight * (f - kk.max)) / kk.sum;
    bdet += coef * ex / kk.weight;
    // d vonMises / d s (vonMisesFailure3DStressSens)
    const double fy = f * ep.ys;
    double bs[6] = {0, 0, 0, 0, 0, 0};
    if (fy != 0.0) {
      const double fact = coef * det * ex * 0.5 / (ep.ys * fy);
      bs[0] = fact * (2.0 * s[0] - s[1] - s[2]);
      bs[1] = fact * (2.0 * s[1] - s[0] - s[2]);
      bs[2] = fact * (2.0 * s[2] - s[0] - s[1]);
      bs[3] = 6.0 * fact * s[3];
      bs[4] = 6.0 * fact * s[4];
      bs[5] = 6.0 * fact * s[5];
    }
    double cbs[6];
    hex_Ce(c, bs, cbs);
    for (int k = 0; k < 6; k++) beu[k] += cbs[k];
  }
  // strains -> displacement gradients -> shape gradients -> J -> Xd
  double bUu[9], bUw[9];
  bUu[0] = beu[0]; bUu[4] = beu[1]; bUu[8] = beu[2];
  bUu[5] = bUu[7] = beu[3]; bUu[2] = bUu[6] = beu[4];
  bUu[1] = bUu[3] = beu[5];
  bUw[0] = bew[0]; bUw[4] = bew[1]; bUw[8] = bew[2];
  bUw[5] = bUw[7] = bew[3]; bUw[2] = bUw[6] = bew[4];
  bUw[1] = bUw[3] = bew[5];
  double bJ[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int mm = 0; mm < 8; mm++)
    for (int j = 0; j < 3; j++) {
      double bg = 0.0;
      for (int i = 0; i < 3; i++)
        bg += bUu[3 * i + j] * u[3 * mm + i] + bUw[3 * i + j] * w[3 * mm + i];
      for (int r = 0; r < 3; r++) bJ[3 * r + j] += Nxi[3 * mm + r] * bg;
    }
  double bXd[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  hex_inv3_rev(J, det, bJ, bdet, bXd);
  for (int mm = 0; mm < 8; mm++)
    for (int i = 0; i < 3; i++)
      bX[3 * mm + i] += Nxi[3 * mm] * bXd[3 * i] +
                        Nxi[3 * mm + 1] * bXd[3 * i + 1] +
                        Nxi[3 * mm + 2] * bXd[3 * i + 2];
}

// All 24 coordinate derivatives of the quantity above, added into dX.
__device__ void hex_xpt_reverse(const ElemParams &ep, const HexXptData &dt,
                                int func, KsStats kk, double coef,
                                double scale, double lambda, double *dX) {
  const double *X = dt.X, *w = dt.w;
  const HexC c = hex_c(ep);
  const double sc = dt.has_psi ? scale : 0.0;
  double bX[24];
  for (int i = 0; i < 24; i++) bX[i] = 0.0;
  for (int q = 0; q < 8; q++)
    hex_xpt_point_rev(ep, dt, c, q, func, kk, coef, sc, bX);
  if (dt.has_psi && lambda != 0.0) {
    for (int tk = 0; tk < dt.ntrac; tk++) {
      const int face = dt.trac_face[tk];
      const double *tr = &dt.trac_val[3 * tk];
      for (int n = 0; n < 4; n++) {
        double N[8];
        // the face point's tangents t1, t2 (columns ta, tb of dX/dxi) as
        // hex_face_point forms them; area = |t1 x t2|
        const int f2 = face >> 1;
        const double uu = gauss2(n & 1), vv = gauss2(n >> 1);
        const double cc = -1.0 + 2.0 * (face & 1);
        double fpt[3];
        if (f2 == 0) { fpt[0] = cc; fpt[1] = uu; fpt[2] = vv; }
        else if (f2 == 1) { fpt[0] = uu; fpt[1] = cc; fpt[2] = vv; }
        else { fpt[0] = uu; fpt[1] = vv; fpt[2] = cc; }
        double Nxi[24];
        hex_shape(fpt, N, Nxi);
        int ta, tb;
        if (f2 == 0) { ta = 2; tb = 1; }
        else if (f2 == 1) { ta = 0; tb = 2; }
        else { ta = 1; tb = 0; }
        if (face == 1) { ta = 1; tb = 2; }
        if (face == 3) { ta = 2; tb = 0; }
        if (face == 5) { ta = 0; tb = 1; }
        double t1[3], t2[3];
        for (int ii = 0; ii < 3; ii++) {
          double a = 0.0, b = 0.0;
          for (int m = 0; m < 8; m++) {
            a += Nxi[3 * m + ta] * X[3 * m + ii];
            b += Nxi[3 * m + tb] * X[3 * m + ii];
          }
          t1[ii] = a;
          t2[ii] = b;
        }
        const double nr[3] = {t1[1] * t2[2] - t1[2] * t2[1],
                              t1[2] * t2[0] - t1[0] * t2[2],
                              t1[0] * t2[1] - t1[1] * t2[0]};
        const double area =
            sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
        double pw = 0.0;
        for (int a = 0; a < 8; a++)
          pw += N[a] * (-tr[0] * w[3 * a] - tr[1] * w[3 * a + 1] -
                        tr[2] * w[3 * a + 2]);
        if (area == 0.0) continue;
        const double barea = sc * lambda * pw;
        const double bnr[3] = {barea * nr[0] / area, barea * nr[1] / area,
                               barea * nr[2] / area};
        // nr = t1 x t2: bt1 = t2 x bnr, bt2 = bnr x t1
        const double bt1[3] = {t2[1] * bnr[2] - t2[2] * bnr[1],
                               t2[2] * bnr[0] - t2[0] * bnr[2],
                               t2[0] * bnr[1] - t2[1] * bnr[0]};
        const double bt2[3] = {bnr[1] * t1[2] - bnr[2] * t1[1],
                               bnr[2] * t1[0] - bnr[0] * t1[2],
                               bnr[0] * t1[1] - bnr[1] * t1[0]};
        for (int m = 0; m < 8; m++)
          for (int ii = 0; ii < 3; ii++)
            bX[3 * m + ii] += Nxi[3 * m + ta] * bt1[ii] +
                              Nxi[3 * m + tb] * bt2[ii];
      }
    }
  }
  for (int i = 0; i < 24; i++) dX[i] += bX[i];
}
