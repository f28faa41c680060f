// MITC4 residual + Jacobian assembly with 8-lane teams (4 elements per warp).
//
// GB300 executes FP64 at 1/64 of the FP32 rate: every warp-wide FP64
// instruction holds the SM's FP64 pipe for 16 cycles whatever its active
// lane count.  So each warp works on four elements at once (one per 8-lane
// team), all four running the same instruction stream, and the element
// matrix is formed with as few FP64 operations as the kinematics allow:
//
//   K = sum_q detXd_q B_q^T C B_q
//     = Bty^T G Bty                         (membrane + transverse shear)
//     + sum_q detXd_q Bb_q^T D Bb_q         (bending)
//     + sum_q detXd_q drill (N_q Bd)^T (N_q Bd)   (drilling)
//
// with Bty the 9 x 24 MITC tying-strain rows, G = sum_q detXd_q M_q^T C_ms
// M_q the 9 x 9 membrane/shear stiffness in tying-strain space (M_q maps the
// tying strains to e0,e1,e2,e6,e7 at Gauss point q), Bb_q the bending rows
// and Bd the 4 nodal drilling rows.  Factoring G = L diag(d) L^T and
// D = L_D L_D^T turns K into a sum of 25 rank-one channels
// K = sum_c z_c z_c^T, so each of the 300 upper-triangle entries costs 25
// FMAs.  The kinematics (normals, transforms, tying strains, drilling
// rows) are those of TACSShellElement::addJacobian
// (src/elements/shell/TACSShellElement.h:436-641) as in shell_kernels.cu.
// Elements of one launch share no node (colouring): the BCSR
// read-modify-write and the residual scatter need no atomics, and the
// first writer of each block and residual row (MeshView::first) stores
// instead of adding, so neither needs a zero fill.
#include <cmath>

#include "tg_internal.h"

namespace tg {
namespace {

#include "shell_common.cuh"

constexpr int kTeam = 8;
constexpr int kTeamsPerWarp = 32 / kTeam;
constexpr int kWarpsPerCta = 1;
constexpr int kTeamsPerCta = kTeamsPerWarp * kWarpsPerCta;
constexpr int kNchan = 25;

struct TeamGeo {
  double Bd[4][24];
  double T[4][9], P[4][9], Q[4][9];
};

struct __align__(16) TeamSmem {
  double X[12];
  double u[24];
  double fn[12];
  double n0[4][3];
  double det[4];
  double sdet[4];
  double prd[4];  // interpolated pressure x -detXd at the 4 points
  double t;
  // rows 0..8 start as Bty; rows 9..23 hold M_q / C M_q, then rows 9..12
  // G (its L D L^T in place) and the pivots' square roots, then the
  // bending and drilling channels
  double Z[kNchan][24];
  TeamGeo g;  // T is reused for the residual's channel projections
  int nodes[4];
  int slot[16];
  unsigned first;  // MeshView::first of the element (0: add everything)
  int pad;
};

// Shape functions of node k or Gauss point q (index < 4: node, else point)
__device__ __forceinline__ void shape_at(int which, double *N, double *Na,
                                         double *Nb) {
  if (which < 4)
    shape2(-1.0 + 2.0 * (which & 1), -1.0 + 2.0 * (which >> 1), N, Na, Nb);
  else
    shape2(gauss2((which - 4) & 1), gauss2((which - 4) >> 1), N, Na, Nb);
}
// The same values read from the CTA's table (filled once per CTA: 8
// evaluation points = 4 nodes + 4 Gauss points, then the 9 tying points),
// so that no phase spends FP64 issue slots re-evaluating constants.
struct ShapeTab {
  double N[17][4], Na[17][4], Nb[17][4];
};
__device__ __forceinline__ void shape_tab(const ShapeTab &T, int which,
                                          double *N, double *Na, double *Nb) {
#pragma unroll
  for (int k = 0; k < 4; k++) {
    N[k] = T.N[which][k];
    Na[k] = T.Na[which][k];
    Nb[k] = T.Nb[which][k];
  }
}

// Row of tying strain t for node mm (TACSShellLinearModel::
// computeTyingStrain, TACSShellElementModel.h:28-140): the displacement
// part cx X,xi + cy X,eta + cn n0 and the director part
// g sum_i X,(c)[i] dmap(fn_mm, i, b), in one form for the five tying
// fields so that lanes with different fields run the same instructions.
__device__ __forceinline__ void tying_row(int f, int mm, const double *N,
                                          const double *Na, const double *Nb,
                                          const double *Xxi, const double *n0,
                                          const double *fn, double *z) {
  double cx = 0.0, cy = 0.0, cn = 0.0, g = 0.0;
  int c = 0;
  if (f == 0) cx = Na[mm];
  else if (f == 1) cy = Nb[mm];
  else if (f == 2) {
    cx = 0.5 * Nb[mm];
    cy = 0.5 * Na[mm];
  } else {
    cn = f == 3 ? 0.5 * Nb[mm] : 0.5 * Na[mm];
    g = 0.5 * N[mm];
    c = f == 3 ? 1 : 0;
  }
#pragma unroll
  for (int a = 0; a < 3; a++)
    z[6 * mm + a] = cx * Xxi[2 * a] + cy * Xxi[2 * a + 1] + cn * n0[a];
  const double x0 = Xxi[c], x1 = Xxi[2 + c], x2 = Xxi[4 + c];
  const double *fm = &fn[3 * mm];
  // rows of dmap: [0, f2, -f1], [-f2, 0, f0], [f1, -f0, 0]
  z[6 * mm + 3] = g * (x1 * -fm[2] + x2 * fm[1]);
  z[6 * mm + 4] = g * (x0 * fm[2] + x2 * -fm[0]);
  z[6 * mm + 5] = g * (x0 * -fm[1] + x1 * fm[0]);
}

__global__ void __launch_bounds__(kWarpsPerCta * 32)
    shell_team_assembly_kernel(ElemParams ep, MeshView m, ColorRange cr,
                               const double *__restrict__ vars, double lambda,
                               double *__restrict__ res,
                               double *__restrict__ mat, int *err_flag) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned char s_tile[36][2];
  __shared__ ShapeTab s_shape;
  TeamSmem *teams = reinterpret_cast<TeamSmem *>(smem_raw);
  const int lane = threadIdx.x & 31;
  const int tl = lane & (kTeam - 1);
  const int team_in_cta = threadIdx.x / kTeam;
  TeamSmem &S = teams[team_in_cta];

  // the 24 x 24 element matrix as an 8 x 8 grid of 3 x 3 tiles (a tile
  // never straddles two 6 x 6 node blocks); upper tiles (ti <= tj)
  for (int k = threadIdx.x; k < 36; k += blockDim.x) {
    int tj = 0, base = 0;
    while (base + tj + 1 <= k) {
      base += tj + 1;
      tj++;
    }
    s_tile[k][0] = (unsigned char)(k - base);
    s_tile[k][1] = (unsigned char)tj;
  }
  for (int k = threadIdx.x; k < 17; k += blockDim.x) {
    if (k < 8)
      shape_at(k, s_shape.N[k], s_shape.Na[k], s_shape.Nb[k]);
    else
      shape2(c_ty_pt[k - 8][0], c_ty_pt[k - 8][1], s_shape.N[k],
             s_shape.Na[k], s_shape.Nb[k]);
  }
  __syncthreads();

  const int gteam = blockIdx.x * kTeamsPerCta + team_in_cta;
  const int nteams = gridDim.x * kTeamsPerCta;
  // uniform trip count across the warp (teams without an element idle)
  const int warp_base = (blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5)) *
                        kTeamsPerWarp;
  const int rounds =
      cr.count > warp_base ? (cr.count - warp_base + nteams - 1) / nteams : 0;

  // per-element constitutive constants (TACSIsoShellConstitutive, tOffset 0)
  const double Dm = ep.E / (1.0 - ep.nu * ep.nu);
  const double A0[6] = {Dm, ep.nu * Dm, 0.0, Dm, 0.0, 0.5 * ep.E / (1.0 + ep.nu)};

  for (int rd = 0; rd < rounds; rd++) {
    const int idx = gteam + rd * nteams;
    const bool active = idx < cr.count;
    const int e = active ? cr.elem_list[idx] : 0;

    // ---------------------------------------------------------- load
    if (active) {
      if (tl < 4) {
        S.nodes[tl] = m.conn[4 * e + tl];
      }
      if (tl == 0) {
        S.t = m.thick[e];
        S.first = m.first ? m.first[e] : 0u;
      }
    }
    __syncwarp();
    if (active) {
      for (int i = tl; i < 12; i += kTeam)
        S.X[i] = m.xpts[3 * S.nodes[i / 3] + i % 3];
      for (int i = tl; i < 24; i += kTeam)
        S.u[i] = vars ? vars[6 * S.nodes[i / 6] + i % 6] : 0.0;
      if (mat)
        for (int i = tl; i < 16; i += kTeam)
          S.slot[i] = find_slot(m.rowp, m.cols, S.nodes[i >> 2], S.nodes[i & 3]);
    }
    __syncwarp();

    // --------------------------------------------------- node normals
    double N[4], Na[4], Nb[4], Xxi[6];
    if (tl < 4) {
      shape_tab(s_shape, tl, N, Na, Nb);
      grad3(Na, Nb, S.X, Xxi);
      double a[3] = {Xxi[0], Xxi[2], Xxi[4]}, b[3] = {Xxi[1], Xxi[3], Xxi[5]};
      double f[3];
      cross3(a, b, f);
      double nrm = sqrt(dot3(f, f));
      if (nrm != 0.0) {
        double s = 1.0 / nrm;
        f[0] *= s; f[1] *= s; f[2] *= s;
      }
      S.fn[3 * tl] = f[0]; S.fn[3 * tl + 1] = f[1]; S.fn[3 * tl + 2] = f[2];
    }
    __syncwarp();

    // ------------- frames at the 4 nodes (lanes 0-3) and 4 points (4-7)
    {
      shape_tab(s_shape, tl, N, Na, Nb);
      grad3(Na, Nb, S.X, Xxi);
      double nv[3];
      if (tl < 4) {
        nv[0] = S.fn[3 * tl]; nv[1] = S.fn[3 * tl + 1]; nv[2] = S.fn[3 * tl + 2];
      } else {
        interp3(N, S.fn, nv);
      }
      double T[9], Xd[9], Xdinv[9], XdinvT[9];
      shell_transform(ep, Xxi, nv, T);
      frame(Xxi, nv, Xd);
      const double det = inv3(Xd, Xdinv);
      mm3(Xdinv, T, XdinvT);
      if (tl < 4) {
        // nodal drilling row (TacsShellComputeDrillStrain +
        // TacsShellAddDrillStrainSens, TACSShellUtilities.h:651-790)
        const int k = tl;
        double tmp[9], du0d[9], dCpt[9];
        const double du0x[9] = {0.0, -0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0};
        mmT3(du0x, XdinvT, tmp);
        mm3(T, tmp, du0d);
        mm3(T, du0x, tmp);
        mmT3(tmp, T, dCpt);
        for (int mm = 0; mm < 4; mm++) {
          for (int a = 0; a < 3; a++)
            S.g.Bd[k][6 * mm + a] = Na[mm] * du0d[3 * a] + Nb[mm] * du0d[3 * a + 1];
          S.g.Bd[k][6 * mm + 3] = 0.0;
          S.g.Bd[k][6 * mm + 4] = 0.0;
          S.g.Bd[k][6 * mm + 5] = 0.0;
        }
        S.g.Bd[k][6 * k + 3] = 0.0 + -(dCpt[7] - dCpt[5]);
        S.g.Bd[k][6 * k + 4] = 0.0 + -(dCpt[2] - dCpt[6]);
        S.g.Bd[k][6 * k + 5] = 0.0 + -(dCpt[3] - dCpt[1]);
      } else {
        // Gauss-point displacement-gradient terms (TacsShellComputeDispGrad,
        // TACSShellUtilities.h:361-420)
        const int q = tl - 4;
        double nxi[6], Xdz[9], nXX[9], Qm[9];
        grad3(Na, Nb, S.fn, nxi);
        Xdz[0] = nxi[0]; Xdz[1] = nxi[1]; Xdz[2] = 0.0;
        Xdz[3] = nxi[2]; Xdz[4] = nxi[3]; Xdz[5] = 0.0;
        Xdz[6] = nxi[4]; Xdz[7] = nxi[5]; Xdz[8] = 0.0;
        mm3(Xdinv, Xdz, nXX);
        for (int i = 0; i < 9; i++) nXX[i] = -nXX[i];
        mm3(nXX, XdinvT, Qm);
        for (int i = 0; i < 9; i++) {
          S.g.T[q][i] = T[i];
          S.g.P[q][i] = XdinvT[i];
          S.g.Q[q][i] = Qm[i];
        }
        S.det[q] = det;
        S.n0[q][0] = nv[0]; S.n0[q][1] = nv[1]; S.n0[q][2] = nv[2];
        S.sdet[q] = sqrt(fabs(det));
        // TACSShellPressure::addResidual (TACSShellPressure.h:56-90): the
        // interpolated pressure times -detXd at this point
        if (m.pres) {
          const double *pe = m.pres + 4 * (size_t)e;
          const double pr = N[0] * pe[0] + N[1] * pe[1] + N[2] * pe[2] +
                            N[3] * pe[3];
          S.prd[q] = pr * -det;
        }
        if (!(det > 0.0) && active && err_flag) atomicCAS(err_flag, 0, 1);
      }
    }
    __syncwarp();

    // ---------------------------------------- tying-strain rows (Bty)
    // (TACSShellLinearModel::computeTyingStrain, TACSShellElementModel.h:28)
    // tying points 0..7 one per lane; point 8 with one node per lane
    {
      double n0[3];
      shape_tab(s_shape, 8 + tl, N, Na, Nb);
      grad3(Na, Nb, S.X, Xxi);
      interp3(N, S.fn, n0);
      const int f = c_ty_field[tl];
      for (int mm = 0; mm < 4; mm++)
        tying_row(f, mm, N, Na, Nb, Xxi, n0, S.fn, S.Z[tl]);
      if (tl < 4) {
        shape_tab(s_shape, 16, N, Na, Nb);
        grad3(Na, Nb, S.X, Xxi);
        interp3(N, S.fn, n0);
        tying_row(c_ty_field[8], tl, N, Na, Nb, Xxi, n0, S.fn, S.Z[8]);
      }
    }
    __syncwarp();

    // ------------------------------- M_q and C M_q (tying -> e0,e1,e2,e6,e7)
    const double t_el = S.t;
    double Ael[6], Del[6], As0, As2, drill;
    {
      const double I = t_el * t_el * t_el / 12.0;
      for (int i = 0; i < 6; i++) {
        Del[i] = I * A0[i];
        Ael[i] = A0[i] * t_el;
      }
      As0 = As2 = (5.0 / 6.0) * Ael[5];
      drill = 0.5 * 0.1 * (As0 + As2);
    }
    double *Mq = &S.Z[9][0];        // [4][5][9]
    double *CMq = &S.Z[9][0] + 180; // [4][5][9]
    for (int k = tl; k < 180; k += kTeam) {
      const int q = k / 45, r = (k % 45) / 9, t = k % 9;
      const double xi = gauss2(q & 1), eta = gauss2(q >> 1);
      const double la0 = (xi - 1.0) * -0.5, la1 = (xi + 1.0) * 0.5;
      const double lb0 = (eta - 1.0) * -0.5, lb1 = (eta + 1.0) * 0.5;
      double nty;
      switch (t) {
        case 0: case 7: nty = lb0; break;
        case 1: case 8: nty = lb1; break;
        case 2: case 5: nty = la0; break;
        case 3: case 6: nty = la1; break;
        default: nty = 1.0;
      }
      const double *P = S.g.P[q];
      const int i = c_ty_ij[c_ty_field[t]][0], j = c_ty_ij[c_ty_field[t]][1];
      const int a = c_erc[r][0], c = c_erc[r][1];
      double s = P[3 * i + a] * P[3 * j + c];
      if (i != j) s += P[3 * j + a] * P[3 * i + c];
      Mq[k] = c_efac[r] * nty * s;
    }
    __syncwarp();
    for (int k = tl; k < 180; k += kTeam) {
      const int q = k / 45, r = (k % 45) / 9, t = k % 9;
      const double *M = &Mq[45 * q];
      double v;
      // C_ms = [A 0; 0 As] acting on (e0, e1, e2, e6, e7)
      if (r == 0) v = Ael[0] * M[t] + Ael[1] * M[9 + t] + Ael[2] * M[18 + t];
      else if (r == 1) v = Ael[1] * M[t] + Ael[3] * M[9 + t] + Ael[4] * M[18 + t];
      else if (r == 2) v = Ael[2] * M[t] + Ael[4] * M[9 + t] + Ael[5] * M[18 + t];
      else if (r == 3) v = As0 * M[27 + t];
      else v = As2 * M[36 + t];
      CMq[k] = v * S.det[q];
    }
    __syncwarp();
    // G = sum_q detXd_q M_q^T C M_q (lower triangle, 45 entries), formed
    // in registers and stored over the consumed M_q (Z rows 9..12)
    double (*G)[9] = reinterpret_cast<double (*)[9]>(&S.Z[9][0]);
    double *sd = &S.Z[9][0] + 81;  // sqrt of the LDL^T pivots of G
    {
      double gv[6];
#pragma unroll
      for (int jj = 0; jj < 6; jj++) {
        const int k = tl + kTeam * jj;
        gv[jj] = 0.0;
        if (k < 45) {
          int a = 0, base = 0;
          while (base + a + 1 <= k) {
            base += a + 1;
            a++;
          }
          const int b = k - base;  // b <= a
          double v = 0.0;
          for (int q = 0; q < 4; q++)
            for (int r = 0; r < 5; r++)
              v += Mq[45 * q + 9 * r + a] * CMq[45 * q + 9 * r + b];
          gv[jj] = v;
        }
      }
      __syncwarp();
#pragma unroll
      for (int jj = 0; jj < 6; jj++) {
        const int k = tl + kTeam * jj;
        if (k < 45) {
          int a = 0, base = 0;
          while (base + a + 1 <= k) {
            base += a + 1;
            a++;
          }
          G[a][k - base] = gv[jj];
        }
      }
    }
    __syncwarp();
    // LDL^T of G (right-looking); L stored below the diagonal
    for (int k = 0; k < 9; k++) {
      const double dk = G[k][k];
      const double inv = dk > 0.0 ? 1.0 / dk : 0.0;
      __syncwarp();
      for (int i = k + 1 + tl; i < 9; i += kTeam) G[i][k] *= inv;
      __syncwarp();
      const int nr = 8 - k;
      for (int p = tl; p < nr * (nr + 1) / 2; p += kTeam) {
        int ii = 0, base = 0;
        while (base + ii + 1 <= p) {
          base += ii + 1;
          ii++;
        }
        const int i = k + 1 + ii, j = k + 1 + (p - base);
        G[i][j] -= G[i][k] * G[j][k] * dk;
      }
      if (tl == 0) sd[k] = dk > 0.0 ? sqrt(dk) : 0.0;
      __syncwarp();
    }
    // membrane/shear channels: z_t = sd_t (L^T Bty)_t, column by column
    for (int c = tl; c < 24; c += kTeam) {
      double b[9];
      for (int t = 0; t < 9; t++) b[t] = S.Z[t][c];
      for (int t = 0; t < 9; t++) {
        double v = b[t];
        for (int t2 = t + 1; t2 < 9; t2++) v += G[t2][t] * b[t2];
        S.Z[t][c] = sd[t] * v;
      }
    }
    __syncwarp();

    // bending channels: sqrt(detXd_q) L_D^T Bb_q with D = L_D L_D^T
    double L00, L10, L20, L11, L21, L22;
    {
      // guarded: a zero thickness gives zero bending channels, not NaN
      L00 = Del[0] > 0.0 ? sqrt(Del[0]) : 0.0;
      L10 = L00 > 0.0 ? Del[1] / L00 : 0.0;
      L20 = L00 > 0.0 ? Del[2] / L00 : 0.0;
      const double d11 = Del[3] - L10 * L10;
      L11 = d11 > 0.0 ? sqrt(d11) : 0.0;
      L21 = L11 > 0.0 ? (Del[4] - L20 * L10) / L11 : 0.0;
      const double d22 = Del[5] - L20 * L20 - L21 * L21;
      L22 = d22 > 0.0 ? sqrt(d22) : 0.0;
    }
    // units (q, node, dof): the 48 displacement dofs first, then the 48
    // rotations, so that every round of the team runs one of the two paths
    for (int k = tl; k < 96; k += kTeam) {
      const bool rot = k >= 48;
      const int kk = rot ? k - 48 : k;
      const int q = kk / 12, mm = (kk - 12 * q) / 3;
      const int a = (rot ? 3 : 0) + (kk - 12 * q - 3 * mm);
      const int c = 6 * mm + a;
      shape_tab(s_shape, 4 + q, N, Na, Nb);
      const double *T = S.g.T[q], *P = S.g.P[q], *Qm = S.g.Q[q];
      double bb[3];
      if (a < 3) {
        const double cu0 = Na[mm] * Qm[0] + Nb[mm] * Qm[3];
        const double cu1 = Na[mm] * Qm[1] + Nb[mm] * Qm[4];
        bb[0] = T[3 * a] * cu0;
        bb[1] = T[3 * a + 1] * cu1;
        bb[2] = T[3 * a] * cu1 + T[3 * a + 1] * cu0;
      } else {
        const int b = a - 3;
        const double cd0 = Na[mm] * P[0] + Nb[mm] * P[3] + N[mm] * Qm[6];
        const double cd1 = Na[mm] * P[1] + Nb[mm] * P[4] + N[mm] * Qm[7];
        const double *f = &S.fn[3 * mm];
        bb[0] = bb[1] = bb[2] = 0.0;
        for (int aa = 0; aa < 3; aa++) {
          const double dm = dmap(f, aa, b);
          bb[0] += (T[3 * aa] * cd0) * dm;
          bb[1] += (T[3 * aa + 1] * cd1) * dm;
          bb[2] += (T[3 * aa] * cd1 + T[3 * aa + 1] * cd0) * dm;
        }
      }
      const double s = S.sdet[q];
      S.Z[9 + 3 * q][c] = s * (L00 * bb[0] + L10 * bb[1] + L20 * bb[2]);
      S.Z[10 + 3 * q][c] = s * (L11 * bb[1] + L21 * bb[2]);
      S.Z[11 + 3 * q][c] = s * (L22 * bb[2]);
    }
    // drilling channels: sqrt(detXd_q drill) sum_k N_q[k] Bd_k
    const double sdrill = drill > 0.0 ? sqrt(drill) : 0.0;
    for (int k = tl; k < 96; k += kTeam) {
      const int q = k / 24, c = k % 24;
      shape_tab(s_shape, 4 + q, N, Na, Nb);
      double v = 0.0;
      for (int kk = 0; kk < 4; kk++) v += N[kk] * S.g.Bd[kk][c];
      S.Z[21 + q][c] = (S.sdet[q] * sdrill) * v;
    }
    __syncwarp();

    // ------------------------------------------------------- residual
    if (res) {
      double *ybuf = &S.g.T[0][0];  // T is not read after the bending rows
      for (int c = tl; c < kNchan; c += kTeam) {
        double v = 0.0;
        for (int i = 0; i < 24; i++) v += S.Z[c][i] * S.u[i];
        ybuf[c] = v;
      }
      __syncwarp();
      for (int i = tl; i < 24; i += kTeam) {
        double r = 0.0;
        for (int c = 0; c < kNchan; c++) r += S.Z[c][i] * ybuf[c];
        // TACSShellPressure::addResidual (TACSShellPressure.h:56-90)
        const int mm = i / 6, a = i - 6 * mm;
        if (m.pres && a < 3) {
          double aux = 0.0;
          for (int q = 0; q < 4; q++)
            aux += s_shape.N[4 + q][mm] * (S.prd[q] * S.n0[q][a]);
          r += lambda * aux;
        }
        if (active) {
          double &dst = res[6 * S.nodes[mm] + a];
          dst = ((S.first >> (16 + mm)) & 1u) ? r : dst + r;
        }
      }
    }

    // ------------- K: 36 upper 3 x 3 tiles, each entry sum_c Z_ci Z_cj
    // (register tiles: 6 shared loads per channel feed 9 products), the
    // off-diagonal tiles mirrored into the transposed block
    if (mat && active) {
      for (int k = tl; k < 36; k += kTeam) {
        const int ti = s_tile[k][0], tj = s_tile[k][1];
        const int i0 = 3 * ti, j0 = 3 * tj;
        double v[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll 5
        for (int c = 0; c < kNchan; c++) {
          const double zi[3] = {S.Z[c][i0], S.Z[c][i0 + 1], S.Z[c][i0 + 2]};
          const double zj[3] = {S.Z[c][j0], S.Z[c][j0 + 1], S.Z[c][j0 + 2]};
#pragma unroll
          for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) v[3 * r + q] += zi[r] * zj[q];
        }
        const int a = ti >> 1, b = tj >> 1;
        const int ii0 = 3 * (ti & 1), jj0 = 3 * (tj & 1);
        const int s_ab = S.slot[4 * a + b];
        // the element's first write of a block stores (no zero fill)
        if (s_ab >= 0) {
          double *blk = mat + 36 * (size_t)s_ab;
          if ((S.first >> (4 * a + b)) & 1u) {
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
              for (int q = 0; q < 3; q++)
                blk[6 * (ii0 + r) + jj0 + q] = v[3 * r + q];
          } else {
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
              for (int q = 0; q < 3; q++)
                blk[6 * (ii0 + r) + jj0 + q] += v[3 * r + q];
          }
        }
        if (ti != tj) {
          const int s_ba = S.slot[4 * b + a];
          if (s_ba >= 0) {
            double *blk = mat + 36 * (size_t)s_ba;
            if ((S.first >> (4 * b + a)) & 1u) {
#pragma unroll
              for (int r = 0; r < 3; r++)
#pragma unroll
                for (int q = 0; q < 3; q++)
                  blk[6 * (jj0 + q) + ii0 + r] = v[3 * r + q];
            } else {
#pragma unroll
              for (int r = 0; r < 3; r++)
#pragma unroll
                for (int q = 0; q < 3; q++)
                  blk[6 * (jj0 + q) + ii0 + r] += v[3 * r + q];
            }
          }
        }
      }
    }
    __syncwarp();
  }
}

int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

}  // namespace

void launch_shell_team_assembly(const ElemParams &ep, const MeshView &m,
                                ColorRange cr, const double *vars,
                                double lambda, double *res, double *mat,
                                int *err_flag, cudaStream_t s) {
  if (cr.count <= 0) return;
  // the shared-memory limit is a per-device kernel attribute: set on each
  // device once, recorded only when the call succeeded
  constexpr int kMaxDevices = 64;
  static bool init[kMaxDevices] = {};
  const size_t smem = sizeof(TeamSmem) * kTeamsPerCta;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices &&
      !init[dev] &&
      cudaFuncSetAttribute(shell_team_assembly_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) == cudaSuccess)
    init[dev] = true;
  // resident CTAs per SM (shared memory bound), once per device
  static int per_sm[kMaxDevices] = {};
  if (dev >= 0 && dev < kMaxDevices && !per_sm[dev]) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, shell_team_assembly_kernel, kWarpsPerCta * 32, smem) ==
            cudaSuccess &&
        nb > 0)
      per_sm[dev] = nb;
  }
  const int resident = (dev >= 0 && dev < kMaxDevices && per_sm[dev])
                           ? per_sm[dev] : 1;
  int need = (cr.count + kTeamsPerCta - 1) / kTeamsPerCta;
  int cap = sm_count() * resident;
  int grid = need < cap ? need : cap;
  if (grid < 1) grid = 1;
  shell_team_assembly_kernel<<<grid, kWarpsPerCta * 32, smem, s>>>(
      ep, m, cr, vars, lambda, res, mat, err_flag);
}

}  // namespace tg
