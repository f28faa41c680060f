// MITC4 shell (TACSQuad4Shell) point-quantity and sensitivity kernels for
// sm_103a: function values (compliance, KS failure), addSVSens, and the
// fused addDVSens + addAdjointResProducts pass.  Residual and Jacobian
// assembly live in shell_team.cu.
//
// One warp owns one element at a time.  The element's strain-displacement
// operators B_q (9 x 24 at each of the 4 Gauss points) are built
// cooperatively in shared memory from exactly the reference kinematics
// (node normals, nodal drilling strains, the 9 MITC tying strains, the
// transform T, Xd^-1 T and the through-thickness term); the strains
// e_q = B_q u then feed the point quantities (TACSShellElement::
// evalPointQuantity / addPointQuantitySVSens / addPointQuantityDVSens /
// addAdjResProduct, src/elements/shell/TACSShellElement.h:918-1352).
// The state-sensitivity pass runs colour by colour (elements of one launch
// share no node), so its scatter needs no atomics and is deterministic, and
// so do the node-coordinate sensitivities (shell_xpt_kernel), which run the
// same kinematics in dual arithmetic.
#include <cmath>
#include <mutex>

#include "dual.cuh"
#include "tg_internal.h"

namespace tg {
namespace {

#include "shell_common.cuh"

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
  double e[4][9];
  double g[4][9];
  double coef[4];
  double t;
  int nodes[4];
};

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

// B_q and detXd_q of element e: from the fixed-geometry class table when
// the view carries one, else formed from the node coordinates
__device__ __forceinline__ void shell_B(ShellSmem &S, const ElemParams &ep,
                                        const MeshView &m, int e, int lane) {
  if (m.geo_B) {
    const double *src = m.geo_B + (size_t)m.geo_cls[e] * 868;
    double *dst = &S.B[0][0][0];
    for (int i = lane; i < 864; i += 32) dst[i] = src[i];
    if (lane < 4) S.det[lane] = src[864 + lane];
    __syncwarp();
  } else {
    shell_build_B(S, ep, lane);
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
    shell_B(S, ep, m, e, lane);
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
    const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
    load_element(S, m, e, vars, nullptr, lane);
    shell_B(S, ep, m, e, lane);
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
        S.coef[q] = exp(kk.weight * (fo.f - kk.max)) / kk.sum * S.det[q];
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
    const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
    load_element(S, m, e, vars, psi, lane);
    shell_B(S, ep, m, e, lane);
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
          double dfdq = S.det[q] * exp(kk.weight * (fo.f - kk.max)) / kk.sum;
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

// ---------------------------------------------------------------------------
// Fixed-geometry forms of the three kernels above.  With the strain
// operators B_q and detXd_q in the class table (m.geo_B: 4 x 9 x 24 then
// 4 dets per geometry class) an element needs no kinematics, so it is
// owned by 4 lanes -- lane 4 j + q on Gauss point q of the warp's j-th
// element, 8 elements per warp -- and every lane does its point's FP64
// work (the warp-per-element forms leave 28 of 32 lanes idle there).  Each
// quantity is formed with the operations of the forms above, in their
// order (the sums over the 4 points included).
constexpr int kGeoWarps = 4;

__device__ __forceinline__ void geo_load_u(const MeshView &m, int e,
                                           const double *vars, double *u) {
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int n = m.conn[4 * e + a];
#pragma unroll
    for (int i = 0; i < 6; i++) u[6 * a + i] = vars ? vars[6 * n + i] : 0.0;
  }
}

// e = B_q v (the first R of the 9 strains; B_q row-major 9 x 24)
template <int R = 9>
__device__ __forceinline__ void geo_strains(const double *Bq,
                                            const double *v, double *e) {
#pragma unroll 1
  for (int r = 0; r < R; r++) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 24; k++) acc += Bq[r * 24 + k] * v[k];
    e[r] = acc;
  }
}

// ((c0 + c1) + c2) + c3 over the element's 4 lanes, on lane q = 0
__device__ __forceinline__ double geo_point_sum(double c) {
  const double c1 = __shfl_down_sync(0xffffffffu, c, 1);
  const double c2 = __shfl_down_sync(0xffffffffu, c, 2);
  const double c3 = __shfl_down_sync(0xffffffffu, c, 3);
  return ((c + c1) + c2) + c3;
}

__global__ void __launch_bounds__(kGeoWarps * 32)
    shell_points_geo_kernel(ElemParams ep, MeshView m,
                            const double *__restrict__ vars,
                            double *__restrict__ elem_fail,
                            double *__restrict__ elem_wdet,
                            double *__restrict__ elem_sed) {
  const int lane = threadIdx.x & 31, q = lane & 3;
  const int gw = blockIdx.x * kGeoWarps + (threadIdx.x >> 5);
  const int nw = gridDim.x * kGeoWarps;
  for (int e0 = 8 * gw; e0 < m.nelem; e0 += 8 * nw) {
    const int e = e0 + (lane >> 2);
    const bool on = e < m.nelem;
    double c = 0.0;
    if (on) {
      const double *tab = m.geo_B + (size_t)m.geo_cls[e] * 868;
      double u[24], ev[9];
      geo_load_u(m, e, vars, u);
      geo_strains<8>(tab + 216 * q, u, ev);  // the 9th is not used here
      ev[8] = 0.0;
      const double t = m.thick[e];
      const ShellStiff cs = shell_stiff(ep, t);
      double sed = 0.0;
      for (int r = 0; r < 9; r++) sed += ev[r] * shell_stress_row(cs, ev, r);
      const FailOut fo = shell_failure(ep, t, ev);
      const double det = tab[864 + q];
      elem_fail[4 * (size_t)e + q] = fo.f;
      elem_wdet[4 * (size_t)e + q] = det;
      c = det * sed;
    }
    const double sum = geo_point_sum(c);
    if (on && q == 0) elem_sed[e] = sum;
  }
}

__global__ void __launch_bounds__(kGeoWarps * 32)
    shell_sv_geo_kernel(ElemParams ep, MeshView m, ColorRange cr,
                        const double *__restrict__ vars, int func, KsStats ks,
                        double alpha, double *__restrict__ dfdu) {
  // each point's 24 weighted B_q^T g_q terms, summed per dof by its lane
  __shared__ double vbuf[kGeoWarps][8][4][24];
  const int lane = threadIdx.x & 31, q = lane & 3, j = lane >> 2;
  const int w = threadIdx.x >> 5;
  const int gw = blockIdx.x * kGeoWarps + w;
  const int nw = gridDim.x * kGeoWarps;
  for (int i0 = 8 * gw; i0 < cr.count; i0 += 8 * nw) {
    const bool on = i0 + j < cr.count;
    const int e = on ? cr.elem_list[i0 + j] : 0;
    if (on) {
      const double *tab = m.geo_B + (size_t)m.geo_cls[e] * 868;
      const double *Bq = tab + 216 * q;
      const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
      double u[24], ev[9], g[9], coef;
      geo_load_u(m, e, vars, u);
      geo_strains<8>(Bq, u, ev);  // the 9th is not used here
      ev[8] = 0.0;
      const double t = m.thick[e], det = tab[864 + q];
      if (func == TG_FUNC_COMPLIANCE) {
        const ShellStiff cs = shell_stiff(ep, t);
        for (int r = 0; r < 9; r++) g[r] = 2.0 * shell_stress_row(cs, ev, r);
        coef = det;
      } else {
        const FailOut fo = shell_failure(ep, t, ev);
        for (int r = 0; r < 6; r++) g[r] = fo.dfde[r];
        g[6] = g[7] = g[8] = 0.0;
        coef = exp(kk.weight * (fo.f - kk.max)) / kk.sum * det;
      }
      for (int k = 0; k < 24; k++) {
        double v = 0.0;
        for (int r = 0; r < 8; r++) v += Bq[r * 24 + k] * g[r];
        vbuf[w][j][q][k] = coef * v;
      }
    }
    __syncwarp();
    if (on) {
      const int node = m.conn[4 * e + q];
      for (int i = 0; i < 6; i++) {
        double acc = 0.0;
        for (int p = 0; p < 4; p++) acc += vbuf[w][j][p][6 * q + i];
        dfdu[6 * node + i] += alpha * acc;
      }
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kGeoWarps * 32)
    shell_dv_geo_kernel(ElemParams ep, MeshView m,
                        const double *__restrict__ vars, int func, KsStats ks,
                        double coef, const double *__restrict__ psi,
                        double scale, double *__restrict__ out) {
  const int lane = threadIdx.x & 31, q = lane & 3;
  const int gw = blockIdx.x * kGeoWarps + (threadIdx.x >> 5);
  const int nw = gridDim.x * kGeoWarps;
  for (int e0 = 8 * gw; e0 < m.nelem; e0 += 8 * nw) {
    const int e = e0 + (lane >> 2);
    const bool on = e < m.nelem;
    double acc = 0.0;
    if (on) {
      const double *tab = m.geo_B + (size_t)m.geo_cls[e] * 868;
      const double *Bq = tab + 216 * q;
      const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
      const double t = m.thick[e], det = tab[864 + q];
      double u[24], e9[9];
      geo_load_u(m, e, vars, u);
      geo_strains(Bq, u, e9);
      if (func >= 0) {
        double ev[9];
        for (int r = 0; r < 9; r++) ev[r] = e9[r];
        ev[8] = 0.0;
        if (func == TG_FUNC_COMPLIANCE) {
          acc += coef * det * shell_stress_dv(ep, t, ev, ev);
        } else {
          const FailOut fo = shell_failure(ep, t, ev);
          const double dfdq = det * exp(kk.weight * (fo.f - kk.max)) / kk.sum;
          acc += coef * dfdq * fo.dfdt;
        }
      }
      if (psi) {
        double w[24], g9[9];
        geo_load_u(m, e, psi, w);
        geo_strains(Bq, w, g9);
        acc += scale * det * shell_stress_dv(ep, t, e9, g9);
      }
    }
    const double sum = geo_point_sum(acc);
    if (on && q == 0) out[e] = sum;
  }
}

// ---------------------------------------------------------------------------
// Node-coordinate sensitivities (TACSAssembler::addXptSens and
// addAdjointResXptSensProducts, src/TACSAssembler.cpp:4858-4920,5136-5205):
// per element, d/dX of scale psi^T R_e + coef f_e (shell residual and
// pressure load; compliance or KS failure terms), defined and derived in
// shell_xpt.cuh in two exact forms: forward (dual numbers,
// shell_xpt_kernel, one thread per element coordinate) and reverse (a
// hand-written adjoint sweep, shell_xpt_rev_kernel, one thread per
// element).  Both scatter colour by colour without atomics.
#include "shell_xpt.cuh"

__device__ __forceinline__ void shell_xpt_load(const MeshView &m, int e,
                                               const double *vars,
                                               const double *psi,
                                               ShellXptData &dt, int *nodes) {
  for (int i = 0; i < 4; i++) nodes[i] = m.conn[4 * e + i];
  for (int i = 0; i < 12; i++) dt.X[i] = m.xpts[3 * nodes[i / 3] + i % 3];
  for (int i = 0; i < 24; i++) {
    const int g = 6 * nodes[i / 6] + i % 6;
    dt.u[i] = vars[g];
    dt.w[i] = psi ? psi[g] : 0.0;
  }
  dt.t = m.thick[e];
  dt.has_psi = psi != nullptr;
  dt.has_pres = m.pres != nullptr;
  for (int k = 0; k < 4; k++) dt.pres[k] = m.pres ? m.pres[4 * e + k] : 0.0;
}

__global__ void __launch_bounds__(128)
    shell_xpt_kernel(ElemParams ep, MeshView m, ColorRange cr,
                     const double *__restrict__ vars, int func, KsStats ks,
                     double coef, const double *__restrict__ psi, double scale,
                     double lambda, double *__restrict__ dfdX) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 12LL * cr.count) return;
  const int e = cr.elem_list[idx / 12], kc = (int)(idx % 12);
  ShellXptData dt;
  int nodes[4];
  shell_xpt_load(m, e, vars, psi, dt, nodes);
  const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
  const double val =
      shell_xpt_forward(ep, dt, kc, func, kk, coef, scale, lambda);
  dfdX[3 * nodes[kc / 3] + kc % 3] += val;
}

__global__ void __launch_bounds__(128)
    shell_xpt_rev_kernel(ElemParams ep, MeshView m, ColorRange cr,
                         const double *__restrict__ vars, int func,
                         KsStats ks, double coef,
                         const double *__restrict__ psi, double scale,
                         double lambda, double *__restrict__ dfdX) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= cr.count) return;
  const int e = cr.elem_list[idx];
  ShellXptData dt;
  int nodes[4];
  shell_xpt_load(m, e, vars, psi, dt, nodes);
  const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
  double dX[12];
  for (int i = 0; i < 12; i++) dX[i] = 0.0;
  shell_xpt_reverse(ep, dt, func, kk, coef, scale, lambda, dX);
  for (int i = 0; i < 12; i++) dfdX[3 * nodes[i / 3] + i % 3] += dX[i];
}

// Fixed-geometry class table (geo_plan.h): for the linear MITC4 element
// with TACSIsoShellConstitutive (tOffset 0) the tangent is
// C(t) = t C1 + t^3 C3 (A, As and the drilling stiffness grow with t, D with
// t^3; TACSIsoShellConstitutive.cpp:181-217), so
//   K(t) = sum_q detXd_q B_q^T C(t) B_q = t K1 + t^3 K3
// with B_q the strain operator of the residual (shell_build_B).  One warp
// per representative element writes K1 and K3 as the 16 node blocks
// (a, b) of 6 x 6; the upper triangle is formed and mirrored, so every
// element matrix is exactly symmetric like the team kernel's.
struct ShellGeoSmem {
  ShellSmem s;
  double CB[4][9][24];  // detXd_q C(t = 1) B_q
};

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    shell_geo_build_kernel(ElemParams ep, MeshView m,
                           const int *__restrict__ reps, int nreps,
                           double *__restrict__ table,
                           double *__restrict__ btab) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ShellGeoSmem &G = reinterpret_cast<ShellGeoSmem *>(smem_raw)[threadIdx.x >> 5];
  ShellSmem &S = G.s;
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  const ShellStiff c1 = shell_stiff(ep, 1.0);
  for (int c = gw; c < nreps; c += nw) {
    load_element(S, m, reps[c], nullptr, nullptr, lane);
    shell_build_B(S, ep, lane);
    if (btab) {  // the strain operators and detXd for the function kernels
      double *bo = btab + (size_t)c * 868;
      const double *bs = &S.B[0][0][0];
      for (int i = lane; i < 864; i += 32) bo[i] = bs[i];
      if (lane < 4) bo[864 + lane] = S.det[lane];
    }
    for (int idx = lane; idx < 96; idx += 32) {
      const int q = idx / 24, j = idx - 24 * q;
      double ev[9];
      for (int r = 0; r < 9; r++) ev[r] = S.B[q][r][j];
      for (int r = 0; r < 9; r++)
        G.CB[q][r][j] = S.det[q] * shell_stress_row(c1, ev, r);
    }
    __syncwarp();
    double *out = table + (size_t)c * 1152;
    for (int idx = lane; idx < 300; idx += 32) {
      int j = 0, base = 0;
      while (base + j + 1 <= idx) {
        base += j + 1;
        j++;
      }
      const int i = idx - base;  // i <= j
      double k1 = 0.0, k3 = 0.0;
      for (int q = 0; q < 4; q++) {
        for (int r = 0; r < 3; r++) k1 += S.B[q][r][i] * G.CB[q][r][j];
        for (int r = 6; r < 9; r++) k1 += S.B[q][r][i] * G.CB[q][r][j];
        for (int r = 3; r < 6; r++) k3 += S.B[q][r][i] * G.CB[q][r][j];
      }
      const int a = i / 6, ri = i - 6 * a, b = j / 6, cj = j - 6 * b;
      out[(4 * a + b) * 36 + 6 * ri + cj] = k1;
      out[576 + (4 * a + b) * 36 + 6 * ri + cj] = k3;
      out[(4 * b + a) * 36 + 6 * cj + ri] = k1;
      out[576 + (4 * b + a) * 36 + 6 * cj + ri] = k3;
    }
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

// Per kernel and device: the dynamic shared-memory limit (a per-device
// attribute of a kernel, set once and kept only once the call succeeded)
// and the CTAs one SM holds at that footprint, which caps the grid (the
// element loops are grid-strided, so a resident grid hides the latency of
// the warp-per-element work best).  Returns the CTAs per SM.
constexpr int kMaxDevices = 64;
struct KernelSlot {
  const void *kernel;
  int dev;
  bool attr;
  int resident;
};
template <typename K>
int prep(K kernel, size_t bytes = sizeof(ShellSmem) * kWarps) {
  static std::mutex mu;
  static KernelSlot slots[64];
  static int nslots = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return 2;
  std::lock_guard<std::mutex> lock(mu);
  KernelSlot *sl = nullptr;
  for (int i = 0; i < nslots; i++)
    if (slots[i].kernel == (const void *)kernel && slots[i].dev == dev)
      sl = &slots[i];
  if (!sl) {
    if (nslots == 64) return 2;
    sl = &slots[nslots++];
    *sl = KernelSlot{(const void *)kernel, dev, false, 0};
  }
  if (!sl->attr &&
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)bytes) == cudaSuccess)
    sl->attr = true;
  if (sl->attr && !sl->resident) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kWarps * 32,
                                                      bytes) == cudaSuccess &&
        nb > 0)
      sl->resident = nb;
  }
  return sl->resident ? sl->resident : 2;
}

// grid of the fixed-geometry forms: 8 elements per warp, at most the CTAs
// the SMs hold
int geo_grid(int count, int ctas_per_sm) {
  const int per_cta = 8 * kWarps;
  const int need = (count + per_cta - 1) / per_cta;
  const int cap = grid_for(1 << 30, ctas_per_sm);
  return need < 1 ? 1 : (need < cap ? need : cap);
}

}  // namespace

void launch_shell_points(const ElemParams &ep, const MeshView &m,
                         const double *vars, double *elem_fail,
                         double *elem_wdet, double *elem_sed,
                         cudaStream_t s) {
  if (m.nelem <= 0) return;
  if (m.geo_B) {
    const int occ = prep(shell_points_geo_kernel, 0);
    shell_points_geo_kernel<<<geo_grid(m.nelem, occ), kGeoWarps * 32, 0,
                              s>>>(ep, m, vars, elem_fail, elem_wdet,
                                   elem_sed);
    return;
  }
  auto k = shell_points_kernel<kWarps>;
  const int occ = prep(k);
  k<<<grid_for(m.nelem, occ), kWarps * 32, sizeof(ShellSmem) * kWarps, s>>>(
      ep, m, vars, elem_fail, elem_wdet, elem_sed);
}

void launch_shell_sv_sens(const ElemParams &ep, const MeshView &m,
                          ColorRange cr, const double *vars, int func,
                          KsStats ks, double alpha, double *dfdu,
                          cudaStream_t s) {
  if (cr.count <= 0) return;
  if (m.geo_B) {
    const int occ = prep(shell_sv_geo_kernel, 0);
    shell_sv_geo_kernel<<<geo_grid(cr.count, occ), kGeoWarps * 32, 0, s>>>(
        ep, m, cr, vars, func, ks, alpha, dfdu);
    return;
  }
  auto k = shell_sv_kernel<kWarps>;
  const int occ = prep(k);
  k<<<grid_for(cr.count, occ), kWarps * 32, sizeof(ShellSmem) * kWarps, s>>>(
      ep, m, cr, vars, func, ks, alpha, dfdu);
}

void launch_shell_dv(const ElemParams &ep, const MeshView &m,
                     const double *vars, int func, KsStats ks, double coef,
                     const double *psi, double scale, double *out,
                     cudaStream_t s) {
  if (m.nelem <= 0) return;
  if (m.geo_B) {
    const int occ = prep(shell_dv_geo_kernel, 0);
    shell_dv_geo_kernel<<<geo_grid(m.nelem, occ), kGeoWarps * 32, 0, s>>>(
        ep, m, vars, func, ks, coef, psi, scale, out);
    return;
  }
  auto k = shell_dv_kernel<kWarps>;
  const int occ = prep(k);
  k<<<grid_for(m.nelem, occ), kWarps * 32, sizeof(ShellSmem) * kWarps, s>>>(
      ep, m, vars, func, ks, coef, psi, scale, out);
}

void launch_shell_geo_build(const ElemParams &ep, const MeshView &m,
                            const int *reps, int nreps, double *table,
                            double *btab, cudaStream_t s) {
  if (nreps <= 0) return;
  auto k = shell_geo_build_kernel<kWarps>;
  const size_t bytes = sizeof(ShellGeoSmem) * kWarps;
  const int occ = prep(k, bytes);
  k<<<grid_for(nreps, occ), kWarps * 32, bytes, s>>>(ep, m, reps, nreps, table,
                                                    btab);
}

void launch_shell_xpt(const ElemParams &ep, const MeshView &m, ColorRange cr,
                      const double *vars, int func, KsStats ks, double coef,
                      const double *psi, double scale, double lambda,
                      double *dfdX, int reverse, cudaStream_t s) {
  if (cr.count <= 0) return;
  if (reverse) {
    shell_xpt_rev_kernel<<<(unsigned)((cr.count + 127) / 128), 128, 0, s>>>(
        ep, m, cr, vars, func, ks, coef, psi, scale, lambda, dfdX);
    return;
  }
  const long long n = 12LL * cr.count;
  shell_xpt_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
      ep, m, cr, vars, func, ks, coef, psi, scale, lambda, dfdX);
}

}  // namespace tg
