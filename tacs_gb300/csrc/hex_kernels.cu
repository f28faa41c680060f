// Trilinear hex8 elasticity kernels (TACSElement3D with
// TACSLinearElasticity3D(TACS_LINEAR_STRAIN) and TACSLinearHexaBasis) for
// sm_103a.  The 36 upper 3x3 node blocks of K = sum_q detXd_q B^T (t C) B
// are formed in the closed isotropic form (the same product B^T C B as
// TACSElementBasis::addWeakMatrix with the isotropic
// TACSMaterialProperties::evalTangentStiffness3D,
// src/constitutive/TACSMaterialProperties.cpp:270-293) and added into the
// 3x3 BCSR blocks; colouring makes the scatter atomic-free.  Assembly runs
// in 8-lane teams; the point-quantity and sensitivity kernels use one warp
// per element.
#include <cmath>

#include "dual.cuh"
#include "tg_internal.h"

namespace tg {
namespace {

#include "hex_common.cuh"

struct HexSmem {
  double X[24];
  double u[24];
  double w[24];
  double det[8];
  double J[8][9];
  double Nx[8][24];
  double e[8][6];
  double g[8][6];
  double coef[8];
  double t;
  int nodes[8];
  int slot[64];
};

__device__ __constant__ unsigned char c_pair[36][2] = {
    {0, 0}, {0, 1}, {0, 2}, {0, 3}, {0, 4}, {0, 5}, {0, 6}, {0, 7}, {1, 1},
    {1, 2}, {1, 3}, {1, 4}, {1, 5}, {1, 6}, {1, 7}, {2, 2}, {2, 3}, {2, 4},
    {2, 5}, {2, 6}, {2, 7}, {3, 3}, {3, 4}, {3, 5}, {3, 6}, {3, 7}, {4, 4},
    {4, 5}, {4, 6}, {4, 7}, {5, 5}, {5, 6}, {5, 7}, {6, 6}, {6, 7}, {7, 7}};

__device__ void hex_load(HexSmem &S, const MeshView &m, int e,
                         const double *vars, const double *vars2, int lane) {
  if (lane < 8) S.nodes[lane] = m.conn[8 * e + lane];
  if (lane == 0) S.t = m.thick[e];
  __syncwarp();
  if (lane < 24) {
    const int nd = S.nodes[lane / 3], k = lane % 3;
    S.X[lane] = m.xpts[3 * nd + k];
    S.u[lane] = vars ? vars[3 * nd + k] : 0.0;
    if (vars2) S.w[lane] = vars2[3 * nd + k];
  }
  __syncwarp();
}

// Gauss-point Jacobians and physical shape gradients
// (TACSElementBasis::getFieldGradient, TACSElementBasis.cpp:266-330)
__device__ void hex_geometry(HexSmem &S, int lane) {
  if (lane < 8) {
    const int q = lane;
    double pt[3] = {gauss2(q & 1), gauss2((q >> 1) & 1), gauss2(q >> 2)};
    double Nxi[24], Xd[9];
    hex_shape(pt, nullptr, Nxi);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double v = 0.0;
#pragma unroll
        for (int mm = 0; mm < 8; mm++) v += Nxi[3 * mm + j] * S.X[3 * mm + i];
        Xd[3 * i + j] = v;
      }
    S.det[q] = inv3(Xd, S.J[q]);
  }
  __syncwarp();
  for (int idx = lane; idx < 64; idx += 32) {
    const int q = idx >> 3, mm = idx & 7;
    double pt[3] = {gauss2(q & 1), gauss2((q >> 1) & 1), gauss2(q >> 2)};
    // gradient of node mm only
    double x[2] = {1.0 - pt[0], 1.0 + pt[0]};
    double y[2] = {1.0 - pt[1], 1.0 + pt[1]};
    double z[2] = {1.0 - pt[2], 1.0 + pt[2]};
    const int i = mm & 1, j = (mm >> 1) & 1, k = mm >> 2;
    const double n0 = 0.125 * (i ? 1.0 : -1.0) * y[j] * z[k];
    const double n1 = 0.125 * x[i] * (j ? 1.0 : -1.0) * z[k];
    const double n2 = 0.125 * x[i] * y[j] * (k ? 1.0 : -1.0);
    const double *J = S.J[q];
#pragma unroll
    for (int c = 0; c < 3; c++)
      S.Nx[q][3 * mm + c] = n0 * J[c] + n1 * J[3 + c] + n2 * J[6 + c];
  }
  __syncwarp();
}

// strains at the 8 points (TACSLinearElasticity3D, linear branch,
// TACSLinearElasticity.cpp:890-900): lanes 0..7
__device__ __forceinline__ void hex_strain(const HexSmem &S, int q,
                                           const double *v, double *e) {
  double Ux[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int mm = 0; mm < 8; mm++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Ux[3 * i + j] += v[3 * mm + i] * S.Nx[q][3 * mm + j];
  e[0] = Ux[0];
  e[1] = Ux[4];
  e[2] = Ux[8];
  e[3] = Ux[5] + Ux[7];
  e[4] = Ux[2] + Ux[6];
  e[5] = Ux[1] + Ux[3];
}
// (B^T s) component for dof (mm, i) at point q
__device__ __forceinline__ double hex_bts(const HexSmem &S, int q, int mm,
                                          int i, const double *s) {
  const double *g = &S.Nx[q][3 * mm];
  if (i == 0) return g[0] * s[0] + g[1] * s[5] + g[2] * s[4];
  if (i == 1) return g[1] * s[1] + g[0] * s[5] + g[2] * s[3];
  return g[2] * s[2] + g[1] * s[3] + g[0] * s[4];
}

// Face-traction residual of one element for node a, direction i
// (TACSTraction3D::addResidual, TACSTraction3D.cpp:87-125).
__device__ double hex_traction(const MeshView &m, int e, const double *X,
                               int a, int i) {
  double aux = 0.0;
  for (int tk = m.trac_ptr[e]; tk < m.trac_ptr[e + 1]; tk++) {
    const int face = m.trac_face[tk];
    const double tr = m.trac_val[3 * tk + i];
    for (int n = 0; n < 4; n++) {
      double N[8];
      const double area = hex_face_point(X, face, n, N);
      aux += area * N[a] * -tr;
    }
  }
  return aux;
}

// Residual and Jacobian with 8-lane teams (4 elements per warp): lane q of
// a team owns Gauss point q for the geometry and the residual and node q's
// 8 block columns for the BCSR lookups; the 36 upper node pairs (a, b) are
// spread over the team, each forming
//   M_ab = sum_q w_q g_qa g_qb^T  (w_q = detXd_q t, g = physical gradient)
//   K_ab = lambda M_ab + mu tr(M_ab) I + mu M_ab^T
// which is B^T (t C) B for the isotropic tangent (lambda = c1, mu = G,
// c0 = lambda + 2 mu).  Residual r = sum_q w_q B_q^T C e_q, summed over the
// team's lanes by shuffles in a fixed order.
struct HexTeam {
  double X[24];
  double u[24];
  double w[8];
  double G[8][8][3];  // [point][node][component]
  double t;
  int nodes[8];
  int slot[64];
};

constexpr int kHexTeamsPerCta = 8;
// CTAs per SM the register allocation aims at (launch bounds): 8 keeps
// the kernel at 128 registers (140 B of spills) and 16 warps per SM; the
// unbounded 192 registers allow 5 CTAs.  Measured on the 128 x 128 x 64
// block: 1 / 6 / 8 give 56.0 / 56.9 / 57.8 M elements/s.
#ifndef TG_HEX_MIN_BLOCKS
#define TG_HEX_MIN_BLOCKS 8
#endif

__global__ void __launch_bounds__(64, TG_HEX_MIN_BLOCKS)
    hex_team_assembly_kernel(ElemParams ep, MeshView m, ColorRange cr,
                             const double *__restrict__ vars, double lambda,
                             double *__restrict__ res,
                             double *__restrict__ mat) {
  __shared__ HexTeam teams[kHexTeamsPerCta];
  const int tm = threadIdx.x >> 3, tl = threadIdx.x & 7;
  HexTeam &S = teams[tm];
  const HexC c = hex_c(ep);
  const int nt = gridDim.x * kHexTeamsPerCta;
  const int rounds = (cr.count + nt - 1) / nt;
  for (int rd = 0; rd < rounds; rd++) {
    const int idx = (rd * gridDim.x + blockIdx.x) * kHexTeamsPerCta + tm;
    const bool active = idx < cr.count;
    const int e = active ? cr.elem_list[idx] : 0;
    if (active) {
      const int nd = m.conn[8 * e + tl];
      S.nodes[tl] = nd;
      if (tl == 0) S.t = m.thick[e];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        S.X[3 * tl + k] = m.xpts[3 * nd + k];
        S.u[3 * tl + k] = vars ? vars[3 * nd + k] : 0.0;
      }
    }
    __syncwarp();
    if (active && mat)
      for (int b = 0; b < 8; b++)
        S.slot[8 * tl + b] = find_slot(m.rowp, m.cols, S.nodes[tl],
                                       S.nodes[b]);
    // geometry at point q = tl (TACSElementBasis::getFieldGradient)
    double Nxi[24], Jinv[9];
    const int q = tl;
    if (active) {
      const double pt[3] = {gauss2(q & 1), gauss2((q >> 1) & 1),
                            gauss2(q >> 2)};
      hex_shape(pt, nullptr, Nxi);
      double Xd[9];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
          double v = 0.0;
#pragma unroll
          for (int mm = 0; mm < 8; mm++) v += Nxi[3 * mm + j] * S.X[3 * mm + i];
          Xd[3 * i + j] = v;
        }
      const double det = inv3(Xd, Jinv);
      S.w[q] = det * S.t;
#pragma unroll
      for (int a = 0; a < 8; a++)
#pragma unroll
        for (int k = 0; k < 3; k++)
          S.G[q][a][k] = Nxi[3 * a] * Jinv[k] + Nxi[3 * a + 1] * Jinv[3 + k] +
                         Nxi[3 * a + 2] * Jinv[6 + k];
    }
    __syncwarp();
    if (res) {
      // r_q = w_q B_q^T C e_q for the 24 dofs at point q = tl
      double r[24];
      {
        double Ux[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (active)
#pragma unroll
          for (int a = 0; a < 8; a++)
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
              for (int j = 0; j < 3; j++)
                Ux[3 * i + j] += S.u[3 * a + i] * S.G[q][a][j];
        double ev[6] = {Ux[0], Ux[4], Ux[8], Ux[5] + Ux[7], Ux[2] + Ux[6],
                        Ux[1] + Ux[3]};
        double sv[6];
        hex_Ce(c, ev, sv);
        const double wq = active ? S.w[q] : 0.0;
#pragma unroll
        for (int k = 0; k < 6; k++) sv[k] *= wq;
#pragma unroll
        for (int a = 0; a < 8; a++) {
          const double g0 = active ? S.G[q][a][0] : 0.0;
          const double g1 = active ? S.G[q][a][1] : 0.0;
          const double g2 = active ? S.G[q][a][2] : 0.0;
          r[3 * a] = g0 * sv[0] + g1 * sv[5] + g2 * sv[4];
          r[3 * a + 1] = g1 * sv[1] + g0 * sv[5] + g2 * sv[3];
          r[3 * a + 2] = g2 * sv[2] + g1 * sv[3] + g0 * sv[4];
        }
      }
      // sum over the team's 8 points
#pragma unroll
      for (int off = 1; off < 8; off <<= 1)
#pragma unroll
        for (int k = 0; k < 24; k++)
          r[k] += __shfl_xor_sync(0xffffffffu, r[k], off);
      // lane tl keeps node tl's three entries (selected with constant
      // indices so r stays in registers)
      double ra[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int a = 0; a < 8; a++)
        if (a == tl) {
          ra[0] = r[3 * a];
          ra[1] = r[3 * a + 1];
          ra[2] = r[3 * a + 2];
        }
      if (active) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
          double rk = ra[i];
          if (m.trac_ptr) rk += lambda * hex_traction(m, e, S.X, tl, i);
          res[3 * S.nodes[tl] + i] += rk;
        }
      }
    }
    if (mat && active) {
      for (int p = tl; p < 36; p += 8) {
        const int a = c_pair[p][0], b = c_pair[p][1];
        double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int qq = 0; qq < 8; qq++) {
          const double wq = S.w[qq];
          const double ga[3] = {wq * S.G[qq][a][0], wq * S.G[qq][a][1],
                                wq * S.G[qq][a][2]};
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) M[3 * i + j] += ga[i] * S.G[qq][b][j];
        }
        const double tr = M[0] + M[4] + M[8];
        double K[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++)
            K[3 * i + j] = c.c1 * M[3 * i + j] + c.G * M[3 * j + i] +
                           (i == j ? c.G * tr : 0.0);
        const int s_ab = S.slot[8 * a + b], s_ba = S.slot[8 * b + a];
        if (s_ab >= 0) {
          double *blk = mat + 9 * (size_t)s_ab;
#pragma unroll
          for (int k = 0; k < 9; k++) blk[k] += K[k];
        }
        if (a != b && s_ba >= 0) {
          double *blk = mat + 9 * (size_t)s_ba;
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) blk[3 * j + i] += K[3 * i + j];
        }
      }
    }
    __syncwarp();
  }
}

// TACSSolidConstitutive::evalFailure (TACSSolidConstitutive.cpp:274-300)
// with vonMisesFailure3D: the von Mises stress of C e over ys
struct HexFail {
  double f, dfde[6];
};
// TACSSolidConstitutive::evalFailure / evalFailureStrainSens
// (TACSSolidConstitutive.cpp:274-330) with vonMisesFailure3D(StressSens)
__device__ HexFail hex_failure(const ElemParams &ep, const HexC &c,
                               const double *e) {
  HexFail o;
  double s[6];
  hex_Ce(c, e, s);
  double f = sqrt(0.5 * ((s[0] - s[1]) * (s[0] - s[1]) +
                         (s[0] - s[2]) * (s[0] - s[2]) +
                         (s[1] - s[2]) * (s[1] - s[2]) +
                         6.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5])));
  double sens[6] = {0, 0, 0, 0, 0, 0};
  if (f != 0.0) {
    double fact = 0.5 / (ep.ys * f);
    sens[0] = fact * (2.0 * s[0] - s[1] - s[2]);
    sens[1] = fact * (2.0 * s[1] - s[0] - s[2]);
    sens[2] = fact * (2.0 * s[2] - s[0] - s[1]);
    sens[3] = 6.0 * fact * s[3];
    sens[4] = 6.0 * fact * s[4];
    sens[5] = 6.0 * fact * s[5];
  }
  o.f = f / ep.ys;
  hex_Ce(c, sens, o.dfde);
  return o;
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    hex_points_kernel(ElemParams ep, MeshView m, const double *__restrict__ vars,
                      double *__restrict__ elem_fail,
                      double *__restrict__ elem_wdet,
                      double *__restrict__ elem_sed) {
  __shared__ HexSmem smem[WARPS];
  HexSmem &S = smem[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  const HexC c = hex_c(ep);
  for (int e = gw; e < m.nelem; e += nw) {
    hex_load(S, m, e, vars, nullptr, lane);
    hex_geometry(S, lane);
    if (lane < 8) {
      double ev[6], s[6];
      hex_strain(S, lane, S.u, ev);
      hex_Ce(c, ev, s);
      double sed = 0.0;
      for (int k = 0; k < 6; k++) sed += ev[k] * (s[k] * S.t);
      HexFail fo = hex_failure(ep, c, ev);
      elem_fail[8 * (size_t)e + lane] = fo.f;
      elem_wdet[8 * (size_t)e + lane] = S.det[lane];
      S.coef[lane] = S.det[lane] * sed;
    }
    __syncwarp();
    if (lane == 0) {
      double acc = 0.0;
      for (int q = 0; q < 8; q++) acc += S.coef[q];
      elem_sed[e] = acc;
    }
    __syncwarp();
  }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    hex_sv_kernel(ElemParams ep, MeshView m, ColorRange cr,
                  const double *__restrict__ vars, int func, KsStats ks,
                  double alpha, double *__restrict__ dfdu) {
  __shared__ HexSmem smem[WARPS];
  HexSmem &S = smem[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  const HexC c = hex_c(ep);
  for (int idx = gw; idx < cr.count; idx += nw) {
    const int e = cr.elem_list[idx];
    const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
    hex_load(S, m, e, vars, nullptr, lane);
    hex_geometry(S, lane);
    if (lane < 8) {
      double ev[6], s[6];
      hex_strain(S, lane, S.u, ev);
      if (func == TG_FUNC_COMPLIANCE) {
        hex_Ce(c, ev, s);
        for (int k = 0; k < 6; k++) S.g[lane][k] = 2.0 * (s[k] * S.t);
        S.coef[lane] = S.det[lane];
      } else {
        HexFail fo = hex_failure(ep, c, ev);
        for (int k = 0; k < 6; k++) S.g[lane][k] = fo.dfde[k];
        S.coef[lane] =
            exp(kk.weight * (fo.f - kk.max)) / kk.sum * S.det[lane];
      }
    }
    __syncwarp();
    if (lane < 24) {
      const int mm = lane / 3, i = lane % 3;
      double acc = 0.0;
      for (int q = 0; q < 8; q++) acc += S.coef[q] * hex_bts(S, q, mm, i, S.g[q]);
      dfdu[3 * S.nodes[mm] + i] += alpha * acc;
    }
    __syncwarp();
  }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    hex_dv_kernel(ElemParams ep, MeshView m, const double *__restrict__ vars,
                  int func, KsStats ks, double coef,
                  const double *__restrict__ psi, double scale,
                  double *__restrict__ out) {
  __shared__ HexSmem smem[WARPS];
  HexSmem &S = smem[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  const HexC c = hex_c(ep);
  for (int e = gw; e < m.nelem; e += nw) {
    hex_load(S, m, e, vars, psi, lane);
    hex_geometry(S, lane);
    if (lane < 8) {
      double ev[6], s[6], acc = 0.0;
      hex_strain(S, lane, S.u, ev);
      hex_Ce(c, ev, s);
      if (func == TG_FUNC_COMPLIANCE) {
        // TACSSolidConstitutive::addStressDVSens(e, e) (.cpp:181-209)
        double v = 0.0;
        for (int k = 0; k < 6; k++) v += s[k] * ev[k];
        acc += coef * S.det[lane] * v;
      }
      // the solid failure index does not depend on t (no addFailureDVSens)
      if (psi) {
        double ep2[6];
        hex_strain(S, lane, S.w, ep2);
        double v = 0.0;
        for (int k = 0; k < 6; k++) v += s[k] * ep2[k];
        acc += scale * S.det[lane] * v;
      }
      S.coef[lane] = acc;
    }
    __syncwarp();
    if (lane == 0) {
      double acc = 0.0;
      for (int q = 0; q < 8; q++) acc += S.coef[q];
      out[e] = acc;
    }
    __syncwarp();
  }
  (void)ks;
}

// ---------------------------------------------------------------------------
// Node-coordinate sensitivities (TACSElement3D::addAdjResXptProduct and
// addPointQuantityXptSens): per element, d/dX of scale psi^T R_e + coef f_e
// (elasticity residual and face tractions; compliance or KS failure
// terms), defined in hex_xpt.cuh in two exact forms: forward (dual
// numbers, hex_xpt_kernel, one thread per element coordinate) and reverse
// (a hand-written adjoint sweep, hex_xpt_rev_kernel, one thread per
// element).  Both scatter colour by colour without atomics.
#include "hex_xpt.cuh"

__device__ __forceinline__ void hex_xpt_load(const MeshView &m, int e,
                                             const double *vars,
                                             const double *psi,
                                             HexXptData &dt, int *nodes) {
  for (int i = 0; i < 8; i++) nodes[i] = m.conn[8 * e + i];
  for (int i = 0; i < 24; i++) {
    const int g = 3 * nodes[i / 3] + i % 3;
    dt.X[i] = m.xpts[g];
    dt.u[i] = vars[g];
    dt.w[i] = psi ? psi[g] : 0.0;
  }
  dt.t = m.thick[e];
  dt.has_psi = psi != nullptr;
  if (m.trac_ptr) {
    const int t0 = m.trac_ptr[e];
    dt.ntrac = m.trac_ptr[e + 1] - t0;
    dt.trac_face = m.trac_face + t0;
    dt.trac_val = m.trac_val + 3 * t0;
  } else {
    dt.ntrac = 0;
    dt.trac_face = nullptr;
    dt.trac_val = nullptr;
  }
}

__global__ void __launch_bounds__(128)
    hex_xpt_kernel(ElemParams ep, MeshView m, ColorRange cr,
                   const double *__restrict__ vars, int func, KsStats ks,
                   double coef, const double *__restrict__ psi, double scale,
                   double lambda, double *__restrict__ dfdX) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 24LL * cr.count) return;
  const int e = cr.elem_list[idx / 24], kc = (int)(idx % 24);
  HexXptData dt;
  int nodes[8];
  hex_xpt_load(m, e, vars, psi, dt, nodes);
  const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
  const double val =
      hex_xpt_forward(ep, dt, kc, func, kk, coef, scale, lambda);
  dfdX[3 * nodes[kc / 3] + kc % 3] += val;
}

__global__ void __launch_bounds__(128)
    hex_xpt_rev_kernel(ElemParams ep, MeshView m, ColorRange cr,
                       const double *__restrict__ vars, int func, KsStats ks,
                       double coef, const double *__restrict__ psi,
                       double scale, double lambda,
                       double *__restrict__ dfdX) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= cr.count) return;
  const int e = cr.elem_list[idx];
  HexXptData dt;
  int nodes[8];
  hex_xpt_load(m, e, vars, psi, dt, nodes);
  const KsStats kk = m.elem_seg ? m.seg_ks[m.elem_seg[e]] : ks;
  double dX[24];
  for (int i = 0; i < 24; i++) dX[i] = 0.0;
  hex_xpt_reverse(ep, dt, func, kk, coef, scale, lambda, dX);
  for (int i = 0; i < 24; i++) dfdX[3 * nodes[i / 3] + i % 3] += dX[i];
}

// Fixed-geometry class table (geo_plan.h): TACSSolidConstitutive's stress
// is t C e, so K(t) = t K1 with K1 = sum_q detXd_q B_q^T C B_q, formed in
// the closed isotropic form of the team kernel at t = 1.  One warp per
// representative element writes the 64 node blocks (a, b) of 3 x 3; pairs
// a <= b are formed and mirrored (K1 exactly symmetric).
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    hex_geo_build_kernel(ElemParams ep, MeshView m,
                         const int *__restrict__ reps, int nreps,
                         double *__restrict__ table) {
  __shared__ HexSmem smem[WARPS];
  HexSmem &S = smem[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const int nw = gridDim.x * WARPS;
  const HexC c = hex_c(ep);
  for (int cl = gw; cl < nreps; cl += nw) {
    hex_load(S, m, reps[cl], nullptr, nullptr, lane);
    hex_geometry(S, lane);
    double *out = table + (size_t)cl * 576;
    for (int p = lane; p < 36; p += 32) {
      const int a = c_pair[p][0], b = c_pair[p][1];
      double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int q = 0; q < 8; q++) {
        const double wq = S.det[q];
        const double ga[3] = {wq * S.Nx[q][3 * a], wq * S.Nx[q][3 * a + 1],
                              wq * S.Nx[q][3 * a + 2]};
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) M[3 * i + j] += ga[i] * S.Nx[q][3 * b + j];
      }
      const double tr = M[0] + M[4] + M[8];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          const double k = c.c1 * M[3 * i + j] + c.G * M[3 * j + i] +
                           (i == j ? c.G * tr : 0.0);
          out[(8 * a + b) * 9 + 3 * i + j] = k;
          out[(8 * b + a) * 9 + 3 * j + i] = k;
        }
    }
    __syncwarp();
  }
}

constexpr int kWarps = 8;

int grid_for(int count) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int need = (count + kWarps - 1) / kWarps;
  int cap = sms * 4;
  if (need < 1) need = 1;
  return need < cap ? need : cap;
}

}  // namespace

void launch_hex_assembly(const ElemParams &ep, const MeshView &m,
                         ColorRange cr, const double *vars, double lambda,
                         double *res, double *mat, int transpose,
                         cudaStream_t s) {
  if (cr.count <= 0) return;
  (void)transpose;  // K is symmetric by construction (mirrored blocks)
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int grid = (cr.count + kHexTeamsPerCta - 1) / kHexTeamsPerCta;
  if (grid > sms * 16) grid = sms * 16;
  hex_team_assembly_kernel<<<grid, 64, 0, s>>>(ep, m, cr, vars, lambda, res,
                                               mat);
}
void launch_hex_geo_build(const ElemParams &ep, const MeshView &m,
                          const int *reps, int nreps, double *table,
                          cudaStream_t s) {
  if (nreps <= 0) return;
  hex_geo_build_kernel<kWarps><<<grid_for(nreps), kWarps * 32, 0, s>>>(
      ep, m, reps, nreps, table);
}
void launch_hex_points(const ElemParams &ep, const MeshView &m,
                       const double *vars, double *elem_fail,
                       double *elem_wdet, double *elem_sed, cudaStream_t s) {
  if (m.nelem <= 0) return;
  hex_points_kernel<kWarps><<<grid_for(m.nelem), kWarps * 32, 0, s>>>(
      ep, m, vars, elem_fail, elem_wdet, elem_sed);
}
void launch_hex_sv_sens(const ElemParams &ep, const MeshView &m,
                        ColorRange cr, const double *vars, int func,
                        KsStats ks, double alpha, double *dfdu,
                        cudaStream_t s) {
  if (cr.count <= 0) return;
  hex_sv_kernel<kWarps><<<grid_for(cr.count), kWarps * 32, 0, s>>>(
      ep, m, cr, vars, func, ks, alpha, dfdu);
}
void launch_hex_dv(const ElemParams &ep, const MeshView &m, const double *vars,
                   int func, KsStats ks, double coef, const double *psi,
                   double scale, double *out, cudaStream_t s) {
  if (m.nelem <= 0) return;
  hex_dv_kernel<kWarps><<<grid_for(m.nelem), kWarps * 32, 0, s>>>(
      ep, m, vars, func, ks, coef, psi, scale, out);
}

void launch_hex_xpt(const ElemParams &ep, const MeshView &m, ColorRange cr,
                    const double *vars, int func, KsStats ks, double coef,
                    const double *psi, double scale, double lambda,
                    double *dfdX, int reverse, cudaStream_t s) {
  if (cr.count <= 0) return;
  if (reverse) {
    hex_xpt_rev_kernel<<<(unsigned)((cr.count + 127) / 128), 128, 0, s>>>(
        ep, m, cr, vars, func, ks, coef, psi, scale, lambda, dfdX);
    return;
  }
  const long long n = 24LL * cr.count;
  hex_xpt_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
      ep, m, cr, vars, func, ks, coef, psi, scale, lambda, dfdX);
}

}  // namespace tg
