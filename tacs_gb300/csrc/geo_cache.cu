// Fixed-geometry assembly for sm_103a: the BCSR Jacobian and the residual
// of linear elements from the class table (geo_plan.h), for repeated
// assemblies at fixed node coordinates (an optimisation loop changes only
// the element scale t and the state u).
//
//   K_ij = sum over the slot's contributions (e, a, b) of
//          t_e K1[cls e](a, b) + t_e^3 K3[cls e](a, b)
//   R_i  = sum_j K_ij u_j + lambda f0_i
//
// the same K and R as TACSAssembler::assembleJacobian / assembleRes
// (src/TACSAssembler.cpp:4133-4405) with the row constraints of
// TACSParallelMat::applyBCs / TACSBVec::applyBCs.  No element math runs
// here: the kernel streams the BCSR values out once (no read-modify-write),
// so its bound is the HBM write of the matrix and the FP64 FMAs of the
// block sums.
//
// One warp per 32 consecutive block rows, lane = row; the warp walks the
// rows' k-th blocks together (k = 0 .. longest row - 1), so on structured
// meshes all lanes of a step have the same number of contributions and the
// FP64 FMAs carry no idle lanes.  Entries that are zero in every class
// are not summed (a compile-time pattern, chosen by the host from the
// table): a flat plate's membrane-bending coupling entries are exactly
// zero.  Each step's 32 blocks are staged in shared
// memory and written back with consecutive lanes on consecutive doubles.
// The residual sums over k in registers: every output has one fixed
// summation order (deterministic).
#include "tg_internal.h"

namespace tg {
namespace {

constexpr int kGeoWarps = 4;

// Entry patterns (bit r * bs + c) of the coefficient blocks.  A flat
// shell in a coordinate plane couples (u, v, theta_z) and (w, theta_x,
// theta_y) only, and its bending part only (theta_x, theta_y): 18 and 4 of
// the 36 entries.  The kernel is instantiated per pattern so that the
// skipped entries cost no instruction at all (a run-time mask still issues
// predicated FMAs); the host picks the pattern that covers the table's
// non-zero entries.
constexpr unsigned long long kAll36 = (1ull << 36) - 1, kAll9 = (1ull << 9) - 1;
constexpr unsigned long long kFlatK1 =
    (0x23ull << 0) | (0x23ull << 6) | (0x1Cull << 12) | (0x1Cull << 18) |
    (0x1Cull << 24) | (0x23ull << 30);
constexpr unsigned long long kFlatK3 = (0x18ull << 18) | (0x18ull << 24);

template <int BS, int NCOEF, int NPE, unsigned long long M1,
          unsigned long long M3>
__global__ void __launch_bounds__(kGeoWarps * 32)
    geo_assembly_kernel(GeoView g, const double *__restrict__ vars,
                        double lambda, int apply_bcs,
                        double *__restrict__ res, double *__restrict__ vals) {
  constexpr int B2 = BS * BS;
  constexpr int STRIDE = B2 + 1;  // odd: conflict-free 8-byte staging
  constexpr int NB = NPE * NPE;
  constexpr int CLS = NCOEF * NB * B2;
  __shared__ double stage[kGeoWarps][32 * STRIDE];
  __shared__ int sslot[kGeoWarps][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = blockIdx.x * kGeoWarps + warp;
  if (gw >= g.nwarps) return;  // whole warps leave together
  const int row = gw * 32 + lane;
  const bool rv = row < g.nrows;
  const int p0 = rv ? g.rowp[row] : 0, p1 = rv ? g.rowp[row + 1] : 0;
  const int kmax = g.warp_kmax[gw];
  const int bcm = (rv && apply_bcs) ? g.node_bc[row] : 0;
  constexpr unsigned long long m1 = M1, m3 = M3, mu = M1 | M3;
  double y[BS];
#pragma unroll
  for (int r = 0; r < BS; r++) y[r] = 0.0;
  double *st = stage[warp];
  for (int k = 0; k < kmax; k++) {
    const int s = p0 + k;
    const bool sv = s < p1;
    double acc[B2];
#pragma unroll
    for (int q = 0; q < B2; q++) acc[q] = 0.0;
    int j = 0;
    if (sv) {
      j = g.cols[s];
      const int c1 = g.cptr[s + 1];
      for (int c = g.cptr[s]; c < c1; c++) {
        const int code = g.contrib[c];
        const int e = code >> 6, ab = code & 63;
        const double te = g.thick[e];
        const double *K = g.table + (size_t)g.cls[e] * CLS + ab * B2;
        if (NCOEF == 2) {
          const double t3 = te * te * te;
#pragma unroll
          for (int q = 0; q < B2; q++) {
            if ((m1 >> q) & 1ull) acc[q] = fma(te, K[q], acc[q]);
            if ((m3 >> q) & 1ull) acc[q] = fma(t3, K[NB * B2 + q], acc[q]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < B2; q++)
            if ((m1 >> q) & 1ull) acc[q] = fma(te, K[q], acc[q]);
        }
      }
      if (res) {
        double uj[BS];
#pragma unroll
        for (int c = 0; c < BS; c++) uj[c] = vars ? vars[BS * j + c] : 0.0;
#pragma unroll
        for (int r = 0; r < BS; r++)
#pragma unroll
          for (int c = 0; c < BS; c++)
            if ((mu >> (BS * r + c)) & 1ull)
              y[r] = fma(acc[BS * r + c], uj[c], y[r]);
      }
      // constrained rows: zero, unit diagonal (BCSRMat::zeroRow)
      if (bcm) {
#pragma unroll
        for (int r = 0; r < BS; r++)
          if ((bcm >> r) & 1)
#pragma unroll
            for (int c = 0; c < BS; c++)
              acc[BS * r + c] = (j == row && r == c) ? 1.0 : 0.0;
      }
    }
    if (vals) {
#pragma unroll
      for (int q = 0; q < B2; q++) st[lane * STRIDE + q] = acc[q];
      sslot[warp][lane] = sv ? s : -1;
      __syncwarp();
      for (int x = lane; x < 32 * B2; x += 32) {
        const int b = x / B2, q = x - B2 * b;
        const int sb = sslot[warp][b];
        if (sb >= 0) vals[(size_t)sb * B2 + q] = st[b * STRIDE + q];
      }
      __syncwarp();
    }
  }
  if (res && rv) {
#pragma unroll
    for (int r = 0; r < BS; r++) {
      const size_t d = (size_t)BS * row + r;
      double v = y[r] + lambda * g.f0[d];
      if ((bcm >> r) & 1) v = vars ? vars[d] : 0.0;
      res[d] = v;
    }
  }
}

template <int B2>
__global__ void geo_mask_kernel(const double *__restrict__ table, int ncoef,
                                long long nblocks,
                                unsigned long long *__restrict__ masks) {
  const long long blk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (blk >= nblocks) return;
  // blocks are ordered (class, coef, a, b): coef = (blk / nb) % ncoef
  const double *K = table + blk * B2;
  unsigned long long m = 0;
  for (int q = 0; q < B2; q++)
    if (K[q] != 0.0) m |= 1ull << q;
  if (m) atomicOr(&masks[(blk / (B2 == 36 ? 16 : 64)) % ncoef], m);
}

template <int BS, int NCOEF, int NPE, unsigned long long M1,
          unsigned long long M3>
void launch_geo(const GeoView &g, const double *vars, double lambda,
                int apply_bcs, double *res, double *vals, cudaStream_t s) {
  const int grid = (g.nwarps + kGeoWarps - 1) / kGeoWarps;
  geo_assembly_kernel<BS, NCOEF, NPE, M1, M3>
      <<<grid, kGeoWarps * 32, 0, s>>>(g, vars, lambda, apply_bcs, res, vals);
}

}  // namespace

void launch_geo_masks(int bs, int ncoef, int nblocks_per_coef_cls, int ncls,
                      const double *table, unsigned long long *masks,
                      cudaStream_t s) {
  const long long n = (long long)ncls * ncoef * nblocks_per_coef_cls;
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (bs == 6)
    geo_mask_kernel<36><<<grid, 256, 0, s>>>(table, ncoef, n, masks);
  else
    geo_mask_kernel<9><<<grid, 256, 0, s>>>(table, ncoef, n, masks);
}

void launch_geo_assembly(int bs, const GeoView &g, const double *vars,
                         double lambda, int apply_bcs, double *res,
                         double *vals, cudaStream_t s) {
  if (g.nwarps <= 0) return;
  if (bs == 6) {
    if ((g.mask1 & ~kFlatK1) == 0 && (g.mask3 & ~kFlatK3) == 0)
      launch_geo<6, 2, 4, kFlatK1, kFlatK3>(g, vars, lambda, apply_bcs, res,
                                            vals, s);
    else
      launch_geo<6, 2, 4, kAll36, kAll36>(g, vars, lambda, apply_bcs, res,
                                          vals, s);
  } else {
    launch_geo<3, 1, 8, kAll9, 0>(g, vars, lambda, apply_bcs, res, vals, s);
  }
}

}  // namespace tg
