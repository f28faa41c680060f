// Launches of the multifrontal block Cholesky kernels (direct_kernels.cuh).
#include <cmath>

#include "direct_kernels.cuh"
#include "tg_internal.h"

namespace tg {

using namespace dk;

namespace {

int grid_1d(size_t n) {
  size_t g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > 4096) g = 4096;
  return (int)g;
}

}  // namespace

void launch_direct_level_assemble(const DirectView &v, const int *sn,
                                  int count, const double *A,
                                  cudaStream_t s) {
  if (count <= 0) return;
  direct_zero_kernel<<<count, 256, 0, s>>>(v, sn, count);
  direct_assemble_kernel<<<count, 256, 0, s>>>(v, sn, count, A);
  direct_extend_add_kernel<<<count, 256, 0, s>>>(v, sn, count);
}

void launch_direct_factor_small(const DirectView &v, const int *sn,
                                int count, int *fail, cudaStream_t s) {
  if (count <= 0) return;
  direct_factor_small_kernel<<<count, 256, 0, s>>>(v, sn, count, fail);
}

void launch_direct_factor_large(const DirectView &v, int sn, int M, int C,
                                int *fail, cudaStream_t s) {
  for (int k0 = 0; k0 < C; k0 += kPanel) {
    const int nb = C - k0 < kPanel ? C - k0 : kPanel;
    direct_panel_kernel<<<1, 256, 0, s>>>(v, sn, k0, nb, fail);
    const int rest = M - (k0 + nb);
    if (rest > 0) {
      const int tiles = (rest + kTile - 1) / kTile;
      direct_trailing_kernel<<<dim3(tiles, tiles), 256, 0, s>>>(v, sn, k0,
                                                                 nb);
    }
  }
}

void launch_direct_forward(const DirectView &v, const int *sn, int count,
                           int max_front, double *y, double *contrib,
                           cudaStream_t s) {
  if (count <= 0) return;
  direct_forward_kernel<<<count, 256, sizeof(double) * max_front, s>>>(
      v, sn, count, y, contrib);
}

void launch_direct_backward(const DirectView &v, const int *sn, int count,
                            int max_front, const double *y, double *x,
                            cudaStream_t s) {
  if (count <= 0) return;
  direct_backward_kernel<<<count, 256, sizeof(double) * max_front, s>>>(
      v, sn, count, y, x);
}

void launch_direct_bc_mask(int n, int bs, const int *bcmask, const double *b,
                           double *out, cudaStream_t s) {
  direct_bc_mask_kernel<<<grid_1d((size_t)n * bs), 256, 0, s>>>(n, bs, bcmask,
                                                                b, out);
}

void launch_direct_rhs(int n, int bs, const int *perm, const double *b,
                       const double *Kpb, const double *pb, double *ypos,
                       cudaStream_t s) {
  direct_rhs_kernel<<<grid_1d((size_t)n * bs), 256, 0, s>>>(n, bs, perm, b,
                                                            Kpb, pb, ypos);
}

void launch_direct_unpermute(int n, int bs, const int *perm,
                             const double *xpos, double *x, cudaStream_t s) {
  direct_unpermute_kernel<<<grid_1d((size_t)n * bs), 256, 0, s>>>(n, bs, perm,
                                                                  xpos, x);
}

void direct_set_smem(int max_front) {
  // the attribute only grows: every factorisation of the process keeps
  // its solve workspace
  static int set = 48 * 1024;
  const int bytes = (int)sizeof(double) * max_front;
  if (bytes > set) {
    set = bytes;
    cudaFuncSetAttribute(direct_forward_kernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(direct_backward_kernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  }
}

}  // namespace tg
