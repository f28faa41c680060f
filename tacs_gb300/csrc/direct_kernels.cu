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

template <class T>
void launch_direct_level_assemble(const DirectView &v, const int *sn,
                                  int count, const double *A, int nchild,
                                  int ychunks, cudaStream_t s) {
  if (count <= 0) return;
  direct_zero_kernel<T><<<count, 256, 0, s>>>(v, sn, count);
  direct_assemble_kernel<T><<<count, 256, 0, s>>>(v, sn, count, A);
  if (ychunks > 0)
    for (int k = 0; k < nchild; k++)
      direct_extend_add_kernel<T>
          <<<dim3(count, ychunks), 256, 0, s>>>(v, sn, count, k);
}

template <class T>
void launch_direct_factor_small(const DirectView &v, const int *sn,
                                int count, int *fail, cudaStream_t s) {
  if (count <= 0) return;
  direct_factor_small_kernel<T><<<count, 256, 0, s>>>(v, sn, count, fail);
}

template <class T>
void launch_direct_panel_step(const DirectView &v, const int *sn, int count,
                              const int *tprefix, int tiles,
                              const int *rprefix, int rblocks, int k0,
                              int *fail, cudaStream_t s) {
  if (count <= 0) return;
  direct_panel_kernel<T><<<count, 256, 0, s>>>(v, sn, count, k0, fail);
  if (rblocks > 0)
    direct_trsm_kernel<T><<<rblocks, 256, 0, s>>>(v, sn, rprefix, count, k0);
  if (tiles > 0)
    direct_trailing_kernel<T><<<tiles, 256, 0, s>>>(v, sn, tprefix, count,
                                                     k0);
}

template <class T>
void launch_direct_forward(const DirectView &v, const int *sn, int count,
                           int max_front, T *y, T *contrib, cudaStream_t s) {
  if (count <= 0) return;
  direct_forward_kernel<T>
      <<<count, 256, sizeof(T) * (max_front + kDirectSolveDiag), s>>>(
          v, sn, count, y, contrib);
}

template <class T>
void launch_direct_backward(const DirectView &v, const int *sn, int count,
                            int max_front, const T *y, T *x, cudaStream_t s) {
  if (count <= 0) return;
  direct_backward_kernel<T>
      <<<count, 256, sizeof(T) * (max_front + kDirectSolveDiag), s>>>(
          v, sn, count, y, x);
}

// Large fronts: kDirectSolveCluster CTAs per front in one thread-block
// cluster; shared memory for the rank owning the most rows.
static size_t cluster_smem(int max_front, size_t elem) {
  const int nbk = (max_front + 31) / 32;
  const int mine = (nbk + kDirectSolveCluster - 1) / kDirectSolveCluster;
  return elem * ((size_t)mine * 32 + kDirectSolveDiag);
}

template <class K, class... Args>
static cudaError_t cluster_launch_dk(K kernel, int count, size_t smem,
                                     cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(count * kDirectSolveCluster));
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kDirectSolveCluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <class T>
void launch_direct_forward_cluster(const DirectView &v, const int *sn,
                                   int count, int max_front, T *y, T *contrib,
                                   cudaStream_t s) {
  if (count <= 0) return;
  cluster_launch_dk(direct_forward_cluster_kernel<T>, count,
                    cluster_smem(max_front, sizeof(T)), s, v, sn, count, y,
                    contrib);
}

template <class T>
void launch_direct_backward_cluster(const DirectView &v, const int *sn,
                                    int count, int max_front, const T *y,
                                    T *x, cudaStream_t s) {
  if (count <= 0) return;
  cluster_launch_dk(direct_backward_cluster_kernel<T>, count,
                    cluster_smem(max_front, sizeof(T)), s, v, sn, count, y, x);
}

// whether the device schedules the solve clusters (at least one active)
bool direct_cluster_solve_ok() {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kDirectSolveCluster);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = cluster_smem(1 << 15, sizeof(double));
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kDirectSolveCluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(
      &n, (void *)direct_forward_cluster_kernel<double>, &cfg);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

template <class T>
void launch_direct_bc_mask(int n, int bs, const int *bcmask, const T *b,
                           T *out, cudaStream_t s) {
  direct_bc_mask_kernel<T><<<grid_1d((size_t)n * bs), 256, 0, s>>>(
      n, bs, bcmask, b, out);
}

template <class T>
void launch_direct_rhs(int n, int bs, const int *perm, const T *b,
                       const T *Kpb, const T *pb, T *ypos, cudaStream_t s) {
  direct_rhs_kernel<T><<<grid_1d((size_t)n * bs), 256, 0, s>>>(
      n, bs, perm, b, Kpb, pb, ypos);
}

template <class T>
void launch_direct_unpermute(int n, int bs, const int *perm, const T *xpos,
                             T *x, cudaStream_t s) {
  direct_unpermute_kernel<T><<<grid_1d((size_t)n * bs), 256, 0, s>>>(
      n, bs, perm, xpos, x);
}

cudaError_t direct_set_smem(int max_front) {
  // per device (the attribute belongs to the kernel on each device); the
  // limit only grows, and is recorded only once every call succeeded
  constexpr int kMaxDevices = 64;
  static int set[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  const int bytes = (int)sizeof(double) * (max_front + kDirectSolveDiag);
  if (bytes <= 48 * 1024 || bytes <= set[dev]) return cudaSuccess;
  const void *ks[4] = {(const void *)direct_forward_kernel<double>,
                       (const void *)direct_backward_kernel<double>,
                       (const void *)direct_forward_kernel<float>,
                       (const void *)direct_backward_kernel<float>};
  for (const void *k : ks) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             bytes);
    if (e != cudaSuccess) return e;
  }
  set[dev] = bytes;
  return cudaSuccess;
}

#define TG_DIRECT_INSTANTIATE(T)                                            \
  template void launch_direct_level_assemble<T>(const DirectView &,        \
                                                const int *, int,          \
                                                const double *, int, int,  \
                                                cudaStream_t);             \
  template void launch_direct_factor_small<T>(const DirectView &,          \
                                              const int *, int, int *,     \
                                              cudaStream_t);               \
  template void launch_direct_panel_step<T>(const DirectView &, const int *, \
                                            int, const int *, int,           \
                                            const int *, int, int, int *,    \
                                            cudaStream_t);                   \
  template void launch_direct_forward<T>(const DirectView &, const int *,  \
                                         int, int, T *, T *, cudaStream_t); \
  template void launch_direct_backward<T>(const DirectView &, const int *, \
                                          int, int, const T *, T *,        \
                                          cudaStream_t);                   \
  template void launch_direct_forward_cluster<T>(                          \
      const DirectView &, const int *, int, int, T *, T *, cudaStream_t);  \
  template void launch_direct_backward_cluster<T>(                         \
      const DirectView &, const int *, int, int, const T *, T *,           \
      cudaStream_t);                                                        \
  template void launch_direct_bc_mask<T>(int, int, const int *, const T *, \
                                         T *, cudaStream_t);               \
  template void launch_direct_rhs<T>(int, int, const int *, const T *,     \
                                     const T *, const T *, T *,            \
                                     cudaStream_t);                        \
  template void launch_direct_unpermute<T>(int, int, const int *,          \
                                           const T *, T *, cudaStream_t);
TG_DIRECT_INSTANTIATE(double)
TG_DIRECT_INSTANTIATE(float)

}  // namespace tg
