// Launches of the multifrontal block Cholesky kernels (direct_kernels.cuh).
#include <algorithm>
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
                                  int count, const double *A, int zchunks,
                                  int nchild, int ychunks, cudaStream_t s) {
  if (count <= 0) return;
  direct_zero_kernel<T>
      <<<dim3(count, zchunks < 65535 ? zchunks : 65535), 256, 0, s>>>(
          v, sn, count);
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
void launch_direct_inverses(const DirectView &v, const int *inv_sn,
                            const int *inv_k0, int count, cudaStream_t s) {
  if (count <= 0) return;
  direct_inverse_kernel<T><<<count, 32, 0, s>>>(v, inv_sn, inv_k0, count);
}

size_t direct_panel_smem(size_t elem) {
  return elem * kDirectTrsmRows * (kDirectPanel + 1);
}

template <class T>
void launch_direct_panel_step(const DirectView &v, const int *sn, int count,
                              const int *tprefix, int tiles,
                              const int *rprefix, int rblocks, int k0,
                              int tile, int *fail, cudaStream_t s) {
  if (count <= 0) return;
  direct_panel_kernel<T><<<count, 256, 0, s>>>(v, sn, count, k0, fail);
  if (rblocks > 0)
    direct_trsm_kernel<T><<<rblocks, 256, direct_panel_smem(sizeof(T)), s>>>(
        v, sn, rprefix, count, k0);
  if (tiles <= 0) return;
  if (tile == 64)
    direct_trailing_kernel<T, 64><<<tiles, 256, 0, s>>>(v, sn, tprefix,
                                                         count, k0);
  else
    direct_trailing_kernel<T, 32><<<tiles, 256, 0, s>>>(v, sn, tprefix,
                                                         count, k0);
}

// the solves' kernels for NR = 1, 2 or 4 right-hand sides at once; a
// level whose fronts have at most 128 rows takes CTAs of 64 threads (more
// of them resident per SM, beside the smaller shared memory)
static int plain_threads(int max_front) {
  return max_front <= 128 ? 64 : kDirectPlainThreads;
}
template <class T>
static void forward_plain(int nr, dim3 g, int nt, size_t smem, cudaStream_t s,
                          const DirectView &v, const int *sn, int count,
                          T *y, T *contrib) {
  if (nr == 4)
    direct_forward_kernel<T, 4><<<g, nt, smem, s>>>(v, sn, count, y, contrib);
  else if (nr == 2)
    direct_forward_kernel<T, 2><<<g, nt, smem, s>>>(v, sn, count, y, contrib);
  else
    direct_forward_kernel<T, 1><<<g, nt, smem, s>>>(v, sn, count, y, contrib);
}
template <class T>
static void backward_plain(int nr, dim3 g, int nt, size_t smem,
                           cudaStream_t s, const DirectView &v, const int *sn,
                           int count, const T *y, T *x) {
  if (nr == 4)
    direct_backward_kernel<T, 4><<<g, nt, smem, s>>>(v, sn, count, y, x);
  else if (nr == 2)
    direct_backward_kernel<T, 2><<<g, nt, smem, s>>>(v, sn, count, y, x);
  else
    direct_backward_kernel<T, 1><<<g, nt, smem, s>>>(v, sn, count, y, x);
}

size_t direct_solve_smem(int front, int nr, size_t elem) {
  return elem * ((size_t)front * nr + direct_plain_extra(nr, (int)elem));
}

template <class T>
void launch_direct_forward(const DirectView &v, const int *sn, int count,
                           int max_front, int nr, T *y, T *contrib,
                           cudaStream_t s) {
  if (count <= 0) return;
  forward_plain<T>(nr, dim3(count), plain_threads(max_front),
                   direct_solve_smem(max_front, nr, sizeof(T)), s, v, sn,
                   count, y, contrib);
}

template <class T>
void launch_direct_backward(const DirectView &v, const int *sn, int count,
                            int max_front, int nr, const T *y, T *x,
                            cudaStream_t s) {
  if (count <= 0) return;
  backward_plain<T>(nr, dim3(count), plain_threads(max_front),
                    direct_solve_smem(max_front, nr, sizeof(T)), s, v, sn,
                    count, y, x);
}

// Large fronts: ncl CTAs per front in one thread-block cluster; shared
// memory for the rank owning the most rows.
size_t direct_cluster_smem(int max_front, int nr, size_t elem, int ncl) {
  const int nbk = (max_front + 31) / 32;
  const int mine = (nbk + ncl - 1) / ncl;
  return elem * ((size_t)mine * 32 * nr);
}

template <class K, class... Args>
static cudaError_t cluster_launch_dk(K kernel, int count, int ncl,
                                     size_t smem, cudaStream_t s,
                                     Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(count * ncl));
  cfg.blockDim = dim3(kDirectClusterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ncl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <class T>
void launch_direct_forward_cluster(const DirectView &v, const int *sn,
                                   int count, int max_front, int nr, int ncl,
                                   T *y, T *contrib, cudaStream_t s) {
  if (count <= 0) return;
  const size_t smem = direct_cluster_smem(max_front, nr, sizeof(T), ncl);
  if (nr == 4)
    cluster_launch_dk(direct_forward_cluster_kernel<T, 4>, count, ncl, smem,
                      s, v, sn, count, ncl, y, contrib);
  else if (nr == 2)
    cluster_launch_dk(direct_forward_cluster_kernel<T, 2>, count, ncl, smem,
                      s, v, sn, count, ncl, y, contrib);
  else
    cluster_launch_dk(direct_forward_cluster_kernel<T, 1>, count, ncl, smem,
                      s, v, sn, count, ncl, y, contrib);
}

template <class T>
void launch_direct_bwd_gemv(const DirectView &v, const int *sn,
                            const int *tprefix, const int64_t *poff,
                            int count, int total, int nr, const T *x,
                            T *part, cudaStream_t s) {
  if (count <= 0 || total <= 0) return;
  const unsigned g = (unsigned)((total + 7) / 8);
  if (nr == 4)
    direct_bwd_gemv_kernel<T, 4><<<g, 256, 0, s>>>(v, sn, tprefix, poff,
                                                   count, total, x, part);
  else if (nr == 2)
    direct_bwd_gemv_kernel<T, 2><<<g, 256, 0, s>>>(v, sn, tprefix, poff,
                                                   count, total, x, part);
  else
    direct_bwd_gemv_kernel<T, 1><<<g, 256, 0, s>>>(v, sn, tprefix, poff,
                                                   count, total, x, part);
}

template <class T>
void launch_direct_backward_cluster(const DirectView &v, const int *sn,
                                    const int64_t *poff, int count,
                                    int max_front, int nr, int ncl,
                                    const T *y, T *x, const T *part,
                                    cudaStream_t s) {
  if (count <= 0) return;
  const size_t smem = direct_cluster_smem(max_front, nr, sizeof(T), ncl);
  if (nr == 4)
    cluster_launch_dk(direct_backward_cluster_kernel<T, 4>, count, ncl, smem,
                      s, v, sn, poff, count, ncl, y, x, part);
  else if (nr == 2)
    cluster_launch_dk(direct_backward_cluster_kernel<T, 2>, count, ncl, smem,
                      s, v, sn, poff, count, ncl, y, x, part);
  else
    cluster_launch_dk(direct_backward_cluster_kernel<T, 1>, count, ncl, smem,
                      s, v, sn, poff, count, ncl, y, x, part);
}

// whether the device schedules the solve clusters of ncl CTAs (at least
// one active), asked with the dynamic shared memory of a 32 k-row front
// (the attribute set first: with the kernel's static shared memory it
// passes 48 KB; clusters above 8 CTAs also need the non-portable size
// allowed, which set_solve_smem sets on every cluster kernel)
bool direct_cluster_solve_ok(int ncl) {
  const size_t bytes = direct_cluster_smem(1 << 15, 1, sizeof(double), ncl);
  if (ncl > 8 &&
      cudaFuncSetAttribute(
          (const void *)direct_forward_cluster_kernel<double, 1>,
          cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (cudaFuncSetAttribute(
          (const void *)direct_forward_cluster_kernel<double, 1>,
          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ncl);
  cfg.blockDim = dim3(kDirectClusterThreads);
  cfg.dynamicSmemBytes = bytes;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ncl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(
      &n, (void *)direct_forward_cluster_kernel<double, 1>, &cfg);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

template <class T>
void launch_direct_rhs(int n, int bs, const int *perm, const T *b, T *ypos,
                       int nrhs, size_t ld, cudaStream_t s) {
  direct_rhs_kernel<T><<<grid_1d((size_t)n * bs * nrhs), 256, 0, s>>>(
      n, bs, perm, b, ypos, nrhs, ld);
}

template <class T>
void launch_direct_bc_couple(const DirectBc &c, int bs, const T *a,
                             const T *b, T *ypos, int nrhs, size_t ld,
                             cudaStream_t s) {
  if (c.nrow == 0) return;
  direct_bc_couple_kernel<T>
      <<<grid_1d((size_t)c.nrow * bs * nrhs), 256, 0, s>>>(
          c.nrow, bs, c.row, c.pos, c.ptr, c.blk, c.cols, c.bcmask, a, b,
          ypos, nrhs, ld);
}

template <class T>
void launch_direct_unpermute(int n, int bs, const int *perm, const T *xpos,
                             T *x, int nrhs, size_t ld, cudaStream_t s) {
  direct_unpermute_kernel<T><<<grid_1d((size_t)n * bs * nrhs), 256, 0, s>>>(
      n, bs, perm, xpos, x, nrhs, ld);
}

// Dynamic shared memory of the solve kernels for fronts of up to
// plain_front rows on one CTA and cluster_front rows on a cluster, nr
// right-hand sides at most.  Per device (the attribute belongs
// to the kernel on each device); the limits only grow, and are recorded
// only once every call succeeded.
template <class T, int NR>
static cudaError_t set_solve_smem(int plain_front, int cluster_front) {
  const size_t pb = direct_solve_smem(plain_front, NR, sizeof(T));
  const size_t cb =
      direct_cluster_smem(cluster_front, NR, sizeof(T), kDirectSolveCluster);
  const void *plain[2] = {(const void *)direct_forward_kernel<T, NR>,
                          (const void *)direct_backward_kernel<T, NR>};
  const void *clus[2] = {(const void *)direct_forward_cluster_kernel<T, NR>,
                         (const void *)direct_backward_cluster_kernel<T, NR>};
  // set whatever the size: the kernels' static shared memory (staged
  // rows, inverse blocks) counts against the same 48 KB default
  cudaError_t e = cudaSuccess;
  for (const void *k : plain)
    if ((e = cudaFuncSetAttribute(k,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)pb)) != cudaSuccess)
      return e;
  if (cluster_front > 0)
    for (const void *k : clus) {
      if ((e = cudaFuncSetAttribute(k,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)cb)) != cudaSuccess)
        return e;
      // wide clusters, where the device schedules them (a failure here
      // only leaves the levels on 8-CTA clusters)
      if (cudaFuncSetAttribute(k,
                               cudaFuncAttributeNonPortableClusterSizeAllowed,
                               1) != cudaSuccess)
        cudaGetLastError();
    }
  return e;
}

cudaError_t direct_set_smem(int plain_front, int cluster_front, int max_nr) {
  constexpr int kMaxDevices = 64;
  static int set_plain[kMaxDevices] = {}, set_cluster[kMaxDevices] = {},
             set_nr[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (plain_front <= set_plain[dev] && cluster_front <= set_cluster[dev] &&
      max_nr <= set_nr[dev])
    return cudaSuccess;
  if (set_nr[dev] == 0) {  // first call on this device: the row solves
    const size_t pb = direct_panel_smem(sizeof(double));
    if ((e = cudaFuncSetAttribute(
             (const void *)direct_trsm_kernel<double>,
             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pb)) !=
        cudaSuccess)
      return e;
    if ((e = cudaFuncSetAttribute(
             (const void *)direct_trsm_kernel<float>,
             cudaFuncAttributeMaxDynamicSharedMemorySize,
             (int)direct_panel_smem(sizeof(float)))) != cudaSuccess)
      return e;
  }
  const int pf = std::max(plain_front, set_plain[dev]);
  const int cf = std::max(cluster_front, set_cluster[dev]);
  const int mn = std::max(max_nr, set_nr[dev]);
  if ((e = set_solve_smem<double, 1>(pf, cf)) != cudaSuccess) return e;
  if ((e = set_solve_smem<float, 1>(pf, cf)) != cudaSuccess) return e;
  if (mn >= 2) {
    if ((e = set_solve_smem<double, 2>(pf, cf)) != cudaSuccess) return e;
    if ((e = set_solve_smem<float, 2>(pf, cf)) != cudaSuccess) return e;
  }
  if (mn >= 4) {
    if ((e = set_solve_smem<double, 4>(pf, cf)) != cudaSuccess) return e;
    if ((e = set_solve_smem<float, 4>(pf, cf)) != cudaSuccess) return e;
  }
  set_plain[dev] = pf;
  set_cluster[dev] = cf;
  set_nr[dev] = mn;
  return cudaSuccess;
}

#define TG_DIRECT_INSTANTIATE(T)                                            \
  template void launch_direct_level_assemble<T>(const DirectView &,        \
                                                const int *, int,          \
                                                const double *, int, int,  \
                                                int, cudaStream_t);        \
  template void launch_direct_inverses<T>(const DirectView &, const int *, \
                                         const int *, int, cudaStream_t);  \
  template void launch_direct_factor_small<T>(const DirectView &,          \
                                              const int *, int, int *,     \
                                              cudaStream_t);               \
  template void launch_direct_panel_step<T>(const DirectView &, const int *, \
                                            int, const int *, int,           \
                                            const int *, int, int, int,      \
                                            int *, cudaStream_t);            \
  template void launch_direct_forward<T>(const DirectView &, const int *,  \
                                         int, int, int, T *, T *,          \
                                         cudaStream_t);                    \
  template void launch_direct_backward<T>(const DirectView &, const int *, \
                                          int, int, int, const T *, T *,   \
                                          cudaStream_t);                   \
  template void launch_direct_forward_cluster<T>(                          \
      const DirectView &, const int *, int, int, int, int, T *, T *,       \
      cudaStream_t);                                                        \
  template void launch_direct_bwd_gemv<T>(                                 \
      const DirectView &, const int *, const int *, const int64_t *, int,  \
      int, int, const T *, T *, cudaStream_t);                              \
  template void launch_direct_backward_cluster<T>(                         \
      const DirectView &, const int *, const int64_t *, int, int, int, int,\
      const T *, T *, const T *, cudaStream_t);                             \
  template void launch_direct_rhs<T>(int, int, const int *, const T *,     \
                                     T *, int, size_t, cudaStream_t);      \
  template void launch_direct_bc_couple<T>(const DirectBc &, int,          \
                                           const T *, const T *, T *, int, \
                                           size_t, cudaStream_t);          \
  template void launch_direct_unpermute<T>(int, int, const int *,          \
                                           const T *, T *, int, size_t,    \
                                           cudaStream_t);
TG_DIRECT_INSTANTIATE(double)
TG_DIRECT_INSTANTIATE(float)

}  // namespace tg
