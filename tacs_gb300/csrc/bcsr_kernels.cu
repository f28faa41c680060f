// Block-CSR linear algebra for sm_103a: the BCSR mat-vec (FP64 / FP32,
// BCSRMatVecMult6/3, src/bpmat/BCSRMatMult6.cpp:82, BCSRMatMult3.cpp:28),
// Dirichlet row zeroing (BCSRMat::zeroRow, src/bpmat/BCSRMat.cpp:2027),
// level-scheduled block ILU(0) factor and triangular solves
// (BCSRMatFactor6/3, BCSRMatApplyLower/Upper, BCSRMatFact6.cpp:946,
// BCSRMatMult6.cpp:319-415), block Jacobi, deterministic reductions and the
// GMRES vector kernels.
#include <cmath>

#include <cooperative_groups.h>

#include "tg_internal.h"

namespace tg {
namespace {

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

int blocks_for(size_t n, int threads, int per_sm = 8) {
  size_t b = (n + threads - 1) / threads;
  size_t cap = (size_t)num_sms() * per_sm;
  if (b < 1) b = 1;
  return (int)(b < cap ? b : cap);
}

// ------------------------------------------------------------ mat-vec
// One thread per (block row, row within block): BS threads read the BS
// rows of each BSxBS block, i.e. the whole contiguous block.  NR right-hand
// sides (vectors ld apart) share each block read from memory.
template <int BS, int NR, typename T>
__global__ void __launch_bounds__(256)
    bcsr_mult_kernel(int nrows, const int *__restrict__ rowp,
                     const int *__restrict__ cols, const T *__restrict__ A,
                     const T *__restrict__ x, T *__restrict__ y, size_t ld) {
  const int per_warp = 32 / BS;
  const int lane = threadIdx.x & 31;
  const int sub = lane / BS, ii = lane - BS * sub;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  if (sub >= per_warp) return;
  for (int row = gw * per_warp + sub; row < nrows; row += nw * per_warp) {
    T acc[NR];
#pragma unroll
    for (int l = 0; l < NR; l++) acc[l] = 0;
    const int end = rowp[row + 1];
#pragma unroll 3
    for (int j = rowp[row]; j < end; j++) {
      const T *a = &A[(size_t)BS * BS * j + BS * ii];
      T av[BS];
#pragma unroll
      for (int jj = 0; jj < BS; jj++) av[jj] = a[jj];
      const size_t xo = (size_t)BS * cols[j];
#pragma unroll
      for (int l = 0; l < NR; l++) {
        const T *xx = &x[l * ld + xo];
        T s = 0;
#pragma unroll
        for (int jj = 0; jj < BS; jj++) s += av[jj] * xx[jj];
        acc[l] += s;
      }
    }
#pragma unroll
    for (int l = 0; l < NR; l++) y[l * ld + (size_t)BS * row + ii] = acc[l];
  }
}

template <int BS, typename T>
void mult_dispatch(int nrows, const int *rowp, const int *cols, const T *A,
                   const T *x, T *y, int nrhs, size_t ld, cudaStream_t s) {
  const int per_warp = 32 / BS;
  size_t warps = (nrows + per_warp - 1) / per_warp;
  int blocks = blocks_for(warps * 32, 256, 16);
  for (int l = 0; l < nrhs;) {
    const int left = nrhs - l;
    if (left >= 4) {
      bcsr_mult_kernel<BS, 4, T><<<blocks, 256, 0, s>>>(nrows, rowp, cols, A,
                                                        x + l * ld, y + l * ld,
                                                        ld);
      l += 4;
    } else if (left >= 2) {
      bcsr_mult_kernel<BS, 2, T><<<blocks, 256, 0, s>>>(nrows, rowp, cols, A,
                                                        x + l * ld, y + l * ld,
                                                        ld);
      l += 2;
    } else {
      bcsr_mult_kernel<BS, 1, T><<<blocks, 256, 0, s>>>(nrows, rowp, cols, A,
                                                        x + l * ld, y + l * ld,
                                                        ld);
      l += 1;
    }
  }
}

// ---------------------------------------------------------------- BCs
__global__ void apply_bcs_mat_kernel(int bs, int nbcs, const int *bc_nodes,
                                     const int *bc_masks, const int *rowp,
                                     const int *cols, double *A) {
  for (int i = blockIdx.x * blockDim.y + threadIdx.y; i < nbcs;
       i += gridDim.x * blockDim.y) {
    const int row = bc_nodes[i], mask = bc_masks[i];
    for (int j = rowp[row]; j < rowp[row + 1]; j++) {
      double *a = &A[(size_t)bs * bs * j];
      for (int k = threadIdx.x; k < bs * bs; k += blockDim.x) {
        const int ii = k / bs, jj = k - bs * ii;
        if (mask & (1 << ii)) {
          a[k] = (cols[j] == row && ii == jj) ? 1.0 : 0.0;
        }
      }
    }
  }
}

__global__ void apply_bcs_res_kernel(int bs, int nbcs, const int *bc_nodes,
                                     const int *bc_masks, const double *vars,
                                     double *res) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nbcs;
       i += gridDim.x * blockDim.x) {
    const int node = bc_nodes[i], mask = bc_masks[i];
    for (int k = 0; k < bs; k++)
      if (mask & (1 << k)) {
        size_t d = (size_t)bs * node + k;
        res[d] = vars ? vars[d] : 0.0;
      }
  }
}

__global__ void fill_kernel(double *x, double v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    x[i] = v;
}
__global__ void d2f_kernel(const double *x, float *y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
__global__ void f2d_kernel(const float *x, double *y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}
__global__ void gather_dv_kernel(int nelem, const int *dvnum, const double *dvs,
                                 double *thick) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nelem;
       e += gridDim.x * blockDim.x)
    if (dvnum[e] >= 0) thick[e] = dvs[dvnum[e]];
}
// dfdx[d] += sum over the elements of design variable d (element order)
__global__ void scatter_dv_kernel(int ndv, const int *dv_ptr,
                                  const int *dv_elems, const double *vals,
                                  double *dfdx) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < ndv;
       d += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = dv_ptr[d]; k < dv_ptr[d + 1]; k++) acc += vals[dv_elems[k]];
    dfdx[d] += acc;
  }
}

// ---------------------------------------------------------- reductions
// Deterministic: fixed partition into npart partial results, then one
// block combines them in a fixed tree order.
template <int OP>  // 0 sum, 1 max, 2 ks-sum
__global__ void reduce_partial_kernel(const double *x, const double *w,
                                      size_t n, const double *dmax, double ksw,
                                      double *partials) {
  __shared__ double sh[256];
  size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  size_t b = chunk * blockIdx.x, e = b + chunk < n ? b + chunk : n;
  double acc = OP == 1 ? -1e300 : 0.0;
  const double mx = (OP == 2) ? *dmax : 0.0;
  for (size_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    if (OP == 0) acc += x[i];
    else if (OP == 1) acc = x[i] > acc ? x[i] : acc;
    else if (OP == 3) acc = fabs(x[i]) > acc ? fabs(x[i]) : acc;
    else acc += w[i] * exp(ksw * (x[i] - mx));
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      if (OP == 1 || OP == 3)
        sh[threadIdx.x] = sh[threadIdx.x + s] > sh[threadIdx.x]
                                         ? sh[threadIdx.x + s]
                                         : sh[threadIdx.x];
      else sh[threadIdx.x] += sh[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}
// max |x| of k vectors n apart (blockIdx.y = vector), in the fixed
// partition of reduce_partial_kernel; the final pass writes vector v's
// maximum to out[v * stride]
__global__ void absmax_multi_partial_kernel(const double *x, size_t n,
                                            double *partials) {
  __shared__ double sh[256];
  const double *xv = x + (size_t)blockIdx.y * n;
  size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  size_t b = chunk * blockIdx.x, e = b + chunk < n ? b + chunk : n;
  double acc = 0.0;
  for (size_t i = b + threadIdx.x; i < e; i += blockDim.x)
    acc = fabs(xv[i]) > acc ? fabs(xv[i]) : acc;
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      sh[threadIdx.x] = sh[threadIdx.x + s] > sh[threadIdx.x]
                            ? sh[threadIdx.x + s]
                            : sh[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}
__global__ void absmax_multi_final_kernel(const double *partials, int npart,
                                          double *out, int stride) {
  __shared__ double sh[256];
  const double *p = partials + (size_t)blockIdx.x * npart;
  double acc = 0.0;
  for (int i = threadIdx.x; i < npart; i += blockDim.x)
    acc = p[i] > acc ? p[i] : acc;
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      sh[threadIdx.x] = sh[threadIdx.x + s] > sh[threadIdx.x]
                            ? sh[threadIdx.x + s]
                            : sh[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[(size_t)blockIdx.x * stride] = sh[0];
}
// r = b - t
__global__ void residual_kernel(const double *b, const double *t, double *r,
                                size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    r[i] = b[i] - t[i];
}
// x += c (c in FP32)
__global__ void f2d_add_kernel(const float *c, double *x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    x[i] += (double)c[i];
}
// sum over each scalar row of |A| (for the infinity norm of A)
__global__ void bcsr_row_abs_sum_kernel(int bs, int nrows,
                                        const int *__restrict__ rowp,
                                        const double *__restrict__ vals,
                                        double *__restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nrows * bs) return;
  const int i = (int)(t / bs), r = (int)(t % bs);
  const size_t b2 = (size_t)bs * bs;
  double acc = 0.0;
  for (int j = rowp[i]; j < rowp[i + 1]; j++)
    for (int q = 0; q < bs; q++) acc += fabs(vals[b2 * j + r * bs + q]);
  out[t] = acc;
}
template <int OP>
__global__ void reduce_final_kernel(const double *partials, int npart,
                                    double *out) {
  __shared__ double sh[256];
  double acc = OP == 1 ? -1e300 : 0.0;
  for (int i = threadIdx.x; i < npart; i += blockDim.x) {
    if (OP == 1) acc = partials[i] > acc ? partials[i] : acc;
    else acc += partials[i];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      if (OP == 1) sh[threadIdx.x] = sh[threadIdx.x + s] > sh[threadIdx.x]
                                         ? sh[threadIdx.x + s]
                                         : sh[threadIdx.x];
      else sh[threadIdx.x] += sh[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// --------------------------------------------------------------- ILU(0)
// Block inverse with partial pivoting then the explicit inverse, column by
// column: BMatComputeInverse (src/bpmat/BCSRMatMult.cpp:308-386).
// Lane 0 factors; lanes 0..n-1 form one column of the inverse each.
template <int BS, typename T>
__device__ void warp_block_inverse(T *a, T *lu, int *piv, int lane,
                                   int *fail_flag, int row) {
  if (lane == 0) {
    for (int k = 0; k < BS * BS; k++) lu[k] = a[k];
    int fail = 0;
    for (int k = 0; k < BS - 1 && !fail; k++) {
      int nk = BS * k, r = k;
      double maxv = fabs((double)lu[nk + k]);
      for (int j = k + 1; j < BS; j++) {
        double t = fabs((double)lu[BS * j + k]);
        if (t > maxv) {
          maxv = t;
          r = j;
        }
      }
      piv[k] = r;
      if (r != k)
        for (int j = 0; j < BS; j++) {
          T t = lu[nk + j];
          lu[nk + j] = lu[BS * r + j];
          lu[BS * r + j] = t;
        }
      if (lu[nk + k] == (T)0) {
        fail = k + 1;
        break;
      }
      for (int i = k + 1; i < BS; i++) lu[BS * i + k] = lu[BS * i + k] / lu[nk + k];
      for (int i = k + 1; i < BS; i++)
        for (int j = k + 1; j < BS; j++) lu[BS * i + j] -= lu[BS * i + k] * lu[nk + j];
    }
    if (!fail && lu[BS * BS - 1] == (T)0) fail = BS;
    piv[BS] = fail;
    if (fail) atomicCAS(fail_flag, 0, row + 1);
  }
  __syncwarp();
  if (piv[BS]) return;
  if (lane < BS) {
    const int k = lane;
    int ip = k;
    for (int i = 0; i < BS - 1; i++) {
      if (ip == piv[i]) ip = i;
      else if (ip == i) ip = piv[i];
    }
    T col[BS];
    for (int i = 0; i < ip; i++) col[i] = 0;
    col[ip] = 1;
    for (int i = ip + 1; i < BS; i++) {
      T v = 0;
      for (int j = ip; j < i; j++) v -= lu[BS * i + j] * col[j];
      col[i] = v;
    }
    for (int i = BS - 1; i >= 0; i--) {
      T v = col[i];
      for (int j = i + 1; j < BS; j++) v -= lu[BS * i + j] * col[j];
      col[i] = v / lu[BS * i + i];
    }
    for (int i = 0; i < BS; i++) a[BS * i + k] = col[i];
  }
  __syncwarp();
}

// One warp per row of one level (IKJ variant of BCSRMatFactor6/3):
// for every lower block j in order: d = A_j D_{cj}^{-1};
// A_k -= d A_p for the matching upper blocks of row cj; A_j = d.
// Then the diagonal block is replaced by its inverse.
template <int BS, typename T>
__global__ void __launch_bounds__(128)
    ilu0_factor_level_kernel(const int *__restrict__ rows, int nrows_lvl,
                             const int *__restrict__ rowp,
                             const int *__restrict__ cols,
                             const int *__restrict__ diag,
                             const int *__restrict__ upd_ptr,
                             const int *__restrict__ upd_tgt,
                             const int *__restrict__ upd_src, T *F,
                             int *fail_flag) {
  __shared__ T sd[4][BS * BS];
  __shared__ T slu[4][BS * BS];
  __shared__ int spiv[4][BS + 1];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = blockIdx.x * 4 + wid;
  const int nw = gridDim.x * 4;
  const int B2 = BS * BS;
  for (int r = gw; r < nrows_lvl; r += nw) {
    const int i = rows[r];
    for (int j = rowp[i]; cols[j] < i; j++) {
      const T *a = &F[(size_t)B2 * j];
      const T *b = &F[(size_t)B2 * diag[cols[j]]];
      for (int k = lane; k < B2; k += 32) {
        const int rr = k / BS, cc = k - BS * rr;
        T s = 0;
#pragma unroll
        for (int q = 0; q < BS; q++) s += a[BS * rr + q] * b[BS * q + cc];
        sd[wid][k] = s;
      }
      __syncwarp();
      for (int u = upd_ptr[j]; u < upd_ptr[j + 1]; u++) {
        T *ak = &F[(size_t)B2 * upd_tgt[u]];
        const T *bp = &F[(size_t)B2 * upd_src[u]];
        for (int k = lane; k < B2; k += 32) {
          const int rr = k / BS, cc = k - BS * rr;
          T s = 0;
#pragma unroll
          for (int q = 0; q < BS; q++) s += sd[wid][BS * rr + q] * bp[BS * q + cc];
          ak[k] -= s;
        }
      }
      __syncwarp();
      for (int k = lane; k < B2; k += 32) F[(size_t)B2 * j + k] = sd[wid][k];
      __syncwarp();
    }
    warp_block_inverse<BS, T>(&F[(size_t)B2 * diag[i]], slu[wid], spiv[wid],
                              lane, fail_flag, i);
  }
}

// Diagonal-block inverses only (block Jacobi)
template <int BS, typename T>
__global__ void __launch_bounds__(128)
    diag_inverse_kernel(int nrows, const int *__restrict__ diag, T *F,
                        int *fail_flag) {
  __shared__ T slu[4][BS * BS];
  __shared__ int spiv[4][BS + 1];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = blockIdx.x * 4 + wid; i < nrows; i += gridDim.x * 4)
    warp_block_inverse<BS, T>(&F[(size_t)BS * BS * diag[i]], slu[wid],
                              spiv[wid], lane, fail_flag, i);
}

// Lower solve of one level: y_i = x_i - sum_{j<i} L_ij y_cj
// (BCSRMatApplyLower6, unit lower); NR vectors ld apart per block read.
template <int BS, int NR, typename T>
__global__ void __launch_bounds__(256)
    ilu_lower_level_kernel(const int *__restrict__ rows, int nrows_lvl,
                           const int *__restrict__ rowp,
                           const int *__restrict__ cols,
                           const T *__restrict__ F, const T *__restrict__ x,
                           T *__restrict__ y, size_t ld) {
  const int per_warp = 32 / BS;
  const int lane = threadIdx.x & 31, sub = lane / BS, ii = lane - BS * sub;
  if (sub >= per_warp) return;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int r = gw * per_warp + sub; r < nrows_lvl; r += nw * per_warp) {
    const int i = rows[r];
    T z[NR];
#pragma unroll
    for (int l = 0; l < NR; l++) z[l] = x[l * ld + (size_t)BS * i + ii];
    for (int j = rowp[i]; cols[j] < i; j++) {
      const T *a = &F[(size_t)BS * BS * j + BS * ii];
      T av[BS];
#pragma unroll
      for (int c = 0; c < BS; c++) av[c] = a[c];
      const size_t yo = (size_t)BS * cols[j];
#pragma unroll
      for (int l = 0; l < NR; l++) {
        const T *yy = &y[l * ld + yo];
        T s = 0;
#pragma unroll
        for (int c = 0; c < BS; c++) s += av[c] * yy[c];
        z[l] -= s;
      }
    }
#pragma unroll
    for (int l = 0; l < NR; l++) y[l * ld + (size_t)BS * i + ii] = z[l];
  }
}

// Upper solve of one level: z_i = y_i - sum_{j>i} U_ij x_cj ; x_i = D_i^-1 z
template <int BS, int NR, typename T>
__global__ void __launch_bounds__(256)
    ilu_upper_level_kernel(const int *__restrict__ rows, int nrows_lvl,
                           const int *__restrict__ rowp,
                           const int *__restrict__ cols,
                           const int *__restrict__ diag,
                           const T *__restrict__ F, const T *__restrict__ yin,
                           T *__restrict__ xout, size_t ld) {
  const int per_warp = 32 / BS;
  const int lane = threadIdx.x & 31, sub = lane / BS, ii = lane - BS * sub;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int nrounds = (nrows_lvl + nw * per_warp - 1) / (nw * per_warp);
  for (int rd = 0; rd < nrounds; rd++) {
    const int r = (rd * nw + gw) * per_warp + sub;
    const bool active = sub < per_warp && r < nrows_lvl;
    T z[NR];
#pragma unroll
    for (int l = 0; l < NR; l++) z[l] = 0;
    int i = 0;
    if (active) {
      i = rows[r];
#pragma unroll
      for (int l = 0; l < NR; l++) z[l] = yin[l * ld + (size_t)BS * i + ii];
      for (int j = diag[i] + 1; j < rowp[i + 1]; j++) {
        const T *a = &F[(size_t)BS * BS * j + BS * ii];
        T av[BS];
#pragma unroll
        for (int c = 0; c < BS; c++) av[c] = a[c];
        const size_t xo = (size_t)BS * cols[j];
#pragma unroll
        for (int l = 0; l < NR; l++) {
          const T *xx = &xout[l * ld + xo];
          T s = 0;
#pragma unroll
          for (int c = 0; c < BS; c++) s += av[c] * xx[c];
          z[l] -= s;
        }
      }
    }
    const int base = lane - ii;
    T dv[BS];
    if (active) {
      const T *dinv = &F[(size_t)BS * BS * diag[i] + BS * ii];
#pragma unroll
      for (int c = 0; c < BS; c++) dv[c] = dinv[c];
    } else {
#pragma unroll
      for (int c = 0; c < BS; c++) dv[c] = 0;
    }
#pragma unroll
    for (int l = 0; l < NR; l++) {
      T out = 0;
#pragma unroll
      for (int c = 0; c < BS; c++) {
        T zc = __shfl_sync(0xffffffffu, z[l], base + c);
        out += dv[c] * zc;
      }
      if (active) xout[l * ld + (size_t)BS * i + ii] = out;
    }
  }
}

template <int BS, typename T>
__global__ void __launch_bounds__(256)
    block_jacobi_kernel(int nrows, const int *__restrict__ diag,
                        const T *__restrict__ F, const T *__restrict__ x,
                        T *__restrict__ y, int nrhs, size_t ld) {
  const int per_warp = 32 / BS;
  const int lane = threadIdx.x & 31, sub = lane / BS, ii = lane - BS * sub;
  if (sub >= per_warp) return;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw * per_warp + sub; i < nrows; i += nw * per_warp) {
    const T *a = &F[(size_t)BS * BS * diag[i] + BS * ii];
    for (int l = 0; l < nrhs; l++) {
      const T *xx = &x[l * ld + (size_t)BS * i];
      T s = 0;
#pragma unroll
      for (int c = 0; c < BS; c++) s += a[c] * xx[c];
      y[l * ld + (size_t)BS * i + ii] = s;
    }
  }
}

// --------------------------------------------------------------- GMRES
// partial dot products of w with the k basis vectors W_j (column j at
// W + j*ld): block (x, j) reduces chunk x of W_j . w into partials[j*nbx+x]
__global__ void __launch_bounds__(256)
    dots_partial_kernel(const double *__restrict__ W, size_t ld, int k,
                        const double *__restrict__ w,
                        double *__restrict__ partials) {
  __shared__ double sh[8];
  const int j = blockIdx.y, nbx = gridDim.x;
  const double *Wj = W + (size_t)j * ld;
  size_t chunk = (ld + nbx - 1) / nbx;
  size_t b = chunk * blockIdx.x, e = b + chunk < ld ? b + chunk : ld;
  double acc = 0.0;
  for (size_t i = b + threadIdx.x; i < e; i += blockDim.x) acc += Wj[i] * w[i];
  for (int off = 16; off > 0; off >>= 1)
    acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
    partials[(size_t)j * nbx + blockIdx.x] = t;
  }
}
__global__ void dots_final_kernel(const double *partials, int nbx, int k,
                                  double *h) {
  const int j = blockIdx.x;
  if (j >= k) return;
  __shared__ double sh[8];
  double acc = 0.0;
  for (int p = threadIdx.x; p < nbx; p += blockDim.x)
    acc += partials[(size_t)j * nbx + p];
  for (int off = 16; off > 0; off >>= 1)
    acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
    h[j] = t;
  }
}
__global__ void gemv_sub_kernel(const double *__restrict__ W, size_t ld, int k,
                                const double *__restrict__ h,
                                double *__restrict__ w) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ld;
       i += (size_t)gridDim.x * blockDim.x) {
    double acc = w[i];
    for (int j = 0; j < k; j++) acc -= h[j] * W[(size_t)j * ld + i];
    w[i] = acc;
  }
}
__global__ void axpy_kernel(double a, const double *x, double *y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void scale_kernel(double a, double *x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    x[i] *= a;
}

template <typename T>
__global__ void gather_blocks_kernel(int nnz, int b2, const int *valmap,
                                     const double *src, T *dst) {
  const size_t n = (size_t)nnz * b2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t k = i / b2, e = i - k * b2;
    const int m = valmap[k];
    dst[i] = m >= 0 ? (T)src[(size_t)m * b2 + e] : (T)0;
  }
}
template <typename T>
__global__ void permute_kernel(int nrows, int bs, const int *perm,
                               const T *src, T *dst, int scatter, int nrhs) {
  const size_t n = (size_t)nrows * bs;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
       i < n * nrhs; i += (size_t)gridDim.x * blockDim.x) {
    const size_t l = i / n, k = i - l * n;
    const size_t r = k / bs, c = k - r * bs;
    const size_t o = l * n + (size_t)perm[r] * bs + c;
    if (scatter) dst[o] = src[i];
    else dst[i] = src[o];
  }
}
// Both ILU(0) triangular solves in one launch.  Each thread-block cluster
// owns a group of independent matrix components and walks their merged
// level schedule (lower levels, then upper levels); the rows of a level are
// striped over the cluster's CTAs, 6 (or 3) lanes per block row as in the
// level kernels above, and a hardware cluster barrier separates the levels.
//
// Latency, not bandwidth, bounds this walk, so only the neighbour values
// produced by earlier levels are loaded after a barrier.  The level
// pointers sit in shared memory; a row's descriptor (row, first block,
// block count, diagonal block and the first MAXB block columns) is loaded
// two levels ahead and its factor entries, right-hand side and, for the
// upper solve, D^-1 row and lower-solve value one level ahead; those loads
// are issued between the barrier's arrive (which releases the level's
// stores) and its wait, so they overlap the barrier instead of delaying the
// release.  Values produced
// inside the launch (tmp, y) are read with ld.global.cg so they come from
// L2, where the barrier's release/acquire ordering makes the other CTAs'
// stores visible.  Same arithmetic per row as the level kernels.
template <int MAXB>
struct RowDesc {
  int i, jbeg, nb, dpos;
  int col[MAXB];
};

template <int MAXB>
__device__ __forceinline__ void load_desc(RowDesc<MAXB> &d,
                                          const int4 *__restrict__ desc,
                                          int pos) {
  constexpr int DW = 1 + MAXB / 4;
  const int4 h = desc[(size_t)DW * pos];
  d.i = h.x;
  d.jbeg = h.y;
  d.nb = h.z;
  d.dpos = h.w;
#pragma unroll
  for (int q = 0; q < MAXB / 4; q++) {
    const int4 c = desc[(size_t)DW * pos + 1 + q];
    d.col[4 * q] = c.x;
    d.col[4 * q + 1] = c.y;
    d.col[4 * q + 2] = c.z;
    d.col[4 * q + 3] = c.w;
  }
}

template <int BS, int NR, int MAXB, typename T>
struct RowData {
  T a[MAXB][BS];
  T base[NR];  // x_i (lower) or tmp_i (upper)
  T dinv[BS];  // upper only
};

template <int BS, int NR, int MAXB, bool UPPER, typename T>
__device__ __forceinline__ void load_data(RowData<BS, NR, MAXB, T> &p,
                                          const RowDesc<MAXB> &d,
                                          const T *__restrict__ F,
                                          const T *__restrict__ basev,
                                          size_t ld, int ii) {
#pragma unroll
  for (int q = 0; q < MAXB; q++) {
    if (q < d.nb) {
      const T *a = &F[(size_t)BS * BS * (d.jbeg + q) + BS * ii];
#pragma unroll
      for (int c = 0; c < BS; c++) p.a[q][c] = a[c];
    }
  }
#pragma unroll
  for (int l = 0; l < NR; l++)
    p.base[l] = UPPER ? __ldcg(&basev[l * ld + (size_t)BS * d.i + ii])
                      : basev[l * ld + (size_t)BS * d.i + ii];
  if (UPPER) {
    const T *dv = &F[(size_t)BS * BS * d.dpos + BS * ii];
#pragma unroll
    for (int c = 0; c < BS; c++) p.dinv[c] = dv[c];
  }
}

// z = base - sum over the row's blocks of A_q v_cq (v read from L2)
template <int BS, int NR, int MAXB, typename T>
__device__ __forceinline__ void row_product(const RowDesc<MAXB> &d,
                                            const RowData<BS, NR, MAXB, T> &p,
                                            const int *__restrict__ cols,
                                            const T *__restrict__ F,
                                            const T *v, size_t ld, int ii,
                                            T *z) {
#pragma unroll
  for (int l = 0; l < NR; l++) {
    z[l] = p.base[l];
    // all neighbour values of this right-hand side load together
    T vv[MAXB][BS];
#pragma unroll
    for (int q = 0; q < MAXB; q++) {
      if (q < d.nb) {
        const size_t vo = (size_t)BS * d.col[q];
#pragma unroll
        for (int c = 0; c < BS; c++) vv[q][c] = __ldcg(&v[l * ld + vo + c]);
      }
    }
#pragma unroll
    for (int q = 0; q < MAXB; q++) {
      if (q < d.nb) {
        T s = 0;
#pragma unroll
        for (int c = 0; c < BS; c++) s += p.a[q][c] * vv[q][c];
        z[l] -= s;
      }
    }
  }
  for (int q = MAXB; q < d.nb; q++) {  // rows with more blocks than MAXB
    const int j = d.jbeg + q;
    const T *a = &F[(size_t)BS * BS * j + BS * ii];
    const size_t vo = (size_t)BS * cols[j];
#pragma unroll
    for (int l = 0; l < NR; l++) {
      const T *w = &v[l * ld + vo];
      T s = 0;
#pragma unroll
      for (int c = 0; c < BS; c++) s += a[c] * __ldcg(w + c);
      z[l] -= s;
    }
  }
}

template <int BS, int NR, int MAXB, typename T>
__global__ void __launch_bounds__(256)
    ilu_cluster_kernel(IluClusterView cv, const int *__restrict__ cols,
                       const T *__restrict__ F, const T *__restrict__ x,
                       T *__restrict__ tmp, T *__restrict__ y, size_t ld) {
  namespace cg = cooperative_groups;
  extern __shared__ int s_lp[];
  cg::cluster_group cl = cg::this_cluster();
  const int cs = (int)cl.num_blocks();
  const int g = blockIdx.x / cs;
  const int rank = (int)cl.block_rank();
  const int per_warp = 32 / BS;
  const int lane = threadIdx.x & 31, sub = lane / BS, ii = lane - BS * sub;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int slots = nwarps * per_warp;  // rows per CTA per pass
  const bool has_slot = sub < per_warp;
  const int k0 = (warp * per_warp + (has_slot ? sub : 0)) * cs + rank;
  const int stride = slots * cs;
  // level pointers of this group: lower (nl + 1) then upper (nu + 1)
  const int l0 = cv.grp_lvl[g], nl = cv.grp_lvl[g + 1] - l0 - 1;
  const int u0 = cv.grp_ulvl[g], nu = cv.grp_ulvl[g + 1] - u0 - 1;
  int *s_up = s_lp + nl + 1;
  for (int t = threadIdx.x; t <= nl; t += blockDim.x) s_lp[t] = cv.lvl_ptr[l0 + t];
  for (int t = threadIdx.x; t <= nu; t += blockDim.x) s_up[t] = cv.ulvl_ptr[u0 + t];
  __syncthreads();
  RowDesc<MAXB> D, Dn;
  RowData<BS, NR, MAXB, T> P;
  // ------------------------------------------------------------ lower
  {
    bool have = nl > 0 && has_slot && s_lp[0] + k0 < s_lp[1];
    bool have_n = nl > 1 && has_slot && s_lp[1] + k0 < s_lp[2];
    if (have) load_desc<MAXB>(D, cv.ldesc, s_lp[0] + k0);
    if (have_n) load_desc<MAXB>(Dn, cv.ldesc, s_lp[1] + k0);
    if (have) load_data<BS, NR, MAXB, false, T>(P, D, F, x, ld, ii);
    for (int L = 0; L < nl; L++) {
      const int b = s_lp[L], e = s_lp[L + 1];
      if (have) {
        T z[NR];
        row_product<BS, NR, MAXB, T>(D, P, cols, F, tmp, ld, ii, z);
#pragma unroll
        for (int l = 0; l < NR; l++)
          tmp[l * ld + (size_t)BS * D.i + ii] = z[l];
        for (int k = k0 + stride; b + k < e; k += stride) {
          RowDesc<MAXB> D2;
          load_desc<MAXB>(D2, cv.ldesc, b + k);
          load_data<BS, NR, MAXB, false, T>(P, D2, F, x, ld, ii);
          row_product<BS, NR, MAXB, T>(D2, P, cols, F, tmp, ld, ii, z);
#pragma unroll
          for (int l = 0; l < NR; l++)
            tmp[l * ld + (size_t)BS * D2.i + ii] = z[l];
        }
      }
      // arrive (releasing this level's stores), then load level L+1's data
      // and level L+2's descriptor while the barrier completes
      auto tok = cl.barrier_arrive();
      have = have_n;
      D = Dn;
      if (have) load_data<BS, NR, MAXB, false, T>(P, D, F, x, ld, ii);
      have_n = L + 2 < nl && has_slot && s_lp[L + 2] + k0 < s_lp[L + 3];
      if (have_n) load_desc<MAXB>(Dn, cv.ldesc, s_lp[L + 2] + k0);
      cl.barrier_wait(std::move(tok));
    }
  }
  // ------------------------------------------------------------ upper
  {
    bool have = nu > 0 && has_slot && s_up[0] + k0 < s_up[1];
    bool have_n = nu > 1 && has_slot && s_up[1] + k0 < s_up[2];
    if (have) load_desc<MAXB>(D, cv.udesc, s_up[0] + k0);
    if (have_n) load_desc<MAXB>(Dn, cv.udesc, s_up[1] + k0);
    if (have) load_data<BS, NR, MAXB, true, T>(P, D, F, tmp, ld, ii);
    const int base_lane = lane - ii;
    for (int L = 0; L < nu; L++) {
      const int b = s_up[L], e = s_up[L + 1];
      // every lane of a warp runs the same rounds: the D^-1 product
      // exchanges z through shuffles
      const int nrounds = (e - b + stride - 1) / stride;
      for (int rd = 0; rd < nrounds; rd++) {
        const int k = k0 + rd * stride;
        const bool active = has_slot && b + k < e;
        if (rd > 0 && active) {
          load_desc<MAXB>(D, cv.udesc, b + k);
          load_data<BS, NR, MAXB, true, T>(P, D, F, tmp, ld, ii);
        }
        T z[NR];
#pragma unroll
        for (int l = 0; l < NR; l++) z[l] = 0;
        if (active) row_product<BS, NR, MAXB, T>(D, P, cols, F, y, ld, ii, z);
#pragma unroll
        for (int l = 0; l < NR; l++) {
          T out = 0;
#pragma unroll
          for (int c = 0; c < BS; c++) {
            const T zc = __shfl_sync(0xffffffffu, z[l], base_lane + c);
            out += (active ? P.dinv[c] : T(0)) * zc;
          }
          if (active) y[l * ld + (size_t)BS * D.i + ii] = out;
        }
      }
      auto tok = cl.barrier_arrive();
      have = have_n;
      D = Dn;
      if (have) load_data<BS, NR, MAXB, true, T>(P, D, F, tmp, ld, ii);
      have_n = L + 2 < nu && has_slot && s_up[L + 2] + k0 < s_up[L + 3];
      if (have_n) load_desc<MAXB>(Dn, cv.udesc, s_up[L + 2] + k0);
      cl.barrier_wait(std::move(tok));
    }
  }
}

// One block per element segment: KS max, KS sum and compliance over the
// segment's points, each a fixed-order block reduction.
__device__ double block_reduce(double v, bool is_max, double *sh) {
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, v, off);
    v = is_max ? fmax(v, o) : v + o;
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = sh[0];
  for (int q = 1; q < (int)(blockDim.x >> 5); q++)
    t = is_max ? fmax(t, sh[q]) : t + sh[q];
  __syncthreads();
  return t;
}
__global__ void __launch_bounds__(256)
    segment_functions_kernel(const double *__restrict__ fail,
                             const double *__restrict__ wdet,
                             const double *__restrict__ sed, int nq,
                             const int *__restrict__ seg_ptr, double ksw,
                             KsStats *__restrict__ out_ks,
                             double *__restrict__ out_comp) {
  __shared__ double sh[8];
  const int g = blockIdx.x;
  const size_t e0 = seg_ptr[g], e1 = seg_ptr[g + 1];
  double mx = -INFINITY;
  for (size_t i = e0 * nq + threadIdx.x; i < e1 * nq; i += blockDim.x)
    mx = fmax(mx, fail[i]);
  mx = block_reduce(mx, true, sh);
  double sm = 0.0;
  for (size_t i = e0 * nq + threadIdx.x; i < e1 * nq; i += blockDim.x)
    sm += wdet[i] * exp(ksw * (fail[i] - mx));
  sm = block_reduce(sm, false, sh);
  double c = 0.0;
  for (size_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) c += sed[e];
  c = block_reduce(c, false, sh);
  if (threadIdx.x == 0) {
    out_ks[g].max = mx;
    out_ks[g].sum = sm;
    out_ks[g].weight = ksw;
    out_comp[g] = c;
  }
}

}  // namespace

// ------------------------------------------------------------- launchers
void launch_bcsr_mult(int bsize, int nrows, const int *rowp, const int *cols,
                      const double *A, const double *x, double *y,
                      cudaStream_t s, int nrhs, size_t ld) {
  if (bsize == 6)
    mult_dispatch<6, double>(nrows, rowp, cols, A, x, y, nrhs, ld, s);
  else mult_dispatch<3, double>(nrows, rowp, cols, A, x, y, nrhs, ld, s);
}
void launch_bcsr_mult_f32(int bsize, int nrows, const int *rowp,
                          const int *cols, const float *A, const float *x,
                          float *y, cudaStream_t s, int nrhs, size_t ld) {
  if (bsize == 6)
    mult_dispatch<6, float>(nrows, rowp, cols, A, x, y, nrhs, ld, s);
  else mult_dispatch<3, float>(nrows, rowp, cols, A, x, y, nrhs, ld, s);
}
void launch_apply_bcs_mat(int bsize, int nbcs, const int *bc_nodes,
                          const int *bc_masks, const int *rowp,
                          const int *cols, double *A, cudaStream_t s) {
  if (nbcs <= 0) return;
  dim3 th(32, 4);
  int blocks = (nbcs + 3) / 4;
  if (blocks > 4096) blocks = 4096;
  apply_bcs_mat_kernel<<<blocks, th, 0, s>>>(bsize, nbcs, bc_nodes, bc_masks,
                                             rowp, cols, A);
}
void launch_apply_bcs_res(int bsize, int nbcs, const int *bc_nodes,
                          const int *bc_masks, const double *vars,
                          double *res, cudaStream_t s) {
  if (nbcs <= 0) return;
  apply_bcs_res_kernel<<<blocks_for(nbcs, 256), 256, 0, s>>>(
      bsize, nbcs, bc_nodes, bc_masks, vars, res);
}
void launch_fill(double *x, double v, size_t n, cudaStream_t s) {
  if (!n) return;
  fill_kernel<<<blocks_for(n, 256), 256, 0, s>>>(x, v, n);
}
void launch_d2f(const double *x, float *y, size_t n, cudaStream_t s) {
  if (!n) return;
  d2f_kernel<<<blocks_for(n, 256), 256, 0, s>>>(x, y, n);
}
void launch_f2d(const float *x, double *y, size_t n, cudaStream_t s) {
  if (!n) return;
  f2d_kernel<<<blocks_for(n, 256), 256, 0, s>>>(x, y, n);
}
void launch_gather_dv(int nelem, const int *dvnum, const double *dvs,
                      double *thick, cudaStream_t s) {
  if (nelem <= 0) return;
  gather_dv_kernel<<<blocks_for(nelem, 256), 256, 0, s>>>(nelem, dvnum, dvs,
                                                          thick);
}
void launch_scatter_dv(int ndv, const int *dv_ptr, const int *dv_elems,
                       const double *vals, double *dfdx, cudaStream_t s) {
  if (ndv <= 0) return;
  scatter_dv_kernel<<<blocks_for(ndv, 256), 256, 0, s>>>(ndv, dv_ptr,
                                                         dv_elems, vals, dfdx);
}
void launch_reduce_max(const double *x, size_t n, double *partials, int npart,
                       double *out, cudaStream_t s) {
  reduce_partial_kernel<1><<<npart, 256, 0, s>>>(x, nullptr, n, nullptr, 0.0,
                                                 partials);
  reduce_final_kernel<1><<<1, 256, 0, s>>>(partials, npart, out);
}
void launch_reduce_absmax(const double *x, size_t n, double *partials,
                          int npart, double *out, cudaStream_t s) {
  reduce_partial_kernel<3><<<npart, 256, 0, s>>>(x, nullptr, n, nullptr, 0.0,
                                                 partials);
  reduce_final_kernel<1><<<1, 256, 0, s>>>(partials, npart, out);
}
void launch_reduce_absmax_multi(const double *x, int k, size_t n,
                                double *partials, int npart, double *out,
                                int stride, cudaStream_t s) {
  if (k <= 0) return;
  absmax_multi_partial_kernel<<<dim3(npart, k), 256, 0, s>>>(x, n, partials);
  absmax_multi_final_kernel<<<k, 256, 0, s>>>(partials, npart, out, stride);
}
void launch_residual(const double *b, const double *t, double *r, size_t n,
                     cudaStream_t s) {
  if (!n) return;
  residual_kernel<<<blocks_for(n, 256), 256, 0, s>>>(b, t, r, n);
}
void launch_f2d_add(const float *c, double *x, size_t n, cudaStream_t s) {
  if (!n) return;
  f2d_add_kernel<<<blocks_for(n, 256), 256, 0, s>>>(c, x, n);
}
void launch_bcsr_row_abs_sum(int bsize, int nrows, const int *rowp,
                             const double *vals, double *out, cudaStream_t s) {
  const long long n = (long long)nrows * bsize;
  if (n <= 0) return;
  bcsr_row_abs_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      bsize, nrows, rowp, vals, out);
}
void launch_reduce_sum(const double *x, size_t n, double *partials, int npart,
                       double *out, cudaStream_t s) {
  reduce_partial_kernel<0><<<npart, 256, 0, s>>>(x, nullptr, n, nullptr, 0.0,
                                                 partials);
  reduce_final_kernel<0><<<1, 256, 0, s>>>(partials, npart, out);
}
void launch_ks_sum(const double *fail, const double *wdet, size_t n,
                   const double *dmax, double ksw, double *partials, int npart,
                   double *out, cudaStream_t s) {
  reduce_partial_kernel<2><<<npart, 256, 0, s>>>(fail, wdet, n, dmax, ksw,
                                                 partials);
  reduce_final_kernel<0><<<1, 256, 0, s>>>(partials, npart, out);
}

void launch_segment_functions(const double *elem_fail, const double *elem_wdet,
                              const double *elem_sed, int nq,
                              const int *seg_elem_ptr, int nseg, double ksw,
                              KsStats *seg_ks, double *seg_comp,
                              cudaStream_t s) {
  if (nseg <= 0) return;
  segment_functions_kernel<<<nseg, 256, 0, s>>>(
      elem_fail, elem_wdet, elem_sed, nq, seg_elem_ptr, ksw, seg_ks, seg_comp);
}

template <typename T>
static void factor_level(const IluPlan &p, int level, T *F, cudaStream_t s) {
  const int b = p.lvl_ptr_h[level], n = p.lvl_ptr_h[level + 1] - b;
  if (n <= 0) return;
  int blocks = (n + 3) / 4;
  if (blocks > num_sms() * 16) blocks = num_sms() * 16;
  if (p.bsize == 6)
    ilu0_factor_level_kernel<6, T><<<blocks, 128, 0, s>>>(
        p.lvl_rows + b, n, p.rowp, p.cols, p.diag, p.upd_ptr, p.upd_tgt,
        p.upd_src, F, p.d_fail);
  else
    ilu0_factor_level_kernel<3, T><<<blocks, 128, 0, s>>>(
        p.lvl_rows + b, n, p.rowp, p.cols, p.diag, p.upd_ptr, p.upd_tgt,
        p.upd_src, F, p.d_fail);
}
void launch_ilu0_factor_level(const IluPlan &p, int level, double *F,
                              cudaStream_t s) {
  factor_level<double>(p, level, F, s);
}
void launch_ilu0_factor_level_f32(const IluPlan &p, int level, float *F,
                                  cudaStream_t s) {
  factor_level<float>(p, level, F, s);
}
void launch_block_inverse_diag(const IluPlan &p, double *F, cudaStream_t s) {
  int blocks = (p.nrows + 3) / 4;
  if (blocks > num_sms() * 16) blocks = num_sms() * 16;
  if (p.bsize == 6)
    diag_inverse_kernel<6, double><<<blocks, 128, 0, s>>>(p.nrows, p.diag, F,
                                                          p.d_fail);
  else
    diag_inverse_kernel<3, double><<<blocks, 128, 0, s>>>(p.nrows, p.diag, F,
                                                          p.d_fail);
}

template <int BS, int NR, typename T>
static void level_pair(const IluPlan &p, bool upper, int L, const T *F,
                       const T *in, T *out, size_t ld, cudaStream_t s) {
  const int per_warp = 32 / BS;
  const std::vector<int> &ptr = upper ? p.ulvl_ptr_h : p.lvl_ptr_h;
  const int b = ptr[L], n = ptr[L + 1] - b;
  int blocks = blocks_for((size_t)((n + per_warp - 1) / per_warp) * 32, 256, 16);
  if (upper)
    ilu_upper_level_kernel<BS, NR, T><<<blocks, 256, 0, s>>>(
        p.ulvl_rows + b, n, p.rowp, p.cols, p.diag, F, in, out, ld);
  else
    ilu_lower_level_kernel<BS, NR, T><<<blocks, 256, 0, s>>>(
        p.lvl_rows + b, n, p.rowp, p.cols, F, in, out, ld);
}

template <int BS, typename T>
static void level_multi(const IluPlan &p, bool upper, int L, const T *F,
                        const T *in, T *out, int nrhs, size_t ld,
                        cudaStream_t s) {
  for (int l = 0; l < nrhs;) {
    const int left = nrhs - l;
    const size_t o = l * ld;
    if (left >= 4) {
      level_pair<BS, 4, T>(p, upper, L, F, in + o, out + o, ld, s);
      l += 4;
    } else if (left >= 2) {
      level_pair<BS, 2, T>(p, upper, L, F, in + o, out + o, ld, s);
      l += 2;
    } else {
      level_pair<BS, 1, T>(p, upper, L, F, in + o, out + o, ld, s);
      l += 1;
    }
  }
}


template <int BS, int NR, typename T>
static void cluster_launch(const IluPlan &p, const T *F, const T *x, T *y,
                           T *tmp, size_t ld, cudaStream_t s) {
  auto kern = ilu_cluster_kernel<BS, NR, (BS == 6 ? 4 : 8), T>;
  // kernel attributes are per device: set on each device, recorded only
  // when the call succeeded
  constexpr int kMaxDevices = 64;
  static bool attr[kMaxDevices] = {};
  static size_t smem_set[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    dev = 0;
  if (!attr[dev] &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed,
                           1) == cudaSuccess)
    attr[dev] = true;
  const size_t smem = sizeof(int) * (size_t)p.cluster.max_lp;
  if (smem > smem_set[dev] && smem > 48 * 1024 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) == cudaSuccess)
    smem_set[dev] = smem;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p.cluster.ngroups * p.cluster.cs);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = p.cluster.cs;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, p.cluster, p.cols, F, x, tmp, y, ld);
}

// Largest cluster size (of 16, 8, 4, 2, 1) the device can schedule for the
// cluster triangular-solve kernel.
int ilu_cluster_max_size() {
  auto kern = ilu_cluster_kernel<6, 4, 4, double>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed,
                       1);
  for (int cs = 16; cs > 1; cs >>= 1) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(256);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n > 0)
      return cs;
    cudaGetLastError();
  }
  return 1;
}

template <typename T>
static void apply_cluster(const IluPlan &p, const T *F, const T *x, T *y,
                          T *tmp, int nrhs, size_t ld, cudaStream_t s) {
  for (int l = 0; l < nrhs;) {
    const int left = nrhs - l;
    const size_t o = l * ld;
    const int nr = left >= 4 ? 4 : (left >= 2 ? 2 : 1);
    if (p.bsize == 6) {
      if (nr == 4) cluster_launch<6, 4, T>(p, F, x + o, y + o, tmp + o, ld, s);
      else if (nr == 2) cluster_launch<6, 2, T>(p, F, x + o, y + o, tmp + o, ld, s);
      else cluster_launch<6, 1, T>(p, F, x + o, y + o, tmp + o, ld, s);
    } else {
      if (nr == 4) cluster_launch<3, 4, T>(p, F, x + o, y + o, tmp + o, ld, s);
      else if (nr == 2) cluster_launch<3, 2, T>(p, F, x + o, y + o, tmp + o, ld, s);
      else cluster_launch<3, 1, T>(p, F, x + o, y + o, tmp + o, ld, s);
    }
    l += nr;
  }
}

template <typename T>
static void apply_levels(const IluPlan &p, const T *F, const T *x, T *y,
                         T *tmp, int nrhs, size_t ld, cudaStream_t s) {
  if (p.cluster.ngroups > 0) {
    apply_cluster<T>(p, F, x, y, tmp, nrhs, ld, s);
    return;
  }
  const int nl = (int)p.lvl_ptr_h.size() - 1;
  for (int L = 0; L < nl; L++) {
    if (p.bsize == 6) level_multi<6, T>(p, false, L, F, x, tmp, nrhs, ld, s);
    else level_multi<3, T>(p, false, L, F, x, tmp, nrhs, ld, s);
  }
  const int nu = (int)p.ulvl_ptr_h.size() - 1;
  for (int L = 0; L < nu; L++) {
    if (p.bsize == 6) level_multi<6, T>(p, true, L, F, tmp, y, nrhs, ld, s);
    else level_multi<3, T>(p, true, L, F, tmp, y, nrhs, ld, s);
  }
}
void launch_ilu0_apply(const IluPlan &p, const double *F, const double *x,
                       double *y, double *tmp, cudaStream_t s, int nrhs,
                       size_t ld) {
  apply_levels<double>(p, F, x, y, tmp, nrhs, ld, s);
}
void launch_ilu0_apply_f32(const IluPlan &p, const float *F, const float *x,
                           float *y, float *tmp, cudaStream_t s, int nrhs,
                           size_t ld) {
  apply_levels<float>(p, F, x, y, tmp, nrhs, ld, s);
}
void launch_block_jacobi_apply(const IluPlan &p, const double *F,
                               const double *x, double *y, cudaStream_t s,
                               int nrhs, size_t ld) {
  const int per_warp = 32 / p.bsize;
  int blocks = blocks_for((size_t)((p.nrows + per_warp - 1) / per_warp) * 32,
                          256, 16);
  if (p.bsize == 6)
    block_jacobi_kernel<6, double><<<blocks, 256, 0, s>>>(p.nrows, p.diag, F,
                                                          x, y, nrhs, ld);
  else
    block_jacobi_kernel<3, double><<<blocks, 256, 0, s>>>(p.nrows, p.diag, F,
                                                          x, y, nrhs, ld);
}
void launch_block_jacobi_apply_f32(const IluPlan &p, const float *F,
                                   const float *x, float *y, cudaStream_t s,
                                   int nrhs, size_t ld) {
  const int per_warp = 32 / p.bsize;
  int blocks = blocks_for((size_t)((p.nrows + per_warp - 1) / per_warp) * 32,
                          256, 16);
  if (p.bsize == 6)
    block_jacobi_kernel<6, float><<<blocks, 256, 0, s>>>(p.nrows, p.diag, F, x,
                                                         y, nrhs, ld);
  else
    block_jacobi_kernel<3, float><<<blocks, 256, 0, s>>>(p.nrows, p.diag, F, x,
                                                         y, nrhs, ld);
}

void launch_dots(const double *W, size_t ld, int k, const double *w,
                 double *partials, int npart, double *h, cudaStream_t s) {
  if (k <= 0) return;
  // npart partials in total: nbx chunks for each of the k vectors
  int nbx = npart / k;
  size_t need = (ld + 2047) / 2048;
  if ((size_t)nbx > need) nbx = (int)need;
  if (nbx < 1) nbx = 1;
  dots_partial_kernel<<<dim3(nbx, k), 256, 0, s>>>(W, ld, k, w, partials);
  dots_final_kernel<<<k, 128, 0, s>>>(partials, nbx, k, h);
}
void launch_gemv_sub(const double *W, size_t ld, int k, const double *h,
                     double *w, size_t n, cudaStream_t s) {
  (void)n;
  gemv_sub_kernel<<<blocks_for(ld, 256), 256, 0, s>>>(W, ld, k, h, w);
}
void launch_axpy(double a, const double *x, double *y, size_t n,
                 cudaStream_t s) {
  if (!n) return;
  axpy_kernel<<<blocks_for(n, 256), 256, 0, s>>>(a, x, y, n);
}
void launch_scale(double a, double *x, size_t n, cudaStream_t s) {
  if (!n) return;
  scale_kernel<<<blocks_for(n, 256), 256, 0, s>>>(a, x, n);
}
void launch_copy(const double *x, double *y, size_t n, cudaStream_t s) {
  if (!n) return;
  cudaMemcpyAsync(y, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
}

void launch_gather_blocks(int nnz, int b2, const int *valmap,
                          const double *src, double *dst, cudaStream_t s) {
  gather_blocks_kernel<double><<<blocks_for((size_t)nnz * b2, 256), 256, 0, s>>>(
      nnz, b2, valmap, src, dst);
}
void launch_gather_blocks_f32(int nnz, int b2, const int *valmap,
                              const double *src, float *dst, cudaStream_t s) {
  gather_blocks_kernel<float><<<blocks_for((size_t)nnz * b2, 256), 256, 0, s>>>(
      nnz, b2, valmap, src, dst);
}
void launch_permute_gather(int nrows, int bs, const int *perm,
                           const double *src, double *dst, cudaStream_t s,
                           int nrhs) {
  permute_kernel<double>
      <<<blocks_for((size_t)nrows * bs * nrhs, 256), 256, 0, s>>>(
          nrows, bs, perm, src, dst, 0, nrhs);
}
void launch_permute_scatter(int nrows, int bs, const int *perm,
                            const double *src, double *dst, cudaStream_t s,
                            int nrhs) {
  permute_kernel<double>
      <<<blocks_for((size_t)nrows * bs * nrhs, 256), 256, 0, s>>>(
          nrows, bs, perm, src, dst, 1, nrhs);
}
void launch_permute_gather_f32(int nrows, int bs, const int *perm,
                               const float *src, float *dst, cudaStream_t s,
                               int nrhs) {
  permute_kernel<float>
      <<<blocks_for((size_t)nrows * bs * nrhs, 256), 256, 0, s>>>(
          nrows, bs, perm, src, dst, 0, nrhs);
}
void launch_permute_scatter_f32(int nrows, int bs, const int *perm,
                                const float *src, float *dst, cudaStream_t s,
                                int nrhs) {
  permute_kernel<float>
      <<<blocks_for((size_t)nrows * bs * nrhs, 256), 256, 0, s>>>(
          nrows, bs, perm, src, dst, 1, nrhs);
}

}  // namespace tg
