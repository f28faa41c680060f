// Kernels of the multifrontal block Cholesky (the numeric phase of the
// direct factorisation; host analysis in direct_symbolic.h, launches in
// direct_kernels.cu).  Included by direct_kernels.cu and, with
// DK_EMULATE defined, by a CPU test harness that runs every CTA as one
// thread in sequence: each kernel is written as phases separated by
// __syncthreads() in which every thread strides over independent entries,
// so one thread executing the phases in order computes the same result.
//
// Storage (one per factorisation): the front of supernode s (M x M
// scalars, M = front rows x bs, lower triangle used) is split between its
// factor panel -- the first C = own columns x bs columns of every front
// row, row-major M x C at lstore + l_off[s] -- and its update matrix --
// the trailing (M - C) x (M - C) part, row-major at pool + u_off[s], in a
// pool shared across tree levels.  A level of the tree is processed as:
// zero the fronts, scatter the matrix's lower blocks (boundary columns
// zeroed so that the factored matrix is the symmetric Kt), add the
// children's update matrices (one CTA per parent, children in a fixed
// order: deterministic), then the partial Cholesky: small fronts one CTA
// each, large fronts by 32-column panels (one CTA factors the panel, a
// grid of 32 x 32 tiles updates the trailing front).  The solves pass
// contribution vectors from children to parents the same way, so no two
// CTAs write one entry.
#pragma once

#ifndef DK_EMULATE
#include <cooperative_groups.h>
#endif

#include "direct_view.h"

#ifdef DK_EMULATE
#define DK_DYN_SMEM(T, name) T *name = reinterpret_cast<T *>(dk_dyn_smem())
#else
#define DK_DYN_SMEM(T, name)                                   \
  extern __shared__ __align__(16) unsigned char dk_smem_raw[]; \
  T *name = reinterpret_cast<T *>(dk_smem_raw)
#endif

namespace tg {
namespace dk {
namespace {

#ifndef DK_EMULATE
template <class T>
__device__ __forceinline__ bool dk_isfinite(T x) { return isfinite(x); }
template <class T>
__device__ __forceinline__ T dk_sqrt(T x) { return sqrt(x); }
#endif


// T = double for the FP64 factorisation, float for the FP32 one (whose
// storage is lstore32 / pool32)
template <class T>
struct Front {
  T *lp;  // M x C row-major panel
  T *up;  // (M - C) x (M - C) row-major update, or nullptr
  int M, C;
  __device__ __forceinline__ T &at(int i, int j) const {  // i >= j
    return j < C ? lp[(size_t)i * C + j]
                 : up[(size_t)(i - C) * (M - C) + (j - C)];
  }
};

__device__ __forceinline__ double *dk_store(const DirectView &v, bool pool,
                                            double *) {
  return pool ? v.pool : v.lstore;
}
__device__ __forceinline__ float *dk_store(const DirectView &v, bool pool,
                                           float *) {
  return pool ? v.pool32 : v.lstore32;
}

template <class T>
__device__ __forceinline__ Front<T> front_of(const DirectView &v, int s) {
  Front<T> f;
  const int bs = v.bs;
  f.M = (v.sn_rowptr[s + 1] - v.sn_rowptr[s]) * bs;
  f.C = (v.sn_col[s + 1] - v.sn_col[s]) * bs;
  f.lp = dk_store(v, false, (T *)nullptr) + (size_t)v.l_off[s] * bs * bs;
  f.up = v.u_off[s] >= 0
             ? dk_store(v, true, (T *)nullptr) + (size_t)v.u_off[s] * bs * bs
             : nullptr;
  return f;
}

// zero the fronts of the level's supernodes (one CTA each)
template <class T>
__global__ void __launch_bounds__(256)
    direct_zero_kernel(DirectView v, const int *__restrict__ sn, int count) {
  if ((int)blockIdx.x >= count) return;
  const Front<T> f = front_of<T>(v, sn[blockIdx.x]);
  const size_t npan = (size_t)f.M * f.C;
  for (size_t k = threadIdx.x; k < npan; k += blockDim.x) f.lp[k] = 0.0;
  if (f.up) {
    const size_t nu = (size_t)(f.M - f.C) * (f.M - f.C);
    for (size_t k = threadIdx.x; k < nu; k += blockDim.x) f.up[k] = 0.0;
  }
}

// the matrix's lower blocks into the fronts; entries in a boundary row or
// column are 0 except the boundary dof's own diagonal (1)
template <class T>
__global__ void __launch_bounds__(256)
    direct_assemble_kernel(DirectView v, const int *__restrict__ sn,
                           int count, const double *__restrict__ A) {
  if ((int)blockIdx.x >= count) return;
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  const int bs = v.bs, b2 = bs * bs;
  const int k0 = v.asm_ptr[s], k1 = v.asm_ptr[s + 1];
  const size_t total = (size_t)(k1 - k0) * b2;
  for (size_t t = threadIdx.x; t < total; t += blockDim.x) {
    const int k = k0 + (int)(t / b2), e = (int)(t % b2);
    const int r = e / bs, q = e - bs * (e / bs);
    const int ir = v.asm_row[k] * bs + r, jc = v.asm_col[k] * bs + q;
    if (jc > ir) continue;  // upper half of a diagonal block
    const int rnode = v.perm[v.sn_rows[v.sn_rowptr[s] + v.asm_row[k]]];
    const int cnode = v.perm[v.sn_col[s] + v.asm_col[k]];
    const bool bc = ((v.bcmask[rnode] >> r) & 1) || ((v.bcmask[cnode] >> q) & 1);
    T val = (T)A[(size_t)v.asm_blk[k] * b2 + e];
    if (bc) val = (rnode == cnode && r == q) ? T(1) : T(0);
    f.at(ir, jc) = val;
  }
}

// The children's update matrices into their parent fronts.  One launch
// per child position kchild (the kchild-th child of every parent of the
// level, children in increasing order across launches, so every parent
// entry receives its children's terms in one fixed order); within a launch
// a parent's child is split over CTAs by kExtendRows rows of its update
// matrix (blockIdx.y), one warp per row and the lanes along it.  A child
// maps its entries one-to-one into its parent, so no two threads of a
// launch write one entry.
constexpr int kExtendRows = kDirectExtendRows;
template <class T>
__global__ void __launch_bounds__(256)
    direct_extend_add_kernel(DirectView v, const int *__restrict__ sn,
                             int count, int kchild) {
  if ((int)blockIdx.x >= count) return;
  const int s = sn[blockIdx.x];
  if (kchild >= v.ch_ptr[s + 1] - v.ch_ptr[s]) return;
  const int c = v.ch_list[v.ch_ptr[s] + kchild];
  const Front<T> f = front_of<T>(v, s);
  const Front<T> fc = front_of<T>(v, c);
  const int um = fc.M - fc.C;
  const int r0 = (int)blockIdx.y * kExtendRows;
  if (r0 >= um) return;
  const int r1 = r0 + kExtendRows < um ? r0 + kExtendRows : um;
  const int bs = v.bs;
  const int *rel = v.ea_rel + v.ea_ptr[c];
  const int ls = blockDim.x < 32 ? (int)blockDim.x : 32;
  const int nw = blockDim.x < 32 ? 1 : (int)blockDim.x / 32;
  const int w = (int)threadIdx.x / 32, lane = (int)threadIdx.x % 32;
  for (int ur = r0 + w; ur < r1; ur += nw) {
    const int i = rel[ur / bs] * bs + ur % bs;
    const T *src = fc.up + (size_t)ur * um;
    for (int uc = lane; uc <= ur; uc += ls)
      f.at(i, rel[uc / bs] * bs + uc % bs) += src[uc];
  }
}

// partial Cholesky of whole small fronts, one CTA each (right-looking in
// place); fail = first failing supernode + 1
template <class T>
__global__ void __launch_bounds__(256)
    direct_factor_small_kernel(DirectView v, const int *__restrict__ sn,
                               int count, int *fail) {
  if ((int)blockIdx.x >= count) return;
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  __shared__ T piv;
  for (int k = 0; k < f.C; k++) {
    if (threadIdx.x == 0) {
      const T d = f.at(k, k);
      if (!(d > 0.0) || !dk_isfinite(d)) {
        atomicCAS(fail, 0, s + 1);
        piv = 1.0;
      } else {
        piv = dk_sqrt(d);
      }
      f.at(k, k) = piv;
    }
    __syncthreads();
    const T inv = T(1) / piv;
    for (int i = k + 1 + threadIdx.x; i < f.M; i += blockDim.x)
      f.at(i, k) *= inv;
    __syncthreads();
    // trailing update of rows and columns > k, lower triangle only:
    // t = a (a + 1) / 2 + b with 0 <= b <= a < w
    const int w = f.M - k - 1;
    const int total = w * (w + 1) / 2;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int a = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
      while ((a + 1) * (a + 2) / 2 <= t) a++;  // exact integer fix-up
      while (a * (a + 1) / 2 > t) a--;
      const int i = k + 1 + a, j = k + 1 + (t - a * (a + 1) / 2);
      f.at(i, j) -= f.at(i, k) * f.at(j, k);
    }
    __syncthreads();
  }
}

// Large fronts, in panel steps batched over the large fronts of a level
// (direct::panel_steps).  A step has three launches: this kernel factors
// the nb x nb diagonal block of columns [k0, k0 + nb) of front
// sn[blockIdx.x] (nb = min(kPanel, C - k0) > 0, one CTA, right-looking);
// direct_trsm_kernel solves the rows below against it; the trailing
// kernel updates the rest of the front.
constexpr int kTile = kDirectTile, kPanel = kDirectPanel;
template <class T>
__global__ void __launch_bounds__(256)
    direct_panel_kernel(DirectView v, const int *__restrict__ sn, int count,
                        int k0, int *fail) {
  if ((int)blockIdx.x >= count) return;
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  const int nb = f.C - k0 < kPanel ? f.C - k0 : kPanel;
  __shared__ T piv;
  for (int k = k0; k < k0 + nb; k++) {
    if (threadIdx.x == 0) {
      const T d = f.at(k, k);
      if (!(d > 0.0) || !dk_isfinite(d)) {
        atomicCAS(fail, 0, s + 1);
        piv = 1.0;
      } else {
        piv = dk_sqrt(d);
      }
      f.at(k, k) = piv;
    }
    __syncthreads();
    const T inv = T(1) / piv;
    const int kend = k0 + nb;
    for (int i = k + 1 + threadIdx.x; i < kend; i += blockDim.x)
      f.at(i, k) *= inv;
    __syncthreads();
    // update the rest of the diagonal block's columns (k, k0 + nb)
    const int w = kend - k - 1;
    if (w > 0) {
      const int rows = kend - k - 1;
      const size_t total = (size_t)rows * w;
      for (size_t t = threadIdx.x; t < total; t += blockDim.x) {
        const int i = k + 1 + (int)(t / w), j = k + 1 + (int)(t % w);
        if (j > i) continue;
        f.at(i, j) -= f.at(i, k) * f.at(j, k);
      }
    }
    __syncthreads();
  }
}

// Rows below a panel's diagonal block: L21 = A21 L11^-T, row by row
// (forward substitution against the diagonal block, held in shared
// memory), one thread per row, kTrsmRows rows per CTA; CTA b belongs to
// the last front f with rprefix[f] <= b and takes its row block
// b - rprefix[f].
constexpr int kTrsmRows = kDirectTrsmRows;
template <class T>
__global__ void __launch_bounds__(256)
    direct_trsm_kernel(DirectView v, const int *__restrict__ sn,
                       const int *__restrict__ rprefix, int count, int k0) {
  const int b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (rprefix[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  const Front<T> f = front_of<T>(v, sn[lo]);
  const int nb = f.C - k0 < kPanel ? f.C - k0 : kPanel;
  const int r0 = k0 + nb + (b - rprefix[lo]) * kTrsmRows;
  const int r1 = r0 + kTrsmRows < f.M ? r0 + kTrsmRows : f.M;
  __shared__ T Ld[kPanel][kPanel + 1];
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t % nb;
    Ld[r][c] = c <= r ? f.at(k0 + r, k0 + c) : T(0);
  }
  __syncthreads();
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    T x[kPanel];
#pragma unroll
    for (int k = 0; k < kPanel; k++) {
      if (k < nb) {
        T acc = f.at(i, k0 + k);
#pragma unroll
        for (int q = 0; q < kPanel; q++)
          if (q < k) acc -= x[q] * Ld[k][q];
        x[k] = acc / Ld[k][k];
      }
    }
#pragma unroll
    for (int k = 0; k < kPanel; k++)
      if (k < nb) f.at(i, k0 + k) = x[k];
  }
}

// Trailing update after a panel step: F(i, j) -= sum_q F(i, q) F(j, q)
// over the panel's columns q, for k1 <= j <= i < M, in 32 x 32 tiles.  One
// CTA per lower-triangular tile of all the step's fronts: CTA b belongs to
// the last front f with tprefix[f] <= b (fronts without tiles are skipped
// that way) and is its tile tau = b - tprefix[f] = ti (ti + 1) / 2 + tj.
template <class T>
__global__ void __launch_bounds__(256)
    direct_trailing_kernel(DirectView v, const int *__restrict__ sn,
                           const int *__restrict__ tprefix, int count,
                           int k0) {
  const int b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tprefix[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  const Front<T> f = front_of<T>(v, sn[lo]);
  const int nb = f.C - k0 < kPanel ? f.C - k0 : kPanel;
  const int tau = b - tprefix[lo];
  int ti = (int)((sqrtf(8.0f * (float)tau + 1.0f) - 1.0f) * 0.5f);
  while ((ti + 1) * (ti + 2) / 2 <= tau) ti++;  // exact integer fix-up
  while (ti * (ti + 1) / 2 > tau) ti--;
  const int tj = tau - ti * (ti + 1) / 2;
  const int k1 = k0 + nb;
  const int i0 = k1 + ti * kTile, j0 = k1 + tj * kTile;
  if (i0 >= f.M || j0 >= f.M) return;
  __shared__ T Ai[kTile][kPanel + 1], Aj[kTile][kPanel + 1];
  for (int t = threadIdx.x; t < kTile * nb; t += blockDim.x) {
    const int r = t / nb, q = t % nb;
    Ai[r][q] = i0 + r < f.M ? f.at(i0 + r, k0 + q) : 0.0;
    Aj[r][q] = j0 + r < f.M ? f.at(j0 + r, k0 + q) : 0.0;
  }
  __syncthreads();
  // a group owns rows (r, r + 16) x columns (c, c + 16) of the tile: one
  // pass over q loads 4 operands for 4 products (half the shared-memory
  // loads per FMA of one entry per pass; each entry keeps its own
  // summation order over q)
  constexpr int kHalf = kTile / 2;
  for (int g = threadIdx.x; g < kHalf * kHalf; g += blockDim.x) {
    const int r = g / kHalf, c = g % kHalf;
    T a00 = 0, a01 = 0, a10 = 0, a11 = 0;
    for (int q = 0; q < nb; q++) {
      const T x0 = Ai[r][q], x1 = Ai[r + kHalf][q];
      const T y0 = Aj[c][q], y1 = Aj[c + kHalf][q];
      a00 += x0 * y0;
      a01 += x0 * y1;
      a10 += x1 * y0;
      a11 += x1 * y1;
    }
    const int ia = i0 + r, ib = ia + kHalf, ja = j0 + c, jb = ja + kHalf;
    if (ia < f.M && ja <= ia) f.at(ia, ja) -= a00;
    if (ia < f.M && jb <= ia) f.at(ia, jb) -= a01;
    if (ib < f.M && ja <= ib) f.at(ib, ja) -= a10;
    if (ib < f.M && jb <= ib) f.at(ib, jb) -= a11;
  }
}

// ----------------------------------------------------------------- solves
// NR right-hand sides at once: every vector of the solve (the factor-order
// vectors y and x, the contribution vectors and the front workspace z)
// holds entry t of right-hand side r at t * NR + r, so that each factor
// entry loaded serves NR products; each right-hand side's sums are formed
// in the same order whatever NR is.
// Both solves go through the panel in blocks of kDirectSolveBlock columns:
// the block's diagonal part is staged in shared memory (rows padded to an
// odd length) and solved by one warp, and the block's off-diagonal part
// updates the rest of the front in one pass whose threads read contiguous
// panel rows (forward) or consecutive columns (backward).  Two CTA
// barriers per block instead of two per column.  Dynamic shared memory:
// the front's M x NR entries of z, then the diagonal block.

// Triangular solve of the staged diagonal block D (nb x nb, row stride
// kDirectSolveBlock + 1) on zb[0..nb) (NR interleaved right-hand sides):
// lower (L zb = zb) or its transpose.  Warp 0 works on it; the others
// wait at the caller's barrier.
template <class T, bool kTranspose, int NR>
__device__ __forceinline__ void dk_block_solve(const T *D, int nb, T *zb) {
  constexpr int P = kDirectSolveBlock + 1;
  if (threadIdx.x >= 32) return;
  const int ls = blockDim.x < 32 ? (int)blockDim.x : 32;
  for (int kk = 0; kk < nb; kk++) {
    const int k = kTranspose ? nb - 1 - kk : kk;
    for (int r = threadIdx.x; r < NR; r += ls) zb[k * NR + r] /= D[k * P + k];
    __syncwarp();
    T zk[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) zk[r] = zb[k * NR + r];
    if (kTranspose) {
      for (int j = threadIdx.x; j < k; j += ls) {
        const T d = D[k * P + j];
#pragma unroll
        for (int r = 0; r < NR; r++) zb[j * NR + r] -= d * zk[r];
      }
    } else {
      for (int j = k + 1 + threadIdx.x; j < nb; j += ls) {
        const T d = D[j * P + k];
#pragma unroll
        for (int r = 0; r < NR; r++) zb[j * NR + r] -= d * zk[r];
      }
    }
    __syncwarp();
  }
}

template <class T>
__device__ __forceinline__ void dk_stage_block(const Front<T> &f, int kb,
                                               int nb, T *D) {
  constexpr int P = kDirectSolveBlock + 1;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t - nb * (t / nb);
    D[r * P + c] = f.lp[(size_t)(kb + r) * f.C + kb + c];
  }
}

// position of front row i of supernode s in a factor-order vector
__device__ __forceinline__ size_t dk_pos(const int *rows, int bs, int i) {
  return (size_t)rows[i / bs] * bs + i % bs;
}

// Forward: z = front rows of the supernode (own rows from y, the rows
// below zero), plus the children's contribution vectors; L11 z1 = z1 and
// z2 -= L21 z1; own rows back to y, z2 to the supernode's contribution.
template <class T, int NR>
__global__ void __launch_bounds__(256)
    direct_forward_kernel(DirectView v, const int *__restrict__ sn, int count,
                          T *y, T *contrib) {
  if ((int)blockIdx.x >= count) return;
  DK_DYN_SMEM(T, z);
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  T *D = z + (size_t)f.M * NR;
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  for (int t = threadIdx.x; t < f.M * NR; t += blockDim.x) {
    const int i = t / NR, r = t - NR * (t / NR);
    z[t] = i < f.C ? y[dk_pos(rows, bs, i) * NR + r] : T(0);
  }
  __syncthreads();
  for (int k = v.ch_ptr[s]; k < v.ch_ptr[s + 1]; k++) {
    const int c = v.ch_list[k];
    const Front<T> fc = front_of<T>(v, c);
    const int um = fc.M - fc.C;
    const int *rel = v.ea_rel + v.ea_ptr[c];
    const T *w = contrib + v.v_off[c] * NR;
    for (int t = threadIdx.x; t < um * NR; t += blockDim.x) {
      const int i = t / NR, r = t - NR * (t / NR);
      z[(rel[i / bs] * bs + i % bs) * NR + r] += w[t];
    }
    __syncthreads();
  }
  for (int kb = 0; kb < f.C; kb += kDirectSolveBlock) {
    const int nb = f.C - kb < kDirectSolveBlock ? f.C - kb : kDirectSolveBlock;
    dk_stage_block(f, kb, nb, D);
    __syncthreads();
    dk_block_solve<T, false, NR>(D, nb, z + kb * NR);
    __syncthreads();
    // rows below the block: z_i -= L(i, kb .. kb+nb) z(kb .. kb+nb)
    for (int i = kb + nb + threadIdx.x; i < f.M; i += blockDim.x) {
      const T *Li = f.lp + (size_t)i * f.C + kb;
      T acc[NR];
#pragma unroll
      for (int r = 0; r < NR; r++) acc[r] = 0;
      for (int c = 0; c < nb; c++) {
        const T l = Li[c];
#pragma unroll
        for (int r = 0; r < NR; r++) acc[r] += l * z[(kb + c) * NR + r];
      }
#pragma unroll
      for (int r = 0; r < NR; r++) z[i * NR + r] -= acc[r];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < f.C * NR; t += blockDim.x) {
    const int i = t / NR, r = t - NR * (t / NR);
    y[dk_pos(rows, bs, i) * NR + r] = z[t];
  }
  if (v.sn_parent[s] >= 0) {
    T *w = contrib + v.v_off[s] * NR;
    for (int t = f.C * NR + threadIdx.x; t < f.M * NR; t += blockDim.x)
      w[t - f.C * NR] = z[t];
  }
}

// Backward: z1 = y1 - L21^T x2 (x2 from the ancestors, already final),
// then L11^T z1 = z1 from the last block up; own rows to x.
template <class T, int NR>
__global__ void __launch_bounds__(256)
    direct_backward_kernel(DirectView v, const int *__restrict__ sn,
                           int count, const T *y, T *x) {
  if ((int)blockIdx.x >= count) return;
  DK_DYN_SMEM(T, z);
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  T *D = z + (size_t)f.M * NR;
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  for (int t = threadIdx.x; t < f.M * NR; t += blockDim.x) {
    const int i = t / NR, r = t - NR * (t / NR);
    const size_t g = dk_pos(rows, bs, i) * NR + r;
    z[t] = i < f.C ? y[g] : x[g];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < f.C; j += blockDim.x) {
    T acc[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) acc[r] = 0;
    for (int i = f.C; i < f.M; i++) {
      const T l = f.lp[(size_t)i * f.C + j];
#pragma unroll
      for (int r = 0; r < NR; r++) acc[r] += l * z[i * NR + r];
    }
#pragma unroll
    for (int r = 0; r < NR; r++) z[j * NR + r] -= acc[r];
  }
  __syncthreads();
  for (int kb = ((f.C - 1) / kDirectSolveBlock) * kDirectSolveBlock; kb >= 0;
       kb -= kDirectSolveBlock) {
    const int nb = f.C - kb < kDirectSolveBlock ? f.C - kb : kDirectSolveBlock;
    dk_stage_block(f, kb, nb, D);
    __syncthreads();
    dk_block_solve<T, true, NR>(D, nb, z + kb * NR);
    __syncthreads();
    // columns before the block: z_j -= sum_k L(kb + k, j) z(kb + k)
    for (int j = threadIdx.x; j < kb; j += blockDim.x) {
      T acc[NR];
#pragma unroll
      for (int r = 0; r < NR; r++) acc[r] = 0;
      for (int k = 0; k < nb; k++) {
        const T l = f.lp[(size_t)(kb + k) * f.C + j];
#pragma unroll
        for (int r = 0; r < NR; r++) acc[r] += l * z[(kb + k) * NR + r];
      }
#pragma unroll
      for (int r = 0; r < NR; r++) z[j * NR + r] -= acc[r];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < f.C * NR; t += blockDim.x) {
    const int i = t / NR, r = t - NR * (t / NR);
    x[dk_pos(rows, bs, i) * NR + r] = z[t];
  }
}

#ifndef DK_EMULATE
// Large fronts: one thread-block cluster of kDirectSolveCluster CTAs per
// front, so that the front's triangular solves use that many SMs' FP64
// pipes (one CTA per front leaves the top of the tree, a handful of fronts
// with thousands of rows, on one SM each).  The front's rows are dealt out
// in 32-row blocks: block b belongs to rank b % nr and sits in that CTA's
// shared memory at slot (b / nr) * 32.  For column block kb its owner
// solves the staged diagonal block and publishes the 32 x NR values; after
// one hardware cluster barrier every rank reads them through distributed
// shared memory and updates its own rows (forward: rows below; backward:
// columns before).  The control flow is the same in every CTA of a
// cluster (each cluster exits together, and every barrier is reached by
// all of its CTAs); a final barrier keeps each CTA's shared memory alive
// until the others are done reading it.  Dynamic shared memory: the owned
// rows (rounded up to whole blocks) x NR, then the diagonal block.
struct ClusterRows {
  int nr, rank;
  __device__ __forceinline__ bool owns(int r) const {
    return ((r >> 5) % nr) == rank;
  }
  __device__ __forceinline__ int slot(int r) const {
    return ((r >> 5) / nr) * 32 + (r & 31);
  }
  // the i-th row owned by this rank, i < count(M)
  __device__ __forceinline__ int row(int i) const {
    return ((i >> 5) * nr + rank) * 32 + (i & 31);
  }
  __device__ __forceinline__ int count(int M) const {
    const int nbk = (M + 31) >> 5;
    const int mine = nbk > rank ? (nbk - rank + nr - 1) / nr : 0;
    return mine * 32;
  }
};

template <class T, int NR>
__global__ void __launch_bounds__(256)
    direct_forward_cluster_kernel(DirectView v, const int *__restrict__ sn,
                                  int count, T *y, T *contrib) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const ClusterRows cr{(int)cl.num_blocks(), (int)cl.block_rank()};
  const int fi = (int)blockIdx.x / cr.nr;  // the same in the whole cluster
  if (fi >= count) return;
  DK_DYN_SMEM(T, z);
  __shared__ T zb[32 * NR], zk[32 * NR];
  const int s = sn[fi];
  const Front<T> f = front_of<T>(v, s);
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  const int nown = cr.count(f.M);
  T *D = z + (size_t)nown * NR;
  for (int t = threadIdx.x; t < nown * NR; t += blockDim.x) {
    const int i = cr.row(t / NR), r = t - NR * (t / NR);
    z[t] = (i < f.C) ? y[dk_pos(rows, bs, i) * NR + r] : T(0);
  }
  __syncthreads();
  for (int k = v.ch_ptr[s]; k < v.ch_ptr[s + 1]; k++) {
    const int c = v.ch_list[k];
    const Front<T> fc = front_of<T>(v, c);
    const int um = fc.M - fc.C;
    const int *rel = v.ea_rel + v.ea_ptr[c];
    const T *w = contrib + v.v_off[c] * NR;
    for (int t = threadIdx.x; t < um * NR; t += blockDim.x) {
      const int i = t / NR, q = t - NR * (t / NR);
      const int r = rel[i / bs] * bs + i % bs;
      if (cr.owns(r)) z[cr.slot(r) * NR + q] += w[t];
    }
    __syncthreads();
  }
  for (int kb = 0; kb < f.C; kb += 32) {
    const int nb = f.C - kb < 32 ? f.C - kb : 32;
    const int owner = (kb >> 5) % cr.nr;
    if (owner == cr.rank) {
      dk_stage_block(f, kb, nb, D);
      __syncthreads();
      dk_block_solve<T, false, NR>(D, nb, z + cr.slot(kb) * NR);
      __syncthreads();
      for (int t = threadIdx.x; t < nb * NR; t += blockDim.x)
        zb[t] = z[cr.slot(kb) * NR + t];
    }
    cl.sync();
    const T *src = cl.map_shared_rank(zb, owner);
    for (int t = threadIdx.x; t < nb * NR; t += blockDim.x) zk[t] = src[t];
    __syncthreads();
    // own rows below the block: z_r -= L(r, kb .. kb+nb) zk
    for (int t = threadIdx.x; t < nown; t += blockDim.x) {
      const int r = cr.row(t);
      if (r < kb + nb || r >= f.M) continue;
      const T *Lr = f.lp + (size_t)r * f.C + kb;
      T acc[NR];
#pragma unroll
      for (int q = 0; q < NR; q++) acc[q] = 0;
      for (int c = 0; c < nb; c++) {
        const T l = Lr[c];
#pragma unroll
        for (int q = 0; q < NR; q++) acc[q] += l * zk[c * NR + q];
      }
#pragma unroll
      for (int q = 0; q < NR; q++) z[t * NR + q] -= acc[q];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < nown * NR; t += blockDim.x) {
    const int r = cr.row(t / NR), q = t - NR * (t / NR);
    if (r < f.C) y[dk_pos(rows, bs, r) * NR + q] = z[t];
    else if (r < f.M && v.sn_parent[s] >= 0)
      contrib[(v.v_off[s] + (r - f.C)) * NR + q] = z[t];
  }
  cl.sync();  // the other ranks may still read zb
}

template <class T, int NR>
__global__ void __launch_bounds__(256)
    direct_backward_cluster_kernel(DirectView v, const int *__restrict__ sn,
                                   int count, const T *y, T *x) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const ClusterRows cr{(int)cl.num_blocks(), (int)cl.block_rank()};
  const int fi = (int)blockIdx.x / cr.nr;
  if (fi >= count) return;
  DK_DYN_SMEM(T, z);
  __shared__ T zb[32 * NR], zk[32 * NR];
  const int s = sn[fi];
  const Front<T> f = front_of<T>(v, s);
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  const int nown = cr.count(f.M);
  T *D = z + (size_t)nown * NR;
  // own rows of the triangle: y1 - L21^T x2 (x2 final, from the ancestors)
  for (int t = threadIdx.x; t < nown; t += blockDim.x) {
    const int j = cr.row(t);
    if (j >= f.C) continue;
    T acc[NR];
#pragma unroll
    for (int q = 0; q < NR; q++) acc[q] = 0;
    for (int i = f.C; i < f.M; i++) {
      const T l = f.lp[(size_t)i * f.C + j];
      const size_t g = dk_pos(rows, bs, i) * NR;
#pragma unroll
      for (int q = 0; q < NR; q++) acc[q] += l * x[g + q];
    }
    const size_t gj = dk_pos(rows, bs, j) * NR;
#pragma unroll
    for (int q = 0; q < NR; q++) z[t * NR + q] = y[gj + q] - acc[q];
  }
  __syncthreads();
  for (int kb = ((f.C - 1) >> 5) << 5; kb >= 0; kb -= 32) {
    const int nb = f.C - kb < 32 ? f.C - kb : 32;
    const int owner = (kb >> 5) % cr.nr;
    if (owner == cr.rank) {
      dk_stage_block(f, kb, nb, D);
      __syncthreads();
      dk_block_solve<T, true, NR>(D, nb, z + cr.slot(kb) * NR);
      __syncthreads();
      for (int t = threadIdx.x; t < nb * NR; t += blockDim.x)
        zb[t] = z[cr.slot(kb) * NR + t];
    }
    cl.sync();
    const T *src = cl.map_shared_rank(zb, owner);
    for (int t = threadIdx.x; t < nb * NR; t += blockDim.x) zk[t] = src[t];
    __syncthreads();
    // own columns before the block: z_j -= sum_k L(kb + k, j) zk_k
    for (int t = threadIdx.x; t < nown; t += blockDim.x) {
      const int j = cr.row(t);
      if (j >= kb) continue;
      T acc[NR];
#pragma unroll
      for (int q = 0; q < NR; q++) acc[q] = 0;
      for (int k = 0; k < nb; k++) {
        const T l = f.lp[(size_t)(kb + k) * f.C + j];
#pragma unroll
        for (int q = 0; q < NR; q++) acc[q] += l * zk[k * NR + q];
      }
#pragma unroll
      for (int q = 0; q < NR; q++) z[t * NR + q] -= acc[q];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < nown * NR; t += blockDim.x) {
    const int r = cr.row(t / NR), q = t - NR * (t / NR);
    if (r < f.C) x[dk_pos(rows, bs, r) * NR + q] = z[t];
  }
  cl.sync();
}
#endif  // DK_EMULATE

// b' = b - K P b + P b (P keeps the boundary dofs) for nrhs right-hand
// sides ld apart (node order): tmp = P b, K tmp by the mat-vec, then the
// right-hand-side kernel, which also permutes into the factor's order and
// interleaves (ypos[t * nrhs + r]); the unpermute kernel undoes both.
template <class T>
__global__ void direct_bc_mask_kernel(int n, int bs, const int *bcmask,
                                      const T *b, T *out, int nrhs,
                                      size_t ld) {
  const size_t N = (size_t)n * bs, tot = N * nrhs;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / N, e = t - N * r;
    const int node = (int)(e / bs), q = (int)(e % bs);
    out[t] = ((bcmask[node] >> q) & 1) ? b[r * ld + e] : T(0);
  }
}
template <class T>
__global__ void direct_rhs_kernel(int n, int bs, const int *perm,
                                  const T *b, const T *Kpb, const T *pb,
                                  T *ypos, int nrhs, size_t ld) {
  const size_t N = (size_t)n * bs, tot = N * nrhs;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t e = t / nrhs, r = t - nrhs * e;
    const int pos = (int)(e / bs), q = (int)(e % bs);
    const size_t g = (size_t)perm[pos] * bs + q;
    ypos[t] = b[r * ld + g] - Kpb[r * N + g] + pb[r * N + g];
  }
}
template <class T>
__global__ void direct_unpermute_kernel(int n, int bs, const int *perm,
                                        const T *xpos, T *x, int nrhs,
                                        size_t ld) {
  const size_t N = (size_t)n * bs, tot = N * nrhs;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t e = t / nrhs, r = t - nrhs * e;
    const int pos = (int)(e / bs), q = (int)(e % bs);
    x[r * ld + (size_t)perm[pos] * bs + q] = xpos[t];
  }
}


}  // namespace
}  // namespace dk
}  // namespace tg
