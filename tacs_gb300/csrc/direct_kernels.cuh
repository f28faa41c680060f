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


// W consecutive entries of T loaded or stored as one vector access (the
// address must be W entries aligned)
template <class T, int W>
struct alignas(sizeof(T) * W) DkVec {
  T v[W];
};

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

__device__ __forceinline__ double *dk_dinv(const DirectView &v, double *) {
  return v.dinv;
}
__device__ __forceinline__ float *dk_dinv(const DirectView &v, float *) {
  return v.dinv32;
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

// zero the fronts of the level's supernodes: front blockIdx.x, entries
// [blockIdx.y kZeroChunk, (blockIdx.y + 1) kZeroChunk) of its panel and
// update matrix taken as one range (the grid's y extent covers the
// level's largest front)
constexpr int kZeroChunk = kDirectZeroChunk;
template <class T>
__global__ void __launch_bounds__(256)
    direct_zero_kernel(DirectView v, const int *__restrict__ sn, int count) {
  if ((int)blockIdx.x >= count) return;
  const Front<T> f = front_of<T>(v, sn[blockIdx.x]);
  const size_t npan = (size_t)f.M * f.C;
  const size_t nu = f.up ? (size_t)(f.M - f.C) * (f.M - f.C) : 0;
  // chunks of kZeroChunk entries, gridDim.y of them at a time (the grid's
  // y extent is at most 65,535; a front of more than ~32 k rows has more
  // chunks than that)
  for (size_t lo = (size_t)blockIdx.y * kZeroChunk; lo < npan + nu;
       lo += (size_t)gridDim.y * kZeroChunk) {
    const size_t hi =
        lo + kZeroChunk < npan + nu ? lo + kZeroChunk : npan + nu;
    for (size_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
      if (k < npan) f.lp[k] = T(0);
      else f.up[k - npan] = T(0);
    }
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
// sn[blockIdx.x] (nb = min(kPanel, C - k0) > 0), staged in shared memory
// and factored by one warp (right-looking, the operations of the one-CTA
// kernel in its order); direct_trsm_kernel solves the rows below against
// it; the trailing kernel updates the rest of the front.
constexpr int kTile = kDirectTile, kPanel = kDirectPanel;
template <class T>
__global__ void __launch_bounds__(256)
    direct_panel_kernel(DirectView v, const int *__restrict__ sn, int count,
                        int k0, int *fail) {
  if ((int)blockIdx.x >= count) return;
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  const int nb = f.C - k0 < kPanel ? f.C - k0 : kPanel;
  __shared__ T Ld[kPanel][kPanel + 1];
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t - nb * (t / nb);
    Ld[r][c] = c <= r ? f.at(k0 + r, k0 + c) : T(0);
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int ls = blockDim.x < 32 ? (int)blockDim.x : 32;
    for (int k = 0; k < nb; k++) {
      if (threadIdx.x == 0) {
        const T d = Ld[k][k];
        if (!(d > 0.0) || !dk_isfinite(d)) {
          atomicCAS(fail, 0, s + 1);
          Ld[k][k] = T(1);
        } else {
          Ld[k][k] = dk_sqrt(d);
        }
      }
      __syncwarp();
      const T inv = T(1) / Ld[k][k];
      for (int i = k + 1 + threadIdx.x; i < nb; i += ls) Ld[i][k] *= inv;
      __syncwarp();
      for (int i = k + 1 + threadIdx.x; i < nb; i += ls)
        for (int j = k + 1; j <= i; j++) Ld[i][j] -= Ld[i][k] * Ld[j][k];
      __syncwarp();
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t - nb * (t / nb);
    if (c <= r) f.at(k0 + r, k0 + c) = Ld[r][c];
  }
}

// Inverses of the factored 32 x 32 diagonal blocks, for the solves (one
// launch after the factorisation, off its critical path): block b is
// panel inv_k0[b] of supernode inv_sn[b]; one warp each.  X = L^-1 row by
// row, X(i, :) = (e_i - sum_{q < i} L(i, q) X(q, :)) / L(i, i) with the
// reciprocal pivots formed once (lane j on column j), stored row-major in
// the block's 32 x 32 slot of dinv, zero elsewhere.
template <class T>
__global__ void __launch_bounds__(32)
    direct_inverse_kernel(DirectView v, const int *__restrict__ inv_sn,
                          const int *__restrict__ inv_k0, int count) {
  const int b = blockIdx.x;
  if (b >= count) return;
  const int s = inv_sn[b], k0 = inv_k0[b];
  const Front<T> f = front_of<T>(v, s);
  const int nb = f.C - k0 < kPanel ? f.C - k0 : kPanel;
  __shared__ T Ld[kPanel][kPanel + 1], X[kPanel][kPanel + 1];
  __shared__ T rd[kPanel];
  const int ls = blockDim.x < 32 ? (int)blockDim.x : 32;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t - nb * (t / nb);
    Ld[r][c] = c <= r ? f.at(k0 + r, k0 + c) : T(0);
  }
  __syncwarp();
  for (int i = threadIdx.x; i < nb; i += ls) rd[i] = T(1) / Ld[i][i];
  __syncwarp();
  for (int i = 0; i < nb; i++) {
    for (int j = threadIdx.x; j < kPanel; j += ls) {
      T x = T(0);
      if (j == i) {
        x = rd[i];
      } else if (j < i) {
        T acc = T(0);
        for (int q = j; q < i; q++) acc += Ld[i][q] * X[q][j];
        x = -acc * rd[i];
      }
      X[i][j] = x;
    }
    __syncwarp();
  }
  T *out = dk_dinv(v, (T *)nullptr) + v.dinv_off[s] +
           (size_t)(k0 / kPanel) * kPanel * kPanel;
  for (int t = threadIdx.x; t < kPanel * kPanel; t += blockDim.x) {
    const int r = t / kPanel, c = t - kPanel * (t / kPanel);
    out[t] = r < nb ? X[r][c] : T(0);
  }
}

// Rows below a panel's diagonal block: L21 = A21 L11^-T, row by row
// (forward substitution against the factored diagonal block, held in
// shared memory), one thread per row, kTrsmRows rows per CTA; CTA b
// belongs to the last front f with rprefix[f] <= b and takes its row block
// b - rprefix[f].  The rows are staged through shared memory, so that
// global loads and stores run along contiguous panel rows.  Dynamic shared
// memory: kTrsmRows x (kPanel + 1) entries.
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
  const int nr = r1 > r0 ? r1 - r0 : 0;
  __shared__ T Ld[kPanel][kPanel + 1];
  DK_DYN_SMEM(T, X);  // kTrsmRows x (kPanel + 1)
  constexpr int P = kPanel + 1;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t - nb * (t / nb);
    Ld[r][c] = c <= r ? f.at(k0 + r, k0 + c) : T(0);
  }
  for (int t = threadIdx.x; t < nr * nb; t += blockDim.x) {
    const int r = t / nb, c = t - nb * (t / nb);
    X[r * P + c] = f.lp[(size_t)(r0 + r) * f.C + k0 + c];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    T *xi = X + i * P;
    for (int k = 0; k < nb; k++) {
      T acc = xi[k];
      for (int q = 0; q < k; q++) acc -= xi[q] * Ld[k][q];
      xi[k] = acc / Ld[k][k];
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nr * nb; t += blockDim.x) {
    const int r = t / nb, c = t - nb * (t / nb);
    f.lp[(size_t)(r0 + r) * f.C + k0 + c] = X[r * P + c];
  }
}

// Trailing update after a panel step: F(i, j) -= sum_q F(i, q) F(j, q)
// over the panel's columns q, for k1 <= j <= i < M, in TILE x TILE tiles
// (32 for the FP64 factorisation, bound by the FP64 pipe; 64 for the FP32
// one, where shared-memory loads per FMA set the pace).  One CTA per
// lower-triangular tile of all the step's fronts: CTA b belongs to the
// last front f with tprefix[f] <= b (fronts without tiles are skipped that
// way) and is its tile tau = b - tprefix[f] = ti (ti + 1) / 2 + tj.  The
// two operand tiles are staged transposed (Ai[q][r] = F(i0 + r, k0 + q)),
// so that thread (ty, tx) = (t / 16, t % 16), owning the R x R entries
// (ty R + a, tx R + c) of the tile (R = TILE / 16), reads its R row
// operands and R column operands of one q as two R-wide vectors: 2 loads
// for R^2 products.  Each entry keeps its own summation order over q (the
// result does not depend on TILE).
template <class T, int TILE>
__global__ void __launch_bounds__(256)
    direct_trailing_kernel(DirectView v, const int *__restrict__ sn,
                           const int *__restrict__ tprefix, int count,
                           int k0) {
  constexpr int R = TILE / 16;
  constexpr int LD = TILE + 16 / (int)sizeof(T);  // 16-byte rows, padded
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
  const int i0 = k1 + ti * TILE, j0 = k1 + tj * TILE;
  if (i0 >= f.M || j0 >= f.M) return;
  alignas(16) __shared__ T Ai[kPanel][LD];
  alignas(16) __shared__ T Aj[kPanel][LD];
  for (int t = threadIdx.x; t < TILE * nb; t += blockDim.x) {
    const int r = t / nb, q = t % nb;
    Ai[q][r] = i0 + r < f.M ? f.at(i0 + r, k0 + q) : T(0);
    Aj[q][r] = j0 + r < f.M ? f.at(j0 + r, k0 + q) : T(0);
  }
  __syncthreads();
  for (int g = threadIdx.x; g < 256; g += blockDim.x) {
    const int ty = g / 16, tx = g % 16;
    T acc[R][R];
#pragma unroll
    for (int a = 0; a < R; a++)
#pragma unroll
      for (int c = 0; c < R; c++) acc[a][c] = 0;
    for (int q = 0; q < nb; q++) {
#ifdef DK_EMULATE
      T x[R], y[R];
      for (int a = 0; a < R; a++) x[a] = Ai[q][ty * R + a];
      for (int c = 0; c < R; c++) y[c] = Aj[q][tx * R + c];
#else
      // 16-byte vectors (R entries, or R / VW vectors of VW)
      constexpr int VW = R * sizeof(T) <= 16 ? R : 16 / (int)sizeof(T);
      T x[R], y[R];
#pragma unroll
      for (int h = 0; h < R; h += VW) {
        const DkVec<T, VW> xv =
            *reinterpret_cast<const DkVec<T, VW> *>(&Ai[q][ty * R + h]);
        const DkVec<T, VW> yv =
            *reinterpret_cast<const DkVec<T, VW> *>(&Aj[q][tx * R + h]);
#pragma unroll
        for (int w = 0; w < VW; w++) {
          x[h + w] = xv.v[w];
          y[h + w] = yv.v[w];
        }
      }
#endif
#pragma unroll
      for (int a = 0; a < R; a++)
#pragma unroll
        for (int c = 0; c < R; c++) acc[a][c] += x[a] * y[c];
    }
#pragma unroll
    for (int a = 0; a < R; a++) {
      const int i = i0 + ty * R + a;
      if (i >= f.M) continue;
#pragma unroll
      for (int c = 0; c < R; c++) {
        const int j = j0 + tx * R + c;
        if (j <= i) f.at(i, j) -= acc[a][c];
      }
    }
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

// A 32 x 32 inverse of a diagonal block (dinv, row-major) into shared
// memory with padded rows: directly, or through registers (256 threads, 4
// entries each, coalesced) loaded before they are needed.
template <class T>
__device__ __forceinline__ void dk_inv_stage(T (*Ls)[33], const T *src) {
  for (int t = threadIdx.x; t < 1024; t += blockDim.x) Ls[t >> 5][t & 31] = src[t];
}
#ifndef DK_EMULATE
template <class T>
__device__ __forceinline__ void dk_inv_load(T (&pre)[4], const T *src) {
#pragma unroll
  for (int q = 0; q < 4; q++) pre[q] = src[threadIdx.x + 256 * q];
}
template <class T>
__device__ __forceinline__ void dk_inv_store(const T (&pre)[4],
                                             T (*Ls)[33]) {
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int t = threadIdx.x + 256 * q;
    Ls[t >> 5][t & 31] = pre[q];
  }
}
#endif

// Block solve with a staged inverse X: forward z = X z, or backward
// z = X^T z, on the block's nb entries (NR interleaved right-hand sides);
// the result also goes to zbuf when given.  Warp 0, lane i on entry i (the
// others return).
template <class T, int NR, bool kTranspose>
__device__ __forceinline__ void dk_inv_solve(const T (*X)[33], int nb, T *z,
                                             T *zbuf) {
#ifdef DK_EMULATE
  T out[32 * NR];
  for (int i = 0; i < nb; i++)
    for (int q = 0; q < NR; q++) {
      T acc = 0;
      if (kTranspose)
        for (int j = i; j < nb; j++) acc += X[j][i] * z[j * NR + q];
      else
        for (int j = 0; j <= i; j++) acc += X[i][j] * z[j * NR + q];
      out[i * NR + q] = acc;
    }
  for (int t = 0; t < nb * NR; t++) {
    z[t] = out[t];
    if (zbuf) zbuf[t] = out[t];
  }
#else
  if (threadIdx.x >= 32) return;
  const int i = threadIdx.x;
  T out[NR];
#pragma unroll
  for (int q = 0; q < NR; q++) out[q] = 0;
  if (i < nb) {
    if (kTranspose) {
      for (int j = i; j < nb; j++) {
        const T a = X[j][i];
#pragma unroll
        for (int q = 0; q < NR; q++) out[q] += a * z[j * NR + q];
      }
    } else {
      for (int j = 0; j <= i; j++) {
        const T a = X[i][j];
#pragma unroll
        for (int q = 0; q < NR; q++) out[q] += a * z[j * NR + q];
      }
    }
  }
  __syncwarp();
  if (i < nb)
#pragma unroll
    for (int q = 0; q < NR; q++) {
      z[i * NR + q] = out[q];
      if (zbuf) zbuf[i * NR + q] = out[q];
    }
#endif
}

#ifndef DK_EMULATE
// z(r0 + i) -= L(r0 + i, kb .. kb + nb) zk for the rows i < 32 of a row
// group with bit i of `valid` set, by one warp: lane c loads column c of
// every row (each row a coalesced load, all 32 issued together), then per
// butterfly the products of 32 / NR rows with the NR right-hand sides
// (entry i NR + q: row i, right-hand side q) are summed across the lanes
// by shuffles so that lane j holds entry j's sum (31 shuffles per 32
// sums).  L0: row r0's column kb; ldl: the panel's row stride; zrow(i):
// row i's NR entries of z.
template <class T, int NR, class ZRow>
__device__ __forceinline__ void dk_warp_rows(const T *L0, size_t ldl, int nb,
                                             const T *zk, unsigned valid,
                                             ZRow zrow) {
  constexpr int RB = 32 / NR;  // rows per butterfly
  const int lane = threadIdx.x & 31;
  T zc[NR];
#pragma unroll
  for (int q = 0; q < NR; q++) zc[q] = lane < nb ? zk[lane * NR + q] : T(0);
  T l[32];
#pragma unroll
  for (int i = 0; i < 32; i++)
    l[i] = ((valid >> i) & 1u) && lane < nb ? L0[(size_t)i * ldl + lane]
                                            : T(0);
#pragma unroll
  for (int g = 0; g < NR; g++) {
    T v[32];
#pragma unroll
    for (int i = 0; i < RB; i++)
#pragma unroll
      for (int q = 0; q < NR; q++) v[i * NR + q] = l[g * RB + i] * zc[q];
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
      const bool up = (lane & h) != 0;
#pragma unroll
      for (int i = 0; i < h; i++) {
        const T send = up ? v[i] : v[i + h];
        const T keep = up ? v[i + h] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
      }
    }
    const int r = g * RB + lane / NR;
    if ((valid >> r) & 1u) zrow(r)[lane % NR] -= v[0];
  }
}
#endif  // DK_EMULATE

// Row i's entries kb .. kb + nb of a panel times the block's solved
// entries zk (NR interleaved right-hand sides), added to acc in column
// order, with loads W entries wide (DkVec): a panel row of C entries starts
// on a W-entry boundary when the panel does and C is a multiple of W (kb
// is a multiple of 32), which dk_vec_width checks per front.
template <class T>
__device__ __forceinline__ int dk_vec_width(const T *lp, int C) {
  const unsigned long long a = (unsigned long long)lp;
  if (sizeof(T) == 4 && C % 4 == 0 && a % 16 == 0) return 4;
  if (C % 2 == 0 && a % (2 * sizeof(T)) == 0 && 2 * sizeof(T) <= 16)
    return 2;
  return 1;
}
template <class T, int NR, int W>
__device__ __forceinline__ void dk_row_dot_w(const T *Li, int nb,
                                             const T *zk, T (&acc)[NR]) {
  if (nb == 32) {  // a whole block: every load issued before the products
    constexpr int NV = 32 / W;
    DkVec<T, W> l[NV];
#pragma unroll
    for (int u = 0; u < NV; u++)
      l[u] = *reinterpret_cast<const DkVec<T, W> *>(Li + u * W);
#pragma unroll
    for (int u = 0; u < NV; u++)
#pragma unroll
      for (int w = 0; w < W; w++)
#pragma unroll
        for (int q = 0; q < NR; q++)
          acc[q] += l[u].v[w] * zk[(u * W + w) * NR + q];
    return;
  }
  int c = 0;
  for (; c + W <= nb; c += W) {
    const DkVec<T, W> l = *reinterpret_cast<const DkVec<T, W> *>(Li + c);
#pragma unroll
    for (int w = 0; w < W; w++)
#pragma unroll
      for (int q = 0; q < NR; q++) acc[q] += l.v[w] * zk[(c + w) * NR + q];
  }
  for (; c < nb; c++)
#pragma unroll
    for (int q = 0; q < NR; q++) acc[q] += Li[c] * zk[c * NR + q];
}
template <class T, int NR>
__device__ __forceinline__ void dk_row_dot(int W, const T *Li, int nb,
                                           const T *zk, T (&acc)[NR]) {
  if constexpr (sizeof(T) == 4) {
    if (W == 4) {
      dk_row_dot_w<T, NR, 4>(Li, nb, zk, acc);
      return;
    }
  }
  if (W == 2)
    dk_row_dot_w<T, NR, 2>(Li, nb, zk, acc);
  else
    dk_row_dot_w<T, NR, 1>(Li, nb, zk, acc);
}

// Columns j0 .. j0 + W of a panel (Lc = its entry in row 0, ldl = C)
// against z over the rows i0, i0 + step, .. < i1: acc[w] += L(i, j0 + w)
// z_i (NR interleaved right-hand sides), one W-wide load per row.
template <class T, int NR, int W>
__device__ __forceinline__ void dk_col_dot_w(const T *Lc, int ldl, int i0,
                                             int i1, int step, const T *z,
                                             T (&acc)[4][NR]) {
#pragma unroll 4
  for (int i = i0; i < i1; i += step) {
    const DkVec<T, W> l =
        *reinterpret_cast<const DkVec<T, W> *>(Lc + (size_t)i * ldl);
#pragma unroll
    for (int w = 0; w < W; w++)
#pragma unroll
      for (int q = 0; q < NR; q++) acc[w][q] += l.v[w] * z[i * NR + q];
  }
}
template <class T, int NR>
__device__ __forceinline__ void dk_col_dot(int W, const T *Lc, int ldl,
                                           int i0, int i1, int step,
                                           const T *z, T (&acc)[4][NR]) {
  if constexpr (sizeof(T) == 4) {
    if (W == 4) {
      dk_col_dot_w<T, NR, 4>(Lc, ldl, i0, i1, step, z, acc);
      return;
    }
  }
  if (W == 2)
    dk_col_dot_w<T, NR, 2>(Lc, ldl, i0, i1, step, z, acc);
  else
    dk_col_dot_w<T, NR, 1>(Lc, ldl, i0, i1, step, z, acc);
}

// acc = sum over c < nb of L(kb + c, j) zk(c) (NR interleaved right-hand
// sides; Lc = the entry (kb, j), ldl = the row stride), in c order; a
// whole block's loads are issued 16 (one right-hand side) or 8 at a time
// before their products.
template <class T, int NR>
__device__ __forceinline__ void dk_col_block(const T *Lc, size_t ldl, int nb,
                                             const T *zk, T (&acc)[NR]) {
#pragma unroll
  for (int q = 0; q < NR; q++) acc[q] = 0;
  if (nb == 32) {
    constexpr int H = NR == 1 ? 16 : 8;  // within the 64-register budget
#pragma unroll 1
    for (int h = 0; h < 32; h += H) {
      T l[H];
#pragma unroll
      for (int c = 0; c < H; c++) l[c] = Lc[(size_t)(h + c) * ldl];
#pragma unroll
      for (int c = 0; c < H; c++)
#pragma unroll
        for (int q = 0; q < NR; q++) acc[q] += l[c] * zk[(h + c) * NR + q];
    }
    return;
  }
  for (int c = 0; c < nb; c++) {
    const T l = Lc[(size_t)c * ldl];
#pragma unroll
    for (int q = 0; q < NR; q++) acc[q] += l * zk[c * NR + q];
  }
}

// position of front row i of supernode s in a factor-order vector
__device__ __forceinline__ size_t dk_pos(const int *rows, int bs, int i) {
  return (size_t)rows[i / bs] * bs + i % bs;
}

// Forward: z = front rows of the supernode (own rows from y, the rows
// below zero), plus the children's contribution vectors; L11 z1 = z1 and
// z2 -= L21 z1; own rows back to y, z2 to the supernode's contribution.
// Per column block: the block solve (with the kept inverse when the
// front was factored by panels, else by substitution), then the rows below
// it.  kDirectPlainThreads threads.
// CTAs per SM the one-CTA forward solve is compiled for (the register
// budget of its row loads in flight against the fronts resident per SM),
// per scalar type and right-hand-side count, as measured on the 48-plate
// batch: FP32 8 (one right-hand side) or 6, FP64 4 (one) or 8
template <class T, int NR>
struct DkForwardBlocks {
  static constexpr int value =
      sizeof(T) == 4 ? (NR == 1 ? 8 : 6) : (NR == 1 ? 4 : 8);
};

template <class T, int NR>
__global__ void __launch_bounds__(kDirectPlainThreads,
                                  DkForwardBlocks<T, NR>::value)
    direct_forward_kernel(DirectView v, const int *__restrict__ sn, int count,
                          T *y, T *contrib) {
  if ((int)blockIdx.x >= count) return;
  DK_DYN_SMEM(T, z);
  __shared__ T Ls[32][33];
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  T *D = z + (size_t)f.M * NR;
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  const bool inv = v.dinv_off[s] >= 0;
  const T *Xg = inv ? dk_dinv(v, (T *)nullptr) + v.dinv_off[s] : nullptr;
  const int W = dk_vec_width(f.lp, f.C);
  for (int i = threadIdx.x; i < f.M; i += blockDim.x) {
    T *zi = z + (size_t)i * NR;
    if (i < f.C) {
      const T *yi = y + dk_pos(rows, bs, i) * NR;
#pragma unroll
      for (int q = 0; q < NR; q++) zi[q] = yi[q];
    } else {
#pragma unroll
      for (int q = 0; q < NR; q++) zi[q] = T(0);
    }
  }
  __syncthreads();
  for (int k = v.ch_ptr[s]; k < v.ch_ptr[s + 1]; k++) {
    const int c = v.ch_list[k];
    const Front<T> fc = front_of<T>(v, c);
    const int um = fc.M - fc.C;
    const int *rel = v.ea_rel + v.ea_ptr[c];
    const T *w = contrib + v.v_off[c] * NR;
    for (int i = threadIdx.x; i < um; i += blockDim.x) {
      T *zi = z + (size_t)(rel[i / bs] * bs + i % bs) * NR;
      const T *wi = w + (size_t)i * NR;
#pragma unroll
      for (int q = 0; q < NR; q++) zi[q] += wi[q];
    }
    __syncthreads();
  }
  for (int kb = 0; kb < f.C; kb += kDirectSolveBlock) {
    const int nb = f.C - kb < kDirectSolveBlock ? f.C - kb : kDirectSolveBlock;
    if (inv) {
      dk_inv_stage(Ls, Xg + (size_t)(kb >> 5) * 1024);
      __syncthreads();
      dk_inv_solve<T, NR, false>(Ls, nb, z + kb * NR, (T *)nullptr);
    } else {
      dk_stage_block(f, kb, nb, D);
      __syncthreads();
      dk_block_solve<T, false, NR>(D, nb, z + kb * NR);
    }
    __syncthreads();
    // rows below the block: z_i -= L(i, kb .. kb+nb) z(kb .. kb+nb), one
    // thread per row (its loads independent and W entries wide, every one
    // serving the NR right-hand sides; measured faster here than
    // warp-per-row-group reductions or rows staged through shared memory)
    for (int i = kb + nb + threadIdx.x; i < f.M; i += blockDim.x) {
      T acc[NR];
#pragma unroll
      for (int q = 0; q < NR; q++) acc[q] = 0;
      dk_row_dot<T, NR>(W, f.lp + (size_t)i * f.C + kb, nb, z + kb * NR,
                        acc);
#pragma unroll
      for (int q = 0; q < NR; q++) z[(size_t)i * NR + q] -= acc[q];
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < f.C; i += blockDim.x) {
    const T *zi = z + (size_t)i * NR;
    T *yi = y + dk_pos(rows, bs, i) * NR;
#pragma unroll
    for (int q = 0; q < NR; q++) yi[q] = zi[q];
  }
  if (v.sn_parent[s] >= 0) {
    T *w = contrib + v.v_off[s] * NR;
    for (int t = f.C * NR + threadIdx.x; t < f.M * NR; t += blockDim.x)
      w[t - f.C * NR] = z[t];
  }
}

// Backward: z1 = y1 - L21^T x2 (x2 from the ancestors, already final),
// then L11^T z1 = z1 from the last block up (with the kept inverse when
// the front was factored by panels); own rows to x.  kDirectPlainThreads
// threads.
template <class T, int NR>
__global__ void __launch_bounds__(kDirectPlainThreads, 6)
    direct_backward_kernel(DirectView v, const int *__restrict__ sn,
                           int count, const T *y, T *x) {
  if ((int)blockIdx.x >= count) return;
  DK_DYN_SMEM(T, z);
  __shared__ T Ls[32][33];
  const int s = sn[blockIdx.x];
  const Front<T> f = front_of<T>(v, s);
  T *D = z + (size_t)f.M * NR;
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  const bool inv = v.dinv_off[s] >= 0;
  const T *Xg = inv ? dk_dinv(v, (T *)nullptr) + v.dinv_off[s] : nullptr;
  for (int i = threadIdx.x; i < f.M; i += blockDim.x) {
    const size_t g = dk_pos(rows, bs, i) * NR;
    const T *src = i < f.C ? y + g : x + g;
    T *zi = z + (size_t)i * NR;
#pragma unroll
    for (int q = 0; q < NR; q++) zi[q] = src[q];
  }
  __syncthreads();
  // own rows: z_j -= sum_{i >= C} L(i, j) z_i.  Tasks form a grid of
  // column groups (W adjacent columns, one W-wide load per row) by P
  // interleaved parts of the rows, at most kDirectPlainThreads tasks; the
  // parts' sums meet in shared memory after z (the staging area of the
  // block solves, free until they start) in a fixed order.
  {
    const int W = dk_vec_width(f.lp, f.C);
    const int ncg = f.C / W;  // W divides C
    int P = kDirectPlainThreads / (ncg > 0 ? ncg : 1);
    P = P < 1 ? 1 : P;
    for (int t = threadIdx.x; t < ncg * P; t += blockDim.x) {
      const int cg = t % ncg, pp = t / ncg, j0 = cg * W;
      T acc[4][NR];
#pragma unroll
      for (int w = 0; w < 4; w++)
#pragma unroll
        for (int q = 0; q < NR; q++) acc[w][q] = 0;
      dk_col_dot<T, NR>(W, f.lp + j0, f.C, f.C + pp, f.M, P, z, acc);
#pragma unroll
      for (int w = 0; w < 4; w++)
#pragma unroll
        for (int q = 0; q < NR; q++) {
          if (w >= W) continue;
          if (P == 1)
            z[(j0 + w) * NR + q] -= acc[w][q];
          else
            D[((size_t)pp * f.C + j0 + w) * NR + q] = acc[w][q];
        }
    }
    if (P > 1) {
      __syncthreads();
      for (int t = threadIdx.x; t < f.C * NR; t += blockDim.x) {
        T sum = 0;
        for (int pp = 0; pp < P; pp++) sum += D[(size_t)pp * f.C * NR + t];
        z[t] -= sum;
      }
    }
  }
  __syncthreads();
  for (int kb = ((f.C - 1) / kDirectSolveBlock) * kDirectSolveBlock; kb >= 0;
       kb -= kDirectSolveBlock) {
    const int nb = f.C - kb < kDirectSolveBlock ? f.C - kb : kDirectSolveBlock;
    if (inv) {
      dk_inv_stage(Ls, Xg + (size_t)(kb >> 5) * 1024);
      __syncthreads();
      dk_inv_solve<T, NR, true>(Ls, nb, z + kb * NR, (T *)nullptr);
    } else {
      dk_stage_block(f, kb, nb, D);
      __syncthreads();
      dk_block_solve<T, true, NR>(D, nb, z + kb * NR);
    }
    __syncthreads();
    // columns before the block: z_j -= sum_k L(kb + k, j) z(kb + k)
    // (a whole block's 32 loads issued 16 at a time, before their products)
    for (int j = threadIdx.x; j < kb; j += blockDim.x) {
      T acc[NR];
#pragma unroll
      for (int r = 0; r < NR; r++) acc[r] = 0;
      if (nb == 32) {
#pragma unroll
        for (int h = 0; h < 32; h += 16) {
          T l[16];
#pragma unroll
          for (int k = 0; k < 16; k++)
            l[k] = f.lp[(size_t)(kb + h + k) * f.C + j];
#pragma unroll
          for (int k = 0; k < 16; k++)
#pragma unroll
            for (int r = 0; r < NR; r++)
              acc[r] += l[k] * z[(kb + h + k) * NR + r];
        }
      } else {
        for (int k = 0; k < nb; k++) {
          const T l = f.lp[(size_t)(kb + k) * f.C + j];
#pragma unroll
          for (int r = 0; r < NR; r++) acc[r] += l * z[(kb + k) * NR + r];
        }
      }
#pragma unroll
      for (int r = 0; r < NR; r++) z[j * NR + r] -= acc[r];
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < f.C; i += blockDim.x) {
    const T *zi = z + (size_t)i * NR;
    T *xi = x + dk_pos(rows, bs, i) * NR;
#pragma unroll
    for (int q = 0; q < NR; q++) xi[q] = zi[q];
  }
}

#ifndef DK_EMULATE
// The backward solve's products L21^T x2 of the fronts solved by clusters
// (the part of their work that does not wait for the chain of diagonal
// blocks), over the whole GPU.  Tile = (front k of the level's list,
// 32-column block, chunk of kDirectGemvRows update rows), one warp each:
// lane = column (each row's load coalesced); the chunk's entries of x2
// are gathered once, lane i holding those of the rows i mod 32, and
// broadcast by shuffles.  part[(poff[k] + chunk C + j) NR + q] = the
// chunk's sum for column j (one writer per entry; the cluster kernel adds
// the chunks in order).  tprefix[k]: the tiles of fronts 0 .. k.
template <class T, int NR>
__global__ void __launch_bounds__(256)
    direct_bwd_gemv_kernel(DirectView v, const int *__restrict__ sn,
                           const int *__restrict__ tprefix,
                           const int64_t *__restrict__ poff, int count,
                           int total, const T *__restrict__ x,
                           T *__restrict__ part) {
  constexpr int U = kDirectGemvRows / 32;
  const int tile = (int)blockIdx.x * 8 + ((int)threadIdx.x >> 5);
  if (tile >= total) return;
  const int lane = (int)threadIdx.x & 31;
  int lo = 0, hi = count - 1;  // the first front whose prefix passes tile
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (tprefix[mid] > tile) hi = mid;
    else lo = mid + 1;
  }
  const int k = lo;
  const int lt = tile - (k > 0 ? tprefix[k - 1] : 0);
  const int s = sn[k];
  const Front<T> f = front_of<T>(v, s);
  const int ncb = (f.C + 31) >> 5;
  const int cb = lt % ncb, rc = lt / ncb;
  const int i0 = f.C + rc * kDirectGemvRows;
  const int nrow = f.M - i0 < kDirectGemvRows ? f.M - i0 : kDirectGemvRows;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  T xr[U][NR];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int r = lane + 32 * u;
    const size_t g = r < nrow ? dk_pos(rows, v.bs, i0 + r) * NR : 0;
#pragma unroll
    for (int q = 0; q < NR; q++) xr[u][q] = r < nrow ? x[g + q] : T(0);
  }
  const int j = cb * 32 + lane;
  const T *Lj = f.lp + (size_t)i0 * f.C + (j < f.C ? j : 0);
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; q++) acc[q] = 0;
#pragma unroll
  for (int u = 0; u < U; u++) {
#pragma unroll 16
    for (int w = 0; w < 32; w++) {
      const int r = 32 * u + w;
      if (r < nrow) {  // the same for the whole warp
        const T l = Lj[(size_t)r * f.C];
#pragma unroll
        for (int q = 0; q < NR; q++)
          acc[q] += l * __shfl_sync(0xffffffffu, xr[u][q], w);
      }
    }
  }
  if (j < f.C)
#pragma unroll
    for (int q = 0; q < NR; q++)
      part[(poff[k] + (int64_t)rc * f.C + j) * NR + q] = acc[q];
}
#endif  // DK_EMULATE

#ifndef DK_EMULATE
// Large fronts: one thread-block cluster of ncl CTAs (kDirectSolveCluster,
// or kDirectSolveClusterWide at the top levels; 256 threads each) per
// front, so that the front's triangular solves use that many SMs (one CTA per front leaves the top of the tree, a handful of
// fronts with thousands of rows, on one SM each).  The front's rows are
// dealt out in 32-row blocks: block b belongs to rank b % nr and sits in
// that CTA's shared memory at slot (b / nr) * 32.  Column block k is
// solved by its owner with the inverse of its diagonal block (kept by the
// factorisation, dinv: a 32 x 32 product instead of 32 dependent steps)
// and published in shared memory; the others read it through distributed
// shared memory after the cluster barrier.  The solve is pipelined one
// block ahead: once block k is known, the owner of block k + 1 first
// applies it to its 32 rows (forward) or columns (backward) of block k + 1,
// solves and publishes that block and arrives at the barrier, and only
// then applies block k to the rest of its rows; the others arrive as soon
// as they have read block k.  So the chain of dependent blocks costs one
// barrier, one 32-row update and one 32 x 32 product per block, and the
// bulk of the work runs beside it.  Every CTA of a cluster executes the
// same sequence of barrier arrivals and waits (block counts depend on the
// front only); a final barrier keeps each CTA's shared memory alive until
// the others are done reading it.  Dynamic shared memory: the owned rows
// (rounded up to whole blocks) x NR.
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
__global__ void __launch_bounds__(kDirectClusterThreads)
    direct_forward_cluster_kernel(DirectView v, const int *__restrict__ sn,
                                  int count, int ncl, T *y, T *contrib) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const ClusterRows cr{(int)cl.num_blocks(), (int)cl.block_rank()};
  // the shared memory is sized for ncl ranks: any other cluster shape
  // leaves (the whole cluster sees the same size)
  if (cr.nr != ncl) return;
  const int fi = (int)blockIdx.x / cr.nr;  // the same in the whole cluster
  if (fi >= count) return;
  DK_DYN_SMEM(T, z);
  __shared__ T zb[2][32 * NR], zk[32 * NR];
  __shared__ T Ls[32][33];
  const int s = sn[fi];
  const Front<T> f = front_of<T>(v, s);
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  const int nown = cr.count(f.M);
  const T *inv = dk_dinv(v, (T *)nullptr) + v.dinv_off[s];
  const int nblk = (f.C + 31) >> 5;
  const int warp = (int)threadIdx.x >> 5, nwarp = (int)blockDim.x >> 5;
  for (int t = threadIdx.x; t < nown; t += blockDim.x) {
    const int i = cr.row(t);
    T *zt = z + (size_t)t * NR;
    if (i < f.C) {
      const T *yi = y + dk_pos(rows, bs, i) * NR;
#pragma unroll
      for (int q = 0; q < NR; q++) zt[q] = yi[q];
    } else {
#pragma unroll
      for (int q = 0; q < NR; q++) zt[q] = T(0);
    }
  }
  __syncthreads();
  for (int k = v.ch_ptr[s]; k < v.ch_ptr[s + 1]; k++) {
    const int c = v.ch_list[k];
    const Front<T> fc = front_of<T>(v, c);
    const int um = fc.M - fc.C;
    const int *rel = v.ea_rel + v.ea_ptr[c];
    const T *w = contrib + v.v_off[c] * NR;
    for (int i = threadIdx.x; i < um; i += blockDim.x) {
      const int r = rel[i / bs] * bs + i % bs;
      if (!cr.owns(r)) continue;
      T *zr = z + (size_t)cr.slot(r) * NR;
      const T *wi = w + (size_t)i * NR;
#pragma unroll
      for (int q = 0; q < NR; q++) zr[q] += wi[q];
    }
    __syncthreads();
  }
  T pre[4];
  if (cr.rank == 0) {  // block 0: its rows are complete
    dk_inv_load(pre, inv);
    dk_inv_store(pre, Ls);
    __syncthreads();
    dk_inv_solve<T, NR, false>(Ls, f.C < 32 ? f.C : 32, z, zb[0]);
    __syncthreads();
  }
  cl.barrier_arrive();
  for (int k = 0; k < nblk; k++) {
    const int kb = k << 5, nb = f.C - kb < 32 ? f.C - kb : 32;
    const int k1 = k + 1, r1 = k1 << 5;
    const bool next_mine = k1 < nblk && k1 % cr.nr == cr.rank;
    const int nb1 = next_mine ? (f.C - r1 < 32 ? f.C - r1 : 32) : 0;
    if (next_mine) dk_inv_load(pre, inv + (size_t)k1 * 1024);
    cl.barrier_wait();
    const T *src = cl.map_shared_rank(&zb[k & 1][0], k % cr.nr);
    for (int t = threadIdx.x; t < nb * NR; t += blockDim.x) zk[t] = src[t];
    __syncthreads();
    if (next_mine) {
      dk_inv_store(pre, Ls);
      if (warp == 0) {
        T *zr1 = z + (size_t)cr.slot(r1) * NR;
        dk_warp_rows<T, NR>(
            f.lp + (size_t)r1 * f.C + kb, f.C, nb, zk,
            nb1 == 32 ? 0xffffffffu : (1u << nb1) - 1u,
            [&](int i) { return zr1 + i * NR; });
      }
      __syncthreads();
      dk_inv_solve<T, NR, false>(Ls, nb1, z + (size_t)cr.slot(r1) * NR,
                                 zb[k1 & 1]);
      __syncthreads();
    }
    if (k1 < nblk) cl.barrier_arrive();
    // the rest of this rank's rows below block k, a 32-row block per warp
    for (int g = warp; g < (nown >> 5); g += nwarp) {
      const int r0 = cr.row(g << 5);
      if (r0 + 32 <= kb + nb || r0 >= f.M) continue;
      unsigned valid = 0;
      for (int i = 0; i < 32; i++) {
        const int r = r0 + i;
        const bool ahead = r >= r1 && r < r1 + nb1;  // done ahead
        if (r >= kb + nb && r < f.M && !ahead) valid |= 1u << i;
      }
      if (!valid) continue;
      T *zg = z + (size_t)(g << 5) * NR;
      dk_warp_rows<T, NR>(f.lp + (size_t)r0 * f.C + kb, f.C, nb, zk,
                              valid, [&](int i) { return zg + i * NR; });
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
__global__ void __launch_bounds__(kDirectClusterThreads, 4)
    direct_backward_cluster_kernel(DirectView v, const int *__restrict__ sn,
                                   const int64_t *__restrict__ poff,
                                   int count, int ncl, const T *y, T *x,
                                   const T *part) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const ClusterRows cr{(int)cl.num_blocks(), (int)cl.block_rank()};
  if (cr.nr != ncl) return;  // as in the forward kernel
  const int fi = (int)blockIdx.x / cr.nr;
  if (fi >= count) return;
  DK_DYN_SMEM(T, z);
  __shared__ T zb[2][32 * NR], zk[32 * NR];
  __shared__ T Ls[32][33];
  const int s = sn[fi];
  const Front<T> f = front_of<T>(v, s);
  const int bs = v.bs;
  const int *rows = v.sn_rows + v.sn_rowptr[s];
  const int nown = cr.count(f.M);
  const T *inv = dk_dinv(v, (T *)nullptr) + v.dinv_off[s];
  const int nblk = (f.C + 31) >> 5;
  // own rows of the triangle: y1 - L21^T x2 (x2 final, from the
  // ancestors), the products summed over the update-row chunks of
  // direct_bwd_gemv_kernel in order
  {
    const int nrc = (f.M - f.C + kDirectGemvRows - 1) / kDirectGemvRows;
    const T *pf = part + poff[fi] * NR;
    for (int t = threadIdx.x; t < nown; t += blockDim.x) {
      const int j = cr.row(t);
      if (j >= f.C) continue;
      const size_t gj = dk_pos(rows, bs, j) * NR;
      T sum[NR];
#pragma unroll
      for (int q = 0; q < NR; q++) sum[q] = 0;
#pragma unroll 4
      for (int rc = 0; rc < nrc; rc++)
#pragma unroll
        for (int q = 0; q < NR; q++)
          sum[q] += pf[((size_t)rc * f.C + j) * NR + q];
#pragma unroll
      for (int q = 0; q < NR; q++) z[t * NR + q] = y[gj + q] - sum[q];
    }
    __syncthreads();
  }
  T pre[4];
  const int kt = nblk - 1;
  if (kt % cr.nr == cr.rank) {  // the last block: its rows are complete
    dk_inv_load(pre, inv + (size_t)kt * 1024);
    dk_inv_store(pre, Ls);
    __syncthreads();
    dk_inv_solve<T, NR, true>(Ls, f.C - (kt << 5),
                              z + (size_t)cr.slot(kt << 5) * NR, zb[kt & 1]);
    __syncthreads();
  }
  cl.barrier_arrive();
  for (int k = kt; k >= 0; k--) {
    const int kb = k << 5, nb = f.C - kb < 32 ? f.C - kb : 32;
    const int k1 = k - 1, r1 = k1 << 5;
    const bool next_mine = k1 >= 0 && k1 % cr.nr == cr.rank;
    if (next_mine) dk_inv_load(pre, inv + (size_t)k1 * 1024);
    cl.barrier_wait();
    const T *src = cl.map_shared_rank(&zb[k & 1][0], k % cr.nr);
    for (int t = threadIdx.x; t < nb * NR; t += blockDim.x) zk[t] = src[t];
    __syncthreads();
    if (next_mine) {
      dk_inv_store(pre, Ls);
      // this rank's columns of block k - 1 (a whole block: 32)
      if (threadIdx.x < 32) {
        const int j = r1 + (int)threadIdx.x;
        T acc[NR];
        dk_col_block<T, NR>(f.lp + (size_t)kb * f.C + j, f.C, nb, zk, acc);
        T *zj = z + (size_t)cr.slot(j) * NR;
#pragma unroll
        for (int q = 0; q < NR; q++) zj[q] -= acc[q];
      }
      __syncthreads();
      dk_inv_solve<T, NR, true>(Ls, 32, z + (size_t)cr.slot(r1) * NR,
                                zb[k1 & 1]);
      __syncthreads();
    }
    if (k1 >= 0) cl.barrier_arrive();
    // the rest of this rank's columns before block k
    for (int t = threadIdx.x; t < nown; t += blockDim.x) {
      const int j = cr.row(t);
      if (j >= kb) continue;
      if (next_mine && j >= r1) continue;  // done ahead
      T acc[NR];
      dk_col_block<T, NR>(f.lp + (size_t)kb * f.C + j, f.C, nb, zk, acc);
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

// b' = b - A_{:,c} b_c on the free dofs, b' = b on the constrained ones
// (c: the constrained dofs, whose rows of A are the identity), for nrhs
// right-hand sides ld apart (node order).  The right-hand-side kernel
// permutes b into the factor's order and interleaves it (ypos[t * nrhs +
// r]); the coupling kernel then subtracts A_{i,c} b_c on the block rows
// that have a block in a constrained column (bc_row[k] at factor position
// bc_pos[k], its blocks bc_blk[bc_ptr[k] .. bc_ptr[k + 1]), BCSR value
// indices), one thread per (row, dof, right-hand side); the unpermute
// kernel undoes the permutation.
template <class T>
__global__ void direct_rhs_kernel(int n, int bs, const int *perm,
                                  const T *b, T *ypos, int nrhs, size_t ld) {
  const size_t N = (size_t)n * bs, tot = N * nrhs;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t e = t / nrhs, r = t - nrhs * e;
    const int pos = (int)(e / bs), q = (int)(e % bs);
    ypos[t] = b[r * ld + (size_t)perm[pos] * bs + q];
  }
}
template <class T>
__global__ void direct_bc_couple_kernel(int nrow, int bs,
                                        const int *__restrict__ bc_row,
                                        const int *__restrict__ bc_pos,
                                        const int *__restrict__ bc_ptr,
                                        const int *__restrict__ bc_blk,
                                        const int *__restrict__ cols,
                                        const int *__restrict__ bcmask,
                                        const T *__restrict__ a, const T *b,
                                        T *ypos, int nrhs, size_t ld) {
  const size_t per = (size_t)bs * nrhs, tot = (size_t)nrow * per;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t k = t / per, e = t - per * k;
    const int q = (int)(e / nrhs), r = (int)(e - (size_t)nrhs * q);
    if ((bcmask[bc_row[k]] >> q) & 1) continue;  // a constrained row
    T acc = 0;
    for (int m = bc_ptr[k]; m < bc_ptr[k + 1]; m++) {
      const int blk = bc_blk[m], j = cols[blk], mask = bcmask[j];
      const T *Aq = a + ((size_t)blk * bs + q) * bs;
      const T *bj = b + r * ld + (size_t)j * bs;
      for (int p = 0; p < bs; p++)
        if ((mask >> p) & 1) acc += Aq[p] * bj[p];
    }
    ypos[((size_t)bc_pos[k] * bs + q) * nrhs + r] -= acc;
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
