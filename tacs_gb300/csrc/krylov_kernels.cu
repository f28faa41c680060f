// Device side of the batched restarted GMRES (GMRES::solve,
// src/bpmat/KSM.cpp:785-970) for sm_103a.
//
// A solve covers nsys independent systems at once: nrhs right-hand sides
// (vectors ld apart) times nseg disjoint row ranges of a block-diagonal
// operator.  Every vector operation is segmented by system through a chunk
// list (chunks never straddle two systems), the Hessenberg matrices, Givens
// rotations and convergence tests live in device memory (one thread per
// system), and the current Arnoldi index is a device integer.  The kernels
// of one Arnoldi step therefore have fixed arguments, so one captured CUDA
// graph of the step is replayed m times per restart with no host round trip.
// Every reduction is a fixed-order two-stage sum, so results do not depend
// on the launch configuration of a run.
#include <cmath>

#include "tg_internal.h"

namespace tg {
namespace {

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

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// partials[c * ldp + j] = sum over chunk c of W_j . w, j < k,
// k = (*kdev) + kofs (kdev may be null).  One block per chunk keeps its
// slice of w in registers and streams the k basis vectors past it, four at
// a time so their loads overlap.
template <int EPT>
__global__ void __launch_bounds__(256)
    kr_dots_partial(const double *__restrict__ W, size_t ld,
                    const int *__restrict__ kdev, int kofs,
                    const double *__restrict__ w, KrylovChunks ch,
                    double *__restrict__ partials, int ldp) {
  __shared__ double sh[8][64];
  const int k = (kdev ? *kdev : 0) + kofs;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = blockIdx.x; c < ch.nchunks; c += gridDim.x) {
    const size_t start = (size_t)ch.start[c];
    const int len = ch.len[c];
    double wr[EPT];
#pragma unroll
    for (int e = 0; e < EPT; e++) {
      const int o = threadIdx.x + 256 * e;
      wr[e] = o < len ? w[start + o] : 0.0;
    }
    for (int j0 = 0; j0 < k; j0 += 64) {
      const int jn = k - j0 < 64 ? k - j0 : 64;
      int jj = 0;
      for (; jj + 4 <= jn; jj += 4) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int e = 0; e < EPT; e++) {
          const int o = threadIdx.x + 256 * e;
          if (o < len) {
#pragma unroll
            for (int q = 0; q < 4; q++)
              acc[q] += W[(size_t)(j0 + jj + q) * ld + start + o] * wr[e];
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
          for (int q = 0; q < 4; q++)
            acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
        if (lane == 0) {
#pragma unroll
          for (int q = 0; q < 4; q++) sh[warp][jj + q] = acc[q];
        }
      }
      for (; jj < jn; jj++) {
        const double *Wj = W + (size_t)(j0 + jj) * ld + start;
        double acc = 0.0;
#pragma unroll
        for (int e = 0; e < EPT; e++) {
          const int o = threadIdx.x + 256 * e;
          if (o < len) acc += Wj[o] * wr[e];
        }
        acc = warp_sum(acc);
        if (lane == 0) sh[warp][jj] = acc;
      }
      __syncthreads();
      if (threadIdx.x < jn) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < 8; q++) t += sh[q][threadIdx.x];
        partials[(size_t)c * ldp + j0 + threadIdx.x] = t;
      }
      __syncthreads();
    }
  }
}

// out[s * ldo + j] = sum over the chunks of system s of partials[c][j]
__global__ void kr_dots_final(const double *__restrict__ partials, int ldp,
                              const int *__restrict__ kdev, int kofs,
                              KrylovChunks ch, double *__restrict__ out,
                              int ldo) {
  const int k = (kdev ? *kdev : 0) + kofs;
  const int s = blockIdx.x;
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (s >= ch.nsys || j >= k) return;
  const int c0 = ch.sys_ptr[s], c1 = ch.sys_ptr[s + 1];
  double t = 0.0;
#pragma unroll 4
  for (int c = c0; c < c1; c++) t += partials[(size_t)c * ldp + j];
  out[(size_t)s * ldo + j] = t;
}

// w -= sum_j coef[sys][j] W_j over k = (*kdev) + kofs vectors; optionally
// normparts[c] = sum over chunk c of the updated w^2
template <int EPT>
__global__ void __launch_bounds__(256)
    kr_gemv_sub(const double *__restrict__ W, size_t ld,
                const int *__restrict__ kdev, int kofs,
                const double *__restrict__ coef, int ldc, KrylovChunks ch,
                double *__restrict__ w, double *__restrict__ normparts) {
  extern __shared__ double scoef[];
  __shared__ double sh[8];
  const int k = (kdev ? *kdev : 0) + kofs;
  for (int c = blockIdx.x; c < ch.nchunks; c += gridDim.x) {
    const size_t start = (size_t)ch.start[c];
    const int len = ch.len[c];
    const double *cf = coef + (size_t)ch.sys[c] * ldc;
    for (int j = threadIdx.x; j < k; j += blockDim.x) scoef[j] = cf[j];
    __syncthreads();
    double sq = 0.0;
#pragma unroll
    for (int e = 0; e < EPT; e++) {
      const int o = threadIdx.x + 256 * e;
      if (o < len) {
        const double *Wc = W + start + o;
        double acc = w[start + o];
        int j = 0;
        for (; j + 4 <= k; j += 4) {
          const double w0 = Wc[(size_t)j * ld], w1 = Wc[(size_t)(j + 1) * ld];
          const double w2 = Wc[(size_t)(j + 2) * ld],
                       w3 = Wc[(size_t)(j + 3) * ld];
          acc -= scoef[j] * w0;
          acc -= scoef[j + 1] * w1;
          acc -= scoef[j + 2] * w2;
          acc -= scoef[j + 3] * w3;
        }
        for (; j < k; j++) acc -= scoef[j] * Wc[(size_t)j * ld];
        w[start + o] = acc;
        sq += acc * acc;
      }
    }
    if (normparts) {
      sq = warp_sum(sq);
      if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = sq;
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < 8; q++) t += sh[q];
        normparts[c] = t;
      }
    }
    __syncthreads();
  }
}

// W_{*it} = v = scale[sys] * w (exact zero for a zero scale, so an inactive
// system carries no stale values into the next step)
__global__ void kr_scale_store(const double *__restrict__ w, KrylovChunks ch,
                               const double *__restrict__ scale,
                               double *__restrict__ W, size_t ld,
                               const int *__restrict__ it,
                               double *__restrict__ v) {
  const size_t base = (size_t)(*it) * ld;
  for (int c = blockIdx.x; c < ch.nchunks; c += gridDim.x) {
    const size_t start = (size_t)ch.start[c];
    const int len = ch.len[c];
    const double a = scale[ch.sys[c]];
    for (int o = threadIdx.x; o < len; o += blockDim.x) {
      const double val = a == 0.0 ? 0.0 : a * w[start + o];
      W[base + start + o] = val;
      v[start + o] = val;
    }
  }
}

// Z_{*it} = z (flexible GMRES keeps every preconditioned basis vector)
__global__ void kr_store_at(const double *__restrict__ z, double *__restrict__ Z,
                            size_t ld, const int *__restrict__ it) {
  const size_t base = (size_t)(*it) * ld;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ld;
       i += (size_t)gridDim.x * blockDim.x)
    Z[base + i] = z[i];
}

// r = b - r (r holds A x on entry)
__global__ void kr_residual(const double *__restrict__ b, double *__restrict__ r,
                            size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}
__global__ void kr_axpy(const double *__restrict__ x, double *__restrict__ y,
                        size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] += x[i];
}
// per-system scale of a segmented vector (used to mask finished systems)
__global__ void kr_mask(double *__restrict__ x, KrylovChunks ch,
                        const double *__restrict__ scale) {
  for (int c = blockIdx.x; c < ch.nchunks; c += gridDim.x) {
    const size_t start = (size_t)ch.start[c];
    const double a = scale[ch.sys[c]];
    if (a == 1.0) continue;
    for (int o = threadIdx.x; o < ch.len[c]; o += blockDim.x)
      x[start + o] = a == 0.0 ? 0.0 : a * x[start + o];
  }
}

__device__ void count_active(const KrylovState &st, int s, int local) {
  // one block covers all systems (nsys <= 1024)
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  if (local) atomicAdd(&cnt, 1);
  __syncthreads();
  if (threadIdx.x == 0) *st.nactive = cnt;
  (void)s;
}

// Start of a restart cycle: the true residual norms are in st.nrm2.
__global__ void kr_cycle_init(KrylovState st) {
  const int s = threadIdx.x;
  int act = 0;
  if (s < st.nsys) {
    const double rn0 = sqrt(st.nrm2[s]);
    if (*st.first) st.rhs_norm[s] = rn0;
    st.res[(size_t)s * (st.m + 1)] = rn0;
    st.niters[s] = 0;
    st.rn[s] = rn0;
    if (!isfinite(rn0)) st.err[s] = 1;
    if (st.converged[s] || st.err[s] || st.done[s]) {
      act = 0;
    } else if (rn0 == 0.0 || rn0 < st.atol ||
               rn0 <= st.rtol[s] * st.rhs_norm[s]) {
      st.converged[s] = 1;
      act = 0;
    } else if (!*st.first && *st.stall && rn0 > 0.9 * st.rn0prev[s]) {
      st.done[s] = 1;  // stalled restart
      act = 0;
    } else {
      act = 1;
    }
    st.rn0prev[s] = rn0;
    st.active[s] = act;
    st.scale[s] = act ? 1.0 / rn0 : 0.0;
  }
  count_active(st, s, act);
  __syncthreads();
  if (threadIdx.x == 0) {
    *st.first = 0;
    *st.it = 0;
  }
}

// Arnoldi step *st.it: Hessenberg column from the two Gram-Schmidt passes
// and the norm, previous rotations, the new rotation, the residual
// estimate and the convergence test; then advances *st.it.
__global__ void kr_arnoldi(KrylovState st) {
  const int s = threadIdx.x;
  const int i = *st.it;
  const int m = st.m;
  int act = 0;
  if (s < st.nsys) {
    act = st.active[s];
    if (!act) {
      st.scale[s] = 0.0;
    } else {
      double *Hc = st.H + (size_t)s * (m + 1) * m + (size_t)(m + 1) * i;
      const double *h1 = st.h1 + (size_t)s * (m + 1);
      const double *h2 = st.h2 + (size_t)s * (m + 1);
      double *Qc = st.Qc + (size_t)s * m, *Qs = st.Qs + (size_t)s * m;
      double *res = st.res + (size_t)s * (m + 1);
      const double nrm = sqrt(st.nrm2[s]);
      st.scale[s] = nrm > 0.0 ? 1.0 / nrm : 0.0;
      // previous rotations: rotation j mixes entries j and j+1, so only the
      // running entry (carry) depends on the previous step; the column's
      // other entries and the rotations load independently
      double carry = h1[0] + h2[0];
      for (int j = 0; j < i; j++) {
        const double b = h1[j + 1] + h2[j + 1];
        const double c = Qc[j], sn = Qs[j];
        Hc[j] = carry * c + b * sn;
        carry = -carry * sn + b * c;
      }
      const double a = carry, b = nrm;
      const double sq = sqrt(a * a + b * b);
      Qc[i] = a / sq;
      Qs[i] = b / sq;
      Hc[i] = a * Qc[i] + b * Qs[i];
      Hc[i + 1] = -a * Qs[i] + b * Qc[i];
      const double r = res[i];
      res[i] = r * Qc[i];
      res[i + 1] = -r * Qs[i];
      const double rn = fabs(res[i + 1]);
      st.rn[s] = rn;
      if (!isfinite(rn)) {
        st.err[s] = 1;
        st.niters[s] = i;  // drop the step that produced it
        act = 0;
      } else {
        st.niters[s] = i + 1;
        if (rn < st.atol || rn < st.rtol[s] * st.rhs_norm[s]) {
          st.converged[s] = 1;
          act = 0;
        }
      }
      if (!act) st.scale[s] = 0.0;
      st.active[s] = act;
    }
  }
  count_active(st, s, act);
  __syncthreads();
  if (threadIdx.x == 0) *st.it = i + 1;
}

// End of a cycle: back-substitution H y = res over each system's own step
// count; coefficients -y are left in res (zero beyond the step count) for
// the update x += M^{-1} sum_j y_j W_j.
__global__ void kr_solve_y(KrylovState st) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= st.nsys) return;
  const int m = st.m;
  const int ni = st.niters[s];
  const double *H = st.H + (size_t)s * (m + 1) * m;
  double *res = st.res + (size_t)s * (m + 1);
  for (int i = ni - 1; i >= 0; i--) {
    double r = res[i];
    for (int j = i + 1; j < ni; j++) r = r - H[(size_t)(m + 1) * j + i] * res[j];
    res[i] = r / H[(size_t)(m + 1) * i + i];
  }
  for (int i = 0; i < ni; i++) res[i] = -res[i];
  for (int i = ni; i <= m; i++) res[i] = 0.0;
  st.iters[s] += ni;
}

// Loop control of a restart cycle's WHILE node: continue while a system is
// active and the cycle has room for another step (kr_arnoldi advances
// *st.it every step, kr_cycle_init resets it: at most m steps per cycle).
__global__ void kr_loop_control(KrylovState st, cudaGraphConditionalHandle h,
                                int m) {
  cudaGraphSetConditional(h, (*st.nactive > 0 && *st.it < m) ? 1u : 0u);
}

int grid_chunks(int nchunks) {
  int cap = sm_count() * 8;
  return nchunks < cap ? (nchunks > 0 ? nchunks : 1) : cap;
}
int grid_elems(size_t n) {
  size_t b = (n + 255) / 256;
  size_t cap = (size_t)sm_count() * 8;
  if (b < 1) b = 1;
  return (int)(b < cap ? b : cap);
}

}  // namespace

void launch_kr_dots(const double *W, size_t ld, const int *kdev, int kofs,
                    int kmax, const double *w, const KrylovChunks &ch,
                    double *partials, double *out, int ldo, cudaStream_t s) {
  const int g = grid_chunks(ch.nchunks);
  switch (ch.ept) {
    case 1: kr_dots_partial<1><<<g, 256, 0, s>>>(W, ld, kdev, kofs, w, ch, partials, kmax); break;
    case 2: kr_dots_partial<2><<<g, 256, 0, s>>>(W, ld, kdev, kofs, w, ch, partials, kmax); break;
    case 4: kr_dots_partial<4><<<g, 256, 0, s>>>(W, ld, kdev, kofs, w, ch, partials, kmax); break;
    default: kr_dots_partial<8><<<g, 256, 0, s>>>(W, ld, kdev, kofs, w, ch, partials, kmax); break;
  }
  dim3 gf(ch.nsys, (kmax + 127) / 128);
  kr_dots_final<<<gf, 128, 0, s>>>(partials, kmax, kdev, kofs, ch, out, ldo);
}

void launch_kr_gemv_sub(const double *W, size_t ld, const int *kdev, int kofs,
                        int kmax, const double *coef, int ldc,
                        const KrylovChunks &ch, double *w, double *normparts,
                        cudaStream_t s) {
  const int g = grid_chunks(ch.nchunks);
  const size_t sm = sizeof(double) * (kmax > 0 ? kmax : 1);
  switch (ch.ept) {
    case 1: kr_gemv_sub<1><<<g, 256, sm, s>>>(W, ld, kdev, kofs, coef, ldc, ch, w, normparts); break;
    case 2: kr_gemv_sub<2><<<g, 256, sm, s>>>(W, ld, kdev, kofs, coef, ldc, ch, w, normparts); break;
    case 4: kr_gemv_sub<4><<<g, 256, sm, s>>>(W, ld, kdev, kofs, coef, ldc, ch, w, normparts); break;
    default: kr_gemv_sub<8><<<g, 256, sm, s>>>(W, ld, kdev, kofs, coef, ldc, ch, w, normparts); break;
  }
}

void launch_kr_norm_final(const double *normparts, const KrylovChunks &ch,
                          double *out, cudaStream_t s) {
  kr_dots_final<<<dim3(ch.nsys, 1), 128, 0, s>>>(normparts, 1, nullptr, 1,
                                                  ch, out, 1);
}

void launch_kr_scale_store(const double *w, const KrylovChunks &ch,
                           const double *scale, double *W, size_t ld,
                           const int *it, double *v, cudaStream_t s) {
  kr_scale_store<<<grid_chunks(ch.nchunks), 256, 0, s>>>(w, ch, scale, W, ld,
                                                          it, v);
}
void launch_kr_store_at(const double *z, double *Z, size_t ld, const int *it,
                        cudaStream_t s) {
  kr_store_at<<<grid_elems(ld), 256, 0, s>>>(z, Z, ld, it);
}
void launch_kr_residual(const double *b, double *r, size_t n, cudaStream_t s) {
  kr_residual<<<grid_elems(n), 256, 0, s>>>(b, r, n);
}
void launch_kr_axpy(const double *x, double *y, size_t n, cudaStream_t s) {
  kr_axpy<<<grid_elems(n), 256, 0, s>>>(x, y, n);
}
void launch_kr_mask(double *x, const KrylovChunks &ch, const double *scale,
                    cudaStream_t s) {
  kr_mask<<<grid_chunks(ch.nchunks), 256, 0, s>>>(x, ch, scale);
}
void launch_kr_cycle_init(const KrylovState &st, cudaStream_t s) {
  kr_cycle_init<<<1, ((st.nsys + 31) / 32) * 32, 0, s>>>(st);
}
void launch_kr_arnoldi(const KrylovState &st, cudaStream_t s) {
  kr_arnoldi<<<1, ((st.nsys + 31) / 32) * 32, 0, s>>>(st);
}
void launch_kr_loop_control(const KrylovState &st,
                            cudaGraphConditionalHandle h, int m,
                            cudaStream_t s) {
  kr_loop_control<<<1, 1, 0, s>>>(st, h, m);
}
void launch_kr_solve_y(const KrylovState &st, cudaStream_t s) {
  kr_solve_y<<<(st.nsys + 127) / 128, 128, 0, s>>>(st);
}

}  // namespace tg
