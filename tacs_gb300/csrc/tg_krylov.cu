// Host side of the batched restarted GMRES: the tg_ksm_* entry points of
// include/tacs_gb300.h (GMRES, src/bpmat/KSM.h / KSM.cpp:785-970).
//
// One restart cycle is three CUDA graphs captured once per multivector
// layout: the cycle start (true residual, per-system norms, first basis
// vector), one Arnoldi step (operator, two classical Gram-Schmidt passes,
// norm, Givens update on the device) replayed up to m times, and the cycle
// end (back-substitution and x += M^{-1} V y).  They are also composed into
// one graph per cycle whose WHILE node repeats the Arnoldi step on the
// device until every system converged or m steps ran; the host then reads
// one integer (systems still iterating) per cycle.  Without conditional
// nodes the host launches the step graph and reads that integer every few
// steps.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tg_objects.h"

namespace {

constexpr int kCheckEvery = 8;
constexpr int kMaxSystems = 1024;

// out = M^{-1} in on the multivector; a FP32 pc is applied through FP32
// copies of in and out
void enqueue_pc(tg_ksm *k, const double *in, double *out, cudaStream_t s) {
  tg_pc *pc = k->pc;
  if (!pc) {
    cudaMemcpyAsync(out, in, k->N * sizeof(double), cudaMemcpyDeviceToDevice,
                    s);
  } else if (pc->precision == TG_PREC_FP64 || k->mixed) {
    // a mixed-precision solve's FP64 passes use the FP64 factor
    pc_launch(pc, k->nrhs, k->n, in, out, k->d_t64, k->d_px, k->d_py, s, 1);
  } else {
    launch_d2f(in, k->d_x32, k->N, s);
    pc_launch(pc, k->nrhs, k->n, k->d_x32, k->d_y32, k->d_t32, k->d_px32,
              k->d_py32, s);
    launch_f2d(k->d_y32, out, k->N, s);
  }
}

// w = A M^{-1} v.  Mode 0: FP64 mat-vec; mode 1 (mixed precision): FP32
// preconditioner and FP32 mat-vec on an FP32 copy of v.
void enqueue_op(tg_ksm *k, int mode, cudaStream_t s) {
  tg_mat *A = k->A;
  const int *rowp = A->a->d_rowp, *cols = A->a->d_cols;
  if (mode == 0) {
    const double *src = k->d_v;
    if (k->pc) {
      enqueue_pc(k, k->d_v, k->d_z, s);
      src = k->d_z;
      if (k->flexible) launch_kr_store_at(k->d_z, k->d_Z, k->N, k->st.it, s);
    }
    launch_bcsr_mult(A->bsize, A->nrows, rowp, cols, A->d_vals, src, k->d_w,
                     s, k->nrhs, k->n);
  } else {
    launch_d2f(k->d_v, k->d_x32, k->N, s);
    pc_launch(k->pc, k->nrhs, k->n, k->d_x32, k->d_y32, k->d_t32, k->d_px32,
              k->d_py32, s);
    if (k->flexible) {
      launch_f2d(k->d_y32, k->d_z, k->N, s);
      launch_kr_store_at(k->d_z, k->d_Z, k->N, k->st.it, s);
    }
    launch_bcsr_mult_f32(A->bsize, A->nrows, rowp, cols, A->d_vals32,
                         k->d_y32, k->d_w32, s, k->nrhs, k->n);
    launch_f2d(k->d_w32, k->d_w, k->N, s);
  }
}

void enqueue_start(tg_ksm *k, cudaStream_t s) {
  tg_mat *A = k->A;
  const size_t N = k->N;
  launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols, A->d_vals,
                   k->d_X, k->d_w, s, k->nrhs, k->n);
  launch_kr_residual(k->d_B, k->d_w, N, s);
  launch_kr_dots(k->d_w, N, nullptr, 1, 1, k->d_w, k->ch, k->d_partials,
                 k->st.nrm2, 1, s);
  launch_kr_cycle_init(k->st, s);
  launch_kr_scale_store(k->d_w, k->ch, k->st.scale, k->d_W, N, k->st.it,
                        k->d_v, s);
}

void enqueue_iter(tg_ksm *k, int mode, cudaStream_t s) {
  const size_t N = k->N;
  const int m = k->m;
  enqueue_op(k, mode, s);
  launch_kr_dots(k->d_W, N, k->st.it, 1, m + 1, k->d_w, k->ch, k->d_partials,
                 k->st.h1, m + 1, s);
  launch_kr_gemv_sub(k->d_W, N, k->st.it, 1, m + 1, k->st.h1, m + 1, k->ch,
                     k->d_w, nullptr, s);
  launch_kr_dots(k->d_W, N, k->st.it, 1, m + 1, k->d_w, k->ch, k->d_partials,
                 k->st.h2, m + 1, s);
  launch_kr_gemv_sub(k->d_W, N, k->st.it, 1, m + 1, k->st.h2, m + 1, k->ch,
                     k->d_w, k->d_normparts, s);
  launch_kr_norm_final(k->d_normparts, k->ch, k->st.nrm2, s);
  launch_kr_arnoldi(k->st, s);
  launch_kr_scale_store(k->d_w, k->ch, k->st.scale, k->d_W, N, k->st.it,
                        k->d_v, s);
}

void enqueue_end(tg_ksm *k, cudaStream_t s) {
  const size_t N = k->N;
  launch_kr_solve_y(k->st, s);
  if (k->flexible) {
    // x += Z y with the stored preconditioned vectors (flexible GMRES)
    launch_kr_gemv_sub(k->d_Z, N, nullptr, k->m, k->m, k->st.res, k->m + 1,
                       k->ch, k->d_X, nullptr, s);
    return;
  }
  cudaMemsetAsync(k->d_z, 0, N * sizeof(double), s);
  launch_kr_gemv_sub(k->d_W, N, nullptr, k->m, k->m, k->st.res, k->m + 1,
                     k->ch, k->d_z, nullptr, s);
  enqueue_pc(k, k->d_z, k->d_z2, s);
  launch_kr_axpy(k->d_z2, k->d_X, N, s);
}

template <typename F>
int capture(cudaGraphExec_t *out, F &&body, int *nodes = nullptr) {
  cudaStream_t cs;
  TG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    body(cs);
    e = cudaStreamEndCapture(cs, &g);
  }
  if (e == cudaSuccess && nodes) {
    size_t n = 0;
    e = cudaGraphGetNodes(g, nullptr, &n);
    *nodes = (int)n;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) return cuda_check(e, "GMRES graph capture");
  return 0;
}

// One restart cycle as one graph: start, loop control, a WHILE node whose
// body is the Arnoldi step of the given operator mode followed by the loop
// control, then the end of the cycle.  The steps run back to back on the
// device with no host round trip; the loop runs at most m times.  Returns
// 0 with *out null (not an error) where the driver or runtime does not
// build conditional nodes.
int capture_cycle(tg_ksm *k, int mode, cudaGraphExec_t *out) {
  *out = nullptr;
  cudaGraph_t g = nullptr;
  cudaStream_t cs = nullptr, cb = nullptr;
  cudaGraphConditionalHandle h{};
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e == cudaSuccess)
    e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cb, cudaStreamNonBlocking);
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    enqueue_start(k, cs);
    launch_kr_loop_control(k->st, h, k->m, cs);
    cudaStreamCaptureStatus cst;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    cudaGraphNode_t wn = nullptr;
    cudaGraphNodeParams np = {};
    e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &nd);
    if (e == cudaSuccess) {
      np.type = cudaGraphNodeTypeConditional;
      np.conditional.handle = h;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      e = cudaGraphAddNode(&wn, cg, deps, nullptr, nd, &np);
    }
    if (e == cudaSuccess)
      e = cudaStreamUpdateCaptureDependencies(cs, &wn, nullptr, 1,
                                              cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess) {
      cudaGraph_t body = np.conditional.phGraph_out[0];
      e = cudaStreamBeginCaptureToGraph(cb, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed);
      if (e == cudaSuccess) {
        enqueue_iter(k, mode, cb);
        launch_kr_loop_control(k->st, h, k->m, cb);
        cudaGraph_t bo = nullptr;
        e = cudaStreamEndCapture(cb, &bo);
      }
    }
    if (e == cudaSuccess) enqueue_end(k, cs);
    cudaGraph_t go = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &go);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  if (cb) cudaStreamDestroy(cb);
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    *out = nullptr;
    cudaGetLastError();  // the per-step graphs remain in use
  }
  return 0;
}

// Allocate buffers, the chunk list and the state for nrhs vectors, and
// capture the cycle graphs.
int ensure_layout(tg_ksm *k, int nrhs) {
  const long long pv = pc_layout_version(k->pc);
  if (k->nrhs == nrhs && k->pc_version == pv) return 0;
  k->free_layout();
  k->pc_version = pv;
  const int nseg = (int)k->seg_rows.size() - 1;
  const int nsys = nseg * nrhs;
  if (nsys > kMaxSystems)
    return fail(TG_ERR_ARG, "GMRES: more than 1024 systems in one solve");
  const int bs = k->A->bsize;
  const size_t n = k->n, N = n * nrhs;
  const int m = k->m;
  if (N > (size_t)0x7fffffff)
    return fail(TG_ERR_ARG, "GMRES: multivector longer than 2^31 entries");
  // chunk size: enough chunks to cover the SMs a few times over
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  int ept = 1;
  while (ept < 8 && (size_t)256 * ept * sms * 4 < N) ept *= 2;
  const int CH = 256 * ept;
  std::vector<int> cstart, clen, csys, sys_ptr(1, 0);
  for (int l = 0; l < nrhs; l++)
    for (int g = 0; g < nseg; g++) {
      const size_t b = l * n + (size_t)k->seg_rows[g] * bs;
      const size_t e = l * n + (size_t)k->seg_rows[g + 1] * bs;
      for (size_t c = b; c < e; c += CH) {
        cstart.push_back((int)c);
        clen.push_back((int)std::min<size_t>(CH, e - c));
        csys.push_back(l * nseg + g);
      }
      sys_ptr.push_back((int)cstart.size());
    }
  const int nchunks = (int)cstart.size();
  int rc = 0;
  if (!rc) rc = dalloc(&k->d_W, N * (m + 1));
  if (!rc && k->flexible) rc = dalloc(&k->d_Z, N * m);
  if (!rc) rc = dalloc(&k->d_v, N);
  if (!rc) rc = dalloc(&k->d_w, N);
  if (!rc) rc = dalloc(&k->d_z, N);
  if (!rc) rc = dalloc(&k->d_z2, N);
  if (!rc) rc = dalloc(&k->d_B, N);
  if (!rc) rc = dalloc(&k->d_X, N);
  if (!rc) rc = dalloc(&k->d_Bo, N);
  if (!rc) rc = dalloc(&k->d_Xo, N);
  tg_pc *pc = k->pc;
  if (!rc && pc && (pc->precision == TG_PREC_FP64 || k->mixed)) {
    rc = dalloc(&k->d_t64, N);
    if (!rc && pc->type == TG_PC_ILU0_COLORED) rc = dalloc(&k->d_px, N);
    if (!rc && pc->type == TG_PC_ILU0_COLORED) rc = dalloc(&k->d_py, N);
  }
  if (!rc && pc && pc->precision == TG_PREC_FP32) {
    rc = dalloc(&k->d_x32, N);
    if (!rc) rc = dalloc(&k->d_y32, N);
    if (!rc) rc = dalloc(&k->d_w32, N);
    if (!rc) rc = dalloc(&k->d_t32, N);
    if (!rc && pc->type == TG_PC_ILU0_COLORED) rc = dalloc(&k->d_px32, N);
    if (!rc && pc->type == TG_PC_ILU0_COLORED) rc = dalloc(&k->d_py32, N);
  }
  if (!rc) rc = dalloc(&k->d_partials, (size_t)(m + 2) * nchunks);
  if (!rc) rc = dalloc(&k->d_normparts, (size_t)nchunks);
  if (!rc) rc = upload(&k->d_cstart, cstart);
  if (!rc) rc = upload(&k->d_clen, clen);
  if (!rc) rc = upload(&k->d_csys, csys);
  if (!rc) rc = upload(&k->d_sys_ptr, sys_ptr);
  // per-system state
  const size_t S1 = (size_t)nsys;
  const size_t nd = S1 * ((size_t)(m + 1) * m + 2 * m + 3 * (m + 1) + 7);
  const size_t ni = S1 * 6 + 4;
  if (!rc) rc = dalloc(&k->d_sd, nd);
  if (!rc) rc = dalloc(&k->d_si, ni);
  if (!rc && !k->h_pinned) {
    cudaError_t e = cudaMallocHost((void **)&k->h_pinned, 4 * sizeof(int));
    if (e != cudaSuccess) rc = cuda_check(e, "cudaMallocHost");
  }
  if (rc) {
    k->free_layout();
    return rc;
  }
  // every basis slot starts at zero: the end-of-cycle update multiplies
  // slots past a system's step count by zero coefficients
  cudaMemset(k->d_W, 0, N * (m + 1) * sizeof(double));
  if (k->d_Z) cudaMemset(k->d_Z, 0, N * m * sizeof(double));
  cudaMemset(k->d_sd, 0, nd * sizeof(double));
  cudaMemset(k->d_si, 0, ni * sizeof(int));
  k->nrhs = nrhs;
  k->N = N;
  k->nsys = nsys;
  k->ch = KrylovChunks{k->d_cstart, k->d_clen, k->d_csys, k->d_sys_ptr,
                       nchunks, nsys, ept};
  KrylovState &st = k->st;
  st.m = m;
  st.nsys = nsys;
  st.atol = k->atol;
  double *p = k->d_sd;
  st.H = p; p += S1 * (m + 1) * m;
  st.Qc = p; p += S1 * m;
  st.Qs = p; p += S1 * m;
  st.res = p; p += S1 * (m + 1);
  st.h1 = p; p += S1 * (m + 1);
  st.h2 = p; p += S1 * (m + 1);
  st.nrm2 = p; p += S1;
  st.scale = p; p += S1;
  st.rhs_norm = p; p += S1;
  st.rn = p; p += S1;
  st.rtol = p; p += S1;
  st.rn0prev = p; p += S1;
  p += S1;
  int *q = k->d_si;
  st.active = q; q += S1;
  st.converged = q; q += S1;
  st.done = q; q += S1;
  st.err = q; q += S1;
  st.niters = q; q += S1;
  st.iters = q; q += S1;
  st.first = q; q += 1;
  st.it = q; q += 1;
  st.nactive = q; q += 1;
  st.stall = q; q += 1;
  // graphs (a mixed solve's FP64 passes read the FP64 factor, which must
  // have its buffers before they are captured)
  if (!rc && k->mixed && k->pc) rc = pc_prepare_fp64(k->pc);
  if (!rc)
    rc = capture(&k->g_start, [&](cudaStream_t cs) { enqueue_start(k, cs); });
  if (!rc)
    rc = capture(&k->g_end, [&](cudaStream_t cs) { enqueue_end(k, cs); });
  for (int mode = 0; mode < (k->mixed ? 2 : 1) && !rc; mode++)
    rc = capture(&k->g_iter[mode],
                 [&](cudaStream_t cs) { enqueue_iter(k, mode, cs); },
                 &k->step_nodes[mode]);
  for (int mode = 0; mode < (k->mixed ? 2 : 1) && !rc; mode++)
    rc = capture_cycle(k, mode, &k->g_cycle[mode]);
  if (rc) k->free_layout();
  return rc;
}

// Set every per-system rtol to v (host -> device)
int set_rtols(tg_ksm *k, const std::vector<double> &v, cudaStream_t s) {
  TG_CUDA(cudaMemcpyAsync(k->st.rtol, v.data(), v.size() * sizeof(double),
                          cudaMemcpyHostToDevice, s));
  return 0;
}

// Restarted GMRES on d_B -> d_X (state reset except done[]).
int run_cycles(tg_ksm *k, int mode, int stall, cudaStream_t s,
               int max_cycles = 0) {
  const size_t S1 = (size_t)k->nsys;
  KrylovState &st = k->st;
  TG_CUDA(cudaMemsetAsync(st.converged, 0, S1 * sizeof(int), s));
  TG_CUDA(cudaMemsetAsync(st.err, 0, S1 * sizeof(int), s));
  TG_CUDA(cudaMemsetAsync(st.iters, 0, S1 * sizeof(int), s));
  const int one = 1;
  TG_CUDA(cudaMemcpyAsync(st.first, &one, sizeof(int), cudaMemcpyHostToDevice,
                          s));
  TG_CUDA(cudaMemcpyAsync(st.stall, &stall, sizeof(int),
                          cudaMemcpyHostToDevice, s));
  volatile int *hp = k->h_pinned;
  const int ncyc = max_cycles > 0 ? std::min(max_cycles, k->nrestart + 1)
                                  : k->nrestart + 1;
  for (int cycle = 0; cycle < ncyc; cycle++) {
    if (k->g_cycle[mode]) {
      // the whole cycle on the device; one read of the active count
      TG_CUDA(cudaGraphLaunch(k->g_cycle[mode], s));
      TG_CUDA(cudaMemcpyAsync(k->h_pinned, st.nactive, sizeof(int),
                              cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaStreamSynchronize(s));
      if (hp[0] == 0) break;
      continue;
    }
    TG_CUDA(cudaGraphLaunch(k->g_start, s));
    TG_CUDA(cudaMemcpyAsync(k->h_pinned, st.nactive, sizeof(int),
                            cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    if (hp[0] == 0) break;
    int done_iters = 0;
    while (done_iters < k->m) {
      const int nb = std::min(kCheckEvery, k->m - done_iters);
      for (int i = 0; i < nb; i++) TG_CUDA(cudaGraphLaunch(k->g_iter[mode], s));
      done_iters += nb;
      TG_CUDA(cudaMemcpyAsync(k->h_pinned, st.nactive, sizeof(int),
                              cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaStreamSynchronize(s));
      if (hp[0] == 0) break;
    }
    TG_CUDA(cudaGraphLaunch(k->g_end, s));
    if (hp[0] == 0) break;  // every system converged (or failed) this cycle
  }
  TG_CUDA(cudaStreamSynchronize(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}

// per-system 2-norms of a multivector (host result)
int seg_norms(tg_ksm *k, const double *x, std::vector<double> &out,
              cudaStream_t s) {
  launch_kr_dots(x, k->N, nullptr, 1, 1, x, k->ch, k->d_partials, k->st.nrm2,
                 1, s);
  out.assign(k->nsys, 0.0);
  TG_CUDA(cudaMemcpyAsync(out.data(), k->st.nrm2, k->nsys * sizeof(double),
                          cudaMemcpyDeviceToHost, s));
  TG_CUDA(cudaStreamSynchronize(s));
  for (auto &v : out) v = std::sqrt(v);
  return 0;
}

template <typename T>
int fetch(std::vector<T> &h, const T *d, size_t n, cudaStream_t s) {
  h.resize(n);
  TG_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost,
                          s));
  TG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

// Restarted GMRES inside iterative refinement on the FP64 true residual.
//
// Mode 0 (FP64 operator): the first pass is the reference's GMRES on
// r0 = b - A x0 with its own tolerance (estimated residual below
// rtol ||r0||); a system reports converged when that pass converged, as in
// the reference, or when its true residual meets rtol ||r0||.  Up to two
// more passes then refine the solution against the true residual when it is
// above rtol ||r0|| (the estimate and the true residual drift apart on
// ill-conditioned shells), stopping when a pass no longer halves it.
// Mode 1 (mixed precision): every pass runs the FP32 preconditioner and
// mat-vec with FP64 Arnoldi to a modest relative tolerance, and a system has
// converged when its FP64 true residual meets rtol ||r0||.  Each pass
// contracts the true residual by about cond(A) x the FP32 rounding of A
// (and by the FP32 factor's own accuracy); when a pass gains less than 1e4x
// for some system, the remaining passes run the all-FP64 solve (an FP64
// factor of the same matrix, made then, and the FP64 mat-vec) to the full
// tolerance, and a system stops when a pass no longer halves its residual.
// A system whose FP64 passes stop there with a true residual at or below
// eps (|A| |x| + |b|), the accuracy FP64 arithmetic can attain, has
// converged (where rtol |r0| lies below that floor no solver meets it).
int solve_refined(tg_ksm *k, int mode, const double *B, double *X,
                  int zero_guess, int *iters, int *flags, double *resn,
                  cudaStream_t s) {
  const size_t N = k->N;
  const int ns = k->nsys;
  tg_mat *A = k->A;
  TG_CUDA(cudaMemcpyAsync(k->d_Bo, B, N * sizeof(double),
                          cudaMemcpyDeviceToDevice, s));
  if (zero_guess) TG_CUDA(cudaMemsetAsync(k->d_Xo, 0, N * sizeof(double), s));
  else
    TG_CUDA(cudaMemcpyAsync(k->d_Xo, X, N * sizeof(double),
                            cudaMemcpyDeviceToDevice, s));
  std::vector<double> r0, rn, prev(ns, 0.0), rt(ns), mask(ns);
  std::vector<int> conv(ns, 0), done(ns, 0), it_total(ns, 0), it, pconv;
  std::vector<int> fresh(ns, 0);  // mixed: system restarted from zero in FP64
  std::vector<int> stuck(ns, 0);  // mixed: FP64 continuation did not converge
  int rc;
  const int max_outer = mode == 0 ? 2 : 30;
  const int mode_in = mode;
  // TG_KSM_TRACE=1 prints each refinement pass's relative true residuals
  const bool trace = std::getenv("TG_KSM_TRACE") != nullptr;
  // Mixed precision: the accuracy an FP64 iterate can attain is about
  // eps (|A| |x| + |b|) per system (normwise backward error at the unit
  // roundoff), with |A| the 2-norm of the row 1-norms (not below the
  // Frobenius or spectral norm).  A system whose FP64 passes stagnate at or
  // below it has converged as far as FP64 arithmetic allows, even where
  // rtol |r0| lies below that floor (thin shells: cond(A) ~ 1e12).
  std::vector<double> anorm, bnorm, xnorm, floor_(ns, 0.0);
  if (mode_in == 1) {
    launch_bcsr_row_abs_sum(A->bsize, A->nrows, A->a->d_rowp, A->d_vals,
                            k->d_X, s);
    for (int l = 1; l < k->nrhs; l++)
      TG_CUDA(cudaMemcpyAsync(k->d_X + (size_t)l * k->n, k->d_X,
                              k->n * sizeof(double), cudaMemcpyDeviceToDevice,
                              s));
    if ((rc = seg_norms(k, k->d_X, anorm, s))) return rc;
    if ((rc = seg_norms(k, k->d_Bo, bnorm, s))) return rc;
  }
  for (int outer = 0; outer <= max_outer; outer++) {
    launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols,
                     A->d_vals, k->d_Xo, k->d_B, s, k->nrhs, k->n);
    launch_kr_residual(k->d_Bo, k->d_B, N, s);
    if ((rc = seg_norms(k, k->d_B, rn, s))) return rc;
    if (outer == 0) r0 = rn;
    int left = 0;
    bool to_fp64 = false, restart_any = false;
    // a correction that made a system's true residual larger is taken back
    if (outer > 0) {
      bool any = false;
      for (int i = 0; i < ns; i++) {
        mask[i] = (!done[i] && std::isfinite(rn[i]) && rn[i] > prev[i])
                      ? 1.0 : 0.0;
        any |= mask[i] != 0.0;
      }
      if (any) {
        TG_CUDA(cudaMemcpyAsync(k->st.scale, mask.data(), ns * sizeof(double),
                                cudaMemcpyHostToDevice, s));
        launch_kr_mask(k->d_X, k->ch, k->st.scale, s);
        launch_axpy(-1.0, k->d_X, k->d_Xo, N, s);
        // the residual of the restored iterate drives the next pass
        launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols,
                         A->d_vals, k->d_Xo, k->d_B, s, k->nrhs, k->n);
        launch_kr_residual(k->d_Bo, k->d_B, N, s);
        for (int i = 0; i < ns; i++)
          if (mask[i] != 0.0) {
            rn[i] = prev[i];
            if (mode == 1) to_fp64 = true;
            else if (mode_in == 1 && !fresh[i]) stuck[i] = 1;
            else done[i] = 1;
          }
      }
    }
    if (mode_in == 1) {
      if ((rc = seg_norms(k, k->d_Xo, xnorm, s))) return rc;
      for (int i = 0; i < ns; i++)
        floor_[i] = 0x1p-53 * (anorm[i] * xnorm[i] + bnorm[i]);
    }
    for (int i = 0; i < ns; i++) {
      if (!std::isfinite(rn[i]))
        return fail(TG_ERR_NONFINITE, "GMRES: non-finite true residual");
      if (done[i]) {
        // a system stopped (taken back) at the FP64 accuracy floor
        if (mode_in == 1 && !conv[i] && rn[i] <= floor_[i]) conv[i] = 1;
        continue;
      }
      const bool met = rn[i] <= k->rtol * r0[i] || rn[i] < k->atol;
      if (met) {
        done[i] = 1;
        conv[i] = 1;
      } else if (mode == 1 && outer > 0 && rn[i] >= 1e-4 * prev[i]) {
        // a pass solved to 1e-6 with the FP32 mat-vec gained less than
        // 1e4x: cond(A) x FP32 rounding is not small for this system, so
        // the remaining passes keep the FP32 preconditioner but apply A in
        // FP64
        to_fp64 = true;
      } else if (stuck[i] || (outer > 0 && rn[i] > 0.5 * prev[i])) {
        if (mode_in == 1 && mode == 0 && rn[i] <= floor_[i]) {
          // the FP64 passes stagnated at the attainable accuracy
          done[i] = 1;
          conv[i] = 1;
        } else if (mode_in == 1 && mode == 0 && !fresh[i]) {
          // the FP64 passes stalled from the mixed-precision iterate (its
          // residual is left in the hardest modes, where restarted GMRES
          // stagnates): solve this system again from zero, all in FP64
          fresh[i] = 1;
          restart_any = true;
        } else {
          done[i] = 1;  // stagnated
        }
      } else if (outer == max_outer) {
        done[i] = 1;
        if (mode_in == 1 && mode == 0 && rn[i] <= floor_[i]) conv[i] = 1;
      }
    }
    if (to_fp64) {
      mode = 0;
      if ((rc = pc_factor_fp64(k->pc, s))) return rc;
    }
    if (restart_any) {
      std::vector<double> keep(ns);
      for (int i = 0; i < ns; i++) {
        const bool reset =
            fresh[i] && (stuck[i] || rn[i] > 0.5 * prev[i]) && !done[i];
        stuck[i] = 0;
        keep[i] = reset ? 0.0 : 1.0;
        if (reset) {
          rn[i] = r0[i];
          prev[i] = 2.0 * r0[i];  // the fresh solve's first pass always runs
        }
      }
      TG_CUDA(cudaMemcpyAsync(k->st.scale, keep.data(), ns * sizeof(double),
                              cudaMemcpyHostToDevice, s));
      launch_kr_mask(k->d_Xo, k->ch, k->st.scale, s);
      // the residual of a reset system is its right-hand side again
      launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols,
                       A->d_vals, k->d_Xo, k->d_B, s, k->nrhs, k->n);
      launch_kr_residual(k->d_Bo, k->d_B, N, s);
    }
    if (trace) {
      std::fprintf(stderr, "[tg_ksm] pass %d mode %d:", outer, mode);
      for (int i = 0; i < ns; i++)
        std::fprintf(stderr, " %d:%.3e%s", i, rn[i] / r0[i],
                     done[i] ? (conv[i] ? "c" : "x") : "");
      std::fprintf(stderr, "\n");
    }
    for (int i = 0; i < ns; i++) {
      if (!done[i]) {
        left++;
        prev[i] = rn[i];
        if (mode_in == 0 && outer == 0)
          rt[i] = k->rtol;
        else if (mode == 0)
          rt[i] = std::max(1e-14, 0.5 * k->rtol * r0[i] / rn[i]);
        else
          rt[i] = std::max(1e-6, 0.1 * k->rtol * r0[i] / rn[i]);
      } else {
        rt[i] = 1.0;
      }
      mask[i] = done[i] ? 0.0 : 1.0;
    }
    if (resn)
      for (int i = 0; i < ns; i++) resn[i] = rn[i];
    if (!left) break;
    // finished systems get a zero right-hand side and stay inactive
    TG_CUDA(cudaMemcpyAsync(k->st.scale, mask.data(), ns * sizeof(double),
                            cudaMemcpyHostToDevice, s));
    launch_kr_mask(k->d_B, k->ch, k->st.scale, s);
    TG_CUDA(cudaMemcpyAsync(k->st.done, done.data(), ns * sizeof(int),
                            cudaMemcpyHostToDevice, s));
    if ((rc = set_rtols(k, rt, s))) return rc;
    TG_CUDA(cudaMemsetAsync(k->d_X, 0, N * sizeof(double), s));
    // passes with the FP64 mat-vec restart until their cycle limit (the
    // first one is the reference's GMRES); passes with the FP32 mat-vec stop
    // a system whose restarts stall at the FP32 accuracy floor
    // a mixed solve's FP64 pass that continues from the FP32 iterate and
    // does not converge within its cycle limit (restarted GMRES can stall on
    // the hard modes such a residual is left in) restarts that system from
    // zero in FP64
    const bool continuing = mode_in == 1 && mode == 0;
    if ((rc = run_cycles(k, mode, mode == 1, s))) return rc;
    if (continuing) {
      std::vector<int> ic;
      if ((rc = fetch(ic, k->st.converged, ns, s))) return rc;
      for (int i = 0; i < ns; i++)
        if (!done[i] && !fresh[i] && !ic[i]) stuck[i] = 1;
    }
    if ((rc = fetch(it, k->st.iters, ns, s))) return rc;
    std::vector<int> err;
    if ((rc = fetch(err, k->st.err, ns, s))) return rc;
    for (int i = 0; i < ns; i++) {
      if (err[i])
        return fail(TG_ERR_NONFINITE, "GMRES: non-finite residual estimate");
      it_total[i] += it[i];
    }
    if (mode_in == 0 && outer == 0) {
      if ((rc = fetch(pconv, k->st.converged, ns, s))) return rc;
      for (int i = 0; i < ns; i++) conv[i] = done[i] ? conv[i] : pconv[i];
    }
    launch_kr_axpy(k->d_X, k->d_Xo, N, s);
  }
  TG_CUDA(cudaMemcpyAsync(X, k->d_Xo, N * sizeof(double),
                          cudaMemcpyDeviceToDevice, s));
  TG_CUDA(cudaStreamSynchronize(s));
  int all = 1;
  for (int i = 0; i < ns; i++) {
    if (iters) iters[i] = it_total[i];
    if (flags) flags[i] = conv[i];
    all &= conv[i];
  }
  return all;
}

}  // namespace

extern "C" {

int tg_ksm_get_graph_info(tg_ksm *k, int *cycle_graph, int *step_nodes,
                          int *step_nodes_fp32) {
  if (!k) return fail(TG_ERR_ARG, "tg_ksm_get_graph_info: NULL");
  if (cycle_graph) *cycle_graph = k->g_cycle[0] ? 1 : 0;
  if (step_nodes) *step_nodes = k->step_nodes[0];
  if (step_nodes_fp32) *step_nodes_fp32 = k->step_nodes[1];
  return 0;
}

int tg_ksm_create(tg_mat *A, tg_pc *pc, int m, int nrestart, int mixed,
                  tg_ksm **out) {
  if (!A || !out || m <= 0 || nrestart < 0)
    return fail(TG_ERR_ARG, "tg_ksm_create: bad arguments");
  if (mixed && (!pc || pc->precision != TG_PREC_FP32))
    return fail(TG_ERR_ARG, "tg_ksm_create: mixed precision needs a FP32 pc");
  tg_ksm *k = new tg_ksm();
  k->A = A;
  A->refcount++;
  k->pc = pc;
  if (pc) pc->refcount++;
  k->m = m;
  k->nrestart = nrestart;
  k->mixed = mixed;
  k->n = (size_t)A->nrows * A->bsize;
  k->seg_rows = {0, A->nrows};
  // an FP32 preconditioner is applied with FP32 rounding that differs
  // between the Arnoldi vectors and their combination, so its solves keep
  // every preconditioned vector (flexible GMRES) and update x from those
  k->flexible = pc && pc->precision == TG_PREC_FP32;
  *out = k;
  return 0;
}
int tg_ksm_decref(tg_ksm *k) {
  if (!k) return 0;
  if (--k->refcount == 0) {
    tg_pc_decref(k->pc);
    tg_mat_decref(k->A);
    delete k;
  }
  return 0;
}
int tg_ksm_set_tolerances(tg_ksm *k, double rtol, double atol) {
  if (!k) return fail(TG_ERR_ARG, "NULL ksm");
  k->rtol = rtol;
  k->atol = atol;
  k->st.atol = atol;
  if (k->nrhs) k->free_layout();  // atol is captured in the graphs
  return 0;
}

int tg_ksm_set_segments(tg_ksm *k, int nseg, const int *row_ptr) {
  if (!k || nseg <= 0 || !row_ptr)
    return fail(TG_ERR_ARG, "tg_ksm_set_segments: bad arguments");
  tg_mat *A = k->A;
  if (row_ptr[0] != 0 || row_ptr[nseg] != A->nrows)
    return fail(TG_ERR_ARG, "tg_ksm_set_segments: row_ptr must span 0..rows");
  for (int g = 0; g < nseg; g++)
    if (row_ptr[g + 1] <= row_ptr[g])
      return fail(TG_ERR_ARG, "tg_ksm_set_segments: empty or unsorted range");
  // the matrix must not couple two ranges
  const std::vector<int> &rowp = A->a->rowp_h, &cols = A->a->cols_h;
  for (int g = 0; g < nseg; g++)
    for (int i = row_ptr[g]; i < row_ptr[g + 1]; i++)
      for (int j = rowp[i]; j < rowp[i + 1]; j++)
        if (cols[j] < row_ptr[g] || cols[j] >= row_ptr[g + 1])
          return fail(TG_ERR_ARG,
                      "tg_ksm_set_segments: the matrix couples two ranges");
  k->seg_rows.assign(row_ptr, row_ptr + nseg + 1);
  k->free_layout();
  return 0;
}

int tg_ksm_solve_multi(tg_ksm *k, int nrhs, const double *B, double *X,
                       int zero_guess, int *iters, int *flags,
                       double *resnorms, void *sv) {
  if (!k || !B || !X || nrhs <= 0)
    return fail(TG_ERR_ARG, "tg_ksm_solve_multi: bad arguments");
  if (k->pc && !k->pc->factored)
    return fail(TG_ERR_STATE, "tg_ksm_solve: the preconditioner is not factored");
  int rc = ensure_layout(k, nrhs);
  if (rc) return rc;
  return solve_refined(k, k->mixed ? 1 : 0, B, X, zero_guess, iters, flags,
                       resnorms, S(sv));
}

int tg_ksm_solve(tg_ksm *k, const double *b, double *x, int zero_guess,
                 int *iters, double *resnorm, void *sv) {
  if (!k || !b || !x) return fail(TG_ERR_ARG, "tg_ksm_solve: NULL argument");
  const int nseg = (int)k->seg_rows.size() - 1;
  std::vector<int> it(nseg), fl(nseg);
  std::vector<double> rn(nseg);
  int rc = tg_ksm_solve_multi(k, 1, b, x, zero_guess, it.data(), fl.data(),
                              rn.data(), sv);
  if (rc < 0) return rc;
  if (iters) *iters = *std::max_element(it.begin(), it.end());
  if (resnorm) *resnorm = *std::max_element(rn.begin(), rn.end());
  return rc;
}

}  // extern "C"
