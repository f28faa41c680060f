// CPU run of the direct factorisation's GPU kernels
// (tacs_gb300/csrc/direct_kernels.cuh): every CTA runs as one thread, in
// sequence, which computes what the GPU does because each kernel is
// written as phases of independent strided work separated by barriers.
// The launch sequence mirrors tg_direct_factor / tg_direct_solve
// (tacs_gb300/csrc/tg_direct.cu).  Built by tests/test_direct_symbolic.py
// with g++ and called through ctypes; test infrastructure only.
#define DK_EMULATE
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

struct EmuDim3 {
  unsigned x, y, z;
};
static EmuDim3 threadIdx{0, 0, 0}, blockIdx{0, 0, 0}, blockDim{1, 1, 1},
    gridDim{1, 1, 1};
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static
#define __launch_bounds__(...)
#define __syncthreads() ((void)0)
#define __syncwarp() ((void)0)
static std::vector<double> g_dyn;
static double *dk_dyn_smem() { return g_dyn.data(); }
static inline int atomicCAS(int *a, int cmp, int val) {
  const int old = *a;
  if (old == cmp) *a = val;
  return old;
}
namespace tg {
namespace dk {
namespace {
template <class T>
inline bool dk_isfinite(T x) { return std::isfinite(x); }
template <class T>
inline T dk_sqrt(T x) { return std::sqrt(x); }
}  // namespace
}  // namespace dk
}  // namespace tg

#include "direct_kernels.cuh"
#include "direct_symbolic.h"

using namespace tg::dk;

template <class K, class... Args>
static void launch(K kernel, unsigned gx, unsigned gy, size_t smem_doubles,
                   Args... args) {
  g_dyn.assign(smem_doubles + 1, 0.0);
  gridDim = {gx, gy, 1};
  for (unsigned y = 0; y < gy; y++)
    for (unsigned x = 0; x < gx; x++) {
      blockIdx = {x, y, 0};
      kernel(args...);
    }
}

static void set_store(tg::DirectView &v, double *l, double *p) {
  v.lstore = l;
  v.pool = p;
}
static void set_dinv(tg::DirectView &v, double *p) {
  v.dinv = p;
  v.dinv32 = nullptr;
}
static void set_dinv(tg::DirectView &v, float *p) {
  v.dinv = nullptr;
  v.dinv32 = p;
}
static void set_store(tg::DirectView &v, float *l, float *p) {
  v.lstore32 = l;
  v.pool32 = p;
}

// the solve passes of tg_direct.cu's solve_levels for NR right-hand sides
template <class T, int NR>
static void de_solve_pass(const tg::DirectView &v,
                          const tg::direct::Analysis &an, int max_front,
                          T *ypos, T *xpos, T *contrib) {
  const int nl = (int)an.level_ptr.size() - 1;
  // in doubles: the GPU's entries of T rounded up
  const size_t smem =
      ((size_t)max_front * NR + tg::direct_plain_extra(NR, (int)sizeof(T))) *
          sizeof(T) / sizeof(double) + 1;
  for (int L = 0; L < nl; L++) {
    const int lb = an.level_ptr[L], le = an.level_ptr[L + 1];
    launch(direct_forward_kernel<T, NR>, le - lb, 1, smem, v,
           (const int *)an.level_sn.data() + lb, le - lb, ypos, contrib);
  }
  for (int L = nl - 1; L >= 0; L--) {
    const int lb = an.level_ptr[L], le = an.level_ptr[L + 1];
    launch(direct_backward_kernel<T, NR>, le - lb, 1, smem, v,
           (const int *)an.level_sn.data() + lb, le - lb, (const T *)ypos,
           xpos);
  }
}

// X = A^-1 B for the assembled BCSR matrix A with row boundary conditions
// (bcmask per node) and nrhs right-hand sides back to back, by the GPU
// kernels run on the CPU in T (double: the FP64 factorisation; float: the
// FP32 one, b and x converted), in passes of 4, 2 and 1 right-hand sides
// as on the GPU.  small_max: fronts of at most this many scalar rows take
// the one-CTA kernel, larger ones the panel path.  Returns 0, or the
// failing supernode + 1.
template <class T>
static int de_solve_t(int n, int bs, const int *rowp, const int *cols,
                      const double *vals, const int *bcmask_in,
                      const double *xyz, int small_max, int nrhs,
                      const double *b_in, double *x_out) {
  std::vector<int> rp(rowp, rowp + n + 1), cs(cols, cols + rowp[n]);
  std::vector<int> perm = tg::direct::nested_dissection(rp, cs, 64, xyz);
  tg::direct::Analysis an = tg::direct::analyse(rp, cs, perm);
  const int ns = (int)an.sn_col.size() - 1;
  const size_t b2 = (size_t)bs * bs, N = (size_t)n * bs;
  std::vector<int> fm(ns), fc(ns), ch_ptr(ns + 1, 0), ch_list(ns + 1);
  std::vector<int64_t> v_off(ns, 0);
  int64_t vacc = 0;
  int max_front = 0;
  for (int s = 0; s < ns; s++) {
    fm[s] = (an.sn_rowptr[s + 1] - an.sn_rowptr[s]) * bs;
    fc[s] = (an.sn_col[s + 1] - an.sn_col[s]) * bs;
    max_front = std::max(max_front, fm[s]);
    v_off[s] = vacc;
    vacc += fm[s] - fc[s];
    if (an.sn_parent[s] >= 0) ch_ptr[an.sn_parent[s] + 1]++;
  }
  for (int s = 0; s < ns; s++) ch_ptr[s + 1] += ch_ptr[s];
  {
    std::vector<int> fill(ch_ptr.begin(), ch_ptr.end() - 1);
    for (int s = 0; s < ns; s++)
      if (an.sn_parent[s] >= 0) ch_list[fill[an.sn_parent[s]]++] = s;
  }
  std::vector<int> bcmask(bcmask_in, bcmask_in + n);
  const tg::direct::BcCoupling bcc =
      tg::direct::bc_coupling(rp, cs, bcmask, an.iperm);
  // sized exactly as tg_direct.cu allocates them, so that a sanitizer
  // build sees any access the GPU would make out of bounds
  const int max_nr = nrhs >= 4 ? 4 : nrhs >= 2 ? 2 : 1;
  std::vector<T> lstore((size_t)an.l_total * b2),
      pool((size_t)an.u_peak * b2), contrib(vacc * max_nr),
      ypos(N * max_nr), xpos(N * max_nr), bt(b_in, b_in + N * nrhs), xt(N * nrhs), vt(vals, vals + rowp[n] * b2);
  const T *b = bt.data();
  T *x = xt.data();
  int failflag = 0;
  tg::DirectView v;
  v.bs = bs;
  v.perm = an.perm.data();
  v.bcmask = bcmask.data();
  v.sn_col = an.sn_col.data();
  v.sn_rowptr = an.sn_rowptr.data();
  v.sn_rows = an.sn_rows.data();
  v.sn_parent = an.sn_parent.data();
  v.ea_ptr = an.ea_ptr.data();
  v.ea_rel = an.ea_rel.data();
  v.asm_ptr = an.asm_ptr.data();
  v.asm_blk = an.asm_blk.data();
  v.asm_row = an.asm_row.data();
  v.asm_col = an.asm_col.data();
  v.ch_ptr = ch_ptr.data();
  v.ch_list = ch_list.data();
  v.l_off = an.l_off.data();
  v.u_off = an.u_off.data();
  v.v_off = v_off.data();
  v.lstore = v.pool = nullptr;
  v.lstore32 = v.pool32 = nullptr;
  // the fronts factored by panels keep the inverses of their diagonal
  // blocks, as in tg_direct.cu
  std::vector<int64_t> dinv_off(ns, -1);
  std::vector<int> inv_sn, inv_k0;
  int64_t dinv_len = 0;
  for (int sn = 0; sn < ns; sn++) {
    if (fm[sn] <= small_max) continue;
    dinv_off[sn] = dinv_len;
    for (int k0 = 0; k0 < fc[sn]; k0 += tg::kDirectPanel) {
      inv_sn.push_back(sn);
      inv_k0.push_back(k0);
      dinv_len += (int64_t)tg::kDirectPanel * tg::kDirectPanel;
    }
  }
  std::vector<T> dinv(dinv_len > 0 ? (size_t)dinv_len : 1);
  v.dinv_off = dinv_off.data();
  set_dinv(v, dinv.data());
  set_store(v, lstore.data(), pool.data());

  // factor: the sequence of tg_direct_factor (small fronts of a level in
  // one launch, large ones in panel steps batched over the level)
  std::vector<int> small_h, small_ptr(1, 0);
  for (size_t L = 0; L + 1 < an.level_ptr.size(); L++) {
    for (int t = an.level_ptr[L]; t < an.level_ptr[L + 1]; t++) {
      const int sn = an.level_sn[t];
      if (fm[sn] <= small_max) small_h.push_back(sn);
    }
    small_ptr.push_back((int)small_h.size());
  }
  // the trailing tile of tg_direct.cu: 64 for the FP32 factorisation
  const int tile = sizeof(T) == sizeof(float) ? tg::kDirectTile32
                                              : tg::kDirectTile;
  const tg::direct::PanelSteps ps = tg::direct::panel_steps(
      an, bs, small_max, tg::kDirectPanel, tile, tg::kDirectTrsmRows);
  size_t step = 0;
  for (size_t L = 0; L + 1 < an.level_ptr.size(); L++) {
    const int lb = an.level_ptr[L], le = an.level_ptr[L + 1];
    const int *lv = an.level_sn.data() + lb;
    const int cnt = le - lb;
    int64_t zmax = 0;  // the zeroing chunks of tg_direct.cu
    for (int t = 0; t < cnt; t++) {
      const int64_t M = fm[lv[t]], Cc = fc[lv[t]];
      zmax = std::max(zmax, M * Cc + (M - Cc) * (M - Cc));
    }
    launch(direct_zero_kernel<T>, cnt,
           (unsigned)((zmax + tg::kDirectZeroChunk - 1) / tg::kDirectZeroChunk),
           0, v, lv, cnt);
    launch(direct_assemble_kernel<T>, cnt, 1, 0, v, lv, cnt, vals);
    int nch = 0, um = 0;  // the extend-add launches of tg_direct.cu
    for (int t = 0; t < cnt; t++) {
      const int sn = lv[t];
      nch = std::max(nch, ch_ptr[sn + 1] - ch_ptr[sn]);
      for (int k = ch_ptr[sn]; k < ch_ptr[sn + 1]; k++)
        um = std::max(um, fm[ch_list[k]] - fc[ch_list[k]]);
    }
    const int ych = (um + tg::kDirectExtendRows - 1) / tg::kDirectExtendRows;
    if (ych > 0)
      for (int k = 0; k < nch; k++)
        launch(direct_extend_add_kernel<T>, cnt, ych, 0, v, lv, cnt, k);
    const int sb = small_ptr[L], se = small_ptr[L + 1];
    if (se > sb)
      launch(direct_factor_small_kernel<T>, se - sb, 1, 0, v,
             (const int *)small_h.data() + sb, se - sb, &failflag);
    for (; step < ps.level.size() && ps.level[step] == (int)L; step++) {
      const int *fr = ps.fronts.data() + ps.front_off[step];
      const int *tp = ps.tprefix.data() + ps.tile_off[step];
      const int *rp = ps.rprefix.data() + ps.tile_off[step];
      launch(direct_panel_kernel<T>, ps.count[step], 1, 0, v, fr,
             ps.count[step], ps.k0[step], &failflag);
      if (ps.rtotal[step] > 0)
        launch(direct_trsm_kernel<T>, ps.rtotal[step], 1,
               (size_t)tg::kDirectTrsmRows * (tg::kDirectPanel + 1), v, fr,
               rp, ps.count[step], ps.k0[step]);
      if (ps.total[step] > 0) {
        if (tile == 64)
          launch(direct_trailing_kernel<T, 64>, ps.total[step], 1, 0, v, fr,
                 tp, ps.count[step], ps.k0[step]);
        else
          launch(direct_trailing_kernel<T, 32>, ps.total[step], 1, 0, v, fr,
                 tp, ps.count[step], ps.k0[step]);
      }
    }
  }
  if (failflag) return failflag;
  // the inverses of the diagonal blocks, after the factorisation
  if (!inv_sn.empty())
    launch(direct_inverse_kernel<T>, (unsigned)inv_sn.size(), 1, 0, v,
           (const int *)inv_sn.data(), (const int *)inv_k0.data(),
           (int)inv_sn.size());

  // solve: the sequence of tg_direct_solve (on the GPU fronts of more than
  // kDirectClusterFront rows take the cluster kernels, one thread-block
  // cluster per front, checked by the GPU tests; here every front takes the
  // one-CTA kernels, which form each row's sums in the same order)
  for (int r0 = 0; r0 < nrhs;) {
    const int left = nrhs - r0;
    const int nr = left >= 4 ? 4 : left >= 2 ? 2 : 1;
    const T *bb = b + (size_t)r0 * N;
    launch(direct_rhs_kernel<T>, 1, 1, 0, n, bs, (const int *)an.perm.data(),
           bb, ypos.data(), nr, N);
    if (!bcc.row.empty())
      launch(direct_bc_couple_kernel<T>, 1, 1, 0, (int)bcc.row.size(), bs,
             (const int *)bcc.row.data(), (const int *)bcc.pos.data(),
             (const int *)bcc.ptr.data(), (const int *)bcc.blk.data(),
             (const int *)cols, (const int *)bcmask.data(),
             (const T *)vt.data(), bb, ypos.data(), nr, N);
    if (nr == 4)
      de_solve_pass<T, 4>(v, an, max_front, ypos.data(), xpos.data(),
                          contrib.data());
    else if (nr == 2)
      de_solve_pass<T, 2>(v, an, max_front, ypos.data(), xpos.data(),
                          contrib.data());
    else
      de_solve_pass<T, 1>(v, an, max_front, ypos.data(), xpos.data(),
                          contrib.data());
    launch(direct_unpermute_kernel<T>, 1, 1, 0, n, bs,
           (const int *)an.perm.data(), (const T *)xpos.data(),
           x + (size_t)r0 * N, nr, N);
    r0 += nr;
  }
  for (size_t k = 0; k < N * nrhs; k++) x_out[k] = (double)x[k];
  return 0;
}

extern "C" {

// precision: 0 FP64, 1 FP32
int de_solve(int n, int bs, const int *rowp, const int *cols,
             const double *vals, const int *bcmask, const double *xyz,
             int small_max, int precision, const double *b, double *x) {
  if (precision == 1)
    return de_solve_t<float>(n, bs, rowp, cols, vals, bcmask, xyz, small_max,
                             1, b, x);
  return de_solve_t<double>(n, bs, rowp, cols, vals, bcmask, xyz, small_max,
                            1, b, x);
}

// nrhs right-hand sides back to back
int de_solve_multi(int n, int bs, const int *rowp, const int *cols,
                   const double *vals, const int *bcmask, const double *xyz,
                   int small_max, int precision, int nrhs, const double *b,
                   double *x) {
  if (precision == 1)
    return de_solve_t<float>(n, bs, rowp, cols, vals, bcmask, xyz, small_max,
                             nrhs, b, x);
  return de_solve_t<double>(n, bs, rowp, cols, vals, bcmask, xyz, small_max,
                            nrhs, b, x);
}

}  // extern "C"

#ifdef DE_MAIN
// Stand-alone driver for a sanitizer build (-fsanitize=address,undefined):
// reads one system written by tests/test_direct_symbolic.py, solves it in
// FP64 and FP32, and prints the two solutions' max |K x - b|.
#include <cstdio>
#include <cstdlib>
static bool read_all(FILE *f, void *p, size_t bytes) {
  return bytes == 0 || fread(p, 1, bytes, f) == bytes;
}
int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[4];  // n, bs, nnz, has_xyz
  if (!read_all(f, hdr, sizeof hdr)) return 2;
  const int n = hdr[0], bs = hdr[1], nnz = hdr[2];
  const size_t N = (size_t)n * bs;
  std::vector<int> rowp(n + 1), cols(nnz), mask(n);
  std::vector<double> vals((size_t)nnz * bs * bs), xyz(3 * (size_t)n), b(N),
      x(N);
  bool ok = read_all(f, rowp.data(), sizeof(int) * rowp.size()) &&
            read_all(f, cols.data(), sizeof(int) * cols.size()) &&
            read_all(f, vals.data(), sizeof(double) * vals.size()) &&
            read_all(f, mask.data(), sizeof(int) * mask.size()) &&
            read_all(f, b.data(), sizeof(double) * N);
  if (ok && hdr[3]) ok = read_all(f, xyz.data(), sizeof(double) * xyz.size());
  fclose(f);
  if (!ok) return 2;
  const int small_max = atoi(argv[2]);
  for (int prec = 0; prec < 2; prec++) {
    const int rc = de_solve(n, bs, rowp.data(), cols.data(), vals.data(),
                            mask.data(), hdr[3] ? xyz.data() : nullptr,
                            small_max, prec, b.data(), x.data());
    if (rc) {
      printf("fail %d\n", rc);
      return 1;
    }
    double res = 0.0;
    for (int i = 0; i < n; i++)
      for (int r = 0; r < bs; r++) {
        double acc = -b[(size_t)i * bs + r];
        for (int j = rowp[i]; j < rowp[i + 1]; j++)
          for (int q = 0; q < bs; q++)
            acc += vals[(size_t)j * bs * bs + r * bs + q] *
                   x[(size_t)cols[j] * bs + q];
        res = std::max(res, std::fabs(acc));
      }
    printf("%d %.6e\n", prec, res);
  }
  return 0;
}
#endif
