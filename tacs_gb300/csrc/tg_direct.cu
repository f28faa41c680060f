// Direct (complete) factorisation of an assembled matrix: the host analysis
// of direct_symbolic.h (nested dissection by the node coordinates,
// supernodes, fronts, storage plan) and the level-by-level multifrontal
// block Cholesky of direct_kernels.cu, behind the C ABI tg_direct_*.
// Replaces the reference's complete factorisation (TACSSchurPc with a
// large levFill, src/bpmat/TACSSchurMat.cpp:1510-1600) with the same
// solution; the matrix's row boundary conditions are handled as
// x = Kt^-1 (b - K P b + P b), Kt being K with the boundary columns zeroed
// too (symmetric positive definite) and P keeping the boundary dofs; the
// correction K P b is formed on the block rows that have a block in a
// constrained column only (direct::bc_coupling).
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "direct_symbolic.h"
#include "tg_objects.h"

// fronts of at most this many scalar rows are factored by one CTA each,
// all fronts of a level in one launch; larger ones by 32-column panels,
// batched over the level's large fronts.
#ifndef TG_DIRECT_SMALL_FRONT
#define TG_DIRECT_SMALL_FRONT 64
#endif
static constexpr int kSmallFront = TG_DIRECT_SMALL_FRONT;
// trailing tile of the FP64 factorisation (32 or 64; the FP32 one uses 64)
#ifndef TG_DIRECT_TILE_F64
#define TG_DIRECT_TILE_F64 32
#endif
// blocks of the max-|x| reductions of the refinement's stopping test
static constexpr int kRedParts = 256;

struct tg_direct {
  int refcount = 1;
  tg_mat *A = nullptr;
  int n = 0, bs = 0, ns = 0, max_front = 0;
  // the largest front solved by one CTA and by one cluster, and the most
  // right-hand sides one solve pass takes (1, 2 or 4; the solve vectors
  // and refinement scratch hold that many)
  int plain_front = 0, cluster_front = 0, max_nr = 1;
  // fronts above cluster_threshold rows are solved by clusters (when the
  // device schedules them); tg_direct_autotune picks it
  bool clusters_ok = false;
  // the device also schedules kDirectSolveClusterWide-CTA clusters; per
  // level the cluster size of its cluster launches
  bool wide_ok = false;
  std::vector<int> csolve_ncl_h;
  int cluster_threshold = tg::kDirectClusterFront;
  long long layout_version = 0;  // build_solve_lists calls
  int precision = TG_PREC_FP64;
  tg::direct::Analysis an;
  std::vector<int> level_ptr_h, level_sn_h, front_m_h, front_c_h;
  // per level: its small fronts (one launch, d_small) and the panel steps
  // of its large ones (steps of level L: step_ptr_h[L] .. [L + 1])
  std::vector<int> small_ptr_h, step_ptr_h;
  // per level: the most children of one of its supernodes and the row
  // blocks of its largest child update matrix (the extend-add launches),
  // and the zeroing chunks of its largest front
  std::vector<int> ext_nch_h, ext_y_h, zero_y_h;
  int tile = tg::kDirectTile;  // trailing tile of the panel steps
  // the solves' fronts per level: one CTA each (d_solve_sn, solve_ptr_h)
  // and, above kDirectClusterFront rows, one thread-block cluster each
  // (d_csolve_sn, csolve_ptr_h)
  std::vector<int> solve_ptr_h, csolve_ptr_h;
  // per level: the largest front solved by one CTA (the launch's shared
  // memory and CTA size)
  std::vector<int> solve_front_h;
  int *d_solve_sn = nullptr, *d_csolve_sn = nullptr;
  std::vector<int> solve_sn_h, csolve_sn_h;
  // the backward solve's L21^T x2 tiles of the cluster fronts: per front
  // of csolve_sn_h the cumulative tiles and the offset of its chunk sums
  // within its level, per level the tiles; the chunk sums' buffer (entries
  // of the factor's precision, for max_nr right-hand sides)
  int *d_gemv_tp = nullptr;
  int64_t *d_gemv_poff = nullptr;
  std::vector<int> gemv_total_h;
  void *d_part = nullptr;
  size_t part_entries = 0;
  tg::direct::PanelSteps steps;
  int *d_small = nullptr, *d_step_fronts = nullptr, *d_step_tprefix = nullptr,
      *d_step_rprefix = nullptr;
  // device copies of the analysis
  int *d_perm = nullptr, *d_bcmask = nullptr, *d_sn_col = nullptr,
      *d_sn_rowptr = nullptr, *d_sn_rows = nullptr, *d_sn_parent = nullptr,
      *d_ea_ptr = nullptr, *d_ea_rel = nullptr, *d_asm_ptr = nullptr,
      *d_asm_blk = nullptr, *d_asm_row = nullptr, *d_asm_col = nullptr,
      *d_ch_ptr = nullptr, *d_ch_list = nullptr, *d_level_sn = nullptr;
  int64_t *d_l_off = nullptr, *d_u_off = nullptr, *d_v_off = nullptr,
          *d_dinv_off = nullptr;
  // inverses of the diagonal blocks of the fronts factored by panels, and
  // the (supernode, first column) list of those blocks
  int *d_inv_sn = nullptr, *d_inv_k0 = nullptr;
  int inv_count = 0;
  double *d_dinv = nullptr;
  float *d_dinv32 = nullptr;
  double *d_lstore = nullptr, *d_pool = nullptr, *d_contrib = nullptr;
  double *d_ypos = nullptr, *d_xpos = nullptr;
  // the right-hand side's coupling to the constrained dofs
  int *d_bc_row = nullptr, *d_bc_pos = nullptr, *d_bc_ptr = nullptr,
      *d_bc_blk = nullptr;
  int bc_nrow = 0;
  // FP32 factorisation: its storage, solve vectors and the matrix in FP32
  float *d_lstore32 = nullptr, *d_pool32 = nullptr, *d_contrib32 = nullptr;
  float *d_ypos32 = nullptr, *d_xpos32 = nullptr, *d_a32 = nullptr,
        *d_r32 = nullptr, *d_c32 = nullptr;
  double *d_r = nullptr, *d_t = nullptr;  // refinement residual, scratch
  // refinement stopping test: reduction partials, 3 device scalars, and
  // ||A||_inf of the values factored last
  double *d_red = nullptr, *d_scal = nullptr;
  double anorm = 0.0;
  int64_t contrib_len = 0;
  int *d_fail = nullptr;
  bool factored = false;
  // a level's one-CTA and cluster solves touch different fronts: the
  // cluster launch runs on side_stream beside the one-CTA launch (forked
  // and joined through the two events), so a level costs the longer of
  // the two rather than their sum.  The side stream has the device's
  // highest priority, so that a cluster's CTAs, which must find room on
  // one GPC together, are placed before the one-CTA fronts take the SMs.
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // the factorisation's launch sequence (every level's assembly, panel
  // steps and the inverses; fixed by the analysis) as one CUDA graph,
  // captured at the second factorisation and replayed after (the first
  // launches the kernels directly: a one-off factorisation gains nothing
  // from a graph, whose capture and instantiation come before its first
  // kernel runs)
  cudaGraphExec_t factor_exec = nullptr;
  int factor_calls = 0;
  tg::DirectBc bc() const {
    tg::DirectBc c;
    c.nrow = bc_nrow;
    c.row = d_bc_row;
    c.pos = d_bc_pos;
    c.ptr = d_bc_ptr;
    c.blk = d_bc_blk;
    c.cols = A->a->d_cols;
    c.bcmask = d_bcmask;
    return c;
  }
  tg::DirectView view() const {
    tg::DirectView v;
    v.bs = bs;
    v.perm = d_perm;
    v.bcmask = d_bcmask;
    v.sn_col = d_sn_col;
    v.sn_rowptr = d_sn_rowptr;
    v.sn_rows = d_sn_rows;
    v.sn_parent = d_sn_parent;
    v.ea_ptr = d_ea_ptr;
    v.ea_rel = d_ea_rel;
    v.asm_ptr = d_asm_ptr;
    v.asm_blk = d_asm_blk;
    v.asm_row = d_asm_row;
    v.asm_col = d_asm_col;
    v.ch_ptr = d_ch_ptr;
    v.ch_list = d_ch_list;
    v.l_off = d_l_off;
    v.u_off = d_u_off;
    v.v_off = d_v_off;
    v.lstore = d_lstore;
    v.pool = d_pool;
    v.lstore32 = d_lstore32;
    v.pool32 = d_pool32;
    v.dinv_off = d_dinv_off;
    v.dinv = d_dinv;
    v.dinv32 = d_dinv32;
    return v;
  }
  ~tg_direct() {
    using tg::dfree;
    dfree(d_perm); dfree(d_bcmask); dfree(d_sn_col); dfree(d_sn_rowptr);
    dfree(d_sn_rows); dfree(d_sn_parent); dfree(d_ea_ptr); dfree(d_ea_rel);
    dfree(d_asm_ptr); dfree(d_asm_blk); dfree(d_asm_row); dfree(d_asm_col);
    dfree(d_ch_ptr); dfree(d_ch_list); dfree(d_level_sn); dfree(d_l_off);
    dfree(d_solve_sn); dfree(d_csolve_sn); dfree(d_gemv_tp);
    dfree(d_gemv_poff);
    if (d_part) cudaFree(d_part);
    dfree(d_u_off); dfree(d_v_off); dfree(d_lstore); dfree(d_pool);
    dfree(d_contrib); dfree(d_ypos); dfree(d_xpos); dfree(d_bc_row);
    dfree(d_bc_pos); dfree(d_bc_ptr); dfree(d_bc_blk);
    dfree(d_fail); dfree(d_small); dfree(d_lstore32);
    dfree(d_step_fronts); dfree(d_step_tprefix); dfree(d_step_rprefix);
    dfree(d_pool32); dfree(d_contrib32); dfree(d_ypos32); dfree(d_xpos32);
    dfree(d_a32); dfree(d_r32);
    dfree(d_c32); dfree(d_r); dfree(d_t); dfree(d_red); dfree(d_scal);
    dfree(d_dinv_off); dfree(d_dinv); dfree(d_dinv32);
    dfree(d_inv_sn); dfree(d_inv_k0);
    if (factor_exec) cudaGraphExecDestroy(factor_exec);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side_stream) cudaStreamDestroy(side_stream);
  }
};

// the largest front the autotuner may leave to the one-CTA solves
static constexpr int kTuneMaxFront = 1536;

// The solves' per-level front lists for a cluster threshold: fronts of more
// than `threshold` rows take the cluster kernels (when the device schedules
// them), the others one CTA each; uploads the lists and sets the kernels'
// shared-memory attributes.
static int build_solve_lists(tg_direct *d, int threshold) {
  const tg::direct::Analysis &an = d->an;
  std::vector<int> a, b;
  d->solve_ptr_h.assign(1, 0);
  d->csolve_ptr_h.assign(1, 0);
  d->csolve_ncl_h.clear();
  d->solve_front_h.clear();
  d->plain_front = d->cluster_front = 0;
  for (size_t L = 0; L + 1 < an.level_ptr.size(); L++) {
    int pf = 0;
    for (int t = an.level_ptr[L]; t < an.level_ptr[L + 1]; t++) {
      const int sn = an.level_sn[t];
      if (d->clusters_ok && d->front_m_h[sn] > threshold) {
        b.push_back(sn);
        d->cluster_front = std::max(d->cluster_front, d->front_m_h[sn]);
      } else {
        a.push_back(sn);
        pf = std::max(pf, d->front_m_h[sn]);
      }
    }
    d->plain_front = std::max(d->plain_front, pf);
    d->solve_ptr_h.push_back((int)a.size());
    d->csolve_ptr_h.push_back((int)b.size());
    const int ncf = d->csolve_ptr_h.back() - d->csolve_ptr_h[L];
    d->csolve_ncl_h.push_back(d->wide_ok && ncf <= tg::kDirectWideFronts
                                  ? tg::kDirectSolveClusterWide
                                  : tg::kDirectSolveCluster);
    d->solve_front_h.push_back(pf);
  }
  d->solve_sn_h = a;
  d->csolve_sn_h = b;
  d->cluster_threshold = threshold;
  d->layout_version++;
  // the backward solve's L21^T x2 tiles of the cluster fronts, per level
  std::vector<int> tp(b.size());
  std::vector<int64_t> poff(b.size());
  d->gemv_total_h.assign(d->csolve_ptr_h.size() - 1, 0);
  size_t part = 0;
  for (size_t L = 0; L + 1 < d->csolve_ptr_h.size(); L++) {
    int tiles = 0;
    int64_t off = 0;
    for (int k = d->csolve_ptr_h[L]; k < d->csolve_ptr_h[L + 1]; k++) {
      const int sn = b[k];
      const int M = d->front_m_h[sn], C = d->front_c_h[sn];
      const int nrc = (M - C + tg::kDirectGemvRows - 1) / tg::kDirectGemvRows;
      tiles += ((C + 31) / 32) * nrc;
      tp[k] = tiles;
      poff[k] = off;
      off += (int64_t)nrc * C;
    }
    d->gemv_total_h[L] = tiles;
    part = std::max(part, (size_t)off);
  }
  tg::dfree(d->d_solve_sn);
  tg::dfree(d->d_csolve_sn);
  tg::dfree(d->d_gemv_tp);
  tg::dfree(d->d_gemv_poff);
  d->d_solve_sn = d->d_csolve_sn = nullptr;
  d->d_gemv_tp = nullptr;
  d->d_gemv_poff = nullptr;
  int rc = upload(&d->d_solve_sn, d->solve_sn_h);
  if (!rc) rc = upload(&d->d_csolve_sn, d->csolve_sn_h);
  if (!rc) rc = upload(&d->d_gemv_tp, tp);
  if (!rc) rc = upload(&d->d_gemv_poff, poff);
  if (!rc && part > d->part_entries) {
    if (d->d_part) cudaFree(d->d_part);
    d->d_part = nullptr;
    d->part_entries = 0;
    const size_t elem =
        d->precision == TG_PREC_FP32 ? sizeof(float) : sizeof(double);
    const cudaError_t e =
        cudaMalloc(&d->d_part, part * (size_t)d->max_nr * elem);
    if (e != cudaSuccess)
      return cuda_check(e, "tg_direct: backward solve chunk sums");
    d->part_entries = part;
  }
  if (rc) return rc;
  const cudaError_t se =
      tg::direct_set_smem(d->plain_front, d->cluster_front, d->max_nr);
  return se == cudaSuccess
             ? 0
             : cuda_check(se, "tg_direct: solve workspace attribute");
}

extern "C" {

int tg_direct_create(tg_mat *A, int use_coords, int precision,
                     tg_direct **out) {
  if (!A || !out) return fail(TG_ERR_ARG, "tg_direct_create: NULL argument");
  *out = nullptr;
  if (precision != TG_PREC_FP64 && precision != TG_PREC_FP32)
    return fail(TG_ERR_ARG, "tg_direct_create: bad precision");
  tg_assembler *a = A->a;
  if (!a || !a->initialized)
    return fail(TG_ERR_STATE, "tg_direct_create: assembler not initialised");
  tg_direct *d = new tg_direct();
  d->A = A;
  A->refcount++;
  {
    int lo_prio = 0, hi_prio = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (e == cudaSuccess)
      e = cudaStreamCreateWithPriority(&d->side_stream, cudaStreamNonBlocking,
                                       hi_prio);
    if (e == cudaSuccess)
      e = cudaEventCreateWithFlags(&d->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess)
      e = cudaEventCreateWithFlags(&d->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      tg_direct_decref(d);
      return cuda_check(e, "tg_direct_create: solve streams");
    }
  }
  d->n = A->nrows;
  d->bs = A->bsize;
  d->precision = precision;
  std::vector<double> xyz;
  if (use_coords) {
    xyz.resize((size_t)3 * a->nnodes);
    cudaError_t e = cudaMemcpy(xyz.data(), a->d_xpts,
                               xyz.size() * sizeof(double),
                               cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      tg_direct_decref(d);
      return cuda_check(e, "tg_direct_create: node coordinates");
    }
  }
  std::vector<int> perm = tg::direct::nested_dissection(
      a->rowp_h, a->cols_h, 64, use_coords ? xyz.data() : nullptr);
  d->an = tg::direct::analyse(a->rowp_h, a->cols_h, perm);
  const tg::direct::Analysis &an = d->an;
  d->ns = (int)an.sn_col.size() - 1;
  d->level_ptr_h = an.level_ptr;
  d->level_sn_h = an.level_sn;
  d->front_m_h.resize(d->ns);
  d->front_c_h.resize(d->ns);
  std::vector<int> ch_ptr(d->ns + 1, 0), ch_list(d->ns > 0 ? d->ns : 1);
  std::vector<int64_t> v_off(d->ns, 0);
  int64_t vacc = 0;
  for (int s = 0; s < d->ns; s++) {
    d->front_m_h[s] = (an.sn_rowptr[s + 1] - an.sn_rowptr[s]) * d->bs;
    d->front_c_h[s] = (an.sn_col[s + 1] - an.sn_col[s]) * d->bs;
    d->max_front = std::max(d->max_front, d->front_m_h[s]);
    v_off[s] = vacc;
    vacc += d->front_m_h[s] - d->front_c_h[s];
    if (an.sn_parent[s] >= 0) ch_ptr[an.sn_parent[s] + 1]++;
  }
  for (int s = 0; s < d->ns; s++) ch_ptr[s + 1] += ch_ptr[s];
  {
    std::vector<int> fill(ch_ptr.begin(), ch_ptr.end() - 1);
    for (int s = 0; s < d->ns; s++)  // children in increasing order
      if (an.sn_parent[s] >= 0) ch_list[fill[an.sn_parent[s]]++] = s;
  }
  std::vector<int> small_h;
  d->small_ptr_h.assign(1, 0);
  for (size_t L = 0; L + 1 < an.level_ptr.size(); L++) {
    for (int t = an.level_ptr[L]; t < an.level_ptr[L + 1]; t++) {
      const int sn = an.level_sn[t];
      if (d->front_m_h[sn] <= kSmallFront) small_h.push_back(sn);
    }
    d->small_ptr_h.push_back((int)small_h.size());
  }
  d->tile = precision == TG_PREC_FP32 ? tg::kDirectTile32 : TG_DIRECT_TILE_F64;
  d->steps = tg::direct::panel_steps(an, d->bs, kSmallFront, tg::kDirectPanel,
                                     d->tile, tg::kDirectTrsmRows);
  d->clusters_ok = tg::direct_cluster_solve_ok(tg::kDirectSolveCluster);
  d->wide_ok = d->clusters_ok &&
               tg::direct_cluster_solve_ok(tg::kDirectSolveClusterWide);
  if (!d->clusters_ok) d->cluster_threshold = 1 << 30;
  // the fronts factored by panels keep the inverses of their diagonal
  // blocks (the solves' block steps become 32 x 32 products)
  std::vector<int64_t> dinv_off(d->ns, -1);
  std::vector<int> inv_sn, inv_k0;
  int64_t dinv_len = 0;
  for (int sn = 0; sn < d->ns; sn++) {
    if (d->front_m_h[sn] <= kSmallFront) continue;
    dinv_off[sn] = dinv_len;
    for (int k0 = 0; k0 < d->front_c_h[sn]; k0 += tg::kDirectPanel) {
      inv_sn.push_back(sn);
      inv_k0.push_back(k0);
      dinv_len += (int64_t)tg::kDirectPanel * tg::kDirectPanel;
    }
  }
  d->inv_count = (int)inv_sn.size();
  for (size_t L = 0; L + 1 < an.level_ptr.size(); L++) {
    int nch = 0, um = 0;
    int64_t zmax = 0;
    for (int t = an.level_ptr[L]; t < an.level_ptr[L + 1]; t++) {
      const int sn = an.level_sn[t];
      const int64_t M = d->front_m_h[sn], C = d->front_c_h[sn];
      zmax = std::max(zmax, M * C + (M - C) * (M - C));
      nch = std::max(nch, ch_ptr[sn + 1] - ch_ptr[sn]);
      for (int k = ch_ptr[sn]; k < ch_ptr[sn + 1]; k++)
        um = std::max(um, d->front_m_h[ch_list[k]] - d->front_c_h[ch_list[k]]);
    }
    d->zero_y_h.push_back(
        (int)((zmax + tg::kDirectZeroChunk - 1) / tg::kDirectZeroChunk));
    d->ext_nch_h.push_back(nch);
    d->ext_y_h.push_back((um + tg::kDirectExtendRows - 1) /
                         tg::kDirectExtendRows);
  }
  {
    const int nlev = (int)an.level_ptr.size() - 1;
    d->step_ptr_h.assign(nlev + 1, 0);
    for (int L : d->steps.level) d->step_ptr_h[L + 1]++;
    for (int L = 0; L < nlev; L++) d->step_ptr_h[L + 1] += d->step_ptr_h[L];
  }
  std::vector<int> bcmask(d->n, 0);
  for (size_t k = 0; k < a->bc_nodes_h.size(); k++)
    bcmask[a->bc_nodes_h[k]] |= a->bc_masks_h[k];
  const size_t b2 = (size_t)d->bs * d->bs;
  const size_t N = (size_t)d->n * d->bs;
  int rc = 0;
  if (!rc) rc = upload(&d->d_perm, an.perm);
  if (!rc) rc = upload(&d->d_bcmask, bcmask);
  {
    const tg::direct::BcCoupling c =
        tg::direct::bc_coupling(a->rowp_h, a->cols_h, bcmask, an.iperm);
    d->bc_nrow = (int)c.row.size();
    if (!rc && d->bc_nrow) rc = upload(&d->d_bc_row, c.row);
    if (!rc && d->bc_nrow) rc = upload(&d->d_bc_pos, c.pos);
    if (!rc && d->bc_nrow) rc = upload(&d->d_bc_ptr, c.ptr);
    if (!rc && d->bc_nrow) rc = upload(&d->d_bc_blk, c.blk);
  }
  if (!rc) rc = upload(&d->d_sn_col, an.sn_col);
  if (!rc) rc = upload(&d->d_sn_rowptr, an.sn_rowptr);
  if (!rc) rc = upload(&d->d_sn_rows, an.sn_rows);
  if (!rc) rc = upload(&d->d_sn_parent, an.sn_parent);
  if (!rc) rc = upload(&d->d_ea_ptr, an.ea_ptr);
  if (!rc) rc = upload(&d->d_ea_rel, an.ea_rel);
  if (!rc) rc = upload(&d->d_asm_ptr, an.asm_ptr);
  if (!rc) rc = upload(&d->d_asm_blk, an.asm_blk);
  if (!rc) rc = upload(&d->d_asm_row, an.asm_row);
  if (!rc) rc = upload(&d->d_asm_col, an.asm_col);
  if (!rc) rc = upload(&d->d_ch_ptr, ch_ptr);
  if (!rc) rc = upload(&d->d_ch_list, ch_list);
  if (!rc) rc = upload(&d->d_level_sn, an.level_sn);
  if (!rc) rc = upload(&d->d_small, small_h);
  if (!rc) rc = upload(&d->d_step_fronts, d->steps.fronts);
  if (!rc) rc = upload(&d->d_step_tprefix, d->steps.tprefix);
  if (!rc) rc = upload(&d->d_step_rprefix, d->steps.rprefix);
  if (!rc) rc = upload(&d->d_l_off, an.l_off);
  if (!rc) rc = upload(&d->d_u_off, an.u_off);
  if (!rc) rc = upload(&d->d_v_off, v_off);
  if (!rc) rc = upload(&d->d_dinv_off, dinv_off);
  if (!rc && d->inv_count) rc = upload(&d->d_inv_sn, inv_sn);
  if (!rc && d->inv_count) rc = upload(&d->d_inv_k0, inv_k0);
  d->contrib_len = vacc;
  // right-hand sides per solve pass: 4, unless the workspace of the largest
  // front would not fit a CTA's shared memory beside the solve kernels'
  // static shared memory (at most 32 KB: staged rows, inverse blocks)
  constexpr size_t kSmemMax = (227 - 32) * 1024;
  // (for every cluster threshold the autotuner may pick)
  const int pf_max = d->clusters_ok ? std::min(d->max_front, kTuneMaxFront)
                                    : d->max_front;
  for (int nr : {4, 2, 1}) {
    d->max_nr = nr;
    if (tg::direct_solve_smem(pf_max, nr, sizeof(double)) <= kSmemMax &&
        tg::direct_cluster_smem(d->max_front, nr, sizeof(double),
                                tg::kDirectSolveCluster) <=
            kSmemMax)
      break;
  }
  const size_t R = (size_t)d->max_nr;
  if (precision == TG_PREC_FP64) {
    if (!rc) rc = dalloc(&d->d_lstore, (size_t)an.l_total * b2);
    if (!rc) rc = dalloc(&d->d_pool, (size_t)an.u_peak * b2);
    if (!rc && dinv_len) rc = dalloc(&d->d_dinv, (size_t)dinv_len);
    if (!rc) rc = dalloc(&d->d_contrib, (size_t)vacc * R);
    if (!rc) rc = dalloc(&d->d_ypos, N * R);
    if (!rc) rc = dalloc(&d->d_xpos, N * R);
  } else {
    if (!rc) rc = dalloc(&d->d_lstore32, (size_t)an.l_total * b2);
    if (!rc) rc = dalloc(&d->d_pool32, (size_t)an.u_peak * b2);
    if (!rc && dinv_len) rc = dalloc(&d->d_dinv32, (size_t)dinv_len);
    if (!rc) rc = dalloc(&d->d_contrib32, (size_t)vacc * R);
    if (!rc) rc = dalloc(&d->d_ypos32, N * R);
    if (!rc) rc = dalloc(&d->d_xpos32, N * R);
    if (!rc) rc = dalloc(&d->d_a32, (size_t)A->nnz * b2);
    if (!rc) rc = dalloc(&d->d_r32, N * R);
    if (!rc) rc = dalloc(&d->d_c32, N * R);
  }
  // refinement (both precisions): residuals, corrections, the max-|x|
  // reductions and their scalars (3 per right-hand side)
  if (!rc) rc = dalloc(&d->d_r, N * R);
  if (!rc) rc = dalloc(&d->d_t, N * R);
  if (!rc) rc = dalloc(&d->d_red, (size_t)kRedParts * R);
  if (!rc) rc = dalloc(&d->d_scal, 3 * R + 2);
  if (!rc) rc = dalloc(&d->d_fail, 1);
  if (!rc && tg::direct_solve_smem(pf_max, 1, sizeof(double)) > kSmemMax)
    rc = fail(TG_ERR_ARG, "tg_direct_create: front too large for a CTA's "
                          "solve workspace");
  if (!rc) rc = build_solve_lists(d, d->cluster_threshold);
  if (rc) {
    tg_direct_decref(d);
    return rc;
  }
  *out = d;
  return 0;
}

int tg_direct_decref(tg_direct *d) {
  if (!d) return 0;
  if (--d->refcount == 0) {
    tg_mat_decref(d->A);
    delete d;
  }
  return 0;
}

}  // extern "C"

template <class T>
static void factor_levels(tg_direct *d, cudaStream_t s) {
  const tg::DirectView v = d->view();
  for (size_t L = 0; L + 1 < d->level_ptr_h.size(); L++) {
    const int b = d->level_ptr_h[L], e = d->level_ptr_h[L + 1];
    tg::launch_direct_level_assemble<T>(v, d->d_level_sn + b, e - b,
                                        d->A->d_vals, d->zero_y_h[L],
                                        d->ext_nch_h[L], d->ext_y_h[L], s);
    // the level's small fronts in one launch, its large ones by panels
    const int sb = d->small_ptr_h[L], se = d->small_ptr_h[L + 1];
    tg::launch_direct_factor_small<T>(v, d->d_small + sb, se - sb, d->d_fail,
                                      s);
    for (int t = d->step_ptr_h[L]; t < d->step_ptr_h[L + 1]; t++) {
      const tg::direct::PanelSteps &ps = d->steps;
      tg::launch_direct_panel_step<T>(
          v, d->d_step_fronts + ps.front_off[t], ps.count[t],
          d->d_step_tprefix + ps.tile_off[t], ps.total[t],
          d->d_step_rprefix + ps.tile_off[t], ps.rtotal[t], ps.k0[t],
          d->tile, d->d_fail, s);
    }
  }
  tg::launch_direct_inverses<T>(v, d->d_inv_sn, d->d_inv_k0, d->inv_count,
                                s);
}

// The stream of a level's cluster solves: the side stream, forked from s
// after the levels before, when the level also has one-CTA solves (which
// stay on s); else s itself.  level_join puts s behind the side stream's
// launches.  Inside a stream capture the fork and join become graph edges.
static cudaStream_t level_fork(tg_direct *d, bool both, cudaStream_t s) {
  if (!both) return s;
  cudaEventRecord(d->ev_fork, s);
  cudaStreamWaitEvent(d->side_stream, d->ev_fork, 0);
  return d->side_stream;
}
static void level_join(tg_direct *d, cudaStream_t sp, cudaStream_t s) {
  if (sp == s) return;
  cudaEventRecord(d->ev_join, sp);
  cudaStreamWaitEvent(s, d->ev_join, 0);
}

// X = A^-1 B in T for nrhs right-hand sides N = n bs apart: per pass of
// at most max_nr of them, b into the factor's order (interleaved) less
// its coupling to the constrained dofs (a: the matrix values in T), the
// level sweeps, back to the node order
template <class T>
static void solve_levels(tg_direct *d, int nrhs, const T *b, T *x,
                         const T *a, T *ypos, T *xpos, T *contrib,
                         cudaStream_t s) {
  const tg::DirectView v = d->view();
  const tg::DirectBc bc = d->bc();
  const size_t N = (size_t)d->n * d->bs;
  const int nl = (int)d->level_ptr_h.size() - 1;
  for (int r0 = 0; r0 < nrhs;) {
    const int left = nrhs - r0;
    const int nr = left >= 4 && d->max_nr >= 4 ? 4
                   : left >= 2 && d->max_nr >= 2 ? 2 : 1;
    const T *bb = b + (size_t)r0 * N;
    T *xx = x + (size_t)r0 * N;
    tg::launch_direct_rhs<T>(d->n, d->bs, d->d_perm, bb, ypos, nr, N, s);
    tg::launch_direct_bc_couple<T>(bc, d->bs, a, bb, ypos, nr, N, s);
    for (int L = 0; L < nl; L++) {
      const int lb = d->solve_ptr_h[L], le = d->solve_ptr_h[L + 1];
      const int cb = d->csolve_ptr_h[L], ce = d->csolve_ptr_h[L + 1];
      const cudaStream_t sc = level_fork(d, le > lb && ce > cb, s);
      tg::launch_direct_forward_cluster<T>(v, d->d_csolve_sn + cb, ce - cb,
                                           d->cluster_front, nr,
                                           d->csolve_ncl_h[L], ypos, contrib,
                                           sc);
      tg::launch_direct_forward<T>(v, d->d_solve_sn + lb, le - lb,
                                   d->solve_front_h[L], nr, ypos, contrib, s);
      level_join(d, sc, s);
    }
    for (int L = nl - 1; L >= 0; L--) {
      const int lb = d->solve_ptr_h[L], le = d->solve_ptr_h[L + 1];
      const int cb = d->csolve_ptr_h[L], ce = d->csolve_ptr_h[L + 1];
      const cudaStream_t sc = level_fork(d, le > lb && ce > cb, s);
      tg::launch_direct_bwd_gemv<T>(v, d->d_csolve_sn + cb, d->d_gemv_tp + cb,
                                    d->d_gemv_poff + cb, ce - cb,
                                    d->gemv_total_h[L], nr, xpos,
                                    (T *)d->d_part, sc);
      tg::launch_direct_backward_cluster<T>(
          v, d->d_csolve_sn + cb, d->d_gemv_poff + cb, ce - cb,
          d->cluster_front, nr, d->csolve_ncl_h[L], ypos, xpos,
          (const T *)d->d_part, sc);
      tg::launch_direct_backward<T>(v, d->d_solve_sn + lb, le - lb,
                                    d->solve_front_h[L], nr, ypos, xpos, s);
      level_join(d, sc, s);
    }
    tg::launch_direct_unpermute<T>(d->n, d->bs, d->d_perm, xpos, xx, nr, N,
                                   s);
    r0 += nr;
  }
}

namespace tg {

long long direct_layout_version(const tg_direct *d) {
  return d ? d->layout_version : 0;
}
tg_mat *direct_matrix(const tg_direct *d) { return d->A; }
int direct_precision(const tg_direct *d) { return d->precision; }
bool direct_is_factored(const tg_direct *d) { return d->factored; }
void direct_incref(tg_direct *d) { d->refcount++; }

int direct_enqueue_solve(tg_direct *d, int nrhs, const void *b, void *x,
                         bool f32, cudaStream_t s) {
  if (!d || !b || !x || nrhs < 1)
    return fail(TG_ERR_ARG, "direct solve: bad arguments");
  if (f32 != (d->precision == TG_PREC_FP32))
    return fail(TG_ERR_ARG, "direct solve: precision of the factorisation");
  if (f32)
    solve_levels<float>(d, nrhs, (const float *)b, (float *)x, d->d_a32,
                        d->d_ypos32, d->d_xpos32, d->d_contrib32, s);
  else
    solve_levels<double>(d, nrhs, (const double *)b, (double *)x,
                         d->A->d_vals, d->d_ypos, d->d_xpos, d->d_contrib,
                         s);
  return 0;
}

}  // namespace tg

// Iterative refinement of nr <= max_nr right-hand sides (N apart): x = 0,
// then per step x += (the factorisation's solve of r = b - A x), r in FP64
// (an FP32 factorisation solves FP32 copies of r), with the stopping tests
// of tg_direct_solve_refined_multi per right-hand side; one that has
// stopped keeps its x (its residual is zeroed before the solve, whose
// correction is then exactly zero).
static int refine_pass(tg_direct *d, int nr, const double *b, double *x,
                       int max_steps, double tol, double ftol, double rtol,
                       int *steps, double *eta_out, cudaStream_t s) {
  tg_mat *A = d->A;
  const size_t N = (size_t)d->n * d->bs;
  const bool f32 = d->precision == TG_PREC_FP32;
  const bool stated = ftol > 0.0 || rtol > 0.0;
  double h[3 * 4];
  double bnorm[4], prev[4], eta[4];
  int slow[4], taken[4];
  bool met[4], done[4];
  tg::launch_reduce_absmax_multi(b, nr, N, d->d_red, kRedParts, d->d_scal, 1,
                                 s);
  TG_CUDA(cudaMemcpyAsync(h, d->d_scal, nr * sizeof(double),
                          cudaMemcpyDeviceToHost, s));
  TG_CUDA(cudaStreamSynchronize(s));
  bool all_done = true;
  for (int r = 0; r < nr; r++) {
    bnorm[r] = h[r];
    prev[r] = eta[r] = 0.0;
    slow[r] = taken[r] = 0;
    met[r] = done[r] = bnorm[r] == 0.0;  // x = 0 is exact
    all_done = all_done && done[r];
  }
  TG_CUDA(cudaMemsetAsync(x, 0, N * nr * sizeof(double), s));
  tg::launch_copy(b, d->d_r, N * nr, s);
  for (int step = 0; step < max_steps && !all_done; step++) {
    if (f32) {
      tg::launch_d2f(d->d_r, d->d_r32, N * nr, s);
      for (int r = 0; r < nr; r++)
        if (done[r])
          TG_CUDA(cudaMemsetAsync(d->d_r32 + r * N, 0, N * sizeof(float), s));
      solve_levels<float>(d, nr, d->d_r32, d->d_c32, d->d_a32, d->d_ypos32,
                          d->d_xpos32, d->d_contrib32, s);
      if (ftol > 0.0)  // the correction itself is tested below
        tg::launch_f2d(d->d_c32, d->d_t, N * nr, s);
    } else {
      for (int r = 0; r < nr; r++)
        if (done[r])
          TG_CUDA(cudaMemsetAsync(d->d_r + r * N, 0, N * sizeof(double), s));
      solve_levels<double>(d, nr, d->d_r, d->d_t, d->A->d_vals, d->d_ypos,
                           d->d_xpos, d->d_contrib, s);
    }
    if (ftol > 0.0)  // the step's correction, max |dx|
      tg::launch_reduce_absmax_multi(d->d_t, nr, N, d->d_red, kRedParts,
                                     d->d_scal + 2, 3, s);
    if (f32 && ftol <= 0.0)
      tg::launch_f2d_add(d->d_c32, x, N * nr, s);
    else
      tg::launch_axpy(1.0, d->d_t, x, N * nr, s);
    // r = b - A x, then max |r| and max |x| per right-hand side
    tg::launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols,
                         A->d_vals, x, d->d_t, s, nr, N);
    tg::launch_residual(b, d->d_t, d->d_r, N * nr, s);
    tg::launch_reduce_absmax_multi(d->d_r, nr, N, d->d_red, kRedParts,
                                   d->d_scal, 3, s);
    tg::launch_reduce_absmax_multi(x, nr, N, d->d_red, kRedParts,
                                   d->d_scal + 1, 3, s);
    TG_CUDA(cudaMemcpyAsync(h, d->d_scal, 3 * nr * sizeof(double),
                            cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    all_done = true;
    for (int r = 0; r < nr; r++) {
      if (done[r]) continue;
      taken[r]++;
      // normwise backward error of x
      const double den = d->anorm * h[3 * r + 1] + bnorm[r];
      eta[r] = den > 0.0 ? h[3 * r] / den : 0.0;
      if (!(eta[r] == eta[r])) {  // NaN: the factorisation is unusable
        met[r] = false;
        done[r] = true;
        continue;
      }
      // stated accuracy: stop as soon as every given test holds
      if (stated && eta[r] <= tol &&
          (ftol <= 0.0 || h[3 * r + 2] <= ftol * h[3 * r + 1]) &&
          (rtol <= 0.0 || h[3 * r] <= rtol * bnorm[r])) {
        met[r] = done[r] = true;
        continue;
      }
      if (eta[r] <= tol) met[r] = true;
      // The backward-error test alone stops early where |A| |x| >> |b|
      // (thin shells): there eta reaches eps sqrt(N) with a residual still
      // far above an FP64 factorisation's.  So the steps go on while they
      // halve eta, and stop at the first step that does not once the
      // tolerance is met (two such steps in a row before it: stagnation).
      // This also ends a stated test that FP64 cannot reach: a residual
      // below the rounding of A x itself (about eps |A| |x|, which on thin
      // shells is far above rtol |b|) is accepted at that floor, as the
      // Krylov solves accept it.
      slow[r] = (taken[r] > 1 && eta[r] > 0.5 * prev[r]) ? slow[r] + 1 : 0;
      if (slow[r] >= (met[r] ? 1 : 2)) done[r] = true;
      prev[r] = eta[r];
      all_done = all_done && done[r];
    }
  }
  int rc = 0;
  for (int r = 0; r < nr; r++) {
    if (steps) steps[r] = taken[r];
    if (eta_out) eta_out[r] = eta[r];
    if (!met[r]) rc = TG_ERR_NOCONV;
  }
  TG_CUDA(cudaGetLastError());
  return rc;
}

extern "C" {

int tg_direct_factor(tg_direct *d, void *s) {
  if (!d) return fail(TG_ERR_ARG, "tg_direct_factor: NULL");
  TG_CUDA(cudaMemsetAsync(d->d_fail, 0, sizeof(int), S(s)));
  if (d->factor_calls++ == 0) {
    if (d->precision == TG_PREC_FP64) {
      factor_levels<double>(d, S(s));
    } else {
      const tg_mat *A = d->A;
      tg::launch_d2f(A->d_vals, d->d_a32,
                     (size_t)A->nnz * A->bsize * A->bsize, S(s));
      factor_levels<float>(d, S(s));
    }
    TG_CUDA(cudaGetLastError());
  } else if (!d->factor_exec) {
    // captured on the side stream (the caller's may be the legacy default
    // stream, which cannot be captured), launched on the caller's
    cudaStream_t cs = d->side_stream;
    TG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    if (d->precision == TG_PREC_FP64) {
      factor_levels<double>(d, cs);
    } else {
      const tg_mat *A = d->A;
      tg::launch_d2f(A->d_vals, d->d_a32,
                     (size_t)A->nnz * A->bsize * A->bsize, cs);
      factor_levels<float>(d, cs);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cs, &g);
    cudaError_t ie = ce;
    if (ce == cudaSuccess)
      ie = cudaGraphInstantiate(&d->factor_exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      d->factor_exec = nullptr;
      return cuda_check(ie, "tg_direct_factor: factorisation graph");
    }
  }
  if (d->factor_exec) TG_CUDA(cudaGraphLaunch(d->factor_exec, S(s)));
  {  // ||A||_inf of these values, for the refinement's backward error
    const tg_mat *A = d->A;
    const size_t N = (size_t)d->n * d->bs;
    tg::launch_bcsr_row_abs_sum(A->bsize, A->nrows, A->a->d_rowp, A->d_vals,
                                d->d_t, S(s));
    tg::launch_reduce_absmax(d->d_t, N, d->d_red, kRedParts, d->d_scal,
                             S(s));
    TG_CUDA(cudaMemcpyAsync(&d->anorm, d->d_scal, sizeof(double),
                            cudaMemcpyDeviceToHost, S(s)));
  }
  int hfail = 0;
  TG_CUDA(cudaMemcpyAsync(&hfail, d->d_fail, sizeof(int),
                          cudaMemcpyDeviceToHost, S(s)));
  TG_CUDA(cudaStreamSynchronize(S(s)));
  TG_CUDA(cudaGetLastError());
  if (hfail) {
    char buf[128];
    snprintf(buf, sizeof(buf),
             "tg_direct_factor: non-positive pivot in supernode %d", hfail - 1);
    return fail(TG_ERR_PIVOT, buf);
  }
  d->factored = true;
  return 0;
}

int tg_direct_solve(tg_direct *d, const double *b, double *x, void *s) {
  return tg_direct_solve_multi(d, 1, b, x, s);
}

int tg_direct_solve_multi(tg_direct *d, int nrhs, const double *b, double *x,
                          void *s) {
  if (!d || !b || !x || nrhs < 1)
    return fail(TG_ERR_ARG, "tg_direct_solve: bad arguments");
  if (!d->factored) return fail(TG_ERR_STATE, "tg_direct_solve: not factored");
  if (d->precision != TG_PREC_FP64)
    return fail(TG_ERR_ARG, "tg_direct_solve: FP32 factorisation "
                            "(use tg_direct_solve_f32)");
  tg::direct_enqueue_solve(d, nrhs, b, x, false, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_direct_solve_f32(tg_direct *d, const float *b, float *x, void *s) {
  if (!d || !b || !x) return fail(TG_ERR_ARG, "tg_direct_solve_f32: NULL");
  if (!d->factored)
    return fail(TG_ERR_STATE, "tg_direct_solve_f32: not factored");
  if (d->precision != TG_PREC_FP32)
    return fail(TG_ERR_ARG, "tg_direct_solve_f32: FP64 factorisation");
  tg::direct_enqueue_solve(d, 1, b, x, true, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_direct_solve_refined(tg_direct *d, const double *b, double *x,
                            int steps, void *s) {
  if (!d || !b || !x || steps < 1)
    return fail(TG_ERR_ARG, "tg_direct_solve_refined: bad arguments");
  if ((const void *)b == (const void *)x)  // b is re-read after x is zeroed
    return fail(TG_ERR_ARG, "tg_direct_solve_refined: b and x alias");
  if (!d->factored)
    return fail(TG_ERR_STATE, "tg_direct_solve_refined: not factored");
  if (d->precision != TG_PREC_FP32)
    return fail(TG_ERR_ARG, "tg_direct_solve_refined: needs the FP32 "
                            "factorisation");
  tg_mat *A = d->A;
  const size_t N = (size_t)d->n * d->bs;
  // x = 0, r = b; then per step: x += FP32-solve(r), r = b - A x (FP64)
  TG_CUDA(cudaMemsetAsync(x, 0, N * sizeof(double), S(s)));
  tg::launch_copy(b, d->d_r, N, S(s));
  for (int k = 0; k < steps; k++) {
    tg::launch_d2f(d->d_r, d->d_r32, N, S(s));
    solve_levels<float>(d, 1, d->d_r32, d->d_c32, d->d_a32, d->d_ypos32,
                        d->d_xpos32, d->d_contrib32, S(s));
    tg::launch_f2d(d->d_c32, d->d_t, N, S(s));
    tg::launch_axpy(1.0, d->d_t, x, N, S(s));
    if (k + 1 < steps) {
      tg::launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols,
                           A->d_vals, x, d->d_t, S(s));
      tg::launch_copy(b, d->d_r, N, S(s));
      tg::launch_axpy(-1.0, d->d_t, d->d_r, N, S(s));
    }
  }
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_direct_solve_refined_tol(tg_direct *d, const double *b, double *x,
                                int max_steps, double tol, int *steps,
                                double *eta_out, void *s) {
  if (d && d->precision != TG_PREC_FP32)
    return fail(TG_ERR_ARG, "tg_direct_solve_refined_tol: needs the FP32 "
                            "factorisation");
  return tg_direct_solve_refined_multi(d, 1, b, x, max_steps, tol, 0.0, 0.0,
                                       steps, eta_out, s);
}

int tg_direct_solve_refined_multi(tg_direct *d, int nrhs, const double *b,
                                  double *x, int max_steps, double tol,
                                  double ftol, double rtol, int *steps,
                                  double *eta_out, void *s) {
  if (!d || !b || !x || nrhs < 1 || max_steps < 1 || !(tol > 0.0) ||
      !(ftol >= 0.0) || !(rtol >= 0.0))
    return fail(TG_ERR_ARG, "tg_direct_solve_refined_tol: bad arguments");
  const size_t N = (size_t)d->n * d->bs;
  // b is re-read after x is zeroed
  const char *bb = (const char *)b, *xb = (const char *)x;
  if (bb < xb + N * nrhs * sizeof(double) && xb < bb + N * nrhs * sizeof(double))
    return fail(TG_ERR_ARG, "tg_direct_solve_refined_tol: b and x alias");
  if (!d->factored)
    return fail(TG_ERR_STATE, "tg_direct_solve_refined_tol: not factored");
  int rc = 0;
  for (int r0 = 0; r0 < nrhs; r0 += d->max_nr) {
    const int nr = nrhs - r0 < d->max_nr ? nrhs - r0 : d->max_nr;
    const int e = refine_pass(d, nr, b + r0 * N, x + r0 * N, max_steps, tol,
                              ftol, rtol, steps ? steps + r0 : nullptr,
                              eta_out ? eta_out + r0 : nullptr, S(s));
    if (e && e != TG_ERR_NOCONV) return e;
    if (e) rc = e;
  }
  if (rc)
    return fail(TG_ERR_NOCONV, "tg_direct_solve_refined_tol: refinement did "
                               "not reach the backward-error tolerance");
  return 0;
}

int tg_direct_autotune(tg_direct *d, int *threshold, double *ms,
                       void *s) {
  if (!d) return fail(TG_ERR_ARG, "tg_direct_autotune: NULL");
  if (!d->factored)
    return fail(TG_ERR_STATE, "tg_direct_autotune: not factored");
  static const int cand[3] = {384, tg::kDirectClusterFront, kTuneMaxFront};
  if (ms)
    for (int k = 0; k < 3; k++) ms[k] = 0.0;
  int best = d->cluster_threshold;
  if (d->clusters_ok) {
    // the choice per matrix shape, precision and device
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, int, int>, int> cache;
    int dev = 0;
    TG_CUDA(cudaGetDevice(&dev));
    const auto key = std::make_tuple(d->n, d->A->nnz, d->bs, d->precision, dev);
    bool cached = false;
    {
      std::lock_guard<std::mutex> lock(mu);
      auto it = cache.find(key);
      if (it != cache.end()) {
        best = it->second;
        cached = true;
      }
    }
    if (!cached) {
      const size_t N = (size_t)d->n * d->bs;
      const bool f32 = d->precision == TG_PREC_FP32;
      tg::launch_fill(d->d_r, 1.0, N, S(s));
      if (f32) tg::launch_d2f(d->d_r, d->d_r32, N, S(s));
      const void *b = f32 ? (const void *)d->d_r32 : (const void *)d->d_r;
      void *x = f32 ? (void *)d->d_c32 : (void *)d->d_t;
      cudaEvent_t e0, e1;
      TG_CUDA(cudaEventCreate(&e0));
      TG_CUDA(cudaEventCreate(&e1));
      float bestms = 0.0f;
      for (int k = 0; k < 3; k++) {
        int rc = build_solve_lists(d, cand[k]);
        if (!rc) rc = tg::direct_enqueue_solve(d, 1, b, x, f32, S(s));  // warm
        if (rc) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return rc;
        }
        TG_CUDA(cudaEventRecord(e0, S(s)));
        for (int r = 0; r < 3; r++)
          tg::direct_enqueue_solve(d, 1, b, x, f32, S(s));
        TG_CUDA(cudaEventRecord(e1, S(s)));
        TG_CUDA(cudaEventSynchronize(e1));
        float t = 0.0f;
        TG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        t /= 3.0f;
        if (ms) ms[k] = t;
        if (k == 0 || t < bestms) {
          bestms = t;
          best = cand[k];
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      std::lock_guard<std::mutex> lock(mu);
      cache[key] = best;
    }
    const int rc = build_solve_lists(d, best);
    if (rc) return rc;
  }
  if (threshold) *threshold = best;
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_direct_get_stats(tg_direct *d, double *stats) {
  if (!d || !stats) return fail(TG_ERR_ARG, "tg_direct_get_stats: NULL");
  const size_t b2 = (size_t)d->bs * d->bs;
  stats[0] = d->ns;
  stats[1] = (double)d->level_ptr_h.size() - 1;
  stats[2] = (double)d->an.l_total * b2 * sizeof(double);
  stats[3] = (double)d->an.u_peak * b2 * sizeof(double);
  stats[4] = (double)d->an.flops_scalar(d->bs);
  stats[5] = d->max_front;
  stats[6] = d->precision;
  stats[7] = (double)d->csolve_sn_h.size();
  stats[8] = d->cluster_threshold;
  return 0;
}

}  // extern "C"
