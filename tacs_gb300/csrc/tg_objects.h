// Host-side objects behind the opaque handles of the C ABI (assembler,
// BCSR matrix, preconditioner, Krylov solver) and the small allocation
// helpers shared by the runtime translation units.  Internal header.
#pragma once

#include <string>
#include <vector>

#include "tg_internal.h"

namespace tg {

template <typename T>
inline int dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) return cuda_check(e, "cudaMalloc");
  return 0;
}
template <typename T>
inline int upload(T **p, const std::vector<T> &h) {
  int rc = dalloc(p, h.size());
  if (rc) return rc;
  if (!h.empty()) {
    cudaError_t e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T),
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_check(e, "cudaMemcpy H2D");
  }
  return 0;
}
template <typename T>
inline void dfree(T *&p) {
  if (p) cudaFree(p);
  p = nullptr;
}

inline int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

}  // namespace tg

using namespace tg;

struct tg_assembler {
  int refcount = 1;
  ElemParams ep{};
  int nnodes = 0, nelem = 0, vpn = 0, npe = 0;
  std::vector<int> conn_h;
  std::vector<int> bc_nodes_h, bc_masks_h;
  std::vector<double> thick_h;
  std::vector<int> dvnum_h;
  std::vector<double> pres_h;  // 4 per element (zeros where unloaded)
  bool has_pres = false;
  std::vector<int> trac_ptr_h, trac_face_h;
  std::vector<double> trac_val_h;
  bool initialized = false;
  int ndv = 0;
  // BCSR pattern
  std::vector<int> rowp_h, cols_h, diag_h;
  // colouring
  std::vector<int> color_ptr_h, color_elems_h;
  // device
  int *d_conn = nullptr;
  double *d_xpts = nullptr, *d_thick = nullptr, *d_pres = nullptr;
  int *d_dvnum = nullptr, *d_trac_ptr = nullptr, *d_trac_face = nullptr;
  double *d_trac_val = nullptr;
  int *d_bc_nodes = nullptr, *d_bc_masks = nullptr;
  int *d_rowp = nullptr, *d_cols = nullptr, *d_diag = nullptr;
  int *d_color_elems = nullptr;
  // first-writer masks of the shell assembly (empty: zero fill and add)
  unsigned *d_first = nullptr;
  int *d_dv_ptr = nullptr, *d_dv_elems = nullptr;
  double *d_elem_fail = nullptr, *d_elem_wdet = nullptr;
  double *d_elem_sed = nullptr, *d_elem_val = nullptr;
  double *d_partials = nullptr, *d_scalars = nullptr;
  int npart = 512;
  KsStats ks{0.0, 1.0, 100.0};
  bool ks_valid = false;
  // node-coordinate derivatives: 0 forward (dual), 1 reverse sweep
  int xpt_mode = TG_XPT_REVERSE;  // the faster of the two exact forms
  // element segments (independent meshes): contiguous element ranges
  int nseg = 0;
  std::vector<int> seg_elem_ptr_h;
  int *d_elem_seg = nullptr, *d_seg_elem_ptr = nullptr;
  KsStats *d_seg_ks = nullptr;
  double *d_seg_comp = nullptr;
  bool seg_ks_valid = false;
  // fixed-geometry assembly (geo_plan.h, geo_cache.cu): the plan depends on
  // the connectivity and constraints, the class table and f0 on the node
  // coordinates (set_nodes invalidates them)
  bool geo_enabled = false;
  bool geo_plan_ready = false, geo_table_valid = false;
  int geo_ncls = 0, geo_nwarps = 0;
  unsigned long long geo_mask[2] = {0, 0};
  size_t geo_table_doubles = 0, geo_plan_bytes = 0;
  int *d_geo_cptr = nullptr, *d_geo_contrib = nullptr, *d_geo_cls = nullptr;
  int *d_geo_node_bc = nullptr, *d_geo_kmax = nullptr, *d_geo_reps = nullptr;
  double *d_geo_table = nullptr, *d_geo_f0 = nullptr;
  double *d_geo_B = nullptr;  // shells: B_q and detXd_q per class
  unsigned long long *d_geo_masks = nullptr;

  int nq() const { return ep.elem_type == TG_ELEM_MITC4 ? 4 : 8; }

  MeshView view() const {
    MeshView m;
    m.nnodes = nnodes;
    m.nelem = nelem;
    m.vpn = vpn;
    m.npe = npe;
    m.conn = d_conn;
    m.xpts = d_xpts;
    m.thick = d_thick;
    m.pres = has_pres ? d_pres : nullptr;
    m.trac_ptr = trac_val_h.empty() ? nullptr : d_trac_ptr;
    m.trac_face = d_trac_face;
    m.trac_val = d_trac_val;
    m.rowp = d_rowp;
    m.cols = d_cols;
    m.elem_seg = nullptr;
    m.seg_ks = nullptr;
    const bool geo = geo_enabled && geo_table_valid && d_geo_B;
    m.geo_B = geo ? d_geo_B : nullptr;
    m.geo_cls = geo ? d_geo_cls : nullptr;
    m.first = d_first;
    return m;
  }
  // view whose KS sensitivities use the per-segment statistics
  MeshView view_segments() const {
    MeshView m = view();
    m.elem_seg = d_elem_seg;
    m.seg_ks = d_seg_ks;
    return m;
  }
  ColorRange color(int c) const {
    ColorRange r;
    r.elem_list = d_color_elems + color_ptr_h[c];
    r.count = color_ptr_h[c + 1] - color_ptr_h[c];
    return r;
  }
  int ncolors() const { return (int)color_ptr_h.size() - 1; }

  ~tg_assembler() {
    dfree(d_conn); dfree(d_xpts); dfree(d_thick); dfree(d_pres);
    dfree(d_dvnum); dfree(d_trac_ptr); dfree(d_trac_face); dfree(d_trac_val);
    dfree(d_bc_nodes); dfree(d_bc_masks); dfree(d_rowp); dfree(d_cols);
    dfree(d_diag); dfree(d_color_elems); dfree(d_dv_ptr); dfree(d_dv_elems);
    dfree(d_first);
    dfree(d_elem_fail); dfree(d_elem_wdet); dfree(d_elem_sed);
    dfree(d_elem_val); dfree(d_partials); dfree(d_scalars);
    dfree(d_elem_seg); dfree(d_seg_elem_ptr); dfree(d_seg_ks);
    dfree(d_seg_comp);
    dfree(d_geo_cptr); dfree(d_geo_contrib); dfree(d_geo_cls);
    dfree(d_geo_node_bc); dfree(d_geo_kmax); dfree(d_geo_reps);
    dfree(d_geo_table); dfree(d_geo_f0); dfree(d_geo_masks); dfree(d_geo_B);
  }
};

struct tg_mat {
  int refcount = 1;
  tg_assembler *a = nullptr;
  int bsize = 0, nrows = 0, nnz = 0;
  double *d_vals = nullptr;
  float *d_vals32 = nullptr;
  ~tg_mat() {
    dfree(d_vals);
    dfree(d_vals32);
  }
};

struct tg_pc {
  int refcount = 1;
  tg_mat *A = nullptr;
  int type = TG_PC_ILU0, precision = TG_PREC_FP64;
  // ILU(k): level of fill and block count of the factor's pattern (fnnz =
  // the matrix's block count for ILU(0) and block Jacobi)
  int lev_fill = 0, fnnz = 0;
  IluPlan plan{};
  int *d_lvl_rows = nullptr, *d_ulvl_rows = nullptr;
  int *d_upd_ptr = nullptr, *d_upd_tgt = nullptr, *d_upd_src = nullptr;
  int *d_fail = nullptr;
  double *d_F = nullptr, *d_tmp = nullptr;
  float *d_F32 = nullptr, *d_x32 = nullptr, *d_y32 = nullptr,
        *d_tmp32 = nullptr;
  double *d_gx = nullptr, *d_gy = nullptr;  // FP64 apply in/out buffers
  // colour-reordered variant and ILU(k): the factor's own pattern, the map
  // from its blocks to the matrix's (-1: fill, starts at zero), and for the
  // colour order the permutation and permuted work vectors
  int *d_prowp = nullptr, *d_pcols = nullptr, *d_pdiag = nullptr;
  int *d_valmap = nullptr, *d_perm = nullptr;
  double *d_px = nullptr, *d_py = nullptr;
  float *d_px32 = nullptr, *d_py32 = nullptr;
  int ncolors = 0;
  // cluster schedule of the triangular solves (natural-order ILU(0))
  int *d_cl_grp_lvl = nullptr, *d_cl_lvl_ptr = nullptr, *d_cl_rows = nullptr;
  int *d_cl_grp_ulvl = nullptr, *d_cl_ulvl_ptr = nullptr,
      *d_cl_urows = nullptr;
  // schedule autotuner: the plan inputs and the measured time per cluster
  // size (index = size; 0 = not measured)
  bool tuned = false;
  std::vector<int> tune_rowp, tune_cols, tune_lvl, tune_ulvl;
  int tune_nl = 0, tune_nu = 0;
  double tune_ms[17] = {0};
  // the level-by-level triangular solves replayed as one CUDA graph
  cudaGraphExec_t apply_exec = nullptr;
  bool factored = false;
  bool fp64_ready = false;  // FP32 pc: FP64 factor of the same matrix in d_F
  // TG_PC_DIRECT: the factorisation in the pc's precision, and for an FP32
  // pc the FP64 one its FP64 fallback passes use
  tg_direct *direct = nullptr, *direct64 = nullptr;
  // direct is the caller's factorisation (tg_pc_create_direct): the pc
  // never factors it
  bool shared_direct = false;
  ~tg_pc() {
    if (direct) tg_direct_decref(direct);
    if (direct64) tg_direct_decref(direct64);
    if (apply_exec) cudaGraphExecDestroy(apply_exec);
    dfree(d_lvl_rows); dfree(d_ulvl_rows); dfree(d_upd_ptr);
    dfree(d_upd_tgt); dfree(d_upd_src); dfree(d_fail); dfree(d_F);
    dfree(d_tmp); dfree(d_F32); dfree(d_x32); dfree(d_y32); dfree(d_tmp32);
    dfree(d_gx); dfree(d_gy); dfree(d_prowp); dfree(d_pcols); dfree(d_pdiag);
    dfree(d_valmap); dfree(d_perm); dfree(d_px); dfree(d_py);
    dfree(d_px32); dfree(d_py32); dfree(d_cl_grp_lvl); dfree(d_cl_lvl_ptr);
    dfree(d_cl_rows); dfree(d_cl_grp_ulvl); dfree(d_cl_ulvl_ptr);
    dfree(d_cl_urows);
  }
};

// Restarted GMRES over nsys = nseg x nrhs systems (tg_krylov.cu).  The
// device buffers are sized for one multivector width (nrhs) at a time and
// the CUDA graphs of a cycle are captured against them.
struct tg_ksm {
  int refcount = 1;
  tg_mat *A = nullptr;
  tg_pc *pc = nullptr;
  int m = 0, nrestart = 0, mixed = 0;
  double rtol = 1e-8, atol = 1e-30;
  size_t n = 0;                 // rows x block size of A
  std::vector<int> seg_rows;    // nseg + 1 block-row offsets of the systems
  int nrhs = 0;                 // current multivector width (0: not laid out)
  // the preconditioner's launch layout the graphs were captured with
  // (pc_layout_version); a change makes the next solve capture again
  long long pc_version = 0;
  size_t N = 0;                 // nrhs * n
  int nsys = 0;
  // multivector buffers
  int flexible = 0;             // keep Z_j = M^{-1} v_j (FP32 preconditioner)
  double *d_W = nullptr, *d_v = nullptr, *d_w = nullptr, *d_z = nullptr;
  double *d_Z = nullptr;
  double *d_z2 = nullptr, *d_B = nullptr, *d_X = nullptr;
  double *d_Bo = nullptr, *d_Xo = nullptr;             // mixed outer loop
  double *d_t64 = nullptr, *d_px = nullptr, *d_py = nullptr;  // FP64 pc
  float *d_x32 = nullptr, *d_y32 = nullptr, *d_w32 = nullptr;
  float *d_t32 = nullptr, *d_px32 = nullptr, *d_py32 = nullptr;
  double *d_partials = nullptr, *d_normparts = nullptr;
  // chunk list
  int *d_cstart = nullptr, *d_clen = nullptr, *d_csys = nullptr;
  int *d_sys_ptr = nullptr;
  KrylovChunks ch{};
  // per-system state (one allocation of doubles, one of ints)
  double *d_sd = nullptr;
  int *d_si = nullptr;
  KrylovState st{};
  int *h_pinned = nullptr;      // nactive read-back
  // graphs: cycle start, one Arnoldi step ([0] FP64 operator, [1] FP32
  // operator for mixed precision) and cycle end
  cudaGraphExec_t g_start = nullptr, g_iter[2] = {nullptr, nullptr},
                  g_end = nullptr;
  // a whole restart cycle per operator mode: start, a device-side WHILE
  // node over the Arnoldi step, end (null where conditional graph nodes are
  // not available: the three graphs above are launched from the host then)
  cudaGraphExec_t g_cycle[2] = {nullptr, nullptr};
  int step_nodes[2] = {0, 0};  // graph nodes (launches) of one Arnoldi step
  void free_layout() {
    if (g_start) cudaGraphExecDestroy(g_start);
    if (g_end) cudaGraphExecDestroy(g_end);
    for (int i = 0; i < 2; i++) {
      if (g_iter[i]) cudaGraphExecDestroy(g_iter[i]);
      if (g_cycle[i]) cudaGraphExecDestroy(g_cycle[i]);
      g_iter[i] = nullptr;
      g_cycle[i] = nullptr;
    }
    g_start = g_end = nullptr;
    dfree(d_W); dfree(d_v); dfree(d_w); dfree(d_z); dfree(d_z2); dfree(d_B);
    dfree(d_Z);
    dfree(d_X); dfree(d_Bo); dfree(d_Xo); dfree(d_t64); dfree(d_px);
    dfree(d_py); dfree(d_x32); dfree(d_y32); dfree(d_w32); dfree(d_t32);
    dfree(d_px32); dfree(d_py32); dfree(d_partials); dfree(d_normparts);
    dfree(d_cstart); dfree(d_clen); dfree(d_csys); dfree(d_sys_ptr);
    dfree(d_sd); dfree(d_si);
    nrhs = 0;
    N = 0;
  }
  ~tg_ksm() {
    free_layout();
    if (h_pinned) cudaFreeHost(h_pinned);
  }
};

static inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

namespace tg {
// M^{-1} on nrhs vectors ld apart (tg_runtime.cu); FP64 buffers for a FP64
// pc, FP32 for a FP32 pc
int pc_launch(tg_pc *pc, int nrhs, size_t ld, const void *in, void *out,
              void *tmp, void *px, void *py, cudaStream_t s, int use_f64 = -1);
// FP64 factor of an FP32 pc's matrix (for FP64 fallback passes)
int pc_factor_fp64(tg_pc *pc, cudaStream_t s);
// Allocate (not factor) whatever pc_factor_fp64 will fill, so that graphs
// captured before the fallback see its buffers
int pc_prepare_fp64(tg_pc *pc);
// Enqueue X = A^-1 B (nrhs vectors of n x bs entries back to back) with a
// direct factorisation whether or not it is factored yet (graph capture;
// tg_direct.cu): FP64 vectors for an FP64 factorisation, FP32 for an FP32
// one
int direct_enqueue_solve(tg_direct *d, int nrhs, const void *b, void *x,
                         bool f32, cudaStream_t s);
// A count that changes whenever the solves of a factorisation are laid out
// again (the autotuner's new launch lists), and of a pc's factorisations:
// graphs captured over older lists must be captured again
long long direct_layout_version(const tg_direct *d);
long long pc_layout_version(const tg_pc *pc);
// a factorisation's matrix, precision and factored state, and one more
// reference to it (tg_pc_create_direct; tg_direct.cu)
tg_mat *direct_matrix(const tg_direct *d);
int direct_precision(const tg_direct *d);
bool direct_is_factored(const tg_direct *d);
void direct_incref(tg_direct *d);
}  // namespace tg
