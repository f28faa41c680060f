// Host runtime of libtacs_gb300: the C ABI declared in include/tacs_gb300.h.
// Owns the device data of assemblers, BCSR matrices, preconditioners and
// Krylov solvers, builds the host-side plans (BCSR pattern, element
// colouring, ILU level sets and update lists, design-variable maps) and
// sequences the sm_103a kernels on the caller's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "tg_internal.h"

namespace tg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_check(cudaError_t e, const char *what) {
  set_error(std::string("CUDA error in ") + what + ": " +
            cudaGetErrorString(e));
  return TG_ERR_CUDA;
}

template <typename T>
static int dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) return cuda_check(e, "cudaMalloc");
  return 0;
}
template <typename T>
static int upload(T **p, const std::vector<T> &h) {
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
static void dfree(T *&p) {
  if (p) cudaFree(p);
  p = nullptr;
}

static int fail(int code, const std::string &msg) {
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
  int *d_dv_ptr = nullptr, *d_dv_elems = nullptr;
  double *d_elem_fail = nullptr, *d_elem_wdet = nullptr;
  double *d_elem_sed = nullptr, *d_elem_val = nullptr;
  double *d_partials = nullptr, *d_scalars = nullptr;
  int npart = 512;
  KsStats ks{0.0, 1.0, 100.0};
  bool ks_valid = false;

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
    dfree(d_elem_fail); dfree(d_elem_wdet); dfree(d_elem_sed);
    dfree(d_elem_val); dfree(d_partials); dfree(d_scalars);
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
  IluPlan plan{};
  int *d_lvl_rows = nullptr, *d_ulvl_rows = nullptr;
  int *d_upd_ptr = nullptr, *d_upd_tgt = nullptr, *d_upd_src = nullptr;
  int *d_fail = nullptr;
  double *d_F = nullptr, *d_tmp = nullptr;
  float *d_F32 = nullptr, *d_x32 = nullptr, *d_y32 = nullptr,
        *d_tmp32 = nullptr;
  double *d_gx = nullptr, *d_gy = nullptr;  // FP64 apply in/out buffers
  // colour-reordered variant: permuted pattern, value map, permutation and
  // permuted work vectors
  int *d_prowp = nullptr, *d_pcols = nullptr, *d_pdiag = nullptr;
  int *d_valmap = nullptr, *d_perm = nullptr;
  double *d_px = nullptr, *d_py = nullptr;
  float *d_px32 = nullptr, *d_py32 = nullptr;
  int ncolors = 0;
  // the level-by-level triangular solves replayed as one CUDA graph
  cudaGraphExec_t apply_exec = nullptr;
  bool factored = false;
  ~tg_pc() {
    if (apply_exec) cudaGraphExecDestroy(apply_exec);
    dfree(d_lvl_rows); dfree(d_ulvl_rows); dfree(d_upd_ptr);
    dfree(d_upd_tgt); dfree(d_upd_src); dfree(d_fail); dfree(d_F);
    dfree(d_tmp); dfree(d_F32); dfree(d_x32); dfree(d_y32); dfree(d_tmp32);
    dfree(d_gx); dfree(d_gy); dfree(d_prowp); dfree(d_pcols); dfree(d_pdiag);
    dfree(d_valmap); dfree(d_perm); dfree(d_px); dfree(d_py);
    dfree(d_px32); dfree(d_py32);
  }
};

struct tg_ksm {
  int refcount = 1;
  tg_mat *A = nullptr;
  tg_pc *pc = nullptr;
  int m = 0, nrestart = 0, mixed = 0;
  double rtol = 1e-8, atol = 1e-30;
  size_t n = 0;
  double *d_W = nullptr, *d_work = nullptr, *d_work2 = nullptr;
  double *d_h = nullptr, *d_h2 = nullptr, *d_partials = nullptr;
  double *d_r = nullptr, *d_d = nullptr;
  float *d_v32 = nullptr, *d_z32 = nullptr, *d_w32 = nullptr;
  int npart = 4096;
  ~tg_ksm() {
    dfree(d_W); dfree(d_work); dfree(d_work2); dfree(d_h); dfree(d_h2);
    dfree(d_partials); dfree(d_r); dfree(d_d); dfree(d_v32); dfree(d_z32);
    dfree(d_w32);
  }
};

static inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

extern "C" {

const char *tg_last_error(void) { return g_last_error.c_str(); }
int tg_version(void) { return 1; }

// ------------------------------------------------------------- assembler
int tg_assembler_create(int elem_type, int num_nodes, int num_elements,
                        const int *conn_host, double rho, double E, double nu,
                        double ys, int transform, const double *ref_axis_host,
                        tg_assembler **out) {
  if (!out) return fail(TG_ERR_ARG, "tg_assembler_create: out is NULL");
  *out = nullptr;
  if (elem_type != TG_ELEM_MITC4 && elem_type != TG_ELEM_HEX8)
    return fail(TG_ERR_ARG, "tg_assembler_create: unknown element type");
  if (num_nodes < 0 || num_elements < 0 || (num_elements > 0 && !conn_host))
    return fail(TG_ERR_ARG, "tg_assembler_create: bad sizes");
  tg_assembler *a = new tg_assembler();
  a->ep.elem_type = elem_type;
  a->ep.rho = rho;
  a->ep.E = E;
  a->ep.nu = nu;
  a->ep.ys = ys;
  a->ep.transform = transform;
  a->ep.ref_axis[0] = 1.0;
  a->ep.ref_axis[1] = a->ep.ref_axis[2] = 0.0;
  if (transform == 1) {
    if (!ref_axis_host) {
      delete a;
      return fail(TG_ERR_ARG, "tg_assembler_create: reference axis missing");
    }
    // TACSShellRefAxisTransform normalises the axis on construction
    double ax[3] = {ref_axis_host[0], ref_axis_host[1], ref_axis_host[2]};
    double nrm = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    double inv = nrm != 0.0 ? 1.0 / nrm : 0.0;
    for (int k = 0; k < 3; k++) a->ep.ref_axis[k] = ax[k] * inv;
  }
  a->nnodes = num_nodes;
  a->nelem = num_elements;
  a->vpn = elem_type == TG_ELEM_MITC4 ? 6 : 3;
  a->npe = elem_type == TG_ELEM_MITC4 ? 4 : 8;
  a->conn_h.assign(conn_host, conn_host + (size_t)a->npe * num_elements);
  for (int c : a->conn_h)
    if (c < 0 || c >= num_nodes) {
      delete a;
      return fail(TG_ERR_ARG, "tg_assembler_create: node index out of range");
    }
  a->thick_h.assign(num_elements, 1.0);
  a->dvnum_h.assign(num_elements, -1);
  *out = a;
  return 0;
}

int tg_assembler_incref(tg_assembler *a) {
  if (!a) return fail(TG_ERR_ARG, "NULL assembler");
  a->refcount++;
  return 0;
}
int tg_assembler_decref(tg_assembler *a) {
  if (!a) return 0;
  if (--a->refcount == 0) delete a;
  return 0;
}

int tg_assembler_get_sizes(tg_assembler *a, int *vpn, int *nnodes,
                           int *nelems, int *ndvs, int *ncolors) {
  if (!a) return fail(TG_ERR_ARG, "NULL assembler");
  if (vpn) *vpn = a->vpn;
  if (nnodes) *nnodes = a->nnodes;
  if (nelems) *nelems = a->nelem;
  if (ndvs) *ndvs = a->ndv;
  if (ncolors) *ncolors = a->initialized ? a->ncolors() : 0;
  return 0;
}

int tg_assembler_add_bcs(tg_assembler *a, int n, const int *nodes,
                         const int *masks) {
  if (!a || n < 0 || (n > 0 && (!nodes || !masks)))
    return fail(TG_ERR_ARG, "tg_assembler_add_bcs: bad arguments");
  if (a->initialized)
    return fail(TG_ERR_STATE, "tg_assembler_add_bcs after initialize");
  for (int i = 0; i < n; i++) {
    if (nodes[i] < 0 || nodes[i] >= a->nnodes)
      return fail(TG_ERR_ARG, "tg_assembler_add_bcs: node out of range");
    // merge with an existing entry for the node (TACSBcMap::addBC)
    bool merged = false;
    for (size_t k = 0; k < a->bc_nodes_h.size(); k++)
      if (a->bc_nodes_h[k] == nodes[i]) {
        a->bc_masks_h[k] |= masks[i];
        merged = true;
        break;
      }
    if (!merged) {
      a->bc_nodes_h.push_back(nodes[i]);
      a->bc_masks_h.push_back(masks[i]);
    }
  }
  return 0;
}

int tg_assembler_set_element_dvs(tg_assembler *a, const double *t,
                                 const int *dvnum) {
  if (!a) return fail(TG_ERR_ARG, "NULL assembler");
  if (t) a->thick_h.assign(t, t + a->nelem);
  if (dvnum) {
    if (a->initialized)
      return fail(TG_ERR_STATE, "design-variable numbers after initialize");
    a->dvnum_h.assign(dvnum, dvnum + a->nelem);
  }
  if (a->initialized && t) {
    cudaError_t e = cudaMemcpy(a->d_thick, a->thick_h.data(),
                               a->nelem * sizeof(double),
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_check(e, "set_element_dvs");
  }
  return 0;
}

int tg_assembler_set_pressure(tg_assembler *a, int n, const int *elems,
                              const double *vals) {
  if (!a || n < 0 || (n > 0 && (!elems || !vals)))
    return fail(TG_ERR_ARG, "tg_assembler_set_pressure: bad arguments");
  if (a->ep.elem_type != TG_ELEM_MITC4)
    return fail(TG_ERR_ARG, "pressure loads are defined for shells");
  if (a->initialized)
    return fail(TG_ERR_STATE, "tg_assembler_set_pressure after initialize");
  a->pres_h.assign((size_t)4 * a->nelem, 0.0);
  for (int k = 0; k < n; k++) {
    if (elems[k] < 0 || elems[k] >= a->nelem)
      return fail(TG_ERR_ARG, "pressure element out of range");
    for (int j = 0; j < 4; j++) a->pres_h[4 * elems[k] + j] += vals[4 * k + j];
  }
  a->has_pres = n > 0;
  return 0;
}

int tg_assembler_set_traction(tg_assembler *a, int n, const int *elems,
                              const int *faces, const double *vals) {
  if (!a || n < 0 || (n > 0 && (!elems || !faces || !vals)))
    return fail(TG_ERR_ARG, "tg_assembler_set_traction: bad arguments");
  if (a->ep.elem_type != TG_ELEM_HEX8)
    return fail(TG_ERR_ARG, "face tractions are defined for hex elements");
  if (a->initialized)
    return fail(TG_ERR_STATE, "tg_assembler_set_traction after initialize");
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return elems[x] < elems[y]; });
  a->trac_ptr_h.assign(a->nelem + 1, 0);
  a->trac_face_h.clear();
  a->trac_val_h.clear();
  for (int k = 0; k < n; k++) {
    if (elems[k] < 0 || elems[k] >= a->nelem || faces[k] < 0 || faces[k] > 5)
      return fail(TG_ERR_ARG, "traction element/face out of range");
    a->trac_ptr_h[elems[k] + 1]++;
  }
  for (int e = 0; e < a->nelem; e++) a->trac_ptr_h[e + 1] += a->trac_ptr_h[e];
  for (int k : order) {
    a->trac_face_h.push_back(faces[k]);
    for (int j = 0; j < 3; j++) a->trac_val_h.push_back(vals[3 * k + j]);
  }
  return 0;
}

// Node-to-node pattern with the diagonal, sorted columns
// (TACSAssembler::createMat / computeLocalNodeToNodeCSR).
static void build_pattern(tg_assembler *a) {
  const int nn = a->nnodes, npe = a->npe;
  std::vector<std::vector<int>> adj(nn);
  for (int i = 0; i < nn; i++) adj[i].push_back(i);
  for (int e = 0; e < a->nelem; e++)
    for (int i = 0; i < npe; i++)
      for (int j = 0; j < npe; j++)
        adj[a->conn_h[npe * e + i]].push_back(a->conn_h[npe * e + j]);
  a->rowp_h.assign(nn + 1, 0);
  a->cols_h.clear();
  a->diag_h.assign(nn, -1);
  for (int i = 0; i < nn; i++) {
    auto &r = adj[i];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    for (int c : r) {
      if (c == i) a->diag_h[i] = (int)a->cols_h.size();
      a->cols_h.push_back(c);
    }
    a->rowp_h[i + 1] = (int)a->cols_h.size();
    std::vector<int>().swap(r);
  }
}

// Greedy element colouring: no two elements of one colour share a node.
static int build_coloring(tg_assembler *a) {
  const int npe = a->npe;
  std::vector<uint64_t> used(a->nnodes, 0);
  std::vector<int> color(a->nelem, 0);
  int ncol = 0;
  for (int e = 0; e < a->nelem; e++) {
    uint64_t m = 0;
    for (int i = 0; i < npe; i++) m |= used[a->conn_h[npe * e + i]];
    int c = 0;
    while (c < 64 && (m >> c) & 1ull) c++;
    if (c >= 64) return fail(TG_ERR_ARG, "element colouring needs > 64 colours");
    color[e] = c;
    ncol = std::max(ncol, c + 1);
    for (int i = 0; i < npe; i++) used[a->conn_h[npe * e + i]] |= (1ull << c);
  }
  a->color_ptr_h.assign(ncol + 1, 0);
  for (int e = 0; e < a->nelem; e++) a->color_ptr_h[color[e] + 1]++;
  for (int c = 0; c < ncol; c++) a->color_ptr_h[c + 1] += a->color_ptr_h[c];
  a->color_elems_h.assign(a->nelem, 0);
  std::vector<int> fill(a->color_ptr_h.begin(), a->color_ptr_h.end() - 1);
  for (int e = 0; e < a->nelem; e++) a->color_elems_h[fill[color[e]]++] = e;
  if (ncol == 0) a->color_ptr_h.assign(1, 0);
  return 0;
}

int tg_assembler_initialize(tg_assembler *a) {
  if (!a) return fail(TG_ERR_ARG, "NULL assembler");
  if (a->initialized) return fail(TG_ERR_STATE, "already initialised");
  build_pattern(a);
  int rc = build_coloring(a);
  if (rc) return rc;
  // design-variable -> elements map (element order)
  a->ndv = 0;
  for (int d : a->dvnum_h) a->ndv = std::max(a->ndv, d + 1);
  std::vector<int> dv_ptr(a->ndv + 1, 0), dv_elems;
  for (int d : a->dvnum_h)
    if (d >= 0) dv_ptr[d + 1]++;
  for (int d = 0; d < a->ndv; d++) dv_ptr[d + 1] += dv_ptr[d];
  dv_elems.assign(dv_ptr[a->ndv], 0);
  {
    std::vector<int> fill(dv_ptr.begin(), dv_ptr.end() - 1);
    for (int e = 0; e < a->nelem; e++)
      if (a->dvnum_h[e] >= 0) dv_elems[fill[a->dvnum_h[e]]++] = e;
  }
  if ((rc = upload(&a->d_conn, a->conn_h))) return rc;
  if ((rc = dalloc(&a->d_xpts, (size_t)3 * a->nnodes))) return rc;
  TG_CUDA(cudaMemset(a->d_xpts, 0, sizeof(double) * 3 * (size_t)a->nnodes));
  if ((rc = upload(&a->d_thick, a->thick_h))) return rc;
  if ((rc = upload(&a->d_dvnum, a->dvnum_h))) return rc;
  if (a->has_pres && (rc = upload(&a->d_pres, a->pres_h))) return rc;
  if (!a->trac_val_h.empty()) {
    if ((rc = upload(&a->d_trac_ptr, a->trac_ptr_h))) return rc;
    if ((rc = upload(&a->d_trac_face, a->trac_face_h))) return rc;
    if ((rc = upload(&a->d_trac_val, a->trac_val_h))) return rc;
  }
  if ((rc = upload(&a->d_bc_nodes, a->bc_nodes_h))) return rc;
  if ((rc = upload(&a->d_bc_masks, a->bc_masks_h))) return rc;
  if ((rc = upload(&a->d_rowp, a->rowp_h))) return rc;
  if ((rc = upload(&a->d_cols, a->cols_h))) return rc;
  if ((rc = upload(&a->d_diag, a->diag_h))) return rc;
  if ((rc = upload(&a->d_color_elems, a->color_elems_h))) return rc;
  if ((rc = upload(&a->d_dv_ptr, dv_ptr))) return rc;
  if ((rc = upload(&a->d_dv_elems, dv_elems))) return rc;
  const size_t nq = (size_t)a->nq() * a->nelem;
  if ((rc = dalloc(&a->d_elem_fail, nq))) return rc;
  if ((rc = dalloc(&a->d_elem_wdet, nq))) return rc;
  if ((rc = dalloc(&a->d_elem_sed, a->nelem))) return rc;
  if ((rc = dalloc(&a->d_elem_val, a->nelem))) return rc;
  if ((rc = dalloc(&a->d_partials, a->npart))) return rc;
  if ((rc = dalloc(&a->d_scalars, 8))) return rc;
  a->initialized = true;
  return 0;
}

int tg_assembler_set_nodes(tg_assembler *a, const double *xpts, void *s) {
  if (!a || !a->initialized)
    return fail(TG_ERR_STATE, "tg_assembler_set_nodes before initialize");
  if (!xpts) return fail(TG_ERR_ARG, "NULL node vector");
  TG_CUDA(cudaMemcpyAsync(a->d_xpts, xpts, sizeof(double) * 3 * a->nnodes,
                          cudaMemcpyDeviceToDevice, S(s)));
  return 0;
}

int tg_assembler_set_design_vars(tg_assembler *a, const double *dvs, void *s) {
  if (!a || !a->initialized)
    return fail(TG_ERR_STATE, "tg_assembler_set_design_vars before initialize");
  if (!dvs) return fail(TG_ERR_ARG, "NULL design vector");
  launch_gather_dv(a->nelem, a->d_dvnum, dvs, a->d_thick, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}

static int check_ready(tg_assembler *a, const char *who) {
  if (!a) return fail(TG_ERR_ARG, std::string(who) + ": NULL assembler");
  if (!a->initialized)
    return fail(TG_ERR_STATE, std::string(who) + ": assembler not initialised");
  return 0;
}

int tg_assemble_res(tg_assembler *a, const double *vars, double lambda,
                    int apply_bcs, double *res, void *s) {
  int rc = check_ready(a, "tg_assemble_res");
  if (rc) return rc;
  if (!res) return fail(TG_ERR_ARG, "tg_assemble_res: NULL residual");
  const size_t n = (size_t)a->vpn * a->nnodes;
  TG_CUDA(cudaMemsetAsync(res, 0, n * sizeof(double), S(s)));
  MeshView m = a->view();
  for (int c = 0; c < a->ncolors(); c++) {
    if (a->ep.elem_type == TG_ELEM_MITC4)
      launch_shell_team_assembly(a->ep, m, a->color(c), vars, lambda, res,
                                 nullptr, nullptr, S(s));
    else
      launch_hex_assembly(a->ep, m, a->color(c), vars, lambda, res, nullptr, 0,
                          S(s));
  }
  if (apply_bcs)
    launch_apply_bcs_res(a->vpn, (int)a->bc_nodes_h.size(), a->d_bc_nodes,
                         a->d_bc_masks, vars, res, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_apply_bcs(tg_assembler *a, double *vec, void *s) {
  int rc = check_ready(a, "tg_apply_bcs");
  if (rc) return rc;
  launch_apply_bcs_res(a->vpn, (int)a->bc_nodes_h.size(), a->d_bc_nodes,
                       a->d_bc_masks, nullptr, vec, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_assemble_jacobian(tg_assembler *a, double alpha, double beta,
                         double gamma, const double *vars, double *res,
                         tg_mat *A, int orient, double lambda, int apply_bcs,
                         void *s) {
  int rc = check_ready(a, "tg_assemble_jacobian");
  if (rc) return rc;
  if (!A || A->a != a)
    return fail(TG_ERR_ARG, "tg_assemble_jacobian: matrix of another assembler");
  if (alpha != 1.0 || beta != 0.0 || gamma != 0.0)
    return fail(TG_ERR_ARG,
                "tg_assemble_jacobian: static elements need alpha=1, beta=gamma=0");
  const size_t n = (size_t)a->vpn * a->nnodes;
  if (res) TG_CUDA(cudaMemsetAsync(res, 0, n * sizeof(double), S(s)));
  TG_CUDA(cudaMemsetAsync(A->d_vals, 0,
                          sizeof(double) * (size_t)A->nnz * A->bsize * A->bsize,
                          S(s)));
  MeshView m = a->view();
  for (int c = 0; c < a->ncolors(); c++) {
    if (a->ep.elem_type == TG_ELEM_MITC4)
      launch_shell_team_assembly(a->ep, m, a->color(c), vars, lambda, res,
                                 A->d_vals, nullptr, S(s));
    else
      launch_hex_assembly(a->ep, m, a->color(c), vars, lambda, res, A->d_vals,
                          orient, S(s));
  }
  if (apply_bcs) {
    if (res)
      launch_apply_bcs_res(a->vpn, (int)a->bc_nodes_h.size(), a->d_bc_nodes,
                           a->d_bc_masks, vars, res, S(s));
    launch_apply_bcs_mat(a->vpn, (int)a->bc_nodes_h.size(), a->d_bc_nodes,
                         a->d_bc_masks, a->d_rowp, a->d_cols, A->d_vals, S(s));
  }
  TG_CUDA(cudaGetLastError());
  return 0;
}

static void launch_points(tg_assembler *a, const double *vars, cudaStream_t s) {
  MeshView m = a->view();
  if (a->ep.elem_type == TG_ELEM_MITC4)
    launch_shell_points(a->ep, m, vars, a->d_elem_fail, a->d_elem_wdet,
                        a->d_elem_sed, s);
  else
    launch_hex_points(a->ep, m, vars, a->d_elem_fail, a->d_elem_wdet,
                      a->d_elem_sed, s);
}

int tg_eval_functions(tg_assembler *a, const double *vars, int nfuncs,
                      const int *funcs, double ks_weight, double *vals,
                      void *s) {
  int rc = check_ready(a, "tg_eval_functions");
  if (rc) return rc;
  if (nfuncs < 0 || (nfuncs > 0 && (!funcs || !vals)) || !vars)
    return fail(TG_ERR_ARG, "tg_eval_functions: bad arguments");
  launch_points(a, vars, S(s));
  const size_t nq = (size_t)a->nq() * a->nelem;
  // d_scalars: [0] compliance, [1] KS max, [2] KS sum
  launch_reduce_sum(a->d_elem_sed, a->nelem, a->d_partials, a->npart,
                    a->d_scalars, S(s));
  launch_reduce_max(a->d_elem_fail, nq, a->d_partials, a->npart,
                    a->d_scalars + 1, S(s));
  launch_ks_sum(a->d_elem_fail, a->d_elem_wdet, nq, a->d_scalars + 1,
                ks_weight, a->d_partials, a->npart, a->d_scalars + 2, S(s));
  double h[3];
  TG_CUDA(cudaMemcpyAsync(h, a->d_scalars, sizeof(h), cudaMemcpyDeviceToHost,
                          S(s)));
  TG_CUDA(cudaStreamSynchronize(S(s)));
  a->ks.max = h[1];
  a->ks.sum = h[2];
  a->ks.weight = ks_weight;
  a->ks_valid = true;
  for (int i = 0; i < nfuncs; i++) {
    if (funcs[i] == TG_FUNC_COMPLIANCE) vals[i] = h[0];
    else if (funcs[i] == TG_FUNC_KS_FAILURE)
      vals[i] = h[1] + std::log(h[2] / 1.0) / ks_weight;
    else return fail(TG_ERR_ARG, "tg_eval_functions: unknown function");
  }
  if (!std::isfinite(h[0]) || !std::isfinite(h[1]) || !std::isfinite(h[2]))
    return fail(TG_ERR_NONFINITE, "tg_eval_functions: non-finite result");
  return 0;
}

int tg_add_sv_sens(tg_assembler *a, const double *vars, int nfuncs,
                   const int *funcs, double alpha, double **dfdu, void *s) {
  int rc = check_ready(a, "tg_add_sv_sens");
  if (rc) return rc;
  if (!vars || nfuncs < 0 || (nfuncs > 0 && (!funcs || !dfdu)))
    return fail(TG_ERR_ARG, "tg_add_sv_sens: bad arguments");
  MeshView m = a->view();
  for (int i = 0; i < nfuncs; i++) {
    if (funcs[i] == TG_FUNC_KS_FAILURE && !a->ks_valid)
      return fail(TG_ERR_STATE,
                  "tg_add_sv_sens: evaluate the KS function first");
    for (int c = 0; c < a->ncolors(); c++) {
      if (a->ep.elem_type == TG_ELEM_MITC4)
        launch_shell_sv_sens(a->ep, m, a->color(c), vars, funcs[i], a->ks,
                             alpha, dfdu[i], S(s));
      else
        launch_hex_sv_sens(a->ep, m, a->color(c), vars, funcs[i], a->ks, alpha,
                           dfdu[i], S(s));
    }
  }
  TG_CUDA(cudaGetLastError());
  return 0;
}

static int elem_dv_pass(tg_assembler *a, const double *vars, int func,
                        double coef, const double *psi, double scale,
                        double *dfdx, cudaStream_t s) {
  MeshView m = a->view();
  if (a->ep.elem_type == TG_ELEM_MITC4)
    launch_shell_dv(a->ep, m, vars, func, a->ks, coef, psi, scale,
                    a->d_elem_val, s);
  else
    launch_hex_dv(a->ep, m, vars, func, a->ks, coef, psi, scale,
                  a->d_elem_val, s);
  launch_scatter_dv(a->ndv, a->d_dv_ptr, a->d_dv_elems, a->d_elem_val, dfdx,
                    s);
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_add_dv_sens(tg_assembler *a, const double *vars, int nfuncs,
                   const int *funcs, double coef, double **dfdx, void *s) {
  int rc = check_ready(a, "tg_add_dv_sens");
  if (rc) return rc;
  if (!vars || nfuncs < 0 || (nfuncs > 0 && (!funcs || !dfdx)))
    return fail(TG_ERR_ARG, "tg_add_dv_sens: bad arguments");
  for (int i = 0; i < nfuncs; i++) {
    if (funcs[i] == TG_FUNC_KS_FAILURE && !a->ks_valid)
      return fail(TG_ERR_STATE, "tg_add_dv_sens: evaluate the KS function first");
    if ((rc = elem_dv_pass(a, vars, funcs[i], coef, nullptr, 0.0, dfdx[i],
                           S(s))))
      return rc;
  }
  return 0;
}

int tg_add_adjoint_res_products(tg_assembler *a, const double *vars,
                                double scale, int nadj, const double **psi,
                                double **dfdx, void *s) {
  int rc = check_ready(a, "tg_add_adjoint_res_products");
  if (rc) return rc;
  if (!vars || nadj < 0 || (nadj > 0 && (!psi || !dfdx)))
    return fail(TG_ERR_ARG, "tg_add_adjoint_res_products: bad arguments");
  for (int k = 0; k < nadj; k++)
    if ((rc = elem_dv_pass(a, vars, -1, 0.0, psi[k], scale, dfdx[k], S(s))))
      return rc;
  return 0;
}

int tg_add_total_derivative(tg_assembler *a, const double *vars, int func,
                            double coef, const double *psi, double scale,
                            double *dfdx, void *s) {
  int rc = check_ready(a, "tg_add_total_derivative");
  if (rc) return rc;
  if (!vars || !dfdx) return fail(TG_ERR_ARG, "tg_add_total_derivative: NULL");
  if (func == TG_FUNC_KS_FAILURE && !a->ks_valid)
    return fail(TG_ERR_STATE, "evaluate the KS function first");
  return elem_dv_pass(a, vars, func, coef, psi, scale, dfdx, S(s));
}

// ------------------------------------------------------------------ BCSR
int tg_mat_create(tg_assembler *a, tg_mat **out) {
  int rc = check_ready(a, "tg_mat_create");
  if (rc) return rc;
  if (!out) return fail(TG_ERR_ARG, "tg_mat_create: out is NULL");
  tg_mat *A = new tg_mat();
  A->a = a;
  a->refcount++;
  A->bsize = a->vpn;
  A->nrows = a->nnodes;
  A->nnz = (int)a->cols_h.size();
  if ((rc = dalloc(&A->d_vals, (size_t)A->nnz * A->bsize * A->bsize))) {
    tg_mat_decref(A);
    return rc;
  }
  cudaMemset(A->d_vals, 0, sizeof(double) * (size_t)A->nnz * A->bsize * A->bsize);
  *out = A;
  return 0;
}
int tg_mat_decref(tg_mat *A) {
  if (!A) return 0;
  if (--A->refcount == 0) {
    tg_assembler_decref(A->a);
    delete A;
  }
  return 0;
}
int tg_mat_get_arrays(tg_mat *A, int *bsize, int *nrows, const int **rowp,
                      const int **cols, double **vals) {
  if (!A) return fail(TG_ERR_ARG, "NULL matrix");
  if (bsize) *bsize = A->bsize;
  if (nrows) *nrows = A->nrows;
  if (rowp) *rowp = A->a->d_rowp;
  if (cols) *cols = A->a->d_cols;
  if (vals) *vals = A->d_vals;
  return 0;
}
int tg_mat_mult(tg_mat *A, const double *x, double *y, void *s) {
  if (!A || !x || !y) return fail(TG_ERR_ARG, "tg_mat_mult: NULL argument");
  launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols, A->d_vals, x,
                   y, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}
static int ensure_f32(tg_mat *A, cudaStream_t s) {
  size_t n = (size_t)A->nnz * A->bsize * A->bsize;
  if (!A->d_vals32) {
    int rc = dalloc(&A->d_vals32, n);
    if (rc) return rc;
  }
  launch_d2f(A->d_vals, A->d_vals32, n, s);
  return 0;
}
int tg_mat_mult_f32(tg_mat *A, const float *x, float *y, void *s) {
  if (!A || !x || !y) return fail(TG_ERR_ARG, "tg_mat_mult_f32: NULL argument");
  if (!A->d_vals32)
    return fail(TG_ERR_STATE, "tg_mat_mult_f32: no FP32 copy (factor a FP32 pc)");
  launch_bcsr_mult_f32(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols,
                       A->d_vals32, x, y, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------- preconditioners
// Level sets of the block lower / upper triangles and the IKJ update list
// of ILU(0) with the pattern of A (BCSRMat(comm, A, levFill = 0, fill),
// src/bpmat/BCSRMat.cpp:138).
static int build_ilu_plan(tg_pc *pc, const std::vector<int> &rowp,
                          const std::vector<int> &cols,
                          const std::vector<int> &diag) {
  const int n = (int)rowp.size() - 1;
  std::vector<int> lvl(n, 0), ulvl(n, 0);
  int nl = 0, nu = 0;
  for (int i = 0; i < n; i++) {
    int L = 0;
    for (int j = rowp[i]; cols[j] < i; j++) L = std::max(L, lvl[cols[j]] + 1);
    lvl[i] = L;
    nl = std::max(nl, L + 1);
  }
  for (int i = n - 1; i >= 0; i--) {
    int L = 0;
    for (int j = diag[i] + 1; j < rowp[i + 1]; j++)
      L = std::max(L, ulvl[cols[j]] + 1);
    ulvl[i] = L;
    nu = std::max(nu, L + 1);
  }
  auto bucket = [&](const std::vector<int> &lv, int nlev, std::vector<int> &ptr,
                    std::vector<int> &rows) {
    ptr.assign(nlev + 1, 0);
    for (int i = 0; i < n; i++) ptr[lv[i] + 1]++;
    for (int L = 0; L < nlev; L++) ptr[L + 1] += ptr[L];
    rows.assign(n, 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < n; i++) rows[fill[lv[i]]++] = i;
  };
  std::vector<int> lrows, urows;
  bucket(lvl, nl, pc->plan.lvl_ptr_h, lrows);
  bucket(ulvl, nu, pc->plan.ulvl_ptr_h, urows);
  // update list per lower entry j of row i: (k, p) with cols[k] == cols[p],
  // p in the strictly-upper part of row cols[j], k > j in row i
  const int nnz = (int)cols.size();
  std::vector<int> upd_ptr(nnz + 1, 0), tgt, src;
  for (int i = 0; i < n; i++) {
    const int row_end = rowp[i + 1];
    for (int j = rowp[i]; j < row_end; j++) {
      if (cols[j] < i) {
        const int cj = cols[j];
        int k = j + 1;
        for (int p = diag[cj] + 1; p < rowp[cj + 1] && k < row_end; p++) {
          while (k < row_end && cols[k] < cols[p]) k++;
          if (k < row_end && cols[k] == cols[p]) {
            tgt.push_back(k);
            src.push_back(p);
          }
        }
      }
      upd_ptr[j + 1] = (int)tgt.size();
    }
  }
  int rc;
  if ((rc = upload(&pc->d_lvl_rows, lrows))) return rc;
  if ((rc = upload(&pc->d_ulvl_rows, urows))) return rc;
  if ((rc = upload(&pc->d_upd_ptr, upd_ptr))) return rc;
  if ((rc = upload(&pc->d_upd_tgt, tgt))) return rc;
  if ((rc = upload(&pc->d_upd_src, src))) return rc;
  return 0;
}

int tg_pc_create(tg_mat *A, int type, int precision, tg_pc **out) {
  if (!A || !out) return fail(TG_ERR_ARG, "tg_pc_create: NULL argument");
  *out = nullptr;
  if (type != TG_PC_ILU0 && type != TG_PC_BLOCK_JACOBI &&
      type != TG_PC_ILU0_COLORED)
    return fail(TG_ERR_ARG, "tg_pc_create: unknown preconditioner type");
  if (precision != TG_PREC_FP64 && precision != TG_PREC_FP32)
    return fail(TG_ERR_ARG, "tg_pc_create: bad precision");
  tg_pc *pc = new tg_pc();
  pc->A = A;
  A->refcount++;
  pc->type = type;
  pc->precision = precision;
  tg_assembler *a = A->a;
  int rc = 0;
  const int *rowp_d = a->d_rowp, *cols_d = a->d_cols, *diag_d = a->d_diag;
  if (type == TG_PC_ILU0) {
    rc = build_ilu_plan(pc, a->rowp_h, a->cols_h, a->diag_h);
  } else if (type == TG_PC_ILU0_COLORED) {
    // greedy colouring of the node graph: nodes of one colour are never
    // neighbours, so with the nodes ordered by colour the ILU(0) factor and
    // both triangular solves proceed one colour at a time
    const int nn = a->nnodes;
    std::vector<int> color(nn, -1);
    int ncol = 0;
    for (int i = 0; i < nn; i++) {
      uint64_t used = 0;
      for (int j = a->rowp_h[i]; j < a->rowp_h[i + 1]; j++) {
        int c = color[a->cols_h[j]];
        if (c >= 0 && c < 64) used |= (1ull << c);
      }
      int c = 0;
      while (c < 64 && ((used >> c) & 1ull)) c++;
      color[i] = c;
      ncol = std::max(ncol, c + 1);
    }
    pc->ncolors = ncol;
    std::vector<int> perm(nn), iperm(nn);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(),
                     [&](int x, int y) { return color[x] < color[y]; });
    for (int r = 0; r < nn; r++) iperm[perm[r]] = r;
    std::vector<int> prowp(nn + 1, 0), pcols, pdiag(nn), valmap;
    pcols.reserve(a->cols_h.size());
    valmap.reserve(a->cols_h.size());
    std::vector<std::pair<int, int>> row;
    for (int r = 0; r < nn; r++) {
      const int o = perm[r];
      row.clear();
      for (int j = a->rowp_h[o]; j < a->rowp_h[o + 1]; j++)
        row.push_back({iperm[a->cols_h[j]], j});
      std::sort(row.begin(), row.end());
      for (auto &e : row) {
        if (e.first == r) pdiag[r] = (int)pcols.size();
        pcols.push_back(e.first);
        valmap.push_back(e.second);
      }
      prowp[r + 1] = (int)pcols.size();
    }
    rc = build_ilu_plan(pc, prowp, pcols, pdiag);
    if (!rc) rc = upload(&pc->d_prowp, prowp);
    if (!rc) rc = upload(&pc->d_pcols, pcols);
    if (!rc) rc = upload(&pc->d_pdiag, pdiag);
    if (!rc) rc = upload(&pc->d_valmap, valmap);
    if (!rc) rc = upload(&pc->d_perm, perm);
    rowp_d = pc->d_prowp;
    cols_d = pc->d_pcols;
    diag_d = pc->d_pdiag;
  }
  const size_t nv = (size_t)A->nnz * A->bsize * A->bsize;
  const size_t n = (size_t)A->nrows * A->bsize;
  if (!rc) rc = dalloc(&pc->d_fail, 1);
  if (!rc) rc = dalloc(&pc->d_F, nv);
  if (!rc) rc = dalloc(&pc->d_tmp, n);
  if (!rc && type == TG_PC_ILU0_COLORED) {
    rc = dalloc(&pc->d_px, n);
    if (!rc) rc = dalloc(&pc->d_py, n);
    if (!rc && precision == TG_PREC_FP32) rc = dalloc(&pc->d_px32, n);
    if (!rc && precision == TG_PREC_FP32) rc = dalloc(&pc->d_py32, n);
  }
  if (!rc) rc = dalloc(&pc->d_gx, n);
  if (!rc) rc = dalloc(&pc->d_gy, n);
  if (!rc && precision == TG_PREC_FP32) {
    rc = dalloc(&pc->d_F32, nv);
    if (!rc) rc = dalloc(&pc->d_x32, n);
    if (!rc) rc = dalloc(&pc->d_y32, n);
    if (!rc) rc = dalloc(&pc->d_tmp32, n);
  }
  if (rc) {
    tg_pc_decref(pc);
    return rc;
  }
  IluPlan &p = pc->plan;
  p.bsize = A->bsize;
  p.nrows = A->nrows;
  p.rowp = rowp_d;
  p.cols = cols_d;
  p.diag = diag_d;
  p.lvl_rows = pc->d_lvl_rows;
  p.ulvl_rows = pc->d_ulvl_rows;
  p.upd_ptr = pc->d_upd_ptr;
  p.upd_tgt = pc->d_upd_tgt;
  p.upd_src = pc->d_upd_src;
  p.d_fail = pc->d_fail;
  *out = pc;
  return 0;
}
int tg_pc_decref(tg_pc *pc) {
  if (!pc) return 0;
  if (--pc->refcount == 0) {
    tg_mat_decref(pc->A);
    delete pc;
  }
  return 0;
}

int tg_pc_factor(tg_pc *pc, void *s) {
  if (!pc) return fail(TG_ERR_ARG, "tg_pc_factor: NULL pc");
  tg_mat *A = pc->A;
  const size_t nv = (size_t)A->nnz * A->bsize * A->bsize;
  TG_CUDA(cudaMemsetAsync(pc->d_fail, 0, sizeof(int), S(s)));
  if (pc->type == TG_PC_ILU0_COLORED) {
    const int nl = (int)pc->plan.lvl_ptr_h.size() - 1;
    const int b2 = A->bsize * A->bsize;
    if (pc->precision == TG_PREC_FP64) {
      launch_gather_blocks(A->nnz, b2, pc->d_valmap, A->d_vals, pc->d_F, S(s));
      for (int L = 0; L < nl; L++)
        launch_ilu0_factor_level(pc->plan, L, pc->d_F, S(s));
    } else {
      launch_gather_blocks_f32(A->nnz, b2, pc->d_valmap, A->d_vals, pc->d_F32,
                               S(s));
      for (int L = 0; L < nl; L++)
        launch_ilu0_factor_level_f32(pc->plan, L, pc->d_F32, S(s));
      int rc = ensure_f32(A, S(s));
      if (rc) return rc;
    }
  } else if (pc->type == TG_PC_ILU0) {
    const int nl = (int)pc->plan.lvl_ptr_h.size() - 1;
    if (pc->precision == TG_PREC_FP64) {
      TG_CUDA(cudaMemcpyAsync(pc->d_F, A->d_vals, nv * sizeof(double),
                              cudaMemcpyDeviceToDevice, S(s)));
      for (int L = 0; L < nl; L++)
        launch_ilu0_factor_level(pc->plan, L, pc->d_F, S(s));
    } else {
      launch_d2f(A->d_vals, pc->d_F32, nv, S(s));
      for (int L = 0; L < nl; L++)
        launch_ilu0_factor_level_f32(pc->plan, L, pc->d_F32, S(s));
      int rc = ensure_f32(A, S(s));
      if (rc) return rc;
    }
  } else {
    TG_CUDA(cudaMemcpyAsync(pc->d_F, A->d_vals, nv * sizeof(double),
                            cudaMemcpyDeviceToDevice, S(s)));
    launch_block_inverse_diag(pc->plan, pc->d_F, S(s));
    if (pc->precision == TG_PREC_FP32) {
      launch_d2f(pc->d_F, pc->d_F32, nv, S(s));
      int rc = ensure_f32(A, S(s));
      if (rc) return rc;
    }
  }
  int hfail = 0;
  TG_CUDA(cudaMemcpyAsync(&hfail, pc->d_fail, sizeof(int),
                          cudaMemcpyDeviceToHost, S(s)));
  TG_CUDA(cudaStreamSynchronize(S(s)));
  TG_CUDA(cudaGetLastError());
  if (hfail) {
    char buf[128];
    snprintf(buf, sizeof(buf),
             "tg_pc_factor: singular diagonal block in row %d", hfail - 1);
    return fail(TG_ERR_PIVOT, buf);
  }
  pc->factored = true;
  return 0;
}

// Apply the factored preconditioner to the pc's internal input buffer
// (d_gx, or d_x32 in FP32) into its output buffer (d_gy / d_y32).  The ILU(0)
// level sequence (2 x number of levels launches) is captured once into a
// CUDA graph and replayed.
static int pc_apply_internal(tg_pc *pc, cudaStream_t s) {
  if (pc->type == TG_PC_BLOCK_JACOBI) {
    if (pc->precision == TG_PREC_FP64)
      launch_block_jacobi_apply(pc->plan, pc->d_F, pc->d_gx, pc->d_gy, s);
    else
      launch_block_jacobi_apply_f32(pc->plan, pc->d_F32, pc->d_x32, pc->d_y32,
                                    s);
    return 0;
  }
  if (!pc->apply_exec) {
    cudaStream_t cs;
    TG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
      const int bs = pc->A->bsize, nr = pc->A->nrows;
      if (pc->type == TG_PC_ILU0_COLORED) {
        if (pc->precision == TG_PREC_FP64) {
          launch_permute_gather(nr, bs, pc->d_perm, pc->d_gx, pc->d_px, cs);
          launch_ilu0_apply(pc->plan, pc->d_F, pc->d_px, pc->d_py, pc->d_tmp,
                            cs);
          launch_permute_scatter(nr, bs, pc->d_perm, pc->d_py, pc->d_gy, cs);
        } else {
          launch_permute_gather_f32(nr, bs, pc->d_perm, pc->d_x32, pc->d_px32,
                                    cs);
          launch_ilu0_apply_f32(pc->plan, pc->d_F32, pc->d_px32, pc->d_py32,
                                pc->d_tmp32, cs);
          launch_permute_scatter_f32(nr, bs, pc->d_perm, pc->d_py32,
                                     pc->d_y32, cs);
        }
      } else if (pc->precision == TG_PREC_FP64) {
        launch_ilu0_apply(pc->plan, pc->d_F, pc->d_gx, pc->d_gy, pc->d_tmp, cs);
      } else {
        launch_ilu0_apply_f32(pc->plan, pc->d_F32, pc->d_x32, pc->d_y32,
                              pc->d_tmp32, cs);
      }
      e = cudaStreamEndCapture(cs, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&pc->apply_exec, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return cuda_check(e, "ILU(0) apply graph capture");
  }
  TG_CUDA(cudaGraphLaunch(pc->apply_exec, s));
  return 0;
}

int tg_pc_apply(tg_pc *pc, const double *x, double *y, void *s) {
  if (!pc || !x || !y) return fail(TG_ERR_ARG, "tg_pc_apply: NULL argument");
  if (!pc->factored) return fail(TG_ERR_STATE, "tg_pc_apply before factor");
  const size_t n = (size_t)pc->A->nrows * pc->A->bsize;
  int rc;
  if (pc->precision == TG_PREC_FP64) {
    TG_CUDA(cudaMemcpyAsync(pc->d_gx, x, n * sizeof(double),
                            cudaMemcpyDeviceToDevice, S(s)));
    if ((rc = pc_apply_internal(pc, S(s)))) return rc;
    TG_CUDA(cudaMemcpyAsync(y, pc->d_gy, n * sizeof(double),
                            cudaMemcpyDeviceToDevice, S(s)));
  } else {
    launch_d2f(x, pc->d_x32, n, S(s));
    if ((rc = pc_apply_internal(pc, S(s)))) return rc;
    launch_f2d(pc->d_y32, y, n, S(s));
  }
  TG_CUDA(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------- KSM
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
  int rc = dalloc(&k->d_W, k->n * (m + 1));
  if (!rc) rc = dalloc(&k->d_work, k->n);
  if (!rc) rc = dalloc(&k->d_work2, k->n);
  if (!rc) rc = dalloc(&k->d_h, m + 2);
  if (!rc) rc = dalloc(&k->d_h2, m + 2);
  if (!rc) rc = dalloc(&k->d_partials, (size_t)k->npart * (m + 2));
  if (!rc) rc = dalloc(&k->d_r, k->n);
  if (!rc) rc = dalloc(&k->d_d, k->n);
  if (!rc && mixed) {
    rc = dalloc(&k->d_v32, k->n);
    if (!rc) rc = dalloc(&k->d_z32, k->n);
    if (!rc) rc = dalloc(&k->d_w32, k->n);
  }
  if (rc) {
    tg_ksm_decref(k);
    return rc;
  }
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
  return 0;
}

// || x ||_2 via the dots kernel (device), returned on the host
static int dnorm(tg_ksm *k, const double *x, double *out, cudaStream_t s) {
  launch_dots(x, k->n, 1, x, k->d_partials, k->npart, k->d_h2, s);
  double v;
  TG_CUDA(cudaMemcpyAsync(&v, k->d_h2, sizeof(double), cudaMemcpyDeviceToHost,
                          s));
  TG_CUDA(cudaStreamSynchronize(s));
  *out = std::sqrt(v);
  return 0;
}

// op(v) = A M^{-1} v, with M^{-1} v kept in z (FP64 or through FP32)
static int apply_op(tg_ksm *k, const double *v, double *z, double *w,
                    cudaStream_t s) {
  tg_mat *A = k->A;
  if (k->mixed) {
    tg_pc *pc = k->pc;
    launch_d2f(v, pc->d_x32, k->n, s);
    int rc = pc_apply_internal(pc, s);
    if (rc) return rc;
    launch_bcsr_mult_f32(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols,
                         A->d_vals32, pc->d_y32, k->d_w32, s);
    launch_f2d(k->d_w32, w, k->n, s);
    if (z) launch_f2d(pc->d_y32, z, k->n, s);
    return 0;
  }
  const double *src = v;
  if (k->pc) {
    int rc = tg_pc_apply(k->pc, v, z, s);
    if (rc) return rc;
    src = z;
  }
  launch_bcsr_mult(A->bsize, A->nrows, A->a->d_rowp, A->a->d_cols, A->d_vals,
                   src, w, s);
  return 0;
}

// One restarted-GMRES solve of A x = b (GMRES::solve, src/bpmat/KSM.cpp:785-
// 970): right preconditioning, Givens rotations, convergence on the
// estimated residual relative to the first cycle's initial residual.  The
// Arnoldi step orthogonalises with two classical Gram-Schmidt passes
// (batched dot products and one update each), which agrees with the
// reference's modified Gram-Schmidt to rounding.
static int gmres_core(tg_ksm *k, const double *b, double *x, int zero_guess,
                      double rtol, double atol, int max_cycles, int *iters,
                      double *resnorm, cudaStream_t s) {
  const int m = k->m;
  const size_t n = k->n;
  double *W = k->d_W;
  std::vector<double> H((size_t)(m + 1) * m, 0.0), res(m + 1, 0.0),
      Qc(m, 0.0), Qs(m, 0.0), h(m + 2), h2(m + 2);
  double rhs_norm = 0.0, rn = 0.0;
  int flag = 0, total = 0;
  for (int count = 0; count < max_cycles; count++) {
    if (zero_guess && count == 0) {
      TG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
      launch_copy(b, W, n, s);
      int rc = dnorm(k, W, &res[0], s);
      if (rc) return rc;
      if (res[0] > 0) launch_scale(1.0 / res[0], W, n, s);
    } else {
      launch_bcsr_mult(k->A->bsize, k->A->nrows, k->A->a->d_rowp,
                       k->A->a->d_cols, k->A->d_vals, x, W, s);
      launch_axpy(-1.0, b, W, n, s);
      int rc = dnorm(k, W, &res[0], s);
      if (rc) return rc;
      if (res[0] > 0) launch_scale(-1.0 / res[0], W, n, s);
    }
    if (count == 0) rhs_norm = res[0];
    rn = res[0];
    int niters = 0;
    if (res[0] < atol || res[0] == 0.0) {
      flag = 1;
      break;
    }
    for (int i = 0; i < m; i++) {
      double *Wi = W + n * i, *Wn = W + n * (i + 1);
      int rc = apply_op(k, Wi, k->d_work, Wn, s);
      if (rc) return rc;
      // CGS2: h = W^T w; w -= W h; twice
      launch_dots(W, n, i + 1, Wn, k->d_partials, k->npart, k->d_h, s);
      launch_gemv_sub(W, n, i + 1, k->d_h, Wn, n, s);
      launch_dots(W, n, i + 1, Wn, k->d_partials, k->npart, k->d_h2, s);
      launch_gemv_sub(W, n, i + 1, k->d_h2, Wn, n, s);
      TG_CUDA(cudaMemcpyAsync(h.data(), k->d_h, sizeof(double) * (i + 1),
                              cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaMemcpyAsync(h2.data(), k->d_h2, sizeof(double) * (i + 1),
                              cudaMemcpyDeviceToHost, s));
      double nrm;
      rc = dnorm(k, Wn, &nrm, s);  // synchronises
      if (rc) return rc;
      double *Hc = &H[(size_t)(m + 1) * i];
      for (int j = 0; j <= i; j++) Hc[j] = h[j] + h2[j];
      Hc[i + 1] = nrm;
      if (nrm > 0) launch_scale(1.0 / nrm, Wn, n, s);
      for (int j = 0; j < i; j++) {
        double h1 = Hc[j], hh = Hc[j + 1];
        Hc[j] = h1 * Qc[j] + hh * Qs[j];
        Hc[j + 1] = -h1 * Qs[j] + hh * Qc[j];
      }
      double h1 = Hc[i], hh = Hc[i + 1];
      double sq = std::sqrt(h1 * h1 + hh * hh);
      Qc[i] = h1 / sq;
      Qs[i] = hh / sq;
      Hc[i] = h1 * Qc[i] + hh * Qs[i];
      Hc[i + 1] = -h1 * Qs[i] + hh * Qc[i];
      h1 = res[i];
      res[i] = h1 * Qc[i];
      res[i + 1] = -h1 * Qs[i];
      niters++;
      rn = std::fabs(res[i + 1]);
      if (!std::isfinite(rn))
        return fail(TG_ERR_NONFINITE, "GMRES: non-finite residual estimate");
      if (rn < atol || rn < rtol * rhs_norm) {
        flag = 1;
        break;
      }
    }
    total += niters;
    for (int i = niters - 1; i >= 0; i--) {
      for (int j = i + 1; j < niters; j++)
        res[i] = res[i] - H[(size_t)(m + 1) * j + i] * res[j];
      res[i] = res[i] / H[(size_t)(m + 1) * i + i];
    }
    // x += M^{-1} (sum_i res_i W_i)
    TG_CUDA(cudaMemcpyAsync(k->d_h, res.data(), sizeof(double) * niters,
                            cudaMemcpyHostToDevice, s));
    TG_CUDA(cudaMemsetAsync(k->d_work, 0, n * sizeof(double), s));
    launch_scale(-1.0, k->d_h, niters, s);
    launch_gemv_sub(W, n, niters, k->d_h, k->d_work, n, s);
    if (k->mixed) {
      tg_pc *pc = k->pc;
      launch_d2f(k->d_work, pc->d_x32, n, s);
      int rc = pc_apply_internal(pc, s);
      if (rc) return rc;
      launch_f2d(pc->d_y32, k->d_work2, n, s);
      launch_axpy(1.0, k->d_work2, x, n, s);
    } else if (k->pc) {
      int rc = tg_pc_apply(k->pc, k->d_work, k->d_work2, s);
      if (rc) return rc;
      launch_axpy(1.0, k->d_work2, x, n, s);
    } else {
      launch_axpy(1.0, k->d_work, x, n, s);
    }
    if (flag) break;
  }
  if (iters) *iters += total;
  if (resnorm) *resnorm = rn;
  TG_CUDA(cudaGetLastError());
  return flag;
}

static int ksm_solve_impl(tg_ksm *k, const double *b, double *x,
                          int zero_guess, int *iters, double *resnorm,
                          cudaStream_t s);

int tg_ksm_solve(tg_ksm *k, const double *b, double *x, int zero_guess,
                 int *iters, double *resnorm, void *sv) {
  if (!k || !b || !x) return fail(TG_ERR_ARG, "tg_ksm_solve: NULL argument");
  return ksm_solve_impl(k, b, x, zero_guess, iters, resnorm, S(sv));
}

static int ksm_solve_impl(tg_ksm *k, const double *b, double *x,
                          int zero_guess, int *iters, double *resnorm,
                          cudaStream_t s) {
  if (iters) *iters = 0;
  if (!k->mixed)
    return gmres_core(k, b, x, zero_guess, k->rtol, k->atol, k->nrestart + 1,
                      iters, resnorm, s);
  // Mixed precision: FP64 iterative refinement on the true residual around
  // GMRES cycles whose preconditioner and mat-vec run in FP32.
  const size_t n = k->n;
  double bnorm;
  int rc = dnorm(k, b, &bnorm, s);
  if (rc) return rc;
  if (zero_guess) TG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
  // Each inner solve runs restarted GMRES with the FP32 operator to a
  // relative 1e-6 (or its restart limit); the FP64 true residual then
  // drives the next correction.  Stops when the true residual meets rtol,
  // or when a correction no longer reduces it (stagnation).
  const int max_outer = 20;
  double rn = bnorm, prev = 0.0;
  for (int outer = 0; outer <= max_outer; outer++) {
    // r = b - A x in FP64
    launch_bcsr_mult(k->A->bsize, k->A->nrows, k->A->a->d_rowp,
                     k->A->a->d_cols, k->A->d_vals, x, k->d_r, s);
    launch_scale(-1.0, k->d_r, n, s);
    launch_axpy(1.0, b, k->d_r, n, s);
    rc = dnorm(k, k->d_r, &rn, s);
    if (rc) return rc;
    if (resnorm) *resnorm = rn;
    if (!std::isfinite(rn))
      return fail(TG_ERR_NONFINITE, "mixed GMRES: non-finite true residual");
    if (rn <= k->rtol * bnorm || rn < k->atol) return 1;
    if (outer > 0 && rn > 0.5 * prev) return 0;  // stagnated
    if (outer == max_outer) break;
    prev = rn;
    int it = 0;
    const double inner = std::max(1e-6, 0.1 * k->rtol * bnorm / rn);
    rc = gmres_core(k, k->d_r, k->d_d, 1, inner, 0.0, k->nrestart + 1, &it,
                    nullptr, s);
    if (rc < 0) return rc;
    if (iters) *iters += it;
    launch_axpy(1.0, k->d_d, x, n, s);
  }
  return 0;
}

}  // extern "C"
