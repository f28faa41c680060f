// Host runtime of libtacs_gb300: the C ABI declared in include/tacs_gb300.h.
// Owns the device data of assemblers, BCSR matrices, preconditioners and
// Krylov solvers, builds the host-side plans (BCSR pattern, element
// colouring, ILU level sets and update lists, design-variable maps) and
// sequences the sm_103a kernels on the caller's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <numeric>
#include <string>
#include <vector>

#include "mesh_graph.h"
#include "geo_plan.h"
#include "tg_objects.h"

namespace tg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_check(cudaError_t e, const char *what) {
  set_error(std::string("CUDA error in ") + what + ": " +
            cudaGetErrorString(e));
  return TG_ERR_CUDA;
}

}  // namespace tg


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
  for (int i = 0; i < n; i++)  // validate before changing anything
    if (nodes[i] < 0 || nodes[i] >= a->nnodes)
      return fail(TG_ERR_ARG, "tg_assembler_add_bcs: node out of range");
  for (int i = 0; i < n; i++) {
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
  if (dvnum && a->initialized)
    return fail(TG_ERR_STATE, "design-variable numbers after initialize");
  if (t) a->thick_h.assign(t, t + a->nelem);
  if (dvnum) a->dvnum_h.assign(dvnum, dvnum + a->nelem);
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
  for (int k = 0; k < n; k++)  // validate before changing anything
    if (elems[k] < 0 || elems[k] >= a->nelem)
      return fail(TG_ERR_ARG, "pressure element out of range");
  a->pres_h.assign((size_t)4 * a->nelem, 0.0);
  for (int k = 0; k < n; k++)
    for (int j = 0; j < 4; j++) a->pres_h[4 * elems[k] + j] += vals[4 * k + j];
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
  for (int k = 0; k < n; k++)  // validate before changing anything
    if (elems[k] < 0 || elems[k] >= a->nelem || faces[k] < 0 || faces[k] > 5)
      return fail(TG_ERR_ARG, "traction element/face out of range");
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return elems[x] < elems[y]; });
  a->trac_ptr_h.assign(a->nelem + 1, 0);
  a->trac_face_h.clear();
  a->trac_val_h.clear();
  for (int k = 0; k < n; k++) a->trac_ptr_h[elems[k] + 1]++;
  for (int e = 0; e < a->nelem; e++) a->trac_ptr_h[e + 1] += a->trac_ptr_h[e];
  for (int k : order) {
    a->trac_face_h.push_back(faces[k]);
    for (int j = 0; j < 3; j++) a->trac_val_h.push_back(vals[3 * k + j]);
  }
  return 0;
}

// Element colouring (mesh_graph.h): no two elements of one colour share a
// node; the colours' element lists in element order.
static void build_coloring(tg_assembler *a) {
  std::vector<int> color;
  const int ncol = graph::color_elements(a->nnodes, a->npe, a->nelem,
                                         a->conn_h.data(), color);
  a->color_ptr_h.assign(ncol + 1, 0);
  for (int e = 0; e < a->nelem; e++) a->color_ptr_h[color[e] + 1]++;
  for (int c = 0; c < ncol; c++) a->color_ptr_h[c + 1] += a->color_ptr_h[c];
  a->color_elems_h.assign(a->nelem, 0);
  std::vector<int> fill(a->color_ptr_h.begin(), a->color_ptr_h.end() - 1);
  for (int e = 0; e < a->nelem; e++) a->color_elems_h[fill[color[e]]++] = e;
}
int tg_assembler_initialize(tg_assembler *a) {
  if (!a) return fail(TG_ERR_ARG, "NULL assembler");
  if (a->initialized) return fail(TG_ERR_STATE, "already initialised");
  graph::node_pattern(a->nnodes, a->npe, a->nelem, a->conn_h.data(),
                      a->rowp_h, a->cols_h, a->diag_h);
  build_coloring(a);
  int rc = 0;
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
  if (a->ep.elem_type == TG_ELEM_MITC4) {
    std::vector<uint32_t> first;
    if (graph::first_writers(a->nnodes, a->nelem, a->conn_h.data(),
                             a->rowp_h, a->cols_h, a->color_ptr_h,
                             a->color_elems_h, first)) {
      std::vector<unsigned> fu(first.begin(), first.end());
      if ((rc = upload(&a->d_first, fu))) return rc;
    }
  }
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
  a->geo_table_valid = false;  // new geometry: classes, table and loads
  return 0;
}

// ------------------------------------------------ fixed-geometry assembly
// The plan (contribution lists, row schedule, node constraint masks) once
// per assembler; the geometry classes, their coefficient table and the
// loads f0 = R(u = 0, lambda = 1) once per node set.
static int geo_prepare(tg_assembler *a, cudaStream_t s) {
  const bool shell = a->ep.elem_type == TG_ELEM_MITC4;
  const int bs = a->vpn, npe = a->npe, ncoef = shell ? 2 : 1;
  int rc = 0;
  if (!a->geo_plan_ready) {
    std::vector<int> cptr, contrib, kmax, node_bc;
    if (geo::contributions(a->nelem, npe, a->conn_h.data(), a->rowp_h,
                           a->cols_h, cptr, contrib))
      return fail(TG_ERR_ARG, "fixed geometry: more than 2^25 elements");
    geo::warp_row_lengths(a->rowp_h, kmax);
    geo::node_bc_masks(a->nnodes, a->bc_nodes_h, a->bc_masks_h, node_bc);
    if ((rc = upload(&a->d_geo_cptr, cptr))) return rc;
    if ((rc = upload(&a->d_geo_contrib, contrib))) return rc;
    if ((rc = upload(&a->d_geo_kmax, kmax))) return rc;
    if ((rc = upload(&a->d_geo_node_bc, node_bc))) return rc;
    if ((rc = dalloc(&a->d_geo_f0, (size_t)bs * a->nnodes))) return rc;
    if ((rc = dalloc(&a->d_geo_masks, 2))) return rc;
    a->geo_nwarps = (int)kmax.size();
    a->geo_plan_bytes = sizeof(int) * (cptr.size() + contrib.size() +
                                       kmax.size() + node_bc.size());
    a->geo_plan_ready = true;
  }
  if (!a->geo_table_valid) {
    std::vector<double> x((size_t)3 * a->nnodes);
    TG_CUDA(cudaMemcpyAsync(x.data(), a->d_xpts, x.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    std::vector<int> cls, reps;
    const int ncls = geo::geometry_classes(a->nelem, npe, a->conn_h.data(),
                                           x.data(), cls, reps);
    dfree(a->d_geo_cls);
    dfree(a->d_geo_reps);
    if ((rc = upload(&a->d_geo_cls, cls))) return rc;
    if ((rc = upload(&a->d_geo_reps, reps))) return rc;
    const size_t per = (size_t)ncoef * npe * npe * bs * bs;
    if ((size_t)ncls * per > a->geo_table_doubles) {
      dfree(a->d_geo_table);
      if ((rc = dalloc(&a->d_geo_table, (size_t)ncls * per))) return rc;
      a->geo_table_doubles = (size_t)ncls * per;
    }
    MeshView m = a->view();
    m.geo_B = nullptr;  // the build forms B itself
    if (shell) {
      dfree(a->d_geo_B);
      if ((rc = dalloc(&a->d_geo_B, (size_t)ncls * 868))) return rc;
      launch_shell_geo_build(a->ep, m, a->d_geo_reps, ncls, a->d_geo_table,
                             a->d_geo_B, s);
    }
    if (!shell)
      launch_hex_geo_build(a->ep, m, a->d_geo_reps, ncls, a->d_geo_table, s);
    TG_CUDA(cudaMemsetAsync(a->d_geo_masks, 0, 2 * sizeof(unsigned long long),
                            s));
    launch_geo_masks(bs, ncoef, npe * npe, ncls, a->d_geo_table,
                     a->d_geo_masks, s);
    TG_CUDA(cudaMemcpyAsync(a->geo_mask, a->d_geo_masks,
                            2 * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s));
    // loads: the residual at u = 0 without constraints (t does not enter)
    const size_t n = (size_t)bs * a->nnodes;
    TG_CUDA(cudaMemsetAsync(a->d_geo_f0, 0, n * sizeof(double), s));
    for (int c = 0; c < a->ncolors(); c++) {
      if (shell)
        launch_shell_team_assembly(a->ep, m, a->color(c), nullptr, 1.0,
                                   a->d_geo_f0, nullptr, nullptr, s);
      else
        launch_hex_assembly(a->ep, m, a->color(c), nullptr, 1.0, a->d_geo_f0,
                            nullptr, 0, s);
    }
    TG_CUDA(cudaStreamSynchronize(s));
    TG_CUDA(cudaGetLastError());
    a->geo_ncls = ncls;
    a->geo_table_valid = true;
  }
  return 0;
}

static GeoView geo_view(const tg_assembler *a) {
  GeoView g;
  g.nrows = a->nnodes;
  g.nwarps = a->geo_nwarps;
  g.rowp = a->d_rowp;
  g.cols = a->d_cols;
  g.cptr = a->d_geo_cptr;
  g.contrib = a->d_geo_contrib;
  g.cls = a->d_geo_cls;
  g.node_bc = a->d_geo_node_bc;
  g.warp_kmax = a->d_geo_kmax;
  g.thick = a->d_thick;
  g.table = a->d_geo_table;
  g.f0 = a->d_geo_f0;
  g.mask1 = a->geo_mask[0];
  g.mask3 = a->geo_mask[1];
  return g;
}

int tg_assembler_set_fixed_geometry(tg_assembler *a, int enable) {
  if (!a || !a->initialized)
    return fail(TG_ERR_STATE, "tg_assembler_set_fixed_geometry before "
                              "initialize");
  a->geo_enabled = enable != 0;
  return 0;
}

int tg_assembler_get_fixed_geometry(tg_assembler *a, int *nclasses,
                                    double *table_bytes, double *plan_bytes) {
  if (!a) return fail(TG_ERR_ARG, "NULL assembler");
  if (nclasses) *nclasses = a->geo_table_valid ? a->geo_ncls : 0;
  if (table_bytes)
    *table_bytes = a->geo_table_valid
                       ? (double)a->geo_ncls * (a->ep.elem_type == TG_ELEM_MITC4
                                                    ? 2 * 16 * 36
                                                    : 64 * 9) * 8.0
                       : 0.0;
  if (plan_bytes) *plan_bytes = (double)a->geo_plan_bytes;
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
  if (a->geo_enabled) {
    if ((rc = geo_prepare(a, S(s)))) return rc;
    launch_geo_assembly(a->vpn, geo_view(a), vars, lambda, apply_bcs, res,
                        nullptr, S(s));
    TG_CUDA(cudaGetLastError());
    return 0;
  }
  MeshView m = a->view();
  // the shell kernels store what they write first (no zero fill)
  const bool first = m.first && a->ep.elem_type == TG_ELEM_MITC4;
  if (!first) TG_CUDA(cudaMemsetAsync(res, 0, n * sizeof(double), S(s)));
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

// ---------------------------------------------------------------- vectors
int tg_vec_axpy(double alpha, const double *x, double *y, long n, void *s) {
  if ((!x || !y) && n > 0) return fail(TG_ERR_ARG, "tg_vec_axpy: NULL");
  launch_axpy(alpha, x, y, (size_t)n, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}
int tg_vec_scale(double alpha, double *x, long n, void *s) {
  if (!x && n > 0) return fail(TG_ERR_ARG, "tg_vec_scale: NULL");
  launch_scale(alpha, x, (size_t)n, S(s));
  TG_CUDA(cudaGetLastError());
  return 0;
}
int tg_vec_dot(const double *x, const double *y, long n, double *out,
               void *s) {
  if (!x || !y || !out) return fail(TG_ERR_ARG, "tg_vec_dot: NULL");
  // reduction scratch, allocated once per device (calls on one device
  // share it, so concurrent dot products on two streams must be ordered)
  constexpr int kParts = 1024;
  static double *scratch[64] = {nullptr};
  int dev = 0;
  TG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(TG_ERR_ARG, "tg_vec_dot: device id");
  if (!scratch[dev]) {
    int rc = dalloc(&scratch[dev], kParts + 1);
    if (rc) return rc;
  }
  launch_dots(x, (size_t)n, 1, y, scratch[dev], kParts, scratch[dev] + kParts,
              S(s));
  TG_CUDA(cudaMemcpyAsync(out, scratch[dev] + kParts, sizeof(double),
                          cudaMemcpyDeviceToHost, S(s)));
  TG_CUDA(cudaStreamSynchronize(S(s)));
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
  if (a->geo_enabled) {
    // element matrices are symmetric: the transpose assembly is the same
    if ((rc = geo_prepare(a, S(s)))) return rc;
    launch_geo_assembly(a->vpn, geo_view(a), vars, lambda, apply_bcs, res,
                        A->d_vals, S(s));
    TG_CUDA(cudaGetLastError());
    return 0;
  }
  MeshView m = a->view();
  // the shell kernels store what they write first (no zero fill)
  const bool first = m.first && a->ep.elem_type == TG_ELEM_MITC4;
  if (!first) {
    if (res) TG_CUDA(cudaMemsetAsync(res, 0, n * sizeof(double), S(s)));
    TG_CUDA(cudaMemsetAsync(
        A->d_vals, 0, sizeof(double) * (size_t)A->nnz * A->bsize * A->bsize,
        S(s)));
  }
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
  // fixed-geometry mode: the class table (and the shells' strain operators)
  // serve the function and sensitivity kernels too
  if (a->geo_enabled && (rc = geo_prepare(a, S(s)))) return rc;
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
      vals[i] = h[1] + std::log(h[2]) / ks_weight;
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

static int elem_dv_pass_view(tg_assembler *a, const MeshView &m,
                             const double *vars, int func, double coef,
                             const double *psi, double scale, double *dfdx,
                             cudaStream_t s) {
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
static int elem_dv_pass(tg_assembler *a, const double *vars, int func,
                        double coef, const double *psi, double scale,
                        double *dfdx, cudaStream_t s) {
  return elem_dv_pass_view(a, a->view(), vars, func, coef, psi, scale, dfdx,
                           s);
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

// ------------------------------------------ node-coordinate sensitivities
static int xpt_pass(tg_assembler *a, const double *vars, int func, double coef,
                    const double *psi, double scale, double lambda,
                    double *dfdX, cudaStream_t s) {
  const MeshView m = a->view();
  for (int c = 0; c < a->ncolors(); c++) {
    if (a->ep.elem_type == TG_ELEM_MITC4)
      launch_shell_xpt(a->ep, m, a->color(c), vars, func, a->ks, coef, psi,
                       scale, lambda, dfdX, a->xpt_mode, s);
    else
      launch_hex_xpt(a->ep, m, a->color(c), vars, func, a->ks, coef, psi,
                     scale, lambda, dfdX, a->xpt_mode, s);
  }
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_set_xpt_mode(tg_assembler *a, int mode) {
  if (!a) return fail(TG_ERR_ARG, "tg_set_xpt_mode: NULL assembler");
  if (mode != TG_XPT_FORWARD && mode != TG_XPT_REVERSE)
    return fail(TG_ERR_ARG, "tg_set_xpt_mode: unknown mode");
  a->xpt_mode = mode;
  return 0;
}

int tg_add_xpt_sens(tg_assembler *a, const double *vars, int nfuncs,
                    const int *funcs, double coef, double **dfdX, void *s) {
  int rc = check_ready(a, "tg_add_xpt_sens");
  if (rc) return rc;
  if (!vars || nfuncs < 0 || (nfuncs > 0 && (!funcs || !dfdX)))
    return fail(TG_ERR_ARG, "tg_add_xpt_sens: bad arguments");
  for (int i = 0; i < nfuncs; i++) {
    if (funcs[i] != TG_FUNC_COMPLIANCE && funcs[i] != TG_FUNC_KS_FAILURE)
      return fail(TG_ERR_ARG, "tg_add_xpt_sens: unknown function");
    if (funcs[i] == TG_FUNC_KS_FAILURE && !a->ks_valid)
      return fail(TG_ERR_STATE,
                  "tg_add_xpt_sens: evaluate the KS function first");
    if (!dfdX[i]) return fail(TG_ERR_ARG, "tg_add_xpt_sens: NULL output");
    if ((rc = xpt_pass(a, vars, funcs[i], coef, nullptr, 0.0, 0.0, dfdX[i],
                       S(s))))
      return rc;
  }
  return 0;
}

int tg_add_adjoint_res_xpt_products(tg_assembler *a, const double *vars,
                                    double scale, int nadj, const double **psi,
                                    double **dfdX, double lambda, void *s) {
  int rc = check_ready(a, "tg_add_adjoint_res_xpt_products");
  if (rc) return rc;
  if (!vars || nadj < 0 || (nadj > 0 && (!psi || !dfdX)))
    return fail(TG_ERR_ARG, "tg_add_adjoint_res_xpt_products: bad arguments");
  for (int k = 0; k < nadj; k++) {
    if (!psi[k] || !dfdX[k])
      return fail(TG_ERR_ARG, "tg_add_adjoint_res_xpt_products: NULL vector");
    if ((rc = xpt_pass(a, vars, -1, 0.0, psi[k], scale, lambda, dfdX[k],
                       S(s))))
      return rc;
  }
  return 0;
}

int tg_add_total_xpt_derivative(tg_assembler *a, const double *vars, int func,
                                double coef, const double *psi, double scale,
                                double *dfdX, void *s) {
  int rc = check_ready(a, "tg_add_total_xpt_derivative");
  if (rc) return rc;
  if (!vars || !dfdX)
    return fail(TG_ERR_ARG, "tg_add_total_xpt_derivative: NULL");
  if (func != TG_FUNC_COMPLIANCE && func != TG_FUNC_KS_FAILURE)
    return fail(TG_ERR_ARG, "tg_add_total_xpt_derivative: unknown function");
  if (func == TG_FUNC_KS_FAILURE && !a->ks_valid)
    return fail(TG_ERR_STATE, "evaluate the KS function first");
  return xpt_pass(a, vars, func, coef, psi, scale, 1.0, dfdX, S(s));
}

// ------------------------------------------------------ element segments
int tg_assembler_set_segments(tg_assembler *a, int nseg,
                              const int *elem_ptr) {
  if (!a || nseg <= 0 || !elem_ptr)
    return fail(TG_ERR_ARG, "tg_assembler_set_segments: bad arguments");
  if (elem_ptr[0] != 0 || elem_ptr[nseg] != a->nelem)
    return fail(TG_ERR_ARG,
                "tg_assembler_set_segments: elem_ptr must span 0..elements");
  std::vector<int> eseg(a->nelem);
  for (int g = 0; g < nseg; g++) {
    if (elem_ptr[g + 1] <= elem_ptr[g])
      return fail(TG_ERR_ARG,
                  "tg_assembler_set_segments: empty or unsorted range");
    for (int e = elem_ptr[g]; e < elem_ptr[g + 1]; e++) eseg[e] = g;
  }
  dfree(a->d_elem_seg); dfree(a->d_seg_elem_ptr); dfree(a->d_seg_ks);
  dfree(a->d_seg_comp);
  a->seg_elem_ptr_h.assign(elem_ptr, elem_ptr + nseg + 1);
  int rc = upload(&a->d_elem_seg, eseg);
  if (!rc) rc = upload(&a->d_seg_elem_ptr, a->seg_elem_ptr_h);
  if (!rc) rc = dalloc(&a->d_seg_ks, (size_t)nseg);
  if (!rc) rc = dalloc(&a->d_seg_comp, (size_t)nseg);
  if (rc) return rc;
  a->nseg = nseg;
  a->seg_ks_valid = false;
  return 0;
}

int tg_eval_functions_segments(tg_assembler *a, const double *vars, int func,
                               double ks_weight, double *vals, void *s) {
  int rc = check_ready(a, "tg_eval_functions_segments");
  if (rc) return rc;
  if (!vars || !vals || a->nseg <= 0)
    return fail(TG_ERR_ARG, "tg_eval_functions_segments: bad arguments");
  if (func != TG_FUNC_COMPLIANCE && func != TG_FUNC_KS_FAILURE)
    return fail(TG_ERR_ARG, "tg_eval_functions_segments: unknown function");
  if (a->geo_enabled && (rc = geo_prepare(a, S(s)))) return rc;
  launch_points(a, vars, S(s));
  launch_segment_functions(a->d_elem_fail, a->d_elem_wdet, a->d_elem_sed,
                           a->nq(), a->d_seg_elem_ptr, a->nseg, ks_weight,
                           a->d_seg_ks, a->d_seg_comp, S(s));
  std::vector<KsStats> ks(a->nseg);
  std::vector<double> comp(a->nseg);
  TG_CUDA(cudaMemcpyAsync(ks.data(), a->d_seg_ks, a->nseg * sizeof(KsStats),
                          cudaMemcpyDeviceToHost, S(s)));
  TG_CUDA(cudaMemcpyAsync(comp.data(), a->d_seg_comp,
                          a->nseg * sizeof(double), cudaMemcpyDeviceToHost,
                          S(s)));
  TG_CUDA(cudaStreamSynchronize(S(s)));
  for (int g = 0; g < a->nseg; g++) {
    vals[g] = func == TG_FUNC_COMPLIANCE
                  ? comp[g]
                  : ks[g].max + std::log(ks[g].sum) / ks_weight;
    if (!std::isfinite(vals[g]))
      return fail(TG_ERR_NONFINITE,
                  "tg_eval_functions_segments: non-finite result");
  }
  a->seg_ks_valid = true;
  return 0;
}

int tg_segment_ks_save(tg_assembler *a, double *ks, void *s) {
  int rc = check_ready(a, "tg_segment_ks_save");
  if (rc) return rc;
  if (!ks || a->nseg <= 0)
    return fail(TG_ERR_ARG, "tg_segment_ks_save: bad arguments");
  if (!a->seg_ks_valid)
    return fail(TG_ERR_STATE, "evaluate the segment KS functions first");
  static_assert(sizeof(KsStats) == 3 * sizeof(double), "KsStats layout");
  TG_CUDA(cudaMemcpyAsync(ks, a->d_seg_ks, a->nseg * sizeof(KsStats),
                          cudaMemcpyDeviceToDevice, S(s)));
  return 0;
}

int tg_segment_ks_restore(tg_assembler *a, const double *ks, void *s) {
  int rc = check_ready(a, "tg_segment_ks_restore");
  if (rc) return rc;
  if (!ks || a->nseg <= 0)
    return fail(TG_ERR_ARG, "tg_segment_ks_restore: bad arguments");
  TG_CUDA(cudaMemcpyAsync(a->d_seg_ks, ks, a->nseg * sizeof(KsStats),
                          cudaMemcpyDeviceToDevice, S(s)));
  a->seg_ks_valid = true;
  return 0;
}

int tg_add_sv_sens_segments(tg_assembler *a, const double *vars, int func,
                            double alpha, double *dfdu, void *s) {
  int rc = check_ready(a, "tg_add_sv_sens_segments");
  if (rc) return rc;
  if (!vars || !dfdu || a->nseg <= 0)
    return fail(TG_ERR_ARG, "tg_add_sv_sens_segments: bad arguments");
  if (func == TG_FUNC_KS_FAILURE && !a->seg_ks_valid)
    return fail(TG_ERR_STATE, "evaluate the segment KS functions first");
  MeshView m = a->view_segments();
  for (int c = 0; c < a->ncolors(); c++) {
    if (a->ep.elem_type == TG_ELEM_MITC4)
      launch_shell_sv_sens(a->ep, m, a->color(c), vars, func, a->ks, alpha,
                           dfdu, S(s));
    else
      launch_hex_sv_sens(a->ep, m, a->color(c), vars, func, a->ks, alpha,
                         dfdu, S(s));
  }
  TG_CUDA(cudaGetLastError());
  return 0;
}

int tg_add_total_derivative_segments(tg_assembler *a, const double *vars,
                                     int func, double coef, const double *psi,
                                     double scale, double *dfdx, void *s) {
  int rc = check_ready(a, "tg_add_total_derivative_segments");
  if (rc) return rc;
  if (!vars || !dfdx || a->nseg <= 0)
    return fail(TG_ERR_ARG, "tg_add_total_derivative_segments: bad arguments");
  if (func == TG_FUNC_KS_FAILURE && !a->seg_ks_valid)
    return fail(TG_ERR_STATE, "evaluate the segment KS functions first");
  return elem_dv_pass_view(a, a->view_segments(), vars, func, coef, psi,
                           scale, dfdx, S(s));
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
// Cluster schedule of the two triangular solves (IluClusterView): the
// connected components of the matrix graph are independent, so components
// are packed into groups (longest-processing-time first on their level
// counts) and each group's levels are merged level by level.  The cluster
// size follows the widest level: about 8 block rows per CTA in FP64 (the
// FP64 pipe binds), 32 in FP32.
static int build_cluster_schedule(tg_pc *pc, const std::vector<int> &rowp,
                                  const std::vector<int> &cols,
                                  const std::vector<int> &lvl,
                                  const std::vector<int> &ulvl, int nl,
                                  int nu, int force_cs = 0) {
  const int n = (int)rowp.size() - 1;
  std::vector<int> parent(n);
  std::iota(parent.begin(), parent.end(), 0);
  std::function<int(int)> find = [&](int a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  for (int i = 0; i < n; i++)
    for (int j = rowp[i]; j < rowp[i + 1]; j++) {
      int a = find(i), b = find(cols[j]);
      if (a != b) parent[std::max(a, b)] = std::min(a, b);
    }
  std::vector<int> comp_of(n), comp_id(n, -1);
  int ncomp = 0;
  for (int i = 0; i < n; i++) {
    int r = find(i);
    if (comp_id[r] < 0) comp_id[r] = ncomp++;
    comp_of[i] = comp_id[r];
  }
  std::vector<int> cnl(ncomp, 0), cnu(ncomp, 0), crows(ncomp, 0);
  for (int i = 0; i < n; i++) {
    const int c = comp_of[i];
    cnl[c] = std::max(cnl[c], lvl[i] + 1);
    cnu[c] = std::max(cnu[c], ulvl[i] + 1);
    crows[c]++;
  }
  std::vector<int> wl(nl, 0), wu(nu, 0);
  for (int i = 0; i < n; i++) {
    wl[lvl[i]]++;
    wu[ulvl[i]]++;
  }
  const int width = std::max(*std::max_element(wl.begin(), wl.end()),
                             *std::max_element(wu.begin(), wu.end()));
  const int per_cta = pc->precision == TG_PREC_FP64 ? 8 : 32;
  const int max_cs = ilu_cluster_max_size();
  int cs = 1;
  // the widest level over all components bounds the per-group width
  while (cs < max_cs && cs * per_cta < width) cs *= 2;
  if (force_cs > 0) cs = std::min(force_cs, max_cs);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int ngroups = std::max(1, std::min(ncomp, std::max(1, 2 * sms / cs)));
  std::vector<int> order(ncomp);
  std::iota(order.begin(), order.end(), 0);
  std::vector<double> cost(ncomp);
  for (int c = 0; c < ncomp; c++)
    cost[c] = cnl[c] + cnu[c] + (double)crows[c] / (cs * 40.0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load(ngroups, 0.0);
  std::vector<int> grp_of_comp(ncomp);
  for (int c : order) {
    int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    grp_of_comp[c] = g;
    load[g] += cost[c];
  }
  std::vector<int> gnl(ngroups, 0), gnu(ngroups, 0);
  for (int c = 0; c < ncomp; c++) {
    gnl[grp_of_comp[c]] = std::max(gnl[grp_of_comp[c]], cnl[c]);
    gnu[grp_of_comp[c]] = std::max(gnu[grp_of_comp[c]], cnu[c]);
  }
  // level pointers: group g, level L -> rows of its components at level L
  auto schedule = [&](const std::vector<int> &lv, const std::vector<int> &gn,
                      std::vector<int> &grp, std::vector<int> &ptr,
                      std::vector<int> &rows) {
    grp.assign(ngroups + 1, 0);
    for (int g = 0; g < ngroups; g++) grp[g + 1] = grp[g] + gn[g] + 1;
    std::vector<int> cnt(grp[ngroups], 0);
    for (int i = 0; i < n; i++) cnt[grp[grp_of_comp[comp_of[i]]] + lv[i]]++;
    ptr.assign(grp[ngroups], 0);
    int acc = 0;
    for (size_t k = 0; k < cnt.size(); k++) {
      ptr[k] = acc;
      acc += cnt[k];
    }
    rows.assign(n, 0);
    std::vector<int> fill(ptr);
    for (int i = 0; i < n; i++)
      rows[fill[grp[grp_of_comp[comp_of[i]]] + lv[i]]++] = i;
  };
  std::vector<int> grp_l, lptr, lrows, grp_u, uptr, urows;
  schedule(lvl, gnl, grp_l, lptr, lrows);
  schedule(ulvl, gnu, grp_u, uptr, urows);
  std::vector<int> diag(n);
  for (int i = 0; i < n; i++) {
    int j = rowp[i];
    while (cols[j] < i) j++;
    diag[i] = j;
  }
  const int maxb = pc->A->bsize == 6 ? 4 : 8;
  const int dw = 4 * (1 + maxb / 4);  // ints per descriptor
  std::vector<int> ldesc(dw * (size_t)n, 0), udesc(dw * (size_t)n, 0);
  for (int k = 0; k < n; k++) {
    const int i = lrows[k];
    int *d = &ldesc[(size_t)dw * k];
    d[0] = i;
    d[1] = rowp[i];
    d[2] = diag[i] - rowp[i];
    d[3] = diag[i];
    for (int q = 0; q < maxb && q < d[2]; q++) d[4 + q] = cols[rowp[i] + q];
    const int u = urows[k];
    int *e = &udesc[(size_t)dw * k];
    e[0] = u;
    e[1] = diag[u] + 1;
    e[2] = rowp[u + 1] - diag[u] - 1;
    e[3] = diag[u];
    for (int q = 0; q < maxb && q < e[2]; q++) e[4 + q] = cols[diag[u] + 1 + q];
  }
  int max_lp = 0;
  for (int g = 0; g < ngroups; g++)
    max_lp = std::max(max_lp, (grp_l[g + 1] - grp_l[g]) +
                                  (grp_u[g + 1] - grp_u[g]));
  dfree(pc->d_cl_grp_lvl); dfree(pc->d_cl_lvl_ptr); dfree(pc->d_cl_rows);
  dfree(pc->d_cl_grp_ulvl); dfree(pc->d_cl_ulvl_ptr); dfree(pc->d_cl_urows);
  int rc = 0;
  if (!rc) rc = upload(&pc->d_cl_grp_lvl, grp_l);
  if (!rc) rc = upload(&pc->d_cl_lvl_ptr, lptr);
  if (!rc) rc = upload(&pc->d_cl_rows, ldesc);
  if (!rc) rc = upload(&pc->d_cl_grp_ulvl, grp_u);
  if (!rc) rc = upload(&pc->d_cl_ulvl_ptr, uptr);
  if (!rc) rc = upload(&pc->d_cl_urows, udesc);
  if (rc) return rc;
  IluClusterView &v = pc->plan.cluster;
  v.ngroups = ngroups;
  v.cs = cs;
  v.max_lp = max_lp;
  v.grp_lvl = pc->d_cl_grp_lvl;
  v.lvl_ptr = pc->d_cl_lvl_ptr;
  v.ldesc = reinterpret_cast<const int4 *>(pc->d_cl_rows);
  v.grp_ulvl = pc->d_cl_grp_ulvl;
  v.ulvl_ptr = pc->d_cl_ulvl_ptr;
  v.udesc = reinterpret_cast<const int4 *>(pc->d_cl_urows);
  return 0;
}

// Pattern of ILU(k) (BCSRMat::computeILUk, src/bpmat/BCSRMat.cpp:625-730):
// row by row, each stored entry (i, c) of row i left of the diagonal
// combines with the strictly upper entries (c, j) of the already finished
// row c; the product would fill (i, j) at level lev(i, c) + lev(c, j) + 1.
// An existing entry keeps the smaller level, a new one is inserted (rows
// stay sorted) when its level is at most lev_fill.  The matrix's own blocks
// have level 0.  valmap gives each factor block's block in the matrix, or
// -1 for fill.
static void iluk_pattern(const std::vector<int> &rowp,
                         const std::vector<int> &cols, int lev_fill,
                         std::vector<int> &frowp, std::vector<int> &fcols,
                         std::vector<int> &fdiag, std::vector<int> &valmap) {
  const int n = (int)rowp.size() - 1;
  std::vector<int> flev;
  frowp.assign(n + 1, 0);
  fdiag.assign(n, 0);
  fcols.clear();
  valmap.clear();
  std::vector<int> rc, rl;
  for (int i = 0; i < n; i++) {
    rc.assign(cols.begin() + rowp[i], cols.begin() + rowp[i + 1]);
    rl.assign(rc.size(), 0);
    auto at = std::lower_bound(rc.begin(), rc.end(), i);
    if (at == rc.end() || *at != i) {
      rl.insert(rl.begin() + (at - rc.begin()), 0);
      rc.insert(at, i);
    }
    for (size_t j = 0; j < rc.size() && rc[j] < i; j++) {
      const int c = rc[j], lc = rl[j];
      size_t p = j + 1;
      for (int q = fdiag[c] + 1; q < frowp[c + 1]; q++) {
        const int col = fcols[q], lev = lc + flev[q] + 1;
        while (p < rc.size() && rc[p] < col) p++;
        if (p < rc.size() && rc[p] == col) {
          if (lev < rl[p]) rl[p] = lev;
        } else if (lev <= lev_fill) {
          rc.insert(rc.begin() + p, col);
          rl.insert(rl.begin() + p, lev);
        }
      }
    }
    int a = rowp[i];
    for (size_t j = 0; j < rc.size(); j++) {
      if (rc[j] == i) fdiag[i] = (int)fcols.size();
      while (a < rowp[i + 1] && cols[a] < rc[j]) a++;
      valmap.push_back(a < rowp[i + 1] && cols[a] == rc[j] ? a : -1);
      fcols.push_back(rc[j]);
      flev.push_back(rl[j]);
    }
    frowp[i + 1] = (int)fcols.size();
  }
}

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
  if (pc->type == TG_PC_ILU0) {
    if ((rc = build_cluster_schedule(pc, rowp, cols, lvl, ulvl, nl, nu)))
      return rc;
    // kept for the schedule autotuner
    pc->tune_rowp = rowp;
    pc->tune_cols = cols;
    pc->tune_lvl = lvl;
    pc->tune_ulvl = ulvl;
    pc->tune_nl = nl;
    pc->tune_nu = nu;
  }
  if ((rc = upload(&pc->d_lvl_rows, lrows))) return rc;
  if ((rc = upload(&pc->d_ulvl_rows, urows))) return rc;
  if ((rc = upload(&pc->d_upd_ptr, upd_ptr))) return rc;
  if ((rc = upload(&pc->d_upd_tgt, tgt))) return rc;
  if ((rc = upload(&pc->d_upd_src, src))) return rc;
  return 0;
}

static int pc_create(tg_mat *A, int type, int lev_fill, int precision,
                     tg_pc **out) {
  if (!A || !out) return fail(TG_ERR_ARG, "tg_pc_create: NULL argument");
  *out = nullptr;
  if (type != TG_PC_ILU0 && type != TG_PC_BLOCK_JACOBI &&
      type != TG_PC_ILU0_COLORED && type != TG_PC_DIRECT)
    return fail(TG_ERR_ARG, "tg_pc_create: unknown preconditioner type");
  if (precision != TG_PREC_FP64 && precision != TG_PREC_FP32)
    return fail(TG_ERR_ARG, "tg_pc_create: bad precision");
  if (lev_fill < 0 || (lev_fill > 0 && type != TG_PC_ILU0))
    return fail(TG_ERR_ARG, "tg_pc_create: fill levels need TG_PC_ILU0");
  tg_pc *pc = new tg_pc();
  pc->A = A;
  A->refcount++;
  pc->type = type;
  pc->precision = precision;
  pc->lev_fill = lev_fill;
  pc->fnnz = A->nnz;
  tg_assembler *a = A->a;
  int rc = 0;
  const int *rowp_d = a->d_rowp, *cols_d = a->d_cols, *diag_d = a->d_diag;
  if (type == TG_PC_DIRECT) {
    // the complete factorisation: only the apply buffers of this object
    const size_t n = (size_t)A->nrows * A->bsize;
    rc = tg_direct_create(A, 1, precision, &pc->direct);
    if (!rc) rc = dalloc(&pc->d_fail, 1);
    if (!rc) rc = dalloc(&pc->d_gx, n);
    if (!rc) rc = dalloc(&pc->d_gy, n);
    if (!rc && precision == TG_PREC_FP32) rc = dalloc(&pc->d_x32, n);
    if (!rc && precision == TG_PREC_FP32) rc = dalloc(&pc->d_y32, n);
    if (rc) {
      tg_pc_decref(pc);
      return rc;
    }
    pc->plan.bsize = A->bsize;
    pc->plan.nrows = A->nrows;
    *out = pc;
    return 0;
  }
  if (type == TG_PC_ILU0 && lev_fill > 0) {
    std::vector<int> frowp, fcols, fdiag, valmap;
    iluk_pattern(a->rowp_h, a->cols_h, lev_fill, frowp, fcols, fdiag,
                 valmap);
    pc->fnnz = (int)fcols.size();
    rc = build_ilu_plan(pc, frowp, fcols, fdiag);
    if (!rc) rc = upload(&pc->d_prowp, frowp);
    if (!rc) rc = upload(&pc->d_pcols, fcols);
    if (!rc) rc = upload(&pc->d_pdiag, fdiag);
    if (!rc) rc = upload(&pc->d_valmap, valmap);
    rowp_d = pc->d_prowp;
    cols_d = pc->d_pcols;
    diag_d = pc->d_pdiag;
  } else if (type == TG_PC_ILU0) {
    rc = build_ilu_plan(pc, a->rowp_h, a->cols_h, a->diag_h);
  } else if (type == TG_PC_ILU0_COLORED) {
    // greedy colouring of the node graph: nodes of one colour are never
    // neighbours, so with the nodes ordered by colour the ILU(0) factor and
    // both triangular solves proceed one colour at a time
    const int nn = a->nnodes;
    std::vector<int> color;
    pc->ncolors = graph::color_nodes(nn, a->rowp_h.data(), a->cols_h.data(),
                                     color);
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
  const size_t nv = (size_t)pc->fnnz * A->bsize * A->bsize;
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
int tg_pc_create(tg_mat *A, int type, int precision, tg_pc **out) {
  return pc_create(A, type, 0, precision, out);
}
int tg_pc_create_direct(tg_direct *d, tg_pc **out) {
  if (!d || !out) return fail(TG_ERR_ARG, "tg_pc_create_direct: NULL argument");
  *out = nullptr;
  tg_pc *pc = new tg_pc();
  pc->A = tg::direct_matrix(d);
  pc->A->refcount++;
  pc->type = TG_PC_DIRECT;
  pc->precision = tg::direct_precision(d);
  pc->fnnz = pc->A->nnz;
  pc->direct = d;
  pc->shared_direct = true;
  tg::direct_incref(d);
  const size_t n = (size_t)pc->A->nrows * pc->A->bsize;
  int rc = dalloc(&pc->d_fail, 1);
  if (!rc) rc = dalloc(&pc->d_gx, n);
  if (!rc) rc = dalloc(&pc->d_gy, n);
  if (!rc && pc->precision == TG_PREC_FP32) rc = dalloc(&pc->d_x32, n);
  if (!rc && pc->precision == TG_PREC_FP32) rc = dalloc(&pc->d_y32, n);
  if (rc) {
    tg_pc_decref(pc);
    return rc;
  }
  pc->plan.bsize = pc->A->bsize;
  pc->plan.nrows = pc->A->nrows;
  *out = pc;
  return 0;
}

int tg_pc_get_fp64_used(tg_pc *pc, int *used) {
  if (!pc || !used) return fail(TG_ERR_ARG, "tg_pc_get_fp64_used: NULL");
  *used = pc->precision == TG_PREC_FP32 && pc->fp64_ready ? 1 : 0;
  return 0;
}

int tg_pc_create_iluk(tg_mat *A, int lev_fill, int precision, tg_pc **out) {
  return pc_create(A, TG_PC_ILU0, lev_fill, precision, out);
}
int tg_pc_get_fill(tg_pc *pc, int *lev_fill, int *nnz_factor) {
  if (!pc) return fail(TG_ERR_ARG, "tg_pc_get_fill: NULL pc");
  if (lev_fill) *lev_fill = pc->lev_fill;
  if (nnz_factor) *nnz_factor = pc->fnnz;
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

}  // extern "C"

namespace tg {

// FP64 factor of an FP32 preconditioner's matrix, for the FP64 passes a
// mixed-precision solve falls back to (kept in d_F beside the FP32 factor).
int pc_prepare_fp64(tg_pc *pc) {
  if (pc->precision == TG_PREC_FP64 || pc->type != TG_PC_DIRECT ||
      pc->direct64)
    return 0;  // the ILU variants keep their FP64 factor from creation
  return tg_direct_create(pc->A, 1, TG_PREC_FP64, &pc->direct64);
}

long long pc_layout_version(const tg_pc *pc) {
  if (!pc || pc->type != TG_PC_DIRECT) return 0;
  // the two factorisations' counts, combined so that either one changing
  // changes the sum's pair
  return direct_layout_version(pc->direct) * 1000003LL +
         direct_layout_version(pc->direct64);
}

int pc_factor_fp64(tg_pc *pc, cudaStream_t s) {
  if (pc->precision == TG_PREC_FP64 || pc->fp64_ready) return 0;
  if (pc->type == TG_PC_DIRECT) {
    int rc = pc_prepare_fp64(pc);
    if (rc) return rc;
    rc = tg_direct_factor(pc->direct64, s);
    if (rc) return rc;
    pc->fp64_ready = true;
    return 0;
  }
  tg_mat *A = pc->A;
  const size_t nv = (size_t)A->nnz * A->bsize * A->bsize;
  TG_CUDA(cudaMemsetAsync(pc->d_fail, 0, sizeof(int), s));
  const int nl = (int)pc->plan.lvl_ptr_h.size() - 1;
  if (pc->type == TG_PC_ILU0_COLORED) {
    launch_gather_blocks(A->nnz, A->bsize * A->bsize, pc->d_valmap, A->d_vals,
                         pc->d_F, s);
    for (int L = 0; L < nl; L++) launch_ilu0_factor_level(pc->plan, L, pc->d_F, s);
  } else if (pc->type == TG_PC_ILU0) {
    if (pc->lev_fill > 0)
      launch_gather_blocks(pc->fnnz, A->bsize * A->bsize, pc->d_valmap,
                           A->d_vals, pc->d_F, s);
    else
      TG_CUDA(cudaMemcpyAsync(pc->d_F, A->d_vals, nv * sizeof(double),
                              cudaMemcpyDeviceToDevice, s));
    for (int L = 0; L < nl; L++) launch_ilu0_factor_level(pc->plan, L, pc->d_F, s);
  } else {
    TG_CUDA(cudaMemcpyAsync(pc->d_F, A->d_vals, nv * sizeof(double),
                            cudaMemcpyDeviceToDevice, s));
    launch_block_inverse_diag(pc->plan, pc->d_F, s);
  }
  int hfail = 0;
  TG_CUDA(cudaMemcpyAsync(&hfail, pc->d_fail, sizeof(int),
                          cudaMemcpyDeviceToHost, s));
  TG_CUDA(cudaStreamSynchronize(s));
  if (hfail)
    return fail(TG_ERR_PIVOT, "FP64 factor: singular diagonal block");
  pc->fp64_ready = true;
  return 0;
}

}  // namespace tg

// Schedule autotuner of the cluster triangular solves: after the first
// factorisation, time both solves (CUDA events, 3 launches after one
// warm-up) for every cluster size the device can schedule and keep the
// fastest.  The width heuristic of build_cluster_schedule is only the
// starting guess: the best size trades the FP64 work per CTA against the
// cluster barrier's latency, which depends on the level widths.
static int autotune_cluster(tg_pc *pc, cudaStream_t s) {
  const size_t n = (size_t)pc->A->nrows * pc->A->bsize;
  const bool f64 = pc->precision == TG_PREC_FP64;
  void *in = f64 ? (void *)pc->d_gx : (void *)pc->d_x32;
  void *out = f64 ? (void *)pc->d_gy : (void *)pc->d_y32;
  void *tmp = f64 ? (void *)pc->d_tmp : (void *)pc->d_tmp32;
  TG_CUDA(cudaMemsetAsync(in, 0, n * (f64 ? 8 : 4), s));
  cudaEvent_t e0, e1;
  TG_CUDA(cudaEventCreate(&e0));
  TG_CUDA(cudaEventCreate(&e1));
  const int max_cs = ilu_cluster_max_size();
  int best_cs = pc->plan.cluster.cs;
  float best = 1e30f;
  for (int cs = 1; cs <= max_cs; cs *= 2) {
    int rc = build_cluster_schedule(pc, pc->tune_rowp, pc->tune_cols,
                                    pc->tune_lvl, pc->tune_ulvl, pc->tune_nl,
                                    pc->tune_nu, cs);
    if (rc) return rc;
    pc_launch(pc, 1, n, in, out, tmp, nullptr, nullptr, s);
    TG_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < 3; r++)
      pc_launch(pc, 1, n, in, out, tmp, nullptr, nullptr, s);
    TG_CUDA(cudaEventRecord(e1, s));
    TG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    TG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    pc->tune_ms[cs] = ms / 3;
    if (ms < best) {
      best = ms;
      best_cs = cs;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int rc = build_cluster_schedule(pc, pc->tune_rowp, pc->tune_cols,
                                  pc->tune_lvl, pc->tune_ulvl, pc->tune_nl,
                                  pc->tune_nu, best_cs);
  if (rc) return rc;
  if (pc->apply_exec) {  // captured against the previous schedule
    cudaGraphExecDestroy(pc->apply_exec);
    pc->apply_exec = nullptr;
  }
  pc->tuned = true;
  TG_CUDA(cudaGetLastError());
  return 0;
}

extern "C" {

int tg_pc_factor(tg_pc *pc, void *s) {
  if (!pc) return fail(TG_ERR_ARG, "tg_pc_factor: NULL pc");
  tg_mat *A = pc->A;
  if (pc->type == TG_PC_DIRECT && pc->shared_direct) {
    if (!tg::direct_is_factored(pc->direct))
      return fail(TG_ERR_STATE, "tg_pc_factor: the shared factorisation is "
                                "not factored");
    int rc = pc->precision == TG_PREC_FP32 ? ensure_f32(A, S(s)) : 0;
    if (rc) return rc;
    pc->factored = true;
    pc->fp64_ready = false;
    return 0;
  }
  if (pc->type == TG_PC_DIRECT) {
    int rc = tg_direct_factor(pc->direct, s);
    if (!rc && pc->precision == TG_PREC_FP32) rc = ensure_f32(A, S(s));
    if (rc) return rc;
    pc->factored = true;
    pc->fp64_ready = false;
    return 0;
  }
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
    const int b2 = A->bsize * A->bsize;
    if (pc->precision == TG_PREC_FP64) {
      if (pc->lev_fill > 0)
        launch_gather_blocks(pc->fnnz, b2, pc->d_valmap, A->d_vals, pc->d_F,
                             S(s));
      else
        TG_CUDA(cudaMemcpyAsync(pc->d_F, A->d_vals, nv * sizeof(double),
                                cudaMemcpyDeviceToDevice, S(s)));
      for (int L = 0; L < nl; L++)
        launch_ilu0_factor_level(pc->plan, L, pc->d_F, S(s));
    } else {
      if (pc->lev_fill > 0)
        launch_gather_blocks_f32(pc->fnnz, b2, pc->d_valmap, A->d_vals,
                                 pc->d_F32, S(s));
      else
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
  pc->fp64_ready = false;
  if (pc->type == TG_PC_ILU0 && !pc->tuned && pc->plan.cluster.ngroups > 0) {
    int rc = autotune_cluster(pc, S(s));
    if (rc) return rc;
  }
  return 0;
}

}  // extern "C"

namespace tg {

// Enqueue M^{-1} on nrhs vectors (ld apart): in -> out.  Buffers are FP64
// for a FP64 pc and FP32 for a FP32 pc; tmp (and px, py for the colour-
// reordered factor) hold nrhs * ld entries.
int pc_launch(tg_pc *pc, int nrhs, size_t ld, const void *in, void *out,
              void *tmp, void *px, void *py, cudaStream_t s, int use_f64) {
  const int bs = pc->A->bsize, nr = pc->A->nrows;
  const bool f64 = use_f64 < 0 ? pc->precision == TG_PREC_FP64 : use_f64 != 0;
  if (pc->type == TG_PC_DIRECT) {
    // the direct solves of all right-hand sides (FP64 solves of an FP32 pc
    // use its FP64 factorisation), several per pass over the factor when
    // they lie back to back.  Enqueued without the factored check: a
    // Krylov graph is captured before the FP64 fallback factors direct64.
    tg_direct *d = f64 ? (pc->precision == TG_PREC_FP64 ? pc->direct
                                                        : pc->direct64)
                       : pc->direct;
    const size_t N = (size_t)nr * bs;
    if (ld == N || nrhs == 1)
      return direct_enqueue_solve(d, nrhs, in, out, !f64, s);
    const size_t esz = f64 ? sizeof(double) : sizeof(float);
    for (int r = 0; r < nrhs; r++) {
      const int rc = direct_enqueue_solve(
          d, 1, (const char *)in + r * ld * esz, (char *)out + r * ld * esz,
          !f64, s);
      if (rc) return rc;
    }
    return 0;
  }
  if (pc->type == TG_PC_BLOCK_JACOBI) {
    if (f64)
      launch_block_jacobi_apply(pc->plan, pc->d_F, (const double *)in,
                                (double *)out, s, nrhs, ld);
    else
      launch_block_jacobi_apply_f32(pc->plan, pc->d_F32, (const float *)in,
                                    (float *)out, s, nrhs, ld);
  } else if (pc->type == TG_PC_ILU0_COLORED) {
    if (f64) {
      launch_permute_gather(nr, bs, pc->d_perm, (const double *)in,
                            (double *)px, s, nrhs);
      launch_ilu0_apply(pc->plan, pc->d_F, (const double *)px, (double *)py,
                        (double *)tmp, s, nrhs, ld);
      launch_permute_scatter(nr, bs, pc->d_perm, (const double *)py,
                             (double *)out, s, nrhs);
    } else {
      launch_permute_gather_f32(nr, bs, pc->d_perm, (const float *)in,
                                (float *)px, s, nrhs);
      launch_ilu0_apply_f32(pc->plan, pc->d_F32, (const float *)px,
                            (float *)py, (float *)tmp, s, nrhs, ld);
      launch_permute_scatter_f32(nr, bs, pc->d_perm, (const float *)py,
                                 (float *)out, s, nrhs);
    }
  } else if (f64) {
    launch_ilu0_apply(pc->plan, pc->d_F, (const double *)in, (double *)out,
                      (double *)tmp, s, nrhs, ld);
  } else {
    launch_ilu0_apply_f32(pc->plan, pc->d_F32, (const float *)in,
                          (float *)out, (float *)tmp, s, nrhs, ld);
  }
  return 0;
}

}  // namespace tg

extern "C" {

// Apply the factored preconditioner to the pc's internal input buffer
// (d_gx, or d_x32 in FP32) into its output buffer (d_gy / d_y32).  The ILU(0)
// level sequence (2 x number of levels launches) is captured once into a
// CUDA graph and replayed.
static int pc_apply_internal(tg_pc *pc, cudaStream_t s) {
  const size_t n = (size_t)pc->A->nrows * pc->A->bsize;
  const bool f64 = pc->precision == TG_PREC_FP64;
  void *in = f64 ? (void *)pc->d_gx : (void *)pc->d_x32;
  void *out = f64 ? (void *)pc->d_gy : (void *)pc->d_y32;
  void *tmp = f64 ? (void *)pc->d_tmp : (void *)pc->d_tmp32;
  void *px = f64 ? (void *)pc->d_px : (void *)pc->d_px32;
  void *py = f64 ? (void *)pc->d_py : (void *)pc->d_py32;
  if (pc->type == TG_PC_BLOCK_JACOBI || pc->type == TG_PC_DIRECT)
    return pc_launch(pc, 1, n, in, out, tmp, px, py, s);
  if (!pc->apply_exec) {
    cudaStream_t cs;
    TG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
      pc_launch(pc, 1, n, in, out, tmp, px, py, cs);
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

int tg_pc_get_schedule(tg_pc *pc, int *cluster_size, int *groups,
                       int *levels, double *tuned_ms) {
  if (!pc) return fail(TG_ERR_ARG, "NULL pc");
  if (pc->type == TG_PC_DIRECT) {  // no level schedule of its own
    if (cluster_size) *cluster_size = 0;
    if (groups) *groups = 0;
    if (levels) *levels = 0;
    if (tuned_ms)
      for (int i = 0; i < 5; i++) tuned_ms[i] = 0.0;
    return 0;
  }
  const IluClusterView &v = pc->plan.cluster;
  if (cluster_size) *cluster_size = v.ngroups ? v.cs : 0;
  if (groups) *groups = v.ngroups;
  if (levels)
    *levels = (int)(pc->plan.lvl_ptr_h.size() + pc->plan.ulvl_ptr_h.size()) - 2;
  if (tuned_ms)
    for (int i = 0; i < 5; i++) tuned_ms[i] = pc->tune_ms[1 << i];
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

}  // extern "C"
