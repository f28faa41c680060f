// Internal declarations shared by the sm_103a kernels and the C++ host
// runtime of libtacs_gb300.  Not part of the public C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tacs_gb300.h"
#include "direct_view.h"
#include "elem_params.h"

namespace tg {

// Device-side view of an assembler used by the element kernels.
struct MeshView {
  int nnodes, nelem, vpn, npe;
  const int *conn;        // npe * nelem
  const double *xpts;     // 3 * nnodes
  const double *thick;    // nelem
  const double *pres;     // 4 * nelem nodal pressures or nullptr
  const int *trac_ptr;    // nelem + 1 (hex tractions) or nullptr
  const int *trac_face;   // per traction entry
  const double *trac_val; // 3 per traction entry
  const int *rowp, *cols; // BCSR pattern
  // element segments (independent meshes in one assembler): when elem_seg
  // is set, the KS sensitivities of element e use seg_ks[elem_seg[e]]
  const int *elem_seg;
  const struct KsStats *seg_ks;
  // fixed-geometry mode (shells): per geometry class the strain operators
  // B_q (4 x 9 x 24) and detXd_q (4), 868 doubles, and the class of each
  // element; nullptr: the kernels form B from the node coordinates
  const double *geo_B;
  const int *geo_cls;
  // shell assembly: the blocks and residual rows element e writes first
  // in the colour order (mesh_graph.h first_writers): stored, not added,
  // so the matrix and residual need no zero fill; nullptr: add everything
  const unsigned *first;
};

// One launch of an element kernel covers the elements of one colour:
// elem_list[0..count) (no two share a node, so the scatter needs no atomics).
struct ColorRange {
  const int *elem_list;
  int count;
};

// ---------------------------------------------------------------- kernels
// (defined in shell_kernels.cu / hex_kernels.cu / bcsr_kernels.cu)

// Residual (and optionally Jacobian) assembly of one colour.
// mat may be nullptr (residual only); res may be nullptr (matrix only).
// 8-lane-team MITC4 assembly (shell_team.cu); err_flag (device int, may be
// nullptr) is set when an element has a non-positive Jacobian determinant.
void launch_shell_team_assembly(const ElemParams &ep, const MeshView &m,
                                ColorRange cr, const double *vars,
                                double lambda, double *res, double *mat,
                                int *err_flag, cudaStream_t s);
void launch_hex_assembly(const ElemParams &ep, const MeshView &m,
                         ColorRange cr, const double *vars, double lambda,
                         double *res, double *mat, int transpose,
                         cudaStream_t s);

// Fixed-geometry assembly (geo_cache.cu; the plan in geo_plan.h).  The
// class table holds, per geometry class, ncoef coefficient matrices
// (shell: K1 at t = 1 of membrane, shear and drilling, K3 at t = 1 of
// bending; hex: K1) as npe x npe node blocks of bs x bs, row-major:
// table[((cls * ncoef + coef) * npe * npe + npe * a + b) * bs * bs + ...].
struct GeoView {
  int nrows, nwarps;
  const int *rowp, *cols;   // BCSR pattern (rows = nodes)
  const int *cptr;          // nnz + 1: contribution ranges per slot
  const int *contrib;       // (e << 6) | (npe a + b), element order
  const int *cls;           // geometry class per element
  const int *node_bc;       // constraint mask per node
  const int *warp_kmax;     // longest row of each 32-row group
  const double *thick;      // element scale t
  const double *table;      // class table
  const double *f0;         // R(u = 0, lambda = 1) without constraints
  // entries (r * bs + c) non-zero in some class: bit set (coefficient 1, 3)
  unsigned long long mask1, mask3;
};
// Builds the class table of the representative elements (one warp each).
// (shells: also the classes' strain operators and detXd into btab, 868
// doubles per class, when btab is not nullptr)
void launch_shell_geo_build(const ElemParams &ep, const MeshView &m,
                            const int *reps, int nreps, double *table,
                            double *btab, cudaStream_t s);
void launch_hex_geo_build(const ElemParams &ep, const MeshView &m,
                          const int *reps, int nreps, double *table,
                          cudaStream_t s);
// OR of the non-zero entry bits of every table block into masks[ncoef].
void launch_geo_masks(int bs, int ncoef, int nblocks_per_coef_cls, int ncls,
                      const double *table, unsigned long long *masks,
                      cudaStream_t s);
// K = sum of t K1 (+ t^3 K3) over each block's contributions, row
// constraints applied when apply_bcs; R = K u + lambda f0 with the
// constrained entries set to u (or 0 without vars).  vals and res may each
// be nullptr.
void launch_geo_assembly(int bs, const GeoView &g, const double *vars,
                         double lambda, int apply_bcs, double *res,
                         double *vals, cudaStream_t s);

// Point quantities.  Pass 1 writes per-element, per-point failure values
// and detXd-weighted strain energies; the KS reduction and the sensitivity
// passes read them back.
// elem_fail: nq per element; elem_wdet: nq per element; elem_sed: 1 per elem
void launch_shell_points(const ElemParams &ep, const MeshView &m,
                         const double *vars, double *elem_fail,
                         double *elem_wdet, double *elem_sed,
                         cudaStream_t s);
void launch_hex_points(const ElemParams &ep, const MeshView &m,
                       const double *vars, double *elem_fail,
                       double *elem_wdet, double *elem_sed, cudaStream_t s);

// dfdu += alpha * df/du for one colour.  func: TG_FUNC_*; for KS the
// statistics ks (or the element's segment statistics) are used.
void launch_shell_sv_sens(const ElemParams &ep, const MeshView &m,
                          ColorRange cr, const double *vars, int func,
                          KsStats ks, double alpha, double *dfdu,
                          cudaStream_t s);
void launch_hex_sv_sens(const ElemParams &ep, const MeshView &m,
                        ColorRange cr, const double *vars, int func,
                        KsStats ks, double alpha, double *dfdu,
                        cudaStream_t s);

// Per-element design derivative: out[e] = coef * df/dt_e (func >= 0, or 0
// when func < 0) + scale * psi_e^T dR_e/dt_e (psi may be nullptr).
void launch_shell_dv(const ElemParams &ep, const MeshView &m,
                     const double *vars, int func, KsStats ks, double coef,
                     const double *psi, double scale, double *out,
                     cudaStream_t s);
void launch_hex_dv(const ElemParams &ep, const MeshView &m, const double *vars,
                   int func, KsStats ks, double coef, const double *psi,
                   double scale, double *out, cudaStream_t s);

// Node-coordinate sensitivities of one colour, added into dfdX (3 per
// node): coef d f/dX for func (TG_FUNC_*, or -1 for none) plus, when psi is
// set, scale psi^T dR/dX with the loads scaled by lambda.
void launch_shell_xpt(const ElemParams &ep, const MeshView &m, ColorRange cr,
                      const double *vars, int func, KsStats ks, double coef,
                      const double *psi, double scale, double lambda,
                      double *dfdX, int reverse, cudaStream_t s);
void launch_hex_xpt(const ElemParams &ep, const MeshView &m, ColorRange cr,
                    const double *vars, int func, KsStats ks, double coef,
                    const double *psi, double scale, double lambda,
                    double *dfdX, int reverse, cudaStream_t s);

// ------------------------------------------------------- BCSR / vectors
// nrhs vectors ld apart (ld may be 0 when nrhs == 1)
void launch_bcsr_mult(int bsize, int nrows, const int *rowp, const int *cols,
                      const double *A, const double *x, double *y,
                      cudaStream_t s, int nrhs = 1, size_t ld = 0);
void launch_bcsr_mult_f32(int bsize, int nrows, const int *rowp,
                          const int *cols, const float *A, const float *x,
                          float *y, cudaStream_t s, int nrhs = 1,
                          size_t ld = 0);
void launch_apply_bcs_mat(int bsize, int nbcs, const int *bc_nodes,
                          const int *bc_masks, const int *rowp,
                          const int *cols, double *A, cudaStream_t s);
void launch_apply_bcs_res(int bsize, int nbcs, const int *bc_nodes,
                          const int *bc_masks, const double *vars,
                          double *res, cudaStream_t s);
void launch_fill(double *x, double v, size_t n, cudaStream_t s);
void launch_d2f(const double *x, float *y, size_t n, cudaStream_t s);
void launch_f2d(const float *x, double *y, size_t n, cudaStream_t s);
void launch_gather_dv(int nelem, const int *dvnum, const double *dvs,
                      double *thick, cudaStream_t s);
void launch_scatter_dv(int ndv, const int *dv_ptr, const int *dv_elems,
                       const double *elem_vals, double *dfdx, cudaStream_t s);

// Deterministic reductions: partial sums per block then one final block.
// Writes result to out (device scalar).
void launch_reduce_max(const double *x, size_t n, double *partials,
                       int npart, double *out, cudaStream_t s);
void launch_reduce_sum(const double *x, size_t n, double *partials,
                       int npart, double *out, cudaStream_t s);
// max |x_i|, and the scalar-row sums of |A| of a BCSR matrix
// max |x| of k vectors n apart into out[v * stride] (partials: npart k)
void launch_reduce_absmax_multi(const double *x, int k, size_t n,
                                double *partials, int npart, double *out,
                                int stride, cudaStream_t s);
// r = b - t; x += c (c in FP32)
void launch_residual(const double *b, const double *t, double *r, size_t n,
                     cudaStream_t s);
void launch_f2d_add(const float *c, double *x, size_t n, cudaStream_t s);
void launch_reduce_absmax(const double *x, size_t n, double *partials,
                          int npart, double *out, cudaStream_t s);
void launch_bcsr_row_abs_sum(int bsize, int nrows, const int *rowp,
                             const double *vals, double *out, cudaStream_t s);
void launch_ks_sum(const double *fail, const double *wdet, size_t n,
                   const double *dmax, double ksw, double *partials,
                   int npart, double *out, cudaStream_t s);
// Per-segment compliance and KS statistics over contiguous element ranges
// seg_elem_ptr[g]..seg_elem_ptr[g+1] (nq points per element).
void launch_segment_functions(const double *elem_fail, const double *elem_wdet,
                              const double *elem_sed, int nq,
                              const int *seg_elem_ptr, int nseg, double ksw,
                              KsStats *seg_ks, double *seg_comp,
                              cudaStream_t s);

// Cluster schedule of the ILU(0) triangular solves: the matrix's
// independent components are grouped, one thread-block cluster of cs CTAs
// per group.  Group g's lower levels are lvl_ptr[grp_lvl[g] ..
// grp_lvl[g+1]) (level pointers into ldesc), its upper levels likewise in
// ulvl_ptr / udesc.  A row descriptor is 1 + MAXB/4 int4s (MAXB = 4 for
// 6x6 blocks, 8 for 3x3): {row, first block, block count, diagonal block}
// and the columns of the first MAXB blocks -- the strictly lower blocks
// rowp[i]..diag[i] for the lower solve, diag[i]+1..rowp[i+1] for the upper
// one.  max_lp: the most level pointers (lower + upper) of any group.
// ngroups == 0: no cluster schedule.
struct IluClusterView {
  int ngroups, cs, max_lp;
  const int *grp_lvl, *lvl_ptr;
  const int4 *ldesc;
  const int *grp_ulvl, *ulvl_ptr;
  const int4 *udesc;
};

// Level-scheduled block ILU(0) (natural order) and block Jacobi.
struct IluPlan {
  int bsize, nrows;
  const int *rowp, *cols, *diag;
  // level sets of the lower solve / factor (rows in increasing order
  // inside a level), and of the upper solve
  std::vector<int> lvl_ptr_h, ulvl_ptr_h;
  const int *lvl_rows, *ulvl_rows;
  // factor update list: for each row, the (target, lower, upper) block
  // triples of the IKJ update, grouped by lower block
  const int *upd_ptr;  // per lower entry j: range into upd_tgt/upd_src
  const int *upd_tgt, *upd_src;
  int *d_fail;  // device int: first failing row + 1
  IluClusterView cluster;  // triangular solves in one cluster launch
};
void launch_ilu0_factor_level(const IluPlan &p, int level, double *F,
                              cudaStream_t s);
void launch_ilu0_factor_level_f32(const IluPlan &p, int level, float *F,
                                  cudaStream_t s);
void launch_block_inverse_diag(const IluPlan &p, double *F, cudaStream_t s);
int ilu_cluster_max_size();
void launch_ilu0_apply(const IluPlan &p, const double *F, const double *x,
                       double *y, double *tmp, cudaStream_t s, int nrhs = 1,
                       size_t ld = 0);
void launch_ilu0_apply_f32(const IluPlan &p, const float *F, const float *x,
                           float *y, float *tmp, cudaStream_t s,
                           int nrhs = 1, size_t ld = 0);
// colour-reordered ILU(0): value gather through a block map and vector
// permutation (dst[r] = src[perm[r]] / dst[perm[r]] = src[r], bs per node)
void launch_gather_blocks(int nnz, int b2, const int *valmap,
                          const double *src, double *dst, cudaStream_t s);
void launch_gather_blocks_f32(int nnz, int b2, const int *valmap,
                              const double *src, float *dst, cudaStream_t s);
void launch_permute_gather(int nrows, int bs, const int *perm,
                           const double *src, double *dst, cudaStream_t s,
                           int nrhs = 1);
void launch_permute_scatter(int nrows, int bs, const int *perm,
                            const double *src, double *dst, cudaStream_t s,
                            int nrhs = 1);
void launch_permute_gather_f32(int nrows, int bs, const int *perm,
                               const float *src, float *dst, cudaStream_t s,
                               int nrhs = 1);
void launch_permute_scatter_f32(int nrows, int bs, const int *perm,
                                const float *src, float *dst, cudaStream_t s,
                                int nrhs = 1);
void launch_block_jacobi_apply(const IluPlan &p, const double *F,
                               const double *x, double *y, cudaStream_t s,
                               int nrhs = 1, size_t ld = 0);
void launch_block_jacobi_apply_f32(const IluPlan &p, const float *F,
                                   const float *x, float *y, cudaStream_t s,
                                   int nrhs = 1, size_t ld = 0);

// GMRES helpers (FP64 Arnoldi)
void launch_dots(const double *W, size_t ld, int k, const double *w,
                 double *partials, int npart, double *h, cudaStream_t s);
void launch_gemv_sub(const double *W, size_t ld, int k, const double *h,
                     double *w, size_t n, cudaStream_t s);
void launch_axpy(double a, const double *x, double *y, size_t n,
                 cudaStream_t s);
void launch_scale(double a, double *x, size_t n, cudaStream_t s);
void launch_copy(const double *x, double *y, size_t n, cudaStream_t s);

// Batched GMRES (krylov_kernels.cu).  A multivector of nrhs vectors (ld
// apart) is split into systems; chunks of at most 256 * ept entries never
// cross a system.  All arrays are device memory.
struct KrylovChunks {
  const int *start;    // offset of the chunk in the multivector
  const int *len;      // entries in the chunk
  const int *sys;      // system of the chunk
  const int *sys_ptr;  // nsys + 1: chunk range of each system
  int nchunks, nsys, ept;
};
struct KrylovState {
  int m, nsys;
  double atol;
  double *H;         // nsys x (m+1) x m, column-major Hessenberg per system
  double *Qc, *Qs;   // nsys x m Givens rotations
  double *res;       // nsys x (m+1) rotated residual, then -y
  double *h1, *h2;   // nsys x (m+1) the two Gram-Schmidt projections
  double *nrm2;      // nsys squared norms
  double *scale;     // nsys basis-vector scale (0 for inactive systems)
  double *rhs_norm;  // nsys first-cycle residual norms
  double *rn;        // nsys latest residual (estimate or true)
  double *rtol;      // nsys relative tolerances
  int *active, *converged, *done, *err, *niters, *iters;  // nsys each
  int *first;        // 1 before the first cycle of a solve
  int *it;           // current Arnoldi index
  int *nactive;      // systems still iterating
  int *stall;        // 1: a restart that gains less than 10% on a
                     // system's true residual ends that system's solve
                     // (FP32 mat-vec passes)
  double *rn0prev;   // nsys true residual at the previous cycle start
};
void launch_kr_dots(const double *W, size_t ld, const int *kdev, int kofs,
                    int kmax, const double *w, const KrylovChunks &ch,
                    double *partials, double *out, int ldo, cudaStream_t s);
void launch_kr_gemv_sub(const double *W, size_t ld, const int *kdev, int kofs,
                        int kmax, const double *coef, int ldc,
                        const KrylovChunks &ch, double *w, double *normparts,
                        cudaStream_t s);
void launch_kr_norm_final(const double *normparts, const KrylovChunks &ch,
                          double *out, cudaStream_t s);
void launch_kr_scale_store(const double *w, const KrylovChunks &ch,
                           const double *scale, double *W, size_t ld,
                           const int *it, double *v, cudaStream_t s);
void launch_kr_store_at(const double *z, double *Z, size_t ld, const int *it,
                        cudaStream_t s);
void launch_kr_residual(const double *b, double *r, size_t n, cudaStream_t s);
void launch_kr_axpy(const double *x, double *y, size_t n, cudaStream_t s);
void launch_kr_mask(double *x, const KrylovChunks &ch, const double *scale,
                    cudaStream_t s);
void launch_kr_cycle_init(const KrylovState &st, cudaStream_t s);
void launch_kr_arnoldi(const KrylovState &st, cudaStream_t s);
void launch_kr_solve_y(const KrylovState &st, cudaStream_t s);
// Sets the conditional handle of a graph's WHILE node to 1 while systems
// are still iterating and fewer than m Arnoldi steps ran this cycle.
void launch_kr_loop_control(const KrylovState &st,
                            cudaGraphConditionalHandle h, int m,
                            cudaStream_t s);

// ------------------------------------------------ direct factorisation
// multifrontal factorisation (direct_kernels.cu), T = double or float
template <class T>
// (zero, matrix scatter, then nchild extend-add launches of ychunks row
// blocks: the largest child count and child update size of the level)
void launch_direct_level_assemble(const DirectView &v, const int *sn,
                                  int count, const double *A, int zchunks,
                                  int nchild, int ychunks, cudaStream_t s);
template <class T>
void launch_direct_factor_small(const DirectView &v, const int *sn,
                                int count, int *fail, cudaStream_t s);
// one panel step of the large fronts of a level (direct::panel_steps):
// the diagonal blocks of fronts sn[0 .. count) at column k0 and the rows
// below them (rblocks row blocks, prefix sums rprefix[0 .. count]), then
// their trailing tiles (tile x tile, 32 or 64; tiles in all, prefix sums
// tprefix[0 .. count])
template <class T>
void launch_direct_panel_step(const DirectView &v, const int *sn, int count,
                              const int *tprefix, int tiles,
                              const int *rprefix, int rblocks, int k0,
                              int tile, int *fail, cudaStream_t s);
// dynamic shared memory of the panel kernel (staged rows)
size_t direct_panel_smem(size_t elem);
// the inverses of the factored diagonal blocks (count blocks: panel
// inv_k0[b] of supernode inv_sn[b]), after the factorisation
template <class T>
void launch_direct_inverses(const DirectView &v, const int *inv_sn,
                            const int *inv_k0, int count, cudaStream_t s);
template <class T>
void launch_direct_forward(const DirectView &v, const int *sn, int count,
                           int max_front, int nr, T *y, T *contrib,
                           cudaStream_t s);
template <class T>
void launch_direct_backward(const DirectView &v, const int *sn, int count,
                            int max_front, int nr, const T *y, T *x,
                            cudaStream_t s);
// the same solves for large fronts, one thread-block cluster of
// kDirectSolveCluster CTAs per front
template <class T>
void launch_direct_forward_cluster(const DirectView &v, const int *sn,
                                   int count, int max_front, int nr, int ncl,
                                   T *y, T *contrib, cudaStream_t s);
// The fronts solved by clusters at one level of the backward solve: first
// their L21^T x2 products in tiles over the whole GPU (total tiles,
// tprefix / poff per front: cumulative tiles and the offset of its chunk
// sums in part, in entries per right-hand side), then the clusters, which
// add the chunk sums in order
template <class T>
void launch_direct_bwd_gemv(const DirectView &v, const int *sn,
                            const int *tprefix, const int64_t *poff,
                            int count, int total, int nr, const T *x,
                            T *part, cudaStream_t s);
template <class T>
void launch_direct_backward_cluster(const DirectView &v, const int *sn,
                                    const int64_t *poff, int count,
                                    int max_front, int nr, int ncl,
                                    const T *y, T *x, const T *part,
                                    cudaStream_t s);
// whether clusters of ncl CTAs are scheduled on this device
bool direct_cluster_solve_ok(int ncl);
// dynamic shared memory of a solve over fronts of `front` rows with nr
// right-hand sides (one CTA per front, or one cluster per front)
size_t direct_solve_smem(int front, int nr, size_t elem);
size_t direct_cluster_smem(int front, int nr, size_t elem, int ncl);
// nrhs right-hand sides ld apart (node order); ypos / xpos interleaved
template <class T>
void launch_direct_rhs(int n, int bs, const int *perm, const T *b, T *ypos,
                       int nrhs, size_t ld, cudaStream_t s);
template <class T>
void launch_direct_bc_couple(const DirectBc &c, int bs, const T *a,
                             const T *b, T *ypos, int nrhs, size_t ld,
                             cudaStream_t s);
template <class T>
void launch_direct_unpermute(int n, int bs, const int *perm, const T *xpos,
                             T *x, int nrhs, size_t ld, cudaStream_t s);
cudaError_t direct_set_smem(int plain_front, int cluster_front, int max_nr);

// error reporting
void set_error(const std::string &msg);
int cuda_check(cudaError_t e, const char *what);

}  // namespace tg

#define TG_CUDA(call)                                 \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return tg::cuda_check(_e, #call); \
  } while (0)
