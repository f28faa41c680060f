/*
  tacs_gb300 -- C ABI of the GB300 (sm_103a) implementation of the TACS
  finite-element hot path: MITC4-shell and hex8 residual / Jacobian assembly
  into 6x6 / 3x3 block-CSR, the BCSR mat-vec, ILU(k) / block-Jacobi
  preconditioning inside GMRES, and the adjoint products.

  Conventions
  - Every call returns 0 on success or a negative TG_ERR_* code; the message
    of the last failure on the calling thread is available from
    tg_last_error().  No call aborts the process.
  - Vectors are raw DEVICE pointers (double, node-major, vars_per_node per
    node -- the layout of TACSBVec::getArray, src/bpmat/TACSBVec.cpp:983).
    Design vectors hold one value per design variable.  Host-pointer
    arguments are named *_host.
  - `stream` is a cudaStream_t passed as void*; NULL means the legacy
    default stream.  Calls only enqueue work (except where noted) and never
    allocate device memory after the object's creation/initialisation.
  - The library owns the device memory of the objects it creates; objects
    are reference counted like TACSObject (src/TACSObject.h:112-146):
    tg_*_create returns a reference, tg_*_decref releases one.
  - Not re-entrant on one object: calls on the same object must be ordered
    on one stream (the reference's objects are not re-entrant either).

  Each entry point names the reference interface it replaces.
*/
#ifndef TACS_GB300_H
#define TACS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TG_OK 0
#define TG_ERR_ARG -1      /* invalid argument / size */
#define TG_ERR_CUDA -2     /* a CUDA runtime call failed */
#define TG_ERR_STATE -3    /* call out of order (e.g. not initialised) */
#define TG_ERR_PIVOT -4    /* zero pivot in a diagonal block inverse */
#define TG_ERR_NOCONV -5   /* iterative solve hit its iteration limit */
#define TG_ERR_NONFINITE -6 /* NaN/Inf detected in a result */

#define TG_ELEM_MITC4 0 /* TACSQuad4Shell, 6 dof/node */
#define TG_ELEM_HEX8 1  /* TACSElement3D(LinearElasticity3D, LinearHexaBasis) */

#define TG_MAT_NORMAL 0    /* MatrixOrientation TACS_MAT_NORMAL */
#define TG_MAT_TRANSPOSE 1 /* TACS_MAT_TRANSPOSE */

#define TG_PC_ILU0 0        /* TACSAdditiveSchwarz(mat, levFill, fill): ILU */
#define TG_PC_BLOCK_JACOBI 1 /* inverted diagonal blocks only */
#define TG_PC_ILU0_COLORED 2 /* ILU(0) of a multicolour node reordering */
#define TG_PC_DIRECT 3       /* complete factorisation (tg_direct); FP32:
                                the factor of a mixed-precision solve */

#define TG_PREC_FP64 0 /* preconditioner and inner mat-vec in FP64 */
#define TG_PREC_FP32 1 /* FP32 factor / apply and inner mat-vec */

#define TG_FUNC_COMPLIANCE 0 /* TACSCompliance */
#define TG_FUNC_KS_FAILURE 1 /* TACSKSFailure, KS_CONTINUOUS */

typedef struct tg_assembler tg_assembler;
typedef struct tg_mat tg_mat;
typedef struct tg_pc tg_pc;
typedef struct tg_ksm tg_ksm;
typedef struct tg_direct tg_direct;

/* ---------------------------------------------------------------- errors */
const char *tg_last_error(void);
int tg_version(void);

/* ------------------------------------------------------------- assembler */
/* TACSAssembler::TACSAssembler + setElementConnectivity + setElements
   (src/TACSAssembler.h:83-91).  conn holds npe node ids per element
   (4 for MITC4 in TACSShellQuadBasis<2> order, 8 for hex8 in
   TACSLinearHexaBasis order).  Material: TACSMaterialProperties(rho, ., E,
   nu, ys) (src/constitutive/TACSMaterialProperties.h:44).  For shells the
   transform is TACSShellNaturalTransform (transform = 0) or
   TACSShellRefAxisTransform(ref_axis) (transform = 1)
   (src/elements/shell/TACSShellElementTransform.h:21,95). */
int tg_assembler_create(int elem_type, int num_nodes, int num_elements,
                        const int *conn_host, double rho, double E, double nu,
                        double ys, int transform, const double *ref_axis_host,
                        tg_assembler **out);
int tg_assembler_incref(tg_assembler *a);
int tg_assembler_decref(tg_assembler *a);
int tg_assembler_get_sizes(tg_assembler *a, int *vars_per_node, int *nnodes,
                           int *nelems, int *ndvs, int *ncolors);

/* TACSAssembler::addBCs(nnodes, nodes, nbcs, vars) with zero values
   (src/TACSAssembler.h:109): dof k of node nodes[i] is constrained when
   bit k of masks[i] is set. */
int tg_assembler_add_bcs(tg_assembler *a, int n, const int *nodes_host,
                         const int *masks_host);

/* Per-element design variables: the thickness t of TACSIsoShellConstitutive
   (src/constitutive/TACSIsoShellConstitutive.h:33) or t of
   TACSSolidConstitutive (TACSSolidConstitutive.h:34) and its design
   variable number tNum (-1: not a design variable). */
int tg_assembler_set_element_dvs(tg_assembler *a, const double *t_host,
                                 const int *dvnum_host);

/* TACSAssembler::initialize (src/TACSAssembler.cpp:2519): builds the BCSR
   non-zero pattern, the element colouring and the device-side maps.
   Synchronous. */
int tg_assembler_initialize(tg_assembler *a);

/* TACSAssembler::setNodes (node vector, 3 doubles per node, device). */
int tg_assembler_set_nodes(tg_assembler *a, const double *xpts,
                           void *stream);
/* TACSAssembler::setDesignVars: values indexed by design-variable number
   (device); every element copies t = dvs[tNum]. */
int tg_assembler_set_design_vars(tg_assembler *a, const double *dvs,
                                 void *stream);

/* Auxiliary loads (TACSAuxElements, src/TACSAuxElements.cpp:78):
   TACSShellPressure with four nodal pressures per element
   (src/elements/shell/TACSShellPressure.h:11-22), and TACSTraction3D face
   tractions in global components (src/elements/TACSTraction3D.cpp:19). */
int tg_assembler_set_pressure(tg_assembler *a, int n, const int *elems_host,
                              const double *vals_host);
int tg_assembler_set_traction(tg_assembler *a, int n, const int *elems_host,
                              const int *faces_host, const double *vals_host);

/* No reference counterpart.  Fixed-geometry assembly: with enable != 0,
   tg_assemble_res and tg_assemble_jacobian produce the same residual and
   matrix (to rounding) from coefficient matrices formed once per distinct
   element geometry: the linear MITC4 element over TACSIsoShellConstitutive
   (tOffset 0) has K = t K1 + t^3 K3, the hex8 element over
   TACSSolidConstitutive K = t K1, and R = K u + lambda R(u = 0); elements
   whose node coordinates relative to their first node are bitwise equal
   share K1 and K3 (one class for a uniform structured mesh).  Each matrix
   block is then summed from its contributions and written once.  The
   classes, coefficients and R(u = 0) are built at the first assembly after
   enabling and after every tg_assembler_set_nodes (synchronous, allocates);
   t (tg_assembler_set_design_vars) and u may change freely.  For shells
   the build also keeps each class's strain operators, which the function
   and sensitivity entry points (tg_eval_functions*, tg_add_sv_sens*,
   tg_add_dv_sens, tg_add_adjoint_res_products, tg_add_total_derivative*)
   then read instead of forming them per element. */
int tg_assembler_set_fixed_geometry(tg_assembler *a, int enable);
/* Geometry classes, coefficient-table bytes (0 before the first build)
   and the bytes of the per-block contribution lists. */
int tg_assembler_get_fixed_geometry(tg_assembler *a, int *nclasses,
                                    double *table_bytes, double *plan_bytes);

/* TACSAssembler::assembleRes(res, lambda, applyBCs)
   (src/TACSAssembler.cpp:4133).  vars: state (device). */
int tg_assemble_res(tg_assembler *a, const double *vars, double lambda,
                    int apply_bcs, double *res, void *stream);

/* TACSAssembler::assembleJacobian(alpha, beta, gamma, res, A, matOr,
   lambda, applyBCs) (src/TACSAssembler.cpp:4291).  Static elements only:
   beta and gamma must be 0.  res may be NULL. */
int tg_assemble_jacobian(tg_assembler *a, double alpha, double beta,
                         double gamma, const double *vars, double *res,
                         tg_mat *A, int mat_orient, double lambda,
                         int apply_bcs, void *stream);

/* TACSAssembler::applyBCs(vec) (zero the constrained entries) */
int tg_apply_bcs(tg_assembler *a, double *vec, void *stream);

/* TACSAssembler::evalFunctions (src/TACSAssembler.cpp:4617) for
   funcs[i] in {TG_FUNC_COMPLIANCE, TG_FUNC_KS_FAILURE}; ks_weight as in
   TACSKSFailure(assembler, ksWeight).  Writes values to vals_host;
   synchronises the stream. */
int tg_eval_functions(tg_assembler *a, const double *vars, int nfuncs,
                      const int *funcs_host, double ks_weight,
                      double *vals_host, void *stream);

/* TACSAssembler::addSVSens(alpha, beta, gamma, funcs, dfdu)
   (src/TACSAssembler.cpp:4941): dfdu[i] += alpha * df_i/du.  Uses the KS
   statistics of the last tg_eval_functions call on this assembler. */
int tg_add_sv_sens(tg_assembler *a, const double *vars, int nfuncs,
                   const int *funcs_host, double alpha, double **dfdu,
                   void *stream);

/* TACSAssembler::addDVSens(coef, funcs, dfdx) (src/TACSAssembler.cpp:4767)
   dfdx[i] += coef * (partial) df_i/dx. */
int tg_add_dv_sens(tg_assembler *a, const double *vars, int nfuncs,
                   const int *funcs_host, double coef, double **dfdx,
                   void *stream);

/* TACSAssembler::addAdjointResProducts(scale, adjoints, dfdx, lambda)
   (src/TACSAssembler.cpp:5033): dfdx[k] += scale * psi_k^T dR/dx. */
int tg_add_adjoint_res_products(tg_assembler *a, const double *vars,
                                double scale, int nadj, const double **psi,
                                double **dfdx, void *stream);

/* Fused total derivative for one function: dfdx = coef * df/dx
   + scale * psi^T dR/dx in one pass (addDVSens followed by
   addAdjointResProducts with the same element strains). */
int tg_add_total_derivative(tg_assembler *a, const double *vars, int func,
                            double coef, const double *psi, double scale,
                            double *dfdx, void *stream);

/* ------------------------------------------- direct factorisation */
/* Complete factorisation of an assembled matrix (the reference's direct
   solve: TACSSchurPc with a large levFill, src/bpmat/TACSSchurMat.cpp:
   1510-1600, same solution): nested dissection (by the node coordinates
   when use_coords), supernodes and fronts analysed once on the host, then
   a level-by-level multifrontal block Cholesky of K with its boundary
   columns zeroed as well, so that x = A^-1 b for the assembled A with its
   row boundary conditions.  precision TG_PREC_FP64, or TG_PREC_FP32 for a
   factorisation in FP32 (from the FP64 matrix) applied by
   tg_direct_solve_f32, e.g. as the preconditioner of an FP64 iteration.
   tg_direct_factor synchronises and returns TG_ERR_PIVOT on a
   non-positive pivot.  Its first call on a tg_direct launches the
   factorisation's kernels on the stream; the second captures them as one
   CUDA graph, which that call and every later one launch.
   stats (9 doubles): supernodes, tree levels, factor bytes (FP64
   storage), update-pool bytes (FP64), dense flops, largest front (scalar
   rows), precision, fronts solved by thread-block clusters, the front
   rows above which they are. */
int tg_direct_create(tg_mat *A, int use_coords, int precision,
                     tg_direct **out);
int tg_direct_factor(tg_direct *d, void *stream);
int tg_direct_solve(tg_direct *d, const double *b, double *x, void *stream);
/* nrhs right-hand sides of n x bs entries back to back (no reference
   counterpart: the batched load cases of one matrix); the solve passes over
   the factor once for up to four of them.  Each right-hand side's result
   is bitwise the one tg_direct_solve gives it. */
int tg_direct_solve_multi(tg_direct *d, int nrhs, const double *b, double *x,
                          void *stream);
int tg_direct_solve_f32(tg_direct *d, const float *b, float *x,
                        void *stream);
/* Mixed precision: x = A^-1 b in FP64 from an FP32 factorisation by
   iterative refinement -- x = 0, then `steps` times x += FP32 solve of
   the FP64 residual r = b - A x (each step gains the FP32 solve's
   relative accuracy, about cond(A) 2^-24). */
int tg_direct_solve_refined(tg_direct *d, const double *b, double *x,
                            int steps, void *stream);
/* The same refinement with a stopping test (no reference counterpart; the
   test of LAPACK's mixed-precision dsgesv, refined further): steps while
   they halve the normwise backward error
   eta = ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), at most
   max_steps; converged when eta reached tol (the steps continue past it
   until one no longer halves eta, since eta <= tol alone still admits a
   residual far above an FP64 factorisation's where |A| |x| >> |b|).
   Returns TG_ERR_NOCONV (x holds the last iterate) when eta stops halving
   for two steps before reaching tol or max_steps pass, which happens when
   cond(A) approaches the inverse of FP32's unit roundoff: factor the
   matrix in FP64 then.  steps and eta (may be NULL)
   receive the steps taken and the final eta.  Synchronises the stream
   once per step.  b and x must be different buffers (both refinement
   calls; tg_direct_solve itself may solve in place). */
int tg_direct_solve_refined_tol(tg_direct *d, const double *b, double *x,
                                int max_steps, double tol, int *steps,
                                double *eta, void *stream);
/* The same for nrhs right-hand sides back to back, refined together (up to
   four per pass over the factor) with the stopping tests applied to each:
   one that has stopped keeps its iterate while the others go on.  Works
   with either factorisation (an FP64 one refines FP64 solves; its first
   step is tg_direct_solve).  With ftol = rtol = 0 the test is the one of
   tg_direct_solve_refined_tol.  With ftol > 0 or rtol > 0 a right-hand
   side has converged, and stops, once every given test holds:
   eta <= tol; a step's correction at most ftol ||x||_inf (its error is
   then about ftol times the contraction of one step, below ftol); the
   residual at most rtol ||b||_inf (the relative residual a Krylov
   solver's tolerance states) -- for callers that need a stated accuracy
   rather than FP64 rounding.  Until then the steps go on as in
   tg_direct_solve_refined_tol, so a right-hand side whose residual cannot
   fall below the rounding of A x (about eps ||A|| ||x||, far above
   rtol ||b|| on thin shells) is accepted there, at the FP64 floor, as the
   Krylov solves accept it.  steps and eta (may be NULL) are arrays of
   nrhs entries; TG_ERR_NOCONV when any right-hand side did not converge
   (eta stopped halving twice above tol, or max_steps passed).  b and x
   must not overlap. */
int tg_direct_solve_refined_multi(tg_direct *d, int nrhs, const double *b,
                                  double *x, int max_steps, double tol,
                                  double ftol, double rtol, int *steps,
                                  double *eta, void *stream);
/* Launch-shape autotuner of the solves (no reference counterpart): times a
   solve of the factored matrix for each threshold above which fronts are
   solved by thread-block clusters (384, 768, 1536 rows; one CTA each
   below) and keeps the fastest.  The choice is cached per (rows, blocks,
   block size, precision, device), so another factorisation of the same
   shape reuses it without timing.  threshold and ms (3 doubles, may be
   NULL) receive the choice and the per-solve times (0 when cached).
   Synchronises the stream. */
int tg_direct_autotune(tg_direct *d, int *threshold, double *ms,
                       void *stream);
int tg_direct_get_stats(tg_direct *d, double *stats);
int tg_direct_decref(tg_direct *d);

/* ------------------------------------- node-coordinate sensitivities */
/* The node vectors dfdX hold 3 doubles per node (TACSAssembler::
   createNodeVec).  Each element's 3 x nodes coordinate derivatives are
   exact (dual arithmetic), the quantity the reference's complex build
   returns.  Launches run colour by colour and are deterministic. */

/* TACSAssembler::addXptSens(coef, funcs, dfdXpt) (src/TACSAssembler.cpp:
   4858): dfdX[i] += coef * d f_i / dX for TG_FUNC_COMPLIANCE /
   TG_FUNC_KS_FAILURE (KS after tg_eval_functions at the same vars). */
int tg_add_xpt_sens(tg_assembler *a, const double *vars, int nfuncs,
                    const int *funcs_host, double coef, double **dfdX,
                    void *stream);

/* TACSAssembler::addAdjointResXptSensProducts(scale, adjoints, dfdXpt,
   lambda) (src/TACSAssembler.cpp:5136): dfdX[k] += scale * psi_k^T dR/dX,
   the pressure and traction loads scaled by lambda. */
int tg_add_adjoint_res_xpt_products(tg_assembler *a, const double *vars,
                                    double scale, int nadj, const double **psi,
                                    double **dfdX, double lambda,
                                    void *stream);

/* Fused shape derivative of one function: dfdX += coef * df/dX
   + scale * psi^T dR/dX (lambda = 1) in one pass. */
int tg_add_total_xpt_derivative(tg_assembler *a, const double *vars, int func,
                                double coef, const double *psi, double scale,
                                double *dfdX, void *stream);

/* How the element coordinate derivatives above are formed (no reference
   counterpart; both are exact): TG_XPT_FORWARD dual arithmetic, one thread
   per element coordinate; TG_XPT_REVERSE (default) a hand-written adjoint
   sweep, one thread per element, 9x (shell) to 20x (hex) faster on
   GB300. */
#define TG_XPT_FORWARD 0
#define TG_XPT_REVERSE 1
int tg_set_xpt_mode(tg_assembler *a, int mode);

/* ------------------------------------------------------ element segments */
/* No reference counterpart (the reference holds one model per assembler).
   elem_ptr (host, nseg+1, elem_ptr[0] = 0 < ... < elem_ptr[nseg] =
   elements) splits the elements into contiguous ranges, e.g. independent
   meshes batched into one assembler; every range then has its own
   compliance and KS aggregate (TACSCompliance / TACSKSFailure evaluated
   over that range's elements only). */
int tg_assembler_set_segments(tg_assembler *a, int nseg, const int *elem_ptr);
/* Per-range function values vals[nseg] (host) of TG_FUNC_COMPLIANCE or
   TG_FUNC_KS_FAILURE; keeps the per-range KS statistics for the calls
   below (evaluate again whenever vars changes).  Synchronises. */
int tg_eval_functions_segments(tg_assembler *a, const double *vars, int func,
                               double ks_weight, double *vals, void *stream);
/* dfdu += alpha * d f_g / du where each element contributes to the function
   of its own range (addSVSens per range, summed into one vector). */
int tg_add_sv_sens_segments(tg_assembler *a, const double *vars, int func,
                            double alpha, double *dfdu, void *stream);
/* tg_add_total_derivative with each element's own range function. */
int tg_add_total_derivative_segments(tg_assembler *a, const double *vars,
                                     int func, double coef, const double *psi,
                                     double scale, double *dfdx, void *stream);
/* No reference counterpart.  The per-range KS statistics that the last
   tg_eval_functions_segments kept (3 doubles per range: the maximum, the
   sum of exp(weight (f - max)) and the weight), copied to / from the
   device buffer ks (3 nseg doubles), so that the sensitivities of several
   state vectors can be formed after all of them were evaluated: save
   after each evaluation, restore before that state's sensitivity calls.
   Asynchronous on the stream. */
int tg_segment_ks_save(tg_assembler *a, double *ks, void *stream);
int tg_segment_ks_restore(tg_assembler *a, const double *ks, void *stream);

/* --------------------------------------------------------------- vectors */
/* TACSBVec::axpy / scale / dot (src/bpmat/TACSBVec.cpp:215-408) on device
   vectors of n doubles.  tg_vec_dot synchronises the stream and writes the
   result to *out (host); it keeps a small reduction buffer per device. */
int tg_vec_axpy(double alpha, const double *x, double *y, long n,
                void *stream);
int tg_vec_scale(double alpha, double *x, long n, void *stream);
int tg_vec_dot(const double *x, const double *y, long n, double *out,
               void *stream);

/* ------------------------------------------------------------------ BCSR */
/* TACSAssembler::createMat (src/TACSAssembler.cpp:3384): a BCSR matrix with
   the assembler's non-zero pattern (node graph plus diagonal, sorted
   columns; BCSRMatData, src/bpmat/BCSRMatImpl.h:27-46). */
int tg_mat_create(tg_assembler *a, tg_mat **out);
int tg_mat_decref(tg_mat *A);
/* BCSRMat::getArrays (src/bpmat/BCSRMat.h:82): device pointers */
int tg_mat_get_arrays(tg_mat *A, int *bsize, int *nrows, const int **rowp,
                      const int **cols, double **vals);
/* BCSRMat::mult / TACSParallelMat::mult (src/bpmat/TACSParallelMat.cpp:248)
   y = A x (device vectors). */
int tg_mat_mult(tg_mat *A, const double *x, double *y, void *stream);
/* FP32 copy of the matrix values and y = A x in FP32 (mixed precision) */
int tg_mat_mult_f32(tg_mat *A, const float *x, float *y, void *stream);

/* ------------------------------------------------------- preconditioners */
/* TACSAdditiveSchwarz(mat, levFill = 0, fill)
   (src/bpmat/TACSParallelMat.cpp:1190) with type TG_PC_ILU0, plus the
   block-Jacobi and colour-reordered ILU(0) variants and TG_PC_DIRECT (the
   complete factorisation of tg_direct_*, the reference's TACSSchurPc with
   a large levFill); precision TG_PREC_FP32 keeps the factor in FP32. */
int tg_pc_create(tg_mat *A, int type, int precision, tg_pc **out);
/* TACSAdditiveSchwarz(mat, levFill, fill) with levFill > 0: block ILU(k)
   on the level-of-fill pattern of BCSRMat::computeILUk
   (src/bpmat/BCSRMat.cpp:625); levFill = 0 is tg_pc_create(TG_PC_ILU0).
   The pattern is built here on the host, once. */
int tg_pc_create_iluk(tg_mat *A, int lev_fill, int precision, tg_pc **out);
/* TACSSerialPivotPc over an existing factorisation
   (src/bpmat/TACSSerialPivotMat.h:66): a TG_PC_DIRECT preconditioner that
   shares d (its precision, its factor, a reference to it) instead of
   factoring the matrix again, so that GMRES can take an FP32
   factorisation that plain iterative refinement does not converge with
   (GMRES-IR).  tg_direct_factor(d) refactors; tg_pc_factor on this pc only
   refreshes the FP32 copy of the matrix values that mixed GMRES uses. */
int tg_pc_create_direct(tg_direct *d, tg_pc **out);
/* No reference counterpart.  *used = 1 when an FP32 pc's FP64 factor of
   the same matrix has been made since its last tg_pc_factor (the mixed
   GMRES passes switched to it), else 0. */
int tg_pc_get_fp64_used(tg_pc *pc, int *used);
/* Level of fill and the factor's block count (nnz(ILU)). */
int tg_pc_get_fill(tg_pc *pc, int *lev_fill, int *nnz_factor);
int tg_pc_decref(tg_pc *pc);
/* TACSAdditiveSchwarz::factor -> BCSRMat::factor (BCSRMatFact6.cpp:946).
   Synchronises; returns TG_ERR_PIVOT (with the row in tg_last_error) on a
   singular diagonal block. */
int tg_pc_factor(tg_pc *pc, void *stream);
/* TACSAdditiveSchwarz::applyFactor -> BCSRMat::applyFactor
   (src/bpmat/BCSRMat.cpp:1326): y = (LU)^{-1} x. */
int tg_pc_apply(tg_pc *pc, const double *x, double *y, void *stream);
/* No reference counterpart.  The schedule of the natural-order ILU(0)
   triangular solves: thread-block cluster size and number of clusters (0
   when the level kernels are used), lower + upper level count, and the
   autotuner's measured time per solve pair in ms for cluster sizes
   1, 2, 4, 8, 16 (tuned_ms, 5 entries, 0 where not measured; may be
   NULL).  The autotuner runs once, at the first tg_pc_factor. */
int tg_pc_get_schedule(tg_pc *pc, int *cluster_size, int *groups,
                       int *levels, double *tuned_ms);

/* ------------------------------------------------------------------- KSM */
/* GMRES(mat, pc, m, nrestart, isFlexible) (src/bpmat/KSM.h) with
   setTolerances(rtol, atol).  mixed != 0 runs the preconditioner and the
   inner mat-vec in FP32 (pc must be TG_PREC_FP32) inside FP64 GMRES with
   FP64 Arnoldi and a true-residual iterative-refinement loop; when the
   FP32 passes stop paying, the remaining passes run the all-FP64 solve
   (an FP64 factor of the same matrix is made then).  With a TG_PREC_FP32
   pc the solver is flexible GMRES (isFlexible = 1: it keeps M^{-1} v_j,
   m more vectors of memory). */
int tg_ksm_create(tg_mat *A, tg_pc *pc, int m, int nrestart, int mixed,
                  tg_ksm **out);
int tg_ksm_decref(tg_ksm *k);
int tg_ksm_set_tolerances(tg_ksm *k, double rtol, double atol);
/* GMRES::solve(b, x, zero_guess) (src/bpmat/KSM.cpp:785).  Synchronous.
   Returns 1 when converged, 0 when not (like the reference), or a negative
   error code.  iters / resnorm (host) receive the iteration count and the
   final (estimated, or true for mixed) residual norm. */
int tg_ksm_solve(tg_ksm *k, const double *b, double *x, int zero_guess,
                 int *iters, double *resnorm, void *stream);
/* No reference counterpart (the reference runs one GMRES per system).
   Splits the block rows into nseg ranges, row_ptr[0] = 0 <
   row_ptr[1] < ... < row_ptr[nseg] = rows (host array), that the matrix
   does not couple (a block-diagonal matrix, e.g. several meshes in one
   assembler; TG_ERR_ARG otherwise).  Every range is then solved as its own
   system with its own Krylov basis, residual and convergence test.  With
   segments set, tg_ksm_solve returns 1 only when every range converged
   and reports the largest iteration count and residual. */
int tg_ksm_set_segments(tg_ksm *k, int nseg, const int *row_ptr);
/* nrhs right-hand sides in one solve: B and X hold nrhs vectors of
   rows x bsize entries one after another (device).  The nseg x nrhs
   systems (index rhs * nseg + range) run as one batched restarted GMRES:
   one mat-vec and one preconditioner application per step cover all of
   them.  iters, flags (1 converged, 0 not) and resnorms receive one entry
   per system (host arrays, may be NULL).  Returns 1 when every system
   converged, 0 when not, or a negative error code.  Synchronous.  At most
   1024 systems per solve. */
int tg_ksm_solve_multi(tg_ksm *k, int nrhs, const double *B, double *X,
                       int zero_guess, int *iters, int *flags,
                       double *resnorms, void *stream);
/* No reference counterpart.  How the solves of the current layout (after a
   first solve) are launched: cycle_graph 1 when each restart cycle is one
   graph whose device-side WHILE node repeats the Arnoldi step (one host
   synchronisation per cycle), 0 when the host launches the step graph and
   checks every few steps; step_nodes / step_nodes_fp32 the graph nodes
   (kernel launches and copies) of one Arnoldi step with the FP64 and (mixed
   precision) FP32 operator.  Any pointer may be NULL. */
int tg_ksm_get_graph_info(tg_ksm *k, int *cycle_graph, int *step_nodes,
                          int *step_nodes_fp32);

/* ------------------------------------------------- allocation-free entry */
/* No counterpart in the reference.  Compliance and KS failure (the values of
   TG_FUNC_COMPLIANCE and TG_FUNC_KS_FAILURE, in that order) of a mesh whose
   arrays the caller owns, computed without allocating any device memory:
   for callers that may not call cudaMalloc (a host framework that hands
   out views of its own pre-allocated device arena, or a loop that has
   frozen its memory footprint and must not allocate, since an allocation
   can implicitly synchronise the device).
   All pointers except ref_axis_host are device pointers: conn (npe per
   element), xpts (3 per node), thick (one t per element), vars (state),
   vals (2 doubles, written).  Working memory is one file-scope device
   array sized for at most TG_NOALLOC_MAX_ELEMENTS elements; every GPU that
   loads the library keeps it (about 4.5 MB) until the process exits.
   Larger meshes are rejected with TG_ERR_ARG.  The first call on each
   device looks up that array's device address (cudaGetSymbolAddress) with
   the device current, so make the first call on a device before any stream
   capture.  All calls share the array: calls that overlap on the GPU (for
   example on two streams) race and must be serialised by the caller. */
#define TG_NOALLOC_MAX_ELEMENTS 32768
int tg_eval_functions_noalloc(int elem_type, int num_elements,
                              const int *conn, const double *xpts,
                              const double *thick, double E, double nu,
                              double ys, int transform,
                              const double *ref_axis_host, const double *vars,
                              double ks_weight, double *vals, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TACS_GB300_H */
