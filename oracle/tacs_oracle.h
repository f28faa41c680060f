/*
  CPU oracle for the TACS finite-element hot path -- TEST INFRASTRUCTURE.

  A plain-C restatement of the reference algorithms (TACS 3.12.1) for:
    - the MITC4 shell element TACSQuad4Shell (residual, Jacobian, adjoint
      products, compliance and KS-failure point quantities),
    - the hex8 TACSElement3D(TACSLinearElasticity3D, TACSLinearHexaBasis),
    - their pressure / face-traction loads,
    - BCSR assembly with row-zero Dirichlet conditions, the BCSR mat-vec,
      block ILU(0) (factor with inverted diagonal blocks, lower/upper apply),
    - restarted right-preconditioned GMRES with modified Gram-Schmidt,
    - compliance / KS failure evaluation, addSVSens, addDVSens and
      addAdjointResProducts.

  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
  this library, and only as the checker or as the timed CPU baseline.  The
  GPU product never links or calls it.

  Parity of this oracle is pinned by the tests/golden fixtures, which hold outputs
  of the reference TACS sources themselves (built by oracle/ref/Makefile),
  including the reference tests' own known answers.
*/
#ifndef TACS_ORACLE_H
#define TACS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Problem description shared by every entry point (all arrays borrowed). */
typedef struct {
  int elem_type;      /* 0 = MITC4 shell (6 dof/node), 1 = hex8 (3 dof/node) */
  int nnodes, nelem;
  const double *xpts; /* 3*nnodes */
  const int *conn;    /* npe*nelem */
  const double *thick;/* nelem: shell thickness / solid "t" */
  const int *dvnum;   /* nelem: design-variable index, -1 = fixed */
  double rho, E, nu, ys;
  int transform;      /* shells: 0 natural, 1 reference axis */
  double ref_axis[3];
  int nbcs;
  const int *bc_nodes, *bc_masks;
  int npres;          /* shell pressure: element ids and 4 nodal values */
  const int *pres_elems;
  const double *pres_vals;
  int ntrac;          /* hex traction: element ids, face ids, 3 values */
  const int *trac_elems, *trac_faces;
  const double *trac_vals;
  double ks_weight;
  int nthreads;       /* threads for the element loops and the mat-vec */
} or_problem;

/* Block-CSR matrix with row-major bsize x bsize blocks. */
typedef struct {
  int bsize, nrows;
  int *rowp, *cols, *diag;
  double *vals;
} or_bcsr;

int or_bcsr_create(const or_problem *p, or_bcsr *A);
void or_bcsr_free(or_bcsr *A);

/* Element kernels (one element, local arrays). */
void or_shell_res(const double X[12], double t, const or_problem *p,
                  const double vars[24], const double pres[4], double res[24]);
void or_shell_jac(const double X[12], double t, const or_problem *p,
                  double res[24], const double vars[24], double mat[576]);
void or_hex_res(const double X[24], double t, const or_problem *p,
                const double vars[24], double res[24]);
void or_hex_jac(const double X[24], double t, const or_problem *p,
                double mat[576]);

/* Global assembly: res / A may be NULL.  apply_bcs as TACSAssembler. */
void or_assemble_res(const or_problem *p, const double *vars, double lambda,
                     int apply_bcs, double *res);
void or_assemble_jac(const or_problem *p, const double *vars, double *res,
                     or_bcsr *A, int transpose, int apply_bcs);
void or_apply_bcs_vec(const or_problem *p, double *x);

/* Linear algebra */
void or_bcsr_mult(const or_bcsr *A, const double *x, double *y, int nthreads);
int or_ilu0_factor(const or_bcsr *A, or_bcsr *F);
/* ILU(lev_fill) on the BCSRMat::computeILUk pattern; F->rowp == NULL on
   the first call builds the pattern (F owns it; free with or_bcsr_free). */
int or_iluk_factor(const or_bcsr *A, int lev_fill, or_bcsr *F); /* F gets a copy */
void or_ilu0_apply(const or_bcsr *F, const double *x, double *y);
int or_gmres(const or_bcsr *A, const or_bcsr *F, const double *b, double *x,
             int m, int nrestart, double rtol, double atol, int *iters,
             int nthreads);

/* Functions (f[0] = compliance, f[1] = KS failure) and sensitivities */
void or_eval_funcs(const or_problem *p, const double *vars, double f[2]);
void or_add_sv_sens(const or_problem *p, const double *vars, int which,
                    double *dfdu);
void or_add_dv_sens(const or_problem *p, const double *vars, int which,
                    double scale, double *dfdx);
void or_add_adj_res_product(const or_problem *p, const double *vars,
                            const double *psi, double scale, double *dfdx);
/* Node-coordinate sensitivities (3 per node), central differences */
void or_add_xpt_sens(const or_problem *p, const double *vars, int which,
                     double coef, double *dfdX);
void or_add_adj_res_xpt_product(const or_problem *p, const double *vars,
                                const double *psi, double scale,
                                double lambda, double *dfdX);

/* Convenience: full static solve + both gradients (the timed CPU step). */
int or_static_adjoint(const or_problem *p, int m, int nrestart, double rtol,
                      double atol, const double *force, double *u,
                      double funcs[2], double *grad_comp, double *grad_ks,
                      int *iters);

#ifdef __cplusplus
}
#endif
#endif
