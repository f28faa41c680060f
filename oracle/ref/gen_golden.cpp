/*
  Golden-vector generator: runs the reference TACS library (oracle/_ref) on a
  problem file and writes every quantity the GPU path is checked against.
  Test infrastructure only.

  usage: gen_golden problem.bin out.bin

  The call sequence mirrors the reference's own static test harness
  (tests/integration_tests/static_analysis_base_test.py:359-427):
    1. at a given state u_test: assembleRes, assembleJacobian (BCSR arrays),
       K*x, ILU(0) apply (TACSAdditiveSchwarz(mat, 0, 10.0)) and ILU(1),
       ILU(2) applies (levFill 1, 2), addSVSens,
       addDVSens and addAdjointResProducts with a given psi_test;
    2. the linear static solve R(u) = K u - f = 0 with GMRES + ILU(0);
    3. compliance and KS failure, their state sensitivities, the adjoint
       solve with the transposed assembly, and the total derivative
       dfdx + (-1) * psi^T dR/dx, and the same for the node coordinates
       (addXptSens + addAdjointResXptSensProducts).
*/
#include "ref_problem.h"

static void write_bcsr(TgWriter &w, const char *prefix, TACSParallelMat *mat) {
  BCSRMat *A, *B;
  mat->getBCSRMat(&A, &B);
  int bsize, nrows, ncols;
  const int *rowp, *cols;
  TacsScalar *vals;
  A->getArrays(&bsize, &nrows, &ncols, &rowp, &cols, &vals);
  std::string p(prefix);
  w.i32((p + "_rowp").c_str(), rowp, nrows + 1);
  w.i32((p + "_cols").c_str(), cols, rowp[nrows]);
  w.f64((p + "_vals").c_str(), vals, (int64_t)rowp[nrows] * bsize * bsize);
}

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  TacsInitialize();
  if (argc < 3) {
    fprintf(stderr, "usage: %s problem.bin out.bin\n", argv[0]);
    return 1;
  }
  TgFile p = tg_read(argv[1]);
  RefModel m = tg_build_model(p);
  TACSAssembler *as = m.assembler;
  TgWriter w(argv[2]);

  const int ndof = m.vpn * m.nnodes;
  TACSBVec *res = as->createVec();
  TACSBVec *vec = as->createVec();
  TACSBVec *out = as->createVec();
  TACSBVec *f = as->createVec();
  res->incref();
  vec->incref();
  out->incref();
  f->incref();
  tg_set_vec(f, m.force);
  TACSParallelMat *mat = as->createMat();
  mat->incref();
  TACSAdditiveSchwarz *pc = new TACSAdditiveSchwarz(mat, 0, 10.0);
  pc->incref();

  TACSFunction *funcs[2];
  double ksw = tg_f(p, "ks_weight", 100.0);
  funcs[0] = new TACSCompliance(as);
  funcs[1] = new TACSKSFailure(as, ksw);
  funcs[0]->incref();
  funcs[1]->incref();
  TacsScalar fvals[2];

  TACSBVec *dfdu[2], *psi[2], *dfdx[2];
  for (int k = 0; k < 2; k++) {
    dfdu[k] = as->createVec();
    psi[k] = as->createVec();
    dfdx[k] = as->createDesignVec();
    dfdu[k]->incref();
    psi[k]->incref();
    dfdx[k]->incref();
  }
  TACSBVec *dfdX[2];
  for (int k = 0; k < 2; k++) {
    dfdX[k] = as->createNodeVec();
    dfdX[k]->incref();
  }
  TacsScalar *arr;

  // ---- 1. unit checks at a prescribed state ----------------------------
  std::vector<double> &u_test = tg_fv(p, "u_test");
  if (!u_test.empty()) {
    tg_set_vec(vec, u_test);
    as->setVariables(vec);

    as->assembleRes(res, 1.0, false);
    res->getArray(&arr);
    w.f64("res_nobc", arr, ndof);
    as->assembleRes(res);
    res->getArray(&arr);
    w.f64("res", arr, ndof);

    as->assembleJacobian(1.0, 0.0, 0.0, res, mat, TACS_MAT_NORMAL, 1.0, false);
    write_bcsr(w, "jac_nobc", mat);
    as->assembleJacobian(1.0, 0.0, 0.0, res, mat);
    res->getArray(&arr);
    w.f64("jac_res", arr, ndof);
    write_bcsr(w, "jac", mat);

    std::vector<double> &x_test = tg_fv(p, "x_test");
    if (!x_test.empty()) {
      tg_set_vec(vec, x_test);
      mat->mult(vec, out);
      out->getArray(&arr);
      w.f64("kx", arr, ndof);
      pc->factor();
      pc->applyFactor(vec, out);
      out->getArray(&arr);
      w.f64("ilu_apply", arr, ndof);
      // ILU(k): TACSAdditiveSchwarz(mat, levFill, fill) with levFill 1, 2
      for (int lev = 1; lev <= 2; lev++) {
        TACSAdditiveSchwarz *pk = new TACSAdditiveSchwarz(mat, lev, 10.0);
        pk->incref();
        pk->factor();
        pk->applyFactor(vec, out);
        out->getArray(&arr);
        w.f64(lev == 1 ? "ilu1_apply" : "ilu2_apply", arr, ndof);
        pk->decref();
      }
      TACSMat *pcmat;
      pc->getMat(&pcmat);
    }

    // Functions and their partial derivatives at the prescribed state
    tg_set_vec(vec, u_test);
    as->setVariables(vec);
    as->evalFunctions(2, funcs, fvals);
    w.f64("funcs_test", fvals, 2);
    for (int k = 0; k < 2; k++) {
      dfdu[k]->zeroEntries();
      dfdx[k]->zeroEntries();
    }
    as->addSVSens(1.0, 0.0, 0.0, 2, funcs, dfdu);
    as->addDVSens(1.0, 2, funcs, dfdx);
    dfdu[0]->getArray(&arr);
    w.f64("dfdu_test_comp", arr, ndof);
    dfdu[1]->getArray(&arr);
    w.f64("dfdu_test_ks", arr, ndof);
    int ndv = dfdx[0]->getArray(&arr);
    w.f64("dfdx_test_comp", arr, ndv);
    dfdx[1]->getArray(&arr);
    w.f64("dfdx_test_ks", arr, ndv);

    std::vector<double> &psi_test = tg_fv(p, "psi_test");
    if (!psi_test.empty()) {
      tg_set_vec(psi[0], psi_test);
      dfdx[0]->zeroEntries();
      as->addAdjointResProducts(1.0, 1, psi, dfdx);
      dfdx[0]->getArray(&arr);
      w.f64("adjres_test", arr, ndv);
    }

    // Node-coordinate sensitivities at the prescribed state (exact in the
    // complex build: the shell and load elements difference by complex
    // step, the solid element is analytic)
    for (int k = 0; k < 2; k++) dfdX[k]->zeroEntries();
    as->addXptSens(1.0, 2, funcs, dfdX);
    dfdX[0]->getArray(&arr);
    w.f64("dfdX_test_comp", arr, 3 * m.nnodes);
    dfdX[1]->getArray(&arr);
    w.f64("dfdX_test_ks", arr, 3 * m.nnodes);
    if (!psi_test.empty()) {
      dfdX[0]->zeroEntries();
      as->addAdjointResXptSensProducts(1.0, 1, psi, dfdX);
      dfdX[0]->getArray(&arr);
      w.f64("adjxpt_test", arr, 3 * m.nnodes);
    }
  }

  // ---- 2. linear static solve -------------------------------------------
  int gm = tg_i(p, "gmres_m", 100), gr = tg_i(p, "gmres_restart", 2);
  double rtol = tg_f(p, "rtol", 1e-12), atol = tg_f(p, "atol", 1e-30);
  GMRES *ksm = new GMRES(mat, pc, gm, gr, 0);
  ksm->incref();
  ksm->setTolerances(rtol, atol);

  as->zeroVariables();
  as->assembleJacobian(1.0, 0.0, 0.0, res, mat);
  pc->factor();
  res->getArray(&arr);
  w.f64("res0", arr, ndof);
  as->applyBCs(f);
  res->axpy(-1.0, f);
  int flag = ksm->solve(res, out);
  out->scale(-1.0);
  as->setVariables(out);
  out->getArray(&arr);
  w.f64("u", arr, ndof);
  int iters = ksm->getIterCount();
  w.i32("gmres_iters", &iters, 1);
  w.i32("gmres_flag", &flag, 1);

  // ---- 3. functions, adjoints and total derivatives --------------------
  as->evalFunctions(2, funcs, fvals);
  w.f64("funcs", fvals, 2);
  for (int k = 0; k < 2; k++) {
    dfdu[k]->zeroEntries();
    dfdx[k]->zeroEntries();
  }
  as->addSVSens(1.0, 0.0, 0.0, 2, funcs, dfdu);
  as->addDVSens(1.0, 2, funcs, dfdx);
  int ndv = dfdx[0]->getArray(&arr);
  w.f64("dfdx_partial_comp", arr, ndv);
  dfdx[1]->getArray(&arr);
  w.f64("dfdx_partial_ks", arr, ndv);
  dfdu[0]->getArray(&arr);
  w.f64("dfdu_comp", arr, ndof);
  dfdu[1]->getArray(&arr);
  w.f64("dfdu_ks", arr, ndof);

  as->assembleJacobian(1.0, 0.0, 0.0, NULL, mat, TACS_MAT_TRANSPOSE);
  pc->factor();
  for (int k = 0; k < 2; k++) {
    as->applyBCs(dfdu[k]);
    ksm->solve(dfdu[k], psi[k]);
  }
  psi[0]->getArray(&arr);
  w.f64("psi_comp", arr, ndof);
  psi[1]->getArray(&arr);
  w.f64("psi_ks", arr, ndof);
  as->addAdjointResProducts(-1.0, 2, psi, dfdx);
  dfdx[0]->getArray(&arr);
  w.f64("grad_comp", arr, ndv);
  dfdx[1]->getArray(&arr);
  w.f64("grad_ks", arr, ndv);

  // total node-coordinate derivatives df/dX - psi^T dR/dX at the solution
  for (int k = 0; k < 2; k++) dfdX[k]->zeroEntries();
  as->addXptSens(1.0, 2, funcs, dfdX);
  as->addAdjointResXptSensProducts(-1.0, 2, psi, dfdX);
  dfdX[0]->getArray(&arr);
  w.f64("grad_xpt_comp", arr, 3 * m.nnodes);
  dfdX[1]->getArray(&arr);
  w.f64("grad_xpt_ks", arr, 3 * m.nnodes);

  TacsFinalize();
  MPI_Finalize();
  return 0;
}
