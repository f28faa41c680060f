/*
  CPU timing of the reference TACS library (oracle/_ref) on one problem
  file: the baseline the GPU path is compared with on this machine's host
  cores.  Test infrastructure only.

  usage: ref_bench problem.bin nthreads reps [xpt]

  Times, best of `reps` after one warm-up call, with std::chrono around
  each reference call and the assembler's own threads
  (TACSAssembler::setNumThreads):
    assembleJacobian(1, 0, 0, res, mat)   residual + Jacobian assembly
    assembleRes(res)                      residual only
  and with a fourth argument also the node-coordinate products
    addXptSens(compliance) and addAdjointResXptSensProducts(psi)
  at a seeded state (the reference runs these serially).
  Prints one JSON line.
*/
#include <chrono>
#include <random>

#include "ref_problem.h"

template <class F>
static double best_ms(int reps, F &&f) {
  f();
  double best = 1e30;
  for (int r = 0; r < reps; r++) {
    auto t0 = std::chrono::steady_clock::now();
    f();
    auto t1 = std::chrono::steady_clock::now();
    double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (ms < best) best = ms;
  }
  return best;
}

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  TacsInitialize();
  if (argc < 4) {
    fprintf(stderr, "usage: %s problem.bin nthreads reps [xpt]\n", argv[0]);
    return 1;
  }
  TgFile p = tg_read(argv[1]);
  const int nthreads = atoi(argv[2]), reps = atoi(argv[3]);
  const bool xpt = argc > 4;
  RefModel m = tg_build_model(p);
  TACSAssembler *as = m.assembler;
  as->setNumThreads(nthreads);

  TACSBVec *res = as->createVec();
  res->incref();
  TACSParallelMat *mat = as->createMat();
  mat->incref();
  const double jac_ms = best_ms(reps, [&] {
    as->assembleJacobian(1.0, 0.0, 0.0, res, mat);
  });
  const double res_ms = best_ms(reps, [&] { as->assembleRes(res); });
  printf("{\"threads\": %d, \"elements\": %d, \"assemble_jacobian_ms\": %.3f, "
         "\"assemble_res_ms\": %.3f, \"elements_per_s\": %.1f",
         nthreads, m.nelem, jac_ms, res_ms, m.nelem / (jac_ms * 1e-3));

  if (xpt) {
    // seeded state and adjoint of unit scale
    std::mt19937_64 gen(7);
    std::normal_distribution<double> nd(0.0, 1.0);
    TACSBVec *u = as->createVec(), *psi = as->createVec();
    u->incref();
    psi->incref();
    TacsScalar *ua, *pa;
    const int n = u->getArray(&ua);
    psi->getArray(&pa);
    for (int k = 0; k < n; k++) {
      ua[k] = 1e-4 * nd(gen);
      pa[k] = nd(gen);
    }
    as->setVariables(u);
    TACSFunction *comp = new TACSCompliance(as);
    comp->incref();
    TacsScalar fval;
    as->evalFunctions(1, &comp, &fval);
    TACSBVec *dX = as->createNodeVec();
    dX->incref();
    const double xs_ms = best_ms(1, [&] {
      dX->zeroEntries();
      as->addXptSens(1.0, 1, &comp, &dX);
    });
    const double xa_ms = best_ms(1, [&] {
      dX->zeroEntries();
      as->addAdjointResXptSensProducts(1.0, 1, &psi, &dX);
    });
    printf(", \"add_xpt_sens_ms\": %.3f, \"add_adjoint_res_xpt_ms\": %.3f",
           xs_ms, xa_ms);
  }
  printf("}\n");
  TacsFinalize();
  MPI_Finalize();
  return 0;
}
