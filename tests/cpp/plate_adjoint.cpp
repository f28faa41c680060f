// Static analysis with adjoint gradients through the C++ interface
// (include/tacs_gb300.hpp), written the way a TACS C++ driver does it
// (examples/plate/plate.cpp with the solve and adjoint recipe of
// tests/integration_tests/static_analysis_base_test.py:359-427): the
// 32 x 32 clamped MITC4 plate under 1e3 Pa, t = 0.01, one thickness design
// variable per element.  Prints one JSON object: the compliance, the KS
// failure value and both gradients.  With the argument "direct" both
// solves use TACSSchurPc (the complete factorisation) instead of GMRES
// with ILU(0).
#include <cstdio>
#include <string>
#include <vector>

#include "tacs_gb300.hpp"

using namespace tacs_gb300;

int main(int argc, char **argv) {
  const bool direct = argc > 1 && std::string(argv[1]) == "direct";
  const int n = 32, nx = n + 1, nnodes = nx * nx, nelems = n * n;
  std::vector<int> ptr(nelems + 1), conn(4 * nelems);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      const int e = i + n * j, n0 = i + nx * j;
      conn[4 * e] = n0;
      conn[4 * e + 1] = n0 + 1;
      conn[4 * e + 2] = n0 + nx;
      conn[4 * e + 3] = n0 + nx + 1;
    }
  for (int e = 0; e <= nelems; e++) ptr[e] = 4 * e;

  TACSAssembler assembler(6, nnodes, nelems);
  assembler.setElementConnectivity(ptr.data(), conn.data());
  TACSElementSpec spec;
  spec.elem_type = TG_ELEM_MITC4;
  spec.rho = 2700.0;
  spec.E = 70e9;
  spec.nu = 0.3;
  spec.ys = 2.7e8;
  spec.t.assign(nelems, 0.01);
  for (int e = 0; e < nelems; e++) spec.tNum.push_back(e);
  assembler.setElements(spec);
  std::vector<int> edge;
  for (int k = 0; k < nnodes; k++) {
    const int i = k % nx, j = k / nx;
    if (i == 0 || j == 0 || i == n || j == n) edge.push_back(k);
  }
  assembler.addBCs((int)edge.size(), edge.data());
  TACSAuxElements aux;
  const double p[4] = {1e3, 1e3, 1e3, 1e3};
  for (int e = 0; e < nelems; e++) aux.addPressure(e, p);
  assembler.setAuxElements(aux);
  assembler.initialize();

  TACSBVec *X = assembler.createNodeVec();
  std::vector<double> xyz(3 * nnodes);
  for (int k = 0; k < nnodes; k++) {
    xyz[3 * k] = (k % nx) / (double)n;
    xyz[3 * k + 1] = (k / nx) / (double)n;
    xyz[3 * k + 2] = 0.0;
  }
  X->setValues(xyz.data());
  assembler.setNodes(X);

  TACSBVec *res = assembler.createVec(), *ans = assembler.createVec();
  BCSRMat *mat = assembler.createMat();
  assembler.zeroVariables();
  assembler.assembleJacobian(1.0, 0.0, 0.0, res, mat);
  TACSAdditiveSchwarz pc(mat, 0, 10.0);
  pc.factor();
  GMRES gmres(mat, &pc, 300, 10, 0);
  gmres.setTolerances(1e-12, 1e-30);
  TACSSchurPc *schur = nullptr;
  if (direct) {
    schur = new TACSSchurPc(mat);
    schur->factor();
  }
  auto solve = [&](TACSBVec *b, TACSBVec *x) {
    if (!direct) return gmres.solve(b, x);
    schur->applyFactor(b, x);
    return 1;
  };
  const int flag = solve(res, ans);
  ans->scale(-1.0);
  assembler.setVariables(ans);

  TACSCompliance comp(&assembler);
  TACSKSFailure ks(&assembler, 100.0);
  TACSFunction *funcs[2] = {&comp, &ks};
  double fvals[2];
  assembler.evalFunctions(2, funcs, fvals);

  std::vector<double> grads[2], gradX[2];
  for (int k = 0; k < 2; k++) {
    TACSBVec *dfdu = assembler.createVec(), *psi = assembler.createVec();
    TACSBVec *dfdx = assembler.createDesignVec();
    TACSBVec *dfdX = assembler.createNodeVec();
    assembler.addSVSens(1.0, 0.0, 0.0, 1, &funcs[k], &dfdu);
    assembler.applyBCs(dfdu);
    solve(dfdu, psi);
    assembler.addDVSens(1.0, 1, &funcs[k], &dfdx);
    assembler.addAdjointResProducts(-1.0, 1, &psi, &dfdx);
    assembler.addXptSens(1.0, 1, &funcs[k], &dfdX);
    assembler.addAdjointResXptSensProducts(-1.0, 1, &psi, &dfdX);
    grads[k].resize(dfdx->getSize());
    dfdx->getValues(grads[k].data());
    gradX[k].resize(dfdX->getSize());
    dfdX->getValues(gradX[k].data());
    delete dfdu;
    delete psi;
    delete dfdx;
    delete dfdX;
  }
  std::printf("{\"flag\": %d, \"funcs\": [%.17g, %.17g]", flag, fvals[0],
              fvals[1]);
  for (int k = 0; k < 2; k++) {
    std::printf(", \"grad%d\": [", k);
    for (size_t i = 0; i < grads[k].size(); i++)
      std::printf("%s%.17g", i ? ", " : "", grads[k][i]);
    std::printf("]");
    std::printf(", \"gradX%d\": [", k);
    for (size_t i = 0; i < gradX[k].size(); i++)
      std::printf("%s%.17g", i ? ", " : "", gradX[k][i]);
    std::printf("]");
  }
  std::printf("}\n");
  delete schur;
  delete X;
  delete res;
  delete ans;
  delete mat;
  return 0;
}
