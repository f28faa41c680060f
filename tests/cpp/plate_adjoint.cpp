// Static analysis with adjoint gradients through the C++ interface
// (include/tacs_gb300.hpp), written with the reference's classes and call
// pattern (an MPI communicator, per-element TACSIsoShellConstitutive /
// TACSQuad4Shell objects through setElements(TACSElement **), TACSShellPressure
// auxiliary elements, createMat / createSchurMat, TACSAdditiveSchwarz or
// TACSSchurPc inside GMRES, incref / decref; the order of examples/plate/
// plate.cpp and of the solve and adjoint recipe of tests/integration_tests/
// static_analysis_base_test.py:359-427): the 32 x 32 clamped MITC4 plate
// under 1e3 Pa, t = 0.01, one thickness design variable per element.
// Prints one JSON object: the compliance, the KS failure value and both
// gradients (thickness and node coordinates).  With the argument "direct"
// the solves use TACSSchurPc (the complete factorisation) as GMRES's
// preconditioner instead of ILU(0).
#include <cstdio>
#include <cstring>
#include <vector>

#include "tacs_gb300.hpp"

using namespace tacs_gb300;

int main(int argc, char **argv) {
  const bool direct = argc > 1 && std::strcmp(argv[1], "direct") == 0;
  MPI_Comm comm = MPI_COMM_WORLD;
  const int n = 32, nx = n + 1, numNodes = nx * nx, numElements = n * n;
  const int varsPerNode = 6;

  TACSAssembler *assembler =
      new TACSAssembler(comm, varsPerNode, numNodes, numElements);
  assembler->incref();

  int *ptr = new int[numElements + 1];
  int *conn = new int[4 * numElements];
  ptr[0] = 0;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      const int e = i + n * j, n0 = i + nx * j;
      conn[4 * e] = n0;
      conn[4 * e + 1] = n0 + 1;
      conn[4 * e + 2] = n0 + nx;
      conn[4 * e + 3] = n0 + nx + 1;
      ptr[e + 1] = 4 * (e + 1);
    }
  assembler->setElementConnectivity(ptr, conn);
  delete[] conn;
  delete[] ptr;

  TacsScalar rho = 2700.0, specific_heat = 0.0, E = 70e9, nu = 0.3;
  TacsScalar ys = 2.7e8, cte = 0.0, kappa = 0.0;
  TACSMaterialProperties *props =
      new TACSMaterialProperties(rho, specific_heat, E, nu, ys, cte, kappa);
  TACSShellTransform *transform = new TACSShellNaturalTransform();
  TACSElement **elements = new TACSElement *[numElements];
  for (int e = 0; e < numElements; e++) {
    TACSShellConstitutive *con = new TACSIsoShellConstitutive(props, 0.01, e);
    elements[e] = new TACSQuad4Shell(transform, con);
  }
  assembler->setElements(elements);
  delete[] elements;

  std::vector<int> edge;
  for (int k = 0; k < numNodes; k++) {
    const int i = k % nx, j = k / nx;
    if (i == 0 || j == 0 || i == n || j == n) edge.push_back(k);
  }
  assembler->addBCs((int)edge.size(), edge.data());

  TACSAuxElements *aux = new TACSAuxElements(numElements);
  TACSElement *pressure = new TACSShellPressure(1e3);
  for (int e = 0; e < numElements; e++) aux->addElement(e, pressure);
  assembler->setAuxElements(aux);

  if (assembler->initialize() != 0) {
    assembler->decref();
    return 1;
  }

  TACSBVec *X = assembler->createNodeVec();
  X->incref();
  std::vector<TacsScalar> xyz(3 * numNodes);
  for (int k = 0; k < numNodes; k++) {
    xyz[3 * k] = (k % nx) / (double)n;
    xyz[3 * k + 1] = (k / nx) / (double)n;
    xyz[3 * k + 2] = 0.0;
  }
  X->copyFromHost(xyz.data());
  assembler->setNodes(X);

  TACSBVec *res = assembler->createVec();
  TACSBVec *ans = assembler->createVec();
  res->incref();
  ans->incref();

  TACSParallelMat *mat =
      direct ? assembler->createSchurMat() : assembler->createMat();
  mat->incref();
  TACSPc *pc = nullptr;
  if (direct)
    pc = new TACSSchurPc(static_cast<TACSSchurMat *>(mat), 1000, 10.0, 1);
  else
    pc = new TACSAdditiveSchwarz(mat, 0, 10.0);
  pc->incref();
  GMRES *gmres = new GMRES(mat, pc, 300, 10, 0);
  gmres->incref();
  gmres->setTolerances(1e-12, 1e-30);

  assembler->zeroVariables();
  assembler->assembleJacobian(1.0, 0.0, 0.0, res, mat);
  pc->factor();
  const int flag = gmres->solve(res, ans);
  ans->scale(-1.0);
  assembler->setVariables(ans);

  TACSFunction *funcs[2] = {new TACSCompliance(assembler),
                            new TACSKSFailure(assembler, 100.0)};
  for (TACSFunction *f : funcs) f->incref();
  TacsScalar fvals[2];
  assembler->evalFunctions(2, funcs, fvals);

  std::vector<TacsScalar> grads[2], gradX[2];
  for (int k = 0; k < 2; k++) {
    TACSBVec *dfdu = assembler->createVec(), *psi = assembler->createVec();
    TACSBVec *dfdx = assembler->createDesignVec();
    TACSBVec *dfdX = assembler->createNodeVec();
    for (TACSBVec *v : {dfdu, psi, dfdx, dfdX}) v->incref();
    assembler->addSVSens(1.0, 0.0, 0.0, 1, &funcs[k], &dfdu);
    assembler->applyBCs(dfdu);
    gmres->solve(dfdu, psi);
    assembler->addDVSens(1.0, 1, &funcs[k], &dfdx);
    assembler->addAdjointResProducts(-1.0, 1, &psi, &dfdx);
    assembler->addXptSens(1.0, 1, &funcs[k], &dfdX);
    assembler->addAdjointResXptSensProducts(-1.0, 1, &psi, &dfdX);
    int size;
    dfdx->getSize(&size);
    grads[k].resize(size);
    dfdx->copyToHost(grads[k].data());
    dfdX->getSize(&size);
    gradX[k].resize(size);
    dfdX->copyToHost(gradX[k].data());
    for (TACSBVec *v : {dfdu, psi, dfdx, dfdX}) v->decref();
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
  for (TACSFunction *f : funcs) f->decref();
  gmres->decref();
  pc->decref();
  mat->decref();
  ans->decref();
  res->decref();
  X->decref();
  assembler->decref();
  return 0;
}
