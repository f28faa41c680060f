/*
  Per-element operation counts of the reference's element routines on the
  checked path, from the counting flavour of the reference build
  (make -C oracle/ref opc; the scalar is oracle/ref/opcount.h).  Test
  infrastructure only: its output is the algorithmic FP64 work per element
  that the GPU kernels' FP64 roofline is quoted against.

  Calls, on one element with generic (seeded, non-degenerate) inputs:
    MITC4 shell (TACSQuad4Shell, TACSIsoShellConstitutive, natural
    transform): addResidual, addJacobian (alpha 1, beta = gamma = 0: the
    call TACSAssembler::assembleJacobian makes), addAdjResProduct, and at
    each of the 4 quadrature points evalPointQuantity /
    addPointQuantitySVSens / addPointQuantityDVSens for the strain energy
    density (compliance) and the failure index (KS failure);
    hex8 (TACSElement3D, TACSLinearElasticity3D, TACSLinearHexaBasis,
    TACSSolidConstitutive): the same calls at its 8 points;
    the shell pressure load (TACSShellPressure) residual.

  Prints one line per routine: name, add, mul, div, sqrt, transcendental,
  and flops = add + mul + div + sqrt.

    make -C oracle/ref opc && oracle/_ref/op_count
*/
#include <cstdio>
#include <cstring>
#include <vector>

#include "TACSElement3D.h"
#include "TACSElementTypes.h"
#include "TACSHexaBasis.h"
#include "TACSIsoShellConstitutive.h"
#include "TACSLinearElasticity.h"
#include "TACSShellElementDefs.h"
#include "TACSSolidConstitutive.h"

TgOpCounts tg_opcounts;

namespace {

void reset() { memset(&tg_opcounts, 0, sizeof(tg_opcounts)); }

void report(const char *name) {
  const TgOpCounts &c = tg_opcounts;
  printf("%-28s %8llu %8llu %6llu %5llu %5llu %9llu\n", name, c.add, c.mul,
         c.div, c.sqrt, c.transc, c.add + c.mul + c.div + c.sqrt);
}

// Deterministic generator for the inputs (values do not change the counts
// of these branch-free element routines beyond degenerate inputs)
struct Lcg {
  unsigned long long s;
  double next() {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(s >> 11) / 9007199254740992.0;
  }
};

void count_element(const char *tag, TACSElement *elem, int nnodes, int vpn,
                   const double *xyz, Lcg &g) {
  const int nv = nnodes * vpn;
  std::vector<TacsScalar> X(3 * nnodes), u(nv), ud(nv, 0.0), udd(nv, 0.0),
      res(nv), mat(nv * nv), psi(nv), dfdx(1), dfdu(nv);
  for (int i = 0; i < 3 * nnodes; i++) X[i] = xyz[i] + 0.01 * g.next();
  for (int i = 0; i < nv; i++) {
    u[i] = 1e-3 * (g.next() - 0.5);
    psi[i] = g.next() - 0.5;
  }
  char name[64];

  reset();
  elem->addResidual(0, 0.0, X.data(), u.data(), ud.data(), udd.data(),
                    res.data());
  snprintf(name, sizeof(name), "%s addResidual", tag);
  report(name);

  reset();
  elem->addJacobian(0, 0.0, 1.0, 0.0, 0.0, X.data(), u.data(), ud.data(),
                    udd.data(), res.data(), mat.data());
  snprintf(name, sizeof(name), "%s addJacobian", tag);
  report(name);

  reset();
  dfdx[0] = 0.0;
  elem->addAdjResProduct(0, 0.0, 1.0, psi.data(), X.data(), u.data(),
                         ud.data(), udd.data(), 1, dfdx.data());
  snprintf(name, sizeof(name), "%s addAdjResProduct", tag);
  report(name);

  // the function integrands at every quadrature point
  const int quantities[2] = {TACS_STRAIN_ENERGY_DENSITY, TACS_FAILURE_INDEX};
  const char *qname[2] = {"energy", "failure"};
  const int nq = elem->getNumQuadraturePoints();
  for (int k = 0; k < 2; k++) {
    TacsScalar detXd, q;
    TacsScalar dfdq = 1.0;
    reset();
    for (int p = 0; p < nq; p++) {
      double pt[3];
      elem->getQuadraturePoint(p, pt);
      elem->evalPointQuantity(0, quantities[k], 0.0, p, pt, X.data(),
                              u.data(), ud.data(), udd.data(), &detXd, &q);
    }
    snprintf(name, sizeof(name), "%s %s values", tag, qname[k]);
    report(name);
    reset();
    for (int p = 0; p < nq; p++) {
      double pt[3];
      elem->getQuadraturePoint(p, pt);
      elem->addPointQuantitySVSens(0, quantities[k], 0.0, 1.0, 0.0, 0.0, p,
                                   pt, X.data(), u.data(), ud.data(),
                                   udd.data(), &dfdq, dfdu.data());
    }
    snprintf(name, sizeof(name), "%s %s SVSens", tag, qname[k]);
    report(name);
    reset();
    for (int p = 0; p < nq; p++) {
      double pt[3];
      elem->getQuadraturePoint(p, pt);
      elem->addPointQuantityDVSens(0, quantities[k], 0.0, 1.0, p, pt,
                                   X.data(), u.data(), ud.data(), udd.data(),
                                   &dfdq, 1, dfdx.data());
    }
    snprintf(name, sizeof(name), "%s %s DVSens", tag, qname[k]);
    report(name);
  }
}

}  // namespace

int main() {
  TacsInitialize();
  Lcg g = {12345};
  printf("%-28s %8s %8s %6s %5s %5s %9s\n", "routine (per element)", "add",
         "mul", "div", "sqrt", "trans", "flops");

  TACSMaterialProperties *props =
      new TACSMaterialProperties(2700.0, 0.0, 70e9, 0.3, 2.7e8, 0.0, 0.0);
  props->incref();

  // MITC4 shell, a unit square in a general plane
  TACSShellTransform *tr = new TACSShellNaturalTransform();
  tr->incref();
  TACSShellConstitutive *scon =
      new TACSIsoShellConstitutive(props, 0.01, 0, 0.0, 10.0);
  TACSElement *shell = new TACSQuad4Shell(tr, scon);
  shell->incref();
  const double quad[12] = {0.0, 0.0, 0.0,  1.0, 0.1, 0.05,
                           0.05, 1.0, 0.1, 1.1, 1.05, 0.2};
  count_element("shell", shell, 4, 6, quad, g);

  // shell pressure load (per-node pressures)
  TacsScalar pn[4] = {1e3, 1.1e3, 0.9e3, 1.05e3};
  TACSElement *pres =
      new TACSShellPressure<6, TACSQuadLinearQuadrature,
                            TACSShellQuadBasis<2> >(pn);
  pres->incref();
  {
    std::vector<TacsScalar> X(quad, quad + 12), u(24, 0.0), res(24, 0.0);
    reset();
    pres->addResidual(0, 0.0, X.data(), u.data(), u.data(), u.data(),
                      res.data());
    report("shell pressure addResidual");
  }

  // hex8, a unit cube
  TACSElementBasis *basis = new TACSLinearHexaBasis();
  basis->incref();
  TACSSolidConstitutive *hcon =
      new TACSSolidConstitutive(props, 1.0, 0, 0.0, 10.0);
  TACSLinearElasticity3D *model =
      new TACSLinearElasticity3D(hcon, TACS_LINEAR_STRAIN);
  TACSElement *hex = new TACSElement3D(model, basis);
  hex->incref();
  double cube[24];
  for (int k = 0; k < 8; k++) {
    cube[3 * k] = (k & 1) ? 1.0 : 0.0;
    cube[3 * k + 1] = (k & 2) ? 1.0 : 0.0;
    cube[3 * k + 2] = (k & 4) ? 1.0 : 0.0;
  }
  count_element("hex", hex, 8, 3, cube, g);

  shell->decref();
  pres->decref();
  hex->decref();
  basis->decref();
  tr->decref();
  props->decref();
  TacsFinalize();
  return 0;
}
