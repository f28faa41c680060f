/*
  Problem-file reader and reference-TACS model builder shared by the checker
  drivers (gen_golden.cpp, ref_bench.cpp).  Test infrastructure only: these
  drivers run the reference TACS library (built from the reference sources by
  this directory's Makefile) to produce golden vectors and CPU timings.

  Problem files are a flat list of named 1-D arrays ("tgarr" format):
    repeat { char name[32]; int32 dtype (0 = f64, 1 = i32); int64 count;
             raw little-endian data }
  They are written by tests/golden/make_golden.py (numpy) and read here.

  The model is built the way the reference's own drivers and tests build it
  (examples/benchmark/benchmark.cpp, tests/integration_tests/
  static_analysis_base_test.py): one constitutive object per element so that
  every element owns one design variable, a TACSAssembler over the given
  connectivity, TACSAuxElements for pressure / traction loads.
*/
#ifndef ORACLE_REF_PROBLEM_H
#define ORACLE_REF_PROBLEM_H

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "TACSAssembler.h"
#include "TACSAuxElements.h"
#include "TACSCompliance.h"
#include "TACSElement3D.h"
#include "TACSHexaBasis.h"
#include "TACSIsoShellConstitutive.h"
#include "TACSKSFailure.h"
#include "TACSLinearElasticity.h"
#include "TACSShellElementDefs.h"
#include "TACSSolidConstitutive.h"
#include "TACSTraction3D.h"

struct TgArray {
  int dtype;  // 0 = f64, 1 = i32
  std::vector<double> f;
  std::vector<int> i;
};

typedef std::map<std::string, TgArray> TgFile;

static inline TgFile tg_read(const char *path) {
  TgFile out;
  FILE *fp = fopen(path, "rb");
  if (!fp) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  char name[33];
  while (fread(name, 1, 32, fp) == 32) {
    name[32] = 0;
    int32_t dtype;
    int64_t count;
    if (fread(&dtype, 4, 1, fp) != 1 || fread(&count, 8, 1, fp) != 1) break;
    TgArray a;
    a.dtype = dtype;
    if (dtype == 0) {
      a.f.resize(count);
      if (count && fread(a.f.data(), 8, count, fp) != (size_t)count) exit(3);
    } else {
      a.i.resize(count);
      if (count && fread(a.i.data(), 4, count, fp) != (size_t)count) exit(3);
    }
    out[std::string(name)] = a;
  }
  fclose(fp);
  return out;
}

struct TgWriter {
  FILE *fp;
  explicit TgWriter(const char *path) {
    fp = fopen(path, "wb");
    if (!fp) {
      fprintf(stderr, "cannot write %s\n", path);
      exit(2);
    }
  }
  ~TgWriter() { fclose(fp); }
  void head(const char *name, int dtype, int64_t count) {
    char buf[32];
    memset(buf, 0, 32);
    strncpy(buf, name, 31);
    fwrite(buf, 1, 32, fp);
    int32_t d = dtype;
    fwrite(&d, 4, 1, fp);
    fwrite(&count, 8, 1, fp);
  }
  void f64(const char *name, const TacsScalar *x, int64_t n) {
    head(name, 0, n);
    for (int64_t k = 0; k < n; k++) {
      double v = TacsRealPart(x[k]);
      fwrite(&v, 8, 1, fp);
    }
  }
  void f64im(const char *name, const TacsScalar *x, int64_t n) {
    head(name, 0, n);
    for (int64_t k = 0; k < n; k++) {
      double v = TacsImagPart(x[k]);
      fwrite(&v, 8, 1, fp);
    }
  }
  void i32(const char *name, const int *x, int64_t n) {
    head(name, 1, n);
    fwrite(x, 4, n, fp);
  }
  void scalar(const char *name, double v) {
    head(name, 0, 1);
    fwrite(&v, 8, 1, fp);
  }
};

static inline double tg_f(TgFile &p, const char *name, double def) {
  auto it = p.find(name);
  if (it == p.end() || it->second.f.empty()) return def;
  return it->second.f[0];
}
static inline int tg_i(TgFile &p, const char *name, int def) {
  auto it = p.find(name);
  if (it == p.end() || it->second.i.empty()) return def;
  return it->second.i[0];
}
static inline std::vector<double> &tg_fv(TgFile &p, const char *name) {
  return p[name].f;
}
static inline std::vector<int> &tg_iv(TgFile &p, const char *name) {
  return p[name].i;
}

/*
  Problem keys (all optional unless noted):
    elem_type (i32: 0 = MITC4 shell / TACSQuad4Shell, 1 = hex8)   required
    nnodes, nelem (i32)                                          required
    xpts (f64, 3*nnodes), conn (i32, npe*nelem)                  required
    mat (f64: rho, E, nu, ys)                                    required
    thick (f64, nelem)      per-element t (shell) or t (solid)
    dvnum (i32, nelem)      design-variable number per element (-1: fixed)
    transform (i32: 0 natural, 1 reference axis), ref_axis (f64, 3)
    bc_nodes, bc_masks (i32)  Dirichlet nodes and dof bit masks
    pres_elems (i32), pres_vals (f64, 4 per element)  shell pressure loads
    trac_elems, trac_faces (i32), trac_vals (f64, 3 per face)  hex tractions
    force (f64, vpn*nnodes)  nodal force vector f (R = K u - f)
    ks_weight (f64)
*/
struct RefModel {
  TACSAssembler *assembler;
  int elem_type, vpn, npe, nnodes, nelem;
  std::vector<double> force;
};

static inline RefModel tg_build_model(TgFile &p) {
  RefModel m;
  m.elem_type = tg_i(p, "elem_type", 0);
  m.nnodes = tg_i(p, "nnodes", 0);
  m.nelem = tg_i(p, "nelem", 0);
  m.vpn = (m.elem_type == 0) ? 6 : 3;
  m.npe = (m.elem_type == 0) ? 4 : 8;

  std::vector<double> &mat = tg_fv(p, "mat");
  TACSMaterialProperties *props =
      new TACSMaterialProperties(mat[0], 0.0, mat[1], mat[2], mat[3], 0.0, 0.0);
  props->incref();

  std::vector<double> &thick = tg_fv(p, "thick");
  std::vector<int> &dvnum = tg_iv(p, "dvnum");

  TACSShellTransform *transform = NULL;
  if (m.elem_type == 0) {
    if (tg_i(p, "transform", 0) == 1) {
      std::vector<double> &ax = tg_fv(p, "ref_axis");
      TacsScalar axis[3] = {ax[0], ax[1], ax[2]};
      transform = new TACSShellRefAxisTransform(axis);
    } else {
      transform = new TACSShellNaturalTransform();
    }
    transform->incref();
  }
  TACSElementBasis *hexbasis = new TACSLinearHexaBasis();
  hexbasis->incref();

  std::vector<TACSElement *> elems(m.nelem);
  for (int e = 0; e < m.nelem; e++) {
    TacsScalar t = thick.empty() ? 1.0 : thick[e];
    int tnum = dvnum.empty() ? -1 : dvnum[e];
    if (m.elem_type == 0) {
      TACSShellConstitutive *con =
          new TACSIsoShellConstitutive(props, t, tnum, 0.0, 10.0);
      elems[e] = new TACSQuad4Shell(transform, con);
    } else {
      TACSSolidConstitutive *con =
          new TACSSolidConstitutive(props, t, tnum, 0.0, 10.0);
      TACSLinearElasticity3D *model =
          new TACSLinearElasticity3D(con, TACS_LINEAR_STRAIN);
      elems[e] = new TACSElement3D(model, hexbasis);
    }
  }

  m.assembler = new TACSAssembler(MPI_COMM_WORLD, m.vpn, m.nnodes, m.nelem);
  m.assembler->incref();
  std::vector<int> ptr(m.nelem + 1);
  for (int e = 0; e <= m.nelem; e++) ptr[e] = m.npe * e;
  m.assembler->setElementConnectivity(ptr.data(), tg_iv(p, "conn").data());
  m.assembler->setElements(elems.data());

  std::vector<int> &bcn = tg_iv(p, "bc_nodes");
  std::vector<int> &bcm = tg_iv(p, "bc_masks");
  for (size_t k = 0; k < bcn.size(); k++) {
    int vars[8], nv = 0;
    for (int d = 0; d < m.vpn; d++) {
      if (bcm[k] & (1 << d)) vars[nv++] = d;
    }
    int node = bcn[k];
    m.assembler->addBCs(1, &node, nv, vars);
  }

  // Aux elements: shell pressure (per-node values) and hex face tractions
  TACSAuxElements *aux = new TACSAuxElements();
  std::vector<int> &pe = tg_iv(p, "pres_elems");
  std::vector<double> &pv = tg_fv(p, "pres_vals");
  for (size_t k = 0; k < pe.size(); k++) {
    TacsScalar pn[4] = {pv[4 * k], pv[4 * k + 1], pv[4 * k + 2],
                        pv[4 * k + 3]};
    TACSElement *pres =
        new TACSShellPressure<6, TACSQuadLinearQuadrature,
                              TACSShellQuadBasis<2> >(pn);
    aux->addElement(pe[k], pres);
  }
  std::vector<int> &te = tg_iv(p, "trac_elems");
  std::vector<int> &tf = tg_iv(p, "trac_faces");
  std::vector<double> &tv = tg_fv(p, "trac_vals");
  for (size_t k = 0; k < te.size(); k++) {
    TacsScalar tr[3] = {tv[3 * k], tv[3 * k + 1], tv[3 * k + 2]};
    TACSElement *trac = new TACSTraction3D(3, tf[k], hexbasis, tr);
    aux->addElement(te[k], trac);
  }
  m.assembler->setAuxElements(aux);
  m.assembler->initialize();

  TACSBVec *X = m.assembler->createNodeVec();
  X->incref();
  TacsScalar *xa;
  X->getArray(&xa);
  std::vector<double> &xp = tg_fv(p, "xpts");
  for (int k = 0; k < 3 * m.nnodes; k++) xa[k] = xp[k];
  m.assembler->setNodes(X);
  X->decref();

  m.force = tg_fv(p, "force");
  if (m.force.empty()) m.force.assign((size_t)m.vpn * m.nnodes, 0.0);
  return m;
}

static inline void tg_set_vec(TACSBVec *v, const std::vector<double> &x) {
  TacsScalar *a;
  int n = v->getArray(&a);
  for (int k = 0; k < n; k++) a[k] = (k < (int)x.size()) ? x[k] : 0.0;
}

#endif
