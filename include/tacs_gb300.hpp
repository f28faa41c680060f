/* C++ host interface of libtacs_gb300 with the reference's class and method
   names (src/TACSAssembler.h, src/bpmat/TACSBVec.h, src/bpmat/BCSRMat.h,
   src/bpmat/KSM.h, src/functions/TACSCompliance.h, TACSKSFailure.h), for
   the hot path only: a C++ caller of TACS switches by its includes and the
   namespace.  Header-only; every call goes through the C ABI in
   tacs_gb300.h and runs on the GPU.  Vectors live in device memory
   (getArray() returns the device pointer; setValues / getValues copy from
   / to the host).  One process, one GPU: no MPI communicator.  Failures
   throw tacs_gb300::TACSError with tg_last_error()'s text. */
#ifndef TACS_GB300_HPP
#define TACS_GB300_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "tacs_gb300.h"

namespace tacs_gb300 {

struct TACSError : std::runtime_error {
  explicit TACSError(const std::string &m) : std::runtime_error(m) {}
};

inline int check(int rc, const char *what) {
  if (rc < 0)
    throw TACSError(std::string(what) + ": " + tg_last_error());
  return rc;
}

enum MatrixOrientation { TACS_MAT_NORMAL = 0, TACS_MAT_TRANSPOSE = 1 };

/* TACSBVec: size doubles of device memory (block size bsize). */
class TACSBVec {
 public:
  TACSBVec(int size, int bsize) : n_(size), bsize_(bsize) {
    if (cudaMalloc((void **)&d_, sizeof(double) * (size > 0 ? size : 1)) !=
        cudaSuccess)
      throw TACSError("TACSBVec: cudaMalloc failed");
    zeroEntries();
  }
  ~TACSBVec() { cudaFree(d_); }
  TACSBVec(const TACSBVec &) = delete;
  TACSBVec &operator=(const TACSBVec &) = delete;

  double *getArray() { return d_; }
  const double *getArray() const { return d_; }
  int getSize() const { return n_; }
  int getBlockSize() const { return bsize_; }
  void zeroEntries() { cudaMemset(d_, 0, sizeof(double) * n_); }
  void setValues(const double *host) {
    cudaMemcpy(d_, host, sizeof(double) * n_, cudaMemcpyHostToDevice);
  }
  void getValues(double *host) const {
    cudaMemcpy(host, d_, sizeof(double) * n_, cudaMemcpyDeviceToHost);
  }
  void copyValues(const TACSBVec *x) {
    cudaMemcpy(d_, x->d_, sizeof(double) * n_, cudaMemcpyDeviceToDevice);
  }
  void scale(double a) { check(tg_vec_scale(a, d_, n_, 0), "TACSBVec::scale"); }
  void axpy(double a, const TACSBVec *x) {
    check(tg_vec_axpy(a, x->d_, d_, n_, 0), "TACSBVec::axpy");
  }
  double dot(const TACSBVec *x) const {
    double v = 0.0;
    check(tg_vec_dot(d_, x->d_, n_, &v, 0), "TACSBVec::dot");
    return v;
  }
  double norm() const;

 private:
  int n_, bsize_;
  double *d_ = nullptr;
};
inline double TACSBVec::norm() const {
  const double v = dot(this);
  return v > 0.0 ? std::sqrt(v) : 0.0;
}

/* Element description standing in for the TACSElement objects of
   setElements: TACSQuad4Shell (TACSShellNaturalTransform or
   TACSShellRefAxisTransform) over TACSIsoShellConstitutive, or
   TACSElement3D(TACSLinearElasticity3D, TACSLinearHexaBasis) over
   TACSSolidConstitutive; one material per assembler, per-element t and
   design-variable number tNum. */
struct TACSElementSpec {
  int elem_type = TG_ELEM_MITC4;
  double rho = 2700.0, E = 70e9, nu = 0.3, ys = 3e8;
  int transform = 0;  // shells: 0 natural, 1 reference axis
  double ref_axis[3] = {1.0, 0.0, 0.0};
  std::vector<double> t;   // per element
  std::vector<int> tNum;   // per element (-1: not a design variable)
};

/* TACSAuxElements with TACSShellPressure (4 nodal pressures) and
   TACSTraction3D (face, 3 components) entries. */
class TACSAuxElements {
 public:
  void addPressure(int elem, const double p[4]) {
    pres_elems.push_back(elem);
    for (int k = 0; k < 4; k++) pres_vals.push_back(p[k]);
  }
  void addTraction(int elem, int face, const double t[3]) {
    trac_elems.push_back(elem);
    trac_faces.push_back(face);
    for (int k = 0; k < 3; k++) trac_vals.push_back(t[k]);
  }
  std::vector<int> pres_elems, trac_elems, trac_faces;
  std::vector<double> pres_vals, trac_vals;
};

class TACSAssembler;

/* TACSFunction: TACSCompliance / TACSKSFailure (KS_CONTINUOUS). */
class TACSFunction {
 public:
  explicit TACSFunction(int kind, double ks_weight = 80.0)
      : kind_(kind), ksw_(ks_weight) {}
  int kind() const { return kind_; }
  double ksWeight() const { return ksw_; }

 private:
  int kind_;
  double ksw_;
};
class TACSCompliance : public TACSFunction {
 public:
  explicit TACSCompliance(TACSAssembler *) : TACSFunction(TG_FUNC_COMPLIANCE) {}
};
class TACSKSFailure : public TACSFunction {
 public:
  TACSKSFailure(TACSAssembler *, double ksWeight = 80.0, double alpha = 1.0)
      : TACSFunction(TG_FUNC_KS_FAILURE, ksWeight) {
    (void)alpha;
  }
};

/* BCSRMat / TACSParallelMat with the assembler's non-zero pattern. */
class BCSRMat {
 public:
  explicit BCSRMat(tg_assembler *a) {
    check(tg_mat_create(a, &m_), "createMat");
  }
  ~BCSRMat() { tg_mat_decref(m_); }
  BCSRMat(const BCSRMat &) = delete;
  BCSRMat &operator=(const BCSRMat &) = delete;
  void mult(const TACSBVec *x, TACSBVec *y) {
    check(tg_mat_mult(m_, x->getArray(), y->getArray(), 0), "BCSRMat::mult");
  }
  /* device arrays of the row-major b x b blocks */
  void getArrays(int *bsize, int *nrows, const int **rowp, const int **cols,
                 double **A) {
    check(tg_mat_get_arrays(m_, bsize, nrows, rowp, cols, A),
          "BCSRMat::getArrays");
  }
  tg_mat *handle() { return m_; }

 private:
  tg_mat *m_ = nullptr;
};

/* TACSAdditiveSchwarz(mat, levFill, fill): block ILU(levFill) on the
   computeILUk pattern (levFill = 0: the matrix's own pattern). */
class TACSAdditiveSchwarz {
 public:
  TACSAdditiveSchwarz(BCSRMat *mat, int levFill, double fill,
                      int precision = TG_PREC_FP64) {
    (void)fill;  // the pattern is sized exactly, no fill estimate needed
    check(tg_pc_create_iluk(mat->handle(), levFill, precision, &pc_),
          "TACSAdditiveSchwarz");
  }
  ~TACSAdditiveSchwarz() { tg_pc_decref(pc_); }
  TACSAdditiveSchwarz(const TACSAdditiveSchwarz &) = delete;
  TACSAdditiveSchwarz &operator=(const TACSAdditiveSchwarz &) = delete;
  void factor() { check(tg_pc_factor(pc_, 0), "factor"); }
  void applyFactor(const TACSBVec *x, TACSBVec *y) {
    check(tg_pc_apply(pc_, x->getArray(), y->getArray(), 0), "applyFactor");
  }
  tg_pc *handle() { return pc_; }

 private:
  tg_pc *pc_ = nullptr;
};

/* TACSSchurPc(mat, levFill, fill, reorderSchur) with its default complete
   fill: the reference's direct solve, here the complete multifrontal
   factorisation (tg_direct); applyFactor(x, y) is y = A^-1 x. */
class TACSSchurPc {
 public:
  explicit TACSSchurPc(BCSRMat *mat, int levFill = 1000000,
                       double fill = 10.0, int reorderSchur = 1) {
    (void)fill;
    (void)reorderSchur;
    if (levFill < 1000)
      throw TACSError("TACSSchurPc: only the complete factorisation "
                      "(levFill >= 1000) is on the GPU");
    check(tg_direct_create(mat->handle(), 1, TG_PREC_FP64, &d_),
          "TACSSchurPc");
  }
  ~TACSSchurPc() { tg_direct_decref(d_); }
  TACSSchurPc(const TACSSchurPc &) = delete;
  TACSSchurPc &operator=(const TACSSchurPc &) = delete;
  void factor() { check(tg_direct_factor(d_, 0), "factor"); }
  void applyFactor(const TACSBVec *x, TACSBVec *y) {
    check(tg_direct_solve(d_, x->getArray(), y->getArray(), 0),
          "applyFactor");
  }

 private:
  tg_direct *d_ = nullptr;
};

/* GMRES(mat, pc, m, nrestart, isFlexible); mixed != 0 needs an FP32 pc. */
class GMRES {
 public:
  GMRES(BCSRMat *mat, TACSAdditiveSchwarz *pc, int m, int nrestart,
        int isFlexible = 0, int mixed = 0) {
    (void)isFlexible;
    check(tg_ksm_create(mat->handle(), pc ? pc->handle() : nullptr, m,
                        nrestart, mixed, &k_),
          "GMRES");
  }
  ~GMRES() { tg_ksm_decref(k_); }
  GMRES(const GMRES &) = delete;
  GMRES &operator=(const GMRES &) = delete;
  void setTolerances(double rtol, double atol) {
    check(tg_ksm_set_tolerances(k_, rtol, atol), "setTolerances");
  }
  int solve(const TACSBVec *b, TACSBVec *x, int zero_guess = 1) {
    return check(tg_ksm_solve(k_, b->getArray(), x->getArray(), zero_guess,
                              &iters_, &resnorm_, 0),
                 "GMRES::solve");
  }
  int getIterCount() const { return iters_; }
  double getResidualNorm() const { return resnorm_; }

 private:
  tg_ksm *k_ = nullptr;
  int iters_ = 0;
  double resnorm_ = 0.0;
};

/* TACSAssembler (one process). */
class TACSAssembler {
 public:
  TACSAssembler(int varsPerNode, int numOwnedNodes, int numElements)
      : vpn_(varsPerNode), nnodes_(numOwnedNodes), nelems_(numElements) {}
  ~TACSAssembler() {
    delete vars_;
    if (a_) tg_assembler_decref(a_);
  }
  TACSAssembler(const TACSAssembler &) = delete;
  TACSAssembler &operator=(const TACSAssembler &) = delete;

  int setElementConnectivity(const int *ptr, const int *conn) {
    conn_.clear();
    for (int e = 0; e < nelems_; e++)
      for (int k = ptr[e]; k < ptr[e + 1]; k++) conn_.push_back(conn[k]);
    return 0;
  }
  int setElements(const TACSElementSpec &spec) {
    spec_ = spec;
    return 0;
  }
  void addBCs(int nnodes, const int *nodes, int nbcs = -1,
              const int *vars = nullptr) {
    int mask = 0;
    if (nbcs < 0) mask = (1 << vpn_) - 1;
    else
      for (int k = 0; k < nbcs; k++) mask |= 1 << vars[k];
    for (int i = 0; i < nnodes; i++) {
      bc_nodes_.push_back(nodes[i]);
      bc_masks_.push_back(mask);
    }
  }
  void setAuxElements(const TACSAuxElements &aux) { aux_ = aux; }
  int initialize() {
    check(tg_assembler_create(spec_.elem_type, nnodes_, nelems_, conn_.data(),
                              spec_.rho, spec_.E, spec_.nu, spec_.ys,
                              spec_.transform, spec_.ref_axis, &a_),
          "TACSAssembler");
    check(tg_assembler_add_bcs(a_, (int)bc_nodes_.size(), bc_nodes_.data(),
                               bc_masks_.data()),
          "addBCs");
    check(tg_assembler_set_element_dvs(a_, spec_.t.data(), spec_.tNum.data()),
          "setElements");
    if (!aux_.pres_elems.empty())
      check(tg_assembler_set_pressure(a_, (int)aux_.pres_elems.size(),
                                      aux_.pres_elems.data(),
                                      aux_.pres_vals.data()),
            "TACSShellPressure");
    if (!aux_.trac_elems.empty())
      check(tg_assembler_set_traction(a_, (int)aux_.trac_elems.size(),
                                      aux_.trac_elems.data(),
                                      aux_.trac_faces.data(),
                                      aux_.trac_vals.data()),
            "TACSTraction3D");
    check(tg_assembler_initialize(a_), "initialize");
    int vpn, nn, ne, ndv, nc;
    check(tg_assembler_get_sizes(a_, &vpn, &nn, &ne, &ndv, &nc), "sizes");
    ndv_ = ndv;
    vars_ = createVec();
    return 0;
  }
  TACSBVec *createVec() { return new TACSBVec(vpn_ * nnodes_, vpn_); }
  TACSBVec *createNodeVec() { return new TACSBVec(3 * nnodes_, 3); }
  TACSBVec *createDesignVec() { return new TACSBVec(ndv_, 1); }
  BCSRMat *createMat() { return new BCSRMat(a_); }
  int getVarsPerNode() const { return vpn_; }
  int getNumOwnedNodes() const { return nnodes_; }
  int getNumElements() const { return nelems_; }

  void setNodes(TACSBVec *X) {
    check(tg_assembler_set_nodes(a_, X->getArray(), 0), "setNodes");
  }
  void setDesignVars(TACSBVec *x) {
    check(tg_assembler_set_design_vars(a_, x->getArray(), 0),
          "setDesignVars");
  }
  void setVariables(TACSBVec *q) { vars_->copyValues(q); }
  void getVariables(TACSBVec *q) { q->copyValues(vars_); }
  void zeroVariables() { vars_->zeroEntries(); }
  void applyBCs(TACSBVec *v) {
    check(tg_apply_bcs(a_, v->getArray(), 0), "applyBCs");
  }

  void assembleRes(TACSBVec *res, double lambda = 1.0, bool applyBCs = true) {
    check(tg_assemble_res(a_, vars_->getArray(), lambda, applyBCs ? 1 : 0,
                          res->getArray(), 0),
          "assembleRes");
  }
  void assembleJacobian(double alpha, double beta, double gamma, TACSBVec *res,
                        BCSRMat *A,
                        MatrixOrientation matOr = TACS_MAT_NORMAL,
                        double lambda = 1.0, bool applyBCs = true) {
    check(tg_assemble_jacobian(a_, alpha, beta, gamma, vars_->getArray(),
                               res ? res->getArray() : nullptr, A->handle(),
                               (int)matOr, lambda, applyBCs ? 1 : 0, 0),
          "assembleJacobian");
  }
  void evalFunctions(int numFuncs, TACSFunction **funcs, double *fvals) {
    for (int i = 0; i < numFuncs; i++) {
      const int kind = funcs[i]->kind();
      check(tg_eval_functions(a_, vars_->getArray(), 1, &kind,
                              funcs[i]->ksWeight(), &fvals[i], 0),
            "evalFunctions");
    }
  }
  void addSVSens(double alpha, double beta, double gamma, int numFuncs,
                 TACSFunction **funcs, TACSBVec **dfdu) {
    (void)beta;
    (void)gamma;
    for (int i = 0; i < numFuncs; i++) {
      double f;
      const int kind = funcs[i]->kind();
      check(tg_eval_functions(a_, vars_->getArray(), 1, &kind,
                              funcs[i]->ksWeight(), &f, 0),
            "addSVSens");
      double *d = dfdu[i]->getArray();
      check(tg_add_sv_sens(a_, vars_->getArray(), 1, &kind, alpha, &d, 0),
            "addSVSens");
    }
  }
  void addDVSens(double coef, int numFuncs, TACSFunction **funcs,
                 TACSBVec **dfdx) {
    for (int i = 0; i < numFuncs; i++) {
      double f;
      const int kind = funcs[i]->kind();
      check(tg_eval_functions(a_, vars_->getArray(), 1, &kind,
                              funcs[i]->ksWeight(), &f, 0),
            "addDVSens");
      double *d = dfdx[i]->getArray();
      check(tg_add_dv_sens(a_, vars_->getArray(), 1, &kind, coef, &d, 0),
            "addDVSens");
    }
  }
  void addAdjointResProducts(double scale, int numAdjoints,
                             TACSBVec **adjoint, TACSBVec **dfdx,
                             double lambda = 1.0) {
    (void)lambda;
    std::vector<const double *> ps(numAdjoints);
    std::vector<double *> ds(numAdjoints);
    for (int i = 0; i < numAdjoints; i++) {
      ps[i] = adjoint[i]->getArray();
      ds[i] = dfdx[i]->getArray();
    }
    check(tg_add_adjoint_res_products(a_, vars_->getArray(), scale,
                                      numAdjoints, ps.data(), ds.data(), 0),
          "addAdjointResProducts");
  }
  // How the coordinate derivatives below are formed (no reference
  // counterpart): false dual numbers per coordinate, true the reverse sweep
  // per element; both exact.
  void setXptReverseMode(bool reverse) {
    check(tg_set_xpt_mode(a_, reverse ? TG_XPT_REVERSE : TG_XPT_FORWARD),
          "setXptReverseMode");
  }
  // TACSAssembler::addXptSens (src/TACSAssembler.cpp:4858): node vectors
  // from createNodeVec, 3 entries per node
  void addXptSens(double coef, int numFuncs, TACSFunction **funcs,
                  TACSBVec **dfdXpt) {
    for (int i = 0; i < numFuncs; i++) {
      double f;
      const int kind = funcs[i]->kind();
      check(tg_eval_functions(a_, vars_->getArray(), 1, &kind,
                              funcs[i]->ksWeight(), &f, 0),
            "addXptSens");
      double *d = dfdXpt[i]->getArray();
      check(tg_add_xpt_sens(a_, vars_->getArray(), 1, &kind, coef, &d, 0),
            "addXptSens");
    }
  }
  // TACSAssembler::addAdjointResXptSensProducts (src/TACSAssembler.cpp:5136)
  void addAdjointResXptSensProducts(double scale, int numAdjoints,
                                    TACSBVec **adjoint, TACSBVec **dfdXpt,
                                    double lambda = 1.0) {
    std::vector<const double *> ps(numAdjoints);
    std::vector<double *> ds(numAdjoints);
    for (int i = 0; i < numAdjoints; i++) {
      ps[i] = adjoint[i]->getArray();
      ds[i] = dfdXpt[i]->getArray();
    }
    check(tg_add_adjoint_res_xpt_products(a_, vars_->getArray(), scale,
                                          numAdjoints, ps.data(), ds.data(),
                                          lambda, 0),
          "addAdjointResXptSensProducts");
  }

 private:
  int vpn_, nnodes_, nelems_, ndv_ = 0;
  std::vector<int> conn_, bc_nodes_, bc_masks_;
  TACSElementSpec spec_;
  TACSAuxElements aux_;
  tg_assembler *a_ = nullptr;
  TACSBVec *vars_ = nullptr;
};

}  // namespace tacs_gb300

#endif /* TACS_GB300_HPP */
