/* C++ host interface of libtacs_gb300 with the reference's class names,
   constructors and method signatures for the hot path (src/TACSAssembler.h,
   src/TACSAuxElements.h, src/bpmat/TACSBVec.h, BCSRMat.h, TACSParallelMat.h,
   TACSSchurMat.h, KSM.h, src/constitutive/TACSMaterialProperties.h,
   TACSIsoShellConstitutive.h, TACSSolidConstitutive.h,
   src/elements/shell/TACSShellElementDefs.h, TACSShellElementTransform.h,
   TACSShellPressure.h, src/elements/TACSElement3D.h, TACSLinearElasticity.h,
   TACSTraction3D.h, basis/TACSHexaBasis.h, src/functions/TACSCompliance.h,
   TACSKSFailure.h): a C++ driver written against the reference compiles
   against this header with `using namespace tacs_gb300;` in place of the
   reference's includes.  Header-only; every numerical call goes through the
   C ABI in tacs_gb300.h and runs on the GPU.

   Differences a caller sees:
   - one process, one GPU.  MPI_Comm is a single-rank stand-in unless
     TACS_GB300_WITH_MPI is defined (then mpi.h's type is used and a
     communicator of more than one rank is rejected by initialize());
   - vector values live in device memory: TACSBVec::getArray returns the
     device pointer; copyFromHost / copyToHost move values from / to host
     memory;
   - element objects describe the element for the GPU kernels: every
     element of one assembler has the same type, material and (shells)
     transform; thickness and design-variable number are per element;
   - errors follow the reference's convention: a message on stderr and a
     non-zero int return (the C ABI's negative status code) where the
     reference returns int, a message only where it returns void.
   Reference counting is intrusive as in the reference (TACSObject::incref /
   decref; an object is deleted when its count returns to zero; objects
   passed to a constructor or setter are incref'd by the receiver). */
#ifndef TACS_GB300_HPP
#define TACS_GB300_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "tacs_gb300.h"

#ifdef TACS_GB300_WITH_MPI
#include <mpi.h>
#else
/* single-rank stand-in for the communicator argument */
typedef int MPI_Comm;
#ifndef MPI_COMM_WORLD
#define MPI_COMM_WORLD 0
#endif
#ifndef MPI_COMM_SELF
#define MPI_COMM_SELF 0
#endif
#endif

namespace tacs_gb300 {

typedef double TacsScalar;

/* Prints the failing call and the library's message (the reference prints
   to stderr and returns a code); returns rc. */
inline int tacs_report(int rc, const char *what) {
  if (rc < 0) std::fprintf(stderr, "[tacs_gb300] %s: %s\n", what,
                           tg_last_error());
  return rc;
}

enum MatrixOrientation { TACS_MAT_NORMAL = 0, TACS_MAT_TRANSPOSE = 1 };
enum ElementStrainType { TACS_LINEAR_STRAIN, TACS_NONLINEAR_STRAIN };

/* TACSObject (src/TACSObject.h:112-146): intrusive reference count. */
class TACSObject {
 public:
  TACSObject() {}
  virtual ~TACSObject() {}
  void incref() { ref_count_++; }
  void decref() {
    if (--ref_count_ <= 0) delete this;
  }
  int refcount() const { return ref_count_; }
  virtual const char *getObjectName() { return "TACSObject"; }

 private:
  TACSObject(const TACSObject &) = delete;
  TACSObject &operator=(const TACSObject &) = delete;
  int ref_count_ = 0;
};

template <class T>
inline void tacs_incref(T *p) {
  if (p) p->incref();
}
template <class T>
inline void tacs_decref(T *p) {
  if (p) p->decref();
}

/* ---- material, constitutive, transforms, bases, models --------------- */

/* TACSMaterialProperties(rho, specific_heat, E, nu, ys, alpha, kappa)
   (src/constitutive/TACSMaterialProperties.h:44): isotropic only. */
class TACSMaterialProperties : public TACSObject {
 public:
  TACSMaterialProperties(TacsScalar rho, TacsScalar specific_heat,
                         TacsScalar E, TacsScalar nu, TacsScalar ys,
                         TacsScalar alpha, TacsScalar kappa)
      : rho_(rho), E_(E), nu_(nu), ys_(ys) {
    (void)specific_heat;
    (void)alpha;
    (void)kappa;
  }
  TacsScalar getDensity() const { return rho_; }
  void getIsotropicProperties(TacsScalar *E, TacsScalar *nu) const {
    if (E) *E = E_;
    if (nu) *nu = nu_;
  }
  TacsScalar getYieldStress() const { return ys_; }
  const char *getObjectName() override { return "TACSMaterialProperties"; }

 private:
  TacsScalar rho_, E_, nu_, ys_;
};

class TACSConstitutive : public TACSObject {
 public:
  TACSConstitutive(TACSMaterialProperties *props, TacsScalar t, int tNum)
      : props_(props), t_(t), tNum_(tNum) {
    tacs_incref(props_);
  }
  ~TACSConstitutive() override { tacs_decref(props_); }
  TACSMaterialProperties *getMaterialProperties() { return props_; }
  TacsScalar thickness() const { return t_; }
  int designVarNum() const { return tNum_; }

 private:
  TACSMaterialProperties *props_;
  TacsScalar t_;
  int tNum_;
};

class TACSShellConstitutive : public TACSConstitutive {
 public:
  using TACSConstitutive::TACSConstitutive;
};

/* TACSIsoShellConstitutive(props, t, tNum, tlb, tub, tOffset, kcorr)
   (src/constitutive/TACSIsoShellConstitutive.h:33); the GPU kernels use
   tOffset = 0 and kcorr = 5/6, other values are rejected by initialize(). */
class TACSIsoShellConstitutive : public TACSShellConstitutive {
 public:
  TACSIsoShellConstitutive(TACSMaterialProperties *props, TacsScalar t = 1.0,
                           int tNum = -1, TacsScalar tlb = 0.0,
                           TacsScalar tub = 10.0, TacsScalar tOffset = 0.0,
                           TacsScalar kcorr = 5.0 / 6.0)
      : TACSShellConstitutive(props, t, tNum), tOffset_(tOffset),
        kcorr_(kcorr) {
    (void)tlb;
    (void)tub;
  }
  bool onGpuPath() const {
    return tOffset_ == 0.0 && std::fabs(kcorr_ - 5.0 / 6.0) < 1e-15;
  }
  const char *getObjectName() override { return "TACSIsoShellConstitutive"; }

 private:
  TacsScalar tOffset_, kcorr_;
};

/* TACSSolidConstitutive(props, t, tNum, tlb, tub)
   (src/constitutive/TACSSolidConstitutive.h:34): stress = t C e. */
class TACSSolidConstitutive : public TACSConstitutive {
 public:
  TACSSolidConstitutive(TACSMaterialProperties *props, TacsScalar t = 1.0,
                        int tNum = -1, TacsScalar tlb = 0.0,
                        TacsScalar tub = 1.0)
      : TACSConstitutive(props, t, tNum) {
    (void)tlb;
    (void)tub;
  }
  const char *getObjectName() override { return "TACSSolidConstitutive"; }
};

/* TACSShellTransform and its two forms
   (src/elements/shell/TACSShellElementTransform.h:21,95). */
class TACSShellTransform : public TACSObject {
 public:
  virtual int kind() const = 0;  // 0 natural, 1 reference axis
  virtual const TacsScalar *axis() const { return nullptr; }
};
class TACSShellNaturalTransform : public TACSShellTransform {
 public:
  TACSShellNaturalTransform() {}
  int kind() const override { return 0; }
};
class TACSShellRefAxisTransform : public TACSShellTransform {
 public:
  explicit TACSShellRefAxisTransform(const TacsScalar axis[]) {
    for (int k = 0; k < 3; k++) axis_[k] = axis[k];
  }
  int kind() const override { return 1; }
  const TacsScalar *axis() const override { return axis_; }

 private:
  TacsScalar axis_[3];
};

class TACSElementBasis : public TACSObject {
 public:
  virtual int numNodes() const = 0;
};
/* TACSLinearHexaBasis (src/elements/basis/TACSHexaBasis.h). */
class TACSLinearHexaBasis : public TACSElementBasis {
 public:
  int numNodes() const override { return 8; }
};

class TACSElementModel : public TACSObject {};
/* TACSLinearElasticity3D(con, strain_type)
   (src/elements/TACSLinearElasticity.h:178): linear strain only. */
class TACSLinearElasticity3D : public TACSElementModel {
 public:
  TACSLinearElasticity3D(TACSSolidConstitutive *con,
                         ElementStrainType strain_type)
      : con_(con), strain_(strain_type) {
    tacs_incref(con_);
  }
  ~TACSLinearElasticity3D() override { tacs_decref(con_); }
  TACSSolidConstitutive *getConstitutive() { return con_; }
  ElementStrainType strainType() const { return strain_; }

 private:
  TACSSolidConstitutive *con_;
  ElementStrainType strain_;
};

/* ---- elements --------------------------------------------------------- */

class TACSElement : public TACSObject {
 public:
  enum Kind { SHELL_QUAD4, SOLID_HEX8, SHELL_PRESSURE, TRACTION_3D, OTHER };
  virtual Kind kind() const { return OTHER; }
};

/* TACSQuad4Shell(transform, con) (src/elements/shell/TACSShellElementDefs.h:
   18-20; the TACSShellElement constructor TACSShellElement.h:39). */
class TACSQuad4Shell : public TACSElement {
 public:
  TACSQuad4Shell(TACSShellTransform *transform, TACSShellConstitutive *con)
      : transform_(transform), con_(con) {
    tacs_incref(transform_);
    tacs_incref(con_);
  }
  ~TACSQuad4Shell() override {
    tacs_decref(transform_);
    tacs_decref(con_);
  }
  Kind kind() const override { return SHELL_QUAD4; }
  TACSShellTransform *getTransform() { return transform_; }
  TACSShellConstitutive *getConstitutive() { return con_; }
  const char *getObjectName() override { return "TACSQuad4Shell"; }

 private:
  TACSShellTransform *transform_;
  TACSShellConstitutive *con_;
};

/* TACSElement3D(model, basis) (src/elements/TACSElement3D.h:26) with a
   TACSLinearElasticity3D model and the TACSLinearHexaBasis. */
class TACSElement3D : public TACSElement {
 public:
  TACSElement3D(TACSElementModel *model, TACSElementBasis *basis)
      : model_(model), basis_(basis) {
    tacs_incref(model_);
    tacs_incref(basis_);
  }
  ~TACSElement3D() override {
    tacs_decref(model_);
    tacs_decref(basis_);
  }
  Kind kind() const override { return SOLID_HEX8; }
  TACSElementModel *getModel() { return model_; }
  TACSElementBasis *getBasis() { return basis_; }
  const char *getObjectName() override { return "TACSElement3D"; }

 private:
  TACSElementModel *model_;
  TACSElementBasis *basis_;
};

/* TACSShellPressure(p[4]) / TACSShellPressure(p)
   (src/elements/shell/TACSShellPressure.h:11,18): nodal pressures. */
class TACSShellPressure : public TACSElement {
 public:
  explicit TACSShellPressure(const TacsScalar p[]) {
    for (int k = 0; k < 4; k++) p_[k] = p[k];
  }
  explicit TACSShellPressure(TacsScalar p) {
    for (int k = 0; k < 4; k++) p_[k] = p;
  }
  Kind kind() const override { return SHELL_PRESSURE; }
  const TacsScalar *values() const { return p_; }

 private:
  TacsScalar p_[4];
};

/* TACSTraction3D(varsPerNode, faceIndex, basis, trac[],
   tractionCoordinateComponent) (src/elements/TACSTraction3D.h:22): a
   constant traction on one face; the coordinate-component form only. */
class TACSTraction3D : public TACSElement {
 public:
  TACSTraction3D(int varsPerNode, int faceIndex, TACSElementBasis *basis,
                 const TacsScalar trac[], int tractionCoordinateComponent = 1)
      : face_(faceIndex), coord_(tractionCoordinateComponent) {
    (void)varsPerNode;
    (void)basis;
    for (int k = 0; k < 3; k++) t_[k] = trac[k];
  }
  Kind kind() const override { return TRACTION_3D; }
  int face() const { return face_; }
  int coordinateComponent() const { return coord_; }
  const TacsScalar *values() const { return t_; }

 private:
  int face_, coord_;
  TacsScalar t_[3];
};

/* TACSAuxElements(num) / addElement(num, elem) (src/TACSAuxElements.h:54,
   63). */
class TACSAuxElements : public TACSObject {
 public:
  explicit TACSAuxElements(int num_elems = 100) { items_.reserve(num_elems); }
  ~TACSAuxElements() override {
    for (auto &it : items_) tacs_decref(it.second);
  }
  void addElement(int num, TACSElement *elem) {
    tacs_incref(elem);
    items_.push_back({num, elem});
  }
  void addElements(int nums[], TACSElement **elem, int num_elems) {
    for (int i = 0; i < num_elems; i++) addElement(nums[i], elem[i]);
  }
  int getNumElements() const { return (int)items_.size(); }
  const std::vector<std::pair<int, TACSElement *>> &items() const {
    return items_;
  }

 private:
  std::vector<std::pair<int, TACSElement *>> items_;
};

/* ---- vectors, matrices, preconditioners, GMRES ------------------------ */

class TACSVec : public TACSObject {};

/* TACSBVec (src/bpmat/TACSBVec.h:67-99): size doubles of device memory
   with block size bsize. */
class TACSBVec : public TACSVec {
 public:
  TACSBVec(int size, int bsize) : n_(size), bsize_(bsize) {
    if (cudaMalloc((void **)&d_, sizeof(double) * (size > 0 ? size : 1)) !=
        cudaSuccess) {
      std::fprintf(stderr, "[tacs_gb300] TACSBVec: cudaMalloc failed\n");
      d_ = nullptr;
      n_ = 0;
    }
    zeroEntries();
  }
  ~TACSBVec() override {
    if (d_) cudaFree(d_);
  }
  /* device pointer; returns the number of entries */
  int getArray(TacsScalar **array) {
    *array = d_;
    return n_;
  }
  void getSize(int *size) const { *size = n_; }
  int getBlockSize() const { return bsize_; }
  void zeroEntries() {
    if (d_) cudaMemset(d_, 0, sizeof(double) * n_);
  }
  void set(TacsScalar val) {
    zeroEntries();
    if (val != 0.0) {
      std::vector<double> h(n_, val);
      copyFromHost(h.data());
    }
  }
  void copyFromHost(const TacsScalar *host) {
    cudaMemcpy(d_, host, sizeof(double) * n_, cudaMemcpyHostToDevice);
  }
  void copyToHost(TacsScalar *host) const {
    cudaMemcpy(host, d_, sizeof(double) * n_, cudaMemcpyDeviceToHost);
  }
  void copyValues(TACSVec *x) {
    TACSBVec *v = dynamic_cast<TACSBVec *>(x);
    if (v) cudaMemcpy(d_, v->d_, sizeof(double) * n_, cudaMemcpyDeviceToDevice);
  }
  void scale(TacsScalar a) { tacs_report(tg_vec_scale(a, d_, n_, 0), "scale"); }
  void axpy(TacsScalar a, TACSVec *x) {
    TACSBVec *v = dynamic_cast<TACSBVec *>(x);
    if (v) tacs_report(tg_vec_axpy(a, v->d_, d_, n_, 0), "axpy");
  }
  TacsScalar dot(TACSVec *x) {
    TACSBVec *v = dynamic_cast<TACSBVec *>(x);
    double r = 0.0;
    if (v) tacs_report(tg_vec_dot(d_, v->d_, n_, &r, 0), "dot");
    return r;
  }
  TacsScalar norm() {
    const double v = dot(this);
    return v > 0.0 ? std::sqrt(v) : 0.0;
  }
  double *device() const { return d_; }

 private:
  int n_, bsize_;
  double *d_ = nullptr;
};

class TACSMat : public TACSObject {
 public:
  virtual void mult(TACSVec *x, TACSVec *y) = 0;
  virtual tg_mat *handle() = 0;
};

/* BCSRMat (src/bpmat/BCSRMat.h): the local block matrix of a
   TACSParallelMat (owned by it).  getArrays returns device arrays of the
   row-major b x b blocks. */
class BCSRMat : public TACSObject {
 public:
  explicit BCSRMat(tg_mat *m) : m_(m) {}
  void getArrays(int *bsize, int *nrows, int *ncols, const int **rowp,
                 const int **cols, TacsScalar **Avals) {
    int nr = 0;
    tacs_report(tg_mat_get_arrays(m_, bsize, &nr, rowp, cols, Avals),
                "BCSRMat::getArrays");
    if (nrows) *nrows = nr;
    if (ncols) *ncols = nr;
  }
  void mult(TacsScalar *x, TacsScalar *y) {
    tacs_report(tg_mat_mult(m_, x, y, 0), "BCSRMat::mult");
  }

 private:
  tg_mat *m_;
};

/* TACSParallelMat (src/bpmat/TACSParallelMat.h:52): the assembler's
   matrix; one rank, so the off-process block B is empty (NULL). */
class TACSParallelMat : public TACSMat {
 public:
  explicit TACSParallelMat(tg_assembler *a) {
    if (tacs_report(tg_mat_create(a, &m_), "createMat") < 0) m_ = nullptr;
    local_ = new BCSRMat(m_);
    local_->incref();
  }
  ~TACSParallelMat() override {
    local_->decref();
    if (m_) tg_mat_decref(m_);
  }
  void mult(TACSVec *x, TACSVec *y) override {
    TACSBVec *xv = dynamic_cast<TACSBVec *>(x);
    TACSBVec *yv = dynamic_cast<TACSBVec *>(y);
    if (xv && yv)
      tacs_report(tg_mat_mult(m_, xv->device(), yv->device(), 0),
                  "TACSParallelMat::mult");
  }
  void getSize(int *nr, int *nc) {
    int b = 0, n = 0;
    const int *rp, *c;
    double *A;
    tacs_report(tg_mat_get_arrays(m_, &b, &n, &rp, &c, &A), "getSize");
    if (nr) *nr = b * n;
    if (nc) *nc = b * n;
  }
  void getBCSRMat(BCSRMat **A, BCSRMat **B) {
    if (A) *A = local_;
    if (B) *B = nullptr;
  }
  tg_mat *handle() override { return m_; }

 private:
  tg_mat *m_ = nullptr;
  BCSRMat *local_ = nullptr;
};

/* TACSSchurMat (src/bpmat/TACSSchurMat.h:59): on one GPU the same storage
   as TACSParallelMat; TACSSchurPc on it factors completely. */
class TACSSchurMat : public TACSParallelMat {
 public:
  using TACSParallelMat::TACSParallelMat;
};

/* TACSPc (src/bpmat/KSM.h:200). */
class TACSPc : public TACSObject {
 public:
  virtual void applyFactor(TACSVec *x, TACSVec *y) = 0;
  virtual void factor() = 0;
  virtual tg_pc *handle() = 0;
};

/* TACSAdditiveSchwarz(mat, levFill, fill)
   (src/bpmat/TACSParallelMat.cpp:1190): block ILU(levFill) on the
   computeILUk pattern.  precision TG_PREC_FP32 (no reference counterpart)
   factors and applies in FP32 for the mixed-precision GMRES. */
class TACSAdditiveSchwarz : public TACSPc {
 public:
  TACSAdditiveSchwarz(TACSParallelMat *mat, int levFill, double fill,
                      int precision = TG_PREC_FP64) {
    (void)fill;  // the pattern is sized exactly, no fill estimate needed
    if (tacs_report(tg_pc_create_iluk(mat->handle(), levFill, precision, &pc_),
                    "TACSAdditiveSchwarz") < 0)
      pc_ = nullptr;
  }
  ~TACSAdditiveSchwarz() override {
    if (pc_) tg_pc_decref(pc_);
  }
  void factor() override { tacs_report(tg_pc_factor(pc_, 0), "factor"); }
  void applyFactor(TACSVec *x, TACSVec *y) override {
    TACSBVec *xv = dynamic_cast<TACSBVec *>(x);
    TACSBVec *yv = dynamic_cast<TACSBVec *>(y);
    if (xv && yv)
      tacs_report(tg_pc_apply(pc_, xv->device(), yv->device(), 0),
                  "applyFactor");
  }
  tg_pc *handle() override { return pc_; }

 private:
  tg_pc *pc_ = nullptr;
};

/* TACSSchurPc(mat, levFill, fill, reorder_schur_complement)
   (src/bpmat/TACSSchurMat.h:149): the complete factorisation (the
   multifrontal tg_direct through a TG_PC_DIRECT preconditioner);
   levFill below 1000 (an incomplete Schur factor) is not on the GPU path.
   applyFactor(x, y) is y = A^-1 x. */
class TACSSchurPc : public TACSPc {
 public:
  TACSSchurPc(TACSSchurMat *mat, int levFill, double fill,
              int reorder_schur_complement) {
    (void)fill;
    (void)reorder_schur_complement;
    if (levFill < 1000) {
      std::fprintf(stderr, "[tacs_gb300] TACSSchurPc: only the complete "
                           "factorisation (levFill >= 1000) is on the GPU\n");
      return;
    }
    if (tacs_report(tg_pc_create(mat->handle(), TG_PC_DIRECT, TG_PREC_FP64,
                                 &pc_),
                    "TACSSchurPc") < 0)
      pc_ = nullptr;
  }
  ~TACSSchurPc() override {
    if (pc_) tg_pc_decref(pc_);
  }
  void factor() override {
    if (pc_) tacs_report(tg_pc_factor(pc_, 0), "factor");
  }
  void applyFactor(TACSVec *x, TACSVec *y) override {
    TACSBVec *xv = dynamic_cast<TACSBVec *>(x);
    TACSBVec *yv = dynamic_cast<TACSBVec *>(y);
    if (pc_ && xv && yv)
      tacs_report(tg_pc_apply(pc_, xv->device(), yv->device(), 0),
                  "applyFactor");
  }
  tg_pc *handle() override { return pc_; }

 private:
  tg_pc *pc_ = nullptr;
};

/* GMRES(mat, pc, m, nrestart, isFlexible) (src/bpmat/KSM.h:395).
   setMixedPrecision(1) (no reference counterpart) runs the FP32
   preconditioner and mat-vec inside FP64 GMRES with true-residual
   refinement; it needs a preconditioner made with TG_PREC_FP32. */
class GMRES : public TACSObject {
 public:
  GMRES(TACSMat *mat, TACSPc *pc, int m, int nrestart, int isFlexible)
      : mat_(mat), pc_(pc), m_(m), nrestart_(nrestart) {
    (void)isFlexible;
    tacs_incref(mat_);
    tacs_incref(pc_);
  }
  ~GMRES() override {
    if (k_) tg_ksm_decref(k_);
    tacs_decref(pc_);
    tacs_decref(mat_);
  }
  void setTolerances(double rtol, double atol) {
    rtol_ = rtol;
    atol_ = atol;
    if (k_) tacs_report(tg_ksm_set_tolerances(k_, rtol, atol), "setTolerances");
  }
  void setMixedPrecision(int mixed) { mixed_ = mixed; }
  /* 1 when converged, 0 when not (or on an error, which is printed) */
  int solve(TACSVec *b, TACSVec *x, int zero_guess = 1) {
    TACSBVec *bv = dynamic_cast<TACSBVec *>(b);
    TACSBVec *xv = dynamic_cast<TACSBVec *>(x);
    if (!bv || !xv) return 0;
    if (!k_) {
      if (tacs_report(tg_ksm_create(mat_->handle(), pc_ ? pc_->handle()
                                                        : nullptr,
                                    m_, nrestart_, mixed_, &k_),
                      "GMRES") < 0) {
        k_ = nullptr;
        return 0;
      }
      tacs_report(tg_ksm_set_tolerances(k_, rtol_, atol_), "setTolerances");
    }
    const int rc = tg_ksm_solve(k_, bv->device(), xv->device(), zero_guess,
                                &iters_, &resnorm_, 0);
    if (rc < 0) {
      tacs_report(rc, "GMRES::solve");
      return 0;
    }
    return rc;
  }
  int getIterCount() const { return iters_; }
  double getResidualNorm() const { return resnorm_; }

 private:
  TACSMat *mat_;
  TACSPc *pc_;
  int m_, nrestart_, mixed_ = 0;
  double rtol_ = 1e-8, atol_ = 1e-30;  // the reference's defaults
  tg_ksm *k_ = nullptr;
  int iters_ = 0;
  double resnorm_ = 0.0;
};

class TACSAssembler;

/* TACSFunction: TACSCompliance (src/functions/TACSCompliance.h) and
   TACSKSFailure with KS_CONTINUOUS (src/functions/TACSKSFailure.h). */
class TACSFunction : public TACSObject {
 public:
  TACSFunction(int kind, double ks_weight) : kind_(kind), ksw_(ks_weight) {}
  int kind() const { return kind_; }
  double ksWeight() const { return ksw_; }

 private:
  int kind_;
  double ksw_;
};
class TACSCompliance : public TACSFunction {
 public:
  explicit TACSCompliance(TACSAssembler *)
      : TACSFunction(TG_FUNC_COMPLIANCE, 0.0) {}
  const char *getObjectName() override { return "TACSCompliance"; }
};
class TACSKSFailure : public TACSFunction {
 public:
  TACSKSFailure(TACSAssembler *, double ksWeight = 80.0, double alpha = 1.0,
                double safetyFactor = 1.0)
      : TACSFunction(TG_FUNC_KS_FAILURE, ksWeight) {
    (void)alpha;
    (void)safetyFactor;
  }
  const char *getObjectName() override { return "TACSKSFailure"; }
};

/* ---- the assembler ---------------------------------------------------- */

/* TACSAssembler (src/TACSAssembler.h:83-299) for one process and one
   GPU. */
class TACSAssembler : public TACSObject {
 public:
  enum OrderingType {
    NATURAL_ORDER,
    RCM_ORDER,
    AMD_ORDER,
    ND_ORDER,
    TACS_AMD_ORDER,
    MULTICOLOR_ORDER
  };

  TACSAssembler(MPI_Comm comm, int varsPerNode, int numOwnedNodes,
                int numElements, int numDependentNodes = 0)
      : comm_(comm), vpn_(varsPerNode), nnodes_(numOwnedNodes),
        nelems_(numElements), ndep_(numDependentNodes) {}
  ~TACSAssembler() override {
    tacs_decref(vars_);
    for (TACSElement *e : elements_) tacs_decref(e);
    tacs_decref(aux_);
    if (a_) tg_assembler_decref(a_);
  }

  int setElementConnectivity(const int *ptr, const int *conn) {
    ptr_.assign(ptr, ptr + nelems_ + 1);
    conn_.assign(conn + ptr[0], conn + ptr[nelems_]);
    return 0;
  }
  int setElements(TACSElement **elements) {
    for (TACSElement *e : elements_) tacs_decref(e);
    elements_.assign(elements, elements + nelems_);
    for (TACSElement *e : elements_) tacs_incref(e);
    return 0;
  }
  void addBCs(int nnodes, const int *nodes, int nbcs = -1,
              const int *vars = nullptr, const TacsScalar *vals = nullptr) {
    int mask = 0;
    if (nbcs < 0) mask = (1 << vpn_) - 1;
    else
      for (int k = 0; k < nbcs; k++) mask |= 1 << vars[k];
    bool nonzero = false;
    if (vals)
      for (int k = 0; k < (nbcs < 0 ? vpn_ : nbcs); k++)
        nonzero |= vals[k] != 0.0;
    if (nonzero)
      std::fprintf(stderr, "[tacs_gb300] addBCs: non-zero prescribed values "
                           "are not on the GPU path (zero used)\n");
    for (int i = 0; i < nnodes; i++) {
      bc_nodes_.push_back(nodes[i]);
      bc_masks_.push_back(mask);
    }
  }
  void setAuxElements(TACSAuxElements *aux) {
    tacs_incref(aux);
    tacs_decref(aux_);
    aux_ = aux;
  }
  void setNumThreads(int) {}  // the GPU replaces the pthreads

  int initialize();

  TACSBVec *createVec() { return new TACSBVec(vpn_ * nnodes_, vpn_); }
  TACSBVec *createNodeVec() { return new TACSBVec(3 * nnodes_, 3); }
  TACSBVec *createDesignVec() { return new TACSBVec(ndv_, 1); }
  TACSParallelMat *createMat() { return new TACSParallelMat(a_); }
  TACSSchurMat *createSchurMat(OrderingType = TACS_AMD_ORDER) {
    return new TACSSchurMat(a_);
  }
  int getVarsPerNode() const { return vpn_; }
  int getNumOwnedNodes() const { return nnodes_; }
  int getNumElements() const { return nelems_; }
  MPI_Comm getMPIComm() const { return comm_; }

  void setNodes(TACSBVec *X) {
    tacs_report(tg_assembler_set_nodes(a_, X->device(), 0), "setNodes");
  }
  void setDesignVars(TACSBVec *x) {
    tacs_report(tg_assembler_set_design_vars(a_, x->device(), 0),
                "setDesignVars");
  }
  void setVariables(TACSBVec *q, TACSBVec *qdot = nullptr,
                    TACSBVec *qddot = nullptr) {
    (void)qdot;
    (void)qddot;
    vars_->copyValues(q);
  }
  void getVariables(TACSBVec *q) { q->copyValues(vars_); }
  void zeroVariables() { vars_->zeroEntries(); }
  void applyBCs(TACSVec *v) {
    TACSBVec *bv = dynamic_cast<TACSBVec *>(v);
    if (bv) tacs_report(tg_apply_bcs(a_, bv->device(), 0), "applyBCs");
  }

  void assembleRes(TACSBVec *res, TacsScalar lambda = 1.0,
                   bool applyBCs = true) {
    tacs_report(tg_assemble_res(a_, vars_->device(), lambda, applyBCs ? 1 : 0,
                                res->device(), 0),
                "assembleRes");
  }
  void assembleJacobian(TacsScalar alpha, TacsScalar beta, TacsScalar gamma,
                        TACSBVec *res, TACSMat *A,
                        MatrixOrientation matOr = TACS_MAT_NORMAL,
                        TacsScalar lambda = 1.0, bool applyBCs = true) {
    tacs_report(tg_assemble_jacobian(a_, alpha, beta, gamma, vars_->device(),
                                     res ? res->device() : nullptr,
                                     A->handle(), (int)matOr, lambda,
                                     applyBCs ? 1 : 0, 0),
                "assembleJacobian");
  }
  void evalFunctions(int numFuncs, TACSFunction **funcs, TacsScalar *fvals) {
    for (int i = 0; i < numFuncs; i++) {
      const int kind = funcs[i]->kind();
      tacs_report(tg_eval_functions(a_, vars_->device(), 1, &kind,
                                    funcs[i]->ksWeight(), &fvals[i], 0),
                  "evalFunctions");
    }
  }
  void addSVSens(TacsScalar alpha, TacsScalar beta, TacsScalar gamma,
                 int numFuncs, TACSFunction **funcs, TACSBVec **dfdu) {
    (void)beta;
    (void)gamma;
    for (int i = 0; i < numFuncs; i++) {
      if (!prime(funcs[i], "addSVSens")) continue;
      const int kind = funcs[i]->kind();
      double *d = dfdu[i]->device();
      tacs_report(tg_add_sv_sens(a_, vars_->device(), 1, &kind, alpha, &d, 0),
                  "addSVSens");
    }
  }
  void addDVSens(TacsScalar coef, int numFuncs, TACSFunction **funcs,
                 TACSBVec **dfdx) {
    for (int i = 0; i < numFuncs; i++) {
      if (!prime(funcs[i], "addDVSens")) continue;
      const int kind = funcs[i]->kind();
      double *d = dfdx[i]->device();
      tacs_report(tg_add_dv_sens(a_, vars_->device(), 1, &kind, coef, &d, 0),
                  "addDVSens");
    }
  }
  void addAdjointResProducts(TacsScalar scale, int numAdjoints,
                             TACSBVec **adjoint, TACSBVec **dfdx,
                             TacsScalar lambda = 1.0) {
    (void)lambda;
    std::vector<const double *> ps(numAdjoints);
    std::vector<double *> ds(numAdjoints);
    for (int i = 0; i < numAdjoints; i++) {
      ps[i] = adjoint[i]->device();
      ds[i] = dfdx[i]->device();
    }
    tacs_report(tg_add_adjoint_res_products(a_, vars_->device(), scale,
                                            numAdjoints, ps.data(), ds.data(),
                                            0),
                "addAdjointResProducts");
  }
  /* How the coordinate derivatives below are formed (no reference
     counterpart): false dual numbers per coordinate, true the reverse sweep
     per element; both exact. */
  void setXptReverseMode(bool reverse) {
    tacs_report(tg_set_xpt_mode(a_, reverse ? TG_XPT_REVERSE : TG_XPT_FORWARD),
                "setXptReverseMode");
  }
  /* TACSAssembler::addXptSens (src/TACSAssembler.cpp:4858): node vectors
     from createNodeVec, 3 entries per node */
  void addXptSens(TacsScalar coef, int numFuncs, TACSFunction **funcs,
                  TACSBVec **dfdXpt) {
    for (int i = 0; i < numFuncs; i++) {
      if (!prime(funcs[i], "addXptSens")) continue;
      const int kind = funcs[i]->kind();
      double *d = dfdXpt[i]->device();
      tacs_report(tg_add_xpt_sens(a_, vars_->device(), 1, &kind, coef, &d, 0),
                  "addXptSens");
    }
  }
  /* TACSAssembler::addAdjointResXptSensProducts
     (src/TACSAssembler.cpp:5136) */
  void addAdjointResXptSensProducts(TacsScalar scale, int numAdjoints,
                                    TACSBVec **adjoint, TACSBVec **dfdXpt,
                                    TacsScalar lambda = 1.0) {
    std::vector<const double *> ps(numAdjoints);
    std::vector<double *> ds(numAdjoints);
    for (int i = 0; i < numAdjoints; i++) {
      ps[i] = adjoint[i]->device();
      ds[i] = dfdXpt[i]->device();
    }
    tacs_report(tg_add_adjoint_res_xpt_products(a_, vars_->device(), scale,
                                                numAdjoints, ps.data(),
                                                ds.data(), lambda, 0),
                "addAdjointResXptSensProducts");
  }

 private:
  /* the KS sensitivities use the statistics of the function's last
     evaluation (the reference's two-stage KSFailure): evaluate first */
  bool prime(TACSFunction *f, const char *what) {
    double v;
    const int kind = f->kind();
    return tacs_report(tg_eval_functions(a_, vars_->device(), 1, &kind,
                                         f->ksWeight(), &v, 0),
                       what) >= 0;
  }
  int fail(const char *msg) {
    std::fprintf(stderr, "[tacs_gb300] TACSAssembler::initialize: %s\n", msg);
    return TG_ERR_ARG;
  }

  MPI_Comm comm_;
  int vpn_, nnodes_, nelems_, ndep_, ndv_ = 0;
  std::vector<int> ptr_, conn_, bc_nodes_, bc_masks_;
  std::vector<TACSElement *> elements_;
  TACSAuxElements *aux_ = nullptr;
  tg_assembler *a_ = nullptr;
  TACSBVec *vars_ = nullptr;
};

/* Reads the element objects into the GPU description (one element type,
   material and transform per assembler; t and tNum per element) and the
   auxiliary loads, then creates the device-side assembler. */
inline int TACSAssembler::initialize() {
#ifdef TACS_GB300_WITH_MPI
  int size = 1;
  MPI_Comm_size(comm_, &size);
  if (size != 1) return fail("one rank per assembler (one GPU)");
#endif
  if (a_) return fail("already initialized");
  if (ndep_ != 0) return fail("dependent nodes are not on the GPU path");
  if ((int)ptr_.size() != nelems_ + 1) return fail("no connectivity");
  if ((int)elements_.size() != nelems_) return fail("no elements");
  int type = -1, transform = 0;
  double axis[3] = {1.0, 0.0, 0.0};
  TACSMaterialProperties *props = nullptr;
  std::vector<double> t(nelems_);
  std::vector<int> tnum(nelems_);
  for (int e = 0; e < nelems_; e++) {
    TACSElement *el = elements_[e];
    if (!el) return fail("null element");
    TACSConstitutive *con = nullptr;
    int et = -1;
    if (el->kind() == TACSElement::SHELL_QUAD4) {
      TACSQuad4Shell *s = static_cast<TACSQuad4Shell *>(el);
      TACSIsoShellConstitutive *iso =
          dynamic_cast<TACSIsoShellConstitutive *>(s->getConstitutive());
      if (!iso || !iso->onGpuPath())
        return fail("shells need TACSIsoShellConstitutive with tOffset = 0 "
                    "and kcorr = 5/6");
      if (!s->getTransform()) return fail("shell without a transform");
      con = iso;
      et = TG_ELEM_MITC4;
      const int tk = s->getTransform()->kind();
      if (e == 0) {
        transform = tk;
        if (tk == 1)
          for (int k = 0; k < 3; k++) axis[k] = s->getTransform()->axis()[k];
      } else if (tk != transform ||
                 (tk == 1 && (axis[0] != s->getTransform()->axis()[0] ||
                              axis[1] != s->getTransform()->axis()[1] ||
                              axis[2] != s->getTransform()->axis()[2]))) {
        return fail("one shell transform per assembler");
      }
    } else if (el->kind() == TACSElement::SOLID_HEX8) {
      TACSElement3D *h = static_cast<TACSElement3D *>(el);
      TACSLinearElasticity3D *m =
          dynamic_cast<TACSLinearElasticity3D *>(h->getModel());
      if (!m || m->strainType() != TACS_LINEAR_STRAIN ||
          !dynamic_cast<TACSLinearHexaBasis *>(h->getBasis()))
        return fail("solids need TACSLinearElasticity3D (linear strain) on "
                    "TACSLinearHexaBasis");
      con = m->getConstitutive();
      et = TG_ELEM_HEX8;
    } else {
      return fail("element type is not on the GPU path");
    }
    if (!con || !con->getMaterialProperties())
      return fail("element without material properties");
    if (e == 0) {
      type = et;
      props = con->getMaterialProperties();
    } else if (et != type) {
      return fail("one element type per assembler");
    } else if (con->getMaterialProperties() != props) {
      TACSMaterialProperties *q = con->getMaterialProperties();
      double E0, nu0, E1, nu1;
      props->getIsotropicProperties(&E0, &nu0);
      q->getIsotropicProperties(&E1, &nu1);
      if (E0 != E1 || nu0 != nu1 ||
          props->getDensity() != q->getDensity() ||
          props->getYieldStress() != q->getYieldStress())
        return fail("one material per assembler");
    }
    t[e] = con->thickness();
    tnum[e] = con->designVarNum();
  }
  if ((type == TG_ELEM_MITC4 && vpn_ != 6) ||
      (type == TG_ELEM_HEX8 && vpn_ != 3))
    return fail("varsPerNode does not match the element type");
  for (int e = 0; e < nelems_; e++)
    if (ptr_[e + 1] - ptr_[e] != (type == TG_ELEM_MITC4 ? 4 : 8))
      return fail("connectivity does not match the element type");
  double E, nu;
  props->getIsotropicProperties(&E, &nu);
  int rc = tg_assembler_create(type, nnodes_, nelems_, conn_.data(),
                               props->getDensity(), E, nu,
                               props->getYieldStress(), transform, axis, &a_);
  if (rc < 0) {
    a_ = nullptr;
    return tacs_report(rc, "TACSAssembler");
  }
  if ((rc = tacs_report(tg_assembler_add_bcs(a_, (int)bc_nodes_.size(),
                                             bc_nodes_.data(),
                                             bc_masks_.data()),
                        "addBCs")) < 0)
    return rc;
  if ((rc = tacs_report(tg_assembler_set_element_dvs(a_, t.data(),
                                                     tnum.data()),
                        "setElements")) < 0)
    return rc;
  if (aux_) {
    std::vector<int> pe, te, tf;
    std::vector<double> pv, tv;
    for (const auto &it : aux_->items()) {
      if (it.first < 0 || it.first >= nelems_)
        return fail("auxiliary element number out of range");
      if (it.second->kind() == TACSElement::SHELL_PRESSURE &&
          type == TG_ELEM_MITC4) {
        pe.push_back(it.first);
        const double *p =
            static_cast<TACSShellPressure *>(it.second)->values();
        pv.insert(pv.end(), p, p + 4);
      } else if (it.second->kind() == TACSElement::TRACTION_3D &&
                 type == TG_ELEM_HEX8) {
        TACSTraction3D *tr = static_cast<TACSTraction3D *>(it.second);
        if (tr->coordinateComponent() != 1)
          return fail("TACSTraction3D: coordinate-component tractions only");
        te.push_back(it.first);
        tf.push_back(tr->face());
        tv.insert(tv.end(), tr->values(), tr->values() + 3);
      } else {
        return fail("auxiliary element is not on the GPU path");
      }
    }
    if (!pe.empty() &&
        (rc = tacs_report(tg_assembler_set_pressure(a_, (int)pe.size(),
                                                    pe.data(), pv.data()),
                          "TACSShellPressure")) < 0)
      return rc;
    if (!te.empty() &&
        (rc = tacs_report(tg_assembler_set_traction(a_, (int)te.size(),
                                                    te.data(), tf.data(),
                                                    tv.data()),
                          "TACSTraction3D")) < 0)
      return rc;
  }
  if ((rc = tacs_report(tg_assembler_initialize(a_), "initialize")) < 0)
    return rc;
  int vpn, nn, ne, ndv, nc;
  if ((rc = tacs_report(tg_assembler_get_sizes(a_, &vpn, &nn, &ne, &ndv, &nc),
                        "initialize")) < 0)
    return rc;
  ndv_ = ndv;
  vars_ = createVec();
  vars_->incref();
  return 0;
}

}  // namespace tacs_gb300

#endif /* TACS_GB300_HPP */
