/*
  Forced-include header (g++ -include) for the operation-counting flavour of
  the reference build (make -C oracle/ref opc).  Test infrastructure only.

  The reference's complex build takes TacsScalar = std::complex<double>
  (TACSObject.h:47-56) and needs from it only arithmetic, comparison with
  doubles, real()/imag() and the usual math functions (TacsComplexStep.h
  adds RealPart, ImagPart, fabs and atan on top).  This header includes the
  real <complex> first and then maps the token `complex` to a scalar that
  does the same real arithmetic and counts every operation, so the unchanged
  reference sources, compiled with -DTACS_USE_COMPLEX, count the FP64
  operations their real build executes on TacsScalar values.

  Counted: add/sub, mul, div, sqrt, transcendental calls; a fused
  multiply-add counts as one mul and one add.  Not counted: sign changes,
  comparisons, and arithmetic the reference does in plain double (quadrature
  weights and basis functions), so the counts are a lower bound on the real
  build's FP64 work.  The complex-step branches (verification helpers and
  node-coordinate derivatives) would not compute derivatives here; the
  counting driver calls only residual, Jacobian and adjoint-product paths,
  which take no such branch.
*/
#ifndef TG_OPCOUNT_H
#define TG_OPCOUNT_H

#include <cmath>
#include <complex>

struct TgOpCounts {
  unsigned long long add, mul, div, sqrt, transc;
};
// defined once, in the counting driver (oracle/ref/op_count.cpp)
extern TgOpCounts tg_opcounts;

namespace std {

template <class T>
class tg_counted;

template <>
class tg_counted<double> {
 public:
  typedef double value_type;
  tg_counted(double r = 0.0, double i = 0.0) : re_(r), im_(i) {}
  double real() const { return re_; }
  double imag() const { return im_; }
  void real(double v) { re_ = v; }
  void imag(double v) { im_ = v; }

  tg_counted &operator+=(const tg_counted &b) {
    tg_opcounts.add++;
    re_ += b.re_;
    return *this;
  }
  tg_counted &operator-=(const tg_counted &b) {
    tg_opcounts.add++;
    re_ -= b.re_;
    return *this;
  }
  tg_counted &operator*=(const tg_counted &b) {
    tg_opcounts.mul++;
    re_ *= b.re_;
    return *this;
  }
  tg_counted &operator/=(const tg_counted &b) {
    tg_opcounts.div++;
    re_ /= b.re_;
    return *this;
  }
  tg_counted &operator+=(double b) { return *this += tg_counted(b); }
  tg_counted &operator-=(double b) { return *this -= tg_counted(b); }
  tg_counted &operator*=(double b) { return *this *= tg_counted(b); }
  tg_counted &operator/=(double b) { return *this /= tg_counted(b); }

 private:
  double re_, im_;  // im_ is carried, never computed with
};

typedef tg_counted<double> tg_cd;

#define TG_OPC_BINARY(op)                                                 \
  inline tg_cd operator op(const tg_cd &a, const tg_cd &b) {             \
    tg_cd r(a);                                                           \
    r op## = b;                                                           \
    return r;                                                             \
  }                                                                       \
  inline tg_cd operator op(const tg_cd &a, double b) {                   \
    tg_cd r(a);                                                           \
    r op## = b;                                                           \
    return r;                                                             \
  }                                                                       \
  inline tg_cd operator op(double a, const tg_cd &b) {                   \
    tg_cd r(a);                                                           \
    r op## = b;                                                           \
    return r;                                                             \
  }
TG_OPC_BINARY(+)
TG_OPC_BINARY(-)
TG_OPC_BINARY(*)
TG_OPC_BINARY(/)
#undef TG_OPC_BINARY

inline tg_cd operator+(const tg_cd &a) { return a; }
inline tg_cd operator-(const tg_cd &a) { return tg_cd(-a.real(), -a.imag()); }
inline bool operator==(const tg_cd &a, const tg_cd &b) {
  return a.real() == b.real() && a.imag() == b.imag();
}
inline bool operator==(const tg_cd &a, double b) {
  return a.real() == b && a.imag() == 0.0;
}
inline bool operator==(double a, const tg_cd &b) { return b == a; }
inline bool operator!=(const tg_cd &a, const tg_cd &b) { return !(a == b); }
inline bool operator!=(const tg_cd &a, double b) { return !(a == b); }
inline bool operator!=(double a, const tg_cd &b) { return !(b == a); }

inline double real(const tg_cd &a) { return a.real(); }
inline double imag(const tg_cd &a) { return a.imag(); }
inline tg_cd conj(const tg_cd &a) { return tg_cd(a.real(), -a.imag()); }
inline double abs(const tg_cd &a) { return std::fabs(a.real()); }

inline tg_cd sqrt(const tg_cd &a) {
  tg_opcounts.sqrt++;
  return tg_cd(std::sqrt(a.real()));
}
#define TG_OPC_TRANSC(fn)                          \
  inline tg_cd fn(const tg_cd &a) {               \
    tg_opcounts.transc++;                         \
    return tg_cd(std::fn(a.real()));              \
  }
TG_OPC_TRANSC(exp)
TG_OPC_TRANSC(log)
TG_OPC_TRANSC(sin)
TG_OPC_TRANSC(cos)
TG_OPC_TRANSC(tan)
TG_OPC_TRANSC(sinh)
TG_OPC_TRANSC(cosh)
TG_OPC_TRANSC(tanh)
TG_OPC_TRANSC(log10)
#undef TG_OPC_TRANSC
inline tg_cd pow(const tg_cd &a, const tg_cd &b) {
  tg_opcounts.transc++;
  return tg_cd(std::pow(a.real(), b.real()));
}
inline tg_cd pow(const tg_cd &a, double b) {
  tg_opcounts.transc++;
  return tg_cd(std::pow(a.real(), b));
}
inline tg_cd pow(const tg_cd &a, int b) {
  tg_opcounts.transc++;
  return tg_cd(std::pow(a.real(), b));
}
inline tg_cd pow(double a, const tg_cd &b) {
  tg_opcounts.transc++;
  return tg_cd(std::pow(a, b.real()));
}

}  // namespace std

// every later `std::complex<double>` of the reference is the counted scalar
#define complex tg_counted

#endif  // TG_OPCOUNT_H
