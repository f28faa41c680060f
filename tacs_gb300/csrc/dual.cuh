// Forward-mode dual numbers: a value and one directional derivative.
//
// The node-coordinate sensitivity kernels instantiate the element
// kinematics with Dual, one thread per nodal coordinate, seeding the
// derivative of that coordinate with 1.  The result is the exact
// derivative, the quantity the reference forms by complex step in its
// complex build (TACSElement::addAdjResXptProduct and
// TACSElement::addPointQuantityXptSens, src/elements/TACSElement.cpp:270,
// 746) and analytically for the solid element (TACSElement3D.cpp:260,618).
//
// Dual lives in its own namespace so that its sqrt/exp/log overloads are
// found only by argument-dependent lookup and never hide the double ones.
#pragma once

#include <cmath>

namespace tg {
namespace ad {

struct Dual {
  double v, d;
  Dual() = default;
  __host__ __device__ constexpr Dual(double x) : v(x), d(0.0) {}
  __host__ __device__ constexpr Dual(double x, double dx) : v(x), d(dx) {}
  __host__ __device__ Dual &operator+=(const Dual &b) {
    v += b.v;
    d += b.d;
    return *this;
  }
  __host__ __device__ Dual &operator-=(const Dual &b) {
    v -= b.v;
    d -= b.d;
    return *this;
  }
  __host__ __device__ Dual &operator*=(const Dual &b) {
    d = d * b.v + v * b.d;
    v *= b.v;
    return *this;
  }
};

__host__ __device__ inline Dual operator-(const Dual &a) {
  return Dual(-a.v, -a.d);
}
__host__ __device__ inline Dual operator+(const Dual &a, const Dual &b) {
  return Dual(a.v + b.v, a.d + b.d);
}
__host__ __device__ inline Dual operator-(const Dual &a, const Dual &b) {
  return Dual(a.v - b.v, a.d - b.d);
}
__host__ __device__ inline Dual operator*(const Dual &a, const Dual &b) {
  return Dual(a.v * b.v, a.d * b.v + a.v * b.d);
}
__host__ __device__ inline Dual operator/(const Dual &a, const Dual &b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__host__ __device__ inline Dual operator+(const Dual &a, double b) {
  return Dual(a.v + b, a.d);
}
__host__ __device__ inline Dual operator+(double a, const Dual &b) {
  return Dual(a + b.v, b.d);
}
__host__ __device__ inline Dual operator-(const Dual &a, double b) {
  return Dual(a.v - b, a.d);
}
__host__ __device__ inline Dual operator-(double a, const Dual &b) {
  return Dual(a - b.v, -b.d);
}
__host__ __device__ inline Dual operator*(const Dual &a, double b) {
  return Dual(a.v * b, a.d * b);
}
__host__ __device__ inline Dual operator*(double a, const Dual &b) {
  return Dual(a * b.v, a * b.d);
}
__host__ __device__ inline Dual operator/(const Dual &a, double b) {
  return Dual(a.v / b, a.d / b);
}
__host__ __device__ inline Dual operator/(double a, const Dual &b) {
  const double q = a / b.v;
  return Dual(q, -q * b.d / b.v);
}

// comparisons act on the value (branches follow the value's path)
__host__ __device__ inline bool operator<(const Dual &a, const Dual &b) {
  return a.v < b.v;
}
__host__ __device__ inline bool operator>(const Dual &a, const Dual &b) {
  return a.v > b.v;
}
__host__ __device__ inline bool operator!=(const Dual &a, double b) {
  return a.v != b;
}
__host__ __device__ inline bool operator>(const Dual &a, double b) {
  return a.v > b;
}
__host__ __device__ inline bool operator<(const Dual &a, double b) {
  return a.v < b;
}

__device__ inline Dual sqrt(const Dual &a) {
  const double s = ::sqrt(a.v);
  return Dual(s, s != 0.0 ? 0.5 * a.d / s : 0.0);
}
__device__ inline Dual exp(const Dual &a) {
  const double e = ::exp(a.v);
  return Dual(e, e * a.d);
}
__device__ inline Dual log(const Dual &a) {
  return Dual(::log(a.v), a.d / a.v);
}
__device__ inline Dual fabs(const Dual &a) { return a.v < 0.0 ? -a : a; }

}  // namespace ad
}  // namespace tg
