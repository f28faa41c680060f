// Small dense helpers shared by the shell and hex element kernels: the
// 2-point Gauss abscissa, 3-vector products, the 3x3 inverse with its
// determinant, and the BCSR block lookup.  Included inside namespace
// tg::<anonymous> by shell_common.cuh and hex_common.cuh (and with them by
// the host-compiled element checks).  The coordinate-dependent helpers
// are templates over the scalar type (double, or ad::Dual).
#pragma once

// TacsGaussQuadPts2 (src/elements/basis/TACSGaussQuadrature.h:26)
#define TG_GPT 0.577350269189626

__device__ __forceinline__ double gauss2(int i) {
  return i ? TG_GPT : -TG_GPT;
}

template <class A, class B>
__device__ __forceinline__ auto dot3(const A *a, const B *b)
    -> decltype(a[0] * b[0]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <class R>
__device__ __forceinline__ void cross3(const R *x, const R *y, R *o) {
  o[0] = x[1] * y[2] - x[2] * y[1];
  o[1] = x[2] * y[0] - x[0] * y[2];
  o[2] = x[0] * y[1] - x[1] * y[0];
}
// inv3x3 (src/elements/TACSElementAlgebra.h:1980)
template <class R>
__device__ R inv3(const R *A, R *Ai) {
  R det = (A[8] * (A[0] * A[4] - A[3] * A[1]) -
           A[7] * (A[0] * A[5] - A[3] * A[2]) +
           A[6] * (A[1] * A[5] - A[2] * A[4]));
  R di = 1.0 / det;
  Ai[0] = (A[4] * A[8] - A[5] * A[7]) * di;
  Ai[1] = -(A[1] * A[8] - A[2] * A[7]) * di;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * di;
  Ai[3] = -(A[3] * A[8] - A[5] * A[6]) * di;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * di;
  Ai[5] = -(A[0] * A[5] - A[2] * A[3]) * di;
  Ai[6] = (A[3] * A[7] - A[4] * A[6]) * di;
  Ai[7] = -(A[0] * A[7] - A[1] * A[6]) * di;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * di;
  return det;
}
// binary search of col in the sorted column list of row
__device__ __forceinline__ int find_slot(const int *rowp, const int *cols,
                                         int row, int col) {
  int lo = rowp[row], hi = rowp[row + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    int c = cols[mid];
    if (c == col) return mid;
    if (c < col) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

