// CPU check of the fixed-geometry plan (tacs_gb300/csrc/geo_plan.h): the
// per-block contribution lists, the geometry classes and the row schedule,
// called through ctypes by tests/test_geo_plan.py; test infrastructure only.
#include <vector>

#include "geo_plan.h"
#include "mesh_graph.h"

extern "C" {

// pattern + contributions of a mesh: rowp[nn+1]; cols, cptr[nnz+1] and
// contrib written up to cap entries each; returns nnz (or -1)
int gp_contributions(int nn, int npe, int nelem, const int *conn, int cap,
                     int *rowp, int *cols, int *cptr, int *contrib,
                     int *ncontrib) {
  std::vector<int> rp, cs, dg, cp, ct;
  tg::graph::node_pattern(nn, npe, nelem, conn, rp, cs, dg);
  if (tg::geo::contributions(nelem, npe, conn, rp, cs, cp, ct)) return -1;
  for (int i = 0; i <= nn; i++) rowp[i] = rp[i];
  for (int k = 0; k < (int)cs.size() && k < cap; k++) cols[k] = cs[k];
  for (int k = 0; k < (int)cp.size() && k < cap; k++) cptr[k] = cp[k];
  for (int k = 0; k < (int)ct.size() && k < cap; k++) contrib[k] = ct[k];
  *ncontrib = (int)ct.size();
  return (int)cs.size();
}

// classes[nelem], reps[<= nelem]; returns the number of classes
int gp_classes(int nelem, int npe, const int *conn, const double *xpts,
               int *cls, int *reps) {
  std::vector<int> c, r;
  const int n = tg::geo::geometry_classes(nelem, npe, conn, xpts, c, r);
  for (int e = 0; e < nelem; e++) cls[e] = c[e];
  for (int k = 0; k < n; k++) reps[k] = r[k];
  return n;
}

// longest row of every 32-row group: kmax[(nrows + 31) / 32]
void gp_row_lengths(int nrows, const int *rowp, int *kmax) {
  std::vector<int> rp(rowp, rowp + nrows + 1), k;
  tg::geo::warp_row_lengths(rp, k);
  for (size_t i = 0; i < k.size(); i++) kmax[i] = k[i];
}

}  // extern "C"
