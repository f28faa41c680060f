// CPU check of the host graph routines (tacs_gb300/csrc/mesh_graph.h):
// the element and node colourings and the node pattern, called through
// ctypes by tests/test_mesh_graph.py; test infrastructure only.
#include <vector>

#include "mesh_graph.h"

extern "C" {

// color[nelem]; returns the number of colours
int mg_color_elements(int nn, int npe, int nelem, const int *conn,
                      int *color) {
  std::vector<int> c;
  const int n = tg::graph::color_elements(nn, npe, nelem, conn, c);
  for (int e = 0; e < nelem; e++) color[e] = c[e];
  return n;
}

// pattern of the mesh, then its node colouring: rowp[nn+1]; cols and the
// colours are written up to cap entries; returns nnz
int mg_pattern_and_node_colors(int nn, int npe, int nelem, const int *conn,
                               int cap, int *rowp, int *cols, int *color,
                               int *ncolors) {
  std::vector<int> rp, cs, dg, c;
  tg::graph::node_pattern(nn, npe, nelem, conn, rp, cs, dg);
  *ncolors = tg::graph::color_nodes(nn, rp.data(), cs.data(), c);
  for (int i = 0; i <= nn; i++) rowp[i] = rp[i];
  for (int k = 0; k < (int)cs.size() && k < cap; k++) cols[k] = cs[k];
  for (int i = 0; i < nn; i++) color[i] = c[i];
  return (int)cs.size();
}

// first-writer masks of a 4-node mesh assembled colour by colour (the
// colouring of color_elements); returns 1 with first[nelem] filled, or 0
int mg_first_writers(int nn, int nelem, const int *conn, unsigned *first) {
  std::vector<int> rp, cs, dg, c;
  tg::graph::node_pattern(nn, 4, nelem, conn, rp, cs, dg);
  const int ncol = tg::graph::color_elements(nn, 4, nelem, conn, c);
  std::vector<int> cptr(ncol + 1, 0), celems(nelem);
  for (int e = 0; e < nelem; e++) cptr[c[e] + 1]++;
  for (int k = 0; k < ncol; k++) cptr[k + 1] += cptr[k];
  std::vector<int> fill(cptr.begin(), cptr.end() - 1);
  for (int e = 0; e < nelem; e++) celems[fill[c[e]]++] = e;
  std::vector<uint32_t> f;
  if (!tg::graph::first_writers(nn, nelem, conn, rp, cs, cptr, celems, f))
    return 0;
  for (int e = 0; e < nelem; e++) first[e] = f[e];
  return 1;
}

}  // extern "C"
