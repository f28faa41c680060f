// Host-side graph work of an assembler (no CUDA): the node-to-node block
// pattern (TACSAssembler::createMat / computeLocalNodeToNodeCSR) and the
// greedy colourings that make the element scatters and the
// colour-reordered ILU(0) free of write conflicts.  Checked on the CPU by
// tests/test_mesh_graph.py (tests/cpp/mesh_graph_check.cpp).
#pragma once

#include <algorithm>
#include <cstdint>
#include <unordered_map>
#include <vector>

namespace tg {
namespace graph {

// Node-to-node pattern with the diagonal and sorted columns; diag[i] is the
// position of (i, i).
inline void node_pattern(int nn, int npe, int nelem, const int *conn,
                         std::vector<int> &rowp, std::vector<int> &cols,
                         std::vector<int> &diag) {
  std::vector<std::vector<int>> adj(nn);
  for (int i = 0; i < nn; i++) adj[i].push_back(i);
  for (int e = 0; e < nelem; e++)
    for (int i = 0; i < npe; i++)
      for (int j = 0; j < npe; j++)
        adj[conn[npe * e + i]].push_back(conn[npe * e + j]);
  rowp.assign(nn + 1, 0);
  cols.clear();
  diag.assign(nn, -1);
  for (int i = 0; i < nn; i++) {
    auto &r = adj[i];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    for (int c : r) {
      if (c == i) diag[i] = (int)cols.size();
      cols.push_back(c);
    }
    rowp[i + 1] = (int)cols.size();
    std::vector<int>().swap(r);
  }
}

// Greedy element colouring in element order: each element takes the
// smallest colour that no element sharing one of its nodes has taken.
// Colours below 64 are tracked as a bit mask per node, higher ones in a
// per-node list (meshes with a node of high valence), with no limit.
// Returns the number of colours; color[e] is element e's colour.
inline int color_elements(int nn, int npe, int nelem, const int *conn,
                          std::vector<int> &color) {
  std::vector<uint64_t> used(nn, 0);
  std::unordered_map<int, std::vector<int>> over;  // node -> colours >= 64
  std::vector<char> taken;
  color.assign(nelem, 0);
  int ncol = 0;
  for (int e = 0; e < nelem; e++) {
    const int *nd = conn + (size_t)npe * e;
    uint64_t m = 0;
    for (int i = 0; i < npe; i++) m |= used[nd[i]];
    int c = 0;
    while (c < 64 && ((m >> c) & 1ull)) c++;
    if (c == 64) {
      taken.assign(ncol > 64 ? ncol - 64 + 1 : 1, 0);
      for (int i = 0; i < npe; i++) {
        auto it = over.find(nd[i]);
        if (it != over.end())
          for (int x : it->second) taken[x - 64] = 1;
      }
      while (c - 64 < (int)taken.size() && taken[c - 64]) c++;
    }
    color[e] = c;
    ncol = std::max(ncol, c + 1);
    for (int i = 0; i < npe; i++) {
      if (c < 64) used[nd[i]] |= (1ull << c);
      else over[nd[i]].push_back(c);
    }
  }
  return ncol;
}

// First writers of a 4-node element assembly launched colour by colour
// (colour_ptr / colour_elems, in launch order): bit 4 a + b of first[e]
// is set when element e is the first to write block (node a, node b) of
// the pattern (rowp, cols), bit 16 + a when it is the first to write
// node a's residual rows.  Elements of one colour share no node, so each
// block and node has exactly one first writer, which can store instead of
// add (no zero fill).  Returns false -- and no masks -- when a node is in
// no element (its rows would never be written).
inline bool first_writers(int nn, int nelem, const int *conn,
                          const std::vector<int> &rowp,
                          const std::vector<int> &cols,
                          const std::vector<int> &color_ptr,
                          const std::vector<int> &color_elems,
                          std::vector<uint32_t> &first) {
  std::vector<char> node_seen(nn, 0), blk_seen(cols.size(), 0);
  first.assign(nelem, 0u);
  for (size_t c = 0; c + 1 < color_ptr.size(); c++)
    for (int k = color_ptr[c]; k < color_ptr[c + 1]; k++) {
      const int e = color_elems[k];
      const int *nd = conn + 4 * (size_t)e;
      uint32_t m = 0;
      for (int a = 0; a < 4; a++) {
        if (!node_seen[nd[a]]) {
          node_seen[nd[a]] = 1;
          m |= 1u << (16 + a);
        }
        for (int b = 0; b < 4; b++) {
          const int *lo = cols.data() + rowp[nd[a]];
          const int *hi = cols.data() + rowp[nd[a] + 1];
          const int *it = std::lower_bound(lo, hi, nd[b]);
          if (it == hi || *it != nd[b]) return false;
          const size_t slot = (size_t)(it - cols.data());
          if (!blk_seen[slot]) {
            blk_seen[slot] = 1;
            m |= 1u << (4 * a + b);
          }
        }
      }
      first[e] = m;
    }
  for (int i = 0; i < nn; i++)
    if (!node_seen[i]) {
      first.clear();
      return false;
    }
  return true;
}

// Greedy colouring of the node graph (rowp, cols) in node order: each node
// takes the smallest colour none of its already coloured neighbours has.
// Returns the number of colours.
inline int color_nodes(int nn, const int *rowp, const int *cols,
                       std::vector<int> &color) {
  color.assign(nn, -1);
  std::vector<int> stamp;  // stamp[c] == i: colour c is taken around node i
  int ncol = 0;
  for (int i = 0; i < nn; i++) {
    for (int j = rowp[i]; j < rowp[i + 1]; j++) {
      const int c = color[cols[j]];
      if (c < 0) continue;
      if (c >= (int)stamp.size()) stamp.resize(c + 1, -1);
      stamp[c] = i;
    }
    int c = 0;
    while (c < (int)stamp.size() && stamp[c] == i) c++;
    color[i] = c;
    ncol = std::max(ncol, c + 1);
  }
  return ncol;
}

}  // namespace graph
}  // namespace tg
