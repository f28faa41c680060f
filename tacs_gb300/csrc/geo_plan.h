// Host-side plan of the fixed-geometry assembly (no CUDA): for linear
// elements whose stiffness is a fixed combination of the element scale t
// (MITC4 with TACSIsoShellConstitutive, tOffset 0: K = t K1 + t^3 K3;
// hex8 with TACSSolidConstitutive: K = t K1), the element matrices depend
// on the node coordinates only through K1 and K3, which are formed once per
// distinct element geometry.  This header builds
//   * the contribution lists: for every block slot (i, j) of the BCSR
//     pattern, the (element, a, b) pairs with conn[e][a] = i and
//     conn[e][b] = j, in element order (so every block's sum has a fixed
//     order), packed as (e << 6) | (npe a + b);
//   * the geometry classes: elements whose node coordinates relative to
//     their first node are bitwise equal share one class; the first such
//     element is the class representative;
//   * the row schedule: rows in groups of 32 (one warp), each group's
//     longest row.
// Checked on the CPU by tests/test_geo_plan.py (tests/cpp/geo_plan_check.cpp).
#pragma once

#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace tg {
namespace geo {

constexpr int kAbBits = 6;  // npe * a + b < 64 for npe <= 8

// Slot of (row, col) in a sorted-column BCSR pattern, -1 if absent.
inline int find_col(const int *rowp, const int *cols, int row, int col) {
  int lo = rowp[row], hi = rowp[row + 1] - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (cols[mid] == col) return mid;
    if (cols[mid] < col) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

// Contribution lists in CSR form over the nnz slots.  Returns 0, or -1 if
// an element's node pair has no slot or the element count does not fit
// the packing (nelem >= 2^25).
inline int contributions(int nelem, int npe, const int *conn,
                         const std::vector<int> &rowp,
                         const std::vector<int> &cols, std::vector<int> &cptr,
                         std::vector<int> &contrib) {
  if (nelem >= (1 << (31 - kAbBits))) return -1;
  const int nnz = (int)cols.size();
  std::vector<int> slot((size_t)nelem * npe * npe);
  cptr.assign(nnz + 1, 0);
  for (int e = 0; e < nelem; e++)
    for (int a = 0; a < npe; a++)
      for (int b = 0; b < npe; b++) {
        const int s = find_col(rowp.data(), cols.data(), conn[npe * e + a],
                               conn[npe * e + b]);
        if (s < 0) return -1;
        slot[((size_t)e * npe + a) * npe + b] = s;
        cptr[s + 1]++;
      }
  for (int s = 0; s < nnz; s++) cptr[s + 1] += cptr[s];
  contrib.assign(cptr[nnz], 0);
  std::vector<int> fill(cptr.begin(), cptr.end() - 1);
  for (int e = 0; e < nelem; e++)  // element order within every slot
    for (int a = 0; a < npe; a++)
      for (int b = 0; b < npe; b++) {
        const int s = slot[((size_t)e * npe + a) * npe + b];
        contrib[fill[s]++] = (e << kAbBits) | (npe * a + b);
      }
  return 0;
}

// Geometry classes by the bit patterns of X_k - X_0 (k = 1..npe-1).
// cls[e] is the class of element e, reps[c] the representative (first
// element) of class c.  Returns the number of classes.
inline int geometry_classes(int nelem, int npe, const int *conn,
                            const double *xpts, std::vector<int> &cls,
                            std::vector<int> &reps) {
  const int nk = 3 * (npe - 1);
  struct Hash {
    size_t operator()(const std::vector<uint64_t> &k) const {
      uint64_t h = 1469598103934665603ull;
      for (uint64_t v : k) {
        h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
        h *= 1099511628211ull;
      }
      return (size_t)h;
    }
  };
  std::unordered_map<std::vector<uint64_t>, int, Hash> map;
  map.reserve(64);
  cls.assign(nelem, 0);
  reps.clear();
  std::vector<uint64_t> key(nk);
  for (int e = 0; e < nelem; e++) {
    const double *x0 = xpts + 3 * (size_t)conn[npe * e];
    for (int k = 1; k < npe; k++) {
      const double *xk = xpts + 3 * (size_t)conn[npe * e + k];
      for (int d = 0; d < 3; d++) {
        const double v = xk[d] - x0[d];
        uint64_t bits;
        std::memcpy(&bits, &v, sizeof(bits));
        key[3 * (k - 1) + d] = bits;
      }
    }
    auto it = map.find(key);
    if (it == map.end()) {
      const int c = (int)reps.size();
      map.emplace(key, c);
      reps.push_back(e);
      cls[e] = c;
    } else {
      cls[e] = it->second;
    }
  }
  return (int)reps.size();
}

// Longest row of each group of 32 consecutive rows.
inline void warp_row_lengths(const std::vector<int> &rowp,
                             std::vector<int> &kmax) {
  const int nrows = (int)rowp.size() - 1;
  const int nw = (nrows + 31) / 32;
  kmax.assign(nw, 0);
  for (int i = 0; i < nrows; i++) {
    const int len = rowp[i + 1] - rowp[i];
    if (len > kmax[i / 32]) kmax[i / 32] = len;
  }
}

// Constraint mask of every node: the OR of its addBCs entries.
inline void node_bc_masks(int nnodes, const std::vector<int> &bc_nodes,
                          const std::vector<int> &bc_masks,
                          std::vector<int> &node_bc) {
  node_bc.assign(nnodes, 0);
  for (size_t k = 0; k < bc_nodes.size(); k++)
    if (bc_nodes[k] >= 0 && bc_nodes[k] < nnodes)
      node_bc[bc_nodes[k]] |= bc_masks[k];
}

}  // namespace geo
}  // namespace tg
