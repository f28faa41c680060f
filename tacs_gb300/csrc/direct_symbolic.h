// Host analysis of the direct (complete) block factorisation of a
// symmetric block pattern: header-only C++ without CUDA, so the library and
// the CPU tests compile the same code.
//
//   nested_dissection   fill-reducing node order (level-structure bisection)
//   analyse             elimination tree, column structures, fundamental
//                       supernodes, their fronts, the supernodal tree and
//                       its levels, the extend-add maps and the map of the
//                       matrix's lower blocks into the fronts
//
// The numeric phase is a multifrontal block Cholesky (the stiffness matrix
// with row-and-column boundary conditions is symmetric positive definite):
// for each supernode, children before parents, its front (the supernode's
// rows x its columns, dense, bs x bs per block) gathers the matrix's lower
// blocks and the children's update matrices, the leading diagonal block is
// factored, the rows below are solved against it, and the Schur update of
// the rows below goes to the parent.  This replaces the complete-fill
// row-by-row factorisation of the reference's direct preconditioner
// (TACSSchurPc with levFill 1000, src/bpmat/TACSSchurMat.cpp:1510-1600,
// and BCSRMat::computeILUk, src/bpmat/BCSRMat.cpp:625) with the same
// solution.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <iterator>
#include <map>
#include <thread>
#include <vector>

namespace tg {
namespace direct {

// Nested dissection by level structures.  A connected part larger than
// `leaf` vertices is split at a level set of a breadth-first search from a
// pseudo-peripheral vertex (the level where the cumulative count passes
// half the part): the levels before it and after it share no edge, so the
// level set separates them.  Each part is ordered before its separator,
// recursively, so the separator rows come last and the complete factor
// fills only within the parts' own blocks and the separators.  Parts of at
// most `leaf` vertices are ordered by reverse Cuthill-McKee (breadth-first
// from a pseudo-peripheral vertex, reversed).  Disconnected parts are
// ordered one after the other.  The pattern must be symmetric; perm[r] is
// the original row placed at position r.
class NestedDissection {
 public:
  // xyz (3 per vertex, may be null): with coordinates a part is bisected
  // at the median of its widest coordinate instead (recursive coordinate
  // bisection), the separator being the smaller of the two sides' rows of
  // vertices that touch the other side -- straight cuts on meshes, where
  // level sets from a corner are bent
  // threads: at most this many threads (0: the host's hardware threads);
  // the order does not depend on it
  NestedDissection(const std::vector<int> &rowp, const std::vector<int> &cols,
                   int leaf, const double *xyz = nullptr, int threads = 0)
      : rowp_(rowp), cols_(cols), leaf_(leaf < 1 ? 1 : leaf), xyz_(xyz),
        threads_(threads) {}

  std::vector<int> order() {
    const int n = (int)rowp_.size() - 1;
    part_.assign(n, 0);
    dist_.assign(n, -1);
    std::vector<int> out;
    out.reserve(n);
    std::vector<int> all(n);
    for (int i = 0; i < n; i++) all[i] = i;
    next_id_ = 1;
    // the two sides of a cut share no edge and so no vertex that either
    // side's recursion writes: the top levels run them on two threads
    // (each side's order is then appended in the same sequence), at most
    // 2^par_depth_ <= hw threads at a time
    const unsigned hw = threads_ > 0 ? (unsigned)threads_
                                     : std::thread::hardware_concurrency();
    par_depth_ = 0;
    while (par_depth_ < 4 && (2u << par_depth_) <= hw) par_depth_++;
    split(all, 0, out, 0);
    return out;
  }

 private:
  const std::vector<int> &rowp_, &cols_;
  int leaf_;
  const double *xyz_;
  int threads_;
  std::atomic<int> next_id_{1};
  int par_depth_ = 0;
  static constexpr size_t kParMin = 4096;  // smallest part split on threads
  std::vector<int> part_;  // subgraph id of each unordered vertex, -1 once
                           // ordered or held for a separator
  std::vector<int> dist_;

  // breadth-first search inside subgraph `id` from src: visit order in
  // `vis`, distances in dist_ (reset by the caller through `vis`)
  void bfs(int id, int src, std::vector<int> &vis) {
    vis.clear();
    vis.push_back(src);
    dist_[src] = 0;
    for (size_t h = 0; h < vis.size(); h++) {
      const int v = vis[h];
      for (int j = rowp_[v]; j < rowp_[v + 1]; j++) {
        const int w = cols_[j];
        if (part_[w] == id && dist_[w] < 0) {
          dist_[w] = dist_[v] + 1;
          vis.push_back(w);
        }
      }
    }
  }
  void clear_dist(const std::vector<int> &vis) {
    for (int v : vis) dist_[v] = -1;
  }
  int degree(int v) const { return rowp_[v + 1] - rowp_[v]; }

  // pseudo-peripheral vertex of the connected part containing start:
  // repeated searches from the farthest, lowest-degree vertex while the
  // eccentricity grows; vis / dist_ keep the search from the returned
  // vertex
  int peripheral(int id, int start, std::vector<int> &vis) {
    int src = start, ecc = -1;
    for (int it = 0; it < 8; it++) {
      bfs(id, src, vis);
      const int far = dist_[vis.back()];
      if (far <= ecc) break;
      ecc = far;
      int best = vis.back();
      for (size_t k = vis.size(); k-- > 0;) {
        const int v = vis[k];
        if (dist_[v] < far) break;
        if (degree(v) < degree(best)) best = v;
      }
      if (best == src) break;
      clear_dist(vis);
      src = best;
    }
    return src;
  }

  void emit_rcm(const std::vector<int> &vis, std::vector<int> &out) {
    for (size_t k = vis.size(); k-- > 0;) {
      out.push_back(vis[k]);
      part_[vis[k]] = -1;
    }
  }

  // order the vertices `verts` (all with part_ == id), one connected part
  // after the other
  void split(const std::vector<int> &verts, int id, std::vector<int> &out,
             int depth) {
    if (verts.empty()) return;
    std::vector<int> vis;
    bfs(id, verts[0], vis);
    clear_dist(vis);
    if (vis.size() == verts.size()) {
      split_connected(verts, id, out, depth);
      return;
    }
    std::vector<std::pair<std::vector<int>, int>> parts;
    for (int v : verts) {
      if (part_[v] != id) continue;
      bfs(id, v, vis);
      clear_dist(vis);
      const int cid = next_id_++;
      for (int w : vis) part_[w] = cid;
      parts.push_back({vis, cid});
    }
    if (depth < par_depth_ && parts.size() > 1 &&
        verts.size() >= 2 * kParMin) {
      // the parts share no edge: ordered by this branch's share of the
      // threads (2^(par_depth_ - depth)), each taking the next part, then
      // appended in sequence
      std::vector<std::vector<int>> outs(parts.size());
      std::atomic<size_t> next{0};
      auto work = [&] {
        for (size_t i; (i = next++) < parts.size();)
          split_connected(parts[i].first, parts[i].second, outs[i],
                          par_depth_);
      };
      std::vector<std::thread> pool;
      const size_t nt =
          std::min(parts.size(), (size_t)1 << (par_depth_ - depth));
      for (size_t t = 1; t < nt; t++) {
        try {
          pool.emplace_back(work);
        } catch (...) {  // fewer threads
          break;
        }
      }
      work();
      for (auto &t : pool) t.join();
      for (auto &o : outs) out.insert(out.end(), o.begin(), o.end());
      return;
    }
    for (auto &pc : parts) split_connected(pc.first, pc.second, out, depth);
  }

  // order the two sides of a cut, a's then b's (no edge joins them)
  void split_two(const std::vector<int> &a, int ida, const std::vector<int> &b,
                 int idb, std::vector<int> &out, int depth) {
    if (depth < par_depth_ && a.size() >= kParMin && b.size() >= kParMin) {
      std::vector<int> oa, ob;
      std::thread t;
      try {
        t = std::thread([&] { split(a, ida, oa, depth + 1); });
      } catch (...) {  // no thread: in sequence
        split(a, ida, oa, depth + 1);
      }
      split(b, idb, ob, depth + 1);
      if (t.joinable()) t.join();
      out.insert(out.end(), oa.begin(), oa.end());
      out.insert(out.end(), ob.begin(), ob.end());
      return;
    }
    split(a, ida, out, depth + 1);
    split(b, idb, out, depth + 1);
  }

  // coordinate bisection of a connected part; false when it cannot cut
  bool split_coords(const std::vector<int> &verts, int id,
                    std::vector<int> &out, int depth) {
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) lo[d] = hi[d] = xyz_[3 * (size_t)verts[0] + d];
    for (int v : verts)
      for (int d = 0; d < 3; d++) {
        lo[d] = std::min(lo[d], xyz_[3 * (size_t)v + d]);
        hi[d] = std::max(hi[d], xyz_[3 * (size_t)v + d]);
      }
    int ax = 0;
    for (int d = 1; d < 3; d++)
      if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    std::vector<std::pair<double, int>> key(verts.size());
    for (size_t k = 0; k < verts.size(); k++)
      key[k] = {xyz_[3 * (size_t)verts[k] + ax], verts[k]};
    const size_t half = key.size() / 2;
    std::nth_element(key.begin(), key.begin() + half, key.end());
    const int ida = next_id_++, idb = next_id_++;
    for (size_t k = 0; k < key.size(); k++)
      part_[key[k].second] = k < half ? ida : idb;
    // rows of each side that touch the other side
    std::vector<int> sa, sb;
    for (int v : verts) {
      const int own = part_[v], other = own == ida ? idb : ida;
      for (int j = rowp_[v]; j < rowp_[v + 1]; j++)
        if (part_[cols_[j]] == other) {
          (own == ida ? sa : sb).push_back(v);
          break;
        }
    }
    std::vector<int> &sep = sa.size() < sb.size() ? sa : sb;
    const int sep_id = sa.size() < sb.size() ? ida : idb;
    std::vector<int> a, b;
    for (int v : verts) {
      if (part_[v] == ida) a.push_back(v);
      else b.push_back(v);
    }
    const size_t na = a.size() - (sep_id == ida ? sep.size() : 0);
    const size_t nb = b.size() - (sep_id == idb ? sep.size() : 0);
    if (na == 0 || nb == 0) {  // undo: the level-structure split decides
      for (int v : verts) part_[v] = id;
      return false;
    }
    for (int v : sep) part_[v] = -1;
    std::vector<int> a2, b2;
    for (int v : a)
      if (part_[v] == ida) a2.push_back(v);
    for (int v : b)
      if (part_[v] == idb) b2.push_back(v);
    split_two(a2, ida, b2, idb, out, depth);
    for (int v : sep) out.push_back(v);
    return true;
  }

  void split_connected(const std::vector<int> &verts, int id,
                       std::vector<int> &out, int depth) {
    if (xyz_ && (int)verts.size() > leaf_ &&
        split_coords(verts, id, out, depth))
      return;
    std::vector<int> vis;
    peripheral(id, verts[0], vis);
    const int nlev = dist_[vis.back()] + 1;
    if ((int)verts.size() <= leaf_ || nlev < 3) {
      clear_dist(vis);
      emit_rcm(vis, out);
      return;
    }
    // separator level: the smallest level set among those where the
    // cumulative count lies between 35 % and 65 % of the part (the median
    // level when none does), kept off the first and last level so that
    // both sides are non-empty
    std::vector<int> count(nlev, 0);
    for (int v : vis) count[dist_[v]]++;
    const double nv = (double)verts.size();
    size_t acc = 0;
    int sep = -1, median = 1;
    for (int L = 1; L < nlev - 1; L++) {
      const size_t before = acc + count[L - 1];
      acc = before;
      const double lo = before / nv, hi = (before + count[L]) / nv;
      if (lo < 0.5) median = L;
      if (hi >= 0.35 && lo <= 0.65 && (sep < 0 || count[L] < count[sep]))
        sep = L;
    }
    if (sep < 0) sep = median;
    const int ida = next_id_++, idb = next_id_++;
    std::vector<int> a, b, sp;
    for (int v : vis) {
      const int d = dist_[v];
      if (d < sep) {
        part_[v] = ida;
        a.push_back(v);
      } else if (d > sep) {
        part_[v] = idb;
        b.push_back(v);
      } else {
        part_[v] = -1;
        sp.push_back(v);
      }
    }
    clear_dist(vis);
    split_two(a, ida, b, idb, out, depth);
    for (int v : sp) out.push_back(v);
  }
};

inline std::vector<int> nested_dissection(const std::vector<int> &rowp,
                                          const std::vector<int> &cols,
                                          int leaf = 64,
                                          const double *xyz = nullptr,
                                          int threads = 0) {
  NestedDissection nd(rowp, cols, leaf, xyz, threads);
  return nd.order();
}



// Result of the analysis.  Indices called "position" are in the permuted
// order (position r holds original row perm[r]).
struct Analysis {
  int n = 0;                  // block rows
  std::vector<int> perm, iperm;
  std::vector<int> parent;    // elimination tree over positions, -1 = root
  // supernode s owns the consecutive positions [sn_col[s], sn_col[s + 1])
  std::vector<int> sn_col;
  // front rows of s: its own positions, then the positions below them in
  // increasing order; rows [sn_rowptr[s], sn_rowptr[s + 1]) of sn_rows
  std::vector<int> sn_rowptr, sn_rows;
  std::vector<int> sn_parent;  // supernodal tree, -1 = root
  // levels of the supernodal tree (0 = leaves; a supernode's children are
  // all on lower levels): supernodes of level L are
  // level_sn[level_ptr[L] .. level_ptr[L + 1])
  std::vector<int> level_ptr, level_sn;
  // extend-add: the update rows of s (its front rows after its own
  // columns) as row offsets inside the parent's front
  std::vector<int> ea_ptr, ea_rel;  // ea_ptr per supernode
  // the matrix's blocks in the lower triangle of the fronts: for block k
  // of supernode s (asm_ptr[s] .. asm_ptr[s + 1]): the matrix block
  // asm_blk[k] goes to front block row asm_row[k], column asm_colidx[k]
  std::vector<int> asm_ptr, asm_blk, asm_row, asm_col;
  // storage plan, in blocks of bs x bs: supernode s keeps its factor
  // panel (front rows x own columns, dense) at l_off[s] of an array of
  // l_total blocks, and its update matrix ((front rows - own columns)^2,
  // dense) at u_off[s] of a pool of u_peak blocks; the pool is reused, an
  // update living from its supernode's level to its parent's level
  std::vector<int64_t> l_off, u_off;
  int64_t l_total = 0, u_peak = 0;
  // totals
  int64_t factor_blocks = 0;   // blocks of L (lower triangle, diagonal incl.)
  int64_t front_blocks = 0;    // sum over fronts of rows x rows
  int64_t zero_blocks = 0;     // explicit zeros added by amalgamation
  int64_t flops_scalar(int bs) const;
};

// Dense work of the numeric phase in scalar flops for block size bs:
// per supernode with m front rows and c own columns (scalar sizes
// M = m bs, C = c bs): Cholesky C^3 / 3, triangular solve (M - C) C^2,
// update (M - C)^2 C.
inline int64_t Analysis::flops_scalar(int bs) const {
  int64_t f = 0;
  for (size_t s = 0; s + 1 < sn_col.size(); s++) {
    const int64_t c = (int64_t)(sn_col[s + 1] - sn_col[s]) * bs;
    const int64_t m = (int64_t)(sn_rowptr[s + 1] - sn_rowptr[s]) * bs;
    f += c * c * c / 3 + (m - c) * c * c + (m - c) * (m - c) * c;
  }
  return f;
}

struct Analysis;
inline void plan_storage(Analysis &a);

struct AnalysisOptions {
  bool amalgamate = true;  // relaxed supernode amalgamation
  int max_columns = 64;    // widest merged supernode (block columns)
};

// rowp / cols: symmetric block pattern with sorted columns and every
// diagonal present (the assembler's); perm: the node order (new -> old).
inline Analysis analyse(const std::vector<int> &rowp,
                        const std::vector<int> &cols,
                        const std::vector<int> &perm,
                        const AnalysisOptions &opt = AnalysisOptions()) {
  Analysis a;
  const int n = (int)rowp.size() - 1;
  a.n = n;
  a.perm = perm;
  a.iperm.assign(n, 0);
  for (int r = 0; r < n; r++) a.iperm[perm[r]] = r;

  // lower neighbours of each position (positions < r), sorted
  std::vector<int> lptr(n + 1, 0), ladj;
  ladj.reserve(cols.size() / 2 + n);
  for (int r = 0; r < n; r++) {
    const int o = perm[r];
    const size_t b = ladj.size();
    for (int j = rowp[o]; j < rowp[o + 1]; j++) {
      const int c = a.iperm[cols[j]];
      if (c < r) ladj.push_back(c);
    }
    std::sort(ladj.begin() + b, ladj.end());
    lptr[r + 1] = (int)ladj.size();
  }

  // elimination tree (Liu's algorithm with path compression)
  a.parent.assign(n, -1);
  std::vector<int> anc(n, -1);
  for (int r = 0; r < n; r++) {
    for (int k = lptr[r]; k < lptr[r + 1]; k++) {
      int i = ladj[k];
      while (anc[i] != -1 && anc[i] != r) {
        const int t = anc[i];
        anc[i] = r;
        i = t;
      }
      if (anc[i] == -1) {
        anc[i] = r;
        a.parent[i] = r;
      }
    }
  }

  // the upper neighbours of each position in A (rows > r), sorted
  std::vector<int> uptr(n + 1, 0), uadj;
  {
    std::vector<int> cnt(n, 0);
    for (int r = 0; r < n; r++)
      for (int k = lptr[r]; k < lptr[r + 1]; k++) cnt[ladj[k]]++;
    for (int r = 0; r < n; r++) uptr[r + 1] = uptr[r] + cnt[r];
    uadj.resize(uptr[n]);
    std::vector<int> fill(uptr.begin(), uptr.end() - 1);
    for (int r = 0; r < n; r++)  // increasing r: rows of each list sorted
      for (int k = lptr[r]; k < lptr[r + 1]; k++)
        uadj[fill[ladj[k]]++] = r;
  }
  // column counts of L (Gilbert, Ng and Peyton's row-subtree method):
  // row i of L has its nonzeros on the subtree of the elimination tree
  // spanned by the columns j < i with A(i, j) != 0; visiting the columns in
  // postorder, j is a leaf of row i's subtree when its first descendant
  // comes after the previous leaf's, each leaf adds one to its column and
  // one less is counted at the least common ancestor of consecutive leaves
  // (found by path compression); the counts are then these differences
  // summed over each subtree.  So the supernodes follow without forming
  // every column's structure.
  std::vector<int> count(n, 0), nchild(n, 0);
  {
    std::vector<int> head(n, -1), next(n, -1);
    for (int j = n - 1; j >= 0; j--) {
      const int p = a.parent[j];
      if (p >= 0) {
        next[j] = head[p];
        head[p] = j;
        nchild[p]++;
      }
    }
    std::vector<int> post, stack;
    post.reserve(n);
    for (int r = 0; r < n; r++) {
      if (a.parent[r] != -1) continue;
      stack.push_back(r);
      while (!stack.empty()) {
        const int j = stack.back();
        const int c = head[j];
        if (c == -1) {
          stack.pop_back();
          post.push_back(j);
        } else {
          head[j] = next[c];
          stack.push_back(c);
        }
      }
    }
    std::vector<int> firstd(n, -1), delta(n, 0), maxfirst(n, -1),
        prevleaf(n, -1), anc(n);
    for (int k = 0; k < n; k++) {
      int j = post[k];
      delta[j] = firstd[j] == -1 ? 1 : 0;  // a leaf of the tree
      for (; j != -1 && firstd[j] == -1; j = a.parent[j]) firstd[j] = k;
    }
    for (int i = 0; i < n; i++) anc[i] = i;
    for (int k = 0; k < n; k++) {
      const int j = post[k];
      if (a.parent[j] != -1) delta[a.parent[j]]--;
      for (int q = uptr[j]; q < uptr[j + 1]; q++) {
        const int i = uadj[q];  // A(i, j) != 0, i > j
        if (firstd[j] <= maxfirst[i]) continue;  // j not a leaf of row i
        maxfirst[i] = firstd[j];
        const int jprev = prevleaf[i];
        prevleaf[i] = j;
        delta[j]++;
        if (jprev == -1) continue;  // row i's first leaf
        int r = jprev;  // the least common ancestor of jprev and j
        while (r != anc[r]) r = anc[r];
        for (int t = jprev; t != r;) {
          const int up = anc[t];
          anc[t] = r;
          t = up;
        }
        delta[r]--;
      }
      if (a.parent[j] != -1) anc[j] = a.parent[j];
    }
    for (int k = 0; k < n; k++) {
      const int j = post[k];
      if (a.parent[j] != -1) delta[a.parent[j]] += delta[j];
    }
    for (int j = 0; j < n; j++) count[j] = delta[j] - 1;  // below the diagonal
  }

  // fundamental supernodes: j + 1 joins j's supernode when it is j's
  // parent, j is its only child and the structures nest (count drops by 1)
  std::vector<int> first;
  first.push_back(0);
  for (int j = 1; j < n; j++) {
    const bool join = a.parent[j - 1] == j && nchild[j] == 1 &&
                      count[j - 1] == count[j] + 1;
    if (!join) first.push_back(j);
  }
  int ns = (int)first.size();
  if (n == 0) ns = 0;
  std::vector<int> last(ns);  // one past the last column
  for (int s = 0; s < ns; s++) last[s] = s + 1 < ns ? first[s + 1] : n;
  std::vector<int> sn_of(n);
  for (int s = 0; s < ns; s++)
    for (int j = first[s]; j < last[s]; j++) sn_of[j] = s;
  // front rows of a supernode: its own positions, then the rows below them
  // (the structure of L below its last column, count[last - 1] rows), so
  // the amalgamation below decides on front sizes alone and the rows are
  // formed only for the supernodes that survive it
  std::vector<int64_t> msize(ns);
  for (int s = 0; s < ns; s++)
    msize[s] = (last[s] - first[s]) + (int64_t)count[last[s] - 1];
  std::vector<int> spar(ns, -1);
  for (int s = 0; s < ns; s++) {
    const int p = a.parent[last[s] - 1];
    spar[s] = p < 0 ? -1 : sn_of[p];
  }

  // relaxed amalgamation: a child whose columns end where its parent's
  // begin is merged into the parent when the explicit zeros this adds to
  // the merged factor stay below a fraction that shrinks with its width
  // (wide dense fronts suit the GPU, but not at the price of much extra
  // work); merged rows = the child's columns + the parent's rows, which
  // hold every row of the child
  std::vector<int64_t> zeros(ns, 0);
  std::vector<char> alive(ns, 1);
  // a merged supernode's parent links resolve through rep (union-find)
  std::vector<int> rep(ns);
  for (int t = 0; t < ns; t++) rep[t] = t;
  auto find = [&](int t) {
    while (rep[t] != t) t = rep[t] = rep[rep[t]];
    return t;
  };
  if (opt.amalgamate) {
    auto entries = [](int64_t c, int64_t m) {
      return c * (c + 1) / 2 + c * (m - c);
    };
    for (int p = ns - 1; p > 0; p--) {
      if (!alive[p]) continue;
      while (true) {
        if (first[p] == 0) break;
        const int c = sn_of[first[p] - 1];
        if (!alive[c] || spar[c] < 0 || find(spar[c]) != p) break;
        const int64_t nc = last[c] - first[c], np = last[p] - first[p];
        const int64_t mc = msize[c], mp = msize[p];
        const int64_t add = nc * (mp - (mc - nc));
        const int64_t z = zeros[c] + zeros[p] + add;
        const int64_t tot = entries(nc + np, nc + mp);
        const int64_t w = nc + np;
        const double frac = w <= 4 ? 0.5 : w <= 16 ? 0.25 : w <= 48 ? 0.1
                                                               : 0.05;
        if (w > opt.max_columns || (double)z > frac * (double)tot) break;
        // merge c into p
        msize[p] = nc + mp;
        for (int j = first[c]; j < last[c]; j++) sn_of[j] = p;
        first[p] = first[c];
        zeros[p] = z;
        alive[c] = 0;
        rep[c] = p;  // c's children now hang on p
      }
    }
  }
  // renumber the surviving supernodes in column order
  std::vector<int> newid(ns, -1);
  int nsurv = 0;
  for (int s = 0; s < ns; s++)
    if (alive[s]) newid[s] = nsurv++;
  a.sn_col.assign(nsurv + 1, 0);
  a.sn_rowptr.assign(nsurv + 1, 0);
  a.sn_parent.assign(nsurv, -1);
  for (int s = 0; s < ns; s++) {
    if (!alive[s]) continue;
    const int t = newid[s];
    a.sn_col[t] = first[s];
    a.sn_parent[t] = spar[s] < 0 ? -1 : newid[find(spar[s])];
    a.sn_rowptr[t + 1] = a.sn_rowptr[t] + (int)msize[s];
    const int64_t m = msize[s], c = last[s] - first[s];
    a.front_blocks += m * m;
    a.factor_blocks += c * (c + 1) / 2 + (m - c) * c;
    a.zero_blocks += zeros[s];
  }
  if (nsurv > 0) a.sn_col[nsurv] = n;
  ns = nsurv;
  // the rows of each surviving supernode (children before parents): its
  // own positions, the upper neighbours of its columns and its children's
  // rows below their own columns, sorted -- the union of its columns'
  // structures in L
  a.sn_rows.assign(a.sn_rowptr[ns], 0);
  {
    std::vector<int> shead(ns, -1), snext(ns, -1), mark(n, -1);
    for (int s = ns - 1; s >= 0; s--) {
      const int p = a.sn_parent[s];
      if (p >= 0) {
        snext[s] = shead[p];
        shead[p] = s;
      }
    }
    for (int s = 0; s < ns; s++) {
      int *r = &a.sn_rows[a.sn_rowptr[s]];
      const int m = a.sn_rowptr[s + 1] - a.sn_rowptr[s];
      int len = 0;
      for (int j = a.sn_col[s]; j < a.sn_col[s + 1]; j++) {
        r[len++] = j;
        mark[j] = s;
      }
      const int own = len;
      for (int j = a.sn_col[s]; j < a.sn_col[s + 1]; j++)
        for (int q = uptr[j]; q < uptr[j + 1]; q++)
          if (mark[uadj[q]] != s && len < m) {
            mark[uadj[q]] = s;
            r[len++] = uadj[q];
          }
      for (int c = shead[s]; c >= 0; c = snext[c]) {
        const int cown = a.sn_col[c + 1] - a.sn_col[c];
        for (int t = a.sn_rowptr[c] + cown; t < a.sn_rowptr[c + 1]; t++) {
          const int i = a.sn_rows[t];
          if (mark[i] != s && len < m) {
            mark[i] = s;
            r[len++] = i;
          }
        }
      }
      std::sort(r + own, r + len);
    }
  }

  // levels: leaves 0, a parent one above its highest child
  std::vector<int> lev(ns, 0);
  int nlev = ns > 0 ? 1 : 0;
  for (int s = 0; s < ns; s++) {  // children precede parents in positions
    const int p = a.sn_parent[s];
    if (p >= 0 && lev[p] < lev[s] + 1) lev[p] = lev[s] + 1;
    nlev = std::max(nlev, lev[s] + 1);
  }
  a.level_ptr.assign(nlev + 1, 0);
  for (int s = 0; s < ns; s++) a.level_ptr[lev[s] + 1]++;
  for (int L = 0; L < nlev; L++) a.level_ptr[L + 1] += a.level_ptr[L];
  a.level_sn.assign(ns, 0);
  {
    std::vector<int> fill(a.level_ptr.begin(), a.level_ptr.end() - 1);
    for (int s = 0; s < ns; s++) a.level_sn[fill[lev[s]]++] = s;
  }

  // extend-add maps: each update row of s as a row of the parent's front
  a.ea_ptr.assign(ns + 1, 0);
  a.ea_rel.clear();
  for (int s = 0; s < ns; s++) {
    const int p = a.sn_parent[s];
    const int own = a.sn_col[s + 1] - a.sn_col[s];
    const int *rows = &a.sn_rows[a.sn_rowptr[s]];
    const int m = a.sn_rowptr[s + 1] - a.sn_rowptr[s];
    if (p >= 0) {
      const int *prow = &a.sn_rows[a.sn_rowptr[p]];
      const int pm = a.sn_rowptr[p + 1] - a.sn_rowptr[p];
      int q = 0;
      for (int k = own; k < m; k++) {  // both lists sorted
        while (q < pm && prow[q] < rows[k]) q++;
        a.ea_rel.push_back(q);  // q < pm: the parent's front holds it
      }
    }
    a.ea_ptr[s + 1] = (int)a.ea_rel.size();
  }

  // the matrix's lower blocks (position i >= j) in the front of j's
  // supernode: block row = index of i in the front rows, block column =
  // j - first column.  Block (i, j) of the permuted matrix is stored in
  // row perm[i] of A at column perm[j]: the mirror of A's block at (row
  // perm[j], column perm[i]), found through the transpose map (with sorted
  // columns, the t-th visit of column c in a pass over rows in increasing
  // order is the t-th entry of row c); the front row of i through a
  // scatter of the supernode's rows
  std::vector<int> mirror(cols.size());
  {
    std::vector<int> cur(rowp.begin(), rowp.end() - 1);
    for (int o = 0; o < n; o++)
      for (int k = rowp[o]; k < rowp[o + 1]; k++) mirror[k] = cur[cols[k]]++;
  }
  std::vector<int> where(n, -1);
  a.asm_ptr.assign(ns + 1, 0);
  const size_t nlow = (cols.size() + (size_t)n) / 2;  // i >= j blocks
  a.asm_blk.clear();
  a.asm_row.clear();
  a.asm_col.clear();
  a.asm_blk.reserve(nlow);
  a.asm_row.reserve(nlow);
  a.asm_col.reserve(nlow);
  for (int s = 0; s < ns; s++) {
    for (int t = a.sn_rowptr[s]; t < a.sn_rowptr[s + 1]; t++)
      where[a.sn_rows[t]] = t - a.sn_rowptr[s];
    for (int j = a.sn_col[s]; j < a.sn_col[s + 1]; j++) {
      const int oj = perm[j];
      // column j of the permuted matrix = row oj of A (symmetric pattern)
      for (int k = rowp[oj]; k < rowp[oj + 1]; k++) {
        const int i = a.iperm[cols[k]];
        if (i < j) continue;
        a.asm_blk.push_back(mirror[k]);
        a.asm_row.push_back(where[i]);
        a.asm_col.push_back(j - a.sn_col[s]);
      }
    }
    a.asm_ptr[s + 1] = (int)a.asm_blk.size();
  }
  plan_storage(a);
  return a;
}

// First-fit allocation in a pool of one address range: an allocation
// takes the free block of lowest offset that is large enough (or the top
// of the range), a release merges with free neighbours.  Free blocks are
// indexed by offset (for merging) and by size class (floor log2 of the
// size: every block of a higher class fits, so the first fit is the
// lowest offset among the higher classes' first blocks and the fitting
// blocks of the request's own class), which keeps each allocation near
// logarithmic where a scan of all free blocks was linear.
class PoolPlan {
 public:
  int64_t alloc(int64_t size) {
    const int c = cls(size);
    int64_t best = -1;
    for (const auto &blk : by_cls_[c])
      if (blk.second >= size) {
        best = blk.first;
        break;
      }
    for (int k = c + 1; k < kClasses; k++)
      if (!by_cls_[k].empty() &&
          (best < 0 || by_cls_[k].begin()->first < best))
        best = by_cls_[k].begin()->first;
    if (best < 0) {
      const int64_t off = top_;
      top_ += size;
      peak_ = std::max(peak_, top_);
      return off;
    }
    const int64_t rest = free_[best] - size;
    erase(best);
    if (rest > 0) insert(best + size, rest);
    return best;
  }
  void release(int64_t off, int64_t size) {
    if (size <= 0) return;
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && off + size == nx->first) {
      size += nx->second;
      erase(nx->first);
    }
    auto pv = free_.lower_bound(off);
    if (pv != free_.begin()) {
      --pv;
      if (pv->first + pv->second == off) {
        off = pv->first;
        size += pv->second;
        erase(off);
      }
    }
    if (off + size == top_) {
      top_ = off;
      return;
    }
    insert(off, size);
  }
  int64_t peak() const { return peak_; }

 private:
  static constexpr int kClasses = 64;
  static int cls(int64_t size) {
    int c = 0;
    while (c + 1 < kClasses && (size >> (c + 1)) > 0) c++;
    return c;
  }
  void insert(int64_t off, int64_t size) {
    free_[off] = size;
    by_cls_[cls(size)].emplace(off, size);
  }
  void erase(int64_t off) {
    auto it = free_.find(off);
    by_cls_[cls(it->second)].erase(off);
    free_.erase(it);
  }
  std::map<int64_t, int64_t> free_;
  std::map<int64_t, int64_t> by_cls_[kClasses];  // offset -> size
  int64_t top_ = 0, peak_ = 0;
};

// Factor panels back to back; updates from a pool: the supernodes of a
// level allocate theirs, and the updates their children handed up are
// released once the level is done.
inline void plan_storage(Analysis &a) {
  const int ns = (int)a.sn_col.size() - 1;
  a.l_off.assign(ns, 0);
  a.u_off.assign(ns, -1);
  int64_t acc = 0;
  for (int s = 0; s < ns; s++) {
    const int64_t m = a.sn_rowptr[s + 1] - a.sn_rowptr[s];
    const int64_t c = a.sn_col[s + 1] - a.sn_col[s];
    a.l_off[s] = acc;
    acc += m * c;
  }
  a.l_total = acc;
  std::vector<int> cptr(ns + 1, 0), cl(ns > 0 ? ns : 1);
  for (int s = 0; s < ns; s++)
    if (a.sn_parent[s] >= 0) cptr[a.sn_parent[s] + 1]++;
  for (int s = 0; s < ns; s++) cptr[s + 1] += cptr[s];
  {
    std::vector<int> fill(cptr.begin(), cptr.end() - 1);
    for (int s = 0; s < ns; s++)
      if (a.sn_parent[s] >= 0) cl[fill[a.sn_parent[s]]++] = s;
  }
  auto usize = [&](int s) {
    const int64_t u = (a.sn_rowptr[s + 1] - a.sn_rowptr[s]) -
                      (a.sn_col[s + 1] - a.sn_col[s]);
    return u * u;
  };
  PoolPlan pool;
  for (size_t L = 0; L + 1 < a.level_ptr.size(); L++) {
    for (int t = a.level_ptr[L]; t < a.level_ptr[L + 1]; t++) {
      const int s = a.level_sn[t];
      if (usize(s) > 0 && a.sn_parent[s] >= 0) a.u_off[s] = pool.alloc(usize(s));
    }
    for (int t = a.level_ptr[L]; t < a.level_ptr[L + 1]; t++) {
      const int s = a.level_sn[t];
      for (int k = cptr[s]; k < cptr[s + 1]; k++)
        if (a.u_off[cl[k]] >= 0) pool.release(a.u_off[cl[k]], usize(cl[k]));
    }
  }
  a.u_peak = pool.peak();
}

// The factor's launch plan for fronts of more than small_max scalar rows:
// they are factored level by level in panel steps of `panel` columns,
// step p of a level taking the p-th panel of every large front of the
// level that has one, then one grid over the lower-triangular
// tile x tile blocks of all their trailing matrices.  Step t covers
// fronts[front_off[t] .. + count[t]) at column k0[t]; tprefix[tile_off[t]
// .. + count[t] + 1) is the prefix sum of their tile counts (total[t] in
// all).  Shared by the runtime and the CPU emulation of its launches.
//   Below each panel's diagonal block, the rows solved against it go in blocks
// of `rows` rows: rprefix[tile_off[t] .. + count[t] + 1) is the prefix sum
// of the fronts' row-block counts (rtotal[t] in all).
struct PanelSteps {
  std::vector<int> level, k0, front_off, count, tile_off, total, rtotal;
  std::vector<int> fronts, tprefix, rprefix;
};

inline PanelSteps panel_steps(const Analysis &an, int bs, int small_max,
                              int panel, int tile, int rows) {
  PanelSteps ps;
  const int nl = (int)an.level_ptr.size() - 1;
  std::vector<int> large;
  for (int L = 0; L < nl; L++) {
    large.clear();
    int maxc = 0;
    for (int t = an.level_ptr[L]; t < an.level_ptr[L + 1]; t++) {
      const int s = an.level_sn[t];
      const int M = (an.sn_rowptr[s + 1] - an.sn_rowptr[s]) * bs;
      const int C = (an.sn_col[s + 1] - an.sn_col[s]) * bs;
      if (M <= small_max) continue;
      large.push_back(s);
      maxc = std::max(maxc, C);
    }
    for (int k0 = 0; k0 < maxc; k0 += panel) {
      ps.level.push_back(L);
      ps.k0.push_back(k0);
      ps.front_off.push_back((int)ps.fronts.size());
      ps.tile_off.push_back((int)ps.tprefix.size());
      int cnt = 0, tiles = 0, rblocks = 0;
      ps.tprefix.push_back(0);
      ps.rprefix.push_back(0);
      for (int s : large) {
        const int M = (an.sn_rowptr[s + 1] - an.sn_rowptr[s]) * bs;
        const int C = (an.sn_col[s + 1] - an.sn_col[s]) * bs;
        if (C <= k0) continue;
        const int nb = std::min(panel, C - k0);
        const int rest = M - (k0 + nb);
        const int nt = rest > 0 ? (rest + tile - 1) / tile : 0;
        ps.fronts.push_back(s);
        tiles += nt * (nt + 1) / 2;
        ps.tprefix.push_back(tiles);
        rblocks += rest > 0 ? (rest + rows - 1) / rows : 0;
        ps.rprefix.push_back(rblocks);
        cnt++;
      }
      ps.count.push_back(cnt);
      ps.total.push_back(tiles);
      ps.rtotal.push_back(rblocks);
    }
  }
  return ps;
}

// The coupling of the right-hand side to the constrained dofs: the
// assembled matrix keeps the columns of the constrained dofs (only their
// rows are the identity), while the factorisation holds the matrix with
// those rows and columns removed, so a solve takes b' = b - A_{:,c} b_c on
// the free dofs.  Listed here: the block rows i with a block in a column
// whose node has a constrained dof (row[k] = i, pos[k] = i's position in
// the factor order, its blocks blk[ptr[k] .. ptr[k + 1]) as indices into
// the BCSR value array), so that the correction touches those blocks only.
struct BcCoupling {
  std::vector<int> row, pos, ptr{0}, blk;
};
inline BcCoupling bc_coupling(const std::vector<int> &rowp,
                              const std::vector<int> &cols,
                              const std::vector<int> &bcmask,
                              const std::vector<int> &iperm) {
  BcCoupling c;
  const int n = (int)rowp.size() - 1;
  for (int i = 0; i < n; i++) {
    const size_t before = c.blk.size();
    for (int k = rowp[i]; k < rowp[i + 1]; k++)
      if (bcmask[cols[k]]) c.blk.push_back(k);
    if (c.blk.size() == before) continue;
    c.row.push_back(i);
    c.pos.push_back(iperm[i]);
    c.ptr.push_back((int)c.blk.size());
  }
  return c;
}

}  // namespace direct
}  // namespace tg
