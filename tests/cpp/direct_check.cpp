// CPU check of the direct factorisation's host analysis
// (tacs_gb300/csrc/direct_symbolic.h): a plain dense multifrontal block
// Cholesky driven by the analysis, and the triangular solves, on the host.
// Built by tests/test_direct_symbolic.py with g++ and called through
// ctypes; test infrastructure only.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "direct_symbolic.h"

using tg::direct::Analysis;

namespace {

// Cholesky of the leading c x c block of the row-major m x m matrix F (lower
// triangle), then L21 = F21 L11^-T and F22 -= L21 L21^T.  Returns 0 or the
// 1-based failing pivot.
int front_factor(double *F, int m, int c) {
  for (int k = 0; k < c; k++) {
    double d = F[(size_t)k * m + k];
    for (int q = 0; q < k; q++) d -= F[(size_t)k * m + q] * F[(size_t)k * m + q];
    if (!(d > 0.0)) return k + 1;
    d = std::sqrt(d);
    F[(size_t)k * m + k] = d;
    for (int i = k + 1; i < m; i++) {
      double s = F[(size_t)i * m + k];
      for (int q = 0; q < k; q++) s -= F[(size_t)i * m + q] * F[(size_t)k * m + q];
      F[(size_t)i * m + k] = s / d;
    }
  }
  for (int i = c; i < m; i++)
    for (int j = c; j <= i; j++) {
      double s = 0.0;
      for (int q = 0; q < c; q++) s += F[(size_t)i * m + q] * F[(size_t)j * m + q];
      F[(size_t)i * m + j] -= s;
    }
  return 0;
}

}  // namespace

extern "C" {

// Analysis statistics for the node order `perm` (nullptr: nested
// dissection with `leaf`, by coordinates when xyz is given): out = {supernodes, levels, factor blocks, front
// blocks, scalar flops for bs}.
int dc_analyse(int n, const int *rowp, const int *cols, const int *perm,
               int leaf, int bs, const double *xyz, double *out) {
  std::vector<int> rp(rowp, rowp + n + 1), cs(cols, cols + rowp[n]);
  std::vector<int> p = perm ? std::vector<int>(perm, perm + n)
                            : tg::direct::nested_dissection(rp, cs, leaf, xyz);
  std::vector<int> seen(n, 0);
  for (int v : p) {
    if (v < 0 || v >= n || seen[v]) return -1;
    seen[v] = 1;
  }
  Analysis a = tg::direct::analyse(rp, cs, p);
  out[0] = (double)(a.sn_col.size() - 1);
  out[1] = (double)(a.level_ptr.size() - 1);
  out[2] = (double)a.factor_blocks;
  out[3] = (double)a.front_blocks;
  out[4] = (double)a.flops_scalar(bs);
  return 0;
}

// Nested-dissection order with at most `threads` threads (0: the host's):
// perm (n entries) is the new -> old order.
int dc_nd(int n, const int *rowp, const int *cols, int leaf,
          const double *xyz, int threads, int *perm) {
  std::vector<int> rp(rowp, rowp + n + 1), cs(cols, cols + rowp[n]);
  std::vector<int> p =
      tg::direct::nested_dissection(rp, cs, leaf, xyz, threads);
  if ((int)p.size() != n) return -1;
  std::copy(p.begin(), p.end(), perm);
  return 0;
}

// Storage plan check: out = {factor panel blocks, update pool peak blocks,
// sum of live update blocks at the busiest level, overlapping live pairs}.
int dc_plan(int n, const int *rowp, const int *cols, int leaf,
            const double *xyz, double *out) {
  std::vector<int> rp(rowp, rowp + n + 1), cs(cols, cols + rowp[n]);
  std::vector<int> perm = tg::direct::nested_dissection(rp, cs, leaf, xyz);
  Analysis a = tg::direct::analyse(rp, cs, perm);
  const int ns = (int)a.sn_col.size() - 1;
  std::vector<int> lev(ns);
  for (size_t L = 0; L + 1 < a.level_ptr.size(); L++)
    for (int t = a.level_ptr[L]; t < a.level_ptr[L + 1]; t++)
      lev[a.level_sn[t]] = (int)L;
  int64_t worst = 0, bad = 0;
  for (size_t L = 0; L + 1 < a.level_ptr.size(); L++) {
    // live at level L: made at or below L, consumed at or above L
    std::vector<std::pair<int64_t, int64_t>> iv;
    int64_t sum = 0;
    for (int s = 0; s < ns; s++) {
      if (a.u_off[s] < 0) continue;
      if (lev[s] > (int)L || lev[a.sn_parent[s]] < (int)L) continue;
      const int64_t u = (a.sn_rowptr[s + 1] - a.sn_rowptr[s]) -
                        (a.sn_col[s + 1] - a.sn_col[s]);
      iv.push_back({a.u_off[s], a.u_off[s] + u * u});
      sum += u * u;
    }
    std::sort(iv.begin(), iv.end());
    for (size_t k = 1; k < iv.size(); k++)
      if (iv[k].first < iv[k - 1].second) bad++;
    for (auto &v : iv)
      if (v.second > a.u_peak) bad++;
    worst = std::max(worst, sum);
  }
  out[0] = (double)a.l_total;
  out[1] = (double)a.u_peak;
  out[2] = (double)worst;
  out[3] = (double)bad;
  return 0;
}

// x = A^-1 b for the symmetric positive definite BCSR matrix (rowp, cols,
// vals; bs x bs row-major blocks), factored by the multifrontal scheme in
// nested-dissection order.
int dc_solve(int n, int bs, const int *rowp, const int *cols,
             const double *vals, const double *b, double *x, int leaf,
             const double *xyz) {
  std::vector<int> rp(rowp, rowp + n + 1), cs(cols, cols + rowp[n]);
  std::vector<int> perm = tg::direct::nested_dissection(rp, cs, leaf, xyz);
  Analysis a = tg::direct::analyse(rp, cs, perm);
  const int ns = (int)a.sn_col.size() - 1;
  const size_t b2 = (size_t)bs * bs;
  // factor panels and the update pool laid out by the analysis' plan
  std::vector<double> Lall((size_t)a.l_total * b2), pool((size_t)a.u_peak * b2);
  auto Lp = [&](int s) { return &Lall[(size_t)a.l_off[s] * b2]; };
  auto Up = [&](int s) { return &pool[(size_t)a.u_off[s] * b2]; };
  for (int L0 = 0; L0 + 1 < (int)a.level_ptr.size(); L0++) {
    for (int t = a.level_ptr[L0]; t < a.level_ptr[L0 + 1]; t++) {
      const int s = a.level_sn[t];
      const int mb = a.sn_rowptr[s + 1] - a.sn_rowptr[s];
      const int cb = a.sn_col[s + 1] - a.sn_col[s];
      const int m = mb * bs, c = cb * bs;
      std::vector<double> F((size_t)m * m, 0.0);
      for (int k = a.asm_ptr[s]; k < a.asm_ptr[s + 1]; k++) {
        const double *blk = &vals[b2 * a.asm_blk[k]];
        const int r0 = a.asm_row[k] * bs, c0 = a.asm_col[k] * bs;
        for (int r = 0; r < bs; r++)
          for (int q = 0; q < bs; q++)
            F[(size_t)(r0 + r) * m + c0 + q] += blk[r * bs + q];
      }
      // children's update matrices (children sit on lower levels)
      for (int ch = 0; ch < s; ch++) {
        if (a.sn_parent[ch] != s) continue;
        const int cm = (a.sn_rowptr[ch + 1] - a.sn_rowptr[ch]) -
                       (a.sn_col[ch + 1] - a.sn_col[ch]);
        const int *rel = &a.ea_rel[a.ea_ptr[ch]];
        const double *Uc = Up(ch);
        const int um = cm * bs;
        for (int k1 = 0; k1 < cm; k1++)
          for (int k2 = 0; k2 <= k1; k2++)
            for (int r = 0; r < bs; r++)
              for (int q = 0; q < bs; q++) {
                const int ur = k1 * bs + r, uc = k2 * bs + q;
                if (uc > ur) continue;
                F[(size_t)(rel[k1] * bs + r) * m + rel[k2] * bs + q] +=
                    Uc[(size_t)ur * um + uc];
              }
      }
      // (the upper halves of the diagonal blocks are never read)
      const int rc = front_factor(F.data(), m, c);
      if (rc) return rc;
      double *Ls = Lp(s);
      for (int i = 0; i < m; i++)
        for (int j = 0; j < c; j++)
          Ls[(size_t)i * c + j] = j <= i ? F[(size_t)i * m + j] : 0.0;
      const int um = m - c;
      if (um > 0 && a.sn_parent[s] >= 0) {
        double *Us = Up(s);
        for (int i = 0; i < um; i++)
          for (int j = 0; j < um; j++)
            Us[(size_t)i * um + j] = j <= i ? F[(size_t)(c + i) * m + c + j]
                                            : 0.0;
      }
    }
  }
  // solves in positions
  std::vector<double> y((size_t)n * bs);
  for (int r = 0; r < n; r++)
    for (int q = 0; q < bs; q++) y[(size_t)r * bs + q] = b[(size_t)perm[r] * bs + q];
  for (int s = 0; s < ns; s++) {
    const int mb = a.sn_rowptr[s + 1] - a.sn_rowptr[s];
    const int cb = a.sn_col[s + 1] - a.sn_col[s];
    const int m = mb * bs, c = cb * bs;
    const int *rows = &a.sn_rows[a.sn_rowptr[s]];
    std::vector<double> z(m);
    for (int k = 0; k < mb; k++)
      for (int q = 0; q < bs; q++) z[k * bs + q] = y[(size_t)rows[k] * bs + q];
    for (int i = 0; i < c; i++) {
      double v = z[i];
      for (int j = 0; j < i; j++) v -= Lp(s)[(size_t)i * c + j] * z[j];
      z[i] = v / Lp(s)[(size_t)i * c + i];
    }
    for (int i = c; i < m; i++) {
      double v = 0.0;
      for (int j = 0; j < c; j++) v += Lp(s)[(size_t)i * c + j] * z[j];
      z[i] -= v;
    }
    for (int k = 0; k < mb; k++)
      for (int q = 0; q < bs; q++) y[(size_t)rows[k] * bs + q] = z[k * bs + q];
  }
  for (int s = ns - 1; s >= 0; s--) {
    const int mb = a.sn_rowptr[s + 1] - a.sn_rowptr[s];
    const int cb = a.sn_col[s + 1] - a.sn_col[s];
    const int m = mb * bs, c = cb * bs;
    const int *rows = &a.sn_rows[a.sn_rowptr[s]];
    std::vector<double> z(m);
    for (int k = 0; k < mb; k++)
      for (int q = 0; q < bs; q++) z[k * bs + q] = y[(size_t)rows[k] * bs + q];
    for (int j = 0; j < c; j++) {
      double v = 0.0;
      for (int i = c; i < m; i++) v += Lp(s)[(size_t)i * c + j] * z[i];
      z[j] -= v;
    }
    for (int i = c - 1; i >= 0; i--) {
      double v = z[i];
      for (int j = i + 1; j < c; j++) v -= Lp(s)[(size_t)j * c + i] * z[j];
      z[i] = v / Lp(s)[(size_t)i * c + i];
    }
    for (int k = 0; k < cb; k++)
      for (int q = 0; q < bs; q++) y[(size_t)rows[k] * bs + q] = z[k * bs + q];
  }
  for (int r = 0; r < n; r++)
    for (int q = 0; q < bs; q++) x[(size_t)perm[r] * bs + q] = y[(size_t)r * bs + q];
  return 0;
}

}  // extern "C"
