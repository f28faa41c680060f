// Device view of a multifrontal factorisation (direct_kernels.cuh): the
// host analysis of direct_symbolic.h uploaded as it is, and the storage.
// Plain C++ so that the kernels also compile for the CPU check.
#pragma once

#include <cstdint>

namespace tg {

// panel width and trailing tile of the large fronts' factorisation (the
// FP32 factorisation uses kDirectTile32)
constexpr int kDirectPanel = 32, kDirectTile = 32, kDirectTile32 = 64;
// rows of a panel's off-diagonal part solved by one CTA (one per thread)
constexpr int kDirectTrsmRows = 256;
// entries of a front zeroed by one CTA
constexpr int kDirectZeroChunk = 16384;
// column block of the triangular solves, and the shared memory of its
// staged diagonal block (rows padded to kDirectSolveBlock + 1 entries)
constexpr int kDirectSolveBlock = 32;
// threads of the one-CTA-per-front solve kernels
constexpr int kDirectPlainThreads = 128;
// Shared memory of the one-CTA solves beyond the front's rows, in entries
// of elem bytes for nr right-hand sides: the staged diagonal block, which
// the backward solve's partial column sums (at most kDirectPlainThreads
// column groups of 16 bytes of entries, nr each) reuse.
constexpr int direct_plain_extra(int nr, int elem) {
  return kDirectPlainThreads * (16 / elem) * nr >
                 kDirectSolveBlock * (kDirectSolveBlock + 1)
             ? kDirectPlainThreads * (16 / elem) * nr
             : kDirectSolveBlock * (kDirectSolveBlock + 1);
}
// rows of a child's update matrix added into its parent by one CTA
constexpr int kDirectExtendRows = 32;
// CTAs of the thread-block cluster that solves one large front, and the
// front rows above which a front is solved that way
constexpr int kDirectSolveCluster = 8;
// the cluster size (non-portable, where the device schedules it) of the
// levels with at most kDirectWideFronts fronts solved by clusters: twice
// the SMs per front where the chain of blocks, not the level's width,
// sets the time
constexpr int kDirectSolveClusterWide = 16;
constexpr int kDirectWideFronts = 19;
// threads of a CTA of the cluster solves
constexpr int kDirectClusterThreads = 256;
// update rows of one tile of the backward solve's L21^T x2 products for
// the fronts solved by clusters (direct_bwd_gemv_kernel)
constexpr int kDirectGemvRows = 128;
constexpr int kDirectClusterFront = 768;
constexpr int kDirectSolveDiag = kDirectSolveBlock * (kDirectSolveBlock + 1);

// The right-hand side's coupling to the constrained dofs
// (direct::bc_coupling, on the device): nrow block rows with their factor
// positions and blocks, the matrix's column indices and the per-node masks
// of constrained dofs.
struct DirectBc {
  int nrow = 0;
  const int *row = nullptr, *pos = nullptr, *ptr = nullptr, *blk = nullptr,
            *cols = nullptr, *bcmask = nullptr;
};

struct DirectView {
  int bs;
  const int *perm, *bcmask;  // position -> node; boundary dof mask per node
  const int *sn_col, *sn_rowptr, *sn_rows, *sn_parent;
  const int *ea_ptr, *ea_rel, *asm_ptr, *asm_blk, *asm_row, *asm_col;
  const int *ch_ptr, *ch_list;
  const int64_t *l_off, *u_off, *v_off;
  double *lstore, *pool;     // FP64 factor panels and update pool
  float *lstore32, *pool32;  // the same storage for an FP32 factorisation
  // inverses of the 32 x 32 diagonal blocks of the fronts factored by
  // panels (row-major, zero above the diagonal and beyond the block):
  // panel p of supernode s at dinv_off[s] + p * 1024, or dinv_off[s] = -1
  // (none kept: a front factored whole by one CTA)
  const int64_t *dinv_off;
  double *dinv;
  float *dinv32;
};

}  // namespace tg
