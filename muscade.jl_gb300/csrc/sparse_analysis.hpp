// Host analysis of the sparse direct solver (no counterpart in the reference,
// which factorises Lλx with UMFPACK at every Newton iteration,
// src/SweepX.jl:207-210).  Used for matrices whose bands are too wide for the
// banded device solvers: 3D frames and lattices.
//
//   1. Compression.  Dofs with the same closed neighbourhood in the pattern
//      (the dofs of one node) form one group; a group whose only neighbour is
//      one other group (the multiplier of a Hold on one node dof) joins it, and
//      groups are merged again by closed neighbourhood.  Within a group the
//      constraint multipliers come last, after the dofs they constrain, so that
//      the factorisation never meets their zero diagonal first.
//   2. Ordering.  Nested dissection of the group graph by recursive coordinate
//      bisection: connected components are independent subtrees; a part is split
//      at the median of its longest coordinate extent, and the vertices of the
//      upper half that touch the lower half form the separator.  Coordinates
//      come from the beam and bar elements' nodes; groups without any take the
//      mean of their neighbours'.
//   3. Symbolic factorisation.  Every leaf part and every separator is one
//      supernode ("front").  A front's index list is its pivots (its own dofs,
//      contiguous in elimination order) followed by the later dofs its pivots
//      couple to, directly or through fill from its subtree.
//   4. Layout.  Each front is a dense m × m column-major block in one buffer;
//      fronts of one height (leaves 0, parent = 1 + max over children) lie
//      together.  Maps give, for every nnz of Lλx, its place in a front, and for
//      every child, where each of its update rows goes in the parent.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mgpu {

struct SparseInput {
  int64_t n = 0;
  const int64_t* colptr = nullptr;  // [n+1] 0-based CSC pattern of Lλx (structurally symmetric)
  const int32_t* rowval = nullptr;  // [nnz]
  const double* xyz = nullptr;      // [n][3] coordinates of each dof's node (NaN when unknown), or nullptr
  const uint8_t* last = nullptr;    // [n] 1 for constraint multipliers, or nullptr
  int leaf_groups = 8;              // nested dissection stops at parts of at most this many groups
};

struct SparseFront {
  int64_t off = 0;     // first entry of the m × m block in the front buffer
  int64_t idx = 0;     // first entry of the index list (elimination positions) in fidx
  int64_t eoff = -1;   // first entry of this front's extend-add map (update rows -> parent's local index)
  int32_t m = 0, p = 0;
  int32_t pos0 = 0;    // elimination position of the first pivot (pivots are pos0 .. pos0+p-1)
  int32_t parent = -1;
  int32_t height = 0;
  int32_t crank = 0;   // rank of this front among its parent's children (extend-add order)
};

struct SparseAnalysis {
  int64_t n = 0, nnz = 0;
  std::vector<int32_t> perm;   // [n] elimination position -> dof
  std::vector<int32_t> ipos;   // [n] dof -> elimination position
  std::vector<SparseFront> fronts;  // postorder: children before parents
  std::vector<int32_t> fidx;   // index lists (elimination positions), per front m entries
  std::vector<int32_t> emap;   // extend-add maps, per non-root front m - p entries
  std::vector<int64_t> amap;   // [nnz] place of each nnz in the front buffer
  std::vector<int32_t> diag;   // [n] CSC position of each diagonal entry, -1 if absent
  int64_t fsize = 0;           // entries of the front buffer (Σ m²)
  int nheight = 0;
  int max_children = 0;
  int ngroups = 0;
  double flops = 0;            // LU flops of the partial factorisations (2 per multiply-add)
  int32_t max_m = 0, max_p = 0;
};

// Returns an empty string on success, else the reason.
std::string sparse_analyse(const SparseInput& in, SparseAnalysis& out);

}  // namespace mgpu
