// Host construction of the assembled-matrix sparsity and of the deterministic
// scatter plans.  Restates asmvec!/asmmat! (src/Assemble.jl:340-448) for the
// SweepX dof group (all X-dofs, identity numbering):
//   * every element contributes the pairs (j,i) of its X-dofs for
//     jeledof, ieledof in column-major order; the CSC pattern is the sorted
//     set of distinct pairs (column j, then row i), colptr/rowval as
//     SparseMatrixCSC, and asm2[ieletyp][i+nX*(j-1), iele] is the nnz index
//     of the pair -- bit-exact with the reference's sortperm construction;
//   * the scatter plans list, for each nnz (and each dof of Lλ), the
//     element entries that add into it, in the reference's accumulation
//     order (element type, then element, then entry), so that the device sum
//     is deterministic and ordered like the reference's loop.
// Counting sort by column + per-column ordering by row replaces the global
// sortperm of (j,i) tuples: it yields the same order and runs in O(pairs).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mgpu {

struct GroupShape {
  int64_t nele;
  int32_t nX;
  const int64_t* indexX;  // [nele][nX] 1-based
};

struct Pattern {
  int64_t n = 0;    // matrix dimension (number of X-dofs)
  int64_t nnz = 0;  // distinct pairs
  std::vector<int64_t> colptr;  // 0-based, n+1
  std::vector<int32_t> rowval;  // 0-based, nnz
  // per group: first pair id and first entry offset in the element matrix buffer
  std::vector<int64_t> pair_base;
  std::vector<int64_t> kbuf_base;  // entry-major buffer: base + (i+nX*j)*nele + e
  std::vector<int64_t> rbuf_base;  // entry-major buffer: base + i*nele + e
  int64_t kbuf_size = 0, rbuf_size = 0;
  std::vector<int32_t> pair_nnz;   // [npair] 0-based nnz of each pair (asm2 - 1)
  // matrix scatter plan: for nnz k, sources msrc[mseg[k] .. mseg[k+1]-1]
  std::vector<uint32_t> mseg;
  std::vector<uint32_t> msrc;
  // vector scatter plan: for dof i, sources vsrc[vseg[i] .. vseg[i+1]-1]
  std::vector<uint32_t> vseg;
  std::vector<uint32_t> vsrc;
};

// Returns an empty string on success, else an error message.
std::string build_pattern(int64_t n, const std::vector<GroupShape>& groups, Pattern& P);

}  // namespace mgpu

#include <cuda_runtime.h>

namespace mgpu {
// The same pattern and plans built on the device (pattern_dev.cu): d_idx[g] the
// group's dof map on the device ([nX][nele], 0-based), on stream st.
std::string build_pattern_device(int64_t n, const std::vector<GroupShape>& groups,
                                 const std::vector<const int32_t*>& d_idx, cudaStream_t st, Pattern& P);

}  // namespace mgpu
