// Device sparse direct solver of the Newton systems whose bands are too wide
// for the banded kernels (3D frames and lattices): multifrontal LU over the
// nested-dissection fronts of sparse_analysis.hpp.  No counterpart in the
// reference, which factorises Lλx with UMFPACK (src/SweepX.jl:207-210).
//
// Per factorisation, on the context stream:
//   * equilibration D Lλx D (D = 1/√|aᵢᵢ|; for a zero-diagonal multiplier the
//     scale that makes its largest column entry one);
//   * fronts height by height, leaves first: the matrix entries of the fronts'
//     pivot rows and columns are placed, the children's Schur complements are
//     added (extend-add, child by child in a fixed order), and each front's
//     pivots are eliminated without row exchanges (the multipliers follow the
//     dofs they constrain, so their zero diagonal is never a pivot) in blocks
//     of NB columns: one kernel factors the diagonal block and solves the
//     block's L and U panels, one updates the trailing block;
//   * FP32 factors inside FP64 iterative refinement (residuals of the FP64
//     Lλx), until the scaled correction is below 1e-14 of the scaled solution
//     or stops shrinking below 1e-10 of it (the FP64 residual's attainable
//     accuracy), at most kSparseSweeps sweeps; when that fails the same
//     kernels factorise in FP64 (MGPU_LINSOLVE_SPARSE), or FP64 throughout
//     (_SPARSE64).
// Every sum runs in a fixed order: results are bitwise repeatable.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

struct mgpu_ctx;

namespace mgpu {

struct SpFrontDev {
  int64_t off, idx, eoff;  // front block, index list, extend-add map
  int32_t m, p, pos0, parent;
  int32_t c0, nc;          // children (in extend-add order) in the child list
};

struct SparseDev {
  std::string why;                 // analysis failure, empty when usable
  int64_t n = 0, nnz = 0, fsize = 0;
  int nfront = 0, nheight = 0, nroot = 0, max_m = 0, max_p = 0;
  double flops = 0;
  // per height: fronts (sorted by pivots, descending), storage range, nnz list
  std::vector<int32_t> h_lf0, h_nlf;           // first entry / count in d_lf
  std::vector<int32_t> h_pmax, h_mmax, h_umax;  // largest pivots / front / update rows per height
  std::vector<int64_t> h_off0, h_off1;         // front storage range
  std::vector<int64_t> h_aq0;                  // nnz of the height's fronts: d_aq[h_aq0[h] .. h_aq0[h+1])
  std::vector<std::vector<int32_t>> h_lfp;     // per height: p of the fronts in d_lf order (host, for step counts)
  // per height: fronts taking the blocked substitutions (a prefix of the list),
  // their most pivot tiles and most row tiles (pivot + update)
  std::vector<int32_t> h_nbig, h_bnp, h_bnt;
  std::vector<int32_t> h_spmax, h_sumax;       // most pivots / update rows of the other fronts
  std::vector<int32_t> h_bnu;                  // most update column blocks of the blocked fronts
  int max_m_small = 0;                         // largest front of the one-block substitutions
  int big_pivots = 0;                          // fronts with this many pivots or more: blocked substitutions
  bool tensor_cores = true;                    // FP32 trailing updates on the tensor cores (TF32 ×3; MGPU_SPARSE_TC=0: SIMT)
  bool tc_left = false;                        // the super-panels' left-looking blocks on the tensor cores too (MGPU_SPARSE_TC_LEFT=1)
  bool super_panels = true;                    // FP32 factorisation by super-panels (MGPU_SPARSE_SUPER=0: per 64-column block)
  // per height and child rank: children to add
  std::vector<std::vector<int32_t>> h_ea0, h_nea, h_eumax;
  SpFrontDev* d_fr = nullptr;
  int32_t* d_lf = nullptr;      // fronts by height
  int32_t* d_ea = nullptr;      // children by (height of parent, rank)
  int32_t* d_clist = nullptr;   // children of each front, in rank order
  int32_t* d_fidx = nullptr;
  int32_t* d_emap = nullptr;
  int64_t* d_amap = nullptr;    // [nnz] place in the front buffer
  int32_t* d_aq = nullptr;      // [nnz] nnz indices by height
  int32_t* d_acol = nullptr;    // [nnz] column of each nnz
  int32_t* d_perm = nullptr;    // [n] elimination position -> dof
  int32_t* d_diag = nullptr;    // [n] CSC position of the diagonal, -1 if none
  int64_t* d_colptr = nullptr;  // the CSC pattern of Lλx
  int32_t* d_rowval = nullptr;
  int64_t* d_rptr = nullptr;    // CSR of Lλx for the residual: rows -> nnz and column
  int32_t* d_rq = nullptr;
  int32_t* d_rcol = nullptr;
  float* F32 = nullptr;         // front buffer (FP32 factors)
  double* F64 = nullptr;        // front buffer (FP64 factors), allocated on first use
  double* D = nullptr;          // [2n] equilibration, then the diagonal part of it
  double* cvec = nullptr;       // children's update vectors (forward substitution)
  double* w = nullptr;          // [n] elimination order work vector
  double* V = nullptr;          // [Σ m] the blocked substitutions' front vectors (at each front's idx)
  double* P = nullptr;          // partial products of the blocked fronts' update columns [Σ p·nu]
  int64_t* d_poff = nullptr;    // [nfront] offset of each blocked front's partials in P
  double* tw = nullptr;         // [n] U₁₂ x_u of each pivot (backward substitution)
  double* yacc = nullptr;       // [n] accumulated scaled solution (elimination order)
  double* r = nullptr;          // [n] residual (model order)
  double* xs = nullptr;         // [n] current solution (model order)
  unsigned long long* nrm = nullptr;  // [2] max |correction|, max |solution| (as ordered bits)
  double* prev = nullptr;       // the previous sweep's max |correction|
  int* flags = nullptr;         // [0] converged, [1] sweeps done, [2] perturbed pivots, [3] non-finite pivot
                                // (bit 1: a chained substitution's wait ran out, bit 2: a tensor-core tile's)
  unsigned* tflag = nullptr;    // [ntflag] per blocked front and pivot tile: epoch of the launch that solved it
  int64_t ntflag = 0;
  int* chain = nullptr;         // [2·nheight + 1] work counters of the chained substitutions, abort word
  unsigned epoch = 0;           // of the last chained launch
  int chain_grid32 = 1, chain_grid64 = 1;  // resident blocks of the chained substitutions
  bool chained = true;          // chained substitutions (MGPU_SPARSE_CHAINED=0: one launch per column block)
  int* hflags = nullptr;        // pinned copy
  int last_sweeps = 0, last_fallback = 0, last_perturbed = 0;
  double last_factor_ms = 0, last_refine_ms = 0;  // CUDA-event times of the last solve's factorisation(s), sweeps
  cudaEvent_t ev[4] = {};
  bool fp64_only = false;       // factorise in FP64 throughout
  bool adaptive = true;         // after an FP64 fallback, keep factorising in FP64
};

constexpr int kSparseSweeps = 12;   // refinement sweeps around FP32 factors
constexpr int kSparseSweeps64 = 6;  // around FP64 factors

// analysis and device upload; dof_xyz[n][3] (NaN where unknown) and last[n]
// (constraint multipliers) may be null.  On failure sp->why says why and the
// solver is not usable.
int sparse_create(mgpu_ctx* c, SparseDev*& sp, const double* dof_xyz, const uint8_t* last);
void sparse_destroy(SparseDev*& sp);
// out = Lλx⁻¹ rhs (model order) with Lλx in ctx->nzval.  Synchronises with the
// host once per solve (the refinement's convergence decides the FP64
// fallback).  *info <- 1 on a non-finite or zero pivot in FP64.
int sparse_factor_solve(mgpu_ctx* c, SparseDev& sp, const double* rhs, double* out, int* info);

}  // namespace mgpu
