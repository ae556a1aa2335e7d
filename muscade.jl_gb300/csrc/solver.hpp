// Linear solver state shared by the Newton drivers (solver.cu) and the
// adjoint (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "band_torn.cuh"
#include "ctx.hpp"
#include "sparse_lu.hpp"

namespace mgpu {

constexpr int kNormBlocks = 128;
constexpr int64_t kTornMinDofs = 512;  // components shorter than this are factorised whole
constexpr int kInfoSlots = 64;  // a captured step holds up to kInfoSlots-1 iterations
constexpr int kFusedMaxP = 32;  // the fused per-component partitioned solve takes components of up to 32 interiors
constexpr int kFusedMaxW = kTbFusedMaxThreads / 32;  // and runs at most that many warps per block

enum SolverPath : int {
  PATH_F32IR = 0,  // row-band warp kernels, FP32 factors + FP64 refinement, FP64 fallback per component
  PATH_F64ROWS = 1,  // row-band warp kernels in FP64
  PATH_BLOCK = 2,  // gbtf2-layout block kernels in FP64 (any band width up to 256)
  PATH_TORN = 3,   // long components cut into interiors and separators, FP64
  PATH_TORN32 = 4,  // the same with FP32 factors inside FP64 iterative refinement, FP64 fallback per component
  PATH_SPARSE = 5,  // multifrontal LU (sparse_lu.hpp), FP32 factors in FP64 refinement, FP64 fallback
  PATH_SPARSE64 = 6  // the same in FP64
};

struct Solver {
  bool ok = false;       // banded scheme applicable
  SparseDev* sparse = nullptr;  // multifrontal solver (built when the bands are too wide, or on request)
  int path = PATH_BLOCK;
  int wm = 0;            // row-band register window (32 or 64), 0 if the row-band kernels do not apply
  int n32 = 0, n64 = 0;  // components whose band fits a 32- / needs a 64-wide window (substitution)
  int32_t *list32 = nullptr, *list64 = nullptr;
  int nlu[4] = {0, 0, 0, 0};  // components by factorisation window: 32, 40, 48, 64
  int32_t* lulist[4] = {nullptr, nullptr, nullptr, nullptr};
  int nref = 8;          // refinement sweeps allowed on the FP32 path
  // row-band layout
  int64_t* rbase = nullptr;   // [ncomp] offset in RB / UC*
  int64_t* lbase = nullptr;   // [ncomp] offset in LM*
  int64_t* rbmap = nullptr;   // [nnz] position of each nnz in RB
  int64_t* rbmapT = nullptr;  // [nnz] position of each nnz in the rows of the transpose
  int wmT = 0;                // as wm, for the transpose (0 when its kl = ku exceeds 31)
  int64_t rb_total = 0, lb_total = 0;
  double* RB = nullptr;       // unfactorised rows (FP64)
  float* RB32 = nullptr;      // the same in FP32
  float* UC32 = nullptr;
  float* LM32 = nullptr;
  double* UC64 = nullptr;
  double* LM64 = nullptr;
  double* bw = nullptr;       // [nX] permuted right-hand side
  double* xw = nullptr;       // [nX] solution (band order)
  double* rw = nullptr;       // [nX] residual
  float* tw32 = nullptr;      // [nX] substitution work
  double* tw64 = nullptr;
  // partitioned (torn) layout of long components: interiors factorised in
  // parallel, separators coupled through a banded Schur complement
  int tearable = 0;           // some component is long enough to be cut
  int nint = 0, nsep = 0;
  int twmI = 0;               // register window of the interior kernels
  int bcr_levels = 0;         // cyclic-reduction levels of the longest separator chain
  int tmaxs = 0;              // largest max(kl, ku) over all components
  TornInt* d_ti = nullptr;    // [nint] interiors (bands of Lλx)
  TornInt* d_tiT = nullptr;   // [nint] the same with kl and ku exchanged (the transpose)
  TornSep* d_ts = nullptr;    // [nsep]
  int64_t *i_rbase = nullptr, *i_lbase = nullptr;
  int32_t *i_n = nullptr, *i_kl = nullptr, *i_ku = nullptr, *i_dof0 = nullptr;
  BcrSep* d_bsep = nullptr;   // [nsep] cyclic-reduction roles
  int64_t* d_brow = nullptr;  // [nsep] first row of each separator in the separator vectors
  int64_t tb_rows = 0, tb_blk = 0, tb_y = 0, tb_lm = 0, tb_tvec = 0;
  int64_t* tbmap = nullptr;   // [nnz] position in TALL = [interior rows | blocks]
  int64_t* tbmapT = nullptr;  // [nnz] the same for the transpose
  double *TALL = nullptr, *TUC = nullptr, *TLM = nullptr, *TY = nullptr;
  double *DLU = nullptr, *FA = nullptr, *WL = nullptr, *WU = nullptr;  // cyclic reduction (band_bcr.cuh)
  int* PV = nullptr;
  double *trhs = nullptr, *txs = nullptr;
  int32_t* tpiv = nullptr;
  // FP32 copies of the partitioned factorisation (refined in FP64)
  float *TALL32 = nullptr, *TUC32 = nullptr, *TLM32 = nullptr, *TY32 = nullptr;
  float *DLU32 = nullptr, *FA32 = nullptr, *WL32 = nullptr, *WU32 = nullptr;
  int32_t* i_comp = nullptr;                     // component of each interior
  int32_t *c_int0 = nullptr, *c_sep0 = nullptr;  // [ncomp+1] first interior / separator of each component
  int maxP = 0;                                  // most interiors in one component
  int fuseW32 = 0, fuseW64 = 0;                  // warps per block of the fused per-component solve, 0: off
  int* iflag = nullptr;                          // fallback flags per interior
  int* nbad = nullptr;                           // components whose FP32 refinement fell short
  int* info32 = nullptr;                         // zero pivots of the FP32 factorisation (caught by the check)
  double *dtmp = nullptr, *rtmp = nullptr;       // refinement correction and residual
  int64_t *rptr = nullptr, *rq = nullptr;        // rows of Lλx: CSC positions ...
  int32_t* rcol = nullptr;                       // ... and columns
  int64_t* dcolptr = nullptr;                    // the CSC pattern on the device
  int32_t* drowval = nullptr;
  int nrefine = 4;                               // FP64 refinement sweeps around the FP32 factors
  bool adaptive = false;                         // AUTO: leave the FP32 path after its first fallback
  int* flag = nullptr;        // [ncomp] FP64 fallback requested
  int* nsweep = nullptr;      // [ncomp] refinement sweeps used
  std::string why;       // reason when not
  int ncomp = 0;
  int64_t band_total = 0;
  int maxkl = 0, maxku = 0;
  // device
  int64_t* cbase = nullptr;   // [ncomp] offset of component band storage
  int32_t* cn = nullptr;      // [ncomp] component size
  int32_t* ckl = nullptr;     // [ncomp]
  int32_t* cku = nullptr;     // [ncomp]
  int32_t* cdof0 = nullptr;   // [ncomp] offset into perm
  int32_t* perm = nullptr;    // [nX] dofs of component c in band order: perm[cdof0[c] + k]
  int64_t* bmap = nullptr;    // [nnz] band position of each nnz
  double* AB = nullptr;       // band storage
  int32_t* ipiv = nullptr;    // [nX] pivot offsets (band order)
  double* rhs = nullptr;      // [nX] permuted right-hand side / solution
  double* rdiag = nullptr;    // [nX] reciprocal pivots (block kernels)
  double* dx = nullptr;       // [nX] Δx in model order
  double* red = nullptr;      // [4] reductions: ΣΔx², ΣLλ²
  double* part = nullptr;     // [2 * kNormBlocks] partial sums of the reductions
  int* info = nullptr;        // [kInfoSlots] first singular component+1 (0 = ok), one slot per iteration of a step
  int32_t* cod = nullptr;     // [nX] component of each dof
  int* frozen = nullptr;      // [ncomp] converged in this step (per-component convergence)
  int* nactive = nullptr;     // [1] components still iterating
  double* hbuf = nullptr;     // pinned host: red[0..1], info
};

// one Newton correction Δx = Lλx \ Lλ -> S.dx and its norms -> S.red; a
// singular factorisation writes component+1 to *info.  Capturable.
int factor_solve(mgpu_ctx* c, int* info);
// out = Lλxᵀ⁻¹ rhs (both in model order) from the Lλx assembled in ctx->nzval,
// with the FP64 row-band kernels; needs Solver::wmT.  Capturable.
int factor_solve_T(mgpu_ctx* c, const double* rhs, double* out, int* info);
// Newton loop of one SweepX step (src/SweepX.jl:190-224) on the resident
// state: uploads the step constants and load values, iterates to convergence
// (or fixed_iter times).  Errors carry the reference's messages.
int newton_step(mgpu_ctx* c, int OX, int64_t step, double t, double dt, const double* tvals_step,
                const mgpu_sweep_opts* opts, mgpu_stats* stats);
unsigned nb(int64_t n, int b);
mgpu_newmark newmark_coefficients(double beta, double gamma, double dt);

}  // namespace mgpu
