// Partitioned ("torn") banded solve for long components, FP64.
//
// A component of n dofs (reverse Cuthill-McKee order, bandwidths kl, ku) is
// cut into P interiors I_0..I_{P-1} and P-1 separators S_1..S_{P-1} of
// s = max(kl, ku) consecutive dofs:  I_0 S_1 I_1 S_2 ... S_{P-1} I_{P-1}.
// With bandwidth <= s no entry couples two interiors, so in the order
// (interiors, separators) the matrix is [A_I E; F D] with A_I block diagonal,
// and the separators carry the block-tridiagonal Schur complement
//     T = D - F A_I^-1 E,
//     T_kk     = D_k - F^R_{k-1} Y^R_{k-1} - F^L_k Y^L_k
//     T_k,k+1  = -F^L_k Y^R_k,         T_k+1,k = -F^R_k Y^L_k
// where Y^L_a = A_a^-1 E^L_a, Y^R_a = A_a^-1 E^R_a are the "spikes" of
// interior a (E^L_a = A[I_a, S_a] is nonzero in the first s rows of I_a only,
// E^R_a = A[I_a, S_{a+1}] in the last s rows, F^L_a = A[S_a, I_a] in the first
// s columns, F^R_a = A[S_{a+1}, I_a] in the last s columns).  A solve is
//     ỹ_a = A_a^-1 b_a,   r_k = b_S_k - F^R_{k-1} ỹ_{k-1} - F^L_k ỹ_k,
//     x_S = T^-1 r,       x_a = ỹ_a - Y^L_a x_S_a - Y^R_a x_S_{a+1}.
// The interiors are factorised by the row-band kernels (band_rows.cuh), all P
// of every component in parallel, and T by block cyclic reduction
// (band_bcr.cuh), log2(P) parallel levels; pivoting is partial within each
// interior and within each s x s block.  A chain of 30,000 dofs becomes
// hundreds of short independent chains and nine reduction levels.
//
// The blocks E, F, D are stored dense, s x s, row-major, each at its own
// offset (-1 when absent); Y^L_a, Y^R_a as m_a x s row-major.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "band_bcr.cuh"
#include "band_rows.cuh"

namespace mgpu {

// per interior: where its data lives
struct TornInt {
  int64_t rbase, lbase;  // row-band storage and multipliers (as RbComp)
  int32_t n, kl, ku;     // size and bands of the interior
  int32_t dof0;          // offset of its dofs in perm
  int32_t s;             // separator width of its component
  int64_t eL, eR, fL, fR;  // offsets of E^L, E^R, F^L, F^R in the block array, -1 if absent
  int64_t yL, yR;          // offsets of Y^L, Y^R (m x s), -1 if absent
  int32_t sepL, sepR;      // global index of the left / right separator, -1 if absent
  int32_t comp;            // connected component it belongs to
};

// per separator
struct TornSep {
  int32_t s;
  int32_t dof0;     // offset of its dofs in perm
  int64_t d;        // offset of D in the block array
  int32_t intL, intR;  // interiors on its left / right
  int64_t trow;     // first row of this separator in the separator vector
  int32_t first;    // 1 when this is the first separator of its component
  int32_t last;     // 1 when it is the last
  int32_t comp;     // connected component it belongs to
};

// only[comp] == 0 skips the component (FP64 fallback after an FP32 factorisation);
// only == nullptr runs all
__device__ __forceinline__ bool tb_skip(const int* only, int comp) { return only && only[comp] == 0; }

// ---------------------------------------------------------------- spikes
// One warp per interior with at least one separator.  Lane r < s computes
// column r of Y^L (right-hand side: column r of E^L), lane s <= r < 2s column
// r-s of Y^R.  Each lane keeps its own column's window in registers: kl+1
// entries for the forward substitution (L with the interchanges), kv+1 for
// the backward one (U).  L, U and the pivots stream through shared memory in
// chunks of 32 columns.  FP64: kl + kv FMA instructions per row, one lane per
// right-hand side.  KLW >= kl+1 sizes the forward window (16 or 32), WM >= kv+1
// the backward one.
template <typename T, int WM, int KLW>
__global__ void __launch_bounds__(32) tb_spikes(int nint, const TornInt* __restrict__ ti,
                                                const T* __restrict__ UC, const T* __restrict__ LM,
                                                const int32_t* __restrict__ ipiv, const T* __restrict__ blk,
                                                T* __restrict__ Y, const int* __restrict__ only) {
  __shared__ __align__(16) T sU[32 * WM];
  __shared__ __align__(16) T sL[32 * 31];
  __shared__ __align__(16) T sYin[32 * 33];  // backward: the chunk's incoming rows, one column per lane
  __shared__ int sP[32];
  const int a = blockIdx.x, lane = threadIdx.x;
  if (a >= nint) return;
  const TornInt I = ti[a];
  if (I.sepL < 0 && I.sepR < 0) return;
  if (tb_skip(only, I.comp)) return;
  const int m = I.n, kl = I.kl, kv = I.kl + I.ku, w = kv + 1, s = I.s;
  const T* U = UC + I.rbase;
  const T* L = LM + I.lbase;
  const int32_t* piv = ipiv + I.dof0;
  const bool isL = lane < s, isR = lane >= s && lane < 2 * s;
  const bool act = (isL && I.sepL >= 0) || (isR && I.sepR >= 0);
  const int col = isL ? lane : lane - s;
  // right-hand side entry of this lane's column at row i
  auto rhs = [&](int i) -> T {
    if (!act || i < 0 || i >= m) return T(0);
    if (isL) return i < s ? blk[I.eL + int64_t(i) * s + col] : T(0);
    const int r = i - (m - s);
    return r >= 0 ? blk[I.eR + int64_t(r) * s + col] : T(0);
  };
  T* Yout = Y + (isL ? I.yL : I.yR);  // only dereferenced when act
  // ---- forward: window rows k..k+kl
  T yw[KLW];
#pragma unroll
  for (int p = 0; p < KLW; ++p) yw[p] = (p <= kl) ? rhs(p) : T(0);
  const int nch = (m + 31) >> 5;
  for (int c = 0; c < nch; ++c) {
    const int k0 = c * 32, k1 = min(m, k0 + 32);
    __syncwarp();
    for (int e = lane; e < (k1 - k0) * kl; e += 32) sL[e] = L[int64_t(k0) * kl + e];
    if (lane < k1 - k0) sP[lane] = piv[k0 + lane] - (k0 + lane);
    __syncwarp();
    for (int k = k0; k < k1; ++k) {
      const int km = min(kl, m - 1 - k);
      const int jp = sP[k - k0];
      if (jp != 0) {
        T v = yw[0];
#pragma unroll
        for (int p = 1; p < KLW; ++p) v = (p == jp) ? yw[p] : v;
        const T y0 = yw[0];
        yw[0] = v;
#pragma unroll
        for (int p = 1; p < KLW; ++p) yw[p] = (p == jp) ? y0 : yw[p];
      }
      const T yk = yw[0];
      if (act) Yout[int64_t(k) * s + col] = yk;
      const T* lk = sL + (k - k0) * kl;
#pragma unroll
      for (int p = 1; p < KLW; ++p) {
        if (p > km) break;  // uniform
        yw[p] = fma(-lk[p - 1], yk, yw[p]);
      }
      const T nx = rhs(k + 1 + kl);
#pragma unroll
      for (int p = 0; p < KLW - 1; ++p) yw[p] = (p < kl) ? yw[p + 1] : yw[p];
#pragma unroll
      for (int p = 0; p < KLW; ++p)
        if (p == kl) yw[p] = nx;
    }
  }
  __syncwarp();
  // ---- backward: window rows k-kv..k (zw[p] holds row k-p)
  T zw[WM];
#pragma unroll
  for (int p = 0; p < WM; ++p) {
    const int i = m - 1 - p;
    zw[p] = (act && p <= kv && i >= 0) ? Yout[int64_t(i) * s + col] : T(0);
  }
  for (int c = nch - 1; c >= 0; --c) {
    const int k0 = c * 32, k1 = min(m, k0 + 32);
    __syncwarp();
    for (int e = lane; e < (k1 - k0) * w; e += 32) sU[e] = U[int64_t(k0) * w + e];
    // rows k-1-kv entering the window during this chunk (forward results, this lane's column):
    // read once per chunk instead of one dependent global load per row
#pragma unroll 4
    for (int q = 0; q < 32; ++q) {
      const int i = k0 + q - 1 - kv;
      sYin[q * 33 + lane] = (act && i >= 0 && q < k1 - k0) ? Yout[int64_t(i) * s + col] : T(0);
    }
    __syncwarp();
    for (int k = k1 - 1; k >= k0; --k) {
      const T* uk = sU + (k - k0) * w;
      const T xk = zw[0] * uk[0];  // 1/U(k,k)
      if (act) Yout[int64_t(k) * s + col] = xk;
      const int pm = min(kv, k);
#pragma unroll
      for (int p = 1; p < WM; ++p) {
        if (p > pm) break;  // uniform
        zw[p] = fma(-uk[p], xk, zw[p]);
      }
      const T nx = sYin[(k - k0) * 33 + lane];
#pragma unroll
      for (int p = 0; p < WM - 1; ++p) zw[p] = (p < kv) ? zw[p + 1] : zw[p];
#pragma unroll
      for (int p = 0; p < WM; ++p)
        if (p == kv) zw[p] = nx;
    }
  }
}

// ---------------------------------------------------------------- Schur complement
// One warp per separator k: its blocks of T (D_k = T_kk, U_k = T_k,k+1 and
// L_k+1 = T_k+1,k) into level 0 of the block cyclic reduction storage
// (band_bcr.cuh: [level][separator][D, L, U][16 x 16]).
template <typename T>
__global__ void __launch_bounds__(32) tb_schur(int nsep, const TornSep* __restrict__ ts,
                                               const TornInt* __restrict__ ti, const T* __restrict__ blk,
                                               const T* __restrict__ Y, T* __restrict__ DLU,
                                               const int* __restrict__ only) {
  const int k = blockIdx.x, lane = threadIdx.x;
  if (k >= nsep) return;
  const TornSep S = ts[k];
  if (tb_skip(only, S.comp)) return;
  const int s = S.s;
  const TornInt IL = ti[S.intL], IR = ti[S.intR];
  T* Dk = DLU + 3 * int64_t(k) * BCR_SS;
  T* Uk = Dk + 2 * BCR_SS;
  T* Lk1 = DLU + (3 * int64_t(k + 1) + 1) * BCR_SS;  // L of the next separator (only when !S.last)
  for (int e = lane; e < s * s; e += 32) {
    const int i = e / s, j = e % s;
    // T_kk = D - F^R_{left} Y^R_{left}[last s rows] - F^L_{right} Y^L_{right}[first s rows]
    const T* FR = blk + IL.fR;
    const T* YR = Y + IL.yR + int64_t(IL.n - s) * s;
    const T* FL = blk + IR.fL;
    const T* YL = Y + IR.yL;
    T a1 = T(0), a2 = T(0);
    for (int q = 0; q < s; ++q) {
      a1 = fma(FR[i * s + q], YR[q * s + j], a1);
      a2 = fma(FL[i * s + q], YL[q * s + j], a2);
    }
    Dk[i * BCR_S + j] = blk[S.d + e] - a1 - a2;
    if (!S.last) {
      // T_k,k+1 = -F^L_{right} Y^R_{right}[first s rows];  T_k+1,k = -F^R_{right} Y^L_{right}[last s rows]
      const T* YRr = Y + IR.yR;
      const T* FRr = blk + IR.fR;
      const T* YLr = Y + IR.yL + int64_t(IR.n - s) * s;
      T b1 = T(0), b2 = T(0);
      for (int q = 0; q < s; ++q) {
        b1 = fma(FL[i * s + q], YRr[q * s + j], b1);
        b2 = fma(FRr[i * s + q], YLr[q * s + j], b2);
      }
      Uk[i * BCR_S + j] = -b1;
      Lk1[i * BCR_S + j] = -b2;
    }
  }
}

// ---------------------------------------------------------------- solve
// separator right-hand sides: r = b_S - F^R_{left} ỹ_{left}[last s] - F^L_{right} ỹ_{right}[first s]
// (b and ỹ in model order; ỹ of the interiors is already in x); arithmetic in
// the factors' type, stored in FP64.  One warp; yl, yr: s entries of scratch.
template <typename T>
__device__ void tb_sep_rhs_warp(const TornSep& S, const TornInt* __restrict__ ti, const T* __restrict__ blk,
                                const int32_t* __restrict__ perm, const double* b, const double* x, double* tr,
                                T* yl, T* yr, int lane) {
  const int s = S.s;
  const TornInt IL = ti[S.intL], IR = ti[S.intR];
  if (lane < s) {
    yl[lane] = T(x[perm[IL.dof0 + IL.n - s + lane]]);
    yr[lane] = T(x[perm[IR.dof0 + lane]]);
  }
  __syncwarp();
  if (lane < s) {
    T v = T(b[perm[S.dof0 + lane]]);
    for (int q = 0; q < s; ++q) {
      v -= blk[IL.fR + lane * s + q] * yl[q];
      v -= blk[IR.fL + lane * s + q] * yr[q];
    }
    tr[S.trow + lane] = double(v);
  }
  __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(32) tb_sep_rhs(int nsep, const TornSep* __restrict__ ts,
                                                 const TornInt* __restrict__ ti, const T* __restrict__ blk,
                                                 const int32_t* __restrict__ perm, const double* __restrict__ b,
                                                 const double* __restrict__ x, double* __restrict__ tr,
                                                 const int* __restrict__ only) {
  __shared__ T yl[BCR_S], yr[BCR_S];
  const int k = blockIdx.x;
  if (k >= nsep) return;
  const TornSep S = ts[k];
  if (tb_skip(only, S.comp)) return;
  tb_sep_rhs_warp(S, ti, blk, perm, b, x, tr, yl, yr, threadIdx.x);
}

// x_a -= Y^L_a x_S_a + Y^R_a x_S_a+1 (interior dofs), x_S = T solution (separator dofs);
// arithmetic in the factors' type (with FP32 factors this is a refinement
// correction).  One warp; xl, xr: s entries of scratch.
template <typename T>
__device__ void tb_back_warp(const TornInt& I, const TornSep* __restrict__ ts, const T* __restrict__ Y,
                             const int32_t* __restrict__ perm, const double* txs, double* x, T* xl, T* xr,
                             int lane) {
  const int s = I.s;
  const bool hl = I.sepL >= 0, hr = I.sepR >= 0;
  if (!(hl || hr)) return;
  if (lane < s) {
    xl[lane] = hl ? T(txs[ts[I.sepL].trow + lane]) : T(0);
    xr[lane] = hr ? T(txs[ts[I.sepR].trow + lane]) : T(0);
  }
  __syncwarp();
  for (int i = lane; i < I.n; i += 32) {
    T v = T(x[perm[I.dof0 + i]]);
    for (int q = 0; q < s; ++q) {
      if (hl) v -= Y[I.yL + int64_t(i) * s + q] * xl[q];
      if (hr) v -= Y[I.yR + int64_t(i) * s + q] * xr[q];
    }
    x[perm[I.dof0 + i]] = double(v);
  }
  if (hr) {
    const TornSep S = ts[I.sepR];
    if (lane < s) x[perm[S.dof0 + lane]] = txs[S.trow + lane];
  }
  __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(32) tb_back(int nint, const TornInt* __restrict__ ti,
                                              const TornSep* __restrict__ ts, const T* __restrict__ Y,
                                              const int32_t* __restrict__ perm, const double* __restrict__ txs,
                                              double* __restrict__ x, const int* __restrict__ only) {
  __shared__ T xl[BCR_S], xr[BCR_S];
  const int a = blockIdx.x;
  if (a >= nint) return;
  const TornInt I = ti[a];
  if (tb_skip(only, I.comp)) return;
  tb_back_warp(I, ts, Y, perm, txs, x, xl, xr, threadIdx.x);
}

// ---------------------------------------------------------------- fused per-component solve
// Everything of one solve of one component in one block, for layouts whose
// components have few interiors (many components, e.g. independent risers):
// W warps take the component's interiors and separators in turn, and the
// cyclic-reduction levels, the back-substitution and (with nref > 1) the
// sweeps of FP64 iterative refinement follow one another behind block
// barriers instead of kernel boundaries.  All vectors stay in the band order
// of the factorisation (contiguous per interior and separator); the
// right-hand side is gathered from model order once and the result scattered
// back once.
//   b = P rhs
//   sweep: t = A~^-1 r  (interiors, separator right-hand sides, cyclic
//          reduction, back-substitution; r = b on the first sweep)
//          x += t (x = t on the first sweep); stop when max|t| <= tol_stop max|x|
//          r = b - A x (FP64, from the unfactorised interior rows and the
//          E, F, D blocks)
//   out = P^T x
// At the end flag[c] = 1 unless max|t| <= tol_ok max|x| and all finite (for
// the FP64 fallback), nsweep[c] = sweeps.  With nref = 1 it is a plain
// solve.  only[c] == 0 skips the component.
struct TbFusedArgs {
  int ncomp;
  const int32_t* cint0;  // [ncomp+1] first interior of each component
  const int32_t* csep0;  // [ncomp+1] first separator of each component
  RbComp cpI;            // interiors as row-band components (bands exchanged for the transpose)
  const TornInt* ti;
  const TornSep* ts;
  const BcrSep* bs;
  int nsep;
  const int32_t* perm;
  const int32_t* tpiv;
  const int64_t* brow;
  const double* tall;    // unfactorised interior rows, then the blocks at tall + tb_rows (FP64)
  int64_t tb_rows;
  double* bw;    // [nX] band-order right-hand side
  double* xw;    // [nX] band-order solution
  double* rw;    // [nX] band-order residual
  double* trhs;  // separator vectors
  double* txs;
  const double* rhs;  // model order
  double* out;        // model order
  const int32_t* ccn;    // [ncomp] component sizes
  const int32_t* ccdof0; // [ncomp] component offsets in perm
  int nref;
  double tol_stop, tol_ok;
  const int* only;
  int* flag;
  int* nsweep;
  int* nbad;  // incremented per flagged component
};

template <typename T>
struct TbFusedFactors {
  const T *UC, *LM, *blk, *Y, *FA, *DLU, *WL, *WU;
  const int* PV;
  T* tw;  // [nX] band-order correction
};

template <typename T, int WM>
__host__ __device__ constexpr int tb_fused_warp_bytes() {
  return ((RbSmem<T, WM>::bytes > int(sizeof(BcrWarp<T>)) ? RbSmem<T, WM>::bytes : int(sizeof(BcrWarp<T>))) + 15) /
         16 * 16;
}

// separator right-hand side in band order: r_S = b_S - F^R_{left} t_{left}[last s] - F^L_{right} t_{right}[first s]
template <typename T>
__device__ void tb_sep_rhs_band(const TornSep& S, const TornInt* __restrict__ ti, const T* __restrict__ blk,
                                const double* b, const T* t, double* tr, int lane) {
  const int s = S.s;
  if (lane < s) {
    const TornInt IL = ti[S.intL], IR = ti[S.intR];
    const T* yl = t + IL.dof0 + IL.n - s;
    const T* yr = t + IR.dof0;
    T v = T(b[S.dof0 + lane]);
    for (int q = 0; q < s; ++q) {
      v -= blk[IL.fR + lane * s + q] * yl[q];
      v -= blk[IR.fL + lane * s + q] * yr[q];
    }
    tr[S.trow + lane] = double(v);
  }
}

// back-substitution in band order: t_a -= Y^L_a x_S_a + Y^R_a x_S_a+1, t_S = x_S.
// One warp; the rows of Y go through shared memory 32 at a time (contiguous
// loads), each lane then takes one row.  sc: scratch of 2*32*16 + 32 T.
template <typename T>
__device__ void tb_back_band(const TornInt& I, const TornSep* __restrict__ ts, const T* __restrict__ Y,
                             const double* txs, T* t, T* sc, int lane) {
  const int s = I.s;
  const bool hl = I.sepL >= 0, hr = I.sepR >= 0;
  if (!(hl || hr)) return;
  T* yl = sc;
  T* yr = sc + 32 * BCR_S;
  T* xl = sc + 64 * BCR_S;
  T* xr = xl + BCR_S;
  if (lane < s) {
    xl[lane] = hl ? T(txs[ts[I.sepL].trow + lane]) : T(0);
    xr[lane] = hr ? T(txs[ts[I.sepR].trow + lane]) : T(0);
  }
#pragma unroll 1
  for (int i0 = 0; i0 < I.n; i0 += 32) {
    const int m = min(32, I.n - i0);
    __syncwarp();
    if (hl)
      for (int e = lane; e < m * s; e += 32) yl[e] = Y[I.yL + int64_t(i0) * s + e];
    if (hr)
      for (int e = lane; e < m * s; e += 32) yr[e] = Y[I.yR + int64_t(i0) * s + e];
    __syncwarp();
    if (lane < m) {
      T v = t[I.dof0 + i0 + lane];
      for (int q = 0; q < s; ++q) {
        if (hl) v -= yl[lane * s + q] * xl[q];
        if (hr) v -= yr[lane * s + q] * xr[q];
      }
      t[I.dof0 + i0 + lane] = v;
    }
  }
  if (hr && lane < s) t[ts[I.sepR].dof0 + lane] = xr[lane];
  __syncwarp();
}

// v - sum_{j < s} a[j] b[j] (s <= 16), ascending j; the loads issued 8 at a time
__device__ __forceinline__ double tb_dot16_sub(const double* a, const double* b, int s, double v) {
#pragma unroll
  for (int jb = 0; jb < 16; jb += 8) {
    if (jb >= s) break;
    double av[8], bv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool ok = jb + u < s;
      av[u] = ok ? a[jb + u] : 0.0;
      bv[u] = ok ? b[jb + u] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (jb + u < s) v = fma(-av[u], bv[u], v);
  }
  return v;
}

// threads per block of the fused solve at most (13 warps): two blocks per SM fit
// in the register file at <= 78 registers per thread
constexpr int kTbFusedMaxThreads = 416;

template <typename T, int WM>
__global__ void __launch_bounds__(kTbFusedMaxThreads, 2) tb_fused(TbFusedArgs A, TbFusedFactors<T> F) {
  extern __shared__ __align__(16) unsigned char tb_dyn[];
  __shared__ double red[2][32];
  __shared__ int fin[32];
  const int cc = blockIdx.x;
  if (cc >= A.ncomp) return;
  if (A.only && A.only[cc] == 0) return;
  const int W = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* my = tb_dyn + size_t(w) * tb_fused_warp_bytes<T, WM>();
  BcrWarp<T>* sw = reinterpret_cast<BcrWarp<T>*>(my);
  const int a0 = A.cint0[cc], a1 = A.cint0[cc + 1], k0 = A.csep0[cc], k1 = A.csep0[cc + 1];
  const int nc = A.ccn[cc];
  const int64_t q0 = A.ccdof0[cc];
  const int32_t* pm = A.perm + q0;
  const int nlev = k1 > k0 ? A.bs[k0].nlev : 0;
  const double* blk64 = A.tall + A.tb_rows;
  T* t = F.tw;
  for (int k = threadIdx.x; k < nc; k += blockDim.x) A.bw[q0 + k] = A.rhs[pm[k]];
  __syncthreads();
  const double* in = A.bw;
  double dn = 0.0, xn = 0.0;
  bool finite = true;
  int sweeps = 0;
  for (int it = 0; it < A.nref; ++it) {
    // interiors: t = A_a^-1 in
    for (int a = a0 + w; a < a1; a += W) {
      const int n = A.cpI.cn[a], kl = A.cpI.ckl[a], kv = kl + A.cpI.cku[a];
      const int64_t d0 = A.cpI.cdof0[a];
      rb_fb<T, WM>(n, kl, kv, kv + 1, F.UC + A.cpI.rbase[a], F.LM + A.cpI.lbase[a], A.tpiv + d0, in + d0, t + d0,
                   my, lane);
      __syncwarp();
    }
    __syncthreads();
    if (k1 > k0) {
      for (int k = k0 + w; k < k1; k += W) tb_sep_rhs_band(A.ts[k], A.ti, F.blk, in, t, A.trhs, lane);
      __syncthreads();
      for (int l = 0; l < nlev; ++l) {
        for (int k = k0 + w; k < k1; k += W) {
          const BcrSep B = A.bs[k];
          if (bcr_role(B.kloc, B.N, l) == 1) bcr_diag_solve_warp(B, k, F.FA, F.PV, A.brow, A.trhs, A.txs, sw, lane);
        }
        __syncthreads();
        for (int k = k0 + w; k < k1; k += W) {
          const BcrSep B = A.bs[k];
          if (bcr_role(B.kloc, B.N, l) == 2) bcr_keep_warp(B, k, l, A.nsep, F.DLU, A.brow, A.trhs, A.txs, sw, lane);
        }
        __syncthreads();
      }
      if (w == 0) bcr_diag_solve_warp(A.bs[k0], k0, F.FA, F.PV, A.brow, A.trhs, A.txs, sw, lane);
      __syncthreads();
      for (int l = nlev - 1; l >= 0; --l) {
        for (int k = k0 + w; k < k1; k += W) {
          const BcrSep B = A.bs[k];
          if (bcr_role(B.kloc, B.N, l) == 1) bcr_back_warp(B, k, l, F.WL, F.WU, A.brow, A.txs, sw, lane);
        }
        __syncthreads();
      }
      for (int a = a0 + w; a < a1; a += W) tb_back_band(A.ti[a], A.ts, F.Y, A.txs, t, reinterpret_cast<T*>(my), lane);
      __syncthreads();
    }
    ++sweeps;
    if (A.nref == 1) break;
    // x += t and the max norms
    dn = 0.0;
    xn = 0.0;
    for (int k = threadIdx.x; k < nc; k += blockDim.x) {
      const int64_t q = q0 + k;
      const double dv = double(t[q]);
      const double xv = it == 0 ? dv : A.xw[q] + dv;
      A.xw[q] = xv;
      finite = finite && isfinite(dv) && isfinite(xv);
      dn = fmax(dn, fabs(dv));
      xn = fmax(xn, fabs(xv));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dn = fmax(dn, __shfl_xor_sync(0xffffffffu, dn, o));
      xn = fmax(xn, __shfl_xor_sync(0xffffffffu, xn, o));
    }
    const bool wfin = __all_sync(0xffffffffu, finite);
    if (lane == 0) {
      red[0][w] = dn;
      red[1][w] = xn;
      fin[w] = wfin;
    }
    __syncthreads();
    dn = 0.0;
    xn = 0.0;
    finite = true;
    for (int q = 0; q < W; ++q) {
      dn = fmax(dn, red[0][q]);
      xn = fmax(xn, red[1][q]);
      finite = finite && fin[q];
    }
    __syncthreads();  // red / fin are rewritten by the next sweep
    if (it + 1 == A.nref || !finite || dn <= A.tol_stop * xn) break;
    // r = b - A x: interior rows (band storage and the E blocks), separator rows
    // (F and D blocks).  The band rows go through the warp's shared scratch 32
    // rows at a time (contiguous loads), each lane then sums one row in
    // ascending column order; its x entries are consecutive across lanes.
    for (int a = a0 + w; a < a1; a += W) {
      const TornInt I = A.ti[a];
      const int n = I.n, kl = I.kl, kv = I.kl + I.ku, wd = kv + 1, s = I.s;
      const double* rows = A.tall + I.rbase;
      const double* xl = I.sepL >= 0 ? A.xw + A.ts[I.sepL].dof0 : nullptr;
      const double* xr = I.sepR >= 0 ? A.xw + A.ts[I.sepR].dof0 : nullptr;
      double* sm = reinterpret_cast<double*>(my);
#pragma unroll 1
      for (int i0 = 0; i0 < n; i0 += 32) {
        const int m = min(32, n - i0);
        __syncwarp();
        for (int e = lane; e < m * wd; e += 32) sm[e] = rows[int64_t(i0) * wd + e];
        __syncwarp();
        if (lane < m) {
          const int i = i0 + lane;
          const int64_t q = I.dof0 + i;
          double v = A.bw[q];
          const int c0 = max(0, kl - i), c1 = min(kv, n - 1 - i + kl);
          const double* row = sm + lane * wd;
          const double* xx = A.xw + q - kl;
#pragma unroll 1
          for (int cb = 0; cb <= c1; cb += 8) {
            double xv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int c = cb + u;
              xv[u] = (c >= c0 && c <= c1) ? xx[c] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
              if (cb + u >= c0 && cb + u <= c1) v = fma(-row[cb + u], xv[u], v);
          }
          if (xl && i < s) v = tb_dot16_sub(blk64 + I.eL + int64_t(i) * s, xl, s, v);
          if (xr && i >= n - s) v = tb_dot16_sub(blk64 + I.eR + int64_t(i - (n - s)) * s, xr, s, v);
          A.rw[q] = v;
        }
      }
    }
#pragma unroll 1
    for (int k = k0 + w; k < k1; k += W) {
      const TornSep S = A.ts[k];
      const int s = S.s;
      if (lane < s) {
        const TornInt IL = A.ti[S.intL], IR = A.ti[S.intR];
        const int64_t q = S.dof0 + lane;
        double v = A.bw[q];
        v = tb_dot16_sub(blk64 + IL.fR + lane * s, A.xw + IL.dof0 + IL.n - s, s, v);
        v = tb_dot16_sub(blk64 + S.d + lane * s, A.xw + S.dof0, s, v);
        v = tb_dot16_sub(blk64 + IR.fL + lane * s, A.xw + IR.dof0, s, v);
        A.rw[q] = v;
      }
    }
    __syncthreads();
    in = A.rw;
  }
  if (A.nref == 1) {
    for (int k = threadIdx.x; k < nc; k += blockDim.x) A.out[pm[k]] = double(t[q0 + k]);
  } else {
    for (int k = threadIdx.x; k < nc; k += blockDim.x) A.out[pm[k]] = A.xw[q0 + k];
    if (threadIdx.x == 0) {
      const int bad = !(finite && dn <= A.tol_ok * xn);
      if (A.flag) A.flag[cc] = bad;
      if (A.nbad && bad) atomicAdd(A.nbad, 1);
      if (A.nsweep) A.nsweep[cc] = sweeps;
    }
  }
}

// per-virtual-component flags (interiors, Schur components) from per-component ones
static __global__ void tb_expand_flags(int n, const int32_t* __restrict__ comp_of, const int* __restrict__ cflag,
                                int* __restrict__ vflag) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) vflag[v] = cflag[comp_of[v]];
}

// r = b - A x, FP64, one thread per row; A given by columns (CSC) with a row
// index (rptr, rq = CSC position, rc = column) for A x, or used as is for Aᵀ x
static __global__ void tb_residual(int64_t n, int transposed, const int64_t* __restrict__ rptr,
                            const int64_t* __restrict__ rq, const int32_t* __restrict__ rc,
                            const int64_t* __restrict__ colptr, const int32_t* __restrict__ rowval,
                            const double* __restrict__ nz, const double* __restrict__ b,
                            const double* __restrict__ x, double* __restrict__ r) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = b[i];
  if (transposed)
    for (int64_t q = colptr[i]; q < colptr[i + 1]; ++q) s = fma(-nz[q], x[rowval[q]], s);
  else
    for (int64_t q = rptr[i]; q < rptr[i + 1]; ++q) s = fma(-nz[rq[q]], x[rc[q]], s);
  r[i] = s;
}

static __global__ void tb_axpy(int64_t n, const double* __restrict__ d, double* __restrict__ x) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] += d[i];
}

// refinement check per component: flag[c] = 1 unless max|d| <= 1e-10 max|x| (NaN fails);
// *nbad counts the flagged components
static __global__ void __launch_bounds__(32) tb_ir_check(const int32_t* __restrict__ cn, const int32_t* __restrict__ cdof0,
                                                  const int32_t* __restrict__ perm, const double* __restrict__ d,
                                                  const double* __restrict__ x, int* __restrict__ flag,
                                                  int* __restrict__ nbad) {
  const int c = blockIdx.x, lane = threadIdx.x;
  const int n = cn[c];
  const int32_t* pm = perm + cdof0[c];
  double dn = 0.0, xn = 0.0;
  bool finite = true;
  for (int k = lane; k < n; k += 32) {
    const double dv = d[pm[k]], xv = x[pm[k]];
    finite = finite && isfinite(dv) && isfinite(xv);
    dn = fmax(dn, fabs(dv));
    xn = fmax(xn, fabs(xv));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dn = fmax(dn, __shfl_xor_sync(0xffffffffu, dn, o));
    xn = fmax(xn, __shfl_xor_sync(0xffffffffu, xn, o));
  }
  finite = __all_sync(0xffffffffu, finite);
  if (lane == 0) {
    const int bad = !(finite && dn <= 1e-10 * xn);
    flag[c] = bad;
    if (bad) atomicAdd(nbad, 1);
  }
}

}  // namespace mgpu
