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
// (b and ỹ in model order; ỹ of the interiors is already in x)
template <typename T>
__global__ void tb_sep_rhs(int nsep, const TornSep* __restrict__ ts, const TornInt* __restrict__ ti,
                           const T* __restrict__ blk, const int32_t* __restrict__ perm,
                           const double* __restrict__ b, const double* __restrict__ x, double* __restrict__ tr,
                           const int* __restrict__ only) {
  const int k = blockIdx.x, lane = threadIdx.x;
  if (k >= nsep) return;
  const TornSep S = ts[k];
  if (tb_skip(only, S.comp)) return;
  const int s = S.s;
  const TornInt IL = ti[S.intL], IR = ti[S.intR];
  for (int i = lane; i < s; i += 32) {
    double v = b[perm[S.dof0 + i]];
    for (int q = 0; q < s; ++q) {
      v -= double(blk[IL.fR + i * s + q]) * x[perm[IL.dof0 + IL.n - s + q]];
      v -= double(blk[IR.fL + i * s + q]) * x[perm[IR.dof0 + q]];
    }
    tr[S.trow + i] = v;
  }
}

// x_a -= Y^L_a x_S_a + Y^R_a x_S_a+1 (interior dofs), x_S = T solution (separator dofs)
template <typename T>
__global__ void tb_back(int nint, const TornInt* __restrict__ ti, const TornSep* __restrict__ ts,
                        const T* __restrict__ Y, const int32_t* __restrict__ perm,
                        const double* __restrict__ txs, double* __restrict__ x, const int* __restrict__ only) {
  const int a = blockIdx.x;
  if (a >= nint) return;
  const TornInt I = ti[a];
  if (tb_skip(only, I.comp)) return;
  const int s = I.s;
  const double* xl = I.sepL >= 0 ? txs + ts[I.sepL].trow : nullptr;
  const double* xr = I.sepR >= 0 ? txs + ts[I.sepR].trow : nullptr;
  if (xl || xr)
    for (int i = threadIdx.x; i < I.n; i += blockDim.x) {
      double v = x[perm[I.dof0 + i]];
      for (int q = 0; q < s; ++q) {
        if (xl) v -= double(Y[I.yL + int64_t(i) * s + q]) * xl[q];
        if (xr) v -= double(Y[I.yR + int64_t(i) * s + q]) * xr[q];
      }
      x[perm[I.dof0 + i]] = v;
    }
  if (I.sepR >= 0) {
    const TornSep S = ts[I.sepR];
    for (int i = threadIdx.x; i < s; i += blockDim.x) x[perm[S.dof0 + i]] = txs[S.trow + i];
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
