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
// The interiors and T are factorised by the row-band kernels (band_rows.cuh)
// with partial pivoting inside each block; the P interiors of every component
// run in parallel, which is the point: a chain of 30,000 dofs becomes ~50
// independent chains and one band of ~50 s.
//
// The blocks E, F, D are stored dense, s x s, row-major, each at its own
// offset (-1 when absent); Y^L_a, Y^R_a as m_a x s row-major.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

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
};

// per separator
struct TornSep {
  int32_t s;
  int32_t dof0;     // offset of its dofs in perm
  int64_t d;        // offset of D in the block array
  int32_t intL, intR;  // interiors on its left / right
  int64_t trow;     // first row of this separator in the T vector
  int64_t tbase;    // row-band storage offset of the T component holding it
  int32_t tkl, tw;  // bands of that T component: kl = ku = 2s-1, w = 4s-1
  int64_t trow0;    // first row of that T component in the T vector
  int32_t first;    // 1 when this is the first separator of its component
  int32_t last;     // 1 when it is the last
};

// ---------------------------------------------------------------- spikes
// One warp per interior with at least one separator.  Lane r < s computes
// column r of Y^L (right-hand side: column r of E^L), lane s <= r < 2s column
// r-s of Y^R.  Each lane keeps its own column's window in registers: kl+1
// entries for the forward substitution (L with the interchanges), kv+1 for
// the backward one (U).  L, U and the pivots stream through shared memory in
// chunks of 32 columns.  FP64: kl + kv FMA instructions per row, one lane per
// right-hand side.  KLW >= kl+1 sizes the forward window (16 or 32), WM >= kv+1
// the backward one.
template <int WM, int KLW>
__global__ void __launch_bounds__(32) tb_spikes(int nint, const TornInt* __restrict__ ti,
                                                const double* __restrict__ UC, const double* __restrict__ LM,
                                                const int32_t* __restrict__ ipiv, const double* __restrict__ blk,
                                                double* __restrict__ Y) {
  __shared__ __align__(16) double sU[32 * WM];
  __shared__ __align__(16) double sL[32 * 31];
  __shared__ __align__(16) double sYin[32 * 33];  // backward: the chunk's incoming rows, one column per lane
  __shared__ int sP[32];
  const int a = blockIdx.x, lane = threadIdx.x;
  if (a >= nint) return;
  const TornInt I = ti[a];
  if (I.sepL < 0 && I.sepR < 0) return;
  const int m = I.n, kl = I.kl, kv = I.kl + I.ku, w = kv + 1, s = I.s;
  const double* U = UC + I.rbase;
  const double* L = LM + I.lbase;
  const int32_t* piv = ipiv + I.dof0;
  const bool isL = lane < s, isR = lane >= s && lane < 2 * s;
  const bool act = (isL && I.sepL >= 0) || (isR && I.sepR >= 0);
  const int col = isL ? lane : lane - s;
  // right-hand side entry of this lane's column at row i
  auto rhs = [&](int i) -> double {
    if (!act || i < 0 || i >= m) return 0.0;
    if (isL) return i < s ? blk[I.eL + int64_t(i) * s + col] : 0.0;
    const int r = i - (m - s);
    return r >= 0 ? blk[I.eR + int64_t(r) * s + col] : 0.0;
  };
  double* Yout = Y + (isL ? I.yL : I.yR);  // only dereferenced when act
  // ---- forward: window rows k..k+kl
  double yw[KLW];
#pragma unroll
  for (int p = 0; p < KLW; ++p) yw[p] = (p <= kl) ? rhs(p) : 0.0;
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
        double v = yw[0];
#pragma unroll
        for (int p = 1; p < KLW; ++p) v = (p == jp) ? yw[p] : v;
        const double y0 = yw[0];
        yw[0] = v;
#pragma unroll
        for (int p = 1; p < KLW; ++p) yw[p] = (p == jp) ? y0 : yw[p];
      }
      const double yk = yw[0];
      if (act) Yout[int64_t(k) * s + col] = yk;
      const double* lk = sL + (k - k0) * kl;
#pragma unroll
      for (int p = 1; p < KLW; ++p)
        if (p <= km) yw[p] = fma(-lk[p - 1], yk, yw[p]);
      const double nx = rhs(k + 1 + kl);
#pragma unroll
      for (int p = 0; p < KLW - 1; ++p) yw[p] = (p < kl) ? yw[p + 1] : yw[p];
#pragma unroll
      for (int p = 0; p < KLW; ++p)
        if (p == kl) yw[p] = nx;
    }
  }
  __syncwarp();
  // ---- backward: window rows k-kv..k (zw[p] holds row k-p)
  double zw[WM];
#pragma unroll
  for (int p = 0; p < WM; ++p) {
    const int i = m - 1 - p;
    zw[p] = (act && p <= kv && i >= 0) ? Yout[int64_t(i) * s + col] : 0.0;
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
      sYin[q * 33 + lane] = (act && i >= 0 && q < k1 - k0) ? Yout[int64_t(i) * s + col] : 0.0;
    }
    __syncwarp();
    for (int k = k1 - 1; k >= k0; --k) {
      const double* uk = sU + (k - k0) * w;
      const double xk = zw[0] * uk[0];  // 1/U(k,k)
      if (act) Yout[int64_t(k) * s + col] = xk;
      const int pm = min(kv, k);
#pragma unroll
      for (int p = 1; p < WM; ++p)
        if (p <= pm) zw[p] = fma(-uk[p], xk, zw[p]);
      const double nx = sYin[(k - k0) * 33 + lane];
#pragma unroll
      for (int p = 0; p < WM - 1; ++p) zw[p] = (p < kv) ? zw[p + 1] : zw[p];
#pragma unroll
      for (int p = 0; p < WM; ++p)
        if (p == kv) zw[p] = nx;
    }
  }
}

// ---------------------------------------------------------------- Schur complement
// One warp per separator k: its block row of T (T_kk, T_k,k+1, T_k+1,k) into
// the row-band storage of its T component (kl = ku = 2s-1).
static __global__ void __launch_bounds__(32) tb_schur(int nsep, const TornSep* __restrict__ ts,
                                               const TornInt* __restrict__ ti, const double* __restrict__ blk,
                                               const double* __restrict__ Y, double* __restrict__ TR) {
  const int k = blockIdx.x, lane = threadIdx.x;
  if (k >= nsep) return;
  const TornSep S = ts[k];
  const int s = S.s;
  const TornInt IL = ti[S.intL], IR = ti[S.intR];
  const int64_t r0 = S.trow - S.trow0;  // first row of this separator in its T component
  auto put = [&](int64_t i, int64_t j, double v) { TR[S.tbase + i * S.tw + (j - i + S.tkl)] = v; };
  for (int e = lane; e < s * s; e += 32) {
    const int i = e / s, j = e % s;
    // T_kk = D - F^R_{left} Y^R_{left}[last s rows] - F^L_{right} Y^L_{right}[first s rows]
    double v = blk[S.d + e];
    const double* FR = blk + IL.fR;
    const double* YR = Y + IL.yR + int64_t(IL.n - s) * s;
    const double* FL = blk + IR.fL;
    const double* YL = Y + IR.yL;
    double a1 = 0.0, a2 = 0.0;
    for (int q = 0; q < s; ++q) {
      a1 = fma(FR[i * s + q], YR[q * s + j], a1);
      a2 = fma(FL[i * s + q], YL[q * s + j], a2);
    }
    put(r0 + i, r0 + j, v - a1 - a2);
    if (!S.last) {
      // T_k,k+1 = -F^L_{right} Y^R_{right}[first s rows];  T_k+1,k = -F^R_{right} Y^L_{right}[last s rows]
      const double* YRr = Y + IR.yR;
      const double* FRr = blk + IR.fR;
      const double* YLr = Y + IR.yL + int64_t(IR.n - s) * s;
      double b1 = 0.0, b2 = 0.0;
      for (int q = 0; q < s; ++q) {
        b1 = fma(FL[i * s + q], YRr[q * s + j], b1);
        b2 = fma(FRr[i * s + q], YLr[q * s + j], b2);
      }
      put(r0 + i, r0 + s + j, -b1);
      put(r0 + s + i, r0 + j, -b2);
    }
  }
}

// ---------------------------------------------------------------- solve
// separator right-hand sides: r = b_S - F^R_{left} ỹ_{left}[last s] - F^L_{right} ỹ_{right}[first s]
// (b and ỹ in model order; ỹ of the interiors is already in x)
static __global__ void tb_sep_rhs(int nsep, const TornSep* __restrict__ ts, const TornInt* __restrict__ ti,
                           const double* __restrict__ blk, const int32_t* __restrict__ perm,
                           const double* __restrict__ b, const double* __restrict__ x, double* __restrict__ tr) {
  const int k = blockIdx.x, lane = threadIdx.x;
  if (k >= nsep) return;
  const TornSep S = ts[k];
  const int s = S.s;
  const TornInt IL = ti[S.intL], IR = ti[S.intR];
  for (int i = lane; i < s; i += 32) {
    double v = b[perm[S.dof0 + i]];
    for (int q = 0; q < s; ++q) {
      v -= blk[IL.fR + i * s + q] * x[perm[IL.dof0 + IL.n - s + q]];
      v -= blk[IR.fL + i * s + q] * x[perm[IR.dof0 + q]];
    }
    tr[S.trow + i] = v;
  }
}

// x_a -= Y^L_a x_S_a + Y^R_a x_S_a+1 (interior dofs), x_S = T solution (separator dofs)
static __global__ void tb_back(int nint, const TornInt* __restrict__ ti, const TornSep* __restrict__ ts,
                        const double* __restrict__ Y, const int32_t* __restrict__ perm,
                        const double* __restrict__ txs, double* __restrict__ x) {
  const int a = blockIdx.x;
  if (a >= nint) return;
  const TornInt I = ti[a];
  const int s = I.s;
  const double* xl = I.sepL >= 0 ? txs + ts[I.sepL].trow : nullptr;
  const double* xr = I.sepR >= 0 ? txs + ts[I.sepR].trow : nullptr;
  if (xl || xr)
    for (int i = threadIdx.x; i < I.n; i += blockDim.x) {
      double v = x[perm[I.dof0 + i]];
      for (int q = 0; q < s; ++q) {
        if (xl) v -= Y[I.yL + int64_t(i) * s + q] * xl[q];
        if (xr) v -= Y[I.yR + int64_t(i) * s + q] * xr[q];
      }
      x[perm[I.dof0 + i]] = v;
    }
  if (I.sepR >= 0) {
    const TornSep S = ts[I.sepR];
    for (int i = threadIdx.x; i < s; i += blockDim.x) x[perm[S.dof0 + i]] = txs[S.trow + i];
  }
}

}  // namespace mgpu
