// Block cyclic reduction of the separators' Schur complement (band_torn.cuh).
//
// Per component the Schur complement is block tridiagonal with N = P-1 blocks
// of s x s:  L_k x_{k-1} + D_k x_k + U_k x_{k+1} = r_k  (L_0 = U_{N-1} = 0).
// Level l (stride h = 2^l) eliminates the active blocks k with (k/h) odd:
//     W_L(k) = D_k^-1 L_k,  W_U(k) = D_k^-1 U_k   (LU of D_k, partial pivoting)
// and the kept blocks e (k/h even) take
//     D_e' = D_e - U_e W_L(e+h) - L_e W_U(e-h),
//     U_e' = -U_e W_U(e+h),   L_e' = -L_e W_L(e-h)
// until block 0 alone remains.  A solve reduces the right-hand side the same
// way (z_k = D_k^-1 r_k, r_e -= U_e z_{e+h} + L_e z_{e-h}), solves block 0 and
// substitutes back level by level (x_k = z_k - W_L(k) x_{k-h} - W_U(k) x_{k+h}).
// The factorisation runs one launch per level over all blocks of all
// components (one warp per block, dense s x s work), so the separators cost
// log2(N) levels instead of a sequential band factorisation of N s rows.  A
// solve either does the same, level by level, or (components of few
// interiors) runs inside the fused per-component solve of band_torn.cuh, one
// block barrier per level.
//
// Storage (per separator k, global index; component offset sep0, local index
// k - sep0; SS = 16 x 16 doubles per block whatever s):
//   DLU[lvl][k] D, L, U of level lvl     FA[k]: LU factors of D at elimination, pivots PV[k]
//   WL[k], WU[k]: D^-1 L and D^-1 U      rhs / z / x: vectors of N s entries per component
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace mgpu {

constexpr int BCR_S = 16;                 // largest block
constexpr int BCR_SS = BCR_S * BCR_S;     // doubles per stored block

struct BcrSep {
  int32_t comp;     // component
  int32_t kloc;     // local block index 0..N-1
  int32_t N;        // blocks of its component
  int32_t s;        // block size
  int32_t sep0;     // global index of block 0 of its component
  int32_t nlev;     // levels of its component: ceil(log2 N)
};

// role of block kloc at level l: 0 inactive, 1 eliminated, 2 kept
__device__ __forceinline__ int bcr_role(int kloc, int N, int l) {
  const int h = 1 << l;
  if (kloc % h != 0 || kloc >= N) return 0;
  return ((kloc / h) & 1) ? 1 : 2;
}

// dense helpers, one warp; A row-major s x s with leading dimension BCR_S
template <typename T>
__device__ void bcr_lu(T* A, int* piv, int s, int lane, int* singular) {
  for (int j = 0; j < s; ++j) {
    // pivot: first largest |A[i][j]|, i >= j
    T best = T(-1);
    int bi = j;
    for (int i = j; i < s; ++i) {
      const T v = fabs(A[i * BCR_S + j]);
      if (v > best) best = v, bi = i;
    }
    if (lane == 0) piv[j] = bi;
    if (bi != j)
      for (int c = lane; c < s; c += 32) {
        const T t = A[j * BCR_S + c];
        A[j * BCR_S + c] = A[bi * BCR_S + c];
        A[bi * BCR_S + c] = t;
      }
    __syncwarp();
    const T p = A[j * BCR_S + j];
    if (p == T(0)) {
      if (lane == 0) *singular = 1;
      continue;
    }
    const T rp = T(1) / p;
    for (int i = j + 1 + lane; i < s; i += 32) A[i * BCR_S + j] *= rp;
    __syncwarp();
    const int m = s - j - 1;
    for (int e = lane; e < m * m; e += 32) {
      const int i = j + 1 + e / m, c = j + 1 + e % m;
      A[i * BCR_S + c] = fma(-A[i * BCR_S + j], A[j * BCR_S + c], A[i * BCR_S + c]);
    }
    __syncwarp();
  }
}

// B (s x nrhs, row-major, ld BCR_S) <- (LU)^-1 P B; lanes over right-hand sides
template <typename T>
__device__ void bcr_lu_solve(const T* F, const int* piv, T* B, int s, int nrhs, int lane) {
  for (int r = lane; r < nrhs; r += 32) {
    for (int j = 0; j < s; ++j)
      if (piv[j] != j) {
        const T t = B[j * BCR_S + r];
        B[j * BCR_S + r] = B[piv[j] * BCR_S + r];
        B[piv[j] * BCR_S + r] = t;
      }
    for (int i = 1; i < s; ++i) {
      T v = B[i * BCR_S + r];
      for (int j = 0; j < i; ++j) v = fma(-F[i * BCR_S + j], B[j * BCR_S + r], v);
      B[i * BCR_S + r] = v;
    }
    for (int i = s - 1; i >= 0; --i) {
      T v = B[i * BCR_S + r];
      for (int j = i + 1; j < s; ++j) v = fma(-F[i * BCR_S + j], B[j * BCR_S + r], v);
      B[i * BCR_S + r] = v / F[i * BCR_S + i];
    }
  }
  __syncwarp();
}

// C (+)= alpha * A B, s x s, lanes over entries of C
template <typename T>
__device__ void bcr_gemm(const T* A, const T* B, T* C, int s, T alpha, bool accumulate, int lane) {
  for (int e = lane; e < s * s; e += 32) {
    const int i = e / s, j = e % s;
    T v = T(0);
    for (int q = 0; q < s; ++q) v = fma(A[i * BCR_S + q], B[q * BCR_S + j], v);
    C[i * BCR_S + j] = accumulate ? fma(alpha, v, C[i * BCR_S + j]) : alpha * v;
  }
  __syncwarp();
}

// level l, eliminated blocks: factor D_k, W_L = D^-1 L, W_U = D^-1 U
template <typename T>
__global__ void __launch_bounds__(32) bcr_eliminate(int nsep, const BcrSep* __restrict__ bs, int l,
                                                    const T* __restrict__ DLU, T* __restrict__ FA,
                                                    int* __restrict__ PV, T* __restrict__ WL, T* __restrict__ WU,
                                                    const int* __restrict__ only, int* __restrict__ info) {
  __shared__ T sA[BCR_SS];
  __shared__ T sB[BCR_S * BCR_S * 2];
  __shared__ int sp[BCR_S];
  __shared__ int sing;
  const int k = blockIdx.x, lane = threadIdx.x;
  if (k >= nsep) return;
  const BcrSep B = bs[k];
  if (only && only[B.comp] == 0) return;
  const int role = l < B.nlev ? bcr_role(B.kloc, B.N, l) : 0;
  if (role != 1) return;
  const int s = B.s, h = 1 << l;
  const int64_t lvl = int64_t(l) * nsep * 3;
  const T* D = DLU + (lvl + 3 * int64_t(k)) * BCR_SS;
  for (int e = lane; e < BCR_SS; e += 32) sA[e] = D[e];
  // right-hand sides [L | U] side by side in sB (row-major, ld BCR_S, columns 0..s-1 L, the next s U)
  const bool hasU = B.kloc + h < B.N;
  for (int e = lane; e < s * s; e += 32) {
    const int i = e / s, j = e % s;
    sB[i * BCR_S + j] = D[BCR_SS + i * BCR_S + j];  // L
  }
  if (lane == 0) sing = 0;
  __syncwarp();
  bcr_lu(sA, sp, s, lane, &sing);
  bcr_lu_solve(sA, sp, sB, s, s, lane);
  T* wl = WL + int64_t(k) * BCR_SS;
  for (int e = lane; e < BCR_SS; e += 32) wl[e] = sB[e];
  __syncwarp();
  T* wu = WU + int64_t(k) * BCR_SS;
  if (hasU) {
    for (int e = lane; e < s * s; e += 32) {
      const int i = e / s, j = e % s;
      sB[i * BCR_S + j] = D[2 * BCR_SS + i * BCR_S + j];  // U
    }
    __syncwarp();
    bcr_lu_solve(sA, sp, sB, s, s, lane);
    for (int e = lane; e < BCR_SS; e += 32) wu[e] = sB[e];
  } else {
    for (int e = lane; e < BCR_SS; e += 32) wu[e] = T(0);
  }
  T* fa = FA + int64_t(k) * BCR_SS;
  for (int e = lane; e < BCR_SS; e += 32) fa[e] = sA[e];
  if (lane < s) PV[int64_t(k) * BCR_S + lane] = sp[lane];
  if (lane == 0 && sing && info) atomicCAS(info, 0, B.comp + 1);
}

// level l, kept blocks: D, L, U of level l+1
template <typename T>
__global__ void __launch_bounds__(32) bcr_update(int nsep, const BcrSep* __restrict__ bs, int l, T* __restrict__ DLU,
                                                 const T* __restrict__ WL, const T* __restrict__ WU,
                                                 const int* __restrict__ only) {
  __shared__ T sD[BCR_SS], sL[BCR_SS], sU[BCR_SS];
  const int k = blockIdx.x, lane = threadIdx.x;
  if (k >= nsep) return;
  const BcrSep B = bs[k];
  if (only && only[B.comp] == 0) return;
  const int role = l < B.nlev ? bcr_role(B.kloc, B.N, l) : 0;
  if (role != 2) return;
  const int s = B.s, h = 1 << l;
  const T* cur = DLU + (int64_t(l) * nsep * 3 + 3 * int64_t(k)) * BCR_SS;
  T* nxt = DLU + (int64_t(l + 1) * nsep * 3 + 3 * int64_t(k)) * BCR_SS;
  for (int e = lane; e < BCR_SS; e += 32) {
    sD[e] = cur[e];
    sL[e] = cur[BCR_SS + e];
    sU[e] = cur[2 * BCR_SS + e];
  }
  __syncwarp();
  const bool up = B.kloc + h < B.N, dn = B.kloc >= h;
  const int64_t kup = k + h, kdn = k - h;
  // D' = D - U W_L(k+h) - L W_U(k-h)
  if (up) bcr_gemm(sU, WL + kup * BCR_SS, sD, s, T(-1), true, lane);
  if (dn) bcr_gemm(sL, WU + kdn * BCR_SS, sD, s, T(-1), true, lane);
  for (int e = lane; e < BCR_SS; e += 32) nxt[e] = sD[e];
  __syncwarp();  // sD is reused as scratch below, with another lane-to-entry assignment
  // U' = -U W_U(k+h), L' = -L W_L(k-h)
  T* nU = nxt + 2 * BCR_SS;
  T* nL = nxt + BCR_SS;
  if (up) {
    bcr_gemm(sU, WU + kup * BCR_SS, sD, s, T(-1), false, lane);  // sD reused as scratch
    for (int e = lane; e < BCR_SS; e += 32) nU[e] = sD[e];
    __syncwarp();
  } else {
    for (int e = lane; e < BCR_SS; e += 32) nU[e] = T(0);
  }
  __syncwarp();
  if (dn) {
    bcr_gemm(sL, WL + kdn * BCR_SS, sD, s, T(-1), false, lane);
    for (int e = lane; e < BCR_SS; e += 32) nL[e] = sD[e];
  } else {
    for (int e = lane; e < BCR_SS; e += 32) nL[e] = T(0);
  }
}

// the last block (kloc = 0) of every component: LU of its final D
template <typename T>
__global__ void __launch_bounds__(32) bcr_root(int nsep, const BcrSep* __restrict__ bs, const T* __restrict__ DLU,
                                               T* __restrict__ FA, int* __restrict__ PV, const int* __restrict__ only,
                                               int* __restrict__ info) {
  __shared__ T sA[BCR_SS];
  __shared__ int sp[BCR_S];
  __shared__ int sing;
  const int k = blockIdx.x, lane = threadIdx.x;
  if (k >= nsep) return;
  const BcrSep B = bs[k];
  if (B.kloc != 0 || (only && only[B.comp] == 0)) return;
  const T* D = DLU + (int64_t(B.nlev) * nsep * 3 + 3 * int64_t(k)) * BCR_SS;
  for (int e = lane; e < BCR_SS; e += 32) sA[e] = D[e];
  if (lane == 0) sing = 0;
  __syncwarp();
  bcr_lu(sA, sp, B.s, lane, &sing);
  T* fa = FA + int64_t(k) * BCR_SS;
  for (int e = lane; e < BCR_SS; e += 32) fa[e] = sA[e];
  if (lane < B.s) PV[int64_t(k) * BCR_S + lane] = sp[lane];
  if (lane == 0 && sing && info) atomicCAS(info, 0, B.comp + 1);
}

// ---- solve: r (FP64, per separator s entries at row0[k]) -> x, stored in FP64
// and computed in the factors' type (with FP32 factors the solve is a
// refinement correction).  One warp per block; the per-block steps are device
// functions shared by the level-by-level kernels below and by the fused
// per-component solve (band_torn.cuh).

// shared scratch of one warp
template <typename T>
struct BcrWarp {
  T A[BCR_SS];
  T B[BCR_SS];
  T v[BCR_S];
  T w[BCR_S];
  int p[BCR_S];
};

// v <- (LU)^-1 P v for one block: F and v in shared memory, the triangular
// sweeps lane-parallel over rows (one column step per warp-synchronous step)
template <typename T>
__device__ void bcr_block_solve(const T* F, const int* piv, T* v, int s, int lane) {
  if (lane == 0)
    for (int j = 0; j < s; ++j)
      if (piv[j] != j) {
        const T t = v[j];
        v[j] = v[piv[j]];
        v[piv[j]] = t;
      }
  __syncwarp();
  for (int j = 0; j < s; ++j) {  // unit lower
    if (lane > j && lane < s) v[lane] = fma(-F[lane * BCR_S + j], v[j], v[lane]);
    __syncwarp();
  }
  for (int j = s - 1; j >= 0; --j) {  // upper
    if (lane == j) v[j] /= F[j * BCR_S + j];
    __syncwarp();
    if (lane < j) v[lane] = fma(-F[lane * BCR_S + j], v[j], v[lane]);
    __syncwarp();
  }
}

template <typename T>
__device__ void bcr_stage(T* dst, const T* src, int lane) {
  for (int e = lane; e < BCR_SS; e += 32) dst[e] = src[e];
}

// z_k = D_k^-1 r_k with the factors FA[k] (an eliminated block at its level, or the root)
template <typename T>
__device__ void bcr_diag_solve_warp(const BcrSep& B, int k, const T* __restrict__ FA, const int* __restrict__ PV,
                                    const int64_t* __restrict__ row0, const double* r, double* z,
                                    BcrWarp<T>* sw, int lane) {
  const int s = B.s;
  const int64_t o = row0[k];
  bcr_stage(sw->A, FA + int64_t(k) * BCR_SS, lane);
  if (lane < s) {
    sw->v[lane] = T(r[o + lane]);
    sw->p[lane] = PV[int64_t(k) * BCR_S + lane];
  }
  __syncwarp();
  bcr_block_solve(sw->A, sw->p, sw->v, s, lane);
  if (lane < s) z[o + lane] = double(sw->v[lane]);
  __syncwarp();
}

// kept block e at level l: r_e -= U_e z_{e+h} + L_e z_{e-h}
template <typename T>
__device__ void bcr_keep_warp(const BcrSep& B, int k, int l, int nsep, const T* __restrict__ DLU,
                              const int64_t* __restrict__ row0, double* r, const double* z, BcrWarp<T>* sw,
                              int lane) {
  const int s = B.s, h = 1 << l;
  const T* cur = DLU + (int64_t(l) * nsep * 3 + 3 * int64_t(k)) * BCR_SS;
  const bool up = B.kloc + h < B.N, dn = B.kloc >= h;
  if (up) bcr_stage(sw->B, cur + 2 * BCR_SS, lane);
  if (dn) bcr_stage(sw->A, cur + BCR_SS, lane);
  if (lane < s) {
    sw->v[lane] = up ? T(z[row0[k + h] + lane]) : T(0);
    sw->w[lane] = dn ? T(z[row0[k - h] + lane]) : T(0);
  }
  __syncwarp();
  if (lane < s) {
    const int64_t o = row0[k];
    T v = T(r[o + lane]);
    for (int q = 0; q < s; ++q) {
      if (up) v = fma(-sw->B[lane * BCR_S + q], sw->v[q], v);
      if (dn) v = fma(-sw->A[lane * BCR_S + q], sw->w[q], v);
    }
    r[o + lane] = double(v);
  }
  __syncwarp();
}

// eliminated block k at level l: x_k = z_k - W_L(k) x_{k-h} - W_U(k) x_{k+h}  (z holds z_k and the kept x)
template <typename T>
__device__ void bcr_back_warp(const BcrSep& B, int k, int l, const T* __restrict__ WL, const T* __restrict__ WU,
                              const int64_t* __restrict__ row0, double* z, BcrWarp<T>* sw, int lane) {
  const int s = B.s, h = 1 << l;
  const bool up = B.kloc + h < B.N;
  const int64_t o = row0[k];
  bcr_stage(sw->A, WL + int64_t(k) * BCR_SS, lane);
  if (up) bcr_stage(sw->B, WU + int64_t(k) * BCR_SS, lane);
  if (lane < s) {
    sw->w[lane] = T(z[row0[k - h] + lane]);
    sw->v[lane] = up ? T(z[row0[k + h] + lane]) : T(0);
  }
  __syncwarp();
  if (lane < s) {
    T a = T(z[o + lane]);
    for (int q = 0; q < s; ++q) {
      a = fma(-sw->A[lane * BCR_S + q], sw->w[q], a);
      if (up) a = fma(-sw->B[lane * BCR_S + q], sw->v[q], a);
    }
    z[o + lane] = double(a);
  }
  __syncwarp();
}

// level-by-level kernels: one warp per separator of every component
// forward, level l: eliminated z_k = D_k^-1 r_k
template <typename T>
__global__ void __launch_bounds__(32) bcr_fwd_elim(int nsep, const BcrSep* __restrict__ bs, int l,
                                                   const T* __restrict__ FA, const int* __restrict__ PV,
                                                   const int64_t* __restrict__ row0, const double* __restrict__ r,
                                                   double* __restrict__ z, const int* __restrict__ only) {
  __shared__ BcrWarp<T> sw;
  const int k = blockIdx.x;
  if (k >= nsep) return;
  const BcrSep B = bs[k];
  if (only && only[B.comp] == 0) return;
  if (!(l < B.nlev && bcr_role(B.kloc, B.N, l) == 1)) return;
  bcr_diag_solve_warp(B, k, FA, PV, row0, r, z, &sw, threadIdx.x);
}

// forward, level l: kept r_e -= U_e z_{e+h} + L_e z_{e-h}
template <typename T>
__global__ void __launch_bounds__(32) bcr_fwd_keep(int nsep, const BcrSep* __restrict__ bs, int l,
                                                   const T* __restrict__ DLU, const int64_t* __restrict__ row0,
                                                   double* __restrict__ r, const double* __restrict__ z,
                                                   const int* __restrict__ only) {
  __shared__ BcrWarp<T> sw;
  const int k = blockIdx.x;
  if (k >= nsep) return;
  const BcrSep B = bs[k];
  if (only && only[B.comp] == 0) return;
  if (!(l < B.nlev && bcr_role(B.kloc, B.N, l) == 2)) return;
  bcr_keep_warp(B, k, l, nsep, DLU, row0, r, z, &sw, threadIdx.x);
}

// root: x_0 = D_0^-1 r_0 (into z, which then holds x for every block as the back-substitution proceeds)
template <typename T>
__global__ void __launch_bounds__(32) bcr_root_solve(int nsep, const BcrSep* __restrict__ bs,
                                                     const T* __restrict__ FA, const int* __restrict__ PV,
                                                     const int64_t* __restrict__ row0, const double* __restrict__ r,
                                                     double* __restrict__ z, const int* __restrict__ only) {
  __shared__ BcrWarp<T> sw;
  const int k = blockIdx.x;
  if (k >= nsep) return;
  const BcrSep B = bs[k];
  if (B.kloc != 0 || (only && only[B.comp] == 0)) return;
  bcr_diag_solve_warp(B, k, FA, PV, row0, r, z, &sw, threadIdx.x);
}

// backward, level l
template <typename T>
__global__ void __launch_bounds__(32) bcr_back(int nsep, const BcrSep* __restrict__ bs, int l,
                                               const T* __restrict__ WL, const T* __restrict__ WU,
                                               const int64_t* __restrict__ row0, double* __restrict__ z,
                                               const int* __restrict__ only) {
  __shared__ BcrWarp<T> sw;
  const int k = blockIdx.x;
  if (k >= nsep) return;
  const BcrSep B = bs[k];
  if (only && only[B.comp] == 0) return;
  if (!(l < B.nlev && bcr_role(B.kloc, B.N, l) == 1)) return;
  bcr_back_warp(B, k, l, WL, WU, row0, z, &sw, threadIdx.x);
}

}  // namespace mgpu
