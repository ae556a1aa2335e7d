// Device sparse direct solver: multifrontal LU over nested-dissection fronts
// (see sparse_lu.hpp and sparse_analysis.hpp).
#include "sparse_lu.hpp"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "ctx.hpp"
#include "sparse_analysis.hpp"
#include "tc.cuh"

namespace mgpu {
namespace {

constexpr int kThreads = 256;
constexpr int kNB32 = 64;  // pivot block of the FP32 factorisation
constexpr int kNB64 = 32;  // of the FP64 factorisation (register rows of the L panel)
constexpr int kTile = 64;  // trailing-update tile
constexpr int kMaxGridY = 65535;

// device-scope loads and stores of flags written by other blocks
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr size_t kUpd32Smem = size_t(2) * 64 * (128 + 4) * sizeof(float);  // sp_update_f32<64> tiles
constexpr double kRefineTol = 1e-14;   // scaled correction / scaled solution: converged
constexpr double kRefineStall = 1e-10;  // ... or stalled below this

inline unsigned nblocks(int64_t n, int b) { return unsigned((n + b - 1) / b); }

// ---------------------------------------------------------------- equilibration
__global__ void sp_scale_diag(int64_t n, const int32_t* __restrict__ diag, const double* __restrict__ nzval,
                              double* __restrict__ D0) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t q = diag[i];
  const double a = q >= 0 ? fabs(nzval[q]) : 0.0;
  D0[i] = a > 0.0 ? 1.0 / sqrt(a) : 0.0;
}

// a dof without a diagonal value (a constraint multiplier): the scale that makes
// its largest column entry one, from the scales of the dofs it couples to
__global__ void sp_scale_zero(int64_t n, const int64_t* __restrict__ colptr, const int32_t* __restrict__ rowval,
                              const double* __restrict__ nzval, const double* __restrict__ D0,
                              double* __restrict__ D) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = D0[i];
  if (d == 0.0) {
    double mx = 0.0;
    for (int64_t q = colptr[i]; q < colptr[i + 1]; ++q) mx = fmax(mx, fabs(nzval[q]) * D0[rowval[q]]);
    d = mx > 0.0 ? 1.0 / mx : 1.0;
  }
  D[i] = d;
}

// ---------------------------------------------------------------- assembly of the fronts
template <class T>
__global__ void sp_assemble(int64_t cnt, const int32_t* __restrict__ aq, const int64_t* __restrict__ amap,
                            const int32_t* __restrict__ rowval, const int32_t* __restrict__ acol,
                            const double* __restrict__ nzval, const double* __restrict__ D, T* __restrict__ F) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int32_t q = aq[t];
  F[amap[q]] = T(nzval[q] * D[rowval[q]] * D[acol[q]]);
}

// extend-add of one child per parent (the children of rank r): the child's
// trailing Schur complement into its parent's front; a warp adds two columns
template <class T>
__global__ void __launch_bounds__(kThreads) sp_extend_add(const SpFrontDev* __restrict__ fr,
                                                          const int32_t* __restrict__ list,
                                                          const int32_t* __restrict__ emap, T* __restrict__ F) {
  const SpFrontDev C = fr[list[blockIdx.y]];
  const SpFrontDev P = fr[C.parent];
  const int uc = C.m - C.p;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int32_t* em = emap + C.eoff;
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
    const int k = blockIdx.x * 16 + w * 2 + kk;
    if (k >= uc) break;
    const T* src = F + C.off + int64_t(C.p + k) * C.m + C.p;
    T* dst = F + P.off + int64_t(em[k]) * P.m;
    for (int l = lane; l < uc; l += 32) dst[em[l]] += src[l];
  }
}

// Stage the kb × kb block at (k0, k0) of a column-major front (leading
// dimension m) into Dg, 8 loads per thread in flight before their stores (a
// load-then-store loop would wait for each load in turn).
template <class T, int NB>
__device__ __forceinline__ void stage_diag_block(const T* __restrict__ A, int m, int k0, int kb, T (*Dg)[NB + 1]) {
  const int n = kb * kb, nt = int(blockDim.x);
  for (int t0 = int(threadIdx.x); t0 < n; t0 += 8 * nt) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + u * nt;
      v[u] = t < n ? A[(k0 + t % kb) + int64_t(k0 + t / kb) * m] : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + u * nt;
      if (t < n) Dg[t % kb][t / kb] = v[u];
    }
  }
}

// ---------------------------------------------------------------- partial LU of the fronts
// The kb × kb diagonal block of pivot block k0, loaded from the front and
// factored in shared memory (no row exchanges; a pivot below tau in magnitude
// is set to ±tau, counted when `count`; a zero pivot with tau = 0 or a
// non-finite one sets flags[3]).  Every block that needs it computes it the same
// way, so the panel kernel reads the block unchanged and the update kernel
// writes it back.
template <class T, int NB>
__device__ void factor_diag(const T* A, int m, int k0, int kb, T (*Dg)[NB + 1], T tau, int* flags, bool count) {
  const int tid = threadIdx.x;
  stage_diag_block<T, NB>(A, m, k0, kb, Dg);
  __syncthreads();
  for (int k = 0; k < kb; ++k) {
    if (tid == 0) {
      const T d = Dg[k][k];
      if (!isfinite(d) || (d == T(0) && tau == T(0))) {
        if (count) atomicOr(flags + 3, 1);
      } else if (fabs(d) < tau) {
        Dg[k][k] = d < T(0) ? -tau : tau;
        if (count) atomicAdd(flags + 2, 1);
      }
    }
    __syncthreads();
    const T piv = Dg[k][k];
    for (int i = k + 1 + tid; i < kb; i += int(blockDim.x)) Dg[i][k] /= piv;
    __syncthreads();
    const int r = kb - k - 1;
    for (int t = tid; t < r * r; t += int(blockDim.x)) {
      const int i = k + 1 + t % r, j = k + 1 + t / r;
      Dg[i][j] -= Dg[i][k] * Dg[k][j];
    }
    __syncthreads();
  }
}

// Pivot block k0 .. k0+kb-1 of every listed front: each block factors the
// diagonal block (factor_diag), then solves either 256 rows of the L panel
// (x U₁₁ = a) or 64 columns of the U panel (L₁₁ y = a).  The diagonal block
// itself is left as it was (other blocks of the launch read it) and written
// by the update kernel.
template <class T, int NB>
__global__ void __launch_bounds__(kThreads) sp_panel(const SpFrontDev* __restrict__ fr,
                                                     const int32_t* __restrict__ flist, int k0, T* __restrict__ F,
                                                     T tau, int* __restrict__ flags) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  if (k0 >= p) return;
  const int kb = min(NB, p - k0);
  const int r0 = k0 + kb, rest = m - r0;
  const int nrc = (rest + kThreads - 1) / kThreads, ncc = (rest + 63) / 64;
  if (int(blockIdx.x) >= nrc + ncc) return;
  T* A = F + Fr.off;
  __shared__ T Dg[NB][NB + 1];
  const int tid = threadIdx.x;
  factor_diag<T, NB>(A, m, k0, kb, Dg, tau, flags, false);
  const int b = blockIdx.x;
  if (b < nrc) {
    const int i = r0 + b * kThreads + tid;
    if (i < m) {
      T x[NB];
#pragma unroll
      for (int c = 0; c < NB; ++c) x[c] = c < kb ? A[i + int64_t(k0 + c) * m] : T(0);
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        if (c < kb) {
          x[c] /= Dg[c][c];
#pragma unroll
          for (int t = c + 1; t < NB; ++t)
            if (t < kb) x[t] -= x[c] * Dg[c][t];
        }
      }
#pragma unroll
      for (int c = 0; c < NB; ++c)
        if (c < kb) A[i + int64_t(k0 + c) * m] = x[c];
    }
  } else if (b < nrc + ncc) {
    const int w = tid >> 5, lane = tid & 31;
    for (int jj = 0; jj < 8; ++jj) {
      const int j = r0 + (b - nrc) * 64 + w * 8 + jj;
      if (j >= m) break;
      T* col = A + int64_t(j) * m + k0;
      T y0 = lane < kb ? col[lane] : T(0);
      T y1 = (NB > 32 && lane + 32 < kb) ? col[lane + 32] : T(0);
      for (int c = 0; c < kb; ++c) {
        const T yc = __shfl_sync(0xffffffffu, c < 32 ? y0 : y1, c & 31);
        if (lane > c && lane < kb) y0 -= Dg[lane][c] * yc;
        if (NB > 32 && lane + 32 > c && lane + 32 < kb) y1 -= Dg[(lane + 32) % NB][c] * yc;
      }
      if (lane < kb) col[lane] = y0;
      if (NB > 32 && lane + 32 < kb) col[lane + 32] = y1;
    }
  }
}

// The same panels once the diagonal block has been factored in place
// (sp_diag_store), so that no block repeats its factorisation: blocks
// [0, nrc) solve 256 rows of the L panel (one row per thread), blocks
// [nrc, nrc + ncc) 64 columns of the U panel, a warp taking eight columns at
// once (lanes over rows) so that eight substitution chains interleave.
template <class T, int NB>
__global__ void __launch_bounds__(kThreads) sp_panel_f(const SpFrontDev* __restrict__ fr,
                                                       const int32_t* __restrict__ flist, int k0,
                                                       T* __restrict__ F) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  if (k0 >= p) return;
  const int kb = min(NB, p - k0);
  const int r0 = k0 + kb, rest = m - r0;
  const int nrc = (rest + kThreads - 1) / kThreads, ncc = (rest + 63) / 64;
  if (int(blockIdx.x) >= nrc + ncc) return;
  T* A = F + Fr.off;
  __shared__ T Dg[NB][NB + 1];
  __shared__ T rdg[NB];  // reciprocal pivots: no division on the rows' substitution chains
  const int tid = threadIdx.x;
  stage_diag_block<T, NB>(A, m, k0, kb, Dg);
  if (tid < kb) rdg[tid] = T(1) / A[(k0 + tid) + int64_t(k0 + tid) * m];
  __syncthreads();
  const int b = blockIdx.x;
  if (b < nrc) {
    // one row per thread, x U₁₁ = a; for NB = 64 in two halves of 32 columns
    // (the second half first takes the first half's products, in the same
    // order as a single pass), so that 32 values, not 64, are live
    const int i = r0 + b * kThreads + tid;
    if (i < m) {
      T* row = A + i;
      constexpr int H = NB > 32 ? NB / 2 : NB;
      {
        T x[H];
#pragma unroll
        for (int c = 0; c < H; ++c) x[c] = c < kb ? row[int64_t(k0 + c) * m] : T(0);
#pragma unroll
        for (int c = 0; c < H; ++c) {
          if (c < kb) {
            x[c] *= rdg[c];
#pragma unroll
            for (int t = c + 1; t < H; ++t)
              if (t < kb) x[t] -= x[c] * Dg[c][t];
          }
        }
#pragma unroll
        for (int c = 0; c < H; ++c)
          if (c < kb) row[int64_t(k0 + c) * m] = x[c];
      }
      if constexpr (NB > H) {
        T y[NB - H];
#pragma unroll
        for (int t = 0; t < NB - H; ++t) y[t] = H + t < kb ? row[int64_t(k0 + H + t) * m] : T(0);
        for (int c = 0; c < H && c < kb; ++c) {
          const T xc = row[int64_t(k0 + c) * m];
#pragma unroll
          for (int t = 0; t < NB - H; ++t)
            if (H + t < kb) y[t] -= xc * Dg[c][H + t];
        }
#pragma unroll
        for (int c = 0; c < NB - H; ++c) {
          if (H + c < kb) {
            y[c] *= rdg[H + c];
#pragma unroll
            for (int t = c + 1; t < NB - H; ++t)
              if (H + t < kb) y[t] -= y[c] * Dg[H + c][H + t];
          }
        }
#pragma unroll
        for (int t = 0; t < NB - H; ++t)
          if (H + t < kb) row[int64_t(k0 + H + t) * m] = y[t];
      }
    }
    return;
  }
  const int w = tid >> 5, lane = tid & 31;
  const int jb = r0 + (b - nrc) * 64 + w * 8;
  T y0[8], y1[8];
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    const bool ok = jb + jj < m;
    const T* col = A + int64_t(jb + jj) * m + k0;
    y0[jj] = ok && lane < kb ? col[lane] : T(0);
    y1[jj] = ok && NB > 32 && lane + 32 < kb ? col[lane + 32] : T(0);
  }
  for (int c = 0; c < kb; ++c) {
    const T l0 = lane > c && lane < kb ? Dg[lane][c] : T(0);
    const T l1 = NB > 32 && lane + 32 > c && lane + 32 < kb ? Dg[(lane + 32) % NB][c] : T(0);
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {  // l0, l1 are zero outside the triangle
      const T yc = __shfl_sync(0xffffffffu, c < 32 ? y0[jj] : y1[jj], c & 31);
      y0[jj] -= l0 * yc;
      if (NB > 32) y1[jj] -= l1 * yc;
    }
  }
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    if (jb + jj >= m) break;
    T* col = A + int64_t(jb + jj) * m + k0;
    if (lane < kb) col[lane] = y0[jj];
    if (NB > 32 && lane + 32 < kb) col[lane + 32] = y1[jj];
  }
}

// trailing update of every listed front after pivot block k0: A₂₂ -= L₂₁ U₁₂,
// one 64 × 64 tile per block (4 × 4 per thread; a warp's rows are consecutive);
// the block after the last tile writes the factored diagonal block
template <class T, int NB>
__global__ void __launch_bounds__(kThreads) sp_update(const SpFrontDev* __restrict__ fr,
                                                      const int32_t* __restrict__ flist, int k0, T* __restrict__ F,
                                                      T tau, int* __restrict__ flags) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  if (k0 >= p) return;
  const int kb = min(NB, p - k0), r0 = k0 + kb, rest = m - r0;
  const int nt = (rest + kTile - 1) / kTile;
  if (int(blockIdx.x) > nt * nt) return;
  T* A = F + Fr.off;
  __shared__ T As[NB][kTile + 1];  // L₂₁ tile, As[c][i]
  __shared__ T Bs[NB][kTile + 1];  // U₁₂ tile, Bs[c][j]
  const int tid = threadIdx.x;
  if (int(blockIdx.x) == nt * nt) {
    static_assert(NB * (NB + 1) <= NB * (kTile + 1), "the diagonal block fits the tile buffer");
    T(*Dg)[NB + 1] = reinterpret_cast<T(*)[NB + 1]>(&As[0][0]);
    factor_diag<T, NB>(A, m, k0, kb, Dg, tau, flags, true);
    for (int t = tid; t < kb * kb; t += kThreads) {
      const int i = t % kb, j = t / kb;
      A[(k0 + i) + int64_t(k0 + j) * m] = Dg[i][j];
    }
    return;
  }
  const int i0 = r0 + (blockIdx.x % nt) * kTile, j0 = r0 + (blockIdx.x / nt) * kTile;
  for (int t = tid; t < NB * kTile; t += kThreads) {
    const int i = t % kTile, c = t / kTile;
    As[c][i] = (c < kb && i0 + i < m) ? A[(i0 + i) + int64_t(k0 + c) * m] : T(0);
  }
  for (int t = tid; t < NB * kTile; t += kThreads) {
    const int c = t % NB, j = t / NB;
    Bs[c][j] = (c < kb && j0 + j < m) ? A[(k0 + c) + int64_t(j0 + j) * m] : T(0);
  }
  __syncthreads();
  const int tr = tid & 15, tc = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
#pragma unroll 8
  for (int c = 0; c < NB; ++c) {
    T a[4], bb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = As[c][tr + 16 * u];
#pragma unroll
    for (int v = 0; v < 4; ++v) bb[v] = Bs[c][tc + 16 * v];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] += a[u] * bb[v];
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int j = j0 + tc + 16 * v;
    if (j >= m) continue;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + tr + 16 * u;
      if (i < m) A[i + int64_t(j) * m] -= acc[u][v];
    }
  }
}

// FP32 trailing update with 128 × 128 tiles (8 × 8 per thread, the L₂₁ and U₁₂
// panels of the tile in dynamic shared memory); otherwise as sp_update
constexpr int kTile32 = 128;
constexpr int kTcMinRest = 512;  // trailing blocks this large take the tensor-core update
constexpr int kPad32 = 4;
template <int NB>
__global__ void __launch_bounds__(kThreads) sp_update_f32(const SpFrontDev* __restrict__ fr,
                                                          const int32_t* __restrict__ flist, int k0,
                                                          float* __restrict__ F, float tau, int* __restrict__ flags) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  if (k0 >= p) return;
  const int kb = min(NB, p - k0), r0 = k0 + kb, rest = m - r0;
  const int nt = (rest + kTile32 - 1) / kTile32;
  if (int(blockIdx.x) > nt * nt) return;
  float* A = F + Fr.off;
  extern __shared__ float smem32[];
  float(*As)[kTile32 + kPad32] = reinterpret_cast<float(*)[kTile32 + kPad32]>(smem32);
  float(*Bs)[kTile32 + kPad32] = reinterpret_cast<float(*)[kTile32 + kPad32]>(smem32 + NB * (kTile32 + kPad32));
  const int tid = threadIdx.x;
  if (int(blockIdx.x) == nt * nt) {
    static_assert(NB * (NB + 1) <= NB * (kTile32 + kPad32), "the diagonal block fits the tile buffer");
    float(*Dg)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(smem32);
    factor_diag<float, NB>(A, m, k0, kb, Dg, tau, flags, true);
    for (int t = tid; t < kb * kb; t += kThreads) {
      const int i = t % kb, j = t / kb;
      A[(k0 + i) + int64_t(k0 + j) * m] = Dg[i][j];
    }
    return;
  }
  const int i0 = r0 + (blockIdx.x % nt) * kTile32, j0 = r0 + (blockIdx.x / nt) * kTile32;
  // the tile's operand loads in batches of 16 per thread, all in flight together
  constexpr int kPer = NB * kTile32 / kThreads;
  static_assert(kPer % 16 == 0, "whole batches");
#pragma unroll
  for (int b0 = 0; b0 < kPer; b0 += 16) {
    float va[16], vb[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int t = (b0 + u) * kThreads + tid;
      const int i = t % kTile32, c = t / kTile32;
      va[u] = (c < kb && i0 + i < m) ? A[(i0 + i) + int64_t(k0 + c) * m] : 0.f;
      const int cb = t % NB, j = t / NB;
      vb[u] = (cb < kb && j0 + j < m) ? A[(k0 + cb) + int64_t(j0 + j) * m] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int t = (b0 + u) * kThreads + tid;
      As[t / kTile32][t % kTile32] = va[u];
      Bs[t % NB][t / NB] = vb[u];
    }
  }
  __syncthreads();
  const int tr = tid & 15, tc = tid >> 4;
  float acc[8][8];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
#pragma unroll 4
  for (int c = 0; c < NB; ++c) {
    const float4 a0 = *reinterpret_cast<const float4*>(&As[c][4 * tr]);
    const float4 a1 = *reinterpret_cast<const float4*>(&As[c][64 + 4 * tr]);
    const float4 b0 = *reinterpret_cast<const float4*>(&Bs[c][4 * tc]);
    const float4 b1 = *reinterpret_cast<const float4*>(&Bs[c][64 + 4 * tc]);
    const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
    const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], bb[v], acc[u][v]);
  }
  // read-modify-write of the tile: two columns' 16 loads in flight at a time
#pragma unroll
  for (int v0 = 0; v0 < 8; v0 += 2) {
    float cv[2][8];
#pragma unroll
    for (int dv = 0; dv < 2; ++dv) {
      const int v = v0 + dv;
      const int j = j0 + (v < 4 ? 4 * tc + v : 64 + 4 * tc + v - 4);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + (u < 4 ? 4 * tr + u : 64 + 4 * tr + u - 4);
        cv[dv][u] = (i < m && j < m) ? A[i + int64_t(j) * m] : 0.f;
      }
    }
#pragma unroll
    for (int dv = 0; dv < 2; ++dv) {
      const int v = v0 + dv;
      const int j = j0 + (v < 4 ? 4 * tc + v : 64 + 4 * tc + v - 4);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + (u < 4 ? 4 * tr + u : 64 + 4 * tr + u - 4);
        if (i < m && j < m) A[i + int64_t(j) * m] = cv[dv][u] - acc[u][v];
      }
    }
  }
}

// ---- FP32 factorisation by super-panels of kSuper pivots: inside a
// super-panel each 64-column block first takes the products of the
// super-panel's earlier blocks (its column block and its row block, the
// left-looking part), then its panel is factored; the trailing block takes
// the whole super-panel's products at once (K = kSuper), so that it is read
// and written once per kSuper pivots instead of once per 64.
constexpr int kSuper = 256;

// C −= L U over 128 × 128 tiles of a rectangle of every listed front, K in
// chunks of 64.  mode 0: rows [k0, m) × columns [k0, min(k0+64, p)), K [s0, k0)
// (the column block); mode 1: rows [k0, min(k0+64, p)) × columns [min(k0+64, p), m),
// K [s0, k0) (the row block); mode 2: rows and columns [e0, m) with
// e0 = min(s0 + kSuper, p), K [s0, e0) (the trailing block).  The products
// are summed apart from C and subtracted once: accumulating them into C would
// round every product at the scale of C, which leaves the FP32 factors of the
// large lattice fronts too coarse for the refinement.
__global__ void __launch_bounds__(kThreads, 2) sp_rect_f32(const SpFrontDev* __restrict__ fr,
                                                        const int32_t* __restrict__ flist, int mode, int s0, int k0,
                                                        int ntc, float* __restrict__ F) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  int ra, rb, ca, cb, ka, kz;
  if (mode == 2) {
    const int e0 = min(s0 + kSuper, p);
    ra = ca = e0;
    rb = cb = m;
    ka = s0;
    kz = e0;
  } else {
    if (k0 >= p) return;
    ka = s0;
    kz = k0;
    if (mode == 0) {
      ra = k0;
      rb = m;
      ca = k0;
      cb = min(k0 + 64, p);
    } else {
      ra = k0;
      rb = min(k0 + 64, p);
      ca = rb;
      cb = m;
    }
  }
  if (kz <= ka) return;
  const int i0 = ra + int(blockIdx.x / ntc) * kTile32;
  const int j0 = ca + int(blockIdx.x % ntc) * kTile32;
  if (i0 >= rb || j0 >= cb) return;
  float* A = F + Fr.off;
  extern __shared__ float smem32[];
  float(*As)[kTile32 + kPad32] = reinterpret_cast<float(*)[kTile32 + kPad32]>(smem32);
  float(*Bs)[kTile32 + kPad32] = reinterpret_cast<float(*)[kTile32 + kPad32]>(smem32 + 64 * (kTile32 + kPad32));
  const int tid = threadIdx.x, tr = tid & 15, tc = tid >> 4;
  float acc[8][8];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
  for (int kc = ka; kc < kz; kc += 64) {
    const int kn = min(64, kz - kc);
    constexpr int kPer = 64 * kTile32 / kThreads;
#pragma unroll
    for (int b0 = 0; b0 < kPer; b0 += 8) {
      float va[8], vb[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int t = (b0 + u) * kThreads + tid;
        const int i = t % kTile32, c = t / kTile32;
        va[u] = (c < kn && i0 + i < rb) ? A[(i0 + i) + int64_t(kc + c) * m] : 0.f;
        const int cc = t % 64, j = t / 64;
        vb[u] = (cc < kn && j0 + j < cb) ? A[(kc + cc) + int64_t(j0 + j) * m] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int t = (b0 + u) * kThreads + tid;
        As[t / kTile32][t % kTile32] = va[u];
        Bs[t % 64][t / 64] = vb[u];
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int c = 0; c < 64; ++c) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[c][4 * tr]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[c][64 + 4 * tr]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[c][4 * tc]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[c][64 + 4 * tc]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], bb[v], acc[u][v]);
    }
    __syncthreads();
  }
  // read-modify-write of the tile, two columns' 16 loads in flight at a time
#pragma unroll
  for (int v0 = 0; v0 < 8; v0 += 2) {
    float cv[2][8];
#pragma unroll
    for (int dv = 0; dv < 2; ++dv) {
      const int v = v0 + dv;
      const int j = j0 + (v < 4 ? 4 * tc + v : 64 + 4 * tc + v - 4);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + (u < 4 ? 4 * tr + u : 64 + 4 * tr + u - 4);
        cv[dv][u] = (i < rb && j < cb) ? A[i + int64_t(j) * m] : 0.f;
      }
    }
#pragma unroll
    for (int dv = 0; dv < 2; ++dv) {
      const int v = v0 + dv;
      const int j = j0 + (v < 4 ? 4 * tc + v : 64 + 4 * tc + v - 4);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + (u < 4 ? 4 * tr + u : 64 + 4 * tr + u - 4);
        if (i < rb && j < cb) A[i + int64_t(j) * m] = cv[dv][u] - acc[u][v];
      }
    }
  }
}

// the trailing block of a super-panel on the tensor cores (what sp_rect_f32
// does in mode 2: rows and columns [e0, m) −= the super-panel's L and U parts,
// K [s0, e0)), one 128 × 128 tile per block
__global__ void __launch_bounds__(tc::kTcThreads) sp_trail_tc(const SpFrontDev* __restrict__ fr,
                                                               const int32_t* __restrict__ flist, int s0, int nt,
                                                               float* __restrict__ F, int* __restrict__ flags) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  const int e0 = min(s0 + kSuper, p);
  if (e0 <= s0) return;
  const int i0 = e0 + int(blockIdx.x / nt) * tc::kTcTile, j0 = e0 + int(blockIdx.x % nt) * tc::kTcTile;
  if (i0 >= m || j0 >= m) return;
  if (ld_relaxed_i32(flags + 3) & 4) return;  // a tile's wait ran out: the factors are discarded
  float* A = F + Fr.off;
  extern __shared__ __align__(128) float smem_tc[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  const bool ok = tc::tile_update_tf32x3(A, m, A, m, A, m, i0, j0, m, m, s0, e0, smem_tc, bar, &tslot);
  if (!ok && threadIdx.x == 0) atomicOr(flags + 3, 4);
}

// the left-looking column block (mode 0) or row block (mode 1) of pivot block
// k0 inside a super-panel on the tensor cores: what sp_rect_f32 does in those
// modes, one 128 × 128 tile per block (the 64-wide side masked)
__global__ void __launch_bounds__(tc::kTcThreads) sp_rect_tc(const SpFrontDev* __restrict__ fr,
                                                              const int32_t* __restrict__ flist, int mode, int s0,
                                                              int k0, int ntc, float* __restrict__ F,
                                                              int* __restrict__ flags) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  if (k0 >= p || k0 <= s0) return;
  int ra, rb, ca, cb;
  if (mode == 0) {
    ra = k0;
    rb = m;
    ca = k0;
    cb = min(k0 + 64, p);
  } else {
    ra = k0;
    rb = min(k0 + 64, p);
    ca = rb;
    cb = m;
  }
  const int i0 = ra + int(blockIdx.x / ntc) * tc::kTcTile, j0 = ca + int(blockIdx.x % ntc) * tc::kTcTile;
  if (i0 >= rb || j0 >= cb) return;
  if (ld_relaxed_i32(flags + 3) & 4) return;
  float* A = F + Fr.off;
  extern __shared__ __align__(128) float smem_tc[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  const bool ok = tc::tile_update_tf32x3(A, m, A, m, A, m, i0, j0, rb, cb, s0, k0, smem_tc, bar, &tslot);
  if (!ok && threadIdx.x == 0) atomicOr(flags + 3, 4);
}

// the diagonal block of pivot block k0 factored in place in every listed front
// (before sp_panel_f, which reads it factored), with the arithmetic of
// factor_diag: NB threads, thread i owning row i of the staged block; one
// block barrier per step (after it, row k is final).  Every thread applies the
// pivot rule to its read of the pivot itself (the rule is idempotent, so the
// owner's write-back of a raised pivot cannot change what another reads).
template <class T, int NB>
__global__ void __launch_bounds__(NB) sp_diag_store(const SpFrontDev* __restrict__ fr,
                                                    const int32_t* __restrict__ flist, int k0, T* __restrict__ F,
                                                    T tau, int* __restrict__ flags) {
  const SpFrontDev Fr = fr[flist[blockIdx.x]];
  const int m = Fr.m, p = Fr.p;
  if (k0 >= p) return;
  const int kb = min(NB, p - k0);
  T* A = F + Fr.off;
  __shared__ T Dg[NB][NB + 1];
  const int i = threadIdx.x;
  stage_diag_block<T, NB>(A, m, k0, kb, Dg);
  for (int k = 0; k < kb; ++k) {
    __syncthreads();
    const T d = Dg[k][k];
    const bool bad = !isfinite(d) || (d == T(0) && tau == T(0));
    const bool raise = !bad && fabs(d) < tau;
    const T piv = raise ? (d < T(0) ? -tau : tau) : d;
    if (i == k) {
      if (bad) atomicOr(flags + 3, 1);
      if (raise) {
        Dg[k][k] = piv;
        atomicAdd(flags + 2, 1);
      }
    } else if (i > k && i < kb) {
      const T l = Dg[i][k] / piv;
      Dg[i][k] = l;
      // eight entries of row k and of row i loaded before any is stored (the
      // compiler cannot tell the rows apart, so a plain loop would wait for
      // each load behind the previous store)
      for (int j0 = k + 1; j0 < kb; j0 += 8) {
        T u[8], r[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          u[q] = j0 + q < kb ? Dg[k][j0 + q] : T(0);
          r[q] = j0 + q < kb ? Dg[i][j0 + q] : T(0);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (j0 + q < kb) Dg[i][j0 + q] = r[q] - l * u[q];
      }
    }
  }
  __syncthreads();
  for (int j = 0; j < kb; ++j)
    if (i < kb) A[(k0 + i) + int64_t(k0 + j) * m] = Dg[i][j];
}

// FP32 trailing update on the tensor cores: one 128 × 128 tile per block
// (tc::tile_update_tf32x3, three TF32 products per k-step, FP32 accumulators in
// tensor memory); the block after the last tile writes the factored diagonal
// block.  flags[3] |= 2 when a tile's MMAs did not complete within the wait.
template <int NB>
__global__ void __launch_bounds__(tc::kTcThreads) sp_update_tc(const SpFrontDev* __restrict__ fr,
                                                                const int32_t* __restrict__ flist, int k0,
                                                                float* __restrict__ F, float tau,
                                                                int* __restrict__ flags) {
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p;
  if (k0 >= p) return;
  const int kb = min(NB, p - k0), r0 = k0 + kb, rest = m - r0;
  const int nt = (rest + tc::kTcTile - 1) / tc::kTcTile;
  if (int(blockIdx.x) > nt * nt) return;
  float* A = F + Fr.off;
  extern __shared__ __align__(128) float smem_tc[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  if (int(blockIdx.x) == nt * nt) {
    float(*Dg)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(smem_tc);
    factor_diag<float, NB>(A, m, k0, kb, Dg, tau, flags, true);
    for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
      const int i = t % kb, j = t / kb;
      A[(k0 + i) + int64_t(k0 + j) * m] = Dg[i][j];
    }
    return;
  }
  const int i0 = r0 + (blockIdx.x % nt) * tc::kTcTile, j0 = r0 + (blockIdx.x / nt) * tc::kTcTile;
  const bool ok = tc::tile_update_tf32x3(A, m, A, m, A, m, i0, j0, m, m, k0, k0 + kb, smem_tc, bar, &tslot);
  if (!ok && threadIdx.x == 0) atomicOr(flags + 3, 4);
}

// C −= A B for host arrays through the same tile routine (column-major, K ≤ 64):
// the tensor-core path's check against a host product
__global__ void __launch_bounds__(tc::kTcThreads) tc_gemm_check(const float* __restrict__ A, int lda,
                                                                 const float* __restrict__ B, int ldb,
                                                                 float* __restrict__ C, int ldc, int M, int N, int K,
                                                                 int* __restrict__ err) {
  extern __shared__ __align__(128) float smem_tc[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  const bool ok = tc::tile_update_tf32x3(A, lda, B, ldb, C, ldc, blockIdx.x * tc::kTcTile, blockIdx.y * tc::kTcTile,
                                         M, N, 0, K, smem_tc, bar, &tslot);
  if (!ok && threadIdx.x == 0) atomicOr(err, 1);
}

// ---------------------------------------------------------------- substitutions (FP64 vectors)
// Per height, leaves first for the forward substitution (roots first for the
// backward one), with two kernels each: one block per front solves the
// triangle of its pivots (blocks of 32 columns: the 32 × 32 diagonal block is
// staged in shared memory and solved by one warp, then all threads update the
// pivot rows below), and a grid of blocks, 256 rows each, does the front's
// rectangular part (L₂₁ y or U₁₂ x_u), one row per thread summing in column
// order.  Vectors are FP64, factors T.
constexpr int kTriThreads = 512;
constexpr int kGemvRows = 256;

// forward, triangle: v = the front's pivot entries plus the children's update
// vectors (in child order); y = L₁₁⁻¹ v[0:p] -> w; v[p:m] (the children's part of
// the update rows) -> cvec, to which sp_fwd_gemv adds −L₂₁ y
template <class T>
__global__ void __launch_bounds__(kTriThreads) sp_fwd_tri(const SpFrontDev* __restrict__ fr,
                                                          const int32_t* __restrict__ flist,
                                                          const int32_t* __restrict__ clist,
                                                          const int32_t* __restrict__ emap, const T* __restrict__ F,
                                                          double* __restrict__ w, double* __restrict__ cvec,
                                                          const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.x]];
  extern __shared__ double v[];
  __shared__ double Dg[32][33];
  __shared__ double yb[32];
  const int m = Fr.m, p = Fr.p, tid = threadIdx.x;
  for (int t = tid; t < m; t += kTriThreads) v[t] = t < p ? w[Fr.pos0 + t] : 0.0;
  __syncthreads();
  for (int k = 0; k < Fr.nc; ++k) {
    const SpFrontDev C = fr[clist[Fr.c0 + k]];
    const int uc = C.m - C.p;
    for (int t = tid; t < uc; t += kTriThreads) v[emap[C.eoff + t]] += cvec[C.eoff + t];
    __syncthreads();
  }
  const T* A = F + Fr.off;
  for (int c0 = 0; c0 < p; c0 += 32) {
    const int cb = min(32, p - c0);
    for (int t = tid; t < cb * 32; t += kTriThreads) {
      const int i = t & 31, j = t >> 5;
      Dg[i][j] = (i < cb && j < i) ? double(A[(c0 + i) + int64_t(c0 + j) * m]) : 0.0;  // strict lower
    }
    __syncthreads();
    if (tid < 32) {
      double y = tid < cb ? v[c0 + tid] : 0.0;
#pragma unroll 4
      for (int c = 0; c < cb; ++c) {  // branch-free: zeros at and above the diagonal
        const double yc = __shfl_sync(0xffffffffu, y, c);
        y -= Dg[tid][c] * yc;
      }
      if (tid < cb) {
        v[c0 + tid] = y;
        yb[tid] = y;
      }
    }
    __syncthreads();
    for (int i = c0 + cb + tid; i < p; i += kTriThreads) {
      double s = 0.0;
      for (int c = 0; c < cb; ++c) s += double(A[i + int64_t(c0 + c) * m]) * yb[c];
      v[i] -= s;
    }
    __syncthreads();
  }
  for (int t = tid; t < p; t += kTriThreads) w[Fr.pos0 + t] = v[t];
  if (Fr.parent >= 0)
    for (int t = p + tid; t < m; t += kTriThreads) cvec[Fr.eoff + (t - p)] = v[t];
}

// forward, rectangle: cvec[f][t] -= Σ_c L₂₁[t, c] y_c for the update rows t of
// every front of the height (y staged in shared memory)
template <class T>
__global__ void __launch_bounds__(kGemvRows) sp_fwd_gemv(const SpFrontDev* __restrict__ fr,
                                                         const int32_t* __restrict__ flist, const T* __restrict__ F,
                                                         const double* __restrict__ w, double* __restrict__ cvec,
                                                         const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p, u = m - p;
  if (Fr.parent < 0 || int(blockIdx.x) * kGemvRows >= u) return;
  extern __shared__ double y[];
  for (int c = threadIdx.x; c < p; c += kGemvRows) y[c] = w[Fr.pos0 + c];
  __syncthreads();
  const int t = blockIdx.x * kGemvRows + threadIdx.x;
  if (t >= u) return;
  const T* L = F + Fr.off + p + t;  // row p+t of the front, column c at L[c*m]
  double s = 0.0;
#pragma unroll 8
  for (int c = 0; c < p; ++c) s += double(L[int64_t(c) * m]) * y[c];
  cvec[Fr.eoff + t] -= s;
}

// backward, rectangle: tw[pos0 + r] = Σ_{j ≥ p} U₁₂[r, j] x_j for the pivot rows r
// (x_u the ancestors' solved values, staged in shared memory)
template <class T>
__global__ void __launch_bounds__(kGemvRows) sp_bwd_gemv(const SpFrontDev* __restrict__ fr,
                                                         const int32_t* __restrict__ flist,
                                                         const int32_t* __restrict__ fidx, const T* __restrict__ F,
                                                         const double* __restrict__ w, double* __restrict__ tw,
                                                         const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p, u = m - p;
  if (int(blockIdx.x) * kGemvRows >= p) return;
  extern __shared__ double xu[];
  for (int j = threadIdx.x; j < u; j += kGemvRows) xu[j] = w[fidx[Fr.idx + p + j]];
  __syncthreads();
  const int r = blockIdx.x * kGemvRows + threadIdx.x;
  if (r >= p) return;
  const T* U = F + Fr.off + r + int64_t(p) * m;  // row r, column p+j at U[j*m]
  double s = 0.0;
#pragma unroll 8
  for (int j = 0; j < u; ++j) s += double(U[int64_t(j) * m]) * xu[j];
  tw[Fr.pos0 + r] = s;
}

// backward, triangle: x[0:p] = U₁₁⁻¹ (y − U₁₂ x_u) -> w
template <class T>
__global__ void __launch_bounds__(kTriThreads) sp_bwd_tri(const SpFrontDev* __restrict__ fr,
                                                          const int32_t* __restrict__ flist, const T* __restrict__ F,
                                                          double* __restrict__ w, const double* __restrict__ tw,
                                                          const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.x]];
  extern __shared__ double v[];
  constexpr int NW = kTriThreads / 32;
  __shared__ double part[NW][33];
  __shared__ double Dg[32][33];
  __shared__ double rdg[32];  // reciprocal pivots of the block
  const int m = Fr.m, p = Fr.p, tid = threadIdx.x;
  for (int t = tid; t < p; t += kTriThreads) v[t] = w[Fr.pos0 + t] - tw[Fr.pos0 + t];
  __syncthreads();
  const T* A = F + Fr.off;
  const int wp = tid >> 5, lane = tid & 31;
  for (int c1 = p; c1 > 0; c1 -= 32) {
    const int c0 = max(0, c1 - 32), cb = c1 - c0;
    double s = 0.0;
    if (lane < cb)
      for (int j = c1 + wp; j < p; j += NW) s += double(A[(c0 + lane) + int64_t(j) * m]) * v[j];
    part[wp][lane] = s;
    for (int t = tid; t < 32 * 32; t += kTriThreads) {
      const int i = t & 31, j = t >> 5;
      const double a = (i < cb && j < cb) ? double(A[(c0 + i) + int64_t(c0 + j) * m]) : 0.0;
      Dg[i][j] = j > i ? a : 0.0;  // strict upper; the diagonal enters as its reciprocal
      if (i == j && i < cb) rdg[i] = 1.0 / a;
    }
    __syncthreads();
    if (tid < 32) {
      double b = 0.0;
      if (lane < cb) {
        b = v[c0 + lane];
#pragma unroll
        for (int q = 0; q < NW; ++q) b -= part[q][lane];
      }
      // branch-free: every step updates every lane (zeros at and below the column)
#pragma unroll 4
      for (int c = cb - 1; c >= 0; --c) {
        const double xc = __shfl_sync(0xffffffffu, b, c) * rdg[c];
        b = fma(-Dg[lane][c], xc, b);
      }
      if (lane < cb) v[c0 + lane] = b * rdg[lane];
    }
    __syncthreads();
  }
  for (int t = tid; t < p; t += kTriThreads) w[Fr.pos0 + t] = v[t];
}

// ---------------------------------------------------------------- blocked substitutions
// The kernels above give a front one block for its triangle, which leaves the
// GPU idle on the few large fronts near the root (the top separator of a
// 60×60×20 lattice has 7,560 pivots: one block would stream its 114 MB
// triangle alone).  Fronts with at least kBigPivots pivots take these kernels
// instead.  The front's vector lives in global memory (V, at the front's
// index-list offset, m entries).  Its rows are cut into tiles of kSB: pivot
// tiles from row 0, update tiles from row p.  One launch per column block:
// every block owning a row tile still to be reduced subtracts that column
// block's products (columns summed 16 at a time in the factors' precision, the
// four partial sums added in FP64 in a fixed order), and the block owning the
// next diagonal tile then solves its triangle from shared memory, so the
// following launch finds that column block solved.
constexpr int kSB = 64;
constexpr int kSBThreads = 256;
constexpr int kBigPivots = 128;  // default threshold (MGPU_SPARSE_BLOCKED_PIVOTS overrides it)

__device__ __forceinline__ int sb_np(int p) { return (p + kSB - 1) / kSB; }
__device__ __forceinline__ int sb_nu(int m, int p) { return (m - p + kSB - 1) / kSB; }
// rows [r0, r1) of row tile t
__device__ __forceinline__ void sb_rows(int t, int m, int p, int& r0, int& r1) {
  const int np = sb_np(p);
  if (t < np) {
    r0 = t * kSB;
    r1 = min(r0 + kSB, p);
  } else {
    r0 = p + (t - np) * kSB;
    r1 = min(r0 + kSB, m);
  }
}

// v[r0..r1) -= A[r0..r1, c0..c0+cb) · x (x in shared memory); the block's 256
// threads: row rr = tid % 64, columns 16·(tid / 64) ..; returns the new value of
// row r0 + tid for tid < 64 (FP64), written back to V as well
template <class T>
__device__ __forceinline__ double sb_update(const T* __restrict__ A, int m, int r0, int r1, int c0, int cb,
                                            const T* xs, double (*part)[kSB], double* __restrict__ Vf) {
  const int tid = threadIdx.x, rr = tid & (kSB - 1), cq = tid >> 6;
  const int r = r0 + rr;
  T sacc = T(0);
  if (r < r1) {
    const T* col = A + r + int64_t(c0) * m;
    const int cbeg = cq * 16;
#pragma unroll
    for (int c = 0; c < 16; ++c)
      if (cbeg + c < cb) sacc = fma(col[int64_t(cbeg + c) * m], xs[cbeg + c], sacc);
  }
  part[cq][rr] = double(sacc);
  __syncthreads();
  double v = 0.0;
  if (tid < kSB && r0 + tid < r1) {
    v = Vf[r0 + tid] - (((part[0][tid] + part[1][tid]) + part[2][tid]) + part[3][tid]);
    Vf[r0 + tid] = v;
  }
  return v;
}

// stage the strict lower (lower = true) or the strict upper triangle of the
// diagonal tile, zeros elsewhere; 8 loads per thread in flight before their stores
template <class T>
__device__ __forceinline__ void sb_stage_diag(const T* __restrict__ A, int m, int r0, int nr, bool lower,
                                              T (*Dg)[kSB + 1]) {
  static_assert(kSB * kSB == 16 * kSBThreads, "two batches of 8 per thread");
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = (8 * h + u) * kSBThreads + threadIdx.x;
      const int i = q & (kSB - 1), c = q >> 6;
      const bool in = i < nr && c < nr && (lower ? c < i : c > i);
      v[u] = in ? A[(r0 + i) + int64_t(r0 + c) * m] : T(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = (8 * h + u) * kSBThreads + threadIdx.x;
      Dg[q & (kSB - 1)][q >> 6] = v[u];
    }
  }
}

// unit lower triangle of the diagonal tile rows [r0, r0+nr): v = L⁻¹ v, in place
// (vals: the tile's current values, threads 0..63); the block's threads stage
// the tile, warp 0 solves (lane l holds rows l and l + 32)
template <class T>
__device__ void sb_tri_lower(const T* __restrict__ A, int m, int r0, int nr, T (*Dg)[kSB + 1], T* vs,
                             double* __restrict__ Vf) {
  const int tid = threadIdx.x;
  sb_stage_diag<T>(A, m, r0, nr, true, Dg);
  __syncthreads();
  if (tid < 32) {
    T a0 = vs[tid], a1 = vs[tid + 32];
#pragma unroll 4
    for (int c = 0; c < nr; ++c) {
      const T yc = __shfl_sync(0xffffffffu, c < 32 ? a0 : a1, c & 31);
      a0 = fma(-Dg[tid][c], yc, a0);
      a1 = fma(-Dg[tid + 32][c], yc, a1);
    }
    if (tid < nr) Vf[r0 + tid] = double(a0);
    if (tid + 32 < nr) Vf[r0 + tid + 32] = double(a1);
  }
}

// x = U⁻¹ v for the staged strict upper triangle of a diagonal tile (warp 0;
// lane l holds rows l and l + 32), with the reciprocals rd[] of its diagonal,
// formed while staging.  Branch-free: every step updates every lane (the
// staged zeros leave the rows at and below the column as they are), and a
// row's value times its reciprocal pivot, the solution, is formed at the
// step of its column for the broadcast and once more at the end in place
// (lane-dependent branches per step made this solve 2.5 times slower than
// the forward one).
template <class T>
__device__ __forceinline__ void sb_solve_upper(const T (*Dg)[kSB + 1], const T* rd, const T* vs, int nr, int r0,
                                               double* __restrict__ Vf) {
  const int tid = threadIdx.x;
  T a0 = vs[tid], a1 = vs[tid + 32];
#pragma unroll 4
  for (int c = nr - 1; c >= 0; --c) {
    const T xc = __shfl_sync(0xffffffffu, c < 32 ? a0 : a1, c & 31) * rd[c];
    a0 = fma(-Dg[tid][c], xc, a0);
    a1 = fma(-Dg[tid + 32][c], xc, a1);
  }
  if (tid < nr) Vf[r0 + tid] = double(a0 * rd[tid]);
  if (tid + 32 < nr) Vf[r0 + tid + 32] = double(a1 * rd[tid + 32]);
}

// upper triangle of the diagonal tile: x = U⁻¹ v, in place
template <class T>
__device__ void sb_tri_upper(const T* __restrict__ A, int m, int r0, int nr, T (*Dg)[kSB + 1], T* vs,
                             double* __restrict__ Vf) {
  const int tid = threadIdx.x;
  __shared__ T rd[kSB];
  sb_stage_diag<T>(A, m, r0, nr, false, Dg);
  if (tid < nr) rd[tid] = T(1) / A[(r0 + tid) + int64_t(r0 + tid) * m];
  __syncthreads();
  if (tid < 32) sb_solve_upper<T>(Dg, rd, vs, nr, r0, Vf);
}

// forward: V = the front's pivot entries, zero update rows
__global__ void sp_fwdb_init(const SpFrontDev* __restrict__ fr, const int32_t* __restrict__ flist,
                             const double* __restrict__ w, double* __restrict__ V, const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t < Fr.m) V[Fr.idx + t] = t < Fr.p ? w[Fr.pos0 + t] : 0.0;
}

// forward: add child number r's update vector (the children in rank order)
__global__ void sp_fwdb_ext(const SpFrontDev* __restrict__ fr, const int32_t* __restrict__ flist,
                            const int32_t* __restrict__ clist, const int32_t* __restrict__ emap, int r,
                            const double* __restrict__ cvec, double* __restrict__ V, const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  if (r >= Fr.nc) return;
  const SpFrontDev C = fr[clist[Fr.c0 + r]];
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t < C.m - C.p) V[Fr.idx + emap[C.eoff + t]] += cvec[C.eoff + t];
}

// forward: the triangle of pivot tile 0
template <class T>
__global__ void __launch_bounds__(kSBThreads) sp_fwdb_first(const SpFrontDev* __restrict__ fr,
                                                            const int32_t* __restrict__ flist,
                                                            const T* __restrict__ F, double* __restrict__ V,
                                                            const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.x]];
  __shared__ T Dg[kSB][kSB + 1];
  __shared__ T vs[kSB];
  double* Vf = V + Fr.idx;
  const int nr = min(kSB, Fr.p);
  if (threadIdx.x < kSB) vs[threadIdx.x] = threadIdx.x < nr ? T(Vf[threadIdx.x]) : T(0);
  sb_tri_lower<T>(F + Fr.off, Fr.m, 0, nr, Dg, vs, Vf);
}

// forward, column block j (solved): the row tiles after it take its products;
// the block of tile j + 1 (a pivot tile) then solves that tile
template <class T>
__global__ void __launch_bounds__(kSBThreads) sp_fwdb_step(const SpFrontDev* __restrict__ fr,
                                                           const int32_t* __restrict__ flist, int j,
                                                           const T* __restrict__ F, double* __restrict__ V,
                                                           const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p, np = sb_np(p), nt = np + sb_nu(m, p);
  const int t = j + 1 + int(blockIdx.x);
  if (j >= np || t >= nt) return;
  __shared__ T xs[kSB];
  __shared__ double part[4][kSB];
  __shared__ T Dg[kSB][kSB + 1];
  __shared__ T vs[kSB];
  const int c0 = j * kSB, cb = min(kSB, p - c0);
  double* Vf = V + Fr.idx;
  const T* A = F + Fr.off;
  if (threadIdx.x < kSB) xs[threadIdx.x] = threadIdx.x < cb ? T(Vf[c0 + threadIdx.x]) : T(0);
  __syncthreads();
  int r0, r1;
  sb_rows(t, m, p, r0, r1);
  const double v = sb_update<T>(A, m, r0, r1, c0, cb, xs, part, Vf);
  if (t != j + 1 || t >= np) return;
  if (threadIdx.x < kSB) vs[threadIdx.x] = T(v);
  sb_tri_lower<T>(A, m, r0, r1 - r0, Dg, vs, Vf);
}

// forward: y to w, the update rows to the parent's extend-add vector
__global__ void sp_fwdb_fin(const SpFrontDev* __restrict__ fr, const int32_t* __restrict__ flist,
                            const double* __restrict__ V, double* __restrict__ w, double* __restrict__ cvec,
                            const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= Fr.m) return;
  if (t < Fr.p)
    w[Fr.pos0 + t] = V[Fr.idx + t];
  else if (Fr.parent >= 0)
    cvec[Fr.eoff + (t - Fr.p)] = V[Fr.idx + t];
}

// backward: V = y of the pivots
__global__ void sp_bwdb_init(const SpFrontDev* __restrict__ fr, const int32_t* __restrict__ flist,
                             const double* __restrict__ w, double* __restrict__ V, const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t < Fr.p) V[Fr.idx + t] = w[Fr.pos0 + t];
}

// backward, the update columns all at once: block (t, b) forms the products of
// pivot tile t with update column block b (x from the ancestors' solution) into
// P[poff(front) + b·p + row]; sp_bwdb_red subtracts them in block order
template <class T>
__global__ void __launch_bounds__(kSBThreads) sp_bwdb_u12(const SpFrontDev* __restrict__ fr,
                                                          const int32_t* __restrict__ flist,
                                                          const int64_t* __restrict__ poff,
                                                          const int32_t* __restrict__ fidx,
                                                          const T* __restrict__ F, const double* __restrict__ w,
                                                          double* __restrict__ P, const int* __restrict__ conv) {
  if (*conv) return;
  const int32_t f = flist[blockIdx.z];
  const SpFrontDev Fr = fr[f];
  const int m = Fr.m, p = Fr.p, t = int(blockIdx.x), b = int(blockIdx.y);
  if (t >= sb_np(p) || b >= sb_nu(m, p)) return;
  __shared__ T xs[kSB];
  __shared__ double part[4][kSB];
  const int c0 = p + b * kSB, cb = min(kSB, m - c0);
  if (threadIdx.x < kSB) xs[threadIdx.x] = threadIdx.x < cb ? T(w[fidx[Fr.idx + c0 + threadIdx.x]]) : T(0);
  __syncthreads();
  const int r0 = t * kSB, r1 = min(r0 + kSB, p);
  const int tid = threadIdx.x, rr = tid & (kSB - 1), cq = tid >> 6;
  const int r = r0 + rr;
  T sacc = T(0);
  if (r < r1) {
    const T* col = F + Fr.off + r + int64_t(c0) * m;
    const int cbeg = cq * 16;
#pragma unroll
    for (int c = 0; c < 16; ++c)
      if (cbeg + c < cb) sacc = fma(col[int64_t(cbeg + c) * m], xs[cbeg + c], sacc);
  }
  part[cq][rr] = double(sacc);
  __syncthreads();
  if (tid < kSB && r0 + tid < r1)
    P[poff[f] + int64_t(b) * p + r0 + tid] = ((part[0][tid] + part[1][tid]) + part[2][tid]) + part[3][tid];
}

__global__ void sp_bwdb_red(const SpFrontDev* __restrict__ fr, const int32_t* __restrict__ flist,
                            const int64_t* __restrict__ poff, const double* __restrict__ P, double* __restrict__ V,
                            const int* __restrict__ conv) {
  if (*conv) return;
  const int32_t f = flist[blockIdx.y];
  const SpFrontDev Fr = fr[f];
  const int r = blockIdx.x * kThreads + threadIdx.x;
  if (r >= Fr.p) return;
  const int nu = sb_nu(Fr.m, Fr.p);
  double s = 0.0;
  for (int b = 0; b < nu; ++b) s += P[poff[f] + int64_t(b) * Fr.p + r];
  V[Fr.idx + r] -= s;
}

// backward: the triangle of the last pivot tile, once the update columns are in
template <class T>
__global__ void __launch_bounds__(kSBThreads) sp_bwdb_last(const SpFrontDev* __restrict__ fr,
                                                           const int32_t* __restrict__ flist,
                                                           const T* __restrict__ F, double* __restrict__ V,
                                                           const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.x]];
  __shared__ T Dg[kSB][kSB + 1];
  __shared__ T vs[kSB];
  double* Vf = V + Fr.idx;
  const int r0 = (sb_np(Fr.p) - 1) * kSB, nr = Fr.p - r0;
  if (threadIdx.x < kSB) vs[threadIdx.x] = threadIdx.x < nr ? T(Vf[r0 + threadIdx.x]) : T(0);
  sb_tri_upper<T>(F + Fr.off, Fr.m, r0, nr, Dg, vs, Vf);
}

// backward, step s over the pivot blocks: column block b = np − 1 − s (solved);
// the pivot tiles above it take its products and the block of tile b − 1 then
// solves that tile
template <class T>
__global__ void __launch_bounds__(kSBThreads) sp_bwdb_step(const SpFrontDev* __restrict__ fr,
                                                           const int32_t* __restrict__ flist, int s,
                                                           const T* __restrict__ F, double* __restrict__ V,
                                                           const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int m = Fr.m, p = Fr.p, np = sb_np(p);
  const int b = np - 1 - s, t = int(blockIdx.x);
  if (b < 1 || t >= b) return;
  __shared__ T xs[kSB];
  __shared__ double part[4][kSB];
  __shared__ T Dg[kSB][kSB + 1];
  __shared__ T vs[kSB];
  double* Vf = V + Fr.idx;
  const T* A = F + Fr.off;
  const int c0 = b * kSB, cb = min(kSB, p - c0);
  if (threadIdx.x < kSB) xs[threadIdx.x] = threadIdx.x < cb ? T(Vf[c0 + threadIdx.x]) : T(0);
  __syncthreads();
  const int r0 = t * kSB, r1 = min(r0 + kSB, p);
  const double v = sb_update<T>(A, m, r0, r1, c0, cb, xs, part, Vf);
  if (t != b - 1) return;
  if (threadIdx.x < kSB) vs[threadIdx.x] = T(v);
  sb_tri_upper<T>(A, m, r0, r1 - r0, Dg, vs, Vf);
}

// ---- chained substitutions: one launch per height and direction.  The
// blocks take work items (row tile t of front f) from a counter in the order
// t·nf + f (forward; backward by distance from the last pivot tile), so that
// every tile an item waits for was taken earlier by a block that is running:
// the waits always end.  A pivot tile, once solved, publishes its values and
// then its flag (the launch's epoch); a tile that needs column block j waits
// for the flag of tile j, its factor entries already loaded.  The arithmetic
// is that of the launch-per-column-block kernels above, in the same order, so
// both give bitwise the same vectors.  Every wait is bounded: when one runs
// out, the block sets the abort word and flags[3], and the other blocks stop
// at their next wait or item.
constexpr int64_t kTileWaitPolls = int64_t(1) << 22;

// flags of front fid's tiles: (idx / 64) + 2·fid leaves every front room for its tiles
__device__ __forceinline__ int64_t sb_flag_base(const SpFrontDev& Fr, int32_t fid) {
  return (Fr.idx >> 6) + 2 * int64_t(fid);
}

// thread 0 waits for *flag == epoch, then the block synchronises; false (for
// the whole block) when the wait ran out or another block gave up
__device__ bool sb_wait(const unsigned* flag, unsigned epoch, int* abort_word, int* flags, int* ok_s) {
  if (threadIdx.x == 0) {
    int ok = 1;
    for (int64_t i = 0;; ++i) {
      if (ld_acquire_u32(flag) == epoch) break;
      if ((i & 63) == 63 && ld_relaxed_i32(abort_word)) {
        ok = 0;
        break;
      }
      if (i >= kTileWaitPolls) {
        atomicExch(abort_word, 1);
        atomicOr(flags + 3, 2);
        ok = 0;
        break;
      }
      if (i > 32) __nanosleep(128);
    }
    *ok_s = ok;
  }
  __syncthreads();
  const bool ok = *ok_s != 0;
  __syncthreads();
  return ok;
}

// next work item of the block (total when there is none left or the launch aborted)
__device__ int sb_claim(int* ctr, int total, const int* abort_word, int* item_s) {
  if (threadIdx.x == 0) *item_s = ld_relaxed_i32(abort_word) ? total : atomicAdd(ctr, 1);
  __syncthreads();
  const int item = *item_s;
  __syncthreads();
  return item;
}

// v -= A[r0..r1, c0..c0+cb) · x for the block's rows, x the solved tile of
// column block j (a[]: this thread's 16 factor entries, loaded before the wait)
template <class T>
__device__ __forceinline__ void sb_chain_load(const T* __restrict__ A, int m, int r0, int r1, int c0, int cb,
                                              T (&a)[16]) {
  const int tid = threadIdx.x, rr = tid & (kSB - 1), cq = tid >> 6;
  const int r = r0 + rr, cbeg = cq * 16;
#pragma unroll
  for (int c = 0; c < 16; ++c)
    a[c] = (r < r1 && cbeg + c < cb) ? A[r + int64_t(c0 + cbeg + c) * m] : T(0);
}
template <class T>
__device__ __forceinline__ void sb_chain_apply(const T (&a)[16], int cb, const double* Vx, T* xs,
                                               double (*part)[kSB], double& v) {
  const int tid = threadIdx.x, rr = tid & (kSB - 1), cq = tid >> 6;
  if (tid < kSB) xs[tid] = tid < cb ? T(__ldcg(Vx + tid)) : T(0);
  __syncthreads();
  const int cbeg = cq * 16;
  T sacc = T(0);
#pragma unroll
  for (int c = 0; c < 16; ++c)
    if (cbeg + c < cb) sacc = fma(a[c], xs[cbeg + c], sacc);
  part[cq][rr] = double(sacc);
  __syncthreads();
  if (tid < kSB) v = v - (((part[0][tid] + part[1][tid]) + part[2][tid]) + part[3][tid]);
  __syncthreads();
}


template <class T>
__global__ void __launch_bounds__(kSBThreads) sp_fwdb_chain(const SpFrontDev* __restrict__ fr,
                                                            const int32_t* __restrict__ flist, int nf, int ntmax,
                                                            const T* __restrict__ F, double* __restrict__ V,
                                                            unsigned* __restrict__ tflag, unsigned epoch,
                                                            int* __restrict__ ctr, int* __restrict__ abort_word,
                                                            int* __restrict__ flags) {
  if (flags[0]) return;
  __shared__ T xs[kSB];
  __shared__ double part[4][kSB];
  __shared__ T Dg[kSB][kSB + 1];
  __shared__ T vs[kSB];
  __shared__ int sync_s[2];
  const int tid = threadIdx.x;
  const int total = ntmax * nf;
  for (;;) {
    const int item = sb_claim(ctr, total, abort_word, &sync_s[0]);
    if (item >= total) return;
    const int t = item / nf;
    const int32_t fid = flist[item % nf];
    const SpFrontDev Fr = fr[fid];
    const int m = Fr.m, p = Fr.p, np = sb_np(p), nt = np + sb_nu(m, p);
    if (t >= nt) continue;
    int r0, r1;
    sb_rows(t, m, p, r0, r1);
    const T* A = F + Fr.off;
    double* Vf = V + Fr.idx;
    unsigned* tf = tflag + sb_flag_base(Fr, fid);
    const bool piv = t < np;
    if (piv) sb_stage_diag<T>(A, m, r0, r1 - r0, true, Dg);
    double v = (tid < kSB && r0 + tid < r1) ? Vf[r0 + tid] : 0.0;
    const int jmax = min(t, np);
    bool ok = true;
    for (int j = 0; j < jmax && ok; ++j) {
      const int c0 = j * kSB, cb = min(kSB, p - c0);
      T a[16];
      sb_chain_load<T>(A, m, r0, r1, c0, cb, a);
      ok = sb_wait(tf + j, epoch, abort_word, flags, &sync_s[1]);
      if (ok) sb_chain_apply<T>(a, cb, Vf + c0, xs, part, v);
    }
    if (!ok) return;
    if (!piv) {
      if (tid < kSB && r0 + tid < r1) Vf[r0 + tid] = v;
      continue;
    }
    const int nr = r1 - r0;
    if (tid < kSB) vs[tid] = T(v);
    __syncthreads();
    if (tid < 32) {
      T a0 = vs[tid], a1 = vs[tid + 32];
#pragma unroll 4
      for (int c = 0; c < nr; ++c) {
        const T yc = __shfl_sync(0xffffffffu, c < 32 ? a0 : a1, c & 31);
        a0 = fma(-Dg[tid][c], yc, a0);
        a1 = fma(-Dg[tid + 32][c], yc, a1);
      }
      if (tid < nr) Vf[r0 + tid] = double(a0);
      if (tid + 32 < nr) Vf[r0 + tid + 32] = double(a1);
      __threadfence();
    }
    __syncthreads();
    if (tid == 0) st_release_u32(tf + t, epoch);
  }
}

template <class T>
__global__ void __launch_bounds__(kSBThreads) sp_bwdb_chain(const SpFrontDev* __restrict__ fr,
                                                            const int32_t* __restrict__ flist, int nf, int npmax,
                                                            const T* __restrict__ F, double* __restrict__ V,
                                                            unsigned* __restrict__ tflag, unsigned epoch,
                                                            int* __restrict__ ctr, int* __restrict__ abort_word,
                                                            int* __restrict__ flags) {
  if (flags[0]) return;
  __shared__ T xs[kSB];
  __shared__ double part[4][kSB];
  __shared__ T Dg[kSB][kSB + 1];
  __shared__ T vs[kSB];
  __shared__ T rd[kSB];
  __shared__ int sync_s[2];
  const int tid = threadIdx.x;
  const int total = npmax * nf;
  for (;;) {
    const int item = sb_claim(ctr, total, abort_word, &sync_s[0]);
    if (item >= total) return;
    const int32_t fid = flist[item % nf];
    const SpFrontDev Fr = fr[fid];
    const int m = Fr.m, p = Fr.p, np = sb_np(p);
    const int t = np - 1 - item / nf;
    if (t < 0) continue;
    const int r0 = t * kSB, r1 = min(r0 + kSB, p), nr = r1 - r0;
    const T* A = F + Fr.off;
    double* Vf = V + Fr.idx;
    unsigned* tf = tflag + sb_flag_base(Fr, fid);
    sb_stage_diag<T>(A, m, r0, nr, false, Dg);
    if (tid < nr) rd[tid] = T(1) / A[(r0 + tid) + int64_t(r0 + tid) * m];
    double v = (tid < kSB && r0 + tid < r1) ? Vf[r0 + tid] : 0.0;
    bool ok = true;
    for (int b = np - 1; b > t && ok; --b) {
      const int c0 = b * kSB, cb = min(kSB, p - c0);
      T a[16];
      sb_chain_load<T>(A, m, r0, r1, c0, cb, a);
      ok = sb_wait(tf + b, epoch, abort_word, flags, &sync_s[1]);
      if (ok) sb_chain_apply<T>(a, cb, Vf + c0, xs, part, v);
    }
    if (!ok) return;
    if (tid < kSB) vs[tid] = T(v);
    __syncthreads();
    if (tid < 32) {
      sb_solve_upper<T>(Dg, rd, vs, nr, r0, Vf);
      __threadfence();
    }
    __syncthreads();
    if (tid == 0) st_release_u32(tf + t, epoch);
  }
}

// backward: x to w
__global__ void sp_bwdb_fin(const SpFrontDev* __restrict__ fr, const int32_t* __restrict__ flist,
                            const double* __restrict__ V, double* __restrict__ w, const int* __restrict__ conv) {
  if (*conv) return;
  const SpFrontDev Fr = fr[flist[blockIdx.y]];
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t < Fr.p) w[Fr.pos0 + t] = V[Fr.idx + t];
}

// ---------------------------------------------------------------- refinement
__global__ void sp_gather_scaled(int64_t n, const int32_t* __restrict__ perm, const double* __restrict__ D,
                                 const double* __restrict__ r, double* __restrict__ w, const int* __restrict__ conv) {
  if (*conv) return;
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int32_t d = perm[k];
  w[k] = D[d] * r[d];
}

__device__ __forceinline__ void max_bits(unsigned long long* dst, double v) {
  // |v| as ordered bits (non-negative doubles order like their bit patterns); NaN wins
  atomicMax(dst, (unsigned long long)__double_as_longlong(isnan(v) ? INFINITY : fabs(v)));
}

__global__ void __launch_bounds__(kThreads) sp_accumulate(int64_t n, int first, const int32_t* __restrict__ perm,
                                                          const double* __restrict__ D, const double* __restrict__ w,
                                                          double* __restrict__ yacc, double* __restrict__ x,
                                                          unsigned long long* __restrict__ nrm,
                                                          const int* __restrict__ conv) {
  if (*conv) return;
  __shared__ double smax[2][kThreads / 32];
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double mw = 0.0, my = 0.0;
  if (k < n) {
    const double z = w[k];
    const double y = first ? z : yacc[k] + z;
    yacc[k] = y;
    const int32_t d = perm[k];
    x[d] = D[d] * y;
    mw = isnan(z) ? INFINITY : fabs(z);
    my = isnan(y) ? INFINITY : fabs(y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mw = fmax(mw, __shfl_xor_sync(0xffffffffu, mw, o));
    my = fmax(my, __shfl_xor_sync(0xffffffffu, my, o));
  }
  if ((threadIdx.x & 31) == 0) {
    smax[0][threadIdx.x >> 5] = mw;
    smax[1][threadIdx.x >> 5] = my;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < kThreads / 32; ++q) {
      mw = fmax(mw, smax[0][q]);
      my = fmax(my, smax[1][q]);
    }
    max_bits(nrm, mw);
    max_bits(nrm + 1, my);
  }
}

// Converged when the scaled correction is below tol of the scaled solution,
// or when it has stopped shrinking (no better than half the previous one)
// while below stall of the solution: the attainable accuracy of the FP64
// residual is then reached.  prev holds the previous correction's norm.
__global__ void sp_check(unsigned long long* nrm, double* prev, int* flags, double tol, double stall) {
  if (flags[0]) return;
  const double nw = __longlong_as_double((long long)nrm[0]), ny = __longlong_as_double((long long)nrm[1]);
  flags[1] += 1;
  if (nw <= tol * ny || (flags[1] > 1 && nw >= 0.5 * *prev && nw <= stall * ny)) flags[0] = 1;
  *prev = nw;
  nrm[0] = 0ull;
  nrm[1] = 0ull;
}

__global__ void __launch_bounds__(kThreads) sp_residual(int64_t n, const int64_t* __restrict__ rptr,
                                                        const int32_t* __restrict__ rq,
                                                        const int32_t* __restrict__ rcol,
                                                        const double* __restrict__ nzval,
                                                        const double* __restrict__ x, const double* __restrict__ b,
                                                        double* __restrict__ r, const int* __restrict__ conv) {
  if (*conv) return;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = b[i];
  for (int64_t t = rptr[i]; t < rptr[i + 1]; ++t) s -= nzval[rq[t]] * x[rcol[t]];
  r[i] = s;
}

template <class T>
cudaError_t upload(T** dst, const std::vector<T>& v) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), std::max<size_t>(v.size(), 1) * sizeof(T));
  if (e != cudaSuccess) return e;
  return v.empty() ? cudaSuccess : cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

template <class T, int NB>
cudaError_t factorise(mgpu_ctx* c, SparseDev& sp, T* F, T tau) {
  cudaStream_t st = c->stream;
  for (int h = 0; h < sp.nheight; ++h) {
    if (sp.h_nlf[h] == 0) continue;
    cudaError_t e = cudaMemsetAsync(F + sp.h_off0[h], 0, (sp.h_off1[h] - sp.h_off0[h]) * sizeof(T), st);
    if (e != cudaSuccess) return e;
    const int64_t na = sp.h_aq0[h + 1] - sp.h_aq0[h];
    if (na > 0) {
      sp_assemble<T><<<nblocks(na, kThreads), kThreads, 0, st>>>(na, sp.d_aq + sp.h_aq0[h], sp.d_amap, sp.d_rowval,
                                                                 sp.d_acol, c->nzval, sp.D, F);
      ++c->launches;
    }
    for (size_t r = 0; r < sp.h_nea[h].size(); ++r) {
      const int cnt = sp.h_nea[h][r];
      for (int f0 = 0; f0 < cnt; f0 += kMaxGridY) {
        const dim3 g(nblocks(sp.h_eumax[h][r], 16), unsigned(std::min(kMaxGridY, cnt - f0)));
        sp_extend_add<T><<<g, kThreads, 0, st>>>(sp.d_fr, sp.d_ea + sp.h_ea0[h][r] + f0, sp.d_emap, F);
        ++c->launches;
      }
    }
    const auto& lp = sp.h_lfp[h];  // pivots of the height's fronts, descending
    if constexpr (std::is_same<T, float>::value) {
      if (sp.super_panels) {
        const int mmax = sp.h_mmax[h];
        for (int s0 = 0; s0 < sp.h_pmax[h]; s0 += kSuper) {
          for (int k0 = s0; k0 < std::min(s0 + kSuper, sp.h_pmax[h]); k0 += NB) {
            int cnt = 0;
            while (cnt < int(lp.size()) && lp[cnt] > k0) ++cnt;
            const int rest = mmax - k0;
            const int nrc = (rest + kThreads - 1) / kThreads, ncc = (rest + 63) / 64;
            for (int f0 = 0; f0 < cnt; f0 += kMaxGridY) {
              const int32_t* fl = sp.d_lf + sp.h_lf0[h] + f0;
              const unsigned gy = unsigned(std::min(kMaxGridY, cnt - f0));
              if (k0 > s0) {
                const int ntr = (rest + kTile32 - 1) / kTile32;
                const int ntc = (rest + kTile32 - 1) / kTile32;  // columns from min(k0 + 64, p)
                if (sp.tensor_cores && sp.tc_left && rest >= kTcMinRest) {
                  sp_rect_tc<<<dim3(unsigned(ntr), gy), tc::kTcThreads, tc::kTcSmem, st>>>(sp.d_fr, fl, 0, s0, k0, 1,
                                                                                          F, sp.flags);
                  sp_rect_tc<<<dim3(unsigned(ntc), gy), tc::kTcThreads, tc::kTcSmem, st>>>(sp.d_fr, fl, 1, s0, k0, ntc,
                                                                                          F, sp.flags);
                } else {
                  sp_rect_f32<<<dim3(unsigned(ntr), gy), kThreads, kUpd32Smem, st>>>(sp.d_fr, fl, 0, s0, k0, 1, F);
                  sp_rect_f32<<<dim3(unsigned(ntc), gy), kThreads, kUpd32Smem, st>>>(sp.d_fr, fl, 1, s0, k0, ntc, F);
                }
                c->launches += 2;
              }
              sp_diag_store<T, NB><<<gy, NB, 0, st>>>(sp.d_fr, fl, k0, F, tau, sp.flags);
              sp_panel_f<T, NB><<<dim3(unsigned(nrc + ncc), gy), kThreads, 0, st>>>(sp.d_fr, fl, k0, F);
              c->launches += 2;
            }
          }
          int cnt = 0;
          while (cnt < int(lp.size()) && lp[cnt] > s0) ++cnt;
          const int nt = (mmax - s0 + kTile32 - 1) / kTile32;
          for (int f0 = 0; f0 < cnt; f0 += kMaxGridY) {
            const int32_t* fl = sp.d_lf + sp.h_lf0[h] + f0;
            const unsigned gy = unsigned(std::min(kMaxGridY, cnt - f0));
            if (sp.tensor_cores && mmax - s0 >= kTcMinRest)
              sp_trail_tc<<<dim3(unsigned(nt * nt), gy), tc::kTcThreads, tc::kTcSmem, st>>>(sp.d_fr, fl, s0, nt, F,
                                                                                          sp.flags);
            else
              sp_rect_f32<<<dim3(unsigned(nt * nt), gy), kThreads, kUpd32Smem, st>>>(sp.d_fr, fl, 2, s0, 0, nt, F);
            ++c->launches;
          }
        }
        continue;
      }
    }
    for (int k0 = 0; k0 < sp.h_pmax[h]; k0 += NB) {
      int cnt = 0;
      while (cnt < int(lp.size()) && lp[cnt] > k0) ++cnt;
      // rows and columns after the pivot block, bounded over the fronts of this step
      const int rest = sp.h_mmax[h] - k0;
      const int nrc = (rest + kThreads - 1) / kThreads, ncc = (rest + 63) / 64;
      const int nt = (rest + kTile - 1) / kTile;
      for (int f0 = 0; f0 < cnt; f0 += kMaxGridY) {
        const int32_t* fl = sp.d_lf + sp.h_lf0[h] + f0;
        const unsigned gy = unsigned(std::min(kMaxGridY, cnt - f0));
        if (nrc + ncc > 0) {
          sp_panel<T, NB><<<dim3(unsigned(nrc + ncc), gy), kThreads, 0, st>>>(sp.d_fr, fl, k0, F, tau, sp.flags);
          ++c->launches;
        }
        if constexpr (std::is_same<T, float>::value) {
          const int nt32 = (rest + kTile32 - 1) / kTile32;
          if (sp.tensor_cores && rest >= kTcMinRest) {
            sp_update_tc<NB><<<dim3(unsigned(nt32 * nt32 + 1), gy), tc::kTcThreads, tc::kTcSmem, st>>>(
                sp.d_fr, fl, k0, F, tau, sp.flags);
            ++c->launches;
          } else {
            sp_update_f32<NB><<<dim3(unsigned(nt32 * nt32 + 1), gy), kThreads, kUpd32Smem, st>>>(sp.d_fr, fl, k0, F,
                                                                                                  tau, sp.flags);
            ++c->launches;
          }
        } else {
          sp_update<T, NB><<<dim3(unsigned(nt * nt + 1), gy), kThreads, 0, st>>>(sp.d_fr, fl, k0, F, tau, sp.flags);
          ++c->launches;
        }
      }
    }
  }
  return cudaGetLastError();
}

// epoch of the next chained launch (never 0, the flags' initial value; on
// wrap-around the flags are cleared)
unsigned next_epoch(SparseDev& sp, cudaStream_t st) {
  if (++sp.epoch == 0) {
    cudaMemsetAsync(sp.tflag, 0, sp.ntflag * sizeof(unsigned), st);
    sp.epoch = 1;
  }
  return sp.epoch;
}

// refinement sweeps with the factors F: x = Lλx⁻¹ b.  Per height, the fronts
// with fewer than sp.big_pivots pivots (the tail of the height's list) take
// the one-block-per-front kernels, the others the blocked ones.
template <class T>
cudaError_t refine(mgpu_ctx* c, SparseDev& sp, const T* F, const double* b, int it0, int it1) {
  cudaStream_t st = c->stream;
  const int64_t n = sp.n;
  const size_t smem = size_t(std::max(sp.max_m_small, 1)) * sizeof(double);
  const int grid = std::is_same<T, float>::value ? sp.chain_grid32 : sp.chain_grid64;
  for (int it = it0; it < it1; ++it) {
    if (sp.chained) {
      const cudaError_t e = cudaMemsetAsync(sp.chain, 0, (2 * size_t(sp.nheight) + 1) * sizeof(int), st);
      if (e != cudaSuccess) return e;
    }
    const double* r = b;
    if (it > 0) {
      sp_residual<<<nblocks(n, kThreads), kThreads, 0, st>>>(n, sp.d_rptr, sp.d_rq, sp.d_rcol, c->nzval, sp.xs, b,
                                                             sp.r, sp.flags);
      ++c->launches;
      r = sp.r;
    }
    sp_gather_scaled<<<nblocks(n, kThreads), kThreads, 0, st>>>(n, sp.d_perm, sp.D, r, sp.w, sp.flags);
    ++c->launches;
    for (int h = 0; h < sp.nheight; ++h) {
      if (!sp.h_nlf[h]) continue;
      const int32_t* fl = sp.d_lf + sp.h_lf0[h];
      const int nbig = sp.h_nbig[h], nsmall = sp.h_nlf[h] - nbig;
      if (nsmall > 0) {
        const int32_t* fs = fl + nbig;
        sp_fwd_tri<T><<<unsigned(nsmall), kTriThreads, smem, st>>>(sp.d_fr, fs, sp.d_clist, sp.d_emap, F, sp.w,
                                                                    sp.cvec, sp.flags);
        ++c->launches;
        const int ur = (sp.h_sumax[h] + kGemvRows - 1) / kGemvRows;
        for (int f0 = 0; f0 < nsmall && ur > 0; f0 += kMaxGridY) {
          sp_fwd_gemv<T><<<dim3(unsigned(ur), unsigned(std::min(kMaxGridY, nsmall - f0))), kGemvRows,
                           size_t(sp.h_spmax[h]) * sizeof(double), st>>>(sp.d_fr, fs + f0, F, sp.w, sp.cvec, sp.flags);
          ++c->launches;
        }
      }
      if (nbig > 0) {
        const unsigned gm = nblocks(sp.h_mmax[h], kThreads);
        sp_fwdb_init<<<dim3(gm, unsigned(nbig)), kThreads, 0, st>>>(sp.d_fr, fl, sp.w, sp.V, sp.flags);
        ++c->launches;
        for (size_t rk = 0; rk < sp.h_nea[h].size(); ++rk) {
          sp_fwdb_ext<<<dim3(nblocks(std::max(sp.h_eumax[h][rk], 1), kThreads), unsigned(nbig)), kThreads, 0, st>>>(
              sp.d_fr, fl, sp.d_clist, sp.d_emap, int(rk), sp.cvec, sp.V, sp.flags);
          ++c->launches;
        }
        if (sp.chained) {
          const int items = sp.h_bnt[h] * nbig;
          sp_fwdb_chain<T><<<unsigned(std::min(items, grid)), kSBThreads, 0, st>>>(
              sp.d_fr, fl, nbig, sp.h_bnt[h], F, sp.V, sp.tflag, next_epoch(sp, st), sp.chain + h,
              sp.chain + 2 * sp.nheight, sp.flags);
          ++c->launches;
        } else {
          sp_fwdb_first<T><<<unsigned(nbig), kSBThreads, 0, st>>>(sp.d_fr, fl, F, sp.V, sp.flags);
          ++c->launches;
          for (int j = 0; j < sp.h_bnp[h]; ++j) {
            const int g = sp.h_bnt[h] - j - 1;
            if (g > 0) {
              sp_fwdb_step<T><<<dim3(unsigned(g), unsigned(nbig)), kSBThreads, 0, st>>>(sp.d_fr, fl, j, F, sp.V,
                                                                                       sp.flags);
              ++c->launches;
            }
          }
        }
        sp_fwdb_fin<<<dim3(gm, unsigned(nbig)), kThreads, 0, st>>>(sp.d_fr, fl, sp.V, sp.w, sp.cvec, sp.flags);
        ++c->launches;
      }
    }
    for (int h = sp.nheight - 1; h >= 0; --h) {
      if (!sp.h_nlf[h]) continue;
      const int32_t* fl = sp.d_lf + sp.h_lf0[h];
      const int nbig = sp.h_nbig[h], nsmall = sp.h_nlf[h] - nbig;
      if (nsmall > 0) {
        const int32_t* fs = fl + nbig;
        const int pr = (sp.h_spmax[h] + kGemvRows - 1) / kGemvRows;
        for (int f0 = 0; f0 < nsmall; f0 += kMaxGridY) {
          sp_bwd_gemv<T><<<dim3(unsigned(pr), unsigned(std::min(kMaxGridY, nsmall - f0))), kGemvRows,
                           size_t(std::max(sp.h_sumax[h], 1)) * sizeof(double), st>>>(sp.d_fr, fs + f0, sp.d_fidx, F,
                                                                                      sp.w, sp.tw, sp.flags);
          ++c->launches;
        }
        sp_bwd_tri<T><<<unsigned(nsmall), kTriThreads, smem, st>>>(sp.d_fr, fs, F, sp.w, sp.tw, sp.flags);
        ++c->launches;
      }
      if (nbig > 0) {
        const unsigned gp = nblocks(sp.h_pmax[h], kThreads);
        sp_bwdb_init<<<dim3(gp, unsigned(nbig)), kThreads, 0, st>>>(sp.d_fr, fl, sp.w, sp.V, sp.flags);
        ++c->launches;
        if (sp.h_bnu[h] > 0) {
          sp_bwdb_u12<T><<<dim3(unsigned(sp.h_bnp[h]), unsigned(sp.h_bnu[h]), unsigned(nbig)), kSBThreads, 0, st>>>(
              sp.d_fr, fl, sp.d_poff, sp.d_fidx, F, sp.w, sp.P, sp.flags);
          sp_bwdb_red<<<dim3(gp, unsigned(nbig)), kThreads, 0, st>>>(sp.d_fr, fl, sp.d_poff, sp.P, sp.V, sp.flags);
          c->launches += 2;
        }
        if (sp.chained) {
          const int items = sp.h_bnp[h] * nbig;
          sp_bwdb_chain<T><<<unsigned(std::min(items, grid)), kSBThreads, 0, st>>>(
              sp.d_fr, fl, nbig, sp.h_bnp[h], F, sp.V, sp.tflag, next_epoch(sp, st), sp.chain + sp.nheight + h,
              sp.chain + 2 * sp.nheight, sp.flags);
          ++c->launches;
        } else {
          sp_bwdb_last<T><<<unsigned(nbig), kSBThreads, 0, st>>>(sp.d_fr, fl, F, sp.V, sp.flags);
          ++c->launches;
          for (int s2 = 0; s2 + 1 < sp.h_bnp[h]; ++s2) {
            sp_bwdb_step<T><<<dim3(unsigned(sp.h_bnp[h]), unsigned(nbig)), kSBThreads, 0, st>>>(sp.d_fr, fl, s2, F,
                                                                                                sp.V, sp.flags);
            ++c->launches;
          }
        }
        sp_bwdb_fin<<<dim3(nblocks(sp.h_pmax[h], kThreads), unsigned(nbig)), kThreads, 0, st>>>(sp.d_fr, fl, sp.V,
                                                                                               sp.w, sp.flags);
        ++c->launches;
      }
    }
    sp_accumulate<<<nblocks(n, kThreads), kThreads, 0, st>>>(n, it == 0, sp.d_perm, sp.D, sp.w, sp.yacc, sp.xs, sp.nrm,
                                                             sp.flags);
    ++c->launches;
    sp_check<<<1, 1, 0, st>>>(sp.nrm, sp.prev, sp.flags, kRefineTol, kRefineStall);
    ++c->launches;
  }
  return cudaGetLastError();
}

// the refinement sweeps in batches: after each batch the host reads the
// convergence flag, so that few sweeps are enqueued after convergence
// (every kernel of a converged sweep returns at once, but is still launched)
template <class T>
cudaError_t refine_batches(mgpu_ctx* c, SparseDev& sp, const T* F, const double* b, int sweeps, int first) {
  int done = 0;
  while (done < sweeps) {
    const int nb_ = done == 0 ? std::min(first, sweeps) : std::min(2, sweeps - done);
    cudaError_t e = refine<T>(c, sp, F, b, done, done + nb_);
    if (e != cudaSuccess) return e;
    done += nb_;
    if (done >= sweeps) break;
    e = cudaMemcpyAsync(sp.hflags, sp.flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return e;
    if (sp.hflags[0] != 0 || sp.hflags[3] != 0) break;
  }
  return cudaSuccess;
}

template <class T>
cudaError_t set_smem(int bytes) {
  for (const void* k : {reinterpret_cast<const void*>(sp_fwd_tri<T>), reinterpret_cast<const void*>(sp_bwd_tri<T>),
                        reinterpret_cast<const void*>(sp_fwd_gemv<T>), reinterpret_cast<const void*>(sp_bwd_gemv<T>)}) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

int sparse_create(mgpu_ctx* c, SparseDev*& spp, const double* dof_xyz, const uint8_t* last) {
  spp = new SparseDev();
  SparseDev& sp = *spp;
  const Pattern& P = c->pat;
  const auto t0 = std::chrono::steady_clock::now();
  SparseInput in;
  in.n = c->nX;
  in.colptr = P.colptr.data();
  in.rowval = P.rowval.data();
  in.xyz = dof_xyz;
  in.last = last;
  in.leaf_groups = 8;
  SparseAnalysis A;
  sp.why = sparse_analyse(in, A);
  if (!sp.why.empty()) return MGPU_OK;
  // the one-block substitutions keep a front's vector in shared memory (fronts
  // with many pivots keep it in global memory)
  sp.big_pivots = kBigPivots;
  if (const char* ev = getenv("MGPU_SPARSE_BLOCKED_PIVOTS")) sp.big_pivots = std::max(1, atoi(ev));
  for (const SparseFront& S : A.fronts)
    if (S.p < sp.big_pivots) sp.max_m_small = std::max(sp.max_m_small, int(S.m));
  if (int64_t(sp.max_m_small) * 8 > 200 * 1024) {
    sp.why = "front of " + std::to_string(sp.max_m_small) + " dofs exceeds the substitution kernels' shared memory";
    return MGPU_OK;
  }
  sp.n = A.n;
  sp.nnz = A.nnz;
  sp.fsize = A.fsize;
  sp.nfront = int(A.fronts.size());
  sp.nheight = A.nheight;
  sp.max_m = A.max_m;
  sp.max_p = A.max_p;
  sp.flops = A.flops;
  const int nf = sp.nfront;
  // fronts, children in rank order
  std::vector<SpFrontDev> fr(nf);
  std::vector<std::vector<int32_t>> kids(nf);
  for (int f = 0; f < nf; ++f)
    if (A.fronts[f].parent >= 0) kids[A.fronts[f].parent].push_back(f);
  std::vector<int32_t> clist;
  for (int f = 0; f < nf; ++f) {
    const SparseFront& S = A.fronts[f];
    std::sort(kids[f].begin(), kids[f].end(), [&](int32_t a, int32_t b) { return A.fronts[a].crank < A.fronts[b].crank; });
    fr[f] = SpFrontDev{S.off, S.idx, S.eoff, S.m, S.p, S.pos0, S.parent, int32_t(clist.size()), int32_t(kids[f].size())};
    clist.insert(clist.end(), kids[f].begin(), kids[f].end());
    if (S.parent < 0) sp.nroot++;
  }
  // fronts by height, pivots descending; storage ranges
  const int H = sp.nheight;
  std::vector<std::vector<int32_t>> byh(H);
  for (int f = 0; f < nf; ++f) byh[A.fronts[f].height].push_back(f);
  std::vector<int32_t> lf;
  sp.h_lf0.resize(H);
  sp.h_nlf.resize(H);
  sp.h_pmax.assign(H, 0);
  sp.h_mmax.assign(H, 0);
  sp.h_umax.assign(H, 0);
  sp.h_off0.assign(H, INT64_MAX);
  sp.h_off1.assign(H, 0);
  sp.h_lfp.resize(H);
  sp.h_nbig.assign(H, 0);
  sp.h_bnp.assign(H, 0);
  sp.h_bnt.assign(H, 0);
  sp.h_spmax.assign(H, 0);
  sp.h_sumax.assign(H, 0);
  sp.h_bnu.assign(H, 0);
  std::vector<int64_t> poff(nf, 0);
  int64_t psize = 0;
  for (int h = 0; h < H; ++h) {
    auto& L = byh[h];
    std::stable_sort(L.begin(), L.end(), [&](int32_t a, int32_t b) { return A.fronts[a].p > A.fronts[b].p; });
    sp.h_lf0[h] = int32_t(lf.size());
    sp.h_nlf[h] = int32_t(L.size());
    for (int32_t f : L) {
      const SparseFront& S = A.fronts[f];
      lf.push_back(f);
      sp.h_lfp[h].push_back(S.p);
      sp.h_pmax[h] = std::max(sp.h_pmax[h], S.p);
      sp.h_mmax[h] = std::max(sp.h_mmax[h], S.m);
      sp.h_umax[h] = std::max(sp.h_umax[h], S.m - S.p);
      sp.h_off0[h] = std::min(sp.h_off0[h], S.off);
      sp.h_off1[h] = std::max(sp.h_off1[h], S.off + int64_t(S.m) * S.m);
      if (S.p >= sp.big_pivots) {  // the prefix of the list (pivots descending)
        const int np = (S.p + kSB - 1) / kSB, nu = (S.m - S.p + kSB - 1) / kSB;
        sp.h_nbig[h]++;
        sp.h_bnp[h] = std::max(sp.h_bnp[h], np);
        sp.h_bnt[h] = std::max(sp.h_bnt[h], np + nu);
        sp.h_bnu[h] = std::max(sp.h_bnu[h], nu);
        poff[f] = psize;
        psize += int64_t(nu) * S.p;
      } else {
        sp.h_spmax[h] = std::max(sp.h_spmax[h], S.p);
        sp.h_sumax[h] = std::max(sp.h_sumax[h], S.m - S.p);
      }
    }
    if (L.empty()) sp.h_off0[h] = sp.h_off1[h] = 0;
  }
  // children to add, by the parent's height and the child's rank
  std::vector<int32_t> ea;
  sp.h_ea0.assign(H, {});
  sp.h_nea.assign(H, {});
  sp.h_eumax.assign(H, {});
  for (int h = 0; h < H; ++h) {
    int maxr = 0;
    for (int32_t f : byh[h]) maxr = std::max<int>(maxr, int(kids[f].size()));
    for (int r = 0; r < maxr; ++r) {
      sp.h_ea0[h].push_back(int32_t(ea.size()));
      int cnt = 0, um = 0;
      for (int32_t f : byh[h])
        if (int(kids[f].size()) > r) {
          const int32_t ch = kids[f][r];
          ea.push_back(ch);
          ++cnt;
          um = std::max(um, A.fronts[ch].m - A.fronts[ch].p);
        }
      sp.h_nea[h].push_back(cnt);
      sp.h_eumax[h].push_back(um);
    }
  }
  // nnz by the height of their front; column of each nnz; rows for the residual
  std::vector<int32_t> fh(nf);
  for (int f = 0; f < nf; ++f) fh[f] = A.fronts[f].height;
  std::vector<int32_t> fpos(A.n);
  for (int f = 0; f < nf; ++f)
    for (int i = 0; i < A.fronts[f].p; ++i) fpos[A.fronts[f].pos0 + i] = f;
  std::vector<int32_t> acol(A.nnz);
  std::vector<int64_t> hcnt(H + 1, 0);
  std::vector<int32_t> qh(A.nnz);
  for (int64_t j = 0; j < A.n; ++j)
    for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
      acol[q] = int32_t(j);
      const int32_t pi = A.ipos[P.rowval[q]], pj = A.ipos[j];
      qh[q] = fh[fpos[std::min(pi, pj)]];
      hcnt[qh[q] + 1]++;
    }
  for (int h = 0; h < H; ++h) hcnt[h + 1] += hcnt[h];
  sp.h_aq0.assign(hcnt.begin(), hcnt.end());
  std::vector<int32_t> aq(A.nnz);
  {
    std::vector<int64_t> fill(hcnt.begin(), hcnt.end() - 1);
    for (int64_t q = 0; q < A.nnz; ++q) aq[fill[qh[q]]++] = int32_t(q);
  }
  std::vector<int64_t> rptr(A.n + 1, 0);
  for (int64_t q = 0; q < A.nnz; ++q) rptr[P.rowval[q] + 1]++;
  for (int64_t i = 0; i < A.n; ++i) rptr[i + 1] += rptr[i];
  std::vector<int32_t> rq(A.nnz), rcol(A.nnz);
  {
    std::vector<int64_t> fill(rptr.begin(), rptr.end() - 1);
    for (int64_t j = 0; j < A.n; ++j)
      for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
        const int64_t t = fill[P.rowval[q]]++;
        rq[t] = int32_t(q);
        rcol[t] = int32_t(j);
      }
  }
  // upload
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
    return e == cudaSuccess;
  };
  ok(upload(&sp.d_fr, fr));
  ok(upload(&sp.d_lf, lf));
  ok(upload(&sp.d_ea, ea));
  ok(upload(&sp.d_clist, clist));
  ok(upload(&sp.d_fidx, A.fidx));
  ok(upload(&sp.d_emap, A.emap));
  ok(upload(&sp.d_amap, A.amap));
  ok(upload(&sp.d_aq, aq));
  ok(upload(&sp.d_acol, acol));
  ok(upload(&sp.d_perm, A.perm));
  ok(upload(&sp.d_diag, A.diag));
  ok(upload(&sp.d_rptr, rptr));
  ok(upload(&sp.d_rq, rq));
  ok(upload(&sp.d_rcol, rcol));
  ok(upload(&sp.d_colptr, P.colptr));
  ok(upload(&sp.d_rowval, P.rowval));
  const int64_t n = A.n;
  ok(cudaMalloc(&sp.F32, std::max<int64_t>(sp.fsize, 1) * sizeof(float)));
  ok(cudaMalloc(&sp.D, 2 * n * sizeof(double)));
  ok(cudaMalloc(&sp.cvec, std::max<size_t>(A.emap.size(), 1) * sizeof(double)));
  ok(cudaMalloc(&sp.w, n * sizeof(double)));
  ok(cudaMalloc(&sp.V, std::max<size_t>(A.fidx.size(), 1) * sizeof(double)));
  ok(cudaMalloc(&sp.P, std::max<int64_t>(psize, 1) * sizeof(double)));
  ok(upload(&sp.d_poff, poff));
  ok(cudaMalloc(&sp.tw, n * sizeof(double)));
  ok(cudaMalloc(&sp.yacc, n * sizeof(double)));
  ok(cudaMalloc(&sp.r, n * sizeof(double)));
  ok(cudaMalloc(&sp.xs, n * sizeof(double)));
  ok(cudaMalloc(&sp.nrm, 2 * sizeof(unsigned long long)));
  ok(cudaMalloc(&sp.prev, sizeof(double)));
  ok(cudaMalloc(&sp.flags, 4 * sizeof(int)));
  ok(cudaMallocHost(&sp.hflags, 4 * sizeof(int)));
  sp.ntflag = int64_t(A.fidx.size()) / 64 + 2 * int64_t(sp.nfront) + 64;
  ok(cudaMalloc(&sp.tflag, sp.ntflag * sizeof(unsigned)));
  ok(cudaMemset(sp.tflag, 0, sp.ntflag * sizeof(unsigned)));
  ok(cudaMalloc(&sp.chain, (2 * size_t(sp.nheight) + 1) * sizeof(int)));
  {
    int dev = 0, nsm = 0, b32 = 0, b64 = 0, f32 = 0, f64 = 0;
    ok(cudaGetDevice(&dev));
    ok(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f32, sp_fwdb_chain<float>, kSBThreads, 0));
    ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b32, sp_bwdb_chain<float>, kSBThreads, 0));
    ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f64, sp_fwdb_chain<double>, kSBThreads, 0));
    ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b64, sp_bwdb_chain<double>, kSBThreads, 0));
    sp.chain_grid32 = std::max(1, nsm * std::max(1, std::min(f32, b32)));
    sp.chain_grid64 = std::max(1, nsm * std::max(1, std::min(f64, b64)));
  }
  if (const char* ev = getenv("MGPU_SPARSE_CHAINED")) sp.chained = atoi(ev) != 0;
  ok(cudaMemset(sp.nrm, 0, 2 * sizeof(unsigned long long)));
  for (cudaEvent_t& ev : sp.ev) ok(cudaEventCreate(&ev));
  const int smem = int(sp.max_m_small * sizeof(double));
  if (smem > 48 * 1024) {
    ok(set_smem<float>(smem));
    ok(set_smem<double>(smem));
  }
  ok(cudaFuncSetAttribute(sp_update_f32<kNB32>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kUpd32Smem)));
  ok(cudaFuncSetAttribute(sp_update_tc<kNB32>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc::kTcSmem)));
  ok(cudaFuncSetAttribute(sp_rect_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kUpd32Smem)));
  ok(cudaFuncSetAttribute(sp_trail_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc::kTcSmem)));
  ok(cudaFuncSetAttribute(sp_rect_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc::kTcSmem)));
  if (const char* ev = getenv("MGPU_SPARSE_TC_LEFT")) sp.tc_left = atoi(ev) != 0;
  if (const char* ev = getenv("MGPU_SPARSE_SUPER")) sp.super_panels = atoi(ev) != 0;
  if (const char* ev = getenv("MGPU_SPARSE_TC")) sp.tensor_cores = atoi(ev) != 0;
  if (e != cudaSuccess) {
    sp.why = std::string("device upload of the sparse solver: ") + cudaGetErrorString(e);
    return set_err(c, e == cudaErrorMemoryAllocation ? MGPU_ERR_NOMEM : MGPU_ERR_CUDA, sp.why);
  }
  if (getenv("MGPU_VERBOSE")) {
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    fprintf(stderr,
            "[muscade_gpu] sparse solver: %d groups, %d fronts, %d heights, largest front %d (%d pivots), "
            "%.3g G front entries, %.3g TFLOP per factorisation, analysis %.2f s\n",
            A.ngroups, nf, H, A.max_m, A.max_p, double(sp.fsize) / 1e9, sp.flops / 1e12, s);
  }
  return MGPU_OK;
}

void sparse_destroy(SparseDev*& sp) {
  if (!sp) return;
  void* ps[] = {sp->d_fr, sp->d_lf, sp->d_ea, sp->d_clist, sp->d_fidx, sp->d_emap, sp->d_amap, sp->d_aq,
                sp->d_acol, sp->d_perm, sp->d_diag, sp->d_colptr, sp->d_rowval, sp->d_rptr, sp->d_rq, sp->d_rcol,
                sp->F32, sp->F64, sp->prev,
                sp->D, sp->cvec, sp->w, sp->V, sp->P, sp->d_poff, sp->tw, sp->yacc, sp->r, sp->xs, sp->nrm,
                sp->flags, sp->tflag, sp->chain};
  for (void* p : ps) cudaFree(p);
  if (sp->hflags) cudaFreeHost(sp->hflags);
  for (cudaEvent_t ev : sp->ev)
    if (ev) cudaEventDestroy(ev);
  delete sp;
  sp = nullptr;
}

int sparse_factor_solve(mgpu_ctx* c, SparseDev& sp, const double* rhs, double* out, int* info) {
  cudaStream_t st = c->stream;
  const int64_t n = sp.n;
  // equilibration from the current values
  sp_scale_diag<<<nblocks(n, kThreads), kThreads, 0, st>>>(n, sp.d_diag, c->nzval, sp.D + n);
  ++c->launches;
  sp_scale_zero<<<nblocks(n, kThreads), kThreads, 0, st>>>(n, sp.d_colptr, sp.d_rowval, c->nzval, sp.D + n,
                                                           sp.D);
  ++c->launches;
  MG_CUDA(cudaMemsetAsync(sp.flags, 0, 4 * sizeof(int), st));
  bool use64 = sp.fp64_only;
  sp.last_factor_ms = sp.last_refine_ms = 0.0;
  auto elapsed = [&](int a, int b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, sp.ev[a], sp.ev[b]);
    return double(ms);
  };
  if (!use64) {
    MG_CUDA(cudaEventRecord(sp.ev[0], st));
    MG_CUDA((factorise<float, kNB32>(c, sp, sp.F32, 1e-10f)));
    MG_CUDA(cudaEventRecord(sp.ev[1], st));
    MG_CUDA(refine_batches<float>(c, sp, sp.F32, rhs, kSparseSweeps, 8));
    MG_CUDA(cudaEventRecord(sp.ev[2], st));
    MG_CUDA(cudaMemcpyAsync(sp.hflags, sp.flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CUDA(cudaStreamSynchronize(st));
    sp.last_factor_ms = elapsed(0, 1);
    sp.last_refine_ms = elapsed(1, 2);
    sp.last_sweeps = sp.hflags[1];
    sp.last_perturbed = sp.hflags[2];
    if (sp.hflags[3] & 6) return set_err(c, MGPU_ERR_CUDA, "sparse solve: a bounded wait on the device ran out");
    sp.last_fallback = 0;
    if (sp.hflags[0] == 0 || sp.hflags[3] != 0) {
      use64 = true;
      sp.last_fallback = 1;
      if (sp.adaptive) sp.fp64_only = true;
    }
  }
  if (use64) {
    if (!sp.F64) {
      cudaError_t e = cudaMalloc(&sp.F64, std::max<int64_t>(sp.fsize, 1) * sizeof(double));
      if (e != cudaSuccess) {
        sp.F64 = nullptr;
        return set_err(c, MGPU_ERR_NOMEM, std::string("FP64 factors of the sparse solver: ") + cudaGetErrorString(e));
      }
    }
    MG_CUDA(cudaMemsetAsync(sp.flags, 0, 4 * sizeof(int), st));
    MG_CUDA(cudaEventRecord(sp.ev[0], st));
    MG_CUDA((factorise<double, kNB64>(c, sp, sp.F64, 0.0)));
    MG_CUDA(cudaEventRecord(sp.ev[1], st));
    MG_CUDA(refine_batches<double>(c, sp, sp.F64, rhs, kSparseSweeps64, 4));
    MG_CUDA(cudaEventRecord(sp.ev[2], st));
    MG_CUDA(cudaMemcpyAsync(sp.hflags, sp.flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CUDA(cudaStreamSynchronize(st));
    sp.last_factor_ms += elapsed(0, 1);
    sp.last_refine_ms += elapsed(1, 2);
    sp.last_sweeps = sp.hflags[1];
    sp.last_perturbed = sp.hflags[2];
    if (sp.hflags[3] & 6) return set_err(c, MGPU_ERR_CUDA, "sparse solve: a bounded wait on the device ran out");
    if (sp.hflags[3] != 0) {  // a zero or non-finite pivot in FP64: the matrix is singular
      const int one = 1;
      MG_CUDA(cudaMemcpy(info, &one, sizeof(int), cudaMemcpyHostToDevice));
    }
  }
  MG_CUDA(cudaMemcpyAsync(out, sp.xs, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  return MGPU_OK;
}

}  // namespace mgpu

// C[M×N] −= A[M×K] B[K×N] (column-major host arrays, K ≤ 64) on the tensor cores
extern "C" int mgpu_tc_gemm_check(int32_t device, int32_t M, int32_t N, int32_t K, const float* A, const float* B,
                                  float* C) {
  using namespace mgpu;
  if (M <= 0 || N <= 0 || K <= 0 || K > 4096 || !A || !B || !C) return MGPU_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MGPU_ERR_CUDA;
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int* derr = nullptr;
  int herr = 0, rc = MGPU_OK;
  const size_t na = size_t(M) * K, nb = size_t(K) * N, nc = size_t(M) * N;
  if (cudaMalloc(&dA, na * 4) != cudaSuccess || cudaMalloc(&dB, nb * 4) != cudaSuccess ||
      cudaMalloc(&dC, nc * 4) != cudaSuccess || cudaMalloc(&derr, sizeof(int)) != cudaSuccess) {
    rc = MGPU_ERR_NOMEM;
  } else if (cudaMemcpy(dA, A, na * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(dB, B, nb * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(dC, C, nc * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemset(derr, 0, sizeof(int)) != cudaSuccess ||
             cudaFuncSetAttribute(tc_gemm_check, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc::kTcSmem)) !=
                 cudaSuccess) {
    rc = MGPU_ERR_CUDA;
  } else {
    const dim3 g((M + tc::kTcTile - 1) / tc::kTcTile, (N + tc::kTcTile - 1) / tc::kTcTile);
    tc_gemm_check<<<g, tc::kTcThreads, tc::kTcSmem>>>(dA, M, dB, K, dC, M, M, N, K, derr);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(C, dC, nc * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = MGPU_ERR_CUDA;
    else if (herr)
      rc = MGPU_ERR_CUDA;
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(derr);
  return rc;
}
