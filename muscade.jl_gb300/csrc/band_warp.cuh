// Banded LU with partial pivoting and its solve, one warp per connected
// component, for bands with kl ≤ 31 and kl+ku+1 ≤ 64 (beam chains, risers,
// frames).  Same algorithm and operation order as band_lu/band_solve
// (LAPACK gbtf2/gbtrs): pivot = first largest |a| in rows k..k+kl, row swap
// over the window, multipliers scaled by 1/pivot, rank-1 update.
//
// The active part of the factorisation lives in registers: the window of
// columns k..k+kl+ku, each held by one (lane, slot) pair, with the rows
// k..k+kl of each column in a per-lane array.  A column step is a local pivot
// search by the lane that holds column k, broadcasts by warp shuffles and a
// register update; no block barriers and no global round trips on the
// critical path.  Finished U rows and L columns stream out to the band
// storage, new rows and columns stream in.
#pragma once
#include <cuda_runtime.h>

namespace mgpu {

constexpr int BW_ROWS = 32;  // kl + 1 ≤ 32
constexpr int BW_SLOTS = 2;  // window kl+ku+1 ≤ 64 columns, two per lane

// a[idx] read/write with a run-time index over a register array (unrolled selects)
template <int N>
__device__ __forceinline__ double rsel(const double (&a)[N], int idx) {
  double v = 0.0;
#pragma unroll
  for (int r = 0; r < N; ++r) v = (r == idx) ? a[r] : v;
  return v;
}
template <int N>
__device__ __forceinline__ void rset(double (&a)[N], int idx, double v) {
#pragma unroll
  for (int r = 0; r < N; ++r) a[r] = (r == idx) ? v : a[r];
}

__global__ void __launch_bounds__(128) band_lu_warp(int ncomp, const int64_t* __restrict__ cbase,
                                                    const int32_t* __restrict__ cn, const int32_t* __restrict__ ckl,
                                                    const int32_t* __restrict__ cku,
                                                    const int32_t* __restrict__ cdof0, double* __restrict__ AB,
                                                    int32_t* __restrict__ ipiv, int* __restrict__ info) {
  const unsigned FULL = 0xffffffffu;
  const int cc = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (cc >= ncomp) return;  // the whole warp leaves together
  const int n = cn[cc], kl = ckl[cc], ku = cku[cc];
  const int kv = kl + ku, ld = 2 * kl + ku + 1, W = kv + 1;
  double* A = AB + cbase[cc];
  int32_t* piv = ipiv + cdof0[cc];
  double act[BW_SLOTS][BW_ROWS];
  int col[BW_SLOTS];
  // window position q = j mod W; position q is lane q&31, slot q>>5
#pragma unroll
  for (int s = 0; s < BW_SLOTS; ++s) {
    const int q = lane + 32 * s;
    const int j = (q < W && q < n) ? q : -1;
    col[s] = j;
#pragma unroll
    for (int r = 0; r < BW_ROWS; ++r) act[s][r] = (j >= 0 && r <= kl && r < n) ? A[kv + r - j + int64_t(ld) * j] : 0.0;
  }
  int q0 = 0;  // window position of column k
  for (int k = 0; k < n; ++k) {
    const int km = min(kl, n - 1 - k);
    const int olane = q0 & 31, oslot = q0 >> 5;
    // prefetch what enters the window after this step (untouched until then):
    // row k+1+kl of the other window columns, and column k+W for the owner of column k
    const int rn = k + 1 + kl, jn = k + W;
    double nrow[BW_SLOTS], ncol[BW_ROWS];
#pragma unroll
    for (int s = 0; s < BW_SLOTS; ++s) {
      const int j = col[s];
      nrow[s] = (j > k && rn < n) ? A[kv + rn - j + int64_t(ld) * j] : 0.0;
    }
    const bool owner = (lane == olane);
#pragma unroll
    for (int r = 0; r < BW_ROWS; ++r)
      ncol[r] = (owner && jn < n && r <= kl && k + 1 + r < n) ? A[kv + (k + 1 + r) - jn + int64_t(ld) * jn] : 0.0;
    // pivot search by the owner of column k
    int jp = 0;
    if (lane == olane) {
      double best = -1.0;
#pragma unroll
      for (int r = 0; r < BW_ROWS; ++r) {
        const double v = fabs(oslot == 0 ? act[0][r] : act[1][r]);
        if (r <= km && v > best) {
          best = v;
          jp = r;
        }
      }
    }
    jp = __shfl_sync(FULL, jp, olane);
    // swap rows k and k+jp in every window column
    if (jp != 0) {
#pragma unroll
      for (int s = 0; s < BW_SLOTS; ++s)
        if (col[s] >= k) {
          const double a0 = act[s][0], ap = rsel(act[s], jp);
          act[s][0] = ap;
          rset(act[s], jp, a0);
        }
    }
    const double pv = __shfl_sync(FULL, oslot == 0 ? act[0][0] : act[1][0], olane);
    if (lane == olane) piv[k] = k + jp;
    if (pv == 0.0) {
      if (lane == 0) atomicCAS(info, 0, cc + 1);
    } else {
      const double rp = 1.0 / pv;
      if (lane == olane) {
#pragma unroll
        for (int r = 1; r < BW_ROWS; ++r) {
          if (r <= km) {
            if (oslot == 0)
              act[0][r] *= rp;
            else
              act[1][r] *= rp;
          }
        }
      }
      // rank-1 update: multipliers broadcast one row at a time
      double u[BW_SLOTS];
#pragma unroll
      for (int s = 0; s < BW_SLOTS; ++s) u[s] = (col[s] > k) ? act[s][0] : 0.0;
#pragma unroll
      for (int r = 1; r < BW_ROWS; ++r) {
        if (r <= km) {  // uniform across the warp
          const double l = __shfl_sync(FULL, oslot == 0 ? act[0][r] : act[1][r], olane);
#pragma unroll
          for (int s = 0; s < BW_SLOTS; ++s)
            if (col[s] > k && u[s] != 0.0) act[s][r] -= l * u[s];
        }
      }
    }
    // write out: column k (U diagonal and L multipliers), row k of the others (U)
#pragma unroll
    for (int s = 0; s < BW_SLOTS; ++s) {
      const int j = col[s];
      if (j == k) {
#pragma unroll
        for (int r = 0; r < BW_ROWS; ++r)
          if (r <= km) A[kv + r + int64_t(ld) * k] = act[s][r];
      } else if (j > k) {
        A[kv + k - j + int64_t(ld) * j] = act[s][0];
      }
    }
    // advance the window to step k+1
#pragma unroll
    for (int s = 0; s < BW_SLOTS; ++s) {
      const int j = col[s];
      if (j == k) {
        if (jn < n) {
          col[s] = jn;
#pragma unroll
          for (int r = 0; r < BW_ROWS; ++r) act[s][r] = ncol[r];
        } else {
          col[s] = -1;
        }
      } else if (j > k) {
        const double nv = nrow[s];  // row k+1+kl entering the active set
#pragma unroll
        for (int r = 0; r < BW_ROWS - 1; ++r) act[s][r] = (r == kl) ? nv : act[s][r + 1];
        act[s][BW_ROWS - 1] = (BW_ROWS - 1 == kl) ? nv : 0.0;
      }
    }
    q0 = (q0 + 1 == W) ? 0 : q0 + 1;
  }
}

// Forward (L with the interchanges) and backward (U, kl+ku superdiagonals)
// substitution, one warp per component, sliding windows of the right-hand side
// held one entry per lane (two slots for the backward window).
__global__ void __launch_bounds__(128) band_solve_warp(int ncomp, const int64_t* __restrict__ cbase,
                                                       const int32_t* __restrict__ cn, const int32_t* __restrict__ ckl,
                                                       const int32_t* __restrict__ cku,
                                                       const int32_t* __restrict__ cdof0,
                                                       const int32_t* __restrict__ perm, const double* __restrict__ AB,
                                                       const int32_t* __restrict__ ipiv, const double* __restrict__ Ll,
                                                       double* __restrict__ rhs, double* __restrict__ dx) {
  const unsigned FULL = 0xffffffffu;
  const int cc = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (cc >= ncomp) return;
  const int n = cn[cc], kl = ckl[cc], ku = cku[cc];
  const int kv = kl + ku, ld = 2 * kl + ku + 1;
  const double* A = AB + cbase[cc];
  const int32_t* piv = ipiv + cdof0[cc];
  const int32_t* pm = perm + cdof0[cc];
  double* b = rhs + cdof0[cc];
  for (int k = lane; k < n; k += 32) b[k] = Ll[pm[k]];
  __syncwarp();
  // forward: lane l holds y[k+l], l ≤ kl
  double y = (lane <= kl && lane < n) ? b[lane] : 0.0;
  for (int k = 0; k < n; ++k) {
    const int km = min(kl, n - 1 - k);
    const int rn = k + 1 + kl;
    const double bnew = (lane == kl && rn < n) ? b[rn] : 0.0;  // prefetch the entering entry
    const double lk = (lane >= 1 && lane <= km) ? A[kv + lane + int64_t(ld) * k] : 0.0;
    const int jp = piv[k] - k;
    if (jp != 0) {
      const double y0 = __shfl_sync(FULL, y, 0);
      const double yj = __shfl_sync(FULL, y, jp);
      if (lane == 0) y = yj;
      if (lane == jp) y = y0;
    }
    const double bk = __shfl_sync(FULL, y, 0);
    if (lane >= 1 && lane <= km) y -= lk * bk;
    if (lane == 0) b[k] = y;  // final forward value
    const double nxt = __shfl_down_sync(FULL, y, 1);
    y = (lane == kl) ? bnew : ((lane < kl) ? nxt : 0.0);
  }
  __syncwarp();
  // backward: position p = lane + 32 s holds y[k-p], p ≤ kv
  double z[BW_SLOTS];
#pragma unroll
  for (int s = 0; s < BW_SLOTS; ++s) {
    const int p = lane + 32 * s;
    const int i = n - 1 - p;
    z[s] = (p <= kv && i >= 0) ? b[i] : 0.0;
  }
  for (int k = n - 1; k >= 0; --k) {
    // loads of this step issued before the dependent arithmetic
    const int inew = k - 1 - kv;
    const double vnew = (inew >= 0 && lane == (kv & 31)) ? b[inew] : 0.0;
    const double d = A[kv + int64_t(ld) * k];
    double uk[BW_SLOTS];
#pragma unroll
    for (int s = 0; s < BW_SLOTS; ++s) {
      const int p = lane + 32 * s;
      uk[s] = (p >= 1 && p <= kv && p <= k) ? A[kv - p + int64_t(ld) * k] : 0.0;
    }
    const double xk = __shfl_sync(FULL, z[0], 0) / d;
    if (lane == 0) b[k] = xk;
#pragma unroll
    for (int s = 0; s < BW_SLOTS; ++s) {
      const int p = lane + 32 * s;
      if (p >= 1 && p <= kv && p <= k) z[s] -= uk[s] * xk;
    }
    // shift the window by one position: p <- p+1, new entry y[k-1-kv] at p = kv
    const double carry = __shfl_sync(FULL, z[1], 0);
    const double d0 = __shfl_down_sync(FULL, z[0], 1);
    const double d1 = __shfl_down_sync(FULL, z[1], 1);
#pragma unroll
    for (int s = 0; s < BW_SLOTS; ++s) {
      const int p = lane + 32 * s;
      double v = (s == 0) ? (lane == 31 ? carry : d0) : (lane == 31 ? 0.0 : d1);
      if (p == kv) v = vnew;
      if (p > kv) v = 0.0;
      z[s] = v;
    }
  }
  __syncwarp();
  for (int k = lane; k < n; k += 32) dx[pm[k]] = b[k];
}

}  // namespace mgpu
