// Banded LU with partial pivoting and its solves, one warp per connected
// component, in a layout built for GB300: factor type T = float (with FP64
// iterative refinement of the solution) or double.
//
// GB300 issues FP64 at 1/64 of the FP32 rate per SM sub-partition, so a warp
// that factorises in FP64 is bound by the number of FP64 *instructions* it
// issues, and one that factorises in FP32 by instruction latency.  Both favour
// a layout where one FMA instruction updates one whole column of the active
// submatrix:
//
//  * lane r holds one active row of the window (columns k..k+kv, kv = kl+ku) in
//    registers; the rank-1 update is kv FMAs per lane per column;
//  * the pivot search is an integer warp reduction on the bits of |a| (no
//    floating-point compares), ties to the first row like LAPACK's idamax;
//  * rows are not moved by an interchange: each lane keeps the position of its
//    row in the pivoted order;
//  * the incoming row is prefetched two columns ahead, spread over the lanes,
//    and handed to the lane whose row just became a U row.
//
// The arithmetic is that of LAPACK gbtf2/gbtrs in the same order (reciprocal
// pivot scaling of the multipliers, a - l*u updates, interchanges applied to
// the right-hand side as the forward substitution meets them), except that the
// backward substitution multiplies by the reciprocal pivot the factorisation
// computed instead of dividing by the pivot: an FP64 division is a chain of
// about ten dependent FP64 instructions, on the critical path of every column.
// With T = double the factors and the solution are bitwise those of the block
// kernels in solver.cu, which do the same.
//
// Storage per component (offsets rbase, lbase, dof0 from the host analysis):
//   A  (FP64, unfactorised rows)  A[i*w + (j - i + kl)],   w = kv + 1
//   UC (T, U by columns)          UC[j*w + p] = U(j-p, j), p = 1..kv;  UC[j*w] = 1/U(j,j)
//   LM (T, multipliers)           LM[k*kl + p - 1] = L(k+p, k), p = 1..kl
//   piv                           row k was interchanged with row piv[k]
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace mgpu {

constexpr unsigned RB_FULL = 0xffffffffu;

// position in the pivoted order of the first largest |v| among candidate lanes;
// *plane = the lane that holds it
__device__ __forceinline__ int rb_argmax(double v, bool cand, int pos, int* plane) {
  unsigned hi = 0u, lo = 0u;
  if (cand) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7fffffffffffffffull;
    hi = static_cast<unsigned>(b >> 32) + 1u;  // 0 is reserved for non-candidates
    lo = static_cast<unsigned>(b);
  }
  const unsigned mh = __reduce_max_sync(RB_FULL, hi);
  const bool in1 = cand && hi == mh;
  const unsigned ml = __reduce_max_sync(RB_FULL, in1 ? lo : 0u);
  const bool in2 = in1 && lo == ml;
  const unsigned jp = __reduce_min_sync(RB_FULL, in2 ? static_cast<unsigned>(pos) : 0xffffffffu);
  *plane = __ffs(__ballot_sync(RB_FULL, in2 && static_cast<unsigned>(pos) == jp)) - 1;
  return static_cast<int>(jp);
}
__device__ __forceinline__ int rb_argmax(float v, bool cand, int pos, int* plane) {
  const unsigned key = cand ? (__float_as_uint(v) & 0x7fffffffu) + 1u : 0u;
  const unsigned mk = __reduce_max_sync(RB_FULL, key);
  const bool in = cand && key == mk;
  const unsigned jp = __reduce_min_sync(RB_FULL, in ? static_cast<unsigned>(pos) : 0xffffffffu);
  *plane = __ffs(__ballot_sync(RB_FULL, in && static_cast<unsigned>(pos) == jp)) - 1;
  return static_cast<int>(jp);
}

__device__ __forceinline__ void rb_cp_async(void* smem, const void* gmem, int bytes) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void rb_cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void rb_cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// What a launch does with the per-component flag array:
enum RbMode : int {
  RB_PRIMARY = 0,   // all components; a zero pivot or a failed refinement sets flag[c]
  RB_FALLBACK = 1,  // only components with flag[c] != 0; a zero pivot is an error (info)
  RB_PLAIN = 2      // all components; a zero pivot is an error (info)
};

struct RbComp {
  const int64_t* rbase;  // [ncomp] offset of the component in A and UC
  const int64_t* lbase;  // [ncomp] offset in LM
  const int32_t* cn;     // [ncomp] size
  const int32_t* ckl;    // [ncomp]
  const int32_t* cku;    // [ncomp]
  const int32_t* cdof0;  // [ncomp] offset in perm / piv / vectors
  const int32_t* list = nullptr;  // components of this launch (block b does list[b]); nullptr: block b does b
};

// ---------------------------------------------------------------- factorisation
// One warp (block of 32) per component; requires kl <= 31 and kv + 1 <= WM.
// Arows: the unfactorised rows in T (an FP32 copy for T = float).  The rows
// that enter the window stream through shared memory in chunks of 32 rows
// (cp.async, double buffered): a register prefetch would not help, because a
// warp-wide instruction that reads a register with a load in flight in any
// lane waits for that load.
template <typename T, int WM>
__global__ void __launch_bounds__(32) rb_lu(RbComp cp, const T* __restrict__ Arows, T* __restrict__ UC,
                                           T* __restrict__ LM, int32_t* __restrict__ ipiv, int mode,
                                           int* __restrict__ flag, int* __restrict__ info) {
  __shared__ __align__(16) T sR[2][32 * WM];
  const int cc = cp.list ? cp.list[blockIdx.x] : int(blockIdx.x), lane = threadIdx.x;
  if (mode == RB_FALLBACK && flag[cc] == 0) return;
  const int n = cp.cn[cc], kl = cp.ckl[cc], kv = kl + cp.cku[cc], w = kv + 1;
  const T* Ac = Arows + cp.rbase[cc];
  T* U = UC + cp.rbase[cc];
  T* L = LM + cp.lbase[cc];
  int32_t* piv = ipiv + cp.cdof0[cc];
  auto issue = [&](int ch) {  // rows [32 ch, 32 ch + 32) of the component into buffer ch & 1
    const int r0 = ch * 32, r1 = min(n, r0 + 32);
    T* dst = sR[ch & 1];
    for (int e = lane; e < (r1 - r0) * w; e += 32) rb_cp_async(dst + e, Ac + int64_t(r0) * w + e, sizeof(T));
  };
  issue((kl + 1) >> 5);  // chunk of the first row that enters (row kl + 1)
  rb_cp_commit();
  T a[WM];
  int pos = (lane <= kl) ? lane : (1 << 30);  // lanes above kl never hold a row
#pragma unroll
  for (int j = 0; j < WM; ++j) {
    const int c = j - lane + kl;  // column j of row `lane` in its storage row
    a[j] = (lane <= kl && lane < n && j <= kv && c <= kv) ? Ac[int64_t(lane) * w + c] : T(0);
  }
  bool singular = false;
  for (int k = 0; k < n; ++k) {
    const int km = min(kl, n - 1 - k);
    const int rn = k + 1 + kl;  // row that enters after this column
    if (rn < n && (k == 0 || (rn & 31) == 0)) {
      __syncwarp();          // every lane is done reading the buffer about to be refilled
      issue((rn >> 5) + 1);  // into the buffer of the chunk just used up
      rb_cp_commit();
      rb_cp_wait<1>();  // chunk rn >> 5 has landed
      __syncwarp();
    }
    int pl;
    const int jp = rb_argmax(a[0], pos <= km, pos, &pl);
    const T pv = __shfl_sync(RB_FULL, a[0], pl);
    if (lane == 0) piv[k] = k + jp;
    if (lane == pl)
      pos = 0;
    else if (pos == 0)
      pos = jp;
    const bool zero = (pv == T(0));
    singular = singular || zero;
    T rp = T(0);  // correctly rounded 1/pv (the value of T(1)/pv, without the general division)
    if (!zero) {
      if constexpr (sizeof(T) == 8)
        rp = __drcp_rn(pv);
      else
        rp = __frcp_rn(pv);
    }
    const bool act = !zero && pos >= 1 && pos <= km;
    const T l = act ? a[0] * rp : a[0];
    if (pos >= 1 && pos <= km) L[int64_t(k) * kl + pos - 1] = l;
    const T le = act ? l : T(0);  // rows outside the update subtract 0*u: no branch per column entry
    // U row k (the pivot row) goes out by columns; rank-1 update of the other rows
    constexpr int NS = (WM + 31) / 32;
    T cap[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) cap[s] = T(0);
#pragma unroll
    for (int j = 1; j < WM; ++j) {
      if (j > kv) break;  // uniform: jump past the columns beyond the band instead of predicating them
      const T u = __shfl_sync(RB_FULL, a[j], pl);
      if ((j & 31) == lane) cap[j >> 5] = u;
      a[j] = fma(-le, u, a[j]);
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const int j = lane + 32 * s;
      if (j <= kv && k + j < n) U[int64_t(k + j) * w + j] = (j == 0) ? rp : cap[s];  // 1/pivot on the diagonal
    }
    // advance to column k+1: drop column k, the pivot lane takes row rn
    const bool me = (lane == pl);
    const T* row = sR[(rn >> 5) & 1] + (rn & 31) * w;
#pragma unroll
    for (int j = 0; j < WM; ++j) {
      const T nv = (rn < n && j <= kv) ? row[j] : T(0);
      const T sh = (j + 1 < WM) ? a[j + 1] : T(0);
      a[j] = me ? nv : sh;
    }
    pos = me ? kl : pos - 1;
  }
  rb_cp_wait<0>();
  if (singular && lane == 0) {
    if (mode == RB_PRIMARY)
      flag[cc] = 1;
    else if (info)
      atomicCAS(info, 0, cc + 1);
  }
}

// ---------------------------------------------------------------- substitution
// Shared memory of one solve block: the forward chunks (L) and the backward
// chunks (U) are used one after the other and share the buffer.
template <typename T, int WM>
struct RbSmem {
  static constexpr int kL = 2 * 32 * 31, kU = 2 * 32 * WM;
  static constexpr int bytes = (kL > kU ? kL : kU) * int(sizeof(T));
};

// t = (LU)^-1 P in for one component, by one warp.  `in` is FP64 (the
// right-hand side or a residual), `t` receives the result in T.  L and U
// stream through shared memory in chunks of 32 columns (cp.async, double
// buffered).  The vector entries ride in circular register windows; the lane
// that finishes entry k refills its slot with entry k+32 (forward) or k-WM
// (backward), and since each lane refills once per chunk, those values and
// the pivots are loaded a whole chunk ahead into registers no per-column
// instruction reads.
template <typename T, int WM>
__device__ void rb_fb(int n, int kl, int kv, int w, const T* __restrict__ U, const T* __restrict__ L,
                      const int32_t* __restrict__ piv, const double* __restrict__ in, T* __restrict__ t,
                      unsigned char* smem, int lane) {
  constexpr int NS = WM / 32, M = WM;  // backward window modulus (a power of two, >= kv + 1)
  T* sL = reinterpret_cast<T*>(smem);
  T* sU = reinterpret_cast<T*>(smem);
  const int nch = (n + 31) >> 5;
  // ---- forward: entry k' lives on lane k' & 31; window k..k+kl
  auto load_fchunk = [&](int c) {
    const int k0 = c * 32, k1 = min(n, k0 + 32);
    T* dl = sL + (c & 1) * (32 * 31);
    for (int e = lane; e < (k1 - k0) * kl; e += 32) rb_cp_async(dl + e, L + int64_t(k0) * kl + e, sizeof(T));
  };
  load_fchunk(0);
  rb_cp_commit();
  T y = (lane < n) ? T(in[lane]) : T(0);
  T nxt = (32 + lane < n) ? T(in[32 + lane]) : T(0);     // refill of this lane in chunk 0
  double inx = (64 + lane < n) ? in[64 + lane] : 0.0;    // refill in chunk 1
  int pk = (lane < n) ? piv[lane] : lane;                // pivots of chunk 0
  int pkn = (32 + lane < n) ? piv[32 + lane] : 32 + lane;  // pivots of chunk 1
  for (int c = 0; c < nch; ++c) {
    if (c + 1 < nch) load_fchunk(c + 1);
    rb_cp_commit();
    const int k0 = c * 32, k1 = min(n, k0 + 32);
    if (c > 0) {
      nxt = T(inx);
      pk = pkn;
      const int e = 32 * (c + 2) + lane, f = 32 * (c + 1) + lane;
      inx = (e < n) ? in[e] : 0.0;
      pkn = (f < n) ? piv[f] : f;
    }
    const unsigned swaps = __ballot_sync(RB_FULL, pk != k0 + lane);
    rb_cp_wait<1>();
    __syncwarp();
    const T* cl = sL + (c & 1) * (32 * 31);
    for (int k = k0; k < k1; ++k) {
      const int km = min(kl, n - 1 - k);
      const int p = (lane - k) & 31;
      const T lk = (p >= 1 && p <= km) ? cl[(k - k0) * kl + p - 1] : T(0);
      if ((swaps >> (k - k0)) & 1u) {
        const int jp = __shfl_sync(RB_FULL, pk, k & 31) - k;
        const T y0 = __shfl_sync(RB_FULL, y, k & 31);
        const T yj = __shfl_sync(RB_FULL, y, (k + jp) & 31);
        if (p == 0) y = yj;
        if (p == jp) y = y0;
      }
      const T bk = __shfl_sync(RB_FULL, y, k & 31);
      if (p >= 1 && p <= km) y = fma(-lk, bk, y);
      if (p == 0) {
        t[k] = y;
        y = nxt;
      }
    }
    __syncwarp();
  }
  rb_cp_wait<0>();
  __threadfence_block();
  __syncwarp();
  // ---- backward: entry k' lives on lane k' & 31, slot (k' mod M) >> 5; window k-kv..k
  auto load_bchunk = [&](int c, int buf) {
    const int k0 = c * 32, k1 = min(n, k0 + 32);
    T* du = sU + buf * (32 * WM);
    for (int e = lane; e < (k1 - k0) * w; e += 32) rb_cp_async(du + e, U + int64_t(k0) * w + e, sizeof(T));
  };
  load_bchunk(nch - 1, 0);
  rb_cp_commit();
  T z[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const int e = (n - 1) - (((n - 1) - (lane + 32 * s)) & (M - 1));  // entry of this slot in (n-1-M, n-1]
    z[s] = (e >= 0) ? t[e] : T(0);
  }
  // lane q refills entry 32 (c - NS) + q while in chunk c
  int e0 = 32 * (nch - 1 - NS) + lane;
  T rfn = (e0 >= 0) ? t[e0] : T(0);
  for (int c = nch - 1, b = 0; c >= 0; --c, b ^= 1) {
    if (c > 0) load_bchunk(c - 1, b ^ 1);
    rb_cp_commit();
    const T rf = rfn;
    e0 = 32 * (c - 1 - NS) + lane;
    rfn = (e0 >= 0) ? t[e0] : T(0);
    const int s0 = c & (NS - 1);  // slot that chunk c refills: (k mod M) >> 5
    rb_cp_wait<1>();
    __syncwarp();
    const T* cu = sU + b * (32 * WM);
    const int k0 = c * 32, k1 = min(n, k0 + 32);
    for (int k = k1 - 1; k >= k0; --k) {
      const T* uk = cu + (k - k0) * w;
      const int ol = k & 31;
      T zo = z[0];
      if (NS > 1 && s0 == 1) zo = z[NS - 1];
      const T zk = __shfl_sync(RB_FULL, zo, ol);
      const T xk = zk * uk[0];
      const int pm = min(kv, k);
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        const int p = (k - lane - 32 * s) & (M - 1);
        if (p >= 1 && p <= pm) z[s] = fma(-uk[p], xk, z[s]);
      }
      if (lane == ol) {
        t[k] = xk;
        if (NS == 1 || s0 == 0)
          z[0] = rf;
        else
          z[NS - 1] = rf;
      }
    }
    __syncwarp();
  }
  rb_cp_wait<0>();
  __syncwarp();
}

// Δx for every component: b = P_rcm Lλ, x = (LU)^-1 b, then (T = float)
// sweeps of iterative refinement r = b - A x (FP64, unfactorised rows),
// x += (LU)^-1 r until the correction is below 1e-12 of x (max norms).  The
// Newton iteration needs no more: a direction exact to 1e-12 moves the
// converged states by ~1e-12 of the last correction.  A component that does
// not contract (rate above 1/2) or would need more than nref sweeps at its
// observed rate is flagged for the FP64 fallback (mode RB_PRIMARY).  Writes dx
// in model order.
template <typename T, int WM>
__global__ void __launch_bounds__(32) rb_solve(RbComp cp, const int32_t* __restrict__ perm,
                                              const double* __restrict__ A, const T* __restrict__ UC,
                                              const T* __restrict__ LM, const int32_t* __restrict__ ipiv,
                                              const double* __restrict__ Ll, double* __restrict__ bw,
                                              double* __restrict__ xw, double* __restrict__ rw, T* __restrict__ tw,
                                              double* __restrict__ dx, int nref, int mode, int* __restrict__ flag,
                                              int* __restrict__ nsweep) {
  __shared__ __align__(16) unsigned char smem[RbSmem<T, WM>::bytes];
  const int cc = cp.list ? cp.list[blockIdx.x] : int(blockIdx.x), lane = threadIdx.x;
  if (mode == RB_FALLBACK && flag[cc] == 0) return;
  if (mode == RB_PRIMARY && flag[cc] != 0) return;  // zero pivot in the primary factorisation
  const int n = cp.cn[cc], kl = cp.ckl[cc], kv = kl + cp.cku[cc], w = kv + 1;
  const int64_t d0 = cp.cdof0[cc];
  const int32_t* pm = perm + d0;
  const double* Ac = A + cp.rbase[cc];
  const T* U = UC + cp.rbase[cc];
  const T* L = LM + cp.lbase[cc];
  const int32_t* piv = ipiv + d0;
  double* b = bw + d0;
  double* x = xw + d0;
  double* r = rw + d0;
  T* t = tw + d0;
  for (int k = lane; k < n; k += 32) b[k] = Ll[pm[k]];
  __syncwarp();
  rb_fb<T, WM>(n, kl, kv, w, U, L, piv, b, t, smem, lane);
  double xn = 0.0, dn = 0.0;
  for (int k = lane; k < n; k += 32) {
    const double v = double(t[k]);
    x[k] = v;
    xn = fmax(xn, fabs(v));
  }
  int sweeps = 0;
  bool ok = true;
  if (nref > 0) {
    double dprev = INFINITY;
    ok = false;
    for (int it = 0; it < nref; ++it) {
      __syncwarp();
      for (int i = lane; i < n; i += 32) {
        double s = b[i];
        const double* row = Ac + int64_t(i) * w;
        const int c0 = max(0, kl - i), c1 = min(kv, n - 1 - i + kl);
        for (int c = c0; c <= c1; ++c) s = fma(-row[c], x[i - kl + c], s);
        r[i] = s;
      }
      __syncwarp();
      rb_fb<T, WM>(n, kl, kv, w, U, L, piv, r, t, smem, lane);
      dn = 0.0;
      xn = 0.0;
      for (int k = lane; k < n; k += 32) {
        const double d = double(t[k]);
        const double v = x[k] + d;
        x[k] = v;
        dn = fmax(dn, fabs(d));
        xn = fmax(xn, fabs(v));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dn = fmax(dn, __shfl_xor_sync(RB_FULL, dn, o));
        xn = fmax(xn, __shfl_xor_sync(RB_FULL, xn, o));
      }
      ++sweeps;
      if (dn <= 1e-12 * xn) {
        ok = true;
        break;
      }
      if (it > 0) {
        const float rho = float(dn / dprev);
        if (!(rho <= 0.5f)) break;  // not contracting (NaN included)
        const float need = logf(float(1e-12 * xn / dn)) / logf(rho);
        if (float(sweeps) + need > float(nref)) break;  // would not make it within nref sweeps
      }
      dprev = dn;
    }
    // NaN/Inf anywhere fails the comparisons above
    if (!(xn <= 1.7976931348623157e308)) ok = false;
  }
  __syncwarp();
  if (lane == 0) {
    if (nsweep) nsweep[cc] = sweeps;
    if (!ok && mode == RB_PRIMARY) flag[cc] = 1;
  }
  if (ok || mode != RB_PRIMARY)
    for (int k = lane; k < n; k += 32) dx[pm[k]] = x[k];
}

// unfactorised rows from the assembled CSC values (positions fixed at create),
// in FP64 and, when A32 is given, in FP32 for the FP32 factorisation
static __global__ void rb_gather(int64_t nnz, const int64_t* __restrict__ map, const double* __restrict__ nzval,
                          double* __restrict__ A, float* __restrict__ A32) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q < nnz) {
    const double v = nzval[q];
    A[map[q]] = v;
    if (A32) A32[map[q]] = float(v);
  }
}

}  // namespace mgpu
