// GB300 assembly path: device model, element kernels, deterministic scatter,
// and the C-ABI entry points of include/muscade_gpu.h.
//
// Per Newton iteration the reference loops over element types and elements,
// evaluates each element with dual numbers and adds values and partials into
// Lλ / Lλx.nzval through the asm maps (src/Assemble.jl:470-608,
// src/SweepX.jl:39-96).  Here:
//   1. one kernel per element type computes every element's residual and
//      Newton tangent (one thread per element, closed-form FP64 tangents) and
//      writes them to element-entry buffers laid out entry-major, so that the
//      stores of a warp are coalesced;
//   2. a gather kernel sums, for every nnz of Lλx and every dof of Lλ, the
//      element entries that map to it, in the order the reference adds them
//      (no floating-point atomics: results are deterministic run to run).  A
//      block takes a run of consecutive nnz, stages all their entries in shared
//      memory with many independent loads in flight, then each thread adds its
//      nnz's entries in order.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "bar_math.hpp"
#include "beam_const.hpp"
#include "ctx.hpp"

using namespace mgpu;

namespace mgpu {

constexpr int BEAM_NCONST = sizeof(BeamConst) / sizeof(double);
constexpr int BAR_NCONST = sizeof(BarConst) / sizeof(double);
static_assert(sizeof(BeamConst) == 50 * sizeof(double), "BeamConst is a flat array of doubles");
static_assert(sizeof(BarConst) == 22 * sizeof(double), "BarConst is a flat array of doubles");

int set_err(mgpu_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

// ------------------------------------------------------------------ kernels
struct AsmArgs {
  const double* x0;
  const double* x1;
  const double* x2;
  const double* u;
  const double* tv;
  const double* av;  // Newmark a (per dof), step mission only
  const double* bv;
  const double* scale;  // per dof or nullptr
  const double* sc;     // step constants: t, a1, a2, a3, b1, b2, b3
  double p0;            // coefficient of ∂/∂X₀ (1)
  int mission;
  int* errflag;
};

template <class T>
__device__ __forceinline__ void load_soa(T& dst, const double* __restrict__ src, int64_t nele, int64_t e) {
  double* d = reinterpret_cast<double*>(&dst);
#pragma unroll
  for (int f = 0; f < int(sizeof(T) / sizeof(double)); ++f) d[f] = __ldg(src + f * nele + e);
}

__device__ __forceinline__ void flag_nan(int* errflag, int64_t gid, bool bad) {
  if (bad) atomicMin(errflag, int(gid < INT_MAX ? gid : INT_MAX - 1));
}

// EulerBeam3D: one thread per element.  DYN selects the Newmark form.
// EI-scale A-dof of the wrapper element EulerBeam3D{adof}: the bending
// constants (EI2, EI3 times Gauss sums of the curvature shapes) scale with it
__device__ __forceinline__ void scale_bending(BeamConst& bc, double s) {
  bc.k3u *= s;
  bc.k3uv *= s;
  bc.k3v *= s;
  bc.k2u *= s;
  bc.k2uv *= s;
  bc.k2v *= s;
}

// Launched with 64, 128 (default) or 256 threads per block (mgpu_autotune
// picks); the bound of 256 leaves the register cap at 255 either way.
template <bool DYN>
__global__ void __launch_bounds__(256) beam_kernel(int64_t nele, const int32_t* __restrict__ idx,
                                                   const int32_t* __restrict__ uidx, const double* __restrict__ cdata,
                                                   const int32_t* __restrict__ aidx, const double* __restrict__ Avec,
                                                   AsmArgs a, double* __restrict__ rout, double* __restrict__ kout,
                                                   int64_t gid0) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  BeamConst bc;
  load_soa(bc, cdata, nele, e);
  if (aidx) scale_bending(bc, __ldg(Avec + __ldg(aidx + e)));
  int dof[12];
  double X0[12], X1[12], X2[12], av[12], bv[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    dof[i] = __ldg(idx + i * nele + e);
    X0[i] = __ldg(a.x0 + dof[i]);
    if constexpr (DYN) {
      X1[i] = __ldg(a.x1 + dof[i]);
      X2[i] = __ldg(a.x2 + dof[i]);
      if (a.mission == MGPU_ASM_STEP) {
        av[i] = __ldg(a.av + dof[i]);
        bv[i] = __ldg(a.bv + dof[i]);
      }
    }
  }
  double U[3];
  const bool has_u = uidx != nullptr;
  if (has_u)
#pragma unroll
    for (int k = 0; k < 3; ++k) U[k] = __ldg(a.u + __ldg(uidx + k * nele + e));
  double R[12], K[144], rd[12];
  const bool step = DYN && a.mission == MGPU_ASM_STEP;
  const Perturb pt{a.p0, DYN ? a.sc[1] : 0.0, DYN ? a.sc[4] : 0.0};  // K + a1 C + b1 M
  beam_element<DYN>(bc, X0, X1, X2, has_u ? U : nullptr, pt, av, bv, R, K, step ? rd : nullptr, nullptr);
  double s[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) s[i] = a.scale ? __ldg(a.scale + dof[i]) : 1.0;
  bool bad = false;
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const double r = (step ? R[i] - rd[i] : R[i]) * s[i];
    bad |= isnan(r);
    rout[i * nele + e] = r;
  }
#pragma unroll
  for (int j = 0; j < 12; ++j)
#pragma unroll
    for (int i = 0; i < 12; ++i) {
      const double k = K[i + 12 * j] * s[i] * s[j];
      bad |= isnan(k);
      kout[(i + 12 * j) * nele + e] = k;
    }
  flag_nan(a.errflag, gid0 + e, bad);
}

__global__ void bar_kernel(int64_t nele, int nder, const int32_t* __restrict__ idx, const int32_t* __restrict__ uidx,
                           const double* __restrict__ cdata, AsmArgs a, double* __restrict__ rout,
                           double* __restrict__ kout, int64_t gid0) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  BarConst bc;
  load_soa(bc, cdata, nele, e);
  int dof[6];
  double X0[6], X1[6], X2[6], av[6], bv[6];
  const bool step = a.mission == MGPU_ASM_STEP;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    dof[i] = __ldg(idx + i * nele + e);
    X0[i] = __ldg(a.x0 + dof[i]);
    X1[i] = nder > 1 ? __ldg(a.x1 + dof[i]) : 0.0;
    X2[i] = nder > 2 ? __ldg(a.x2 + dof[i]) : 0.0;
    av[i] = step ? __ldg(a.av + dof[i]) : 0.0;
    bv[i] = step ? __ldg(a.bv + dof[i]) : 0.0;
  }
  double U[3];
  const bool has_u = uidx != nullptr;
  if (has_u)
    for (int k = 0; k < 3; ++k) U[k] = __ldg(a.u + __ldg(uidx + k * nele + e));
  double R[6], K[36], rd[6];
  bar_element(bc, nder, X0, X1, X2, has_u ? U : nullptr, a.sc[0], a.p0, nder > 1 ? a.sc[1] : 0.0,
              nder > 1 ? a.sc[4] : 0.0, step ? av : nullptr,
              step ? bv : nullptr, R, K, rd, nullptr);
  double s[6];
  for (int i = 0; i < 6; ++i) s[i] = a.scale ? __ldg(a.scale + dof[i]) : 1.0;
  bool bad = false;
  for (int i = 0; i < 6; ++i) {
    const double r = (step ? R[i] - rd[i] : R[i]) * s[i];
    bad |= isnan(r);
    rout[i * nele + e] = r;
  }
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i) {
      const double k = K[i + 6 * j] * s[i] * s[j];
      bad |= isnan(k);
      kout[(i + 6 * j) * nele + e] = k;
    }
  flag_nan(a.errflag, gid0 + e, bad);
}

// DofConstraint{:X} in equal mode with gap g = Σ aᵢ xᵢ − c(t):
// R = [−aᵢ λ ; −g]  (src/BasicElements.jl:426-438)
__global__ void constraint_kernel(int64_t nele, int nX, const int32_t* __restrict__ idx,
                                  const double* __restrict__ cdata, const double* __restrict__ tv, AsmArgs a,
                                  double* __restrict__ rout, double* __restrict__ kout, int64_t gid0) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  const int nx = nX - 1;
  const int dl = __ldg(idx + nx * nele + e);
  const double lam = __ldg(a.x0 + dl);
  const double sl = a.scale ? __ldg(a.scale + dl) : 1.0;
  double gap = -__ldg(tv + e);
  bool bad = false;
  for (int i = 0; i < nx; ++i) {
    const int di = __ldg(idx + i * nele + e);
    const double ci = __ldg(cdata + i * nele + e);
    gap += ci * __ldg(a.x0 + di);
    const double si = a.scale ? __ldg(a.scale + di) : 1.0;
    const double r = -ci * lam * si;
    bad |= isnan(r);
    rout[i * nele + e] = r;
    for (int j = 0; j < nX; ++j) kout[(i + nX * j) * nele + e] = (j == nx) ? -ci * si * sl * a.p0 : 0.0;
  }
  rout[nx * nele + e] = -gap * sl;
  bad |= isnan(gap);
  for (int j = 0; j < nX; ++j) {
    double k = 0.0;
    if (j < nx) {
      const int dj = __ldg(idx + j * nele + e);
      const double sj = a.scale ? __ldg(a.scale + dj) : 1.0;
      k = -__ldg(cdata + j * nele + e) * sl * sj * a.p0;
    }
    kout[(nx + nX * j) * nele + e] = k;
  }
  flag_nan(a.errflag, gid0 + e, bad);
}

// DofLoad: R = −F(t), zero tangent entry (src/BasicElements.jl:281-284)
__global__ void load_kernel(int64_t nele, const int32_t* __restrict__ idx, const double* __restrict__ tv, AsmArgs a,
                            double* __restrict__ rout, double* __restrict__ kout, int64_t gid0) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  const int d = __ldg(idx + e);
  const double s = a.scale ? __ldg(a.scale + d) : 1.0;
  const double r = -__ldg(tv + e) * s;
  rout[e] = r;
  kout[e] = 0.0;
  flag_nan(a.errflag, gid0 + e, isnan(r));
}

// SingleDofCost and SingleUdof in SweepX: the residual of a Lagrangian
// element is ∂L/∂Λ (src/Assemble.jl:661-677), 0 for a cost and −u for the
// U-dof load of SingleUdof (L = cost(u,t) − λu); the tangents are zero.
__global__ void cost_kernel(int64_t nele, int udof, const int32_t* __restrict__ idx,
                            const int32_t* __restrict__ uidx, AsmArgs a, double* __restrict__ rout,
                            double* __restrict__ kout, int64_t gid0) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  double r = 0.0;
  if (udof) {
    const int d = __ldg(idx + e);
    const double s = a.scale ? __ldg(a.scale + d) : 1.0;
    r = -__ldg(a.u + __ldg(uidx + e)) * s;
  }
  rout[e] = r;
  kout[e] = 0.0;
  flag_nan(a.errflag, gid0 + e, isnan(r));
}

// Deterministic gather-sum:
//   out[k] = ((0 + buf[src[q0]]) + buf[src[q0+1]]) + ... ,  q = seg[k] .. seg[k+1]-1.
// A block takes kGatherOut consecutive outputs.  Their plan positions form one
// run [seg[k0], seg[k0+kGatherOut]); the block stages the run's entries in
// shared memory: each thread first loads kGatherPer plan entries (coalesced),
// then issues the kGatherPer gathered loads of the values, all independent, so
// that many loads are in flight per SM.  The gathered values of consecutive
// nnz come from consecutive elements of one entry plane (neighbouring nodes,
// neighbouring elements), so sectors are reused through L1 within a block.
// The sums are FP64 additions, and GB300 issues few of them: the first term
// needs none (0 + v is v, with −0 turned into +0 as the addition would), and
// the outputs of more than one term are listed and shared out one per thread,
// so that a warp's lanes add about as many terms each instead of waiting on
// the longest sum of 32 neighbouring outputs.  A run longer than one staging
// pass takes the general loop (one output per thread, pass by pass).
constexpr int kGatherThreads = 256;
constexpr int kGatherOut = 1024;    // outputs per block (4 per thread)
constexpr int kGatherPer = 8;       // staged entries per thread and pass
constexpr int kGatherStage = kGatherThreads * kGatherPer;

// 0 + v: v itself, except that −0 becomes +0
__device__ __forceinline__ double plus_zero(double v) {
  return __double_as_longlong(v) == (long long)0x8000000000000000ULL ? 0.0 : v;
}

__global__ void __launch_bounds__(kGatherThreads) scatter_kernel(int64_t n, const uint32_t* __restrict__ seg,
                                                                 const uint32_t* __restrict__ src,
                                                                 const double* __restrict__ buf,
                                                                 double* __restrict__ out) {
  __shared__ uint32_t sseg[kGatherOut + 1];
  __shared__ double sval[kGatherStage];
  __shared__ int16_t slist[kGatherOut];
  __shared__ int nlist;
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t k0 = int64_t(blockIdx.x) * kGatherOut;
  const int nk = int(n - k0 < kGatherOut ? n - k0 : kGatherOut);
  for (int t = tid; t <= nk; t += kGatherThreads) sseg[t] = __ldg(seg + k0 + t);
  if (tid == 0) nlist = 0;
  __syncthreads();
  const int64_t qa = sseg[0], qb = sseg[nk];
  constexpr int R = kGatherOut / kGatherThreads;
  if (qb - qa <= kGatherStage) {
    const int wn = int(qb - qa);
    uint32_t sidx[kGatherPer];
#pragma unroll
    for (int u = 0; u < kGatherPer; ++u) {
      const int t = u * kGatherThreads + tid;
      sidx[u] = t < wn ? __ldg(src + qa + t) : 0u;
    }
    double v[kGatherPer];
#pragma unroll
    for (int u = 0; u < kGatherPer; ++u) v[u] = (u * kGatherThreads + tid < wn) ? __ldg(buf + sidx[u]) : 0.0;
#pragma unroll
    for (int u = 0; u < kGatherPer; ++u) sval[u * kGatherThreads + tid] = v[u];
    __syncthreads();
    // outputs of zero or one term now; the others to the list
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int kk = r * kGatherThreads + tid;
      int len = 0, a = 0;
      if (kk < nk) {
        a = int(sseg[kk] - qa);
        len = int(sseg[kk + 1] - sseg[kk]);
        if (len <= 1) out[k0 + kk] = len ? plus_zero(sval[a]) : 0.0;
      }
      const bool longer = len > 1;
      const unsigned mask = __ballot_sync(0xffffffffu, longer);
      int base = 0;
      if (lane == 0 && mask) base = atomicAdd(&nlist, __popc(mask));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (longer) slist[base + __popc(mask & ((1u << lane) - 1u))] = int16_t(kk);
    }
    __syncthreads();
    for (int i = tid; i < nlist; i += kGatherThreads) {
      const int kk = slist[i];
      const int a = int(sseg[kk] - qa), b = int(sseg[kk + 1] - qa);
      double acc = plus_zero(sval[a]);
      for (int q = a + 1; q < b; ++q) acc += sval[q];
      out[k0 + kk] = acc;
    }
    return;
  }
  double acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = 0.0;
  for (int64_t w0 = qa; w0 < qb; w0 += kGatherStage) {
    const int wn = int(qb - w0 < kGatherStage ? qb - w0 : kGatherStage);
    uint32_t sidx[kGatherPer];
#pragma unroll
    for (int u = 0; u < kGatherPer; ++u) {
      const int t = u * kGatherThreads + tid;
      sidx[u] = t < wn ? __ldg(src + w0 + t) : 0u;
    }
    double v[kGatherPer];
#pragma unroll
    for (int u = 0; u < kGatherPer; ++u) v[u] = (u * kGatherThreads + tid < wn) ? __ldg(buf + sidx[u]) : 0.0;
#pragma unroll
    for (int u = 0; u < kGatherPer; ++u) sval[u * kGatherThreads + tid] = v[u];
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int kk = r * kGatherThreads + tid;
      if (kk < nk) {
        const int64_t a = sseg[kk], b = sseg[kk + 1];
        const int64_t lo = a > w0 ? a : w0;
        const int64_t hi = b < w0 + wn ? b : w0 + wn;
        for (int64_t q = lo; q < hi; ++q) acc[r] += sval[q - w0];
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int kk = r * kGatherThreads + tid;
    if (kk < nk) out[k0 + kk] = acc[r];
  }
}

__global__ void newmark_ab_kernel(int64_t n, const double* x1, const double* x2, const double* __restrict__ sc,
                                  double* av, double* bv) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a2 = sc[2], a3 = sc[3], b2 = sc[5], b3 = sc[6];
  av[i] = a2 * x1[i] + a3 * x2[i];
  bv[i] = b2 * x1[i] + b3 * x2[i];
}

__global__ void set_int_kernel(int* p, int v) { *p = v; }

__global__ void fill_kernel(double* p, int64_t n, double v) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

static inline unsigned nblk(int64_t n, int b) { return unsigned((n + b - 1) / b); }

// ------------------------------------------------------------------ assembly
int upload_stepc(mgpu_ctx* c, double t, const mgpu_newmark* nm) {
  const int k = c->stepc_slot;
  c->stepc_slot = (k + 1) % kStepcSlots;
  MG_CUDA(cudaEventSynchronize(c->stepc_ev[k]));  // the copy that last read this slot is done
  double* h = c->hstepc + 8 * k;
  h[0] = t;
  h[1] = nm ? nm->a1 : 0.0;
  h[2] = nm ? nm->a2 : 0.0;
  h[3] = nm ? nm->a3 : 0.0;
  h[4] = nm ? nm->b1 : 0.0;
  h[5] = nm ? nm->b2 : 0.0;
  h[6] = nm ? nm->b3 : 0.0;
  h[7] = 0.0;
  MG_CUDA(cudaMemcpyAsync(c->stepc, h, 8 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  MG_CUDA(cudaEventRecord(c->stepc_ev[k], c->stream));
  return MGPU_OK;
}

void launch_reset_errflag(mgpu_ctx* c) {
  set_int_kernel<<<1, 1, 0, c->stream>>>(c->errflag, INT_MAX);
  ++c->launches;
}

int launch_assembly(mgpu_ctx* c, int mission, cudaEvent_t* ev_groups, double p0) {
  const int64_t nX = c->nX;
  AsmArgs a;
  a.x0 = c->x;
  a.x1 = c->x + nX;
  a.x2 = c->x + 2 * nX;
  a.u = c->u;
  a.tv = c->tv;
  a.av = c->ab;
  a.bv = c->ab + nX;
  a.scale = c->scale;
  a.sc = c->stepc;
  a.mission = mission;
  a.errflag = c->errflag;
  const bool dyn = mission != MGPU_ASM_STATIC;
  a.p0 = p0;
  if (dyn && c->nXder_resident != 3) return set_err(c, MGPU_ERR_ARG, "Newmark assembly needs X, X' and X''");
  if (mission == MGPU_ASM_STEP && nX > 0) {
    newmark_ab_kernel<<<nblk(nX, 256), 256, 0, c->stream>>>(nX, a.x1, a.x2, c->stepc, c->ab, c->ab + nX);
    ++c->launches;
  }
  int64_t gid0 = 0;
  for (size_t g = 0; g < c->groups.size(); ++g) {
    const DevGroup& G = c->groups[g];
    if (G.nele == 0) {
      if (ev_groups) cudaEventRecord(ev_groups[g], c->stream);
      continue;
    }
    double* rout = c->rbuf + c->pat.rbuf_base[g];
    double* kout = c->kbuf + c->pat.kbuf_base[g];
    AsmArgs ag = a;
    if (G.tval_base >= 0) ag.tv = c->tv + G.tval_base;
    switch (G.kind) {
      case MGPU_EULERBEAM3D:
        if (dyn)
          beam_kernel<true><<<nblk(G.nele, c->elem_block), c->elem_block, 0, c->stream>>>(G.nele, G.idx, G.uidx, G.cdata, G.aidx,
                                                                      c->Avec, ag, rout, kout, gid0);
        else
          beam_kernel<false><<<nblk(G.nele, c->elem_block), c->elem_block, 0, c->stream>>>(G.nele, G.idx, G.uidx, G.cdata, G.aidx,
                                                                       c->Avec, ag, rout, kout, gid0);
        break;
      case MGPU_BAR3D:
        bar_kernel<<<nblk(G.nele, c->elem_block), c->elem_block, 0, c->stream>>>(G.nele, dyn ? 3 : 1, G.idx, G.uidx, G.cdata, ag, rout,
                                                             kout, gid0);
        break;
      case MGPU_DOFCONSTRAINT_X:
        constraint_kernel<<<nblk(G.nele, 256), 256, 0, c->stream>>>(G.nele, G.nX, G.idx, G.cdata, ag.tv, ag, rout,
                                                                    kout, gid0);
        break;
      case MGPU_DOFLOAD:
        load_kernel<<<nblk(G.nele, 256), 256, 0, c->stream>>>(G.nele, G.idx, ag.tv, ag, rout, kout, gid0);
        break;
      case MGPU_DOFCOST:
      case MGPU_SINGLEUDOF:
        cost_kernel<<<nblk(G.nele, 256), 256, 0, c->stream>>>(G.nele, G.kind == MGPU_SINGLEUDOF, G.idx, G.uidx, ag,
                                                              rout, kout, gid0);
        break;
      case MGPU_ACOST:  // no X-dofs: nothing in SweepX's Lλ and Lλx
        break;
    }
    if (G.kind != MGPU_ACOST) ++c->launches;
    gid0 += G.nele;
    if (ev_groups) cudaEventRecord(ev_groups[g], c->stream);
  }
  if (c->pat.nnz > 0) {
    scatter_kernel<<<nblk(c->pat.nnz, kGatherOut), kGatherThreads, 0, c->stream>>>(c->pat.nnz, c->mseg, c->msrc,
                                                                                  c->kbuf, c->nzval);
    ++c->launches;
  }
  if (nX > 0) {
    scatter_kernel<<<nblk(nX, kGatherOut), kGatherThreads, 0, c->stream>>>(nX, c->vseg, c->vsrc, c->rbuf, c->Ll);
    ++c->launches;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(c, MGPU_ERR_CUDA, std::string("assembly launch: ") + cudaGetErrorString(e));
  return MGPU_OK;
}

int check_nan(mgpu_ctx* c) {
  int h[1];
  MG_CUDA(cudaMemcpyAsync(h, c->errflag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MG_CUDA(cudaStreamSynchronize(c->stream));
  return nan_error(c, h[0]);
}

int nan_error(mgpu_ctx* c, int flag) {
  if (flag != INT_MAX) {
    // locate type and element
    int64_t gid = flag, base = 0;
    for (size_t g = 0; g < c->groups.size(); ++g) {
      if (gid < base + c->groups[g].nele) {
        const char* names[] = {"?", "EulerBeam3D", "Bar3D", "DofConstraint", "DofLoad", "DofCost", "SingleUdof",
                               "Acost"};
        int k = c->groups[g].kind;
        return set_err(c, MGPU_ERR_NAN,
                       std::string("residual(") + names[(k >= 1 && k <= 7) ? k : 0] +
                           ",...) returned NaN in R, FB or derivatives (ieletyp=" + std::to_string(g + 1) +
                           ", iele=" + std::to_string(gid - base + 1) + ")");
      }
      base += c->groups[g].nele;
    }
    return set_err(c, MGPU_ERR_NAN, "residual returned NaN");
  }
  return MGPU_OK;
}

static int reset_errflag(mgpu_ctx* c) {
  launch_reset_errflag(c);
  MG_CUDA(cudaGetLastError());
  return MGPU_OK;
}

}  // namespace mgpu

// ------------------------------------------------------------------ C ABI
constexpr int64_t kDevicePatternPairs = int64_t(1) << 22;  // element entries from which the device builds the pattern

template <class T>
static int dalloc(mgpu_ctx* c, T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
  if (e != cudaSuccess) return set_err(c, MGPU_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return MGPU_OK;
}

#define MG_TRY(x)              \
  do {                         \
    int rc_ = (x);             \
    if (rc_ != MGPU_OK) return rc_; \
  } while (0)

extern "C" int mgpu_solver_create(mgpu_ctx* c);   // solver.cu
extern "C" void mgpu_solver_destroy(mgpu_ctx* c);  // solver.cu

extern "C" const char* mgpu_last_error(const mgpu_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int mgpu_create(mgpu_ctx** out, const mgpu_model_desc* d) {
  if (!out || !d) return MGPU_ERR_ARG;
  *out = nullptr;
  mgpu_ctx* c = new mgpu_ctx();
  *out = c;
  c->device = d->device;
  MG_CUDA(cudaSetDevice(d->device));
  MG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->nX = d->nX;
  c->nU = d->nU;
  if (d->nX < 0 || d->nU < 0 || d->ngroup < 0 || (d->ngroup > 0 && !d->groups))
    return set_err(c, MGPU_ERR_ARG, "invalid model description");
  std::vector<GroupShape> shapes;
  int64_t ntv = 0;
  for (int g = 0; g < d->ngroup; ++g) {
    const mgpu_group& G = d->groups[g];
    int exp_nX = -1, exp_data = -1;
    switch (G.kind) {
      case MGPU_EULERBEAM3D: exp_nX = 12; exp_data = BEAM_NFIELD; break;
      case MGPU_BAR3D: exp_nX = 6; exp_data = 38; break;
      case MGPU_DOFCONSTRAINT_X: exp_nX = G.nX; exp_data = G.nX - 1; break;
      case MGPU_DOFLOAD: exp_nX = 1; exp_data = 0; break;
      case MGPU_DOFCOST: exp_nX = 1; exp_data = 2; break;
      case MGPU_SINGLEUDOF: exp_nX = 1; exp_data = 1; break;
      case MGPU_ACOST: exp_nX = 0; exp_data = 2; break;
      default:
        return set_err(c, MGPU_ERR_UNSUPPORTED,
                       "element type " + std::to_string(g + 1) + " (kind " + std::to_string(G.kind) +
                           ") is not supported by the GPU path");
    }
    if (G.nX != exp_nX || (G.nX < 1 && G.kind != MGPU_ACOST) || (exp_data > 0 && G.ndata != exp_data) ||
        G.nele < 0 || (G.nele > 0 && G.nX > 0 && !G.indexX) || (G.nele > 0 && exp_data > 0 && !G.edata))
      return set_err(c, MGPU_ERR_ARG, "element type " + std::to_string(g + 1) + ": unexpected layout");
    if ((G.kind == MGPU_EULERBEAM3D || G.kind == MGPU_BAR3D) && !(G.nU == 0 || G.nU == 3))
      return set_err(c, MGPU_ERR_ARG, "beam/bar elements have 0 or 3 U-dofs");
    if ((G.kind == MGPU_DOFCONSTRAINT_X || G.kind == MGPU_DOFLOAD || G.kind == MGPU_DOFCOST ||
         G.kind == MGPU_ACOST) && G.nU != 0)
      return set_err(c, MGPU_ERR_ARG, "constraints, loads and DofCost/Acost elements have no U-dofs");
    if (G.kind == MGPU_SINGLEUDOF && G.nU != 1) return set_err(c, MGPU_ERR_ARG, "SingleUdof has one U-dof");
    if (G.nU > 0 && G.nele > 0 && !G.indexU) return set_err(c, MGPU_ERR_ARG, "missing indexU");
    if (G.indexA && G.kind != MGPU_EULERBEAM3D && G.kind != MGPU_ACOST)
      return set_err(c, MGPU_ERR_UNSUPPORTED, "A-dofs are supported on EulerBeam3D (EI scale) and Acost only");
    if (G.kind == MGPU_ACOST && G.nele > 0 && !G.indexA) return set_err(c, MGPU_ERR_ARG, "Acost needs indexA");
    if (G.kind == MGPU_DOFCOST)
      for (int64_t e = 0; e < G.nele; ++e) {
        const double dd = G.edata[2 * e + 1];
        if (!(dd == 0.0 || dd == 1.0 || dd == 2.0))
          return set_err(c, MGPU_ERR_ARG, "DofCost: the derivative must be 0, 1 or 2");
      }
    if (G.indexA)
      for (int64_t k = 0; k < G.nele; ++k)
        if (G.indexA[k] < 1 || G.indexA[k] > d->nA) return set_err(c, MGPU_ERR_ARG, "A-dof index out of range");
    for (int64_t k = 0; k < G.nele * G.nU; ++k)
      if (G.indexU[k] < 1 || G.indexU[k] > d->nU) return set_err(c, MGPU_ERR_ARG, "U-dof index out of range");
    shapes.push_back(GroupShape{G.nele, G.nX, G.indexX});
    if (has_tval(G.kind)) ntv += G.nele;
  }
  c->ntval = ntv;
  // ---- per-group device data
  int64_t tvb = 0;
  for (int g = 0; g < d->ngroup; ++g) {
    const mgpu_group& G = d->groups[g];
    DevGroup D;
    D.kind = G.kind;
    D.nX = G.nX;
    D.nU = G.nU;
    D.ndata = G.ndata;
    D.nele = G.nele;
    D.h_indexX.assign(G.indexX, G.indexX + G.nele * G.nX);
    std::vector<int32_t> idx(size_t(G.nX) * G.nele);
    for (int64_t e = 0; e < G.nele; ++e)
      for (int i = 0; i < G.nX; ++i) idx[size_t(i) * G.nele + e] = int32_t(G.indexX[e * G.nX + i] - 1);
    MG_TRY(dalloc(c, &D.idx, idx.size()));
    MG_CUDA(cudaMemcpy(D.idx, idx.data(), idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (G.nU > 0) {
      std::vector<int32_t> uidx(size_t(G.nU) * G.nele);
      for (int64_t e = 0; e < G.nele; ++e)
        for (int i = 0; i < G.nU; ++i) uidx[size_t(i) * G.nele + e] = int32_t(G.indexU[e * G.nU + i] - 1);
      MG_TRY(dalloc(c, &D.uidx, uidx.size()));
      MG_CUDA(cudaMemcpy(D.uidx, uidx.data(), uidx.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    if (G.indexA && G.nele > 0) {
      D.h_indexA.assign(G.indexA, G.indexA + G.nele);
      std::vector<int32_t> aidx(G.nele);
      for (int64_t e = 0; e < G.nele; ++e) aidx[e] = int32_t(G.indexA[e] - 1);
      MG_TRY(dalloc(c, &D.aidx, aidx.size()));
      MG_CUDA(cudaMemcpy(D.aidx, aidx.data(), aidx.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    std::vector<double> cd;
    if (G.kind == MGPU_EULERBEAM3D) D.h_edata.assign(G.edata, G.edata + G.nele * BEAM_NFIELD);
    if (G.kind == MGPU_EULERBEAM3D) {
      D.nfield = BEAM_NCONST;
      cd.resize(size_t(D.nfield) * G.nele);
      for (int64_t e = 0; e < G.nele; ++e) {
        BeamConst bc;
        beam_const_from_fields(G.edata + e * BEAM_NFIELD, bc);
        const double* p = reinterpret_cast<const double*>(&bc);
        for (int f = 0; f < D.nfield; ++f) cd[size_t(f) * G.nele + e] = p[f];
      }
    } else if (G.kind == MGPU_BAR3D) {
      D.nfield = BAR_NCONST;
      cd.resize(size_t(D.nfield) * G.nele);
      for (int64_t e = 0; e < G.nele; ++e) {
        BarConst bc;
        bar_const_from_fields(G.edata + e * 38, bc);
        const double* p = reinterpret_cast<const double*>(&bc);
        for (int f = 0; f < D.nfield; ++f) cd[size_t(f) * G.nele + e] = p[f];
      }
    } else if (G.ndata > 0) {  // constraint coefficients, cost weights and targets
      D.nfield = G.ndata;
      cd.resize(size_t(D.nfield) * G.nele);
      for (int64_t e = 0; e < G.nele; ++e)
        for (int f = 0; f < D.nfield; ++f) cd[size_t(f) * G.nele + e] = G.edata[e * D.nfield + f];
    }
    if (!cd.empty()) {
      MG_TRY(dalloc(c, &D.cdata, cd.size()));
      MG_CUDA(cudaMemcpy(D.cdata, cd.data(), cd.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (has_tval(G.kind)) {
      D.tval_base = tvb;
      tvb += G.nele;
    }
    if (G.kind == MGPU_DOFCOST || G.kind == MGPU_SINGLEUDOF || G.kind == MGPU_ACOST) {
      // gradient entries each element writes: (dof, derivative), (X-dof, U-dof) or the A-dof
      std::vector<std::pair<int64_t, int64_t>> keys(G.nele), ukeys;
      for (int64_t e = 0; e < G.nele; ++e) {
        if (G.kind == MGPU_DOFCOST) {
          const int d = int(G.edata[2 * e + 1]);
          D.maxder = std::max(D.maxder, d);
          keys[e] = {G.indexX[e], d};
        } else if (G.kind == MGPU_SINGLEUDOF) {
          keys[e] = {G.indexX[e], 0};
          ukeys.push_back({G.indexU[e], 0});
        } else {
          keys[e] = {G.indexA[e], 0};
        }
      }
      for (auto* v : {&keys, &ukeys}) {
        std::sort(v->begin(), v->end());
        D.distinct = D.distinct && std::adjacent_find(v->begin(), v->end()) == v->end();
      }
    }
    c->groups.push_back(std::move(D));
  }
  // ---- pattern and gather plans: on the host, or on the device (a radix sort of the
  // element entries) when MGPU_DEVICE_PATTERN is set or the model has 4 M entries or more
  const auto t_pat0 = std::chrono::steady_clock::now();
  int64_t npairs = 0;
  for (const GroupShape& G : shapes) npairs += G.nele * G.nX * G.nX;
  bool dev_pattern = npairs >= kDevicePatternPairs;
  if (const char* ev = getenv("MGPU_DEVICE_PATTERN")) dev_pattern = atoi(ev) != 0;
  std::string perr;
  if (dev_pattern) {
    std::vector<const int32_t*> didx;
    for (const DevGroup& D : c->groups) didx.push_back(D.idx);
    perr = build_pattern_device(d->nX, shapes, didx, c->stream, c->pat);
  } else {
    perr = build_pattern(d->nX, shapes, c->pat);
  }
  if (!perr.empty()) return set_err(c, MGPU_ERR_ARG, perr);
  c->device_pattern = dev_pattern;
  const auto t_pat1 = std::chrono::steady_clock::now();
  // ---- node coordinates of the dofs (element geometry) and the constraint multipliers
  c->dof_xyz.assign(3 * size_t(c->nX), NAN);
  c->dof_last.assign(size_t(c->nX), 0);
  for (int g = 0; g < d->ngroup; ++g) {
    const mgpu_group& G = d->groups[g];
    if (G.kind == MGPU_EULERBEAM3D || G.kind == MGPU_BAR3D) {
      // midpoint cₘ and c₂ − c₁ (tgₘ) in the element record: fields 0-2 and 18-20 (beam), 3-5 (bar)
      const int nd = G.kind == MGPU_EULERBEAM3D ? 6 : 3, ftg = G.kind == MGPU_EULERBEAM3D ? 18 : 3;
      for (int64_t e = 0; e < G.nele; ++e) {
        const double* ed = G.edata + e * G.ndata;
        for (int i = 0; i < 2 * nd; ++i) {
          const int64_t dof = G.indexX[e * G.nX + i] - 1;
          const double sgn = i < nd ? -0.5 : 0.5;
          for (int k = 0; k < 3; ++k) c->dof_xyz[3 * dof + k] = ed[k] + sgn * ed[ftg + k];
        }
      }
    } else if (G.kind == MGPU_DOFCONSTRAINT_X) {
      for (int64_t e = 0; e < G.nele; ++e) c->dof_last[G.indexX[e * G.nX + G.nX - 1] - 1] = 1;
    }
  }
  // ---- buffers and scatter plans
  const Pattern& P = c->pat;
  MG_TRY(dalloc(c, &c->kbuf, P.kbuf_size));
  MG_TRY(dalloc(c, &c->rbuf, P.rbuf_size));
  MG_TRY(dalloc(c, &c->mseg, P.mseg.size()));
  MG_TRY(dalloc(c, &c->msrc, P.msrc.size()));
  MG_TRY(dalloc(c, &c->vseg, P.vseg.size()));
  MG_TRY(dalloc(c, &c->vsrc, P.vsrc.size()));
  MG_CUDA(cudaMemcpy(c->mseg, P.mseg.data(), P.mseg.size() * 4, cudaMemcpyHostToDevice));
  MG_CUDA(cudaMemcpy(c->msrc, P.msrc.data(), P.msrc.size() * 4, cudaMemcpyHostToDevice));
  MG_CUDA(cudaMemcpy(c->vseg, P.vseg.data(), P.vseg.size() * 4, cudaMemcpyHostToDevice));
  MG_CUDA(cudaMemcpy(c->vsrc, P.vsrc.data(), P.vsrc.size() * 4, cudaMemcpyHostToDevice));
  MG_TRY(dalloc(c, &c->nzval, P.nnz));
  MG_TRY(dalloc(c, &c->Ll, c->nX));
  MG_TRY(dalloc(c, &c->x, 3 * c->nX));
  MG_CUDA(cudaMemset(c->x, 0, 3 * std::max<int64_t>(c->nX, 1) * sizeof(double)));
  MG_TRY(dalloc(c, &c->u, c->nU));
  MG_CUDA(cudaMemset(c->u, 0, std::max<int64_t>(c->nU, 1) * sizeof(double)));
  MG_TRY(dalloc(c, &c->tv, c->ntval));
  MG_CUDA(cudaMemset(c->tv, 0, std::max<int64_t>(c->ntval, 1) * sizeof(double)));
  MG_TRY(dalloc(c, &c->ab, 2 * c->nX));
  MG_TRY(dalloc(c, &c->errflag, 2));
  c->nA = d->nA;
  MG_TRY(dalloc(c, &c->Avec, std::max<int64_t>(c->nA, 1)));
  {
    std::vector<double> ones(std::max<int64_t>(c->nA, 1), 1.0);
    MG_CUDA(cudaMemcpy(c->Avec, ones.data(), ones.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  MG_TRY(dalloc(c, &c->stepc, 8));
  MG_CUDA(cudaMemset(c->stepc, 0, 8 * sizeof(double)));
  MG_CUDA(cudaMallocHost(&c->hstepc, kStepcSlots * 8 * sizeof(double)));
  for (int k = 0; k < kStepcSlots; ++k) MG_CUDA(cudaEventCreateWithFlags(&c->stepc_ev[k], cudaEventDisableTiming));
  if (d->scaleX) {
    bool ones = true;
    for (int64_t i = 0; i < d->nX; ++i) ones &= (d->scaleX[i] == 1.0);
    if (!ones) {
      MG_TRY(dalloc(c, &c->scale, c->nX));
      MG_CUDA(cudaMemcpy(c->scale, d->scaleX, c->nX * sizeof(double), cudaMemcpyHostToDevice));
    }
  }
  MG_TRY(reset_errflag(c));
  const auto t_sol0 = std::chrono::steady_clock::now();
  MG_TRY(mgpu_solver_create(c));
  if (getenv("MGPU_VERBOSE")) {
    const auto t_sol1 = std::chrono::steady_clock::now();
    auto sec = [](auto a, auto b) { return std::chrono::duration<double>(b - a).count(); };
    fprintf(stderr, "[muscade_gpu] create: pattern %.3f s (nnz %lld), solver analysis %.3f s\n", sec(t_pat0, t_pat1),
            (long long)c->pat.nnz, sec(t_sol0, t_sol1));
  }
  MG_CUDA(cudaStreamSynchronize(c->stream));
  return MGPU_OK;
}

extern "C" void mgpu_destroy(mgpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  mgpu_solver_destroy(c);
  for (auto& G : c->groups) {
    cudaFree(G.idx);
    cudaFree(G.uidx);
    cudaFree(G.aidx);
    cudaFree(G.cdata);
  }
  if (c->cstream) cudaStreamSynchronize(c->cstream);
  void* ps[] = {c->kbuf, c->rbuf, c->mseg, c->msrc, c->vseg, c->vsrc, c->nzval, c->Ll, c->x,
                c->u,    c->tv,   c->ab,   c->scale, c->errflag, c->flush, c->stepc, c->Avec,
                c->anz[0], c->anz[1], c->aLl[0], c->aLl[1], c->aerr};
  for (void* p : ps) cudaFree(p);
  if (c->hstepc) cudaFreeHost(c->hstepc);
  for (double* h : c->astage)
    if (h) cudaFreeHost(h);
  if (c->haerr) cudaFreeHost(c->haerr);
  for (int k = 0; k < 2; ++k)
    for (cudaEvent_t e : {c->a_h2d[k], c->a_comp[k], c->a_d2h[k]})
      if (e) cudaEventDestroy(e);
  if (c->cstream) cudaStreamDestroy(c->cstream);
  for (cudaEvent_t e : c->stepc_ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int mgpu_host_register(void* ptr, int64_t bytes) {
  if (!ptr || bytes <= 0) return MGPU_ERR_ARG;
  return cudaHostRegister(ptr, size_t(bytes), cudaHostRegisterDefault) == cudaSuccess ? MGPU_OK : MGPU_ERR_CUDA;
}

extern "C" int mgpu_host_unregister(void* ptr) {
  if (!ptr) return MGPU_ERR_ARG;
  return cudaHostUnregister(ptr) == cudaSuccess ? MGPU_OK : MGPU_ERR_CUDA;
}

extern "C" int mgpu_set_A(mgpu_ctx* c, const double* A) {
  if (!c || (c->nA > 0 && !A)) return set_err(c, MGPU_ERR_ARG, "mgpu_set_A: bad arguments");
  MG_CUDA(cudaSetDevice(c->device));
  if (c->nA > 0) MG_CUDA(cudaMemcpy(c->Avec, A, c->nA * sizeof(double), cudaMemcpyHostToDevice));
  return MGPU_OK;
}

extern "C" int64_t mgpu_nnz(const mgpu_ctx* c) { return c ? c->pat.nnz : -1; }
extern "C" int64_t mgpu_ntval(const mgpu_ctx* c) { return c ? c->ntval : -1; }
extern "C" int64_t mgpu_launch_count(const mgpu_ctx* c) { return c ? c->launches : -1; }

extern "C" int mgpu_get_pattern(const mgpu_ctx* cc, int64_t* colptr, int64_t* rowval) {
  if (!cc || !colptr || !rowval) return MGPU_ERR_ARG;
  for (int64_t j = 0; j <= cc->nX; ++j) colptr[j] = cc->pat.colptr[j] + 1;
  for (int64_t k = 0; k < cc->pat.nnz; ++k) rowval[k] = int64_t(cc->pat.rowval[k]) + 1;
  return MGPU_OK;
}

extern "C" int mgpu_get_asm(const mgpu_ctx* cc, int32_t g, int64_t* asm1, int64_t* asm2) {
  if (!cc || g < 0 || g >= int32_t(cc->groups.size())) return MGPU_ERR_ARG;
  const DevGroup& G = cc->groups[g];
  const int nX = G.nX;
  for (int64_t e = 0; e < G.nele; ++e) {
    if (asm1)
      for (int i = 0; i < nX; ++i) asm1[e * nX + i] = G.h_indexX[e * nX + i];  // X dof group = all X dofs
    if (asm2)
      for (int k = 0; k < nX * nX; ++k)
        asm2[e * nX * nX + k] = int64_t(cc->pat.pair_nnz[cc->pat.pair_base[g] + e * nX * nX + k]) + 1;
  }
  return MGPU_OK;
}

extern "C" int mgpu_upload_state(mgpu_ctx* c, int32_t nXder, const double* x, const double* u, const double* tvals) {
  if (!c || !x || nXder < 1 || nXder > 3) return set_err(c, MGPU_ERR_ARG, "mgpu_upload_state: bad arguments");
  MG_CUDA(cudaSetDevice(c->device));
  MG_CUDA(cudaMemcpyAsync(c->x, x, nXder * c->nX * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (nXder < 3)
    MG_CUDA(cudaMemsetAsync(c->x + nXder * c->nX, 0, (3 - nXder) * c->nX * sizeof(double), c->stream));
  if (c->nU > 0 && u) MG_CUDA(cudaMemcpyAsync(c->u, u, c->nU * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->ntval > 0 && tvals)
    MG_CUDA(cudaMemcpyAsync(c->tv, tvals, c->ntval * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  c->nXder_resident = nXder;
  return MGPU_OK;
}

extern "C" int mgpu_assemble_resident(mgpu_ctx* c, int32_t mission, double t, const mgpu_newmark* nm) {
  if (!c || mission < 0 || mission > 2 || (mission != MGPU_ASM_STATIC && !nm))
    return set_err(c, MGPU_ERR_ARG, "mgpu_assemble_resident: bad arguments");
  MG_CUDA(cudaSetDevice(c->device));
  MG_TRY(upload_stepc(c, t, mission != MGPU_ASM_STATIC ? nm : nullptr));
  return launch_assembly(c, mission, nullptr, 1.0);
}

extern "C" int mgpu_download(mgpu_ctx* c, double* Ll, double* nzval) {
  if (!c) return MGPU_ERR_ARG;
  MG_CUDA(cudaSetDevice(c->device));
  if (Ll) MG_CUDA(cudaMemcpyAsync(Ll, c->Ll, c->nX * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (nzval) MG_CUDA(cudaMemcpyAsync(nzval, c->nzval, c->pat.nnz * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  MG_CUDA(cudaStreamSynchronize(c->stream));
  return check_nan(c);
}

extern "C" int mgpu_assemble(mgpu_ctx* c, int32_t mission, int32_t nXder, const double* x, const double* u, double t,
                             const double* tvals, const mgpu_newmark* nm, double* Ll, double* nzval) {
  if (!c) return MGPU_ERR_ARG;
  MG_TRY(reset_errflag(c));
  MG_TRY(mgpu_upload_state(c, nXder, x, u, tvals));
  MG_TRY(mgpu_assemble_resident(c, mission, t, nm));
  return mgpu_download(c, Ll, nzval);
}

// Pipelined assembly.  Slot s = ticket mod 2 owns a device copy of the outputs
// (nzval, Lλ, NaN flag) and a page-locked staging area for the inputs.  The
// compute stream uploads the staged inputs into the resident state, assembles
// into the slot's outputs and records a_comp[s]; the copy stream then returns
// them to the caller's buffers and records a_d2h[s].  Slot s is reused two calls
// later, after its copies are done (host wait on a_h2d[s] before restaging,
// stream wait on a_d2h[s] before assembling into it again).
static int async_setup(mgpu_ctx* c) {
  if (c->cstream) return MGPU_OK;
  MG_CUDA(cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking));
  const size_t nst = size_t(3 * c->nX + c->nU + c->ntval);
  for (int k = 0; k < 2; ++k) {
    MG_CUDA(cudaMalloc(&c->anz[k], std::max<int64_t>(c->pat.nnz, 1) * sizeof(double)));
    MG_CUDA(cudaMalloc(&c->aLl[k], std::max<int64_t>(c->nX, 1) * sizeof(double)));
    MG_CUDA(cudaMallocHost(&c->astage[k], std::max<size_t>(nst, 1) * sizeof(double)));
    MG_CUDA(cudaEventCreateWithFlags(&c->a_h2d[k], cudaEventDisableTiming));
    MG_CUDA(cudaEventCreateWithFlags(&c->a_comp[k], cudaEventDisableTiming));
    MG_CUDA(cudaEventCreateWithFlags(&c->a_d2h[k], cudaEventDisableTiming));
  }
  MG_CUDA(cudaMalloc(&c->aerr, 2 * sizeof(int)));
  MG_CUDA(cudaMallocHost(&c->haerr, 2 * sizeof(int)));
  return MGPU_OK;
}

extern "C" int mgpu_assemble_async(mgpu_ctx* c, int32_t mission, int32_t nXder, const double* x, const double* u,
                                   double t, const double* tvals, const mgpu_newmark* nm, double* Ll, double* nzval,
                                   int64_t* ticket) {
  if (!c || !x || nXder < 1 || nXder > 3 || mission < 0 || mission > 2 || (mission != MGPU_ASM_STATIC && !nm))
    return set_err(c, MGPU_ERR_ARG, "mgpu_assemble_async: bad arguments");
  MG_CUDA(cudaSetDevice(c->device));
  MG_TRY(async_setup(c));
  const int64_t tk = c->aticket++;
  const int s = int(tk & 1);
  // the staging area and the outputs of this slot are free once its previous copies are done
  if (c->a_used[s]) MG_CUDA(cudaEventSynchronize(c->a_h2d[s]));
  double* st = c->astage[s];
  std::memcpy(st, x, size_t(nXder) * c->nX * sizeof(double));
  double* su = st + 3 * c->nX;
  double* stv = su + c->nU;
  if (c->nU > 0 && u) std::memcpy(su, u, c->nU * sizeof(double));
  if (c->ntval > 0 && tvals) std::memcpy(stv, tvals, c->ntval * sizeof(double));
  if (c->a_used[s]) MG_CUDA(cudaStreamWaitEvent(c->stream, c->a_d2h[s], 0));
  MG_TRY(mgpu_upload_state(c, nXder, st, (c->nU > 0 && u) ? su : nullptr, (c->ntval > 0 && tvals) ? stv : nullptr));
  MG_CUDA(cudaEventRecord(c->a_h2d[s], c->stream));
  MG_TRY(upload_stepc(c, t, mission != MGPU_ASM_STATIC ? nm : nullptr));
  // assemble into this slot's outputs (the kernels take the pointers at launch)
  double* nz0 = c->nzval;
  double* Ll0 = c->Ll;
  int* err0 = c->errflag;
  c->nzval = c->anz[s];
  c->Ll = c->aLl[s];
  c->errflag = c->aerr + s;
  launch_reset_errflag(c);
  const int rc = launch_assembly(c, mission, nullptr, 1.0);
  c->nzval = nz0;
  c->Ll = Ll0;
  c->errflag = err0;
  if (rc) return rc;
  MG_CUDA(cudaEventRecord(c->a_comp[s], c->stream));
  MG_CUDA(cudaStreamWaitEvent(c->cstream, c->a_comp[s], 0));
  if (Ll) MG_CUDA(cudaMemcpyAsync(Ll, c->aLl[s], c->nX * sizeof(double), cudaMemcpyDeviceToHost, c->cstream));
  if (nzval)
    MG_CUDA(cudaMemcpyAsync(nzval, c->anz[s], c->pat.nnz * sizeof(double), cudaMemcpyDeviceToHost, c->cstream));
  MG_CUDA(cudaMemcpyAsync(c->haerr + s, c->aerr + s, sizeof(int), cudaMemcpyDeviceToHost, c->cstream));
  MG_CUDA(cudaEventRecord(c->a_d2h[s], c->cstream));
  c->a_used[s] = true;
  if (ticket) *ticket = tk;
  return MGPU_OK;
}

extern "C" int mgpu_assemble_wait(mgpu_ctx* c, int64_t ticket) {
  if (!c || ticket < 0 || ticket >= c->aticket || ticket < c->aticket - 2)
    return set_err(c, MGPU_ERR_ARG, "mgpu_assemble_wait: ticket is not one of the last two assemblies");
  MG_CUDA(cudaSetDevice(c->device));
  const int s = int(ticket & 1);
  MG_CUDA(cudaEventSynchronize(c->a_d2h[s]));
  return nan_error(c, c->haerr[s]);
}

extern "C" int mgpu_time_assemble(mgpu_ctx* c, int32_t mission, double t, const mgpu_newmark* nm, int32_t reps,
                                  int32_t flush_l2, double* ms_total, double* ms_groups, double* ms_scatter) {
  if (!c || reps < 1 || (mission != MGPU_ASM_STATIC && !nm)) return set_err(c, MGPU_ERR_ARG, "mgpu_time_assemble: bad arguments");
  MG_CUDA(cudaSetDevice(c->device));
  if (flush_l2 && !c->flush) {
    c->flush_bytes = size_t(512) << 20;  // larger than the 129 MB L2
    MG_TRY(dalloc(c, reinterpret_cast<double**>(&c->flush), c->flush_bytes / 8));
  }
  MG_TRY(reset_errflag(c));
  MG_TRY(upload_stepc(c, t, mission != MGPU_ASM_STATIC ? nm : nullptr));
  const int ng = int(c->groups.size());
  const int ne = ng + 2;  // start, one per group, end
  std::vector<cudaEvent_t> ev(size_t(ne) * reps);
  for (auto& e : ev) MG_CUDA(cudaEventCreate(&e));
  for (int r = 0; r < reps; ++r) {
    if (flush_l2)
      fill_kernel<<<nblk(c->flush_bytes / 8, 256), 256, 0, c->stream>>>(c->flush, c->flush_bytes / 8, double(r));
    cudaEvent_t* E = &ev[size_t(ne) * r];
    MG_CUDA(cudaEventRecord(E[0], c->stream));
    MG_TRY(launch_assembly(c, mission, E + 1, 1.0));
    MG_CUDA(cudaEventRecord(E[ng + 1], c->stream));
  }
  MG_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<double> tg(ng, 0.0);
  double tt = 0, ts = 0;
  for (int r = 0; r < reps; ++r) {
    cudaEvent_t* E = &ev[size_t(ne) * r];
    float a = 0;
    cudaEventElapsedTime(&a, E[0], E[ng + 1]);
    tt += a;
    for (int g = 0; g < ng; ++g) {
      cudaEventElapsedTime(&a, E[g], E[g + 1]);
      tg[g] += a;
    }
    cudaEventElapsedTime(&a, E[ng], E[ng + 1]);
    ts += a;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (ms_total) *ms_total = tt / reps;
  if (ms_groups)
    for (int g = 0; g < ng; ++g) ms_groups[g] = tg[g] / reps;
  if (ms_scatter) *ms_scatter = ts / reps;
  return check_nan(c);
}

// Element-level evaluation (diffed_residual-like) for group g.
__global__ void eval_beam_kernel(int64_t nele, int nder, const double* X, const double* U, const double* cdata,
                                 double p0, double p1, double p2, double* R, double* dR, double* dRdU) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  BeamConst bc;
  load_soa(bc, cdata, nele, e);
  const double* Xe = X + e * nder * 12;
  double K[144], H[36];
  if (nder == 3)
    beam_element<true>(bc, Xe, Xe + 12, Xe + 24, U ? U + 3 * e : nullptr, Perturb{p0, p1, p2}, nullptr, nullptr,
                       R + 12 * e, K, nullptr, dRdU ? H : nullptr);
  else
    beam_element<false>(bc, Xe, Xe, Xe, U ? U + 3 * e : nullptr, Perturb{p0, p1, p2}, nullptr, nullptr, R + 12 * e, K,
                        nullptr, dRdU ? H : nullptr);
  for (int k = 0; k < 144; ++k) dR[144 * e + k] = K[k];
  if (dRdU)
    for (int k = 0; k < 36; ++k) dRdU[36 * e + k] = H[k];
}
__global__ void eval_bar_kernel(int64_t nele, int nder, const double* X, const double* U, const double* cdata, double t,
                                double p0, double p1, double p2, double* R, double* dR, double* dRdU) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  BarConst bc;
  load_soa(bc, cdata, nele, e);
  const double* Xe = X + e * nder * 6;
  double H[18];
  bar_element(bc, nder, Xe, Xe + 6, Xe + 12, U ? U + 3 * e : nullptr, t, p0, p1, p2, nullptr, nullptr, R + 6 * e,
              dR + 36 * e, nullptr, dRdU ? H : nullptr);
  if (dRdU)
    for (int k = 0; k < 18; ++k) dRdU[18 * e + k] = H[k];
}

extern "C" int mgpu_element_eval(mgpu_ctx* c, int32_t g, int32_t nXder, const double* X, const double* U, double t,
                                 double p0, double p1, double p2, double* R, double* dR, double* dRdU) {
  if (!c || g < 0 || g >= int32_t(c->groups.size()) || !X || !R || !dR || !(nXder == 1 || nXder == 3))
    return set_err(c, MGPU_ERR_ARG, "mgpu_element_eval: bad arguments (nXder must be 1 or 3)");
  const DevGroup& G = c->groups[g];
  if (G.kind != MGPU_EULERBEAM3D && G.kind != MGPU_BAR3D)
    return set_err(c, MGPU_ERR_ARG, "mgpu_element_eval: only beam and bar groups");
  MG_CUDA(cudaSetDevice(c->device));
  const int nX = G.nX;
  const int64_t n = G.nele;
  double *dX = nullptr, *dU = nullptr, *dRv = nullptr, *dK = nullptr, *dH = nullptr;
  MG_TRY(dalloc(c, &dX, size_t(n) * nXder * nX));
  MG_TRY(dalloc(c, &dRv, size_t(n) * nX));
  MG_TRY(dalloc(c, &dK, size_t(n) * nX * nX));
  const bool withU = U != nullptr;
  if (withU) {
    MG_TRY(dalloc(c, &dU, size_t(n) * 3));
    MG_TRY(dalloc(c, &dH, size_t(n) * nX * 3));
    MG_CUDA(cudaMemcpy(dU, U, n * 3 * sizeof(double), cudaMemcpyHostToDevice));
  }
  MG_CUDA(cudaMemcpy(dX, X, size_t(n) * nXder * nX * sizeof(double), cudaMemcpyHostToDevice));
  if (G.kind == MGPU_EULERBEAM3D)
    eval_beam_kernel<<<nblk(n, 64), 64, 0, c->stream>>>(n, nXder, dX, dU, G.cdata, p0, p1, p2, dRv, dK,
                                                         (withU && dRdU) ? dH : nullptr);
  else
    eval_bar_kernel<<<nblk(n, 64), 64, 0, c->stream>>>(n, nXder, dX, dU, G.cdata, t, p0, p1, p2, dRv, dK,
                                                        (withU && dRdU) ? dH : nullptr);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cudaStreamSynchronize(c->stream));
  MG_CUDA(cudaMemcpy(R, dRv, size_t(n) * nX * sizeof(double), cudaMemcpyDeviceToHost));
  MG_CUDA(cudaMemcpy(dR, dK, size_t(n) * nX * nX * sizeof(double), cudaMemcpyDeviceToHost));
  if (withU && dRdU) MG_CUDA(cudaMemcpy(dRdU, dH, size_t(n) * nX * 3 * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(dX);
  cudaFree(dU);
  cudaFree(dRv);
  cudaFree(dK);
  cudaFree(dH);
  return MGPU_OK;
}

// ------------------------------------------------------------------ element results
__global__ void beam_results_kernel(int64_t nele, int64_t nstate, int64_t nX, const int32_t* __restrict__ idx,
                                    const double* __restrict__ fields, const int32_t* __restrict__ aidx,
                                    const double* __restrict__ Avec, const double* __restrict__ X,
                                    double* __restrict__ out) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= nele * nstate) return;
  const int64_t e = q % nele, k = q / nele;
  double X0[12];
  for (int i = 0; i < 12; ++i) X0[i] = X[k * nX + __ldg(idx + i * nele + e)];
  const double a = aidx ? Avec[aidx[e]] : 1.0;
  beam_results(fields + e * BEAM_NFIELD, X0, a, out + q * 50);
}

extern "C" int mgpu_beam_results(mgpu_ctx* c, int32_t g, int64_t nstate, const double* X, double* out) {
  if (!c || g < 0 || g >= int32_t(c->groups.size()) || nstate < 0 || (nstate > 0 && (!X || !out)))
    return set_err(c, MGPU_ERR_ARG, "mgpu_beam_results: bad arguments");
  const DevGroup& G = c->groups[g];
  if (G.kind != MGPU_EULERBEAM3D) return set_err(c, MGPU_ERR_ARG, "mgpu_beam_results: not an EulerBeam3D group");
  const int64_t n = G.nele * nstate;
  if (n == 0) return MGPU_OK;
  MG_CUDA(cudaSetDevice(c->device));
  double *df = nullptr, *dX = nullptr, *dout = nullptr;
  auto cleanup = [&]() {
    cudaStreamSynchronize(c->stream);
    cudaFree(df);
    cudaFree(dX);
    cudaFree(dout);
  };
  cudaError_t e = cudaMalloc(&df, G.h_edata.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dX, size_t(nstate) * c->nX * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dout, size_t(n) * 50 * sizeof(double));
  if (e != cudaSuccess) {
    cleanup();
    return set_err(c, MGPU_ERR_NOMEM, std::string("mgpu_beam_results: ") + cudaGetErrorString(e));
  }
  e = cudaMemcpyAsync(df, G.h_edata.data(), G.h_edata.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dX, X, size_t(nstate) * c->nX * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    beam_results_kernel<<<nblk(n, 128), 128, 0, c->stream>>>(G.nele, nstate, c->nX, G.idx, df, G.aidx, c->Avec, dX,
                                                             dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, dout, size_t(n) * 50 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cleanup();
  if (e != cudaSuccess) return set_err(c, MGPU_ERR_CUDA, std::string("mgpu_beam_results: ") + cudaGetErrorString(e));
  return MGPU_OK;
}
