// Element-level Lagrangians with their first and second derivatives
// (mgpu_element_lagrangian), the analogue of diffed_lagrangian{2}
// (src/Diagnostic.jl:852-927) for the basic and cost elements.  DirectXUA
// differentiates each element's Lagrangian twice over its variables in the
// order Λ, X⁽⁰⁾..X⁽ᴼˣ⁾, U, A (revariate{2}, src/DirectXUA.jl:152-171) and adds
// the gradient and Hessian into its per-step blocks (:122-151).  Every
// Lagrangian here is at most quadratic in its variables, so the derivatives
// are written out:
//   DofLoad        L = Λ·R = −Λ₁ F(t)                       (src/BasicElements.jl:281-284)
//   DofConstraint  L = Σᵢ Λᵢ (−aᵢ μ) − Λ_μ (Σᵢ aᵢ xᵢ − c(t))  (R of :426-438, μ the multiplier dof)
//   DofCost        L = w (x⁽ᵈ⁾ − y(t))²                      (:32-50, :198-208 with a quadratic cost)
//   SingleUdof     L = w (u − y(t))² − Λ₁ u                  (:239-248)
//   Acost          L = w (a − y)²                            (:77-86, :163-167)
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace mgpu {

struct LagLayout {
  int nX, nXder, nU, nA, np;
  __device__ int lam(int i) const { return i; }
  __device__ int x(int d, int i) const { return nX + d * nX + i; }
  __device__ int u(int j) const { return nX * (1 + nXder) + j; }
  __device__ int a(int k) const { return nX * (1 + nXder) + nU + k; }
};

// one thread per element; g and h are zeroed by the caller
__global__ void lagrangian_kernel(int64_t nele, int kind, LagLayout ly, const double* __restrict__ cdata,
                                  const double* __restrict__ lam, const double* __restrict__ X,
                                  const double* __restrict__ U, const double* __restrict__ A,
                                  const double* __restrict__ tv, double* __restrict__ L, double* __restrict__ g,
                                  double* __restrict__ h) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  const int nX = ly.nX, np = ly.np;
  const double* Le = lam + e * nX;
  const double* Xe = X + e * int64_t(ly.nXder) * nX;
  const double* Ue = U + e * ly.nU;
  const double* Ae = A + e * ly.nA;
  double* ge = g ? g + e * np : nullptr;
  double* he = h ? h + e * int64_t(np) * np : nullptr;
  auto G = [&](int p, double v) {
    if (ge) ge[p] += v;
  };
  auto H = [&](int p, int q, double v) {
    if (!he) return;
    he[p + np * q] += v;
    if (p != q) he[q + np * p] += v;
  };
  double l = 0.0;
  switch (kind) {
    case MGPU_DOFLOAD: {
      const double F = tv[e];
      l = -Le[0] * F;
      G(ly.lam(0), -F);
      break;
    }
    case MGPU_DOFCONSTRAINT_X: {
      const int nx = nX - 1;
      const double mu = Xe[nx];
      double gap = -tv[e], sa = 0.0;
      for (int i = 0; i < nx; ++i) {
        const double ai = cdata[i * nele + e];
        gap += ai * Xe[i];
        sa += ai * Le[i];
      }
      for (int i = 0; i < nx; ++i) {
        const double ai = cdata[i * nele + e];
        l += Le[i] * (-ai * mu);
        G(ly.lam(i), -ai * mu);
        G(ly.x(0, i), -Le[nx] * ai);
        H(ly.lam(i), ly.x(0, nx), -ai);
        H(ly.lam(nx), ly.x(0, i), -ai);
      }
      l += -Le[nx] * gap;
      G(ly.lam(nx), -gap);
      G(ly.x(0, nx), -sa);
      break;
    }
    case MGPU_DOFCOST: {
      const double w = cdata[e];
      const int d = int(cdata[nele + e]);
      const double r = Xe[d * nX] - tv[e];
      l = w * r * r;
      G(ly.x(d, 0), 2.0 * w * r);
      H(ly.x(d, 0), ly.x(d, 0), 2.0 * w);
      break;
    }
    case MGPU_SINGLEUDOF: {
      const double w = cdata[e], u = Ue[0], r = u - tv[e];
      l = w * r * r - Le[0] * u;
      G(ly.lam(0), -u);
      G(ly.u(0), 2.0 * w * r - Le[0]);
      H(ly.u(0), ly.u(0), 2.0 * w);
      H(ly.lam(0), ly.u(0), -1.0);
      break;
    }
    case MGPU_ACOST: {
      const double w = cdata[e], r = Ae[0] - cdata[nele + e];
      l = w * r * r;
      G(ly.a(0), 2.0 * w * r);
      H(ly.a(0), ly.a(0), 2.0 * w);
      break;
    }
  }
  if (L) L[e] = l;
}

}  // namespace mgpu

using namespace mgpu;

extern "C" int mgpu_element_lagrangian(mgpu_ctx* c, int32_t ig, int32_t nXder, const double* lam, const double* X,
                                       const double* U, const double* A, const double* tv, double* L, double* dL,
                                       double* d2L) {
  if (!c || ig < 0 || ig >= int32_t(c->groups.size()) || nXder < 1 || nXder > 3)
    return set_err(c, MGPU_ERR_ARG, "mgpu_element_lagrangian: bad arguments (nXder must be 1, 2 or 3)");
  const DevGroup& Gr = c->groups[ig];
  const int kind = Gr.kind;
  if (kind == MGPU_EULERBEAM3D || kind == MGPU_BAR3D)
    return set_err(c, MGPU_ERR_UNSUPPORTED, "mgpu_element_lagrangian: beams and bars are residual elements "
                                            "without second order; use mgpu_element_eval");
  const int nX = Gr.nX, nU = Gr.nU, nA = kind == MGPU_ACOST ? 1 : 0;
  const int64_t n = Gr.nele;
  if ((nX > 0 && (!lam || !X)) || (nU > 0 && !U) || (nA > 0 && !A) || (has_tval(kind) && !tv))
    return set_err(c, MGPU_ERR_ARG, "mgpu_element_lagrangian: missing input");
  if (kind == MGPU_DOFCOST && Gr.maxder >= nXder)
    return set_err(c, MGPU_ERR_ARG, "mgpu_element_lagrangian: a DofCost reads a time derivative beyond nXder");
  LagLayout ly{nX, nXder, nU, nA, nX * (1 + nXder) + nU + nA};
  if (n == 0) return MGPU_OK;
  MG_CUDA(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  std::vector<void*> owned;
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    for (void* p : owned) cudaFree(p);
  };
  auto up = [&](const double* h, size_t cnt, double** d) -> bool {
    *d = nullptr;
    if (cudaMalloc(reinterpret_cast<void**>(d), std::max<size_t>(cnt, 1) * sizeof(double)) != cudaSuccess) return false;
    owned.push_back(*d);
    if (h && cnt > 0 && cudaMemcpyAsync(*d, h, cnt * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return false;
    if (!h && cudaMemsetAsync(*d, 0, std::max<size_t>(cnt, 1) * sizeof(double), st) != cudaSuccess) return false;
    return true;
  };
  const size_t np = size_t(ly.np);
  double *dlam, *dX, *dU, *dA, *dtv, *dLv, *dg, *dh;
  const bool ok = up(lam, size_t(n) * nX, &dlam) && up(X, size_t(n) * nXder * nX, &dX) && up(U, size_t(n) * nU, &dU) &&
                  up(A, size_t(n) * nA, &dA) && up(has_tval(kind) ? tv : nullptr, size_t(n), &dtv) &&
                  up(nullptr, size_t(n), &dLv) && up(nullptr, size_t(n) * np, &dg) &&
                  up(nullptr, d2L ? size_t(n) * np * np : 0, &dh);
  if (!ok) {
    cleanup();
    return set_err(c, MGPU_ERR_NOMEM, "mgpu_element_lagrangian: device allocation or copy failed");
  }
  lagrangian_kernel<<<unsigned((n + 127) / 128), 128, 0, st>>>(n, kind, ly, Gr.cdata, dlam, dX, dU, dA, dtv, dLv, dg,
                                                              d2L ? dh : nullptr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && L) e = cudaMemcpyAsync(L, dLv, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && dL) e = cudaMemcpyAsync(dL, dg, n * np * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && d2L) e = cudaMemcpyAsync(d2L, dh, n * np * np * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return set_err(c, MGPU_ERR_CUDA, std::string("mgpu_element_lagrangian: ") + cudaGetErrorString(e));
  return MGPU_OK;
}
