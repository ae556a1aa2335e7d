// Discrete adjoint of SweepX{OX} for cost sensitivities with respect to the
// A-dofs and the time values of the loads.
//
// The reference obtains ∂C/∂A in DirectXUA as the A-block of the Lagrangian
// gradient once the (Λ, X, U) blocks have converged (src/DirectXUA.jl:438-513),
// over an all-steps system with finite differences in time.  Here the time
// discretisation is the Newmark-β of SweepX (src/SweepX.jl:3-15, 98-132): the
// cost, the Lagrangian of the model's cost elements and of optional sensors,
//     C = Σ_n w_n [Σ_DofCost w_e (x_n⁽ᵈᵉ⁾[i_e] − y_e(t_n))² + Σ_SingleUdof w_e (u[j_e] − y_e(t_n))²
//                  + Σ_s c_s (x_n[d_s] − y_{n,s})²] + Σ_Acost w_e (a[k_e] − y_e)²,
// w_n = Δt_n (OX = 2) or 1 (OX = 0), is differentiated through the converged
// steps (the implicit-function adjoint of R(x_n, v_n(x_n, S_{n-1}),
// a_n(x_n, S_{n-1}); u, A) = 0):
//
//   g_n      = x̄_n + a1 v̄_n + b1 ā_n            (x̄_n, v̄_n, ā_n include ∂C/∂x_n, ∂C/∂v_n, ∂C/∂a_n)
//   J_nᵀ μ_n = g_n                               J_n = K + a1 C + b1 M at step n
//   dC/dA   −= μ_nᵀ ∂R_n/∂A,   dC/dF_n = −μ_nᵀ ∂R_n/∂F_n,   dC/du −= μ_nᵀ ∂R_n/∂u
//   p = v̄_n − C_nᵀ μ_n,   q = ā_n − M_nᵀ μ_n
//   x̄_{n-1} = −a1 p − b1 q,  v̄_{n-1} = (1 − a2) p − b2 q,  ā_{n-1} = −a3 p + (1 − b3) q
//
// with a1..b3 the Newmark coefficients of step n.  With dof scaling the
// device matrices are S J S and the residual S R: the solve uses S g and the
// products S⁻¹ (S C S)ᵀ μ.  States are recomputed from √N checkpoints: the
// forward pass keeps the state at the start of every segment of `ckpt` steps;
// the reverse pass recomputes one segment (the same deterministic kernels, so
// the same iterates bit for bit) and walks back through it.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "beam_math.hpp"
#include "solver.hpp"

namespace mgpu {

// Σ_s c_s (x[d_s] − y_s)², one block, fixed order
__global__ void __launch_bounds__(256) adj_cost_value(int64_t ncost, const int32_t* __restrict__ dof,
                                                      const double* __restrict__ cw, const double* __restrict__ y,
                                                      const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double sm[256];
  double a = 0.0;
  for (int64_t s = threadIdx.x; s < ncost; s += 256) {
    const double r = x[dof[s]] - y[s];
    a += cw[s] * r * r;
  }
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) sm[threadIdx.x] += sm[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

// x̄[d_s] += f · 2 c_s (x[d_s] − y_s)   (sensor dofs are distinct)
__global__ void adj_cost_grad(int64_t ncost, const int32_t* __restrict__ dof, const double* __restrict__ cw,
                              const double* __restrict__ y, const double* __restrict__ x, double f,
                              double* __restrict__ xb) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s < ncost) xb[dof[s]] += f * 2.0 * cw[s] * (x[dof[s]] - y[s]);
}

// Σ_e w_e (v_e − y_e)² over a DofCost group (v = x⁽ᵈᵉ⁾[i_e]) or a SingleUdof
// group (v = u[j_e]); cdata holds w (and d), tv the targets.  One block, fixed order.
__global__ void __launch_bounds__(256) adj_group_cost(int64_t nele, int udof, const int32_t* __restrict__ idx,
                                                      const int32_t* __restrict__ uidx,
                                                      const double* __restrict__ cdata,
                                                      const double* __restrict__ tv, const double* __restrict__ x,
                                                      int64_t nX, const double* __restrict__ u,
                                                      double* __restrict__ out) {
  __shared__ double sm[256];
  double a = 0.0;
  for (int64_t e = threadIdx.x; e < nele; e += 256) {
    const double v = udof ? u[uidx[e]] : x[int64_t(cdata[nele + e]) * nX + idx[e]];
    const double r = v - tv[e];
    a += cdata[e] * r * r;
  }
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) sm[threadIdx.x] += sm[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

// Step n's direct partials of a cost group, scaled by the step weight f:
// DofCost: x̄/v̄/ā[i_e] += f 2 w_e (x⁽ᵈᵉ⁾ − y_e);  SingleUdof: ū[j_e] += f 2 w_e (u − y_e)
// and ū[j_e] += μ[i_e] s_i (R = −u s on the X-dof);  dC/dy_e = −f 2 w_e (v − y_e)
// into dtv (may be null).  `serial`: one thread walks the elements in order
// (groups in which two elements write the same entry), else one per element.
__global__ void adj_group_grad(int64_t nele, int udof, int serial, const int32_t* __restrict__ idx,
                               const int32_t* __restrict__ uidx, const double* __restrict__ cdata,
                               const double* __restrict__ tv, const double* __restrict__ x, int64_t nX,
                               const double* __restrict__ u, const double* __restrict__ mu,
                               const double* __restrict__ scale, double f, double* __restrict__ xb,
                               double* __restrict__ vb, double* __restrict__ ab, double* __restrict__ ub,
                               double* __restrict__ dtv) {
  const int64_t e0 = serial ? 0 : int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t e1 = serial ? nele : e0 + 1;
  for (int64_t e = e0; e < e1 && e < nele; ++e) {
    const int i = idx[e];
    if (udof) {
      const int j = uidx[e];
      const double r = u[j] - tv[e];
      ub[j] += f * 2.0 * cdata[e] * r + mu[i] * (scale ? scale[i] : 1.0);
      if (dtv) dtv[e] = -f * 2.0 * cdata[e] * r;
    } else {
      const int d = int(cdata[nele + e]);
      const double r = x[int64_t(d) * nX + i] - tv[e];
      double* bar = d == 0 ? xb : d == 1 ? vb : ab;
      bar[i] += f * 2.0 * cdata[e] * r;
      if (dtv) dtv[e] = -f * 2.0 * cdata[e] * r;
    }
  }
}

// The once-off A-costs: cost += Σ_e w_e (a[k_e] − y_e)², dC/da[k_e] += 2 w_e (a − y_e), in element order.
__global__ void adj_acost(int64_t nele, const int32_t* __restrict__ aidx, const double* __restrict__ cdata,
                          const double* __restrict__ A, double* __restrict__ gradA, double* __restrict__ cost) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double c = 0.0;
  for (int64_t e = 0; e < nele; ++e) {
    const double r = A[aidx[e]] - cdata[nele + e];
    c += cdata[e] * r * r;
    gradA[aidx[e]] += 2.0 * cdata[e] * r;
  }
  *cost = c;
}

// g = S (x̄ + a1 v̄ + b1 ā)
__global__ void adj_rhs(int64_t n, int OX, double a1, double b1, const double* __restrict__ scale,
                        const double* __restrict__ xb, const double* __restrict__ vb, const double* __restrict__ ab,
                        double* __restrict__ g) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = xb[i];
  if (OX == 2) v += a1 * vb[i] + b1 * ab[i];
  g[i] = v * (scale ? scale[i] : 1.0);
}

// y_j = S⁻¹_j Σ_q nz[q] μ[row[q]] over column j (the transposed product, one thread per column)
__global__ void adj_csc_tmatvec(int64_t n, const int64_t* __restrict__ colptr, const int32_t* __restrict__ rowval,
                                const double* __restrict__ nz, const double* __restrict__ mu,
                                const double* __restrict__ scale, double* __restrict__ y) {
  const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double s = 0.0;
  for (int64_t q = colptr[j]; q < colptr[j + 1]; ++q) s += nz[q] * mu[rowval[q]];
  y[j] = scale ? s / scale[j] : s;
}

__global__ void adj_propagate(int64_t n, double a1, double a2, double a3, double b1, double b2, double b3,
                              const double* __restrict__ tC, const double* __restrict__ tM, double* __restrict__ xb,
                              double* __restrict__ vb, double* __restrict__ ab) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p = vb[i] - tC[i], q = ab[i] - tM[i];
  xb[i] = -a1 * p - b1 * q;
  vb[i] = (1.0 - a2) * p - b2 * q;
  ab[i] = -a3 * p + (1.0 - b3) * q;
}

// Per EI-scaled beam: contrib[e] = −μᵀ ∂(S R_e)/∂A_e.  R is linear in the
// bending constants, so ∂R_e/∂A_e is the residual of the element with every
// other stiffness, mass and load term set to zero (the state's bending forces).
__global__ void __launch_bounds__(128) adj_beam_dRdA(int64_t nele, const int32_t* __restrict__ idx,
                                                     const double* __restrict__ cdata, const double* __restrict__ x0,
                                                     const double* __restrict__ mu,
                                                     const double* __restrict__ scale, double* __restrict__ contrib) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  BeamConst bc;
  double* d = reinterpret_cast<double*>(&bc);
  for (int f = 0; f < int(sizeof(BeamConst) / sizeof(double)); ++f) d[f] = __ldg(cdata + f * nele + e);
  bc.ke = 0.0;
  bc.kt = 0.0;
  bc.mu = 0.0;
  bc.iota1 = 0.0;
  bc.w = 0.0;
  for (int k = 0; k < 3; ++k) bc.Ca[k] = bc.Cl[k] = bc.Cq[k] = 0.0;
  int dof[12];
  double X0[12], R[12], K[144];
  for (int i = 0; i < 12; ++i) {
    dof[i] = __ldg(idx + i * nele + e);
    X0[i] = __ldg(x0 + dof[i]);
  }
  beam_element<false>(bc, X0, X0, X0, nullptr, Perturb{1.0, 0.0, 0.0}, nullptr, nullptr, R, K, nullptr, nullptr);
  double s = 0.0;
  for (int i = 0; i < 12; ++i) s += mu[dof[i]] * R[i] * (scale ? scale[dof[i]] : 1.0);
  contrib[e] = -s;
}

// gradA[a] += Σ contrib over the elements of A-dof a (in element order)
__global__ void adj_agrad(int64_t nA, const int64_t* __restrict__ aptr, const int32_t* __restrict__ aele,
                          const double* __restrict__ contrib, double* __restrict__ gradA) {
  const int64_t a = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (a >= nA) return;
  double s = 0.0;
  for (int64_t q = aptr[a]; q < aptr[a + 1]; ++q) s += contrib[aele[q]];
  gradA[a] += s;
}

// dC/dF for DofLoad (R = −F s) and for the offset c of DofConstraint (R_λ = −(Σaᵢxᵢ − c) s_λ)
__global__ void adj_dtv(int64_t nele, int nX, int sign, const int32_t* __restrict__ idx,
                        const double* __restrict__ mu, const double* __restrict__ scale, double* __restrict__ out) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  const int d = __ldg(idx + int64_t(nX - 1) * nele + e);
  out[e] = sign * mu[d] * (scale ? scale[d] : 1.0);
}

}  // namespace mgpu

using namespace mgpu;

extern "C" int mgpu_adjoint_sweepx(mgpu_ctx* c, int32_t OX, int64_t nstep, const double* times, double t0,
                                   int32_t nXder0, const double* x0, const double* u, const double* tvals,
                                   const mgpu_sweep_opts* opts, int64_t ncost, const int64_t* cost_dof,
                                   const double* cost_w, const double* cost_y, int32_t ckpt, double* cost,
                                   double* dCdA, double* dCdtv, double* dCdU, mgpu_stats* stats) {
  if (!c || !times || !opts || !stats || !cost || !(OX == 0 || OX == 2) || nstep < 1 || nXder0 < 0 ||
      nXder0 > OX + 1 || (nXder0 > 0 && !x0) || ncost < 0 || (ncost > 0 && (!cost_dof || !cost_w || !cost_y)) ||
      (c->ntval > 0 && !tvals) || (c->nA > 0 && !dCdA))
    return set_err(c, MGPU_ERR_ARG, "mgpu_adjoint_sweepx: bad arguments");
  if (opts->fixed_iter > 0 || opts->per_component)
    return set_err(c, MGPU_ERR_ARG, "mgpu_adjoint_sweepx: the adjoint needs converged steps (fixed_iter = 0, "
                                    "per_component = 0)");
  *stats = mgpu_stats{0, 0, 0, 0, 0.0, 0.0};
  // cost element groups
  std::vector<int> cgroups;  // DofCost and SingleUdof groups, model order
  for (size_t gi = 0; gi < c->groups.size(); ++gi) {
    const DevGroup& G = c->groups[gi];
    if ((G.kind == MGPU_DOFCOST || G.kind == MGPU_SINGLEUDOF) && G.nele > 0) cgroups.push_back(int(gi));
    if (G.kind == MGPU_DOFCOST && G.nele > 0 && G.maxder > OX)
      return set_err(c, MGPU_ERR_ARG, "mgpu_adjoint_sweepx: a DofCost on a time derivative of X needs OX = 2");
    if (dCdU && (G.kind == MGPU_EULERBEAM3D || G.kind == MGPU_BAR3D) && G.nU > 0 && G.nele > 0)
      return set_err(c, MGPU_ERR_UNSUPPORTED, "mgpu_adjoint_sweepx: dCdU covers the U-dofs of SingleUdof elements; "
                                              "this model has beams or bars with U-dofs");
  }
  const int64_t ncs = 1 + int64_t(cgroups.size());  // per step: sensors, then each cost group
  Solver& S = *c->solver;
  if (!S.ok) return set_err(c, MGPU_ERR_UNSUPPORTED, "no device solver for this model: " + S.why);
  if (!S.wmT)
    return set_err(c, MGPU_ERR_UNSUPPORTED, "the adjoint needs the row-band solver (kl, ku <= 31, kl+ku+1 <= 64)");
  const int64_t n = c->nX;
  std::vector<int32_t> cdof(ncost);
  {
    std::vector<char> seen(n, 0);
    for (int64_t s = 0; s < ncost; ++s) {
      if (cost_dof[s] < 1 || cost_dof[s] > n) return set_err(c, MGPU_ERR_ARG, "cost dof out of range");
      if (seen[cost_dof[s] - 1]++) return set_err(c, MGPU_ERR_ARG, "cost dofs must be distinct");
      cdof[s] = int32_t(cost_dof[s] - 1);
    }
  }
  MG_CUDA(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  if (ckpt <= 0) ckpt = int32_t(std::ceil(std::sqrt(double(nstep))));
  ckpt = int32_t(std::min<int64_t>(ckpt, nstep));
  const int64_t nseg = (nstep + ckpt - 1) / ckpt;
  // A-dof -> beams (CSR over the EI-scaled beams of all groups, element order)
  std::vector<int64_t> aptr(c->nA + 1, 0);
  std::vector<int32_t> aele;
  std::vector<int64_t> abase;  // per group: offset of its beams in contrib (-1 if none)
  int64_t nbA = 0;
  for (auto& G : c->groups) {  // the EI-scaled beams (an Acost's A-dof enters through adj_acost)
    const bool eib = G.kind == MGPU_EULERBEAM3D && G.aidx;
    abase.push_back(eib ? nbA : -1);
    if (eib) nbA += G.nele;
  }
  {
    std::vector<std::vector<int32_t>> lists(c->nA);
    for (size_t g = 0; g < c->groups.size(); ++g)
      if (abase[g] >= 0)
        for (int64_t e = 0; e < c->groups[g].nele; ++e)
          lists[c->groups[g].h_indexA[e] - 1].push_back(int32_t(abase[g] + e));
    for (int64_t a = 0; a < c->nA; ++a) {
      aptr[a + 1] = aptr[a] + int64_t(lists[a].size());
      aele.insert(aele.end(), lists[a].begin(), lists[a].end());
    }
  }
  // device buffers
  std::vector<void*> owned;
  int rc = MGPU_OK;
  auto alloc = [&](auto** p, size_t count) -> bool {
    using T = typename std::remove_pointer<typename std::remove_reference<decltype(*p)>::type>::type;
    if (cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return false;
    owned.push_back(*p);
    return true;
  };
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    for (void* p : owned) cudaFree(p);
    cudaGetLastError();
  };
  const size_t ns = size_t(3) * n;
  double *ck, *seg, *xb, *vb, *ab, *g, *mu, *tC, *tM, *costs, *cw, *cy, *gradA, *contrib, *ub, *acost,
      *dtv = nullptr;
  int32_t *dcd, *aeled, *rowv;
  int64_t *aptrd, *colp;
  bool ok = alloc(&ck, nseg * ns) && alloc(&seg, size_t(ckpt) * ns) && alloc(&xb, n) && alloc(&vb, n) &&
            alloc(&ab, n) && alloc(&g, n) && alloc(&mu, n) && alloc(&tC, n) && alloc(&tM, n) &&
            alloc(&costs, nstep * ncs) && alloc(&ub, c->nU) && alloc(&acost, 1) && alloc(&cw, ncost) && alloc(&cy, size_t(nstep) * ncost) &&
            alloc(&gradA, c->nA) && alloc(&contrib, nbA) && alloc(&dcd, ncost) && alloc(&aeled, aele.size()) &&
            alloc(&aptrd, aptr.size()) && alloc(&colp, n + 1) && alloc(&rowv, c->pat.nnz);
  if (ok && dCdtv && c->ntval > 0) ok = alloc(&dtv, size_t(nstep) * c->ntval);
  if (!ok) {
    cleanup();
    return set_err(c, MGPU_ERR_NOMEM, "device allocation failed for the adjoint");
  }
  {
    std::vector<int32_t> rv(c->pat.rowval.begin(), c->pat.rowval.end());
    ok = cudaMemcpy(colp, c->pat.colptr.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(rowv, rv.data(), rv.size() * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess &&
         (ncost == 0 ||
          (cudaMemcpy(dcd, cdof.data(), ncost * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess &&
           cudaMemcpy(cw, cost_w, ncost * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
           cudaMemcpy(cy, cost_y, size_t(nstep) * ncost * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess)) &&
         cudaMemcpy(aptrd, aptr.data(), aptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess &&
         (aele.empty() ||
          cudaMemcpy(aeled, aele.data(), aele.size() * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess) &&
         cudaMemsetAsync(gradA, 0, std::max<int64_t>(c->nA, 1) * sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(ub, 0, std::max<int64_t>(c->nU, 1) * sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(acost, 0, sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(costs, 0, nstep * ncs * sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(xb, 0, n * sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(vb, 0, n * sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(ab, 0, n * sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(tC, 0, n * sizeof(double), st) == cudaSuccess &&
         cudaMemsetAsync(tM, 0, n * sizeof(double), st) == cudaSuccess;
    if (!ok) {
      cleanup();
      return set_err(c, MGPU_ERR_CUDA, "adjoint: upload failed");
    }
  }
#define ADJ_TRY(x)  \
  do {              \
    rc = (x);       \
    if (rc) {       \
      cleanup();    \
      return rc;    \
    }               \
  } while (0)
#define ADJ_CUDA(call)                                                                                  \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) {                                                                            \
      rc = set_err(c, MGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));               \
      cleanup();                                                                                        \
      return rc;                                                                                        \
    }                                                                                                   \
  } while (0)
  // initial state
  ADJ_CUDA(cudaMemsetAsync(c->x, 0, ns * sizeof(double), st));
  if (nXder0 > 0) ADJ_CUDA(cudaMemcpyAsync(c->x, x0, nXder0 * n * sizeof(double), cudaMemcpyHostToDevice, st));
  if (c->nU > 0 && u) ADJ_CUDA(cudaMemcpyAsync(c->u, u, c->nU * sizeof(double), cudaMemcpyHostToDevice, st));
  c->nXder_resident = OX + 1;
  auto tprev = [&](int64_t k) { return k == 0 ? t0 : times[k - 1]; };  // time of the state before step k+1
  auto tvk = [&](int64_t k) { return c->ntval > 0 ? tvals + k * c->ntval : nullptr; };
  // ---- forward pass: checkpoints and costs
  for (int64_t k = 0; k < nstep; ++k) {
    if (k % ckpt == 0) ADJ_CUDA(cudaMemcpyAsync(ck + (k / ckpt) * ns, c->x, ns * sizeof(double),
                                               cudaMemcpyDeviceToDevice, st));
    const double t = times[k], dt = t - tprev(k);
    if (OX > 0 && !(dt > 0)) {
      cleanup();
      return set_err(c, MGPU_ERR_ARG, "Time step length not strictly positive at step=" + std::to_string(k + 1));
    }
    ADJ_TRY(newton_step(c, OX, k, t, dt, tvk(k), opts, stats));
    stats->nstep_done = int(k + 1);
    if (ncost > 0) adj_cost_value<<<1, 256, 0, st>>>(ncost, dcd, cw, cy + k * ncost, c->x, costs + k * ncs);
    for (size_t q = 0; q < cgroups.size(); ++q) {
      const DevGroup& G = c->groups[cgroups[q]];
      adj_group_cost<<<1, 256, 0, st>>>(G.nele, G.kind == MGPU_SINGLEUDOF, G.idx, G.uidx, G.cdata,
                                        c->tv + G.tval_base, c->x, n, c->u, costs + k * ncs + 1 + q);
    }
  }
  {
    std::vector<double> hc(nstep * ncs, 0.0);
    // the context stream does not synchronise with the legacy stream: copy on it and wait
    ADJ_CUDA(cudaMemcpyAsync(hc.data(), costs, nstep * ncs * sizeof(double), cudaMemcpyDeviceToHost, st));
    ADJ_CUDA(cudaStreamSynchronize(st));
    double C = 0.0;
    for (int64_t k = 0; k < nstep; ++k) {
      double ck_ = 0.0;
      for (int64_t q = 0; q < ncs; ++q) ck_ += hc[k * ncs + q];
      C += (OX == 2 ? times[k] - tprev(k) : 1.0) * ck_;
    }
    *cost = C;
  }
  // ---- reverse pass, segment by segment
  mgpu_stats rstats{0, 0, 0, 0, 0.0, 0.0};
  for (int64_t sgi = nseg - 1; sgi >= 0; --sgi) {
    const int64_t k0 = sgi * ckpt, k1 = std::min<int64_t>(nstep, k0 + ckpt);
    ADJ_CUDA(cudaMemcpyAsync(c->x, ck + sgi * ns, ns * sizeof(double), cudaMemcpyDeviceToDevice, st));
    for (int64_t k = k0; k < k1; ++k) {
      ADJ_TRY(newton_step(c, OX, k, times[k], times[k] - tprev(k), tvk(k), opts, &rstats));
      ADJ_CUDA(cudaMemcpyAsync(seg + (k - k0) * ns, c->x, ns * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    for (int64_t k = k1 - 1; k >= k0; --k) {
      const double t = times[k], dt = t - tprev(k), wk = OX == 2 ? dt : 1.0;
      const mgpu_newmark nm = OX == 2 ? newmark_coefficients(opts->beta, opts->gamma, dt) : mgpu_newmark{0, 0, 0, 0, 0, 0};
      ADJ_CUDA(cudaMemcpyAsync(c->x, seg + (k - k0) * ns, ns * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if (c->ntval > 0)
        ADJ_CUDA(cudaMemcpyAsync(c->tv, tvk(k), c->ntval * sizeof(double), cudaMemcpyHostToDevice, st));
      if (ncost > 0)
        adj_cost_grad<<<nb(ncost, 256), 256, 0, st>>>(ncost, dcd, cw, cy + k * ncost, c->x, wk, xb);
      for (int gi : cgroups) {  // DofCost partials (SingleUdof's need μ, below)
        const DevGroup& G = c->groups[gi];
        if (G.kind != MGPU_DOFCOST) continue;
        double* dt = dtv ? dtv + k * c->ntval + G.tval_base : nullptr;
        if (G.distinct)
          adj_group_grad<<<nb(G.nele, 256), 256, 0, st>>>(G.nele, 0, 0, G.idx, nullptr, G.cdata, c->tv + G.tval_base,
                                                          c->x, n, c->u, nullptr, c->scale, wk, xb, vb, ab, ub, dt);
        else
          adj_group_grad<<<1, 1, 0, st>>>(G.nele, 0, 1, G.idx, nullptr, G.cdata, c->tv + G.tval_base, c->x, n, c->u,
                                          nullptr, c->scale, wk, xb, vb, ab, ub, dt);
      }
      adj_rhs<<<nb(n, 256), 256, 0, st>>>(n, OX, nm.a1, nm.b1, c->scale, xb, vb, ab, g);
      // μ = J⁻ᵀ S g
      ADJ_TRY(upload_stepc(c, t, OX == 2 ? &nm : nullptr));
      launch_reset_errflag(c);
      ADJ_CUDA(cudaMemsetAsync(S.info, 0, sizeof(int), st));
      ADJ_TRY(launch_assembly(c, OX == 2 ? MGPU_ASM_ITER : MGPU_ASM_STATIC, nullptr, 1.0));
      ADJ_TRY(factor_solve_T(c, g, mu, S.info));
      // EI-scale sensitivities
      for (size_t gi = 0; gi < c->groups.size(); ++gi)
        if (abase[gi] >= 0 && c->groups[gi].nele > 0) {
          const DevGroup& G = c->groups[gi];
          adj_beam_dRdA<<<nb(G.nele, 128), 128, 0, st>>>(G.nele, G.idx, G.cdata, c->x, mu, c->scale,
                                                         contrib + abase[gi]);
        }
      if (c->nA > 0) adj_agrad<<<nb(c->nA, 256), 256, 0, st>>>(c->nA, aptrd, aeled, contrib, gradA);
      // U-dof sensitivities of SingleUdof: the cost's partial and −μᵀ∂R/∂u
      for (int gi : cgroups) {
        const DevGroup& G = c->groups[gi];
        if (G.kind != MGPU_SINGLEUDOF) continue;
        double* dt = dtv ? dtv + k * c->ntval + G.tval_base : nullptr;
        if (G.distinct)
          adj_group_grad<<<nb(G.nele, 256), 256, 0, st>>>(G.nele, 1, 0, G.idx, G.uidx, G.cdata, c->tv + G.tval_base,
                                                          c->x, n, c->u, mu, c->scale, wk, xb, vb, ab, ub, dt);
        else
          adj_group_grad<<<1, 1, 0, st>>>(G.nele, 1, 1, G.idx, G.uidx, G.cdata, c->tv + G.tval_base, c->x, n, c->u,
                                          mu, c->scale, wk, xb, vb, ab, ub, dt);
      }
      // load-value sensitivities
      if (dtv) {
        for (auto& G : c->groups) {
          if (G.kind == MGPU_DOFLOAD && G.nele > 0)
            adj_dtv<<<nb(G.nele, 256), 256, 0, st>>>(G.nele, 1, 1, G.idx, mu, c->scale,
                                                     dtv + k * c->ntval + G.tval_base);
          if (G.kind == MGPU_DOFCONSTRAINT_X && G.nele > 0)
            adj_dtv<<<nb(G.nele, 256), 256, 0, st>>>(G.nele, G.nX, -1, G.idx, mu, c->scale,
                                                     dtv + k * c->ntval + G.tval_base);
        }
      }
      if (OX == 2) {
        // Cᵀ μ and Mᵀ μ from the damping and mass matrices of the step
        const mgpu_newmark onlyC{1.0, 0, 0, 0.0, 0, 0}, onlyM{0.0, 0, 0, 1.0, 0, 0};
        ADJ_TRY(upload_stepc(c, t, &onlyC));
        ADJ_TRY(launch_assembly(c, MGPU_ASM_ITER, nullptr, 0.0));
        adj_csc_tmatvec<<<nb(n, 256), 256, 0, st>>>(n, colp, rowv, c->nzval, mu, c->scale, tC);
        ADJ_TRY(upload_stepc(c, t, &onlyM));
        ADJ_TRY(launch_assembly(c, MGPU_ASM_ITER, nullptr, 0.0));
        adj_csc_tmatvec<<<nb(n, 256), 256, 0, st>>>(n, colp, rowv, c->nzval, mu, c->scale, tM);
        adj_propagate<<<nb(n, 256), 256, 0, st>>>(n, nm.a1, nm.a2, nm.a3, nm.b1, nm.b2, nm.b3, tC, tM, xb, vb, ab);
      } else {
        ADJ_CUDA(cudaMemsetAsync(xb, 0, n * sizeof(double), st));
      }
      int hinfo = 0, hflag = INT_MAX;
      ADJ_CUDA(cudaMemcpyAsync(&hinfo, S.info, sizeof(int), cudaMemcpyDeviceToHost, st));
      ADJ_CUDA(cudaMemcpyAsync(&hflag, c->errflag, sizeof(int), cudaMemcpyDeviceToHost, st));
      ADJ_CUDA(cudaStreamSynchronize(st));
      if (hflag != INT_MAX) {
        rc = nan_error(c, hflag);
        cleanup();
        return rc;
      }
      if (hinfo != 0) {
        cleanup();
        return set_err(c, MGPU_ERR_SINGULAR, "adjoint: transposed factorization failed at step=" + std::to_string(k + 1));
      }
    }
  }
  // the once-off A-costs, in group order
  for (const DevGroup& G : c->groups)
    if (G.kind == MGPU_ACOST && G.nele > 0) {
      adj_acost<<<1, 1, 0, st>>>(G.nele, G.aidx, G.cdata, c->Avec, gradA, acost);
      double ha = 0.0;
      ADJ_CUDA(cudaMemcpyAsync(&ha, acost, sizeof(double), cudaMemcpyDeviceToHost, st));
      ADJ_CUDA(cudaStreamSynchronize(st));
      *cost += ha;
    }
  ADJ_CUDA(cudaStreamSynchronize(st));
  if (c->nA > 0) ADJ_CUDA(cudaMemcpy(dCdA, gradA, c->nA * sizeof(double), cudaMemcpyDeviceToHost));
  if (dCdU && c->nU > 0) ADJ_CUDA(cudaMemcpy(dCdU, ub, c->nU * sizeof(double), cudaMemcpyDeviceToHost));
  if (dtv) ADJ_CUDA(cudaMemcpy(dCdtv, dtv, size_t(nstep) * c->ntval * sizeof(double), cudaMemcpyDeviceToHost));
  cleanup();
#undef ADJ_TRY
#undef ADJ_CUDA
  return MGPU_OK;
}

// ====================================================================== forward sensitivities
// The forward-mode counterpart of the adjoint above: for a few A-dofs θ, the
// derivatives of the converged states, step by step.  Differentiating
// R(xₙ, vₙ, aₙ; θ) = 0 with vₙ = a1 xₙ + gᵥ(Sₙ₋₁), aₙ = b1 xₙ + gₐ(Sₙ₋₁):
//   Jₙ sₓ = −∂R/∂θ − Cₙ gᵥ′ − Mₙ gₐ′,   sᵥ = a1 sₓ + gᵥ′,   sₐ = b1 sₓ + gₐ′
//   gᵥ′ = −a1 sₓ⁻ + (1 − a2) sᵥ⁻ − a3 sₐ⁻,   gₐ′ = −b1 sₓ⁻ − b2 sᵥ⁻ + (1 − b3) sₐ⁻
// (⁻ the previous step's sensitivities, zero before the first), and
// dC/dθ = Σₙ wₙ (∂cₙ/∂x·sₓ + ∂cₙ/∂v·sᵥ + ∂cₙ/∂a·sₐ) + ∂C_A/∂θ.  This is what
// SweepXA assembles for its sensitivity solve (src/SweepXA.jl:49-221), here
// on the Newmark discretisation of SweepX.

namespace mgpu {

// Σ_i a[i] b[i] over one block in a fixed order, added to *out
__global__ void __launch_bounds__(256) sens_dot_add(int64_t n, const double* __restrict__ a,
                                                    const double* __restrict__ b, double* __restrict__ out) {
  __shared__ double sm[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += 256) s += a[i] * b[i];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) sm[threadIdx.x] += sm[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out += sm[0];
}

// gᵥ′, gₐ′ from the previous sensitivities; gv/ga scaled by 1/S for the products with S X S
__global__ void sens_carry(int64_t n, double a1, double a2, double a3, double b1, double b2, double b3,
                           const double* __restrict__ sx, const double* __restrict__ sv, const double* __restrict__ sa,
                           const double* __restrict__ scale, double* __restrict__ gv, double* __restrict__ ga,
                           double* __restrict__ gvs, double* __restrict__ gas) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = -a1 * sx[i] + (1.0 - a2) * sv[i] - a3 * sa[i];
  const double a = -b1 * sx[i] - b2 * sv[i] + (1.0 - b3) * sa[i];
  gv[i] = v;
  ga[i] = a;
  const double s = scale ? scale[i] : 1.0;
  gvs[i] = v / s;
  gas[i] = a / s;
}

// rhs_i −= Σ_t nz[rq[t]] x[rcol[t]] over row i (CSR of the pattern, fixed order)
__global__ void sens_csr_sub(int64_t n, const int64_t* __restrict__ rptr, const int32_t* __restrict__ rq,
                             const int32_t* __restrict__ rcol, const double* __restrict__ nz,
                             const double* __restrict__ x, double* __restrict__ rhs) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int64_t t = rptr[i]; t < rptr[i + 1]; ++t) s += nz[rq[t]] * x[rcol[t]];
  rhs[i] -= s;
}

// ∂R_e/∂θ of the listed EI-scaled beams (the bending-only residual, R being
// linear in the bending stiffnesses), one thread per beam, into Re[list][12]
__global__ void __launch_bounds__(128) sens_beam_dRdA(int64_t nlist, const int32_t* __restrict__ list,
                                                      int64_t nele, const int32_t* __restrict__ idx,
                                                      const double* __restrict__ cdata,
                                                      const double* __restrict__ x0, double* __restrict__ Re) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= nlist) return;
  const int64_t e = list[q];
  BeamConst bc;
  double* d = reinterpret_cast<double*>(&bc);
  for (int f = 0; f < int(sizeof(BeamConst) / sizeof(double)); ++f) d[f] = __ldg(cdata + f * nele + e);
  bc.ke = 0.0;
  bc.kt = 0.0;
  bc.mu = 0.0;
  bc.iota1 = 0.0;
  bc.w = 0.0;
  for (int k = 0; k < 3; ++k) bc.Ca[k] = bc.Cl[k] = bc.Cq[k] = 0.0;
  double X0[12], R[12], K[144];
  for (int i = 0; i < 12; ++i) X0[i] = __ldg(x0 + __ldg(idx + i * nele + e));
  beam_element<false>(bc, X0, X0, X0, nullptr, Perturb{1.0, 0.0, 0.0}, nullptr, nullptr, R, K, nullptr, nullptr);
  for (int i = 0; i < 12; ++i) Re[q * 12 + i] = R[i];
}

// rhs[d] −= S_d Re[q][i] over the beams q of one θ, in list order (one thread)
__global__ void sens_beam_rhs(int64_t q0, int64_t q1, const int32_t* __restrict__ list, int64_t nele,
                              const int32_t* __restrict__ idx, const double* __restrict__ Re,
                              const double* __restrict__ scale, double* __restrict__ rhs) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int64_t q = q0; q < q1; ++q) {
    const int64_t e = list[q];
    for (int i = 0; i < 12; ++i) {
      const int dd = idx[i * nele + e];
      rhs[dd] -= Re[q * 12 + i] * (scale ? scale[dd] : 1.0);
    }
  }
}

// sₓ = S z;  sᵥ = a1 sₓ + gᵥ′, sₐ = b1 sₓ + gₐ′
__global__ void sens_update(int64_t n, int OX, double a1, double b1, const double* __restrict__ z,
                            const double* __restrict__ scale, const double* __restrict__ gv,
                            const double* __restrict__ ga, double* __restrict__ sx, double* __restrict__ sv,
                            double* __restrict__ sa) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = z[i] * (scale ? scale[i] : 1.0);
  sx[i] = s;
  if (OX == 2) {
    sv[i] = a1 * s + gv[i];
    sa[i] = b1 * s + ga[i];
  }
}

// dC/dθ += 2 w (a − y) for the A-costs on θ (element order, one thread)
__global__ void sens_acost(int64_t nele, const int32_t* __restrict__ aidx, const double* __restrict__ cdata,
                           const double* __restrict__ A, int32_t theta, double* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int64_t e = 0; e < nele; ++e)
    if (aidx[e] == theta) *out += 2.0 * cdata[e] * (A[theta] - cdata[nele + e]);
}

}  // namespace mgpu

extern "C" int mgpu_sensitivity_sweepx(mgpu_ctx* c, int32_t OX, int64_t nstep, const double* times, double t0,
                                       int32_t nXder0, const double* x0, const double* u, const double* tvals,
                                       const mgpu_sweep_opts* opts, int64_t ncost, const int64_t* cost_dof,
                                       const double* cost_w, const double* cost_y, int32_t nsel, const int64_t* sel,
                                       double* dXdA, double* dCdA, mgpu_stats* stats) {
  if (!c || !times || !opts || !stats || !(OX == 0 || OX == 2) || nstep < 1 || nXder0 < 0 || nXder0 > OX + 1 ||
      (nXder0 > 0 && !x0) || ncost < 0 || (ncost > 0 && (!cost_dof || !cost_w || !cost_y)) ||
      (c->ntval > 0 && !tvals) || nsel < 1 || !sel)
    return set_err(c, MGPU_ERR_ARG, "mgpu_sensitivity_sweepx: bad arguments");
  if (opts->fixed_iter > 0 || opts->per_component)
    return set_err(c, MGPU_ERR_ARG, "mgpu_sensitivity_sweepx: the sensitivities need converged steps (fixed_iter = 0, "
                                    "per_component = 0)");
  *stats = mgpu_stats{0, 0, 0, 0, 0.0, 0.0};
  const int64_t n = c->nX;
  for (int32_t q = 0; q < nsel; ++q)
    if (sel[q] < 1 || sel[q] > c->nA) return set_err(c, MGPU_ERR_ARG, "selected A-dof out of range");
  std::vector<int32_t> cdof(ncost);
  for (int64_t s = 0; s < ncost; ++s) {
    if (cost_dof[s] < 1 || cost_dof[s] > n) return set_err(c, MGPU_ERR_ARG, "cost dof out of range");
    cdof[s] = int32_t(cost_dof[s] - 1);
  }
  for (const DevGroup& G : c->groups)
    if (G.kind == MGPU_DOFCOST && G.nele > 0 && G.maxder > OX)
      return set_err(c, MGPU_ERR_ARG, "mgpu_sensitivity_sweepx: a DofCost on a time derivative of X needs OX = 2");
  Solver& S = *c->solver;
  if (!S.ok && S.path != PATH_SPARSE && S.path != PATH_SPARSE64)
    return set_err(c, MGPU_ERR_UNSUPPORTED, "no device solver for this model: " + S.why);
  MG_CUDA(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  // the beams of each selected θ (group, element) and the CSR of the pattern
  std::vector<int64_t> lptr(nsel + 1, 0);
  std::vector<int32_t> lele;
  std::vector<int32_t> lgrp;
  for (int32_t q = 0; q < nsel; ++q) {
    for (size_t g = 0; g < c->groups.size(); ++g) {
      const DevGroup& G = c->groups[g];
      if (G.kind != MGPU_EULERBEAM3D || !G.aidx) continue;
      for (int64_t e = 0; e < G.nele; ++e)
        if (G.h_indexA[e] == sel[q]) {
          lele.push_back(int32_t(e));
          lgrp.push_back(int32_t(g));
        }
    }
    lptr[q + 1] = int64_t(lele.size());
  }
  std::vector<int64_t> rptr(n + 1, 0);
  for (int64_t q = 0; q < c->pat.nnz; ++q) rptr[c->pat.rowval[q] + 1]++;
  for (int64_t i = 0; i < n; ++i) rptr[i + 1] += rptr[i];
  std::vector<int32_t> rq(c->pat.nnz), rcol(c->pat.nnz);
  {
    std::vector<int64_t> fill(rptr.begin(), rptr.end() - 1);
    for (int64_t j = 0; j < n; ++j)
      for (int64_t q = c->pat.colptr[j]; q < c->pat.colptr[j + 1]; ++q) {
        const int64_t t = fill[c->pat.rowval[q]]++;
        rq[t] = int32_t(q);
        rcol[t] = int32_t(j);
      }
  }
  std::vector<void*> owned;
  auto alloc = [&](auto** p, size_t count) -> bool {
    using T = typename std::remove_pointer<typename std::remove_reference<decltype(*p)>::type>::type;
    if (cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return false;
    owned.push_back(*p);
    return true;
  };
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    for (void* p : owned) cudaFree(p);
    cudaGetLastError();
  };
  const size_t ns = size_t(nsel) * n;
  double *sx, *sv, *sa, *gv, *ga, *gvs, *gas, *rhs, *nzC, *nzM, *gx, *gvc, *gac, *dC, *Re, *cw, *cy, *ub;
  int32_t *dcd, *dl, *drq, *drcol;
  int64_t* drptr;
  bool ok = alloc(&sx, ns) && alloc(&sv, ns) && alloc(&sa, ns) && alloc(&gv, n) && alloc(&ga, n) && alloc(&gvs, n) &&
            alloc(&gas, n) && alloc(&rhs, n) && alloc(&gx, n) && alloc(&gvc, n) && alloc(&gac, n) &&
            alloc(&dC, nsel) && alloc(&Re, lele.size() * 12) && alloc(&cw, ncost) && alloc(&cy, size_t(nstep) * ncost) &&
            alloc(&ub, c->nU) && alloc(&dcd, ncost) && alloc(&dl, lele.size()) && alloc(&drq, rq.size()) &&
            alloc(&drcol, rcol.size()) && alloc(&drptr, rptr.size());
  if (ok && OX == 2) ok = alloc(&nzC, c->pat.nnz) && alloc(&nzM, c->pat.nnz);
  if (!ok) {
    cleanup();
    return set_err(c, MGPU_ERR_NOMEM, "device allocation failed for the sensitivities");
  }
  ok = cudaMemcpy(drptr, rptr.data(), rptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess &&
       (rq.empty() || cudaMemcpy(drq, rq.data(), rq.size() * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess) &&
       (rcol.empty() ||
        cudaMemcpy(drcol, rcol.data(), rcol.size() * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess) &&
       (lele.empty() ||
        cudaMemcpy(dl, lele.data(), lele.size() * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess) &&
       (ncost == 0 ||
        (cudaMemcpy(dcd, cdof.data(), ncost * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(cw, cost_w, ncost * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(cy, cost_y, size_t(nstep) * ncost * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess)) &&
       cudaMemsetAsync(sx, 0, ns * sizeof(double), st) == cudaSuccess &&
       cudaMemsetAsync(sv, 0, ns * sizeof(double), st) == cudaSuccess &&
       cudaMemsetAsync(sa, 0, ns * sizeof(double), st) == cudaSuccess &&
       cudaMemsetAsync(dC, 0, nsel * sizeof(double), st) == cudaSuccess;
  if (!ok) {
    cleanup();
    return set_err(c, MGPU_ERR_CUDA, "sensitivities: upload failed");
  }
  int rc = MGPU_OK;
#define SENS_TRY(x) \
  do {              \
    rc = (x);       \
    if (rc) {       \
      cleanup();    \
      return rc;    \
    }               \
  } while (0)
#define SENS_CUDA(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      rc = set_err(c, MGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
      cleanup();                                                                          \
      return rc;                                                                          \
    }                                                                                     \
  } while (0)
  const size_t nsx = size_t(3) * n;
  SENS_CUDA(cudaMemsetAsync(c->x, 0, nsx * sizeof(double), st));
  if (nXder0 > 0) SENS_CUDA(cudaMemcpyAsync(c->x, x0, nXder0 * n * sizeof(double), cudaMemcpyHostToDevice, st));
  if (c->nU > 0 && u) SENS_CUDA(cudaMemcpyAsync(c->u, u, c->nU * sizeof(double), cudaMemcpyHostToDevice, st));
  c->nXder_resident = OX + 1;
  double told = t0;
  for (int64_t k = 0; k < nstep; ++k) {
    const double t = times[k], dt = t - told;
    told = t;
    if (OX > 0 && !(dt > 0)) {
      cleanup();
      return set_err(c, MGPU_ERR_ARG, "Time step length not strictly positive at step=" + std::to_string(k + 1));
    }
    const double* tvk = c->ntval > 0 ? tvals + k * c->ntval : nullptr;
    SENS_TRY(newton_step(c, OX, k, t, dt, tvk, opts, stats));
    stats->nstep_done = int(k + 1);
    const double wk = OX == 2 ? dt : 1.0;
    const mgpu_newmark nm = OX == 2 ? newmark_coefficients(opts->beta, opts->gamma, dt) : mgpu_newmark{0, 0, 0, 0, 0, 0};
    // the cost's partials at step k
    SENS_CUDA(cudaMemsetAsync(gx, 0, n * sizeof(double), st));
    SENS_CUDA(cudaMemsetAsync(gvc, 0, n * sizeof(double), st));
    SENS_CUDA(cudaMemsetAsync(gac, 0, n * sizeof(double), st));
    if (ncost > 0) adj_cost_grad<<<nb(ncost, 256), 256, 0, st>>>(ncost, dcd, cw, cy + k * ncost, c->x, wk, gx);
    for (const DevGroup& G : c->groups)
      if (G.kind == MGPU_DOFCOST && G.nele > 0) {
        if (G.distinct)
          adj_group_grad<<<nb(G.nele, 256), 256, 0, st>>>(G.nele, 0, 0, G.idx, nullptr, G.cdata, c->tv + G.tval_base,
                                                          c->x, n, c->u, nullptr, c->scale, wk, gx, gvc, gac, ub,
                                                          nullptr);
        else
          adj_group_grad<<<1, 1, 0, st>>>(G.nele, 0, 1, G.idx, nullptr, G.cdata, c->tv + G.tval_base, c->x, n, c->u,
                                          nullptr, c->scale, wk, gx, gvc, gac, ub, nullptr);
      }
    // damping and mass matrices of the step (S C S, S M S)
    if (OX == 2) {
      const mgpu_newmark onlyC{1.0, 0, 0, 0.0, 0, 0}, onlyM{0.0, 0, 0, 1.0, 0, 0};
      SENS_TRY(upload_stepc(c, t, &onlyC));
      SENS_TRY(launch_assembly(c, MGPU_ASM_ITER, nullptr, 0.0));
      SENS_CUDA(cudaMemcpyAsync(nzC, c->nzval, c->pat.nnz * sizeof(double), cudaMemcpyDeviceToDevice, st));
      SENS_TRY(upload_stepc(c, t, &onlyM));
      SENS_TRY(launch_assembly(c, MGPU_ASM_ITER, nullptr, 0.0));
      SENS_CUDA(cudaMemcpyAsync(nzM, c->nzval, c->pat.nnz * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    // the tangent at the converged state, factorised with each θ's right-hand side in Lλ
    SENS_TRY(upload_stepc(c, t, OX == 2 ? &nm : nullptr));
    launch_reset_errflag(c);
    SENS_TRY(launch_assembly(c, OX == 2 ? MGPU_ASM_ITER : MGPU_ASM_STATIC, nullptr, 1.0));
    for (int32_t q = 0; q < nsel; ++q) {
      double* sxq = sx + size_t(q) * n;
      double* svq = sv + size_t(q) * n;
      double* saq = sa + size_t(q) * n;
      SENS_CUDA(cudaMemsetAsync(rhs, 0, n * sizeof(double), st));
      if (OX == 2) {
        sens_carry<<<nb(n, 256), 256, 0, st>>>(n, nm.a1, nm.a2, nm.a3, nm.b1, nm.b2, nm.b3, sxq, svq, saq, c->scale, gv,
                                               ga, gvs, gas);
        sens_csr_sub<<<nb(n, 256), 256, 0, st>>>(n, drptr, drq, drcol, nzC, gvs, rhs);
        sens_csr_sub<<<nb(n, 256), 256, 0, st>>>(n, drptr, drq, drcol, nzM, gas, rhs);
      }
      const int64_t q0 = lptr[q], q1 = lptr[q + 1];
      for (int64_t r0 = q0; r0 < q1;) {  // beams of θ by group
        int64_t r1 = r0;
        while (r1 < q1 && lgrp[r1] == lgrp[r0]) ++r1;
        const DevGroup& G = c->groups[lgrp[r0]];
        sens_beam_dRdA<<<nb(r1 - r0, 128), 128, 0, st>>>(r1 - r0, dl + r0, G.nele, G.idx, G.cdata, c->x, Re + r0 * 12);
        sens_beam_rhs<<<1, 1, 0, st>>>(0, r1 - r0, dl + r0, G.nele, G.idx, Re + r0 * 12, c->scale, rhs);
        r0 = r1;
      }
      // S J S z = rhs
      SENS_CUDA(cudaMemcpyAsync(c->Ll, rhs, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      SENS_CUDA(cudaMemsetAsync(S.info, 0, sizeof(int), st));
      SENS_TRY(factor_solve(c, S.info));
      sens_update<<<nb(n, 256), 256, 0, st>>>(n, OX, nm.a1, nm.b1, S.dx, c->scale, gv, ga, sxq, svq, saq);
      sens_dot_add<<<1, 256, 0, st>>>(n, gx, sxq, dC + q);
      if (OX == 2) {
        sens_dot_add<<<1, 256, 0, st>>>(n, gvc, svq, dC + q);
        sens_dot_add<<<1, 256, 0, st>>>(n, gac, saq, dC + q);
      }
      if (dXdA) {
        double* out = dXdA + (size_t(k) * nsel + q) * size_t(OX + 1) * n;
        SENS_CUDA(cudaMemcpyAsync(out, sxq, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (OX == 2) {
          SENS_CUDA(cudaMemcpyAsync(out + n, svq, n * sizeof(double), cudaMemcpyDeviceToHost, st));
          SENS_CUDA(cudaMemcpyAsync(out + 2 * n, saq, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        }
      }
      int hinfo = 0, hflag = INT_MAX;
      SENS_CUDA(cudaMemcpyAsync(&hinfo, S.info, sizeof(int), cudaMemcpyDeviceToHost, st));
      SENS_CUDA(cudaMemcpyAsync(&hflag, c->errflag, sizeof(int), cudaMemcpyDeviceToHost, st));
      SENS_CUDA(cudaStreamSynchronize(st));
      if (hflag != INT_MAX) {
        rc = nan_error(c, hflag);
        cleanup();
        return rc;
      }
      if (hinfo != 0) {
        cleanup();
        return set_err(c, MGPU_ERR_SINGULAR,
                       "sensitivities: factorization failed at step=" + std::to_string(k + 1));
      }
    }
  }
  for (int32_t q = 0; q < nsel; ++q)
    for (const DevGroup& G : c->groups)
      if (G.kind == MGPU_ACOST && G.nele > 0)
        sens_acost<<<1, 1, 0, st>>>(G.nele, G.aidx, G.cdata, c->Avec, int32_t(sel[q] - 1), dC + q);
  SENS_CUDA(cudaStreamSynchronize(st));
  if (dCdA) SENS_CUDA(cudaMemcpy(dCdA, dC, nsel * sizeof(double), cudaMemcpyDeviceToHost));
  cleanup();
#undef SENS_TRY
#undef SENS_CUDA
  return MGPU_OK;
}
