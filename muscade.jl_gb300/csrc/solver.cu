// Device linear solve and Newton loop of SweepX{0} / SweepX{2}.
//
// The reference factorises Lλx with UMFPACK at every Newton iteration and
// solves Δx = Lλx \ Lλ (src/SweepX.jl:207-210).  The matrices of the models
// this path targets are sparse and, after reordering, narrow-banded within each
// connected component (chains of beams, risers, frames; Hold multipliers sit
// next to the dofs they constrain).  At create time the host splits the
// matrix graph into connected components and orders each with reverse
// Cuthill-McKee; the device then factorises all components at once, one
// thread block per component, with banded LU and partial pivoting (the
// algorithm of LAPACK's gbtf2), and solves with the factors.  The solution is
// the same Δx the reference computes, to rounding.  Components whose band is
// too wide for this scheme are rejected at solve time with MGPU_ERR_UNSUPPORTED
// (there is no CPU fallback).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "band_rows.cuh"
#include "ctx.hpp"
#include "solver.hpp"

using namespace mgpu;

namespace mgpu {


// ---------------------------------------------------------------- host analysis
static void analyse(mgpu_ctx* c, Solver& S) {
  const Pattern& P = c->pat;
  const int64_t n = c->nX;
  if (n == 0) {
    S.why = "empty model";
    return;
  }
  // union-find over the symmetric pattern
  std::vector<int32_t> par(n);
  std::iota(par.begin(), par.end(), 0);
  auto find = [&](int32_t a) {
    while (par[a] != a) {
      par[a] = par[par[a]];
      a = par[a];
    }
    return a;
  };
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
      int32_t a = find(int32_t(j)), b = find(P.rowval[q]);
      if (a != b) par[std::max(a, b)] = std::min(a, b);
    }
  std::vector<int32_t> comp(n, -1), root2comp(n, -1);
  int ncomp = 0;
  for (int64_t i = 0; i < n; ++i) {
    int32_t r = find(int32_t(i));
    if (root2comp[r] < 0) root2comp[r] = ncomp++;
    comp[i] = root2comp[r];
  }
  // symmetric adjacency lists
  std::vector<int64_t> deg(n + 1, 0);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
      int64_t i = P.rowval[q];
      if (i != j) {
        deg[i + 1]++;
        deg[j + 1]++;
      }
    }
  for (int64_t i = 0; i < n; ++i) deg[i + 1] += deg[i];
  std::vector<int32_t> adj(deg[n]);
  {
    std::vector<int64_t> f(deg.begin(), deg.end() - 1);
    for (int64_t j = 0; j < n; ++j)
      for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
        int64_t i = P.rowval[q];
        if (i != j) {
          adj[f[i]++] = int32_t(j);
          adj[f[j]++] = int32_t(i);
        }
      }
  }
  auto degree = [&](int32_t v) { return deg[v + 1] - deg[v]; };
  // members of each component in increasing dof order
  std::vector<std::vector<int32_t>> members(ncomp);
  for (int64_t i = 0; i < n; ++i) members[comp[i]].push_back(int32_t(i));
  std::vector<int32_t> order;  // RCM order, component after component
  order.reserve(n);
  std::vector<int32_t> level(n, -1), mark(n, 0);
  std::vector<int32_t> comp_start(ncomp + 1, 0);
  for (int cc = 0; cc < ncomp; ++cc) {
    const auto& M = members[cc];
    // pseudo-peripheral start: repeat BFS from the farthest, lowest-degree node
    int32_t start = M[0];
    for (int32_t v : M)
      if (degree(v) < degree(start)) start = v;
    for (int it = 0; it < 3; ++it) {
      std::queue<int32_t> qu;
      for (int32_t v : M) level[v] = -1;
      level[start] = 0;
      qu.push(start);
      int32_t last = start;
      while (!qu.empty()) {
        int32_t v = qu.front();
        qu.pop();
        last = v;
        for (int64_t q = deg[v]; q < deg[v + 1]; ++q)
          if (level[adj[q]] < 0) {
            level[adj[q]] = level[v] + 1;
            qu.push(adj[q]);
          }
      }
      int32_t best = last;
      for (int32_t v : M)
        if (level[v] == level[last] && degree(v) < degree(best)) best = v;
      if (best == start) break;
      start = best;
    }
    // Cuthill-McKee from start
    std::vector<int32_t> cm;
    cm.reserve(M.size());
    cm.push_back(start);
    mark[start] = 1;
    std::vector<int32_t> nb;
    for (size_t h = 0; h < cm.size(); ++h) {
      int32_t v = cm[h];
      nb.clear();
      for (int64_t q = deg[v]; q < deg[v + 1]; ++q)
        if (!mark[adj[q]]) {
          mark[adj[q]] = 1;
          nb.push_back(adj[q]);
        }
      std::sort(nb.begin(), nb.end(), [&](int32_t a, int32_t b) {
        return degree(a) != degree(b) ? degree(a) < degree(b) : a < b;
      });
      cm.insert(cm.end(), nb.begin(), nb.end());
    }
    comp_start[cc] = int32_t(order.size());
    for (auto it = cm.rbegin(); it != cm.rend(); ++it) order.push_back(*it);
  }
  comp_start[ncomp] = int32_t(order.size());
  std::vector<int32_t> pos(n);
  for (int64_t k = 0; k < n; ++k) pos[order[k]] = int32_t(k);
  // bandwidths per component
  std::vector<int32_t> kl(ncomp, 0), ku(ncomp, 0);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
      int64_t i = P.rowval[q];
      int cc = comp[j];
      int32_t d = pos[i] - pos[j];
      if (d > kl[cc]) kl[cc] = d;
      if (-d > ku[cc]) ku[cc] = -d;
    }
  std::vector<int64_t> base(ncomp + 1, 0);
  for (int cc = 0; cc < ncomp; ++cc) {
    int64_t nc = comp_start[cc + 1] - comp_start[cc];
    base[cc + 1] = base[cc] + int64_t(2 * kl[cc] + ku[cc] + 1) * nc;
    S.maxkl = std::max(S.maxkl, kl[cc]);
    S.maxku = std::max(S.maxku, ku[cc]);
  }
  S.ncomp = ncomp;
  S.band_total = base[ncomp];
  if (S.maxkl > 256 || S.maxku > 256 || S.band_total > (int64_t(1) << 33)) {
    S.why = "matrix band too wide for the banded device solver (kl=" + std::to_string(S.maxkl) +
            ", ku=" + std::to_string(S.maxku) + ")";
    return;
  }
  // band position of each nnz
  std::vector<int64_t> bmap(P.nnz);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
      int64_t i = P.rowval[q];
      int cc = comp[j];
      int64_t kj = pos[j] - comp_start[cc], ki = pos[i] - comp_start[cc];
      int64_t ld = 2 * kl[cc] + ku[cc] + 1;
      bmap[q] = base[cc] + (kl[cc] + ku[cc] + ki - kj) + ld * kj;
    }
  // upload
  auto up = [&](auto** dst, const auto& v) -> bool {
    using T = typename std::remove_reference<decltype(v[0])>::type;
    if (cudaMalloc(reinterpret_cast<void**>(dst), std::max<size_t>(v.size(), 1) * sizeof(T)) != cudaSuccess)
      return false;
    return cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
  };
  std::vector<int64_t> cb(base.begin(), base.end() - 1);
  std::vector<int32_t> cn(ncomp), c0(ncomp);
  for (int cc = 0; cc < ncomp; ++cc) {
    cn[cc] = comp_start[cc + 1] - comp_start[cc];
    c0[cc] = comp_start[cc];
  }
  bool good = up(&S.cbase, cb) && up(&S.cn, cn) && up(&S.ckl, kl) && up(&S.cku, ku) && up(&S.cdof0, c0) &&
              up(&S.perm, order) && up(&S.bmap, bmap);
  // row-band layout: applies when every component has kl <= 31 and kl+ku+1 <= 64
  int maxw = 0;
  for (int cc = 0; cc < ncomp; ++cc) maxw = std::max(maxw, kl[cc] + ku[cc] + 1);
  if (S.maxkl <= 31 && maxw <= 64) {
    S.wm = maxw <= 32 ? 32 : 64;
    {
      std::vector<int32_t> l32, l64, lu[4];
      for (int cc = 0; cc < ncomp; ++cc) {
        const int w = kl[cc] + ku[cc] + 1;
        (w <= 32 ? l32 : l64).push_back(cc);
        lu[w <= 32 ? 0 : w <= 40 ? 1 : w <= 48 ? 2 : 3].push_back(cc);
      }
      S.n32 = int(l32.size());
      S.n64 = int(l64.size());
      if (!l32.empty()) good = good && up(&S.list32, l32);
      if (!l64.empty()) good = good && up(&S.list64, l64);
      for (int q = 0; q < 4; ++q) {
        S.nlu[q] = int(lu[q].size());
        if (!lu[q].empty()) good = good && up(&S.lulist[q], lu[q]);
      }
    }
    std::vector<int64_t> rb(ncomp + 1, 0), lb(ncomp + 1, 0);
    for (int cc = 0; cc < ncomp; ++cc) {
      const int64_t nc = comp_start[cc + 1] - comp_start[cc];
      rb[cc + 1] = rb[cc] + nc * (kl[cc] + ku[cc] + 1);
      lb[cc + 1] = lb[cc] + nc * std::max(kl[cc], ku[cc]);  // room for the multipliers of Lλx and of its transpose
    }
    S.rb_total = rb[ncomp];
    S.lb_total = lb[ncomp];
    std::vector<int64_t> rbmap(P.nnz), rbmapT(P.nnz);
    for (int64_t j = 0; j < n; ++j)
      for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
        const int64_t i = P.rowval[q];
        const int cc = comp[j];
        const int64_t kj = pos[j] - comp_start[cc], ki = pos[i] - comp_start[cc];
        const int64_t w = kl[cc] + ku[cc] + 1;
        rbmap[q] = rb[cc] + ki * w + (kj - ki + kl[cc]);
        rbmapT[q] = rb[cc] + kj * w + (ki - kj + ku[cc]);  // entry (j, i) of the transpose: kl and ku exchange
      }
    S.wmT = S.maxku <= 31 ? S.wm : 0;
    std::vector<int64_t> rbv(rb.begin(), rb.end() - 1), lbv(lb.begin(), lb.end() - 1);
    const size_t nr = std::max<int64_t>(S.rb_total, 1), nl = std::max<int64_t>(S.lb_total, 1);
    good = good && up(&S.rbase, rbv) && up(&S.lbase, lbv) && up(&S.rbmap, rbmap) && up(&S.rbmapT, rbmapT);
    good = good && cudaMalloc(&S.RB, nr * sizeof(double)) == cudaSuccess &&
           cudaMemset(S.RB, 0, nr * sizeof(double)) == cudaSuccess;
    good = good && cudaMalloc(&S.RB32, nr * sizeof(float)) == cudaSuccess &&
           cudaMemset(S.RB32, 0, nr * sizeof(float)) == cudaSuccess;
    good = good && cudaMalloc(&S.UC32, nr * sizeof(float)) == cudaSuccess &&
           cudaMalloc(&S.LM32, nl * sizeof(float)) == cudaSuccess &&
           cudaMalloc(&S.UC64, nr * sizeof(double)) == cudaSuccess &&
           cudaMalloc(&S.LM64, nl * sizeof(double)) == cudaSuccess;
    good = good && cudaMalloc(&S.bw, n * sizeof(double)) == cudaSuccess &&
           cudaMalloc(&S.xw, n * sizeof(double)) == cudaSuccess &&
           cudaMalloc(&S.rw, n * sizeof(double)) == cudaSuccess &&
           cudaMalloc(&S.tw32, n * sizeof(float)) == cudaSuccess &&
           cudaMalloc(&S.tw64, n * sizeof(double)) == cudaSuccess;
    good = good && cudaMalloc(&S.flag, ncomp * sizeof(int)) == cudaSuccess &&
           cudaMemset(S.flag, 0, ncomp * sizeof(int)) == cudaSuccess &&
           cudaMalloc(&S.nsweep, ncomp * sizeof(int)) == cudaSuccess &&
           cudaMemset(S.nsweep, 0, ncomp * sizeof(int)) == cudaSuccess;
    // ---- torn layout of the long components (needs s = max(kl, ku) <= 16 for the
    // Schur-complement band 2s-1 <= 31)
    // P interiors per component: as many as keep interiors of at least
    // max(2s, 48) dofs (the separators cost log2(P) cyclic-reduction levels),
    // but no more than needed to give every SM sub-partition ~4 warps: with
    // many components (batched models) the GPU is already full and cutting only
    // adds work
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || nsm <= 0) nsm = 152;
    const int64_t target_warps = int64_t(16) * nsm;
    const int64_t pcap = std::max<int64_t>(1, (target_warps + ncomp - 1) / std::max(ncomp, 1));
    std::vector<int> Pc(ncomp, 1), sc(ncomp, 0);
    for (int cc = 0; cc < ncomp; ++cc) {
      const int64_t nc = comp_start[cc + 1] - comp_start[cc];
      const int sw = std::max(1, std::max(kl[cc], ku[cc]));
      sc[cc] = sw;
      if (sw > 16 || nc < kTornMinDofs) continue;
      const int64_t mmin = std::max(2 * sw, 48);
      const int64_t pmax = std::min((nc + sw) / (mmin + sw), pcap);
      Pc[cc] = int(std::max<int64_t>(1, pmax));
      if (Pc[cc] > 1) S.tearable = 1;
    }
    if (S.tearable) {
      std::vector<TornInt> ti, tiT;
      std::vector<TornSep> ts;
      std::vector<int64_t> irb, ilb, brow;
      std::vector<int32_t> in_, ikl, iku, idof, icomp;
      std::vector<BcrSep> bsep;
      int64_t orow = 0, oblk = 0, oy = 0, olm = 0, otv = 0;
      // segment of each band position: >= 0 interior index (global), < 0 -(separator index + 1)
      std::vector<int32_t> seg(n), loc(n);
      int maxwI = 0;
      std::vector<int32_t> cint0(ncomp + 1, 0), csep0(ncomp + 1, 0);
      for (int cc = 0; cc < ncomp; ++cc) {
        const int64_t c0 = comp_start[cc], nc = comp_start[cc + 1] - c0;
        const int P = Pc[cc], sw = sc[cc], w = kl[cc] + ku[cc] + 1;
        cint0[cc] = int32_t(ti.size());
        csep0[cc] = int32_t(ts.size());
        S.maxP = std::max(S.maxP, P);
        maxwI = std::max(maxwI, w);
        const int64_t tot = nc - int64_t(P - 1) * sw;
        int64_t p0 = 0;
        const int sep0 = int(ts.size()), int0 = int(ti.size());
        for (int a = 0; a < P; ++a) {
          const int64_t m = tot / P + (a < tot % P ? 1 : 0);
          TornInt I{};
          I.rbase = orow;
          I.lbase = olm;
          I.n = int32_t(m);
          I.kl = kl[cc];
          I.ku = ku[cc];
          I.dof0 = int32_t(c0 + p0);
          I.s = sw;
          I.eL = I.eR = I.fL = I.fR = I.yL = I.yR = -1;
          I.sepL = a > 0 ? sep0 + a - 1 : -1;
          I.sepR = a < P - 1 ? sep0 + a : -1;
          I.comp = cc;
          if (I.sepL >= 0) {
            I.eL = oblk, oblk += int64_t(sw) * sw;
            I.fL = oblk, oblk += int64_t(sw) * sw;
            I.yL = oy, oy += m * sw;
          }
          if (I.sepR >= 0) {
            I.eR = oblk, oblk += int64_t(sw) * sw;
            I.fR = oblk, oblk += int64_t(sw) * sw;
            I.yR = oy, oy += m * sw;
          }
          orow += m * w;
          olm += m * std::max(kl[cc], ku[cc]);
          for (int64_t q = 0; q < m; ++q) {
            seg[c0 + p0 + q] = int32_t(ti.size());
            loc[c0 + p0 + q] = int32_t(q);
          }
          irb.push_back(I.rbase), ilb.push_back(I.lbase), in_.push_back(I.n), ikl.push_back(I.kl),
              iku.push_back(I.ku), idof.push_back(I.dof0), icomp.push_back(cc);
          ti.push_back(I);
          TornInt IT = I;
          std::swap(IT.kl, IT.ku);
          tiT.push_back(IT);
          p0 += m;
          if (a < P - 1) {
            TornSep Sp{};
            Sp.s = sw;
            Sp.dof0 = int32_t(c0 + p0);
            Sp.d = oblk, oblk += int64_t(sw) * sw;
            Sp.intL = int0 + a;
            Sp.intR = int0 + a + 1;
            Sp.trow = otv + int64_t(a) * sw;
            Sp.first = a == 0;
            Sp.last = a == P - 2;
            Sp.comp = cc;
            for (int64_t q = 0; q < sw; ++q) {
              seg[c0 + p0 + q] = -(int32_t(ts.size()) + 1);
              loc[c0 + p0 + q] = int32_t(q);
            }
            ts.push_back(Sp);
            p0 += sw;
          }
        }
        if (P > 1) {
          // block cyclic reduction of this component's N = P-1 separator blocks
          const int N = P - 1;
          int nlev = 0;
          while ((1 << nlev) < N) ++nlev;
          for (int k = sep0; k < int(ts.size()); ++k) {
            BcrSep B{};
            B.comp = cc;
            B.kloc = k - sep0;
            B.N = N;
            B.s = sw;
            B.sep0 = sep0;
            B.nlev = nlev;
            bsep.push_back(B);
            brow.push_back(ts[k].trow);
          }
          S.bcr_levels = std::max(S.bcr_levels, nlev);
          otv += int64_t(N) * sw;
        }
      }
      S.nint = int(ti.size());
      S.nsep = int(ts.size());
      cint0[ncomp] = S.nint;
      csep0[ncomp] = S.nsep;
      S.twmI = maxwI <= 32 ? 32 : 64;
      // fused per-component solve (one block per component) when every component has
      // few interiors; warps per block bounded by ~112 KB of shared memory (two blocks per SM)
      {
        const char* fe = getenv("MGPU_TORN_FUSED");
        const bool allow = !(fe && fe[0] == '0');
        const int b32 = S.twmI == 32 ? tb_fused_warp_bytes<float, 32>() : tb_fused_warp_bytes<float, 64>();
        const int b64 = S.twmI == 32 ? tb_fused_warp_bytes<double, 32>() : tb_fused_warp_bytes<double, 64>();
        const int budget = 112 * 1024;
        if (allow && S.maxP <= kFusedMaxP) {
          S.fuseW32 = std::max(1, std::min({S.maxP, budget / b32, kFusedMaxW}));
          S.fuseW64 = std::max(1, std::min({S.maxP, budget / b64, kFusedMaxW}));
          if (S.twmI == 32) {
            cudaFuncSetAttribute(tb_fused<float, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, S.fuseW32 * b32);
            cudaFuncSetAttribute(tb_fused<double, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, S.fuseW64 * b64);
          } else {
            cudaFuncSetAttribute(tb_fused<float, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, S.fuseW32 * b32);
            cudaFuncSetAttribute(tb_fused<double, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, S.fuseW64 * b64);
          }
        }
      }
      int maxs = 0;
      for (int cc = 0; cc < ncomp; ++cc) maxs = std::max(maxs, std::max(kl[cc], ku[cc]));
      S.tmaxs = maxs;
      S.tb_rows = orow;
      S.tb_blk = oblk;
      S.tb_y = oy;
      S.tb_lm = olm;
      S.tb_tvec = otv;
      // every nnz to its place in TALL = [interior rows | blocks], for Lλx and for its transpose
      std::vector<int64_t> tbmap(P.nnz), tbmapT(P.nnz);
      auto place = [&](int64_t pi, int64_t pj, bool transposed) -> int64_t {
        const int si = seg[pi], sj = seg[pj];
        const int li = loc[pi], lj = loc[pj];
        if (si >= 0 && sj >= 0) {  // same interior
          if (si != sj) return -1;
          const TornInt& I = ti[si];
          const int w = I.kl + I.ku + 1, klx = transposed ? I.ku : I.kl;
          return I.rbase + int64_t(li) * w + (lj - li + klx);
        }
        if (si >= 0) {  // interior row, separator column: E
          const TornInt& I = ti[si];
          const int k = -sj - 1;
          if (k == I.sepL) return S.tb_rows + I.eL + int64_t(li) * I.s + lj;
          return S.tb_rows + I.eR + int64_t(li - (I.n - I.s)) * I.s + lj;
        }
        if (sj >= 0) {  // separator row, interior column: F
          const TornInt& I = ti[sj];
          const int k = -si - 1;
          if (k == I.sepL) return S.tb_rows + I.fL + int64_t(li) * I.s + lj;
          return S.tb_rows + I.fR + int64_t(li) * I.s + (lj - (I.n - I.s));
        }
        if (si != sj) return -1;
        return S.tb_rows + ts[-si - 1].d + int64_t(li) * ts[-si - 1].s + lj;  // same separator: D
      };
      for (int64_t j = 0; j < n; ++j)
        for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
          const int64_t i = P.rowval[q];
          tbmap[q] = place(pos[i], pos[j], false);
          tbmapT[q] = place(pos[j], pos[i], true);
          if (tbmap[q] < 0 || tbmapT[q] < 0) S.tearable = 0;  // an entry outside the bands (cannot happen)
        }
      auto upv = [&](auto** dst, const auto& v) -> bool { return v.empty() ? true : up(dst, v); };
      good = good && upv(&S.d_ti, ti) && upv(&S.d_tiT, tiT) && upv(&S.d_ts, ts) && upv(&S.i_rbase, irb) &&
             upv(&S.i_lbase, ilb) && upv(&S.i_n, in_) && upv(&S.i_kl, ikl) && upv(&S.i_ku, iku) &&
             upv(&S.i_dof0, idof) && upv(&S.d_bsep, bsep) && upv(&S.d_brow, brow) && up(&S.tbmap, tbmap) &&
             up(&S.tbmapT, tbmapT) && up(&S.c_int0, cint0) && up(&S.c_sep0, csep0);
      // cyclic-reduction storage: levels 0..L of D, L, U per separator, factors and W per separator
      const size_t nblk = size_t(std::max(S.nsep, 1)) * BCR_SS;
      const size_t ndlu = size_t(S.bcr_levels + 1) * 3 * nblk;
      const size_t nall = size_t(std::max<int64_t>(orow + oblk, 1));
      good = good && cudaMalloc(&S.TALL, nall * sizeof(double)) == cudaSuccess &&
             cudaMemset(S.TALL, 0, nall * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.TUC, std::max<int64_t>(orow, 1) * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.TLM, std::max<int64_t>(olm, 1) * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.TY, std::max<int64_t>(oy, 1) * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.DLU, ndlu * sizeof(double)) == cudaSuccess &&
             cudaMemset(S.DLU, 0, ndlu * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.FA, nblk * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.WL, nblk * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.WU, nblk * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.PV, size_t(std::max(S.nsep, 1)) * BCR_S * sizeof(int)) == cudaSuccess &&
             cudaMalloc(&S.trhs, std::max<int64_t>(otv, 1) * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.txs, std::max<int64_t>(otv, 1) * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.tpiv, n * sizeof(int32_t)) == cudaSuccess;
      // FP32 factorisation and FP64 refinement
      auto fal = [&](float** p, int64_t cnt) {
        return cudaMalloc(p, std::max<int64_t>(cnt, 1) * sizeof(float)) == cudaSuccess;
      };
      good = good && fal(&S.TALL32, orow + oblk) &&
             cudaMemset(S.TALL32, 0, std::max<int64_t>(orow + oblk, 1) * sizeof(float)) == cudaSuccess &&
             fal(&S.TUC32, orow) && fal(&S.TLM32, olm) && fal(&S.TY32, oy) && fal(&S.DLU32, int64_t(ndlu)) &&
             cudaMemset(S.DLU32, 0, ndlu * sizeof(float)) == cudaSuccess && fal(&S.FA32, int64_t(nblk)) &&
             fal(&S.WL32, int64_t(nblk)) && fal(&S.WU32, int64_t(nblk));
      good = good && upv(&S.i_comp, icomp) &&
             cudaMalloc(&S.iflag, std::max(S.nint, 1) * sizeof(int)) == cudaSuccess &&
             cudaMalloc(&S.nbad, sizeof(int)) == cudaSuccess && cudaMalloc(&S.info32, sizeof(int)) == cudaSuccess &&
             cudaMalloc(&S.dtmp, n * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&S.rtmp, n * sizeof(double)) == cudaSuccess;
      {
        // rows of the pattern: CSC positions and columns, row by row
        std::vector<int64_t> rptr(n + 1, 0), rq(P.nnz);
        std::vector<int32_t> rcol(P.nnz);
        for (int64_t q = 0; q < P.nnz; ++q) rptr[P.rowval[q] + 1]++;
        for (int64_t i = 0; i < n; ++i) rptr[i + 1] += rptr[i];
        std::vector<int64_t> fill(rptr.begin(), rptr.end() - 1);
        for (int64_t j = 0; j < n; ++j)
          for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
            const int64_t at = fill[P.rowval[q]]++;
            rq[at] = q;
            rcol[at] = int32_t(j);
          }
        std::vector<int32_t> rv(P.rowval.begin(), P.rowval.end());
        good = good && up(&S.rptr, rptr) && up(&S.rq, rq) && up(&S.rcol, rcol) && up(&S.dcolptr, P.colptr) &&
               up(&S.drowval, rv);
      }
    }
  }
  good = good && cudaMalloc(&S.AB, std::max<int64_t>(S.band_total, 1) * sizeof(double)) == cudaSuccess;
  good = good && cudaMalloc(&S.ipiv, n * sizeof(int32_t)) == cudaSuccess;
  good = good && cudaMalloc(&S.rhs, n * sizeof(double)) == cudaSuccess;
  good = good && cudaMalloc(&S.rdiag, n * sizeof(double)) == cudaSuccess;
  good = good && cudaMalloc(&S.dx, n * sizeof(double)) == cudaSuccess;
  good = good && cudaMalloc(&S.red, 4 * sizeof(double)) == cudaSuccess;
  good = good && cudaMalloc(&S.part, 2 * kNormBlocks * sizeof(double)) == cudaSuccess;
  good = good && cudaMalloc(&S.info, kInfoSlots * sizeof(int)) == cudaSuccess &&
         cudaMemset(S.info, 0, kInfoSlots * sizeof(int)) == cudaSuccess;
  {
    std::vector<int32_t> cod(n);
    for (int64_t j = 0; j < n; ++j) cod[j] = comp[j];
    good = good && up(&S.cod, cod);
  }
  good = good && cudaMalloc(&S.frozen, std::max(ncomp, 1) * sizeof(int)) == cudaSuccess &&
         cudaMemset(S.frozen, 0, std::max(ncomp, 1) * sizeof(int)) == cudaSuccess;
  good = good && cudaMalloc(&S.nactive, sizeof(int)) == cudaSuccess;
  good = good && cudaMallocHost(&S.hbuf, 8 * sizeof(double)) == cudaSuccess;
  if (!good) {
    S.why = "device allocation failed for the solver";
    return;
  }
  S.ok = true;
}

// ---------------------------------------------------------------- kernels
__global__ void band_gather(int64_t nnz, const int64_t* __restrict__ bmap, const double* __restrict__ nzval,
                            double* __restrict__ AB) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < nnz) AB[bmap[k]] = nzval[k];
}

// Banded LU with partial pivoting (LAPACK gbtf2 algorithm), one block per
// component.  Also writes the reciprocal pivots, which the backward
// substitution multiplies by (gbtrs divides; the results differ by rounding).
__global__ void __launch_bounds__(128) band_lu(const int64_t* cbase, const int32_t* cn, const int32_t* ckl,
                                               const int32_t* cku, const int32_t* cdof0, double* AB, int32_t* ipiv,
                                               double* rdg, int* info) {
  const int cc = blockIdx.x;
  const int n = cn[cc], kl = ckl[cc], ku = cku[cc];
  const int kv = kl + ku, ld = 2 * kl + ku + 1;
  double* A = AB + cbase[cc];
  int32_t* piv = ipiv + cdof0[cc];
  double* rdiag = rdg + cdof0[cc];  // reciprocal pivots for the backward substitution
  __shared__ double sval[128];
  __shared__ int sidx[128];
  __shared__ int s_jp, s_ju;
  __shared__ double s_piv;
  if (threadIdx.x == 0) s_ju = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const int km = min(kl, n - 1 - k);
    // pivot search over rows k..k+km of column k (first index of max |a|)
    double best = -1.0;
    int bi = 0;
    for (int i = threadIdx.x; i <= km; i += blockDim.x) {
      const double v = fabs(A[kv + i + int64_t(ld) * k]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    sval[threadIdx.x] = best;
    sidx[threadIdx.x] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        const double v2 = sval[threadIdx.x + s];
        const int i2 = sidx[threadIdx.x + s];
        if (v2 > sval[threadIdx.x] || (v2 == sval[threadIdx.x] && i2 < sidx[threadIdx.x])) {
          sval[threadIdx.x] = v2;
          sidx[threadIdx.x] = i2;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const int jp = sidx[0];
      s_jp = jp;
      piv[k] = k + jp;
      const double p = A[kv + jp + int64_t(ld) * k];
      s_piv = p;
      if (p == 0.0 && *info == 0) atomicCAS(info, 0, cc + 1);
      rdiag[k] = 1.0 / p;
      s_ju = max(s_ju, min(k + ku + jp, n - 1));
    }
    __syncthreads();
    const int jp = s_jp, ju = s_ju;
    const double p = s_piv;
    if (p != 0.0) {
      // swap rows k and k+jp in columns k..ju
      if (jp != 0)
        for (int j = k + threadIdx.x; j <= ju; j += blockDim.x) {
          double* a = A + kv + (k - j) + int64_t(ld) * j;
          double* b = A + kv + (k + jp - j) + int64_t(ld) * j;
          const double t = *a;
          *a = *b;
          *b = t;
        }
      __syncthreads();
      // multipliers (scaled by the reciprocal pivot, like gbtf2)
      const double rp = 1.0 / p;
      for (int i = 1 + threadIdx.x; i <= km; i += blockDim.x) A[kv + i + int64_t(ld) * k] *= rp;
      __syncthreads();
      // rank-1 update of columns k+1..ju, rows k+1..k+km
      const int w = ju - k;
      const int tot = w * km;
      for (int q = threadIdx.x; q < tot; q += blockDim.x) {
        const int jj = q / km + 1, i = q % km + 1;
        const int j = k + jj;
        const double u = A[kv - jj + int64_t(ld) * j];  // row k of column j
        if (u != 0.0) A[kv + i - jj + int64_t(ld) * j] -= A[kv + i + int64_t(ld) * k] * u;
      }
    }
    __syncthreads();
  }
}

// Solve with the band factors: permute, L with interchanges, U; one block per component.
__global__ void __launch_bounds__(128) band_solve(const int64_t* cbase, const int32_t* cn, const int32_t* ckl,
                                                  const int32_t* cku, const int32_t* cdof0, const int32_t* perm,
                                                  const double* AB, const int32_t* ipiv, const double* rdg,
                                                  const double* Ll, double* rhs, double* dx) {
  const int cc = blockIdx.x;
  const int n = cn[cc], kl = ckl[cc], ku = cku[cc];
  const int kv = kl + ku, ld = 2 * kl + ku + 1;
  const double* A = AB + cbase[cc];
  const int32_t* piv = ipiv + cdof0[cc];
  const int32_t* pm = perm + cdof0[cc];
  double* b = rhs + cdof0[cc];
  for (int k = threadIdx.x; k < n; k += blockDim.x) b[k] = Ll[pm[k]];
  __syncthreads();
  // forward: L y = P b
  for (int k = 0; k < n; ++k) {
    const int km = min(kl, n - 1 - k);
    const int p = piv[k];
    if (threadIdx.x == 0 && p != k) {
      const double t = b[k];
      b[k] = b[p];
      b[p] = t;
    }
    __syncthreads();
    const double bk = b[k];
    for (int i = 1 + threadIdx.x; i <= km; i += blockDim.x) b[k + i] -= A[kv + i + int64_t(ld) * k] * bk;
    __syncthreads();
  }
  // backward: U x = y  (U has kl+ku superdiagonals)
  for (int k = n - 1; k >= 0; --k) {
    if (threadIdx.x == 0) b[k] *= rdg[cdof0[cc] + k];  // reciprocal pivot from band_lu
    __syncthreads();
    const double bk = b[k];
    const int m = min(kv, k);
    for (int i = 1 + threadIdx.x; i <= m; i += blockDim.x) b[k - i] -= A[kv - i + int64_t(ld) * k] * bk;
    __syncthreads();
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) dx[pm[k]] = b[k];
}

// Σ Δx², Σ Lλ²: kNormBlocks partial sums (fixed assignment and tree order), then
// one block adds the partials in index order -- deterministic for a given n
__global__ void __launch_bounds__(256) norms_partial(int64_t n, const double* dx, const double* Ll, double* part) {
  __shared__ double s1[256], s2[256];
  double a = 0.0, b = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * 256 + threadIdx.x; i < n; i += int64_t(gridDim.x) * 256) {
    a += dx[i] * dx[i];
    b += Ll[i] * Ll[i];
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s1[threadIdx.x] += s1[threadIdx.x + s];
      s2[threadIdx.x] += s2[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
  }
}
__global__ void norms_final(int nb, const double* part, double* red) {
  if (threadIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int k = 0; k < nb; ++k) {
    a += part[2 * k];
    b += part[2 * k + 1];
  }
  red[0] = a;
  red[1] = b;
}

// Per-component convergence for independent models solved together: ΣΔx² and
// ΣLλ² over the component's dofs (one warp, fixed order); a component that
// meets the test is frozen for the rest of the step, the others are counted.
__global__ void __launch_bounds__(32) comp_converge(const int32_t* __restrict__ cn, const int32_t* __restrict__ cdof0,
                                                    const int32_t* __restrict__ perm, const double* __restrict__ dx,
                                                    const double* __restrict__ Ll, double cdx2, double cLl2,
                                                    int* __restrict__ frozen, int* __restrict__ nactive) {
  const int cc = blockIdx.x, lane = threadIdx.x;
  if (frozen[cc]) return;
  const int n = cn[cc];
  const int32_t* pm = perm + cdof0[cc];
  double a = 0.0, b = 0.0;
  for (int k = lane; k < n; k += 32) {
    const int d = pm[k];
    a += dx[d] * dx[d];
    b += Ll[d] * Ll[d];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    if (a <= cdx2 && b <= cLl2)
      frozen[cc] = 1;
    else
      atomicAdd(nactive, 1);
  }
}

// Newmarkβdecrement!  (src/SweepX.jl:98-132, decrement! src/Assemble.jl:206-211)
// (frozen, cod): dofs of converged components keep their state (per-component convergence)
__global__ void decrement_kernel(int64_t n, int OX, int first, const double* dx, const double* scale,
                                 const double* __restrict__ sc, double* x, const int* __restrict__ frozen,
                                 const int32_t* __restrict__ cod) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (frozen && frozen[cod[i]]) return;
  const double a1 = sc[1], a2 = sc[2], a3 = sc[3], b1 = sc[4], b2 = sc[5], b3 = sc[6];
  const double s = scale ? scale[i] : 1.0;
  const double d = dx[i];
  if (OX == 2) {
    double* x1 = x + n;
    double* x2 = x + 2 * n;
    double d1 = a1 * d, d2 = b1 * d;
    if (first) {
      const double xp = x1[i] / s, xpp = x2[i] / s;  // getdof! returns scaled values
      d1 += a2 * xp + a3 * xpp;
      d2 += b2 * xp + b3 * xpp;
    }
    x1[i] -= d1 * s;
    x2[i] -= d2 * s;
  }
  x[i] -= d * s;
}

}  // namespace mgpu

static bool sparse_usable(const Solver& S) { return S.sparse && S.sparse->why.empty(); }
static bool is_sparse(int path) { return path == PATH_SPARSE || path == PATH_SPARSE64; }

// the multifrontal solver, analysed on first need
static int ensure_sparse(mgpu_ctx* c, Solver& S) {
  if (S.sparse) return MGPU_OK;
  const int rc = sparse_create(c, S.sparse, c->dof_xyz.empty() ? nullptr : c->dof_xyz.data(),
                               c->dof_last.empty() ? nullptr : c->dof_last.data());
  if (rc != MGPU_OK) {
    sparse_destroy(S.sparse);
    return rc;
  }
  // the Newton loop's buffers (the banded analysis allocates them only when it applies)
  const int64_t n = std::max<int64_t>(c->nX, 1);
  if (!S.dx) MG_CUDA(cudaMalloc(&S.dx, n * sizeof(double)));
  if (!S.red) MG_CUDA(cudaMalloc(&S.red, 4 * sizeof(double)));
  if (!S.part) MG_CUDA(cudaMalloc(&S.part, 2 * kNormBlocks * sizeof(double)));
  if (!S.info) {
    MG_CUDA(cudaMalloc(&S.info, kInfoSlots * sizeof(int)));
    MG_CUDA(cudaMemset(S.info, 0, kInfoSlots * sizeof(int)));
  }
  if (!S.hbuf) MG_CUDA(cudaMallocHost(&S.hbuf, 8 * sizeof(double)));
  return MGPU_OK;
}

extern "C" int mgpu_solver_create(mgpu_ctx* c) {
  c->solver = new Solver();
  Solver& S = *c->solver;
  analyse(c, S);
  cudaGetLastError();  // analysis errors are reported at solve time
  // default: the FP64 row-band kernels where they apply, else the FP64 block
  // kernels; the multifrontal solver where the bands are too wide
  // (mgpu_set_linear_solver changes it)
  S.path = S.tearable ? PATH_TORN32 : S.wm ? PATH_F64ROWS : PATH_BLOCK;
  S.adaptive = S.tearable;
  if (!S.ok && c->nX > 0) S.path = PATH_SPARSE;  // analysed on first use (a model may only be assembled)
  if (getenv("MGPU_VERBOSE")) {
    static const char* names[] = {"row-band FP32 + FP64 refinement", "row-band FP64", "block FP64",
                                  "partitioned FP64", "partitioned FP32 + FP64 refinement"};
    fprintf(stderr, "[muscade_gpu] solver: %s, %d components, max kl %d, max ku %d, %s\n",
            S.ok ? "banded" : S.why.c_str(), S.ncomp, S.maxkl, S.maxku,
            is_sparse(S.path) ? "multifrontal" : names[S.path]);
  }
  return MGPU_OK;
}

extern "C" int mgpu_set_linear_solver(mgpu_ctx* c, int32_t kind) {
  if (!c || !c->solver || kind < MGPU_LINSOLVE_AUTO || kind > MGPU_LINSOLVE_SPARSE64)
    return set_err(c, MGPU_ERR_ARG, "mgpu_set_linear_solver: bad arguments");
  Solver& S = *c->solver;
  MG_CUDA(cudaSetDevice(c->device));
  if (kind == MGPU_LINSOLVE_SPARSE || kind == MGPU_LINSOLVE_SPARSE64) {
    const int rc = ensure_sparse(c, S);
    if (rc != MGPU_OK) return rc;
    if (!sparse_usable(S)) return set_err(c, MGPU_ERR_UNSUPPORTED, "multifrontal solver: " + S.sparse->why);
    S.path = kind == MGPU_LINSOLVE_SPARSE ? PATH_SPARSE : PATH_SPARSE64;
    S.sparse->fp64_only = kind == MGPU_LINSOLVE_SPARSE64;
    S.sparse->adaptive = true;
    return MGPU_OK;
  }
  if (kind == MGPU_LINSOLVE_AUTO && !S.ok) {  // the multifrontal solver, analysed on first use
    S.path = PATH_SPARSE;
    if (S.sparse) S.sparse->fp64_only = false;
    return MGPU_OK;
  }
  if (!S.ok)
    return set_err(c, MGPU_ERR_UNSUPPORTED, "banded solver kinds need narrow bands: " + S.why);
  if (kind == MGPU_LINSOLVE_TORN || kind == MGPU_LINSOLVE_TORN32) {
    if (!S.tearable)
      return set_err(c, MGPU_ERR_UNSUPPORTED,
                     "partitioned solve needs a component of at least 512 dofs with max(kl, ku) <= 16");
    S.path = kind == MGPU_LINSOLVE_TORN ? PATH_TORN : PATH_TORN32;
    S.adaptive = false;
    return MGPU_OK;
  }
  if ((kind == MGPU_LINSOLVE_F32IR || kind == MGPU_LINSOLVE_F64) && !S.wm)
    return set_err(c, MGPU_ERR_UNSUPPORTED,
                   "linear solver kind needs kl <= 31 and kl+ku+1 <= 64 in every component (kl=" +
                       std::to_string(S.maxkl) + ", ku=" + std::to_string(S.maxku) + ")");
  S.adaptive = kind == MGPU_LINSOLVE_AUTO && S.tearable;
  S.path = kind == MGPU_LINSOLVE_AUTO ? (S.tearable ? PATH_TORN32 : S.wm ? PATH_F64ROWS : PATH_BLOCK)
           : kind == MGPU_LINSOLVE_F32IR ? PATH_F32IR
           : kind == MGPU_LINSOLVE_F64   ? PATH_F64ROWS
                                         : PATH_BLOCK;
  return MGPU_OK;
}

extern "C" int mgpu_linear_solver_info(mgpu_ctx* c, mgpu_linsolve_info* info) {
  if (!c || !c->solver || !info) return set_err(c, MGPU_ERR_ARG, "mgpu_linear_solver_info: bad arguments");
  Solver& S = *c->solver;
  if (is_sparse(S.path)) {
    MG_CUDA(cudaSetDevice(c->device));
    const int rc = ensure_sparse(c, S);
    if (rc != MGPU_OK) return rc;
    if (!sparse_usable(S)) return set_err(c, MGPU_ERR_UNSUPPORTED, "multifrontal solver: " + S.sparse->why);
    const SparseDev& sp = *S.sparse;
    info->kind = S.path == PATH_SPARSE ? MGPU_LINSOLVE_SPARSE : MGPU_LINSOLVE_SPARSE64;
    info->ncomp = sp.nroot;
    info->max_kl = info->max_ku = sp.max_m;
    info->last_fallback = sp.last_fallback;
    info->last_sweeps = sp.last_sweeps;
    return MGPU_OK;
  }
  info->kind = S.path == PATH_F32IR    ? MGPU_LINSOLVE_F32IR
               : S.path == PATH_F64ROWS ? MGPU_LINSOLVE_F64
               : S.path == PATH_TORN    ? MGPU_LINSOLVE_TORN
               : S.path == PATH_TORN32  ? MGPU_LINSOLVE_TORN32
                                        : MGPU_LINSOLVE_BLOCK;
  info->ncomp = S.ncomp;
  info->max_kl = S.maxkl;
  info->max_ku = S.maxku;
  info->last_fallback = 0;
  info->last_sweeps = 0;
  if ((S.path == PATH_F32IR || S.path == PATH_TORN32) && S.ncomp > 0 && S.flag) {
    std::vector<int> f(S.ncomp), w(S.ncomp);
    MG_CUDA(cudaStreamSynchronize(c->stream));
    MG_CUDA(cudaMemcpy(f.data(), S.flag, S.ncomp * sizeof(int), cudaMemcpyDeviceToHost));
    MG_CUDA(cudaMemcpy(w.data(), S.nsweep, S.ncomp * sizeof(int), cudaMemcpyDeviceToHost));
    for (int i = 0; i < S.ncomp; ++i) {
      info->last_fallback += f[i] != 0;
      info->last_sweeps = std::max(info->last_sweeps, w[i]);
    }
    if (S.path == PATH_TORN32 && !S.fuseW32) info->last_sweeps = S.nrefine;
  }
  return MGPU_OK;
}

extern "C" int mgpu_autotune(mgpu_ctx* c, int32_t mission, const mgpu_newmark* nm, mgpu_tune_report* rep) {
  if (!c || !c->solver || !rep || mission < 0 || mission > 2 || (mission != MGPU_ASM_STATIC && !nm))
    return set_err(c, MGPU_ERR_ARG, "mgpu_autotune: bad arguments");
  Solver& S = *c->solver;
  MG_CUDA(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  cudaEvent_t e0, e1;
  MG_CUDA(cudaEventCreate(&e0));
  MG_CUDA(cudaEventCreate(&e1));
  int rc = upload_stepc(c, 0.0, mission != MGPU_ASM_STATIC ? nm : nullptr);
  auto time3 = [&](auto&& f) -> double {  // mean of 3 after one warm-up, -1 on failure
    if (f() != MGPU_OK) return -1.0;
    cudaEventRecord(e0, st);
    for (int r = 0; r < 3; ++r)
      if (f() != MGPU_OK) return -1.0;
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / 3.0;
  };
  // element kernels
  const int blocks[3] = {64, 128, 256};
  int best_b = c->elem_block;
  double best_t = 1e300;
  for (int k = 0; k < 3 && rc == MGPU_OK; ++k) {
    c->elem_block = blocks[k];
    launch_reset_errflag(c);
    const double t = time3([&] { return launch_assembly(c, mission, nullptr); });
    rep->ms_elem[k] = t;
    if (t >= 0 && t < best_t) best_t = t, best_b = blocks[k];
  }
  c->elem_block = best_b;
  rep->elem_block = best_b;
  // linear solvers on the assembled matrix
  for (double& t : rep->ms_linsolve) t = -1.0;
  if (rc == MGPU_OK) rc = launch_assembly(c, mission, nullptr);
  const int saved_path = S.path;
  const bool saved_adaptive = S.adaptive;
  int best_k = -1;
  best_t = 1e300;
  if (rc == MGPU_OK && S.ok) {
    for (int kind = MGPU_LINSOLVE_F32IR; kind <= MGPU_LINSOLVE_TORN32; ++kind) {
      const bool applicable = (kind == MGPU_LINSOLVE_F32IR || kind == MGPU_LINSOLVE_F64) ? S.wm != 0
                              : (kind == MGPU_LINSOLVE_TORN || kind == MGPU_LINSOLVE_TORN32) ? S.tearable != 0
                                                                                             : true;
      if (!applicable) continue;
      S.path = kind == MGPU_LINSOLVE_F32IR ? PATH_F32IR
               : kind == MGPU_LINSOLVE_F64 ? PATH_F64ROWS
               : kind == MGPU_LINSOLVE_BLOCK ? PATH_BLOCK
               : kind == MGPU_LINSOLVE_TORN ? PATH_TORN
                                            : PATH_TORN32;
      S.adaptive = false;
      MG_CUDA(cudaMemsetAsync(S.info, 0, sizeof(int), st));
      const double t = time3([&] { return factor_solve(c, S.info); });
      int hinfo = 0;
      MG_CUDA(cudaMemcpy(&hinfo, S.info, sizeof(int), cudaMemcpyDeviceToHost));
      rep->ms_linsolve[kind] = hinfo == 0 ? t : -1.0;
      if (hinfo == 0 && t >= 0 && t < best_t) best_t = t, best_k = kind;
    }
  }
  if (best_k < 0) {
    S.path = saved_path;
    S.adaptive = saved_adaptive;
  } else {
    S.path = best_k == MGPU_LINSOLVE_F32IR ? PATH_F32IR
             : best_k == MGPU_LINSOLVE_F64 ? PATH_F64ROWS
             : best_k == MGPU_LINSOLVE_BLOCK ? PATH_BLOCK
             : best_k == MGPU_LINSOLVE_TORN ? PATH_TORN
                                            : PATH_TORN32;
    S.adaptive = best_k == MGPU_LINSOLVE_TORN32;  // still leaves FP32 after a fallback
  }
  rep->linsolve = best_k < 0 ? MGPU_LINSOLVE_AUTO : best_k;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  launch_reset_errflag(c);
  MG_CUDA(cudaStreamSynchronize(st));
  return rc;
}

extern "C" int mgpu_sparse_info(mgpu_ctx* c, mgpu_sparse_report* rep) {
  if (!c || !c->solver || !rep) return set_err(c, MGPU_ERR_ARG, "mgpu_sparse_info: bad arguments");
  Solver& S = *c->solver;
  MG_CUDA(cudaSetDevice(c->device));
  if (is_sparse(S.path) || !S.ok) {
    const int rc = ensure_sparse(c, S);
    if (rc != MGPU_OK) return rc;
  }
  if (!sparse_usable(S))
    return set_err(c, MGPU_ERR_UNSUPPORTED,
                   std::string("no multifrontal solver for this model") + (S.sparse ? ": " + S.sparse->why : ""));
  const SparseDev& sp = *S.sparse;
  rep->nfront = sp.nfront;
  rep->nheight = sp.nheight;
  rep->nroot = sp.nroot;
  rep->max_front = sp.max_m;
  rep->max_pivots = sp.max_p;
  rep->front_entries = sp.fsize;
  rep->flops = sp.flops;
  rep->fp64 = sp.fp64_only ? 1 : 0;
  rep->last_fallback = sp.last_fallback;
  rep->last_sweeps = sp.last_sweeps;
  rep->last_perturbed = sp.last_perturbed;
  rep->last_factor_ms = sp.last_factor_ms;
  rep->last_refine_ms = sp.last_refine_ms;
  return MGPU_OK;
}

extern "C" void mgpu_solver_destroy(mgpu_ctx* c) {
  Solver* S = c->solver;
  if (!S) return;
  sparse_destroy(S->sparse);
  void* ps[] = {S->cbase, S->cn, S->ckl, S->cku, S->cdof0, S->perm, S->bmap, S->AB, S->ipiv, S->rhs, S->dx,
                S->red, S->info, S->rbase, S->lbase, S->rbmap, S->rbmapT, S->RB, S->RB32, S->UC32, S->LM32, S->UC64, S->LM64,
                S->bw, S->xw, S->rw, S->tw32, S->tw64, S->flag, S->nsweep, S->rdiag, S->part, S->cod, S->frozen,
                S->nactive, S->d_ti, S->d_tiT, S->d_ts, S->i_rbase, S->i_lbase, S->i_n, S->i_kl, S->i_ku,
                S->i_dof0, S->d_bsep, S->d_brow, S->tbmap, S->tbmapT, S->TALL, S->TUC, S->TLM, S->TY, S->DLU,
                S->FA, S->WL, S->WU, S->PV, S->trhs, S->txs, S->tpiv, S->TALL32, S->TUC32, S->TLM32, S->TY32,
                S->DLU32, S->FA32, S->WL32, S->WU32, S->i_comp,
                S->iflag, S->nbad, S->info32, S->dtmp, S->rtmp, S->rptr, S->rq, S->rcol, S->dcolptr,
                S->drowval, S->c_int0, S->c_sep0, S->list32, S->list64, S->lulist[0], S->lulist[1], S->lulist[2], S->lulist[3]};
  for (void* p : ps) cudaFree(p);
  if (S->hbuf) cudaFreeHost(S->hbuf);
  delete S;
  c->solver = nullptr;
}

namespace mgpu {
unsigned nb(int64_t n, int b) { return unsigned((n + b - 1) / b); }

// one Newton correction: factor Lλx, Δx = Lλx \ Lλ, norms -> S.red (device);
// a singular factorisation writes its component+1 to *info.  Capturable.
// Row-band factorisation and solve of all components: those whose band fits a
// 32-wide register window (kl+ku+1 <= 32) in one launch of the 32-wide
// kernels, the others in one of the 64-wide ones (a window wider than the band
// costs predicated FP64 instructions in every column).
template <typename T>
static void rb_launch(Solver& S, RbComp cp, cudaStream_t st, const T* rows, T* uc, T* lm, const double* rhs, T* tw,
                      double* out, int nref, int mode, int* nsweep, int* info) {
  // factorisation: windows of 32, 40, 48 or 64 (registers, and so resident warps, follow the window)
  if (S.nlu[0] > 0) {
    cp.list = S.lulist[0];
    rb_lu<T, 32><<<S.nlu[0], 32, 0, st>>>(cp, rows, uc, lm, S.ipiv, mode, S.flag, info);
  }
  if (S.nlu[1] > 0) {
    cp.list = S.lulist[1];
    rb_lu<T, 40><<<S.nlu[1], 32, 0, st>>>(cp, rows, uc, lm, S.ipiv, mode, S.flag, info);
  }
  if (S.nlu[2] > 0) {
    cp.list = S.lulist[2];
    rb_lu<T, 48><<<S.nlu[2], 32, 0, st>>>(cp, rows, uc, lm, S.ipiv, mode, S.flag, info);
  }
  if (S.nlu[3] > 0) {
    cp.list = S.lulist[3];
    rb_lu<T, 64><<<S.nlu[3], 32, 0, st>>>(cp, rows, uc, lm, S.ipiv, mode, S.flag, info);
  }
  // substitution: circular windows of 32 or 64 (a power of two)
  if (S.n32 > 0) {
    cp.list = S.list32;
    rb_solve<T, 32><<<S.n32, 32, 0, st>>>(cp, S.perm, S.RB, uc, lm, S.ipiv, rhs, S.bw, S.xw, S.rw, tw, out, nref, mode,
                                          S.flag, nsweep);
  }
  if (S.n64 > 0) {
    cp.list = S.list64;
    rb_solve<T, 64><<<S.n64, 32, 0, st>>>(cp, S.perm, S.RB, uc, lm, S.ipiv, rhs, S.bw, S.xw, S.rw, tw, out, nref, mode,
                                          S.flag, nsweep);
  }
}

// Buffers of the partitioned factorisation in one precision.
template <typename T>
struct TornBufs {
  T *rows, *uc, *lm, *y, *dlu, *fa, *wl, *wu;
};
static TornBufs<double> torn_bufs(Solver& S, double*) {
  return {S.TALL, S.TUC, S.TLM, S.TY, S.DLU, S.FA, S.WL, S.WU};
}
static TornBufs<float> torn_bufs(Solver& S, float*) {
  return {S.TALL32, S.TUC32, S.TLM32, S.TY32, S.DLU32, S.FA32, S.WL32, S.WU32};
}

// Partitioned factorisation of Lλx or of its transpose, already gathered into
// TALL (and TALL32).  cflag: only the components with cflag[c] != 0 (their
// interiors and Schur components flagged in iflag/tflag), or all when null.
template <typename T>
static void torn_factor(mgpu_ctx* c, bool tr, const int* cflag, int* info) {
  Solver& S = *c->solver;
  cudaStream_t st = c->stream;
  const TornBufs<T> B = torn_bufs(S, static_cast<T*>(nullptr));
  const RbComp cpI = tr ? RbComp{S.i_rbase, S.i_lbase, S.i_n, S.i_ku, S.i_kl, S.i_dof0}
                        : RbComp{S.i_rbase, S.i_lbase, S.i_n, S.i_kl, S.i_ku, S.i_dof0};
  const TornInt* ti = tr ? S.d_tiT : S.d_ti;
  const int mode = cflag ? RB_FALLBACK : RB_PLAIN;
  const T* blk = B.rows + S.tb_rows;
  if (S.twmI == 32)
    rb_lu<T, 32><<<S.nint, 32, 0, st>>>(cpI, B.rows, B.uc, B.lm, S.tpiv, mode, S.iflag, info);
  else
    rb_lu<T, 64><<<S.nint, 32, 0, st>>>(cpI, B.rows, B.uc, B.lm, S.tpiv, mode, S.iflag, info);
  if (S.nsep == 0) return;
  // forward window: kl+1 of the matrix being factorised (ku for the transpose); both <= s <= 16
  const bool narrow = S.tmaxs <= 15;
  if (S.twmI == 32 && narrow)
    tb_spikes<T, 32, 16><<<S.nint, 32, 0, st>>>(S.nint, ti, B.uc, B.lm, S.tpiv, blk, B.y, cflag);
  else if (S.twmI == 32)
    tb_spikes<T, 32, 32><<<S.nint, 32, 0, st>>>(S.nint, ti, B.uc, B.lm, S.tpiv, blk, B.y, cflag);
  else if (narrow)
    tb_spikes<T, 64, 16><<<S.nint, 32, 0, st>>>(S.nint, ti, B.uc, B.lm, S.tpiv, blk, B.y, cflag);
  else
    tb_spikes<T, 64, 32><<<S.nint, 32, 0, st>>>(S.nint, ti, B.uc, B.lm, S.tpiv, blk, B.y, cflag);
  tb_schur<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_ts, ti, blk, B.y, B.dlu, cflag);
  for (int l = 0; l < S.bcr_levels; ++l) {
    bcr_eliminate<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_bsep, l, B.dlu, B.fa, S.PV, B.wl, B.wu, cflag, info);
    bcr_update<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_bsep, l, B.dlu, B.wl, B.wu, cflag);
  }
  bcr_root<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_bsep, B.dlu, B.fa, S.PV, cflag, info);
}

// out = A⁻¹ rhs (model order, FP64 in and out) with the factors of torn_factor<T>
template <typename T>
static void torn_apply(mgpu_ctx* c, bool tr, const double* rhs, double* out, const int* cflag) {
  Solver& S = *c->solver;
  cudaStream_t st = c->stream;
  const TornBufs<T> B = torn_bufs(S, static_cast<T*>(nullptr));
  const RbComp cpI = tr ? RbComp{S.i_rbase, S.i_lbase, S.i_n, S.i_ku, S.i_kl, S.i_dof0}
                        : RbComp{S.i_rbase, S.i_lbase, S.i_n, S.i_kl, S.i_ku, S.i_dof0};
  const TornInt* ti = tr ? S.d_tiT : S.d_ti;
  const int mode = cflag ? RB_FALLBACK : RB_PLAIN;
  const T* blk = B.rows + S.tb_rows;
  T* tw = sizeof(T) == 4 ? reinterpret_cast<T*>(S.tw32) : reinterpret_cast<T*>(S.tw64);
  if (S.twmI == 32)
    rb_solve<T, 32><<<S.nint, 32, 0, st>>>(cpI, S.perm, S.TALL, B.uc, B.lm, S.tpiv, rhs, S.bw, S.xw, S.rw, tw, out, 0,
                                           mode, S.iflag, nullptr);
  else
    rb_solve<T, 64><<<S.nint, 32, 0, st>>>(cpI, S.perm, S.TALL, B.uc, B.lm, S.tpiv, rhs, S.bw, S.xw, S.rw, tw, out, 0,
                                           mode, S.iflag, nullptr);
  if (S.nsep == 0) return;
  tb_sep_rhs<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_ts, ti, blk, S.perm, rhs, out, S.trhs, cflag);
  // separators: block cyclic reduction (trhs reduced in place, txs receives z and then x)
  for (int l = 0; l < S.bcr_levels; ++l) {
    bcr_fwd_elim<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_bsep, l, B.fa, S.PV, S.d_brow, S.trhs, S.txs, cflag);
    bcr_fwd_keep<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_bsep, l, B.dlu, S.d_brow, S.trhs, S.txs, cflag);
  }
  bcr_root_solve<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_bsep, B.fa, S.PV, S.d_brow, S.trhs, S.txs, cflag);
  for (int l = S.bcr_levels - 1; l >= 0; --l)
    bcr_back<T><<<S.nsep, 32, 0, st>>>(S.nsep, S.d_bsep, l, B.wl, B.wu, S.d_brow, S.txs, cflag);
  tb_back<T><<<S.nint, 32, 0, st>>>(S.nint, ti, S.d_ts, B.y, S.perm, S.txs, out, cflag);
}

// Fused per-component partitioned solve (band_torn.cuh tb_fused): nref
// sweeps of refinement around the factors of torn_factor<T> (nref = 1 with
// d == x: a plain solve).
template <typename T>
static void torn_fused(mgpu_ctx* c, bool tr, const double* rhs, double* out, int nref, const int* only, int* flag,
                       int* nsweep, int* nbad) {
  Solver& S = *c->solver;
  const TornBufs<T> B = torn_bufs(S, static_cast<T*>(nullptr));
  TbFusedArgs A{};
  A.ncomp = S.ncomp;
  A.cint0 = S.c_int0;
  A.csep0 = S.c_sep0;
  A.cpI = tr ? RbComp{S.i_rbase, S.i_lbase, S.i_n, S.i_ku, S.i_kl, S.i_dof0}
             : RbComp{S.i_rbase, S.i_lbase, S.i_n, S.i_kl, S.i_ku, S.i_dof0};
  A.ti = tr ? S.d_tiT : S.d_ti;
  A.ts = S.d_ts;
  A.bs = S.d_bsep;
  A.nsep = S.nsep;
  A.perm = S.perm;
  A.tpiv = S.tpiv;
  A.brow = S.d_brow;
  A.tall = S.TALL;
  A.tb_rows = S.tb_rows;
  A.bw = S.bw;
  A.xw = S.xw;
  A.rw = S.rw;
  A.trhs = S.trhs;
  A.txs = S.txs;
  A.rhs = rhs;
  A.out = out;
  A.ccn = S.cn;
  A.ccdof0 = S.cdof0;
  A.nref = nref;
  A.tol_stop = 1e-12;
  A.tol_ok = 1e-10;
  A.only = only;
  A.flag = flag;
  A.nsweep = nsweep;
  A.nbad = nbad;
  TbFusedFactors<T> F{};
  F.UC = B.uc;
  F.LM = B.lm;
  F.blk = B.rows + S.tb_rows;
  F.Y = B.y;
  F.FA = B.fa;
  F.DLU = B.dlu;
  F.WL = B.wl;
  F.WU = B.wu;
  F.PV = S.PV;
  F.tw = sizeof(T) == 4 ? reinterpret_cast<T*>(S.tw32) : reinterpret_cast<T*>(S.tw64);
  const int W = sizeof(T) == 4 ? S.fuseW32 : S.fuseW64;
  if (S.twmI == 32)
    tb_fused<T, 32><<<S.ncomp, 32 * W, size_t(W) * tb_fused_warp_bytes<T, 32>(), c->stream>>>(A, F);
  else
    tb_fused<T, 64><<<S.ncomp, 32 * W, size_t(W) * tb_fused_warp_bytes<T, 64>(), c->stream>>>(A, F);
}

// Partitioned solve of Lλx (or its transpose) x = rhs.  FP64 directly, or
// (PATH_TORN32) FP32 factors inside up to S.nrefine sweeps of FP64 iterative
// refinement, then the FP64 factorisation for the components whose last
// correction is not below 1e-10 of their solution.  With few interiors per
// component (fuseW32 > 0) each solve is one launch of the fused
// per-component kernel; otherwise the solve goes level by level over all
// components.  Capturable (no host decision).
static int torn_solve(mgpu_ctx* c, bool tr, const double* rhs, double* out, int* info) {
  Solver& S = *c->solver;
  cudaStream_t st = c->stream;
  const int64_t n = c->nX;
  const bool mixed = S.path == PATH_TORN32;
  rb_gather<<<nb(c->pat.nnz, 256), 256, 0, st>>>(c->pat.nnz, tr ? S.tbmapT : S.tbmap, c->nzval, S.TALL,
                                                 mixed ? S.TALL32 : nullptr);
  const bool fused = S.fuseW32 > 0;
  if (!mixed) {
    torn_factor<double>(c, tr, nullptr, info);
    if (fused)
      torn_fused<double>(c, tr, rhs, out, 1, nullptr, nullptr, nullptr, nullptr);
    else
      torn_apply<double>(c, tr, rhs, out, nullptr);
    MG_CUDA(cudaGetLastError());
    return MGPU_OK;
  }
  torn_factor<float>(c, tr, nullptr, S.info32);
  if (fused) {
    // sweeps with an early stop per component, the check, then FP64 for the flagged components
    MG_CUDA(cudaMemsetAsync(S.nbad, 0, sizeof(int), st));
    torn_fused<float>(c, tr, rhs, out, S.nrefine, nullptr, S.flag, S.nsweep, S.nbad);
    tb_expand_flags<<<nb(S.nint, 256), 256, 0, st>>>(S.nint, S.i_comp, S.flag, S.iflag);
    torn_factor<double>(c, tr, S.flag, info);
    torn_fused<double>(c, tr, rhs, out, 1, S.flag, nullptr, nullptr, nullptr);
    MG_CUDA(cudaGetLastError());
    return MGPU_OK;
  }
  MG_CUDA(cudaMemsetAsync(out, 0, n * sizeof(double), st));
  const double* r = rhs;
  for (int sweep = 0; sweep < S.nrefine; ++sweep) {
    torn_apply<float>(c, tr, r, S.dtmp, nullptr);
    tb_axpy<<<nb(n, 256), 256, 0, st>>>(n, S.dtmp, out);
    if (sweep + 1 < S.nrefine) {
      tb_residual<<<nb(n, 256), 256, 0, st>>>(n, tr ? 1 : 0, S.rptr, S.rq, S.rcol, S.dcolptr, S.drowval, c->nzval,
                                               rhs, out, S.rtmp);
      r = S.rtmp;
    }
  }
  MG_CUDA(cudaMemsetAsync(S.nbad, 0, sizeof(int), st));
  tb_ir_check<<<S.ncomp, 32, 0, st>>>(S.cn, S.cdof0, S.perm, S.dtmp, out, S.flag, S.nbad);
  tb_expand_flags<<<nb(S.nint, 256), 256, 0, st>>>(S.nint, S.i_comp, S.flag, S.iflag);
  torn_factor<double>(c, tr, S.flag, info);
  torn_apply<double>(c, tr, rhs, out, S.flag);
  MG_CUDA(cudaGetLastError());
  return MGPU_OK;
}

int factor_solve(mgpu_ctx* c, int* info) {
  Solver& S = *c->solver;
  cudaStream_t st = c->stream;
  if (is_sparse(S.path)) {
    const int rc = sparse_factor_solve(c, *S.sparse, c->Ll, S.dx, info);
    if (rc) return rc;
    if (S.sparse->fp64_only && S.path == PATH_SPARSE) S.path = PATH_SPARSE64;  // after a fallback
  } else if (S.path == PATH_TORN || S.path == PATH_TORN32) {
    const int rc = torn_solve(c, false, c->Ll, S.dx, info);
    if (rc) return rc;
  } else if (S.path == PATH_BLOCK) {
    MG_CUDA(cudaMemsetAsync(S.AB, 0, S.band_total * sizeof(double), st));
    band_gather<<<nb(c->pat.nnz, 256), 256, 0, st>>>(c->pat.nnz, S.bmap, c->nzval, S.AB);
    band_lu<<<S.ncomp, 128, 0, st>>>(S.cbase, S.cn, S.ckl, S.cku, S.cdof0, S.AB, S.ipiv, S.rdiag, info);
    band_solve<<<S.ncomp, 128, 0, st>>>(S.cbase, S.cn, S.ckl, S.cku, S.cdof0, S.perm, S.AB, S.ipiv, S.rdiag, c->Ll,
                                        S.rhs, S.dx);
  } else {
    // one warp per component, one per block, so that the components spread over all SMs
    const RbComp cp{S.rbase, S.lbase, S.cn, S.ckl, S.cku, S.cdof0};
    rb_gather<<<nb(c->pat.nnz, 256), 256, 0, st>>>(c->pat.nnz, S.rbmap, c->nzval, S.RB,
                                                   S.path == PATH_F32IR ? S.RB32 : nullptr);
    const int mode64 = S.path == PATH_F32IR ? RB_FALLBACK : RB_PLAIN;
    if (S.path == PATH_F32IR) {
      MG_CUDA(cudaMemsetAsync(S.flag, 0, S.ncomp * sizeof(int), st));
      rb_launch<float>(S, cp, st, S.RB32, S.UC32, S.LM32, c->Ll, S.tw32, S.dx, S.nref, RB_PRIMARY, S.nsweep, info);
    }
    // FP64: the whole solve (PATH_F64ROWS) or the components flagged above
    rb_launch<double>(S, cp, st, S.RB, S.UC64, S.LM64, c->Ll, S.tw64, S.dx, 0, mode64, nullptr, info);
  }
  norms_partial<<<kNormBlocks, 256, 0, st>>>(c->nX, S.dx, c->Ll, S.part);
  norms_final<<<1, 32, 0, st>>>(kNormBlocks, S.part, S.red);
  c->launches += 2;
  MG_CUDA(cudaGetLastError());
  return MGPU_OK;
}

int factor_solve_T(mgpu_ctx* c, const double* rhs, double* out, int* info) {
  Solver& S = *c->solver;
  if (is_sparse(S.path))
    return set_err(c, MGPU_ERR_UNSUPPORTED, "transposed solve needs a banded solver kind (not the multifrontal one)");
  if (S.path == PATH_TORN || S.path == PATH_TORN32) return torn_solve(c, true, rhs, out, info);
  if (!S.wmT)
    return set_err(c, MGPU_ERR_UNSUPPORTED,
                   "transposed solve needs the row-band kernels (kl, ku <= 31 and kl+ku+1 <= 64 in every component)");
  cudaStream_t st = c->stream;
  const RbComp cpT{S.rbase, S.lbase, S.cn, S.cku, S.ckl, S.cdof0};  // the transpose: kl and ku exchange
  rb_gather<<<nb(c->pat.nnz, 256), 256, 0, st>>>(c->pat.nnz, S.rbmapT, c->nzval, S.RB, nullptr);
  rb_launch<double>(S, cpT, st, S.RB, S.UC64, S.LM64, rhs, S.tw64, out, 0, RB_PLAIN, nullptr, info);
  MG_CUDA(cudaGetLastError());
  return MGPU_OK;
}
}  // namespace mgpu

namespace mgpu {
mgpu_newmark newmark_coefficients(double beta, double gamma, double dt) {
  // Newmarkβcoefficients (src/SweepX.jl:3-15)
  return mgpu_newmark{gamma / (beta * dt), gamma / beta, (gamma / (2 * beta) - 1) * dt, 1 / (beta * dt * dt),
                      1 / (beta * dt), 1 / (2 * beta)};
}

static int singular_error(mgpu_ctx* c, mgpu_stats* stats, int64_t step, int it) {
  stats->fail_step = int(step + 1);
  stats->fail_iter = it;
  char msg[128];
  snprintf(msg, sizeof msg, "matrix factorization failed at step=%d, iiter=%d", int(step + 1), it);
  return set_err(c, MGPU_ERR_SINGULAR, msg);
}

int newton_step(mgpu_ctx* c, int OX, int64_t step, double t, double dt, const double* tvals_step,
                const mgpu_sweep_opts* opts, mgpu_stats* stats) {
  Solver& S = *c->solver;
  cudaStream_t st = c->stream;
  const int64_t n = c->nX;
  const bool percomp = opts->per_component != 0;
  const double cdx2 = opts->maxdx * opts->maxdx, cLl2 = opts->maxLl * opts->maxLl;
  const mgpu_newmark nm = OX == 2 ? newmark_coefficients(opts->beta, opts->gamma, dt) : mgpu_newmark{0, 0, 0, 0, 0, 0};
  int rc = upload_stepc(c, t, OX == 2 ? &nm : nullptr);
  if (rc) return rc;
  if (c->ntval > 0)
    MG_CUDA(cudaMemcpyAsync(c->tv, tvals_step, c->ntval * sizeof(double), cudaMemcpyHostToDevice, st));
  if (percomp) MG_CUDA(cudaMemsetAsync(S.frozen, 0, std::max(S.ncomp, 1) * sizeof(int), st));
  const int itmax = opts->fixed_iter > 0 ? opts->fixed_iter : opts->maxiter;
  for (int it = 1; it <= itmax; ++it) {
    stats->niter_total++;
    const int first = it == 1;
    const int mission = OX == 0 ? MGPU_ASM_STATIC : (first ? MGPU_ASM_STEP : MGPU_ASM_ITER);
    launch_reset_errflag(c);
    MG_CUDA(cudaMemsetAsync(S.info, 0, sizeof(int), st));
    rc = launch_assembly(c, mission, nullptr);
    if (rc) return rc;
    rc = factor_solve(c, S.info);
    if (rc) return rc;
    decrement_kernel<<<nb(n, 256), 256, 0, st>>>(n, OX, first, S.dx, c->scale, c->stepc, c->x,
                                                  percomp ? S.frozen : nullptr, S.cod);
    ++c->launches;
    if (percomp) {
      MG_CUDA(cudaMemsetAsync(S.nactive, 0, sizeof(int), st));
      comp_converge<<<S.ncomp, 32, 0, st>>>(S.cn, S.cdof0, S.perm, S.dx, c->Ll, cdx2, cLl2, S.frozen, S.nactive);
    }
    MG_CUDA(cudaMemcpyAsync(S.hbuf, S.red, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    int* hi = reinterpret_cast<int*>(S.hbuf + 2);
    MG_CUDA(cudaMemcpyAsync(hi, S.info, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CUDA(cudaMemcpyAsync(hi + 1, c->errflag, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (percomp) MG_CUDA(cudaMemcpyAsync(hi + 2, S.nactive, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (S.path == PATH_TORN32) MG_CUDA(cudaMemcpyAsync(hi + 3, S.nbad, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CUDA(cudaStreamSynchronize(st));
    if (S.path == PATH_TORN32 && hi[3] > 0 && S.adaptive) S.path = PATH_TORN;  // FP32 refinement falls short here
    const double dx2 = S.hbuf[0], Ll2 = S.hbuf[1];
    stats->last_dx = std::sqrt(dx2);
    stats->last_Ll = std::sqrt(Ll2);
    if (hi[1] != INT_MAX) {
      stats->fail_step = int(step + 1);
      stats->fail_iter = it;
      return nan_error(c, hi[1]);
    }
    if (hi[0] != 0) return singular_error(c, stats, step, it);
    if (opts->fixed_iter > 0) {
      if (it == opts->fixed_iter) break;
      continue;
    }
    const bool done = percomp ? hi[2] == 0 : (dx2 <= cdx2 && Ll2 <= cLl2);
    if (done) break;
    if (it == opts->maxiter) {
      stats->fail_step = int(step + 1);
      stats->fail_iter = it;
      std::string which;
      if (percomp) {
        std::vector<int> fz(S.ncomp);
        MG_CUDA(cudaMemcpy(fz.data(), S.frozen, S.ncomp * sizeof(int), cudaMemcpyDeviceToHost));
        int first_open = 0;
        while (first_open < S.ncomp && fz[first_open]) ++first_open;
        which = " (" + std::to_string(hi[2]) + " components, the first is component " + std::to_string(first_open + 1) +
                ")";
      }
      char msg[256];
      snprintf(msg, sizeof msg, "no convergence of step %3d after %3d iterations |Δx|=%g / %g, |Lλ|=%g / %g",
               int(step + 1), it, std::sqrt(dx2), opts->maxdx, Ll2, opts->maxLl);
      return set_err(c, MGPU_ERR_NOCONV, msg + which);
    }
  }
  return MGPU_OK;
}

// Fixed-iteration steps replayed from one captured CUDA graph: per step the
// host uploads t, the Newmark coefficients and the load values (pinned,
// double-buffered), launches the graph, and queues the state and the error
// flags back; it waits only at the end.  Errors are then reported for the
// first failing step, with the states of the steps before it.
static int sweep_graph(mgpu_ctx* c, int OX, int64_t nstep, const double* times, double t0, const double* tvals,
                       const mgpu_sweep_opts* opts, double* states, mgpu_stats* stats) {
  Solver& S = *c->solver;
  cudaStream_t st = c->stream;
  const int64_t n = c->nX;
  const int nder = OX + 1, nit = opts->fixed_iter;
  // steps with a positive time step (the reference stops at the first that is not)
  int64_t nrun = nstep;
  {
    double told = t0;
    for (int64_t k = 0; k < nstep; ++k) {
      if (OX > 0 && !(times[k] - told > 0)) {
        nrun = k;
        break;
      }
      told = times[k];
    }
  }
  const int64_t slot = 8 + c->ntval;
  double* hbuf = nullptr;
  int* hflags = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool registered = false;
  int rc = MGPU_OK;
  const size_t state_bytes = size_t(nstep) * nder * n * sizeof(double);
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (hbuf) cudaFreeHost(hbuf);
    if (hflags) cudaFreeHost(hflags);
    if (registered) cudaHostUnregister(states);
    cudaGetLastError();
  };
#define MG_G(call)                                                                                        \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) {                                                                              \
      rc = set_err(c, MGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                 \
      cleanup();                                                                                          \
      return rc;                                                                                          \
    }                                                                                                     \
  } while (0)
  MG_G(cudaMallocHost(&hbuf, 2 * slot * sizeof(double)));
  MG_G(cudaMallocHost(&hflags, std::max<int64_t>(nrun, 1) * (nit + 1) * sizeof(int)));
  for (auto& e : ev) MG_G(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  if (state_bytes > 0) {
    registered = cudaHostRegister(states, state_bytes, cudaHostRegisterDefault) == cudaSuccess;
    if (!registered) cudaGetLastError();  // pageable copies still work, synchronously
  }
  // capture one step
  MG_G(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  launch_reset_errflag(c);
  cudaMemsetAsync(S.info, 0, kInfoSlots * sizeof(int), st);
  for (int it = 1; it <= nit && rc == MGPU_OK; ++it) {
    const int mission = OX == 0 ? MGPU_ASM_STATIC : (it == 1 ? MGPU_ASM_STEP : MGPU_ASM_ITER);
    rc = launch_assembly(c, mission, nullptr);
    if (rc == MGPU_OK) rc = factor_solve(c, S.info + it);
    if (rc == MGPU_OK)
      decrement_kernel<<<nb(n, 256), 256, 0, st>>>(n, OX, it == 1, S.dx, c->scale, c->stepc, c->x, nullptr,
                                                    nullptr);
  }
  {
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc != MGPU_OK) {
      cleanup();
      return rc;
    }
    MG_G(e);
  }
  MG_G(cudaGraphInstantiate(&exec, graph, 0));
  double told = t0;
  for (int64_t step = 0; step < nrun; ++step) {
    const double t = times[step], dt = t - told;
    told = t;
    const mgpu_newmark nm = OX == 2 ? newmark_coefficients(opts->beta, opts->gamma, dt) : mgpu_newmark{0, 0, 0, 0, 0, 0};
    const int k = int(step & 1);
    MG_G(cudaEventSynchronize(ev[k]));  // the upload two steps back has read this slot
    double* h = hbuf + k * slot;
    const double v[8] = {t, nm.a1, nm.a2, nm.a3, nm.b1, nm.b2, nm.b3, 0.0};
    for (int q = 0; q < 8; ++q) h[q] = v[q];
    for (int64_t q = 0; q < c->ntval; ++q) h[8 + q] = tvals[step * c->ntval + q];
    MG_G(cudaMemcpyAsync(c->stepc, h, 8 * sizeof(double), cudaMemcpyHostToDevice, st));
    if (c->ntval > 0) MG_G(cudaMemcpyAsync(c->tv, h + 8, c->ntval * sizeof(double), cudaMemcpyHostToDevice, st));
    MG_G(cudaEventRecord(ev[k], st));
    MG_G(cudaGraphLaunch(exec, st));
    MG_G(cudaMemcpyAsync(states + step * nder * n, c->x, nder * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    int* f = hflags + step * (nit + 1);
    MG_G(cudaMemcpyAsync(f, c->errflag, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_G(cudaMemcpyAsync(f + 1, S.info + 1, nit * sizeof(int), cudaMemcpyDeviceToHost, st));
  }
  MG_G(cudaMemcpyAsync(S.hbuf, S.red, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (S.path == PATH_TORN32)
    MG_G(cudaMemcpyAsync(reinterpret_cast<int*>(S.hbuf + 2), S.nbad, sizeof(int), cudaMemcpyDeviceToHost, st));
  MG_G(cudaStreamSynchronize(st));
  stats->last_dx = std::sqrt(S.hbuf[0]);
  stats->last_Ll = std::sqrt(S.hbuf[1]);
  if (S.path == PATH_TORN32 && *reinterpret_cast<int*>(S.hbuf + 2) > 0 && S.adaptive) S.path = PATH_TORN;
  for (int64_t step = 0; step < nrun; ++step) {
    const int* f = hflags + step * (nit + 1);
    // within a step the NaN check of an iteration precedes its factorisation
    int bad_it = 0;
    for (int it = 1; it <= nit && !bad_it; ++it)
      if (f[it] != 0) bad_it = it;
    if (f[0] != INT_MAX || bad_it) {
      stats->nstep_done = int(step);
      stats->niter_total = int(step) * nit + (bad_it ? bad_it : 1);
      if (f[0] != INT_MAX) {
        stats->fail_step = int(step + 1);
        stats->fail_iter = 0;
        rc = nan_error(c, f[0]);
      } else {
        rc = singular_error(c, stats, step, bad_it);
      }
      cleanup();
      return rc;
    }
  }
  stats->nstep_done = int(nrun);
  stats->niter_total = int(nrun) * nit;
  cleanup();
#undef MG_G
  if (nrun < nstep) {
    stats->fail_step = int(nrun + 1);
    char msg[128];
    snprintf(msg, sizeof msg, "Time step length not strictly positive at step=%3d", int(nrun + 1));
    return set_err(c, MGPU_ERR_ARG, msg);
  }
  return MGPU_OK;
}
}  // namespace mgpu

// ---------------------------------------------------------------- the Newton loop on the device
// SweepX{0} as one graph launch: a conditional WHILE node over the load steps
// whose body copies the step's constants and load values into place, runs a
// nested WHILE node over the Newton iterations and stores the converged state.
// The iteration body is the captured iteration (assembly, factorisation and
// solve, decrement, convergence test) followed by a controller kernel that
// counts the iteration and ends the loop when every model has converged (or
// the whole system, without per_component), when maxiter is reached, or on a
// NaN or singular factorisation.  The host reads nothing until the sweep ends.
namespace {
struct DevLoop {
  int* step = nullptr;     // current step
  int* iter = nullptr;     // iterations of the current step
  int* status = nullptr;   // [nstep] 0 converged, 1 no convergence, 2 singular, 3 NaN, -1 not run
  int* iters = nullptr;    // [nstep] iterations taken
  double* stepc = nullptr;  // [nstep][8] t and the Newmark coefficients (zero for SweepX{0})
  double* tv = nullptr;    // [nstep][ntval]
  double* states = nullptr;  // [nstep][n]
};

__global__ void dl_step_begin(const int* __restrict__ step, const double* __restrict__ stepc_all,
                              const double* __restrict__ tv_all, int64_t ntval, double* __restrict__ stepc,
                              double* __restrict__ tv, int* __restrict__ iter, int* __restrict__ frozen, int ncomp,
                              cudaGraphConditionalHandle hi) {
  const int64_t k = *step;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < 8) stepc[i] = stepc_all[k * 8 + i];
  if (i < ntval) tv[i] = tv_all[k * ntval + i];
  if (frozen && i < ncomp) frozen[i] = 0;
  if (i == 0) {
    *iter = 0;
    cudaGraphSetConditional(hi, 1u);
  }
}

__global__ void dl_iter_ctl(const int* __restrict__ step, int* __restrict__ iter, int maxiter, int percomp,
                            const int* __restrict__ nactive, const double* __restrict__ red, double cdx2, double cLl2,
                            const int* __restrict__ info, const int* __restrict__ errflag, int* __restrict__ status,
                            int* __restrict__ iters, cudaGraphConditionalHandle hi) {
  const int it = ++*iter;
  const bool conv = percomp ? *nactive == 0 : (red[0] <= cdx2 && red[1] <= cLl2);
  const bool nan = *errflag != INT_MAX, sing = *info != 0;
  const int k = *step;
  iters[k] = it;
  if (nan || sing || conv || it >= maxiter) {
    status[k] = nan ? 3 : sing ? 2 : conv ? 0 : 1;
    cudaGraphSetConditional(hi, 0u);
  } else {
    cudaGraphSetConditional(hi, 1u);
  }
}

__global__ void dl_store(const int* __restrict__ step, const double* __restrict__ x, int64_t n,
                         double* __restrict__ states) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) states[int64_t(*step) * n + i] = x[i];
}

__global__ void dl_step_next(int* __restrict__ step, int nstep, const int* __restrict__ status,
                             cudaGraphConditionalHandle hs) {
  const int k = *step;
  *step = k + 1;
  cudaGraphSetConditional(hs, (status[k] == 0 && k + 1 < nstep) ? 1u : 0u);
}

cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, size_t ndeps,
                       const void* func, unsigned grid, unsigned block, void** args) {
  cudaKernelNodeParams kp = {};
  kp.func = const_cast<void*>(func);
  kp.gridDim = dim3(grid);
  kp.blockDim = dim3(block);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  kp.extra = nullptr;
  return cudaGraphAddKernelNode(node, g, deps, ndeps, &kp);
}
}  // namespace

static int sweep_device_loop(mgpu_ctx* c, int64_t nstep, const double* times, const double* tvals,
                             const mgpu_sweep_opts* opts, double* states, mgpu_stats* stats) {
  Solver& S = *c->solver;
  cudaStream_t st = c->stream;
  const int64_t n = c->nX;
  const bool percomp = opts->per_component != 0;
  DevLoop d;
  cudaGraph_t g = nullptr, bs = nullptr, bi = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> owned;
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
    for (void* p : owned) cudaFree(p);
    cudaGetLastError();
  };
  auto fail = [&](cudaError_t e, const char* what) {
    const int rc = set_err(c, MGPU_ERR_CUDA, std::string("device Newton loop: ") + what + ": " + cudaGetErrorString(e));
    cleanup();
    return rc;
  };
  auto alloc = [&](auto** p, size_t count) -> cudaError_t {
    using T = typename std::remove_pointer<typename std::remove_reference<decltype(*p)>::type>::type;
    const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) owned.push_back(*p);
    return e;
  };
  cudaError_t e = cudaSuccess;
  for (auto r : {alloc(&d.step, 1), alloc(&d.iter, 1), alloc(&d.status, nstep), alloc(&d.iters, nstep),
                 alloc(&d.stepc, size_t(nstep) * 8), alloc(&d.tv, size_t(nstep) * c->ntval),
                 alloc(&d.states, size_t(nstep) * n)})
    if (e == cudaSuccess) e = r;
  if (e != cudaSuccess) {
    cleanup();
    return set_err(c, MGPU_ERR_NOMEM, "device Newton loop: device allocation failed");
  }
  {
    std::vector<double> sc(size_t(nstep) * 8, 0.0);
    for (int64_t k = 0; k < nstep; ++k) sc[k * 8] = times[k];
    std::vector<int> minus(nstep, -1);
    if ((e = cudaMemcpy(d.stepc, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (c->ntval > 0 && (e = cudaMemcpy(d.tv, tvals, size_t(nstep) * c->ntval * sizeof(double),
                                         cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (e = cudaMemcpy(d.status, minus.data(), nstep * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(d.step, 0, sizeof(int))) != cudaSuccess || (e = cudaMemset(d.iters, 0, nstep * sizeof(int))) != cudaSuccess)
      return fail(e, "upload");
  }
  // graph: WHILE(steps) { begin ; WHILE(iterations) { iteration ; controller } ; store ; next }
  cudaGraphConditionalHandle hs, hi;
  if ((e = cudaGraphCreate(&g, 0)) != cudaSuccess) return fail(e, "graph");
  if ((e = cudaGraphConditionalHandleCreate(&hs, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
    return fail(e, "conditional handle");
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hs;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t nsteps;
  if ((e = cudaGraphAddNode(&nsteps, g, nullptr, nullptr, 0, &cp)) != cudaSuccess) return fail(e, "step loop node");
  bs = cp.conditional.phGraph_out[0];
  if ((e = cudaGraphConditionalHandleCreate(&hi, bs, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
    return fail(e, "conditional handle");
  const int64_t ntv = c->ntval;
  int* frozen = percomp ? S.frozen : nullptr;
  int ncomp = S.ncomp;
  cudaGraphNode_t kbegin, niter, kstore, knext;
  {
    void* args[] = {&d.step, &d.stepc, &d.tv, const_cast<int64_t*>(&ntv), &c->stepc, &c->tv, &d.iter, &frozen, &ncomp,
                    &hi};
    const int64_t cnt = std::max<int64_t>(std::max<int64_t>(ntv, 8), percomp ? ncomp : 0);
    if ((e = add_kernel(bs, &kbegin, nullptr, 0, reinterpret_cast<const void*>(dl_step_begin), nb(cnt, 256), 256,
                        args)) != cudaSuccess)
      return fail(e, "step begin node");
  }
  cudaGraphNodeParams ip = {};
  ip.type = cudaGraphNodeTypeConditional;
  ip.conditional.handle = hi;
  ip.conditional.type = cudaGraphCondTypeWhile;
  ip.conditional.size = 1;
  if ((e = cudaGraphAddNode(&niter, bs, &kbegin, nullptr, 1, &ip)) != cudaSuccess) return fail(e, "iteration loop node");
  bi = ip.conditional.phGraph_out[0];
  {
    double* xs = c->x;
    int64_t nn = n;
    void* args[] = {&d.step, &xs, &nn, &d.states};
    if ((e = add_kernel(bs, &kstore, &niter, 1, reinterpret_cast<const void*>(dl_store), nb(n, 256), 256, args)) !=
        cudaSuccess)
      return fail(e, "store node");
    int ns = int(nstep);
    void* args2[] = {&d.step, &ns, &d.status, &hs};
    if ((e = add_kernel(bs, &knext, &kstore, 1, reinterpret_cast<const void*>(dl_step_next), 1, 1, args2)) !=
        cudaSuccess)
      return fail(e, "next-step node");
  }
  // the iteration body, captured
  const double cdx2 = opts->maxdx * opts->maxdx, cLl2 = opts->maxLl * opts->maxLl;
  if ((e = cudaStreamBeginCaptureToGraph(st, bi, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return fail(e, "capture");
  {
    launch_reset_errflag(c);
    cudaMemsetAsync(S.info, 0, sizeof(int), st);
    int rc = launch_assembly(c, MGPU_ASM_STATIC, nullptr);
    if (rc == MGPU_OK) rc = factor_solve(c, S.info);
    if (rc == MGPU_OK) {
      decrement_kernel<<<nb(n, 256), 256, 0, st>>>(n, 0, 1, S.dx, c->scale, c->stepc, c->x, frozen, S.cod);
      if (percomp) {
        cudaMemsetAsync(S.nactive, 0, sizeof(int), st);
        comp_converge<<<S.ncomp, 32, 0, st>>>(S.cn, S.cdof0, S.perm, S.dx, c->Ll, cdx2, cLl2, S.frozen, S.nactive);
      }
      dl_iter_ctl<<<1, 1, 0, st>>>(d.step, d.iter, opts->maxiter, int(percomp), S.nactive, S.red, cdx2, cLl2, S.info,
                                   c->errflag, d.status, d.iters, hi);
    }
    cudaGraph_t out = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &out);
    if (rc != MGPU_OK) {
      cleanup();
      return rc;
    }
    if (ec != cudaSuccess) return fail(ec, "capture of the iteration");
  }
  if ((e = cudaGraphInstantiate(&exec, g, 0)) != cudaSuccess) return fail(e, "instantiate");
  if ((e = cudaGraphLaunch(exec, st)) != cudaSuccess) return fail(e, "launch");
  std::vector<int> status(nstep), iters(nstep);
  if ((e = cudaMemcpyAsync(status.data(), d.status, nstep * sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(iters.data(), d.iters, nstep * sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail(e, "sweep");
  int64_t done = 0;
  while (done < nstep && status[done] == 0) ++done;
  for (int64_t k = 0; k < nstep && k <= done && k < int64_t(iters.size()); ++k) stats->niter_total += iters[k];
  if (done > 0 && (e = cudaMemcpy(states, d.states, size_t(done) * n * sizeof(double), cudaMemcpyDeviceToHost)) !=
                      cudaSuccess)
    return fail(e, "states");
  stats->nstep_done = int(done);
  int rc = MGPU_OK;
  if (done < nstep) {
    const int k = int(done);
    stats->fail_step = k + 1;
    stats->fail_iter = iters[k];
    if (status[k] == 3) {
      int flag = INT_MAX;
      cudaMemcpy(&flag, c->errflag, sizeof(int), cudaMemcpyDeviceToHost);
      rc = nan_error(c, flag);
    } else if (status[k] == 2) {
      rc = singular_error(c, stats, k, iters[k]);
    } else {
      char msg[160];
      snprintf(msg, sizeof msg, "no convergence of step %3d after %3d iterations", k + 1, iters[k]);
      rc = set_err(c, MGPU_ERR_NOCONV, msg);
    }
  }
  cleanup();
  return rc;
}

extern "C" int mgpu_sweepx(mgpu_ctx* c, int32_t OX, int64_t nstep, const double* times, double t0, int32_t nXder0,
                           const double* x0, const double* u, const double* tvals, const mgpu_sweep_opts* opts,
                           double* states, mgpu_stats* stats) {
  if (!c || !times || !opts || !states || !stats || !(OX == 0 || OX == 2) || nstep < 0 || nXder0 < 0 ||
      nXder0 > OX + 1 || (nXder0 > 0 && !x0) || (c->ntval > 0 && nstep > 0 && !tvals))
    return set_err(c, MGPU_ERR_ARG, "mgpu_sweepx: bad arguments");
  if (opts->per_component && opts->fixed_iter > 0)
    return set_err(c, MGPU_ERR_ARG, "mgpu_sweepx: per_component needs the convergence test (fixed_iter = 0)");
  *stats = mgpu_stats{0, 0, 0, 0, 0.0, 0.0};
  Solver& S = *c->solver;
  const bool sparse = is_sparse(S.path);
  MG_CUDA(cudaSetDevice(c->device));
  if (sparse) {
    const int rc = ensure_sparse(c, S);
    if (rc != MGPU_OK) return rc;
    if (!sparse_usable(S))
      return set_err(c, MGPU_ERR_UNSUPPORTED, "no device solver for this model: " + S.why + "; multifrontal solver: " +
                                                  S.sparse->why);
  }
  if (!S.ok && !sparse)
    return set_err(c, MGPU_ERR_UNSUPPORTED,
                   "no device solver for this model: " + S.why +
                       (S.sparse ? "; multifrontal solver: " + S.sparse->why : std::string()));
  if (sparse && opts->per_component)
    return set_err(c, MGPU_ERR_UNSUPPORTED, "per-component convergence needs a banded solver kind");
  MG_CUDA(cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  const int64_t n = c->nX;
  // initial state
  MG_CUDA(cudaMemsetAsync(c->x, 0, 3 * n * sizeof(double), st));
  if (nXder0 > 0) MG_CUDA(cudaMemcpyAsync(c->x, x0, nXder0 * n * sizeof(double), cudaMemcpyHostToDevice, st));
  if (c->nU > 0 && u) MG_CUDA(cudaMemcpyAsync(c->u, u, c->nU * sizeof(double), cudaMemcpyHostToDevice, st));
  c->nXder_resident = OX + 1;
  // the multifrontal solve decides its FP64 fallback on the host: launched step by step
  if (opts->fixed_iter > 0 && opts->fixed_iter < kInfoSlots && !opts->no_graph && !sparse)
    return sweep_graph(c, OX, nstep, times, t0, tvals, opts, states, stats);
  if (opts->device_loop) {
    if (OX != 0 || sparse || opts->fixed_iter > 0 || S.path == PATH_TORN32)
      return set_err(c, MGPU_ERR_UNSUPPORTED, "the device Newton loop runs SweepX{0} with a banded FP64 or F32IR "
                                              "solver and the convergence test");
    if (nstep == 0) return MGPU_OK;
    return sweep_device_loop(c, nstep, times, tvals, opts, states, stats);
  }
  const int nder = OX + 1;
  double told = t0;
  for (int64_t step = 0; step < nstep; ++step) {
    const double t = times[step];
    const double dt = t - told;
    told = t;
    if (OX > 0 && !(dt > 0)) {
      stats->fail_step = int(step + 1);
      char msg[128];
      snprintf(msg, sizeof msg, "Time step length not strictly positive at step=%3d", int(step + 1));
      return set_err(c, MGPU_ERR_ARG, msg);
    }
    const int rc = newton_step(c, OX, step, t, dt, c->ntval > 0 ? tvals + step * c->ntval : nullptr, opts, stats);
    if (rc) return rc;
    MG_CUDA(cudaMemcpyAsync(states + step * nder * n, c->x, nder * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    MG_CUDA(cudaStreamSynchronize(st));
    stats->nstep_done = int(step + 1);
  }
  return MGPU_OK;
}
