// Bar3D residual and Newton tangent for the element kernels.
//
// Reference behaviour: toolbox/BarElement.jl:136-202 (resultants, residual).
// The bar's Gauss-point kinematics are explicit: x = cₘ + ½(u₁+u₂) + tg ζ with
// tg = tgₘ + u₂ − u₁, so velocities and accelerations are linear in X₁, X₂ and
// the residual is an explicit function of (X₀, X₁, X₂).  Its tangent along the
// Newton variation X₀+p0δ, X₁+p1δ, X₂+p2δ (and the Newmark δr direction) is
// computed with a first-order dual carrying one partial per dof plus one.
#pragma once
#include "tj.hpp"

namespace mgpu {

template <int N>
struct Dn {
  double x;
  double d[N];
};
template <int N>
MG_HD Dn<N> dn_c(double c) {
  Dn<N> r;
  r.x = c;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N>
MG_HD Dn<N> operator+(const Dn<N>& a, const Dn<N>& b) {
  Dn<N> r;
  r.x = a.x + b.x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
MG_HD Dn<N> operator-(const Dn<N>& a, const Dn<N>& b) {
  Dn<N> r;
  r.x = a.x - b.x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
MG_HD Dn<N> operator*(const Dn<N>& a, const Dn<N>& b) {
  Dn<N> r;
  r.x = a.x * b.x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fma(a.d[i], b.x, a.x * b.d[i]);
  return r;
}
template <int N>
MG_HD Dn<N> operator*(const Dn<N>& a, double s) {
  Dn<N> r;
  r.x = a.x * s;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * s;
  return r;
}
template <int N>
MG_HD Dn<N> operator+(const Dn<N>& a, double s) {
  Dn<N> r = a;
  r.x += s;
  return r;
}
template <int N>
MG_HD Dn<N> dn_apply(const Dn<N>& a, double f0, double f1) {
  Dn<N> r;
  r.x = f0;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = f1 * a.d[i];
  return r;
}

struct BarConst {
  double tgm[3];
  double L0, Ls;
  double EA, mu, w, Cat, Clt, Cqt, Can, Cln, Cqn;
  double wgp[4], zgp[4];
};

// Bar fields (BarElement.jl:89-101 declaration order, 38 doubles) -> constants.
MG_HD void bar_const_from_fields(const double* f, BarConst& c) {
  for (int k = 0; k < 3; ++k) c.tgm[k] = f[3 + k];
  c.L0 = f[9];
  c.Ls = f[10];
  c.EA = f[11];
  c.mu = f[12];
  c.w = f[13];
  c.Cat = f[14];
  c.Clt = f[15];
  c.Cqt = f[16];
  c.Can = f[17];
  c.Cln = f[18];
  c.Cqn = f[19];
  for (int g = 0; g < 4; ++g) {
    c.wgp[g] = f[20 + g];
    c.zgp[g] = f[24 + g];
  }
}

// R[6], K[36] (column-major), rdir[6] optional, H[18] optional (∂R/∂U).
MG_HD void bar_element(const BarConst& c, int nder, const double* X0, const double* X1, const double* X2,
                       const double* U, double t, double p0, double p1, double p2, const double* av, const double* bv,
                       double* R, double* K, double* rdir, double* H) {
  constexpr int N = 7;  // six dof directions + δr
  Dn<N> x0[6], x1[6], x2[6];
  for (int i = 0; i < 6; ++i) {
    x0[i] = dn_c<N>(X0[i]);
    x1[i] = dn_c<N>(nder > 1 ? X1[i] : 0.0);
    x2[i] = dn_c<N>(nder > 2 ? X2[i] : 0.0);
    x0[i].d[i] = p0;
    x1[i].d[i] = p1;
    x2[i].d[i] = p2;
    x1[i].d[6] = av ? av[i] : 0.0;
    x2[i].d[6] = bv ? bv[i] : 0.0;
  }
  Dn<N> tg[3];
  for (int i = 0; i < 3; ++i) tg[i] = x0[3 + i] - x0[i] + c.tgm[i];
  const Dn<N> L2 = tg[0] * tg[0] + tg[1] * tg[1] + tg[2] * tg[2];
  const double Lv = sqrt(L2.x);
  const Dn<N> L = dn_apply(L2, Lv, 0.5 / Lv);
  const Dn<N> iL = dn_apply(L, 1.0 / Lv, -1.0 / (Lv * Lv));
  Dn<N> dl[3];
  for (int i = 0; i < 3; ++i) dl[i] = tg[i] * iL;
  const Dn<N> eps = L * (1.0 / c.Ls) + (-1.0);
  const Dn<N> fint = eps * c.EA;
  Dn<N> edX[6];
  for (int i = 0; i < 3; ++i) {
    edX[i] = dl[i] * (-1.0 / c.L0);
    edX[3 + i] = dl[i] * (1.0 / c.L0);
  }
  const double fw3 = ((t < -5.0 ? t : -5.0) + 10.0) / 5.0 * c.w;
  Dn<N> Ro[6];
  for (int i = 0; i < 6; ++i) Ro[i] = dn_c<N>(0.0);
  for (int g = 0; g < 4; ++g) {
    const double z = c.zgp[g];
    const double ps1 = -z + 0.5, ps2 = z + 0.5;
    Dn<N> v[3], a[3];
    for (int i = 0; i < 3; ++i) {
      // ∂1(x), ∂2(x) of x = c + tg ζ = ψ₁ u₁ + ψ₂ u₂ + const
      v[i] = x1[i] * ps1 + x1[3 + i] * ps2;
      a[i] = x2[i] * ps1 + x2[3 + i] * ps2;
    }
    const Dn<N> at = a[0] * dl[0] + a[1] * dl[1] + a[2] * dl[2];
    const Dn<N> vt = v[0] * dl[0] + v[1] * dl[1] + v[2] * dl[2];
    Dn<N> an[3], vn[3];
    for (int i = 0; i < 3; ++i) {
      an[i] = a[i] - at * dl[i];
      vn[i] = v[i] - vt * dl[i];
    }
    Dn<N> fqt = vt * vt * c.Cqt;
    if (vt.x < 0.0) fqt = fqt * -1.0;
    Dn<N> fq2 = vn[1] * vn[1] * c.Cqn;
    if (vn[1].x < 0.0) fq2 = fq2 * -1.0;
    Dn<N> fq3 = vn[2] * vn[2] * c.Cqn;
    if (vn[2].x < 0.0) fq3 = fq3 * -1.0;
    Dn<N> fe[3];
    fe[0] = a[0] * c.mu + at * c.Cat + vt * c.Clt + fqt;
    fe[1] = a[1] * c.mu + an[1] * c.Can + vn[1] * c.Cln + fq2;
    fe[2] = a[2] * c.mu + an[2] * c.Can + vn[2] * c.Cln + fq3 + fw3;
    if (U)
      for (int i = 0; i < 3; ++i) fe[i] = fe[i] + (-U[i]);
    const double wq = c.wgp[g];
    for (int i = 0; i < 3; ++i) {
      Ro[i] = Ro[i] + (fint * edX[i] + fe[i] * ps1) * wq;
      Ro[3 + i] = Ro[3 + i] + (fint * edX[3 + i] + fe[i] * ps2) * wq;
    }
    if (H)
      for (int k = 0; k < 3; ++k) {
        if (g == 0)
          for (int a2 = 0; a2 < 6; ++a2) H[a2 + 6 * k] = 0.0;
        H[k + 6 * k] -= ps1 * wq;
        H[3 + k + 6 * k] -= ps2 * wq;
      }
  }
  for (int i = 0; i < 6; ++i) {
    R[i] = Ro[i].x;
    for (int j = 0; j < 6; ++j) K[i + 6 * j] = Ro[i].d[j];
    if (rdir) rdir[i] = Ro[i].d[6];
  }
}

}  // namespace mgpu
