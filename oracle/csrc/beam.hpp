// Oracle (test infrastructure only): EulerBeam3D restated with nested duals.
//
// Follows toolbox/BeamElement.jl:
//   BeamCrossSection / resultants  :6-64
//   shape functions                :74-79
//   constructor                    :122-148
//   residual                       :151-174
//   kinematics                     :177-189
//   corotated                      :193-208
// and the time-derivative packing of src/Taylor.jl:24-65 (motion/motion⁻¹).
//
// The reference obtains the kinematic Jacobians ε∂X₀, κ∂X₀, x∂X₀, vₛₘ∂X₀ by
// re-seeding X₀ (revariate, Taylor.jl:143-166) and composing the result back
// onto the outer derivatives (chainrule/composeJacobian, Taylor.jl:271-323).
// That composition is exact forward-mode differentiation; here the same
// Jacobians are obtained by evaluating the kinematics with an inner Dual whose
// values are the outer-dual X₀, which yields the identical derivatives.
#pragma once
#include "rotations.hpp"

namespace oracle {

struct BeamMat {  // BeamCrossSection field order (BeamElement.jl:6-22)
  double EA, EI2, EI3, GJ, mu, iota1, w, Ca1, Cl1, Cq1, Ca2, Cl2, Cq2, Ca3, Cl3, Cq3;
};

// EulerBeam3D fields (BeamElement.jl:87-103), flattened in declaration order.
struct BeamEle {
  double cm[3];
  double rm[9];
  double zgp[4];
  double znod[2];
  double tgm[3];
  double tge[3];
  double ya[4], yu[4], yv[4], ka[4], ku[4], kv[4];
  double L;
  double dL[4];
  BeamMat mat;
};
static_assert(sizeof(BeamEle) == 69 * sizeof(double), "BeamEle layout");

// Constructor BeamElement.jl:122-148.  Returns 0, or 1 when orient2 is nearly
// parallel to the element (the reference raises an error there).
inline int beam_construct(const double c1[3], const double c2[3], const double orient2_in[3], const BeamMat& mat,
                          BeamEle& o) {
  for (int i = 0; i < 3; ++i) o.cm[i] = (c1[i] + c2[i]) / 2.0;
  for (int i = 0; i < 3; ++i) o.tgm[i] = c2[i] - c1[i];
  double L = std::sqrt(o.tgm[0] * o.tgm[0] + o.tgm[1] * o.tgm[1] + o.tgm[2] * o.tgm[2]);
  double t[3] = {o.tgm[0] / L, o.tgm[1] / L, o.tgm[2] / L};
  double o2[3] = {orient2_in[0], orient2_in[1], orient2_in[2]};
  double no2 = std::sqrt(o2[0] * o2[0] + o2[1] * o2[1] + o2[2] * o2[2]);
  for (int i = 0; i < 3; ++i) o2[i] /= no2;
  double dt = o2[0] * t[0] + o2[1] * t[1] + o2[2] * t[2];
  double n[3] = {o2[0] - t[0] * dt, o2[1] - t[1] * dt, o2[2] - t[2] * dt};
  double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  if (!(nn > 1e-3)) return 1;
  for (int i = 0; i < 3; ++i) n[i] /= nn;
  double b[3] = {t[1] * n[2] - t[2] * n[1], t[2] * n[0] - t[0] * n[2], t[0] * n[1] - t[1] * n[0]};
  for (int i = 0; i < 3; ++i) {
    o.rm[i] = t[i];
    o.rm[3 + i] = n[i];
    o.rm[6 + i] = b[i];
  }
  o.tge[0] = L; o.tge[1] = 0.0; o.tge[2] = 0.0;
  double s30 = std::sqrt(30.0);
  o.dL[0] = L / 2 * (18 - s30) / 36;
  o.dL[1] = L / 2 * (18 + s30) / 36;
  o.dL[2] = L / 2 * (18 + s30) / 36;
  o.dL[3] = L / 2 * (18 - s30) / 36;
  double s65 = std::sqrt(6.0 / 5.0);
  o.zgp[0] = -1.0 / 2 * std::sqrt(3.0 / 7 + 2.0 / 7 * s65);
  o.zgp[1] = -1.0 / 2 * std::sqrt(3.0 / 7 - 2.0 / 7 * s65);
  o.zgp[2] = +1.0 / 2 * std::sqrt(3.0 / 7 - 2.0 / 7 * s65);
  o.zgp[3] = +1.0 / 2 * std::sqrt(3.0 / 7 + 2.0 / 7 * s65);
  o.znod[0] = -0.5; o.znod[1] = 0.5;
  for (int g = 0; g < 4; ++g) {
    double z = o.zgp[g];
    o.ya[g] = 2 * z;
    o.yu[g] = -4 * (z * z * z) + 3 * z;
    o.yv[g] = (z * z - 1.0 / 4) * L;
    o.ka[g] = 2.0 / L;
    o.ku[g] = (-24 * z) / (L * L);
    o.kv[g] = 2.0 / L;
  }
  o.L = L;
  o.mat = mat;
  return 0;
}

// corotated{Mode}  BeamElement.jl:193-208
template <class S>
inline void corotated(const BeamEle& o, const S* X0, V3<S>& vsm, M3<S>& rsm, V3<S>& ul2, V3<S>& vl2, V3<S>& csm) {
  V3<S> u1, v1, u2, v2;
  for (int i = 0; i < 3; ++i) {
    u1.v[i] = X0[i];
    v1.v[i] = X0[3 + i];
    u2.v[i] = X0[6 + i];
    v2.v[i] = X0[9 + i];
  }
  M3<S> rs1 = Rodrigues(v1);
  M3<S> rs2 = Rodrigues(v2);
  V3<S> w = Rodriguesinv(mul(rs2, transpose(rs1)));
  V3<S> dv;
  for (int i = 0; i < 3; ++i) dv.v[i] = 0.5 * w.v[i];
  rsm = mulc(mul(Rodrigues(dv), rs1), o.rm);
  vsm = Rodriguesinv(rsm);
  V3<S> cs, a;
  for (int i = 0; i < 3; ++i) cs.v[i] = 0.5 * (u1.v[i] + u2.v[i]);
  for (int i = 0; i < 3; ++i) a.v[i] = u2.v[i] + o.tgm[i] * o.znod[1] - cs.v[i];
  ul2 = mulTv(rsm, a);
  for (int i = 0; i < 3; ++i) ul2.v[i] = ul2.v[i] - o.tge[i] * o.znod[1];
  vl2 = mulTv(rsm, dv);
  for (int i = 0; i < 3; ++i) csm.v[i] = cs.v[i] + o.cm[i];
}

// kinematics{Mode}  BeamElement.jl:177-189
template <class S>
struct BeamKin {
  V3<S> kappa[4], x[4];
  S eps;
  V3<S> vsm;
  M3<S> rsm;
  V3<S> vl2, ul2, csm;
};
template <class S>
inline void kinematics(const BeamEle& o, const S* X0, BeamKin<S>& k) {
  corotated(o, X0, k.vsm, k.rsm, k.ul2, k.vl2, k.csm);
  const double L = o.L;
  k.eps = sqrt(sq(k.ul2.v[0] + L / 2) + sq(k.ul2.v[1]) + sq(k.ul2.v[2])) * 2.0 / L - 1.0;
  for (int g = 0; g < 4; ++g) {
    double ya = o.ya[g], yu = o.yu[g], yv = o.yv[g], ka = o.ka[g], ku = o.ku[g], kv = o.kv[g];
    k.kappa[g].v[0] = ka * k.vl2.v[0];
    k.kappa[g].v[1] = ku * k.ul2.v[1] + kv * k.vl2.v[2];
    k.kappa[g].v[2] = ku * k.ul2.v[2] - kv * k.vl2.v[1];
    V3<S> y;
    y.v[0] = ya * k.ul2.v[0];
    y.v[1] = yu * k.ul2.v[1] + yv * k.vl2.v[2];
    y.v[2] = yu * k.ul2.v[2] - yv * k.vl2.v[1];
    V3<S> p;
    for (int i = 0; i < 3; ++i) p.v[i] = o.tge[i] * o.zgp[g] + y.v[i];
    V3<S> xr = mulv(k.rsm, p);
    for (int i = 0; i < 3; ++i) k.x[g].v[i] = xr.v[i] + k.csm.v[i];
  }
}

// ---- motion / motion⁻¹ (Taylor.jl:24-65) --------------------------------------
// ND=1: the jet is the outer type itself; ND=2: Dual<O,1>; ND=3: Dual<Dual<O,1>,1>.
template <class O, int ND> struct Jet;
template <class O> struct Jet<O, 1> {
  using T = O;
  static T make(const O* a) { return a[0]; }
  static O d0(const T& a) { return a; }
  static O d1(const T&) { return O(0.0); }
  static O d2(const T&) { return O(0.0); }
};
template <class O> struct Jet<O, 2> {
  using T = Dual<O, 1>;
  static T make(const O* a) {
    T r(a[0], 0);
    r.dx[0] = a[1];
    return r;
  }
  static O d0(const T& a) { return a.x; }
  static O d1(const T& a) { return a.dx[0]; }
  static O d2(const T&) { return O(0.0); }
};
template <class O> struct Jet<O, 3> {
  using T = Dual<Dual<O, 1>, 1>;
  static T make(const O* a) {
    Dual<O, 1> inner(a[0], 0);
    inner.dx[0] = a[1];
    Dual<O, 1> inner2(a[1], 0);
    inner2.dx[0] = a[2];
    T r(inner, 0);
    r.dx[0] = inner2;
    return r;
  }
  static O d0(const T& a) { return a.x.x; }
  static O d1(const T& a) { return a.x.dx[0]; }
  static O d2(const T& a) { return a.dx[0].dx[0]; }
};

// resultants  BeamElement.jl:28-64
template <class O>
inline void beam_resultants(const BeamMat& m, const O& eps, const V3<O>& kappa, const V3<O> x[3], const M3<O> r[3],
                            const V3<O>& vi2, O fi_out[1], V3<O>& mi, V3<O>& fe, V3<O>& me) {
  const M3<O>& r0 = r[0];
  V3<O> xl1 = mulTv(r0, x[1]);  // xᵧ₁ ∘₁ r₀
  V3<O> xl2 = mulTv(r0, x[2]);
  V3<O> fi;
  for (int i = 0; i < 3; ++i) fi.v[i] = m.mu * x[2].v[i];
  V3<O> fal;
  fal.v[0] = m.Ca1 * xl2.v[0];
  fal.v[1] = m.Ca2 * xl2.v[1];
  fal.v[2] = m.Ca3 * xl2.v[2];
  V3<O> fag = mulv(r0, fal);
  V3<O> fll;
  fll.v[0] = m.Cl1 * xl1.v[0];
  fll.v[1] = m.Cl2 * xl1.v[1];
  fll.v[2] = m.Cl3 * xl1.v[2];
  V3<O> flg = mulv(r0, fll);
  O fq1 = m.Cq1 * sq(xl1.v[0]);
  if (xl1.v[0] < 0.0) fq1 = -fq1;
  O fq2 = m.Cq2 * sq(xl1.v[1]);
  if (xl1.v[1] < 0.0) fq2 = -fq2;
  O fq3 = m.Cq3 * sq(xl1.v[2]);
  if (xl1.v[2] < 0.0) fq3 = -fq3;
  V3<O> fql;
  fql.v[0] = fq1; fql.v[1] = fq2; fql.v[2] = fq3;
  V3<O> fqg = mulv(r0, fql);
  for (int i = 0; i < 3; ++i) fe.v[i] = fi.v[i] + fag.v[i] + flg.v[i] + fqg.v[i];
  fe.v[2] = fe.v[2] + m.w;
  O m1l = m.iota1 * vi2.v[0];
  for (int i = 0; i < 3; ++i) me.v[i] = r0.m[i] * m1l;  // ∂0(rₛₘ)[:,1] * m₁ₗ
  fi_out[0] = m.EA * eps;
  mi.v[0] = m.GJ * kappa.v[0];
  mi.v[1] = m.EI3 * kappa.v[1];
  mi.v[2] = m.EI2 * kappa.v[2];
}

// residual  BeamElement.jl:151-174.  X: ND jets of 12 outer values; U: 3 values
// (per unit length, only used when udof).  Output R[12] in the outer type.
template <class O, int ND>
inline void beam_residual(const BeamEle& o, const O (*X)[12], const O* U, bool udof, O* R) {
  using J = Jet<O, ND>;
  using JT = typename J::T;
  // --- direct kinematics on the time jets
  JT Xm[12];
  for (int i = 0; i < 12; ++i) {
    O a[3];
    for (int d = 0; d < ND; ++d) a[d] = X[d][i];
    Xm[i] = J::make(a);
  }
  BeamKin<JT> kd;
  kinematics(o, Xm, kd);
  // motion⁻¹ of gp quantities, ε and rₛₘ
  V3<O> gx[4][3], gk[4];
  for (int g = 0; g < 4; ++g)
    for (int i = 0; i < 3; ++i) {
      gx[g][0].v[i] = J::d0(kd.x[g].v[i]);
      gx[g][1].v[i] = J::d1(kd.x[g].v[i]);
      gx[g][2].v[i] = J::d2(kd.x[g].v[i]);
      gk[g].v[i] = J::d0(kd.kappa[g].v[i]);
    }
  O eps = J::d0(kd.eps);
  M3<O> r[3];
  for (int k = 0; k < 9; ++k) {
    r[0].m[k] = J::d0(kd.rsm.m[k]);
    r[1].m[k] = J::d1(kd.rsm.m[k]);
    r[2].m[k] = J::d2(kd.rsm.m[k]);
  }
  // intrinsicrotationrates  Rotations.jl:177-182 (only the acceleration is used)
  V3<O> vi2;
  if (ND < 3) {
    for (int i = 0; i < 3; ++i) vi2.v[i] = O(0.0);
  } else {
    M3<O> a = mul(transpose(r[1]), r[1]);
    M3<O> b = mul(transpose(r[0]), r[2]);
    M3<O> c;
    for (int k = 0; k < 9; ++k) c.m[k] = a.m[k] + b.m[k];
    vi2 = spininv(c);
  }
  // --- Jacobians wrt X₀ through an inner dual seeded at the outer X₀
  using T = Dual<O, 12>;
  T TX0[12];
  for (int i = 0; i < 12; ++i) {
    TX0[i] = T(X[0][i], 0);
    TX0[i].dx[i] = O(1.0);
  }
  BeamKin<T> kt;
  kinematics(o, TX0, kt);
  // --- quadrature
  for (int j = 0; j < 12; ++j) R[j] = O(0.0);
  for (int g = 0; g < 4; ++g) {
    O fi[1];
    V3<O> mi, fe, me;
    beam_resultants(o.mat, eps, gk[g], gx[g], r, vi2, fi, mi, fe, me);
    if (udof)
      for (int i = 0; i < 3; ++i) fe.v[i] = fe.v[i] - U[i];
    for (int j = 0; j < 12; ++j) {
      O s = fi[0] * kt.eps.dx[j];
      for (int i = 0; i < 3; ++i) {
        s = s + mi.v[i] * kt.kappa[g].v[i].dx[j];
        s = s + fe.v[i] * kt.x[g].v[i].dx[j];
        s = s + me.v[i] * kt.vsm.v[i].dx[j];
      }
      R[j] = R[j] + s * o.dL[g];
    }
  }
}

}  // namespace oracle
