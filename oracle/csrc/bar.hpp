// Oracle (test infrastructure only): Bar3D restated with nested duals.
//
// Follows toolbox/BarElement.jl:
//   AxisymmetricBarCrossSection    :36-48
//   shape functions ψ₁, ψ₂         :57-58
//   constructor (ϵₛ = eps())       :118-133
//   resultants                     :136-161
//   residual                       :167-202
#pragma once
#include "beam.hpp"

namespace oracle {

struct BarMat {  // AxisymmetricBarCrossSection field order
  double EA, mu, w, Cat, Clt, Cqt, Can, Cln, Cqn;
};
struct BarEle {  // Bar3D fields in declaration order (BarElement.jl:89-101)
  double cm[3];
  double tgm[3];
  double tge[3];
  double L0;
  double Ls;
  BarMat mat;
  double wgp[4];
  double zgp[4];
  double znod[2];
  double psi1[4];
  double psi2[4];
};
static_assert(sizeof(BarEle) == 38 * sizeof(double), "BarEle layout");

inline void bar_construct(const double c1[3], const double c2[3], const BarMat& mat, double epss, BarEle& o) {
  for (int i = 0; i < 3; ++i) o.cm[i] = (c1[i] + c2[i]) / 2.0;
  for (int i = 0; i < 3; ++i) o.tgm[i] = c2[i] - c1[i];
  o.L0 = std::sqrt(o.tgm[0] * o.tgm[0] + o.tgm[1] * o.tgm[1] + o.tgm[2] * o.tgm[2]);
  o.Ls = (1 - epss) * o.L0;
  o.tge[0] = o.L0; o.tge[1] = 0; o.tge[2] = 0;
  double L0 = o.L0, s30 = std::sqrt(30.0), s65 = std::sqrt(6.0 / 5.0);
  o.wgp[0] = L0 / 2 * (18 - s30) / 36;
  o.wgp[1] = L0 / 2 * (18 + s30) / 36;
  o.wgp[2] = L0 / 2 * (18 + s30) / 36;
  o.wgp[3] = L0 / 2 * (18 - s30) / 36;
  o.zgp[0] = -1.0 / 2 * std::sqrt(3.0 / 7 + 2.0 / 7 * s65);
  o.zgp[1] = -1.0 / 2 * std::sqrt(3.0 / 7 - 2.0 / 7 * s65);
  o.zgp[2] = +1.0 / 2 * std::sqrt(3.0 / 7 - 2.0 / 7 * s65);
  o.zgp[3] = +1.0 / 2 * std::sqrt(3.0 / 7 + 2.0 / 7 * s65);
  o.znod[0] = -0.5; o.znod[1] = 0.5;
  for (int g = 0; g < 4; ++g) {
    o.psi1[g] = -o.zgp[g] + 1.0 / 2;
    o.psi2[g] = o.zgp[g] + 1.0 / 2;
  }
  o.mat = mat;
}

template <class O, int ND>
inline void bar_residual(const BarEle& o, const O (*X)[6], const O* U, bool udof, double t, O* R) {
  using J = Jet<O, ND>;
  using JT = typename J::T;
  JT x_[6];
  for (int i = 0; i < 6; ++i) {
    O a[3];
    for (int d = 0; d < ND; ++d) a[d] = X[d][i];
    x_[i] = J::make(a);
  }
  JT c[3], tg[3];
  for (int i = 0; i < 3; ++i) {
    c[i] = o.cm[i] + 0.5 * (x_[i] + x_[3 + i]);
    tg[i] = o.tgm[i] + x_[3 + i] - x_[i];
  }
  JT L = sqrt(sq(tg[0]) + sq(tg[1]) + sq(tg[2]));
  JT d_[3];
  for (int i = 0; i < 3; ++i) d_[i] = tg[i] / L;
  JT eps_ = L / o.Ls - 1.0;
  O eps = J::d0(eps_);
  V3<O> dlt;  // δ₀
  for (int i = 0; i < 3; ++i) dlt.v[i] = J::d0(d_[i]);
  O edX[6];
  for (int i = 0; i < 3; ++i) {
    edX[i] = (1.0 / o.L0) * (-dlt.v[i]);
    edX[3 + i] = (1.0 / o.L0) * dlt.v[i];
  }
  for (int j = 0; j < 6; ++j) R[j] = O(0.0);
  const BarMat& m = o.mat;
  for (int g = 0; g < 4; ++g) {
    double z = o.zgp[g];
    double p1 = -z + 1.0 / 2, p2 = z + 1.0 / 2;
    V3<O> v, a;  // ∂1(x), ∂2(x) of x = c + tg ζ
    for (int i = 0; i < 3; ++i) {
      JT xg = c[i] + tg[i] * z;
      v.v[i] = J::d1(xg);
      a.v[i] = J::d2(xg);
    }
    // resultants BarElement.jl:136-161
    V3<O> fi;
    for (int i = 0; i < 3; ++i) fi.v[i] = m.mu * a.v[i];
    double fw3 = ((t < -5.0 ? t : -5.0) + 10.0) / 5.0 * m.w;
    O at = a.v[0] * dlt.v[0] + a.v[1] * dlt.v[1] + a.v[2] * dlt.v[2];
    V3<O> an;
    for (int i = 0; i < 3; ++i) an.v[i] = a.v[i] - at * dlt.v[i];
    V3<O> fa;
    fa.v[0] = m.Cat * at;
    fa.v[1] = m.Can * an.v[1];
    fa.v[2] = m.Can * an.v[2];
    O vt = v.v[0] * dlt.v[0] + v.v[1] * dlt.v[1] + v.v[2] * dlt.v[2];
    V3<O> vn;
    for (int i = 0; i < 3; ++i) vn.v[i] = v.v[i] - vt * dlt.v[i];
    O fqt = m.Cqt * sq(vt);
    if (vt < 0.0) fqt = -fqt;
    O fqn2 = m.Cqn * sq(vn.v[1]);
    if (vn.v[1] < 0.0) fqn2 = -fqn2;
    O fqn3 = m.Cqn * sq(vn.v[2]);
    if (vn.v[2] < 0.0) fqn3 = -fqn3;
    V3<O> fd;
    fd.v[0] = m.Clt * vt + fqt;
    fd.v[1] = m.Cln * vn.v[1] + fqn2;
    fd.v[2] = m.Cln * vn.v[2] + fqn3;
    V3<O> fe;
    for (int i = 0; i < 3; ++i) fe.v[i] = fi.v[i] + fa.v[i] + fd.v[i];
    fe.v[2] = fe.v[2] + fw3;
    O fint = m.EA * eps;
    if (udof)
      for (int i = 0; i < 3; ++i) fe.v[i] = fe.v[i] - U[i];
    // x∂X₀ = [ψ₁ I, ψ₂ I]
    for (int i = 0; i < 3; ++i) {
      R[i] = R[i] + (fint * edX[i] + fe.v[i] * p1) * o.wgp[g];
      R[3 + i] = R[3 + i] + (fint * edX[3 + i] + fe.v[i] * p2) * o.wgp[g];
    }
  }
}

}  // namespace oracle
