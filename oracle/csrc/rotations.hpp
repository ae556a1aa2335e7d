// Oracle (test infrastructure only): 3D rotation algebra of the reference,
// restated generically over the scalar type so that the same code evaluates
// values, time jets and nested derivatives.
//
// Follows toolbox/Rotations.jl:
//   sinc1 and its derivatives  :13-51  (custom derivative rules :47-51)
//   scac                        :61-68
//   spin / spin⁻¹ / trace       :81-96
//   Rodrigues⁻¹                 :105
//   norm3 (zeroed below 1e-14)  :106-112
//   spin²                       :114-122
//   Rodrigues                   :131-135
//   intrinsicrotationrates      :177-182
// Matrices are 3x3 column-major (m[i+3*j] = M[i+1,j+1]) like Julia's SMatrix.
#pragma once
#include <cmath>
#include "dual.hpp"

namespace oracle {

// ---------------------------------------------------------------- sinc1 ----
// sinc1(x) = sinc(x/π) with Julia's Base.sinc: below |x/π|<1e-3 a degree-4
// polynomial in x/π, otherwise sinpi(x/π)/(π x/π).
inline double sinpi_(double y) {
  double r = y - 2.0 * std::nearbyint(y * 0.5);  // exact reduction to [-1,1]
  if (r == 0.0 || std::fabs(r) == 1.0) return 0.0;
  return std::sin(M_PI * r);
}
inline double sinc1_0(double x) {
  double y = x / M_PI;
  if (std::fabs(y) < 1e-3) {
    const double p2 = M_PI * M_PI;
    double y2 = y * y;
    return 1.0 + y2 * (-p2 / 6.0 + y2 * (p2 * p2 / 120.0));
  }
  return sinpi_(y) / (M_PI * y);
}
inline double sinc1_1(double x) {  // sinc1′  Rotations.jl:14-22
  if (std::fabs(x) > 1e-3) {
    double s = std::sin(x), c = std::cos(x);
    return c / x - s / (x * x);
  }
  double x2 = x * x;
  return x * (-1.0 / 3.0 + x2 / 30.0);
}
inline double sinc1_2(double x) {  // sinc1″  :23-31
  if (std::fabs(x) > 1e-1) {
    double s = std::sin(x), c = std::cos(x);
    return -s / x - 2.0 * c / (x * x) + 2.0 * s / (x * x * x);
  }
  double x2 = x * x;
  return -1.0 / 3.0 + x2 * (1.0 / 10.0 + x2 * (-1.0 / 168.0 + x2 * (1.0 / 6480.0)));
}
inline double sinc1_3(double x) {  // sinc1‴  :32-40
  if (std::fabs(x) > 0.4) {
    double s = std::sin(x), c = std::cos(x);
    double x2 = x * x;
    return -c / x + 3.0 * s / x2 + 6.0 * c / (x2 * x) - 6.0 * s / (x2 * x2);
  }
  double x2 = x * x;
  return x * (1.0 / 5.0 + x2 * (-1.0 / 42.0 + x2 * (1.0 / 1080.0 + x2 * (-1.0 / 55440.0 + x2 * (1.0 / 4717440.0)))));
}
inline double sinc1_4(double x) {  // sinc1⁗  :41-44
  double x2 = x * x;
  return 1.0 / 5.0 +
         x2 * (-1.0 / 14.0 +
               x2 * (1.0 / 216.0 +
                     x2 * (-1.0 / 7920.0 +
                           x2 * (1.0 / 524160.0 +
                                 x2 * (-1.0 / 54432000.0 +
                                       x2 * (1.0 / 54432000.0 + x2 * (-1.0 / 8143027200.0 + x2 * (1.0 / 1656387532800.0))))))));
}
inline double sinc1_5(double x) { return x * NAN; }  // sinc1⁗′ :45

template <int K> inline double sinc1k(double x);
template <> inline double sinc1k<0>(double x) { return sinc1_0(x); }
template <> inline double sinc1k<1>(double x) { return sinc1_1(x); }
template <> inline double sinc1k<2>(double x) { return sinc1_2(x); }
template <> inline double sinc1k<3>(double x) { return sinc1_3(x); }
template <> inline double sinc1k<4>(double x) { return sinc1_4(x); }
template <> inline double sinc1k<5>(double x) { return sinc1_5(x); }

// derivative rule: d sinc1^(K)(a) = sinc1^(K+1)(a.x) a.dx  (Rotations.jl:47-51)
template <int K, class T, int N>
inline Dual<T, N> sinc1k(const Dual<T, N>& a) {
  return chain(a, sinc1k<K>(a.x), sinc1k<(K < 5 ? K + 1 : 5)>(a.x));
}
template <class S> inline S sinc1(const S& x) { return sinc1k<0>(x); }

// ----------------------------------------------------------------- scac ----
template <class S>
inline S scac(const S& x) {
  S dx = x - 1.0;
  if (std::fabs(VALUE(dx)) > 1e-3) return sinc1(acos(x));
  return 1.0 + dx * (1.0 / 3.0 + dx * (-2.0 / 90.0 + dx * (0.0052911879917544626 +
                                                          dx * (-0.0016229317117234072 + dx * (0.0005625)))));
}

// ---------------------------------------------------------------- 3x3 -------
template <class S> struct V3 { S v[3]; };
template <class S> struct M3 { S m[9]; };  // column-major

template <class S> inline M3<S> spin(const V3<S>& v) {
  M3<S> M;
  M.m[0] = S(0.0); M.m[1] = v.v[2];  M.m[2] = -v.v[1];
  M.m[3] = -v.v[2]; M.m[4] = S(0.0); M.m[5] = v.v[0];
  M.m[6] = v.v[1]; M.m[7] = -v.v[0]; M.m[8] = S(0.0);
  return M;
}
// M[i,j] (1-based) -> m[(i-1)+3(j-1)]
#define MIJ(M, i, j) (M).m[((i)-1) + 3 * ((j)-1)]
template <class S> inline V3<S> spininv(const M3<S>& m) {
  V3<S> r;
  r.v[0] = (MIJ(m, 3, 2) - MIJ(m, 2, 3)) / 2.0;
  r.v[1] = (MIJ(m, 1, 3) - MIJ(m, 3, 1)) / 2.0;
  r.v[2] = (MIJ(m, 2, 1) - MIJ(m, 1, 2)) / 2.0;
  return r;
}
template <class S> inline S trace(const M3<S>& m) { return MIJ(m, 1, 1) + MIJ(m, 2, 2) + MIJ(m, 3, 3); }

template <class S> inline S norm3(const V3<S>& v) {
  S n = sqrt(v.v[0] * v.v[0] + v.v[1] * v.v[1] + v.v[2] * v.v[2]);
  if (VALUE(n) < 1e-14) n = S(0.0);
  return n;
}
template <class S> inline M3<S> spin2(const M3<S>& Sm) {
  S ab = MIJ(Sm, 2, 3) * MIJ(Sm, 3, 1);
  S ca = MIJ(Sm, 1, 2) * MIJ(Sm, 2, 3);
  S bc = MIJ(Sm, 3, 1) * MIJ(Sm, 1, 2);
  S ma2 = MIJ(Sm, 3, 2) * MIJ(Sm, 2, 3);
  S mb2 = MIJ(Sm, 3, 1) * MIJ(Sm, 1, 3);
  S mc2 = MIJ(Sm, 2, 1) * MIJ(Sm, 1, 2);
  M3<S> r;
  r.m[0] = mc2 + mb2; r.m[1] = ab; r.m[2] = ca;
  r.m[3] = ab; r.m[4] = ma2 + mc2; r.m[5] = bc;
  r.m[6] = ca; r.m[7] = bc; r.m[8] = ma2 + mb2;
  return r;
}
template <class S> inline M3<S> Rodrigues(const V3<S>& v) {
  M3<S> Sm = spin(v);
  S th = norm3(v);
  S A = sinc1(th);
  S h = sinc1(th / 2.0);
  S B = h * h / 2.0;
  M3<S> S2 = spin2(Sm);
  M3<S> R;
  for (int k = 0; k < 9; ++k) R.m[k] = A * Sm.m[k] + B * S2.m[k];
  R.m[0] = R.m[0] + 1.0; R.m[4] = R.m[4] + 1.0; R.m[8] = R.m[8] + 1.0;
  return R;
}
template <class S> inline V3<S> Rodriguesinv(const M3<S>& m) {
  V3<S> a = spininv(m);
  S d = scac((trace(m) - 1.0) / 2.0);
  V3<S> r;
  for (int k = 0; k < 3; ++k) r.v[k] = a.v[k] / d;
  return r;
}

// products -------------------------------------------------------------------
template <class S> inline M3<S> mul(const M3<S>& a, const M3<S>& b) {
  M3<S> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      S s = a.m[i] * b.m[3 * j];
      s = s + a.m[i + 3] * b.m[1 + 3 * j];
      s = s + a.m[i + 6] * b.m[2 + 3 * j];
      r.m[i + 3 * j] = s;
    }
  return r;
}
template <class S> inline M3<S> mulc(const M3<S>& a, const double* b) {  // a * constant matrix
  M3<S> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      S s = a.m[i] * b[3 * j];
      s = s + a.m[i + 3] * b[1 + 3 * j];
      s = s + a.m[i + 6] * b[2 + 3 * j];
      r.m[i + 3 * j] = s;
    }
  return r;
}
template <class S> inline M3<S> transpose(const M3<S>& a) {
  M3<S> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[i + 3 * j] = a.m[j + 3 * i];
  return r;
}
template <class S> inline V3<S> mulv(const M3<S>& a, const V3<S>& b) {
  V3<S> r;
  for (int i = 0; i < 3; ++i) r.v[i] = a.m[i] * b.v[0] + a.m[i + 3] * b.v[1] + a.m[i + 6] * b.v[2];
  return r;
}
template <class S> inline V3<S> mulTv(const M3<S>& a, const V3<S>& b) {  // aᵀ b
  V3<S> r;
  for (int i = 0; i < 3; ++i) r.v[i] = a.m[3 * i] * b.v[0] + a.m[3 * i + 1] * b.v[1] + a.m[3 * i + 2] * b.v[2];
  return r;
}

}  // namespace oracle
