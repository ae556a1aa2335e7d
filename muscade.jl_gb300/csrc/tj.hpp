// Truncated multivariate Taylor arithmetic over the 6 nodal rotation dofs of a
// beam element, with an optional second-order time jet.
//
// A value y carries the coefficients of the monomials
//     1, ε_j, ε_i ε_j                       (static part, "T2": 1+6+21)
//     τ, τ², τ ε_j, τ² ε_j                  (time jet, only when DYN)
// where ε are perturbations of the rotation dofs X₀[3:5], X₀[9:11] and τ is
// time:  y(τ, ε) = v + g·ε + ½ εᵀHε + vt τ + vtt τ² + (gt·ε) τ + (gtt·ε) τ²
// truncated to that monomial set.  The set is closed under products (its
// complement is a monomial ideal), so products and compositions computed here
// are exact for every retained coefficient.  `h` stores the Hessian H packed
// (i ≤ j), so that the coefficient of ε_iε_j (i<j) is h_ij and of ε_i² is ½h_ii.
//
// This carries exactly the derivative information the reference's nested
// duals carry on this path (Newton variation × time derivatives × the
// revariated Jacobian, src/Taylor.jl and src/Adiff.jl), restricted to the six
// variables the rotation maps depend on.
#pragma once
#include <math.h>
#include <type_traits>

// Arithmetic type of the element math: real on the device; a counting type
// when the host flop-count tool instantiates the same code.
#ifndef MGPU_REAL
#define MGPU_REAL double
#endif

#ifdef __CUDACC__
#define MG_HD __host__ __device__ __forceinline__
#else
#define MG_HD inline
#endif

namespace mgpu {

using real = MGPU_REAL;
#ifndef MGPU_HAVE_TO_D
MG_HD double to_d(double x) { return x; }
#endif

constexpr int NV = 6;
constexpr int NH = 21;

// packed index of (i,j), i<=j
MG_HD constexpr int hidx(int i, int j) { return i * NV - (i * (i - 1)) / 2 + (j - i); }

struct NoJet {};
struct TimeJet {
  real vt, vtt;
  real gt[NV], gtt[NV];
};

template <bool DYN>
struct TJ : public std::conditional<DYN, TimeJet, NoJet>::type {
  real v;
  real g[NV];
  real h[NH];
};

template <bool DYN>
MG_HD TJ<DYN> tj_const(real c) {
  TJ<DYN> r;
  r.v = c;
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = 0.0;
#pragma unroll
  for (int i = 0; i < NH; ++i) r.h[i] = 0.0;
  if constexpr (DYN) {
    r.vt = 0.0;
    r.vtt = 0.0;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = 0.0;
      r.gtt[i] = 0.0;
    }
  }
  return r;
}

// independent variable ε_j with value x₀, rate x₁ and acceleration x₂
template <bool DYN>
MG_HD TJ<DYN> tj_var(real x0, int j, real x1 = 0.0, real x2 = 0.0) {
  TJ<DYN> r = tj_const<DYN>(x0);
  r.g[j] = 1.0;
  if constexpr (DYN) {
    r.vt = x1;
    r.vtt = 0.5 * x2;
  }
  return r;
}

template <bool DYN>
MG_HD TJ<DYN> operator+(const TJ<DYN>& a, const TJ<DYN>& b) {
  TJ<DYN> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = a.g[i] + b.g[i];
#pragma unroll
  for (int i = 0; i < NH; ++i) r.h[i] = a.h[i] + b.h[i];
  if constexpr (DYN) {
    r.vt = a.vt + b.vt;
    r.vtt = a.vtt + b.vtt;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = a.gt[i] + b.gt[i];
      r.gtt[i] = a.gtt[i] + b.gtt[i];
    }
  }
  return r;
}
template <bool DYN>
MG_HD TJ<DYN> operator-(const TJ<DYN>& a, const TJ<DYN>& b) {
  TJ<DYN> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = a.g[i] - b.g[i];
#pragma unroll
  for (int i = 0; i < NH; ++i) r.h[i] = a.h[i] - b.h[i];
  if constexpr (DYN) {
    r.vt = a.vt - b.vt;
    r.vtt = a.vtt - b.vtt;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = a.gt[i] - b.gt[i];
      r.gtt[i] = a.gtt[i] - b.gtt[i];
    }
  }
  return r;
}
template <bool DYN>
MG_HD TJ<DYN> tj_scale(const TJ<DYN>& a, real s) {
  TJ<DYN> r;
  r.v = a.v * s;
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = a.g[i] * s;
#pragma unroll
  for (int i = 0; i < NH; ++i) r.h[i] = a.h[i] * s;
  if constexpr (DYN) {
    r.vt = a.vt * s;
    r.vtt = a.vtt * s;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = a.gt[i] * s;
      r.gtt[i] = a.gtt[i] * s;
    }
  }
  return r;
}
template <bool DYN>
MG_HD TJ<DYN> operator-(const TJ<DYN>& a) {
  return tj_scale(a, -1.0);
}
template <bool DYN>
MG_HD TJ<DYN> operator*(const TJ<DYN>& a, real s) { return tj_scale(a, s); }
template <bool DYN>
MG_HD TJ<DYN> operator*(real s, const TJ<DYN>& a) { return tj_scale(a, s); }
template <bool DYN>
MG_HD TJ<DYN> operator+(const TJ<DYN>& a, real s) {
  TJ<DYN> r = a;
  r.v += s;
  return r;
}

// product, truncated to the retained monomials
template <bool DYN>
MG_HD TJ<DYN> operator*(const TJ<DYN>& a, const TJ<DYN>& b) {
  TJ<DYN> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = fma(a.g[i], b.v, a.v * b.g[i]);
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = i; j < NV; ++j) {
      const int k = hidx(i, j);
      real s = fma(a.h[k], b.v, a.v * b.h[k]);
      s = fma(a.g[i], b.g[j], s);
      r.h[k] = fma(a.g[j], b.g[i], s);
    }
  if constexpr (DYN) {
    r.vt = fma(a.vt, b.v, a.v * b.vt);
    r.vtt = fma(a.vtt, b.v, fma(a.vt, b.vt, a.v * b.vtt));
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = fma(a.gt[i], b.v, fma(a.vt, b.g[i], fma(a.g[i], b.vt, a.v * b.gt[i])));
      real s = fma(a.gtt[i], b.v, a.vtt * b.g[i]);
      s = fma(a.gt[i], b.vt, s);
      s = fma(a.vt, b.gt[i], s);
      s = fma(a.g[i], b.vtt, s);
      r.gtt[i] = fma(a.v, b.gtt[i], s);
    }
  }
  return r;
}

// a*b + c, truncated: the product's terms accumulated into c with FMAs (the
// same flops as a product and a sum, 2·(1 + 6 + 21 [+ 1 + 6 + ...]) fewer
// instructions)
template <bool DYN>
MG_HD TJ<DYN> tj_fma(const TJ<DYN>& a, const TJ<DYN>& b, const TJ<DYN>& c) {
  TJ<DYN> r;
  r.v = fma(a.v, b.v, c.v);
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = fma(a.g[i], b.v, fma(a.v, b.g[i], c.g[i]));
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = i; j < NV; ++j) {
      const int k = hidx(i, j);
      real s = fma(a.v, b.h[k], c.h[k]);
      s = fma(a.h[k], b.v, s);
      s = fma(a.g[i], b.g[j], s);
      r.h[k] = fma(a.g[j], b.g[i], s);
    }
  if constexpr (DYN) {
    r.vt = fma(a.vt, b.v, fma(a.v, b.vt, c.vt));
    r.vtt = fma(a.vtt, b.v, fma(a.vt, b.vt, fma(a.v, b.vtt, c.vtt)));
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = fma(a.gt[i], b.v, fma(a.vt, b.g[i], fma(a.g[i], b.vt, fma(a.v, b.gt[i], c.gt[i]))));
      real s = fma(a.vtt, b.g[i], c.gtt[i]);
      s = fma(a.gtt[i], b.v, s);
      s = fma(a.gt[i], b.vt, s);
      s = fma(a.vt, b.gt[i], s);
      s = fma(a.g[i], b.vtt, s);
      r.gtt[i] = fma(a.v, b.gtt[i], s);
    }
  }
  return r;
}

// c - a*b, truncated (negated FMA operands, no extra instructions)
template <bool DYN>
MG_HD TJ<DYN> tj_fnma(const TJ<DYN>& a, const TJ<DYN>& b, const TJ<DYN>& c) {
  TJ<DYN> r;
  r.v = fma(-a.v, b.v, c.v);
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = fma(-a.g[i], b.v, fma(-a.v, b.g[i], c.g[i]));
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = i; j < NV; ++j) {
      const int k = hidx(i, j);
      real s = fma(-a.v, b.h[k], c.h[k]);
      s = fma(-a.h[k], b.v, s);
      s = fma(-a.g[i], b.g[j], s);
      r.h[k] = fma(-a.g[j], b.g[i], s);
    }
  if constexpr (DYN) {
    r.vt = fma(-a.vt, b.v, fma(-a.v, b.vt, c.vt));
    r.vtt = fma(-a.vtt, b.v, fma(-a.vt, b.vt, fma(-a.v, b.vtt, c.vtt)));
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = fma(-a.gt[i], b.v, fma(-a.vt, b.g[i], fma(-a.g[i], b.vt, fma(-a.v, b.gt[i], c.gt[i]))));
      real s = fma(-a.vtt, b.g[i], c.gtt[i]);
      s = fma(-a.gtt[i], b.v, s);
      s = fma(-a.gt[i], b.vt, s);
      s = fma(-a.vt, b.gt[i], s);
      s = fma(-a.g[i], b.vtt, s);
      r.gtt[i] = fma(-a.v, b.gtt[i], s);
    }
  }
  return r;
}

// a*s + c with s real
template <bool DYN>
MG_HD TJ<DYN> tj_fma(const TJ<DYN>& a, real s, const TJ<DYN>& c) {
  TJ<DYN> r;
  r.v = fma(a.v, s, c.v);
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = fma(a.g[i], s, c.g[i]);
#pragma unroll
  for (int i = 0; i < NH; ++i) r.h[i] = fma(a.h[i], s, c.h[i]);
  if constexpr (DYN) {
    r.vt = fma(a.vt, s, c.vt);
    r.vtt = fma(a.vtt, s, c.vtt);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = fma(a.gt[i], s, c.gt[i]);
      r.gtt[i] = fma(a.gtt[i], s, c.gtt[i]);
    }
  }
  return r;
}

// Σ a[i] b[i] (Taylor · Taylor) and Σ a[i] x[i] (Taylor · real), three terms
template <bool DYN>
MG_HD TJ<DYN> tj_dot3(const TJ<DYN> a[3], const TJ<DYN> b[3]) {
  return tj_fma(a[2], b[2], tj_fma(a[1], b[1], a[0] * b[0]));
}
template <bool DYN>
MG_HD TJ<DYN> tj_dot3(const TJ<DYN> a[3], const real x[3]) {
  return tj_fma(a[2], x[2], tj_fma(a[1], x[1], a[0] * x[0]));
}

// composition f(a) from f and its first three derivatives at a.v
template <bool DYN>
MG_HD TJ<DYN> tj_apply(const TJ<DYN>& a, real f0, real f1, real f2, real f3) {
  TJ<DYN> r;
  r.v = f0;
#pragma unroll
  for (int i = 0; i < NV; ++i) r.g[i] = f1 * a.g[i];
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = i; j < NV; ++j) {
      const int k = hidx(i, j);
      r.h[k] = fma(f1, a.h[k], f2 * a.g[i] * a.g[j]);
    }
  if constexpr (DYN) {
    r.vt = f1 * a.vt;
    r.vtt = fma(f1, a.vtt, 0.5 * f2 * a.vt * a.vt);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      r.gt[i] = fma(f1, a.gt[i], f2 * a.g[i] * a.vt);
      real s = f2 * a.g[i] * a.vtt;
      s = fma(f1, a.gtt[i], s);
      s = fma(0.5 * f3 * a.g[i], a.vt * a.vt, s);
      r.gtt[i] = fma(f2 * a.vt, a.gt[i], s);
    }
  }
  return r;
}

template <bool DYN>
MG_HD bool tj_is_zero_value(const TJ<DYN>& a) {
  return a.v == 0.0;
}

}  // namespace mgpu
