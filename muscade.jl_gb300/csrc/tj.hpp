// Truncated multivariate Taylor arithmetic over the nodal rotation dofs of a
// beam element, with an optional second-order time jet.
//
// A value y over N variables carries the coefficients of the monomials
//     1, ε_j, ε_i ε_j                       (static part: 1 + N + N(N+1)/2)
//     τ, τ², τ ε_j, τ² ε_j                  (time jet, only when DYN)
// where ε are perturbations of rotation dofs and τ is time:
//     y(τ, ε) = v + g·ε + ½ εᵀHε + vt τ + vtt τ² + (gt·ε) τ + (gtt·ε) τ²
// truncated to that monomial set.  The set is closed under products (its
// complement is a monomial ideal), so products and compositions computed here
// are exact for every retained coefficient.  `h` stores the Hessian H packed
// (i ≤ j), so that the coefficient of ε_iε_j (i<j) is h_ij and of ε_i² is ½h_ii.
//
// The element's rotation core works on all six rotation dofs X₀[3:5], X₀[9:11]
// (N = 6).  A nodal rotation Rod(vₐ) depends on the three dofs of one node only;
// it is evaluated over those three (N = 3) and enters the six-variable values
// through the block products tj_cross (node 1 × node 2) and tj_mixA (six
// variables × node 1), which skip the coefficients that are zero by structure.
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

// packed index of (i,j), i<=j, over N variables
template <int N = NV>
MG_HD constexpr int hidx(int i, int j) {
  return i * N - (i * (i - 1)) / 2 + (j - i);
}

struct NoJet {};
template <int N>
struct TimeJet {
  real vt, vtt;
  real gt[N], gtt[N];
};

template <bool DYN, int N = NV>
struct TJ : public std::conditional<DYN, TimeJet<N>, NoJet>::type {
  static constexpr int nh = N * (N + 1) / 2;
  real v;
  real g[N];
  real h[N * (N + 1) / 2];
};

template <bool DYN, int N = NV>
MG_HD TJ<DYN, N> tj_const(real c) {
  TJ<DYN, N> r;
  r.v = c;
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = 0.0;
#pragma unroll
  for (int i = 0; i < TJ<DYN, N>::nh; ++i) r.h[i] = 0.0;
  if constexpr (DYN) {
    r.vt = 0.0;
    r.vtt = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      r.gt[i] = 0.0;
      r.gtt[i] = 0.0;
    }
  }
  return r;
}

// independent variable ε_j with value x₀, rate x₁ and acceleration x₂
template <bool DYN, int N = NV>
MG_HD TJ<DYN, N> tj_var(real x0, int j, real x1 = 0.0, real x2 = 0.0) {
  TJ<DYN, N> r = tj_const<DYN, N>(x0);
  r.g[j] = 1.0;
  if constexpr (DYN) {
    r.vt = x1;
    r.vtt = 0.5 * x2;
  }
  return r;
}

template <bool DYN, int N>
MG_HD TJ<DYN, N> operator+(const TJ<DYN, N>& a, const TJ<DYN, N>& b) {
  TJ<DYN, N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = a.g[i] + b.g[i];
#pragma unroll
  for (int i = 0; i < TJ<DYN, N>::nh; ++i) r.h[i] = a.h[i] + b.h[i];
  if constexpr (DYN) {
    r.vt = a.vt + b.vt;
    r.vtt = a.vtt + b.vtt;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      r.gt[i] = a.gt[i] + b.gt[i];
      r.gtt[i] = a.gtt[i] + b.gtt[i];
    }
  }
  return r;
}
template <bool DYN, int N>
MG_HD TJ<DYN, N> operator-(const TJ<DYN, N>& a, const TJ<DYN, N>& b) {
  TJ<DYN, N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = a.g[i] - b.g[i];
#pragma unroll
  for (int i = 0; i < TJ<DYN, N>::nh; ++i) r.h[i] = a.h[i] - b.h[i];
  if constexpr (DYN) {
    r.vt = a.vt - b.vt;
    r.vtt = a.vtt - b.vtt;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      r.gt[i] = a.gt[i] - b.gt[i];
      r.gtt[i] = a.gtt[i] - b.gtt[i];
    }
  }
  return r;
}
template <bool DYN, int N>
MG_HD TJ<DYN, N> tj_scale(const TJ<DYN, N>& a, real s) {
  TJ<DYN, N> r;
  r.v = a.v * s;
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = a.g[i] * s;
#pragma unroll
  for (int i = 0; i < TJ<DYN, N>::nh; ++i) r.h[i] = a.h[i] * s;
  if constexpr (DYN) {
    r.vt = a.vt * s;
    r.vtt = a.vtt * s;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      r.gt[i] = a.gt[i] * s;
      r.gtt[i] = a.gtt[i] * s;
    }
  }
  return r;
}
template <bool DYN, int N>
MG_HD TJ<DYN, N> operator-(const TJ<DYN, N>& a) {
  return tj_scale(a, -1.0);
}
template <bool DYN, int N>
MG_HD TJ<DYN, N> operator*(const TJ<DYN, N>& a, real s) {
  return tj_scale(a, s);
}
template <bool DYN, int N>
MG_HD TJ<DYN, N> operator*(real s, const TJ<DYN, N>& a) {
  return tj_scale(a, s);
}
template <bool DYN, int N>
MG_HD TJ<DYN, N> operator+(const TJ<DYN, N>& a, real s) {
  TJ<DYN, N> r = a;
  r.v += s;
  return r;
}

// product, truncated to the retained monomials
template <bool DYN, int N>
MG_HD TJ<DYN, N> operator*(const TJ<DYN, N>& a, const TJ<DYN, N>& b) {
  TJ<DYN, N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = fma(a.g[i], b.v, a.v * b.g[i]);
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i; j < N; ++j) {
      const int k = hidx<N>(i, j);
      real s = fma(a.h[k], b.v, a.v * b.h[k]);
      s = fma(a.g[i], b.g[j], s);
      r.h[k] = fma(a.g[j], b.g[i], s);
    }
  if constexpr (DYN) {
    r.vt = fma(a.vt, b.v, a.v * b.vt);
    r.vtt = fma(a.vtt, b.v, fma(a.vt, b.vt, a.v * b.vtt));
#pragma unroll
    for (int i = 0; i < N; ++i) {
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
// same flops as a product and a sum, 2·(1 + N + N(N+1)/2 [+ ...]) fewer
// instructions)
template <bool DYN, int N>
MG_HD TJ<DYN, N> tj_fma(const TJ<DYN, N>& a, const TJ<DYN, N>& b, const TJ<DYN, N>& c) {
  TJ<DYN, N> r;
  r.v = fma(a.v, b.v, c.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = fma(a.g[i], b.v, fma(a.v, b.g[i], c.g[i]));
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i; j < N; ++j) {
      const int k = hidx<N>(i, j);
      real s = fma(a.v, b.h[k], c.h[k]);
      s = fma(a.h[k], b.v, s);
      s = fma(a.g[i], b.g[j], s);
      r.h[k] = fma(a.g[j], b.g[i], s);
    }
  if constexpr (DYN) {
    r.vt = fma(a.vt, b.v, fma(a.v, b.vt, c.vt));
    r.vtt = fma(a.vtt, b.v, fma(a.vt, b.vt, fma(a.v, b.vtt, c.vtt)));
#pragma unroll
    for (int i = 0; i < N; ++i) {
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
template <bool DYN, int N>
MG_HD TJ<DYN, N> tj_fnma(const TJ<DYN, N>& a, const TJ<DYN, N>& b, const TJ<DYN, N>& c) {
  TJ<DYN, N> r;
  r.v = fma(-a.v, b.v, c.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = fma(-a.g[i], b.v, fma(-a.v, b.g[i], c.g[i]));
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i; j < N; ++j) {
      const int k = hidx<N>(i, j);
      real s = fma(-a.v, b.h[k], c.h[k]);
      s = fma(-a.h[k], b.v, s);
      s = fma(-a.g[i], b.g[j], s);
      r.h[k] = fma(-a.g[j], b.g[i], s);
    }
  if constexpr (DYN) {
    r.vt = fma(-a.vt, b.v, fma(-a.v, b.vt, c.vt));
    r.vtt = fma(-a.vtt, b.v, fma(-a.vt, b.vt, fma(-a.v, b.vtt, c.vtt)));
#pragma unroll
    for (int i = 0; i < N; ++i) {
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
template <bool DYN, int N>
MG_HD TJ<DYN, N> tj_fma(const TJ<DYN, N>& a, real s, const TJ<DYN, N>& c) {
  TJ<DYN, N> r;
  r.v = fma(a.v, s, c.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = fma(a.g[i], s, c.g[i]);
#pragma unroll
  for (int i = 0; i < TJ<DYN, N>::nh; ++i) r.h[i] = fma(a.h[i], s, c.h[i]);
  if constexpr (DYN) {
    r.vt = fma(a.vt, s, c.vt);
    r.vtt = fma(a.vtt, s, c.vtt);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      r.gt[i] = fma(a.gt[i], s, c.gt[i]);
      r.gtt[i] = fma(a.gtt[i], s, c.gtt[i]);
    }
  }
  return r;
}

// Σ a[i] b[i] (Taylor · Taylor) and Σ a[i] x[i] (Taylor · real), three terms
template <bool DYN, int N>
MG_HD TJ<DYN, N> tj_dot3(const TJ<DYN, N> a[3], const TJ<DYN, N> b[3]) {
  return tj_fma(a[2], b[2], tj_fma(a[1], b[1], a[0] * b[0]));
}
template <bool DYN, int N>
MG_HD TJ<DYN, N> tj_dot3(const TJ<DYN, N> a[3], const real x[3]) {
  return tj_fma(a[2], x[2], tj_fma(a[1], x[1], a[0] * x[0]));
}

// Σ a[i] y_i with y_i(τ) = y0_i + y1_i τ + y2_i τ² independent of ε (a time jet
// without gradient): the products skip y's zero gradient and Hessian
template <bool DYN>
MG_HD TJ<DYN> tj_dot3_time(const TJ<DYN> a[3], const real y0[3], const real y1[3], const real y2[3]) {
  TJ<DYN> r = tj_dot3(a, y0);
  if constexpr (DYN) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      r.vtt = fma(a[k].vt, y1[k], fma(a[k].v, y2[k], r.vtt));
      r.vt = fma(a[k].v, y1[k], r.vt);
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        r.gtt[i] = fma(a[k].gt[i], y1[k], fma(a[k].g[i], y2[k], r.gtt[i]));
        r.gt[i] = fma(a[k].g[i], y1[k], r.gt[i]);
      }
    }
  }
  return r;
}

// ---- block products of the two-node structure (six variables = node 1's
// three, then node 2's three).  ACC: accumulate into c, else c is not read.
template <bool ACC>
MG_HD real tj_mac(real c, real a, real b) {
  if constexpr (ACC)
    return fma(a, b, c);
  else
    return a * b;
}

// x·y (+ c) with x over node 1's variables and y over node 2's: the
// within-node Hessian blocks are x.h·y.v and x.v·y.h, the cross block x.g ⊗ y.g
template <bool ACC, bool DYN>
MG_HD TJ<DYN> tj_cross(const TJ<DYN, 3>& x, const TJ<DYN, 3>& y, const TJ<DYN>& c) {
  TJ<DYN> r;
  r.v = tj_mac<ACC>(c.v, x.v, y.v);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    r.g[i] = tj_mac<ACC>(c.g[i], x.g[i], y.v);
    r.g[3 + i] = tj_mac<ACC>(c.g[3 + i], x.v, y.g[i]);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      r.h[hidx(i, j)] = tj_mac<ACC>(c.h[hidx(i, j)], x.h[hidx<3>(i, j)], y.v);
      r.h[hidx(3 + i, 3 + j)] = tj_mac<ACC>(c.h[hidx(3 + i, 3 + j)], x.v, y.h[hidx<3>(i, j)]);
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.h[hidx(i, 3 + j)] = tj_mac<ACC>(c.h[hidx(i, 3 + j)], x.g[i], y.g[j]);
  if constexpr (DYN) {
    r.vt = fma(x.vt, y.v, tj_mac<ACC>(c.vt, x.v, y.vt));
    r.vtt = fma(x.vtt, y.v, fma(x.vt, y.vt, tj_mac<ACC>(c.vtt, x.v, y.vtt)));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      r.gt[i] = fma(x.gt[i], y.v, tj_mac<ACC>(c.gt[i], x.g[i], y.vt));
      r.gt[3 + i] = fma(x.vt, y.g[i], tj_mac<ACC>(c.gt[3 + i], x.v, y.gt[i]));
      r.gtt[i] = fma(x.gtt[i], y.v, fma(x.gt[i], y.vt, tj_mac<ACC>(c.gtt[i], x.g[i], y.vtt)));
      r.gtt[3 + i] = fma(x.vtt, y.g[i], fma(x.vt, y.gt[i], tj_mac<ACC>(c.gtt[3 + i], x.v, y.gtt[i])));
    }
  }
  return r;
}

// a·b (+ c) with a over the six variables and b over node 1's three
template <bool ACC, bool DYN>
MG_HD TJ<DYN> tj_mixA(const TJ<DYN>& a, const TJ<DYN, 3>& b, const TJ<DYN>& c) {
  TJ<DYN> r;
  r.v = tj_mac<ACC>(c.v, a.v, b.v);
#pragma unroll
  for (int p = 0; p < NV; ++p) {
    real s = tj_mac<ACC>(c.g[p], a.g[p], b.v);
    if (p < 3) s = fma(a.v, b.g[p], s);
    r.g[p] = s;
  }
#pragma unroll
  for (int p = 0; p < NV; ++p)
#pragma unroll
    for (int q = p; q < NV; ++q) {
      const int k = hidx(p, q);
      real s = tj_mac<ACC>(c.h[k], a.h[k], b.v);
      if (q < 3) s = fma(a.v, b.h[hidx<3>(p, q)], s);
      if (q < 3) s = fma(a.g[p], b.g[q], s);
      if (p < 3) s = fma(a.g[q], b.g[p], s);
      r.h[k] = s;
    }
  if constexpr (DYN) {
    r.vt = fma(a.vt, b.v, tj_mac<ACC>(c.vt, a.v, b.vt));
    r.vtt = fma(a.vtt, b.v, fma(a.vt, b.vt, tj_mac<ACC>(c.vtt, a.v, b.vtt)));
#pragma unroll
    for (int p = 0; p < NV; ++p) {
      real s = tj_mac<ACC>(c.gt[p], a.gt[p], b.v);
      s = fma(a.g[p], b.vt, s);
      if (p < 3) {
        s = fma(a.vt, b.g[p], s);
        s = fma(a.v, b.gt[p], s);
      }
      r.gt[p] = s;
      real u = tj_mac<ACC>(c.gtt[p], a.gtt[p], b.v);
      u = fma(a.gt[p], b.vt, u);
      u = fma(a.g[p], b.vtt, u);
      if (p < 3) {
        u = fma(a.vtt, b.g[p], u);
        u = fma(a.vt, b.gt[p], u);
        u = fma(a.v, b.gtt[p], u);
      }
      r.gtt[p] = u;
    }
  }
  return r;
}

// composition f(a) from f and its first three derivatives at a.v
template <bool DYN, int N>
MG_HD TJ<DYN, N> tj_apply(const TJ<DYN, N>& a, real f0, real f1, real f2, real f3) {
  TJ<DYN, N> r;
  r.v = f0;
#pragma unroll
  for (int i = 0; i < N; ++i) r.g[i] = f1 * a.g[i];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i; j < N; ++j) {
      const int k = hidx<N>(i, j);
      r.h[k] = fma(f1, a.h[k], f2 * a.g[i] * a.g[j]);
    }
  if constexpr (DYN) {
    r.vt = f1 * a.vt;
    r.vtt = fma(f1, a.vtt, 0.5 * f2 * a.vt * a.vt);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      r.gt[i] = fma(f1, a.gt[i], f2 * a.g[i] * a.vt);
      real s = f2 * a.g[i] * a.vtt;
      s = fma(f1, a.gtt[i], s);
      s = fma(0.5 * f3 * a.g[i], a.vt * a.vt, s);
      r.gtt[i] = fma(f2 * a.vt, a.gt[i], s);
    }
  }
  return r;
}

}  // namespace mgpu
