// Oracle (test infrastructure only): forward-mode nested dual numbers.
//
// CPU restatement of the differentiation runtime the reference uses on the
// assemble-and-solve path: the nested dual type  ∂ℝ{P,N,R}  of
// src/Adiff.jl:13-16 (value `x`, N partials `dx`, values and partials may
// themselves be duals), its arithmetic rules (src/Adiff.jl:204-304) and the
// VALUE / value / ∂ extractors (src/Adiff.jl:136-195).  Nesting order plays
// the role of the reference's precedence P: the outermost Dual is the newest
// variation.
//
// This file is checked by the oracle tests against the reference's golden
// values; it is never linked into the product library.
#pragma once
#include <cmath>
#include <cstddef>

namespace oracle {

template <class T, int N>
struct Dual {
  T x;
  T dx[N];
  Dual() : x(0.0) {
    for (int i = 0; i < N; ++i) dx[i] = T(0.0);
  }
  Dual(double c) : x(c) {  // constant at any nesting depth
    for (int i = 0; i < N; ++i) dx[i] = T(0.0);
  }
  Dual(const T& v, int) : x(v) {  // value, zero partials (tag int to disambiguate)
    for (int i = 0; i < N; ++i) dx[i] = T(0.0);
  }
};

// VALUE: completely strip partials (src/Adiff.jl:136-139)
inline double VALUE(double a) { return a; }
template <class T, int N>
inline double VALUE(const Dual<T, N>& a) { return VALUE(a.x); }

// ---- arithmetic -----------------------------------------------------------
template <class T, int N>
inline Dual<T, N> operator+(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r(a.x + b.x, 0);
  for (int i = 0; i < N; ++i) r.dx[i] = a.dx[i] + b.dx[i];
  return r;
}
template <class T, int N>
inline Dual<T, N> operator-(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r(a.x - b.x, 0);
  for (int i = 0; i < N; ++i) r.dx[i] = a.dx[i] - b.dx[i];
  return r;
}
template <class T, int N>
inline Dual<T, N> operator-(const Dual<T, N>& a) {
  Dual<T, N> r(-a.x, 0);
  for (int i = 0; i < N; ++i) r.dx[i] = -a.dx[i];
  return r;
}
template <class T, int N>
inline Dual<T, N> operator*(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r(a.x * b.x, 0);
  for (int i = 0; i < N; ++i) r.dx[i] = a.dx[i] * b.x + a.x * b.dx[i];
  return r;
}
template <class T, int N>
inline Dual<T, N> operator/(const Dual<T, N>& a, const Dual<T, N>& b) {
  T inv = T(1.0) / b.x;
  T q = a.x * inv;
  Dual<T, N> r(q, 0);
  for (int i = 0; i < N; ++i) r.dx[i] = (a.dx[i] - q * b.dx[i]) * inv;
  return r;
}
// with plain doubles
template <class T, int N>
inline Dual<T, N> operator+(const Dual<T, N>& a, double b) { Dual<T, N> r = a; r.x = a.x + b; return r; }
template <class T, int N>
inline Dual<T, N> operator+(double b, const Dual<T, N>& a) { return a + b; }
template <class T, int N>
inline Dual<T, N> operator-(const Dual<T, N>& a, double b) { Dual<T, N> r = a; r.x = a.x - b; return r; }
template <class T, int N>
inline Dual<T, N> operator-(double b, const Dual<T, N>& a) { return (-a) + b; }
template <class T, int N>
inline Dual<T, N> operator*(const Dual<T, N>& a, double b) {
  Dual<T, N> r(a.x * b, 0);
  for (int i = 0; i < N; ++i) r.dx[i] = a.dx[i] * b;
  return r;
}
template <class T, int N>
inline Dual<T, N> operator*(double b, const Dual<T, N>& a) { return a * b; }
template <class T, int N>
inline Dual<T, N> operator/(const Dual<T, N>& a, double b) { return a * (1.0 / b); }
template <class T, int N>
inline Dual<T, N> operator/(double a, const Dual<T, N>& b) { return Dual<T, N>(a) / b; }

template <class T, int N>
inline Dual<T, N>& operator+=(Dual<T, N>& a, const Dual<T, N>& b) { a = a + b; return a; }
template <class T, int N>
inline Dual<T, N>& operator-=(Dual<T, N>& a, const Dual<T, N>& b) { a = a - b; return a; }

// comparisons act on VALUE (src/Adiff.jl:198-201)
template <class T, int N> inline bool operator<(const Dual<T, N>& a, double b) { return VALUE(a) < b; }
template <class T, int N> inline bool operator>(const Dual<T, N>& a, double b) { return VALUE(a) > b; }

// ---- univariate functions: value + chain rule -------------------------------
// chain(a, f(a.x), f'(a.x))
template <class T, int N>
inline Dual<T, N> chain(const Dual<T, N>& a, const T& f, const T& fp) {
  Dual<T, N> r(f, 0);
  for (int i = 0; i < N; ++i) r.dx[i] = fp * a.dx[i];
  return r;
}

using std::sqrt;
using std::sin;
using std::cos;
using std::acos;

template <class T, int N>
inline Dual<T, N> sqrt(const Dual<T, N>& a) {
  T s = sqrt(a.x);
  return chain(a, s, T(0.5) / s);
}
template <class T, int N>
inline Dual<T, N> sin(const Dual<T, N>& a) { return chain(a, sin(a.x), cos(a.x)); }
template <class T, int N>
inline Dual<T, N> cos(const Dual<T, N>& a) { return chain(a, cos(a.x), -sin(a.x)); }
template <class T, int N>
inline Dual<T, N> acos(const Dual<T, N>& a) {
  return chain(a, acos(a.x), T(-1.0) / sqrt(T(1.0) - a.x * a.x));
}

// ---- helpers ----------------------------------------------------------------
template <class S> inline S sq(const S& a) { return a * a; }

// zero of the same type as `a` (the reference's `zero(eltype(v))`)
template <class S> inline S zero_like(const S&) { return S(0.0); }

}  // namespace oracle
