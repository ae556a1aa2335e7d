// Host check of the truncated Taylor arithmetic (muscade.jl_gb300/csrc/tj.hpp):
// the block products of the two-node structure against the general
// six-variable product of the embedded values, and the FMA forms against
// product-plus-sum, on seeded random values with and without the time jet.
// Prints the largest relative difference per check; exit code 0.
#include <cmath>
#include <cstdio>
#include <random>

#include "tj.hpp"

using namespace mgpu;

static std::mt19937_64 rng(2026);
static double U() { return std::uniform_real_distribution<double>(-1.0, 1.0)(rng); }

template <bool D, int N>
static TJ<D, N> rnd() {
  TJ<D, N> a;
  a.v = U();
  for (int i = 0; i < N; ++i) a.g[i] = U();
  for (int i = 0; i < TJ<D, N>::nh; ++i) a.h[i] = U();
  if constexpr (D) {
    a.vt = U();
    a.vtt = U();
    for (int i = 0; i < N; ++i) {
      a.gt[i] = U();
      a.gtt[i] = U();
    }
  }
  return a;
}

// a value over node 1's (off = 0) or node 2's (off = 3) variables as a six-variable value
template <bool D>
static TJ<D> embed(const TJ<D, 3>& x, int off) {
  TJ<D> r = tj_const<D>(x.v);
  for (int i = 0; i < 3; ++i) r.g[off + i] = x.g[i];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) r.h[hidx(off + i, off + j)] = x.h[hidx<3>(i, j)];
  if constexpr (D) {
    r.vt = x.vt;
    r.vtt = x.vtt;
    for (int i = 0; i < 3; ++i) {
      r.gt[off + i] = x.gt[i];
      r.gtt[off + i] = x.gtt[i];
    }
  }
  return r;
}

template <bool D>
static double diff(const TJ<D>& a, const TJ<D>& b) {
  double m = std::fabs(a.v - b.v), s = std::fabs(b.v);
  for (int i = 0; i < NV; ++i) m = std::fmax(m, std::fabs(a.g[i] - b.g[i])), s = std::fmax(s, std::fabs(b.g[i]));
  for (int i = 0; i < NH; ++i) m = std::fmax(m, std::fabs(a.h[i] - b.h[i])), s = std::fmax(s, std::fabs(b.h[i]));
  if constexpr (D) {
    m = std::fmax(m, std::fmax(std::fabs(a.vt - b.vt), std::fabs(a.vtt - b.vtt)));
    for (int i = 0; i < NV; ++i) {
      m = std::fmax(m, std::fmax(std::fabs(a.gt[i] - b.gt[i]), std::fabs(a.gtt[i] - b.gtt[i])));
      s = std::fmax(s, std::fmax(std::fabs(b.gt[i]), std::fabs(b.gtt[i])));
    }
  }
  return m / std::fmax(s, 1e-300);
}

template <bool D>
static void run(const char* tag) {
  double e_cross = 0, e_cross_acc = 0, e_mix = 0, e_mix_acc = 0, e_fma = 0, e_fnma = 0, e_sfma = 0;
  for (int rep = 0; rep < 200; ++rep) {
    const TJ<D, 3> x = rnd<D, 3>(), y = rnd<D, 3>();
    const TJ<D> a = rnd<D, 6>(), b = rnd<D, 6>(), c = rnd<D, 6>();
    const TJ<D> X = embed(x, 0), Y = embed(y, 3);
    e_cross = std::fmax(e_cross, diff(tj_cross<false>(x, y, c), X * Y));
    e_cross_acc = std::fmax(e_cross_acc, diff(tj_cross<true>(x, y, c), X * Y + c));
    e_mix = std::fmax(e_mix, diff(tj_mixA<false>(a, x, c), a * X));
    e_mix_acc = std::fmax(e_mix_acc, diff(tj_mixA<true>(a, x, c), a * X + c));
    e_fma = std::fmax(e_fma, diff(tj_fma(a, b, c), a * b + c));
    e_fnma = std::fmax(e_fnma, diff(tj_fnma(a, b, c), c - a * b));
    const double s = U();
    e_sfma = std::fmax(e_sfma, diff(tj_fma(a, s, c), a * s + c));
  }
  printf("%s cross %.3e cross_acc %.3e mixA %.3e mixA_acc %.3e fma %.3e fnma %.3e scalar_fma %.3e\n", tag, e_cross,
         e_cross_acc, e_mix, e_mix_acc, e_fma, e_fnma, e_sfma);
}

int main() {
  run<false>("static");
  run<true>("dynamic");
  return 0;
}
