// Algorithmic FP64 operation count of the beam element kernels: the same
// element code (beam_math.hpp) instantiated on the host with a counting
// scalar.  Every add/sub, mul, fma, div, sqrt and elementary function the
// kernel evaluates for one element is counted once; flops = add + mul + 2 fma
// + div + sqrt + functions.  Prints one JSON object.
#include <cmath>
#include <cstdio>

namespace cnt {
struct Counter {
  long long add = 0, mul = 0, fma = 0, div = 0, sqrt = 0, fun = 0;
};
inline Counter& C() {
  static Counter c;
  return c;
}
struct CountD {
  double v;
  CountD() : v(0.0) {}
  CountD(double x) : v(x) {}
  CountD& operator+=(const CountD& o) { C().add++; v += o.v; return *this; }
  CountD& operator-=(const CountD& o) { C().add++; v -= o.v; return *this; }
};
inline CountD operator+(CountD a, CountD b) { C().add++; return CountD(a.v + b.v); }
inline CountD operator-(CountD a, CountD b) { C().add++; return CountD(a.v - b.v); }
inline CountD operator*(CountD a, CountD b) { C().mul++; return CountD(a.v * b.v); }
inline CountD operator/(CountD a, CountD b) { C().div++; return CountD(a.v / b.v); }
inline CountD operator-(CountD a) { return CountD(-a.v); }
inline bool operator<(CountD a, CountD b) { return a.v < b.v; }
inline bool operator>(CountD a, CountD b) { return a.v > b.v; }
inline bool operator==(CountD a, CountD b) { return a.v == b.v; }
inline bool operator!=(CountD a, CountD b) { return a.v != b.v; }
inline CountD fma(CountD a, CountD b, CountD c) { C().fma++; return CountD(std::fma(a.v, b.v, c.v)); }
inline CountD sqrt(CountD a) { C().sqrt++; return CountD(std::sqrt(a.v)); }
inline CountD sin(CountD a) { C().fun++; return CountD(std::sin(a.v)); }
inline CountD cos(CountD a) { C().fun++; return CountD(std::cos(a.v)); }
inline CountD acos(CountD a) { C().fun++; return CountD(std::acos(a.v)); }
inline void sincos(CountD a, CountD* s, CountD* c) { C().fun++; s->v = std::sin(a.v); c->v = std::cos(a.v); }
inline CountD fabs(CountD a) { return CountD(std::fabs(a.v)); }
inline bool isnan(CountD a) { return std::isnan(a.v); }
inline double to_d(CountD a) { return a.v; }
}  // namespace cnt

using cnt::CountD;
using cnt::fma;
using cnt::sqrt;
using cnt::sin;
using cnt::cos;
using cnt::acos;
using cnt::sincos;
using cnt::fabs;
using cnt::to_d;
#define MGPU_REAL CountD
#define MGPU_HAVE_TO_D 1
#include "beam_const.hpp"

int main() {
  // a generic element and state: rotated nodes (generic branches of sinc1/scac)
  double f[69] = {0};
  const double c1[3] = {0.0, 0.0, 0.0}, c2[3] = {1.0, 0.3, 0.2};
  // fields of an element from c1 to c2 with orient2 = (0,1,0) built by hand is
  // not needed for counting: any consistent frame works
  double t[3] = {c2[0], c2[1], c2[2]};
  double L = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  for (int i = 0; i < 3; ++i) t[i] /= L;
  double nvec[3] = {-t[1], t[0], 0.0};
  double nn = std::sqrt(nvec[0] * nvec[0] + nvec[1] * nvec[1]);
  for (int i = 0; i < 3; ++i) nvec[i] /= nn;
  double b[3] = {t[1] * nvec[2] - t[2] * nvec[1], t[2] * nvec[0] - t[0] * nvec[2], t[0] * nvec[1] - t[1] * nvec[0]};
  for (int i = 0; i < 3; ++i) {
    f[3 + i] = t[i];
    f[6 + i] = nvec[i];
    f[9 + i] = b[i];
    f[18 + i] = c2[i] - c1[i];
  }
  const double z[4] = {-0.4305681557970263, -0.16999052179242816, 0.16999052179242816, 0.4305681557970263};
  const double w[4] = {0.17392742256872692, 0.3260725774312731, 0.3260725774312731, 0.17392742256872692};
  for (int g = 0; g < 4; ++g) {
    f[24 + g] = 2 * z[g];
    f[28 + g] = -4 * z[g] * z[g] * z[g] + 3 * z[g];
    f[32 + g] = (z[g] * z[g] - 0.25) * L;
    f[36 + g] = 2 / L;
    f[40 + g] = -24 * z[g] / (L * L);
    f[44 + g] = 2 / L;
    f[49 + g] = w[g] * L;
  }
  f[48] = L;
  const double mat[16] = {1e8, 1e4, 1e4, 1e4, 10.0, 1.0, 0.0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < 16; ++k) f[53 + k] = mat[k];
  mgpu::BeamConst bc;
  mgpu::beam_const_from_fields(f, bc);
  double X0[12] = {1e-3, 2e-3, -1e-3, 0.1, -0.2, 0.15, 3e-3, -2e-3, 1e-3, 0.12, -0.18, 0.2};
  double X1[12], X2[12];
  for (int i = 0; i < 12; ++i) {
    X1[i] = 0.01 * (i + 1);
    X2[i] = -0.02 * (i + 1);
  }
  double R[12], K[144], rd[12];
  cnt::C() = cnt::Counter();
  mgpu::beam_element<false>(bc, X0, X0, X0, nullptr, mgpu::Perturb{1, 0, 0}, nullptr, nullptr, R, K, nullptr, nullptr);
  cnt::Counter s = cnt::C();
  cnt::C() = cnt::Counter();
  mgpu::beam_element<true>(bc, X0, X1, X2, nullptr, mgpu::Perturb{1, 0.5, 0.25}, nullptr, nullptr, R, K, nullptr,
                           nullptr);
  cnt::Counter d = cnt::C();
  auto fl = [](const cnt::Counter& c) { return c.add + c.mul + 2 * c.fma + c.div + c.sqrt + c.fun; };
  printf("{\"fp64_flops_per_beam_static\": %lld, \"fp64_flops_per_beam_newmark_iter\": %lld, "
         "\"static\": {\"add\": %lld, \"mul\": %lld, \"fma\": %lld, \"div\": %lld, \"sqrt\": %lld, \"fun\": %lld}, "
         "\"newmark_iter\": {\"add\": %lld, \"mul\": %lld, \"fma\": %lld, \"div\": %lld, \"sqrt\": %lld, \"fun\": %lld}, "
         "\"convention\": \"flops = add + mul + 2*fma + div + sqrt + elementary functions, one element, counted once\"}\n",
         fl(s), fl(d), s.add, s.mul, s.fma, s.div, s.sqrt, s.fun, d.add, d.mul, d.fma, d.div, d.sqrt, d.fun);
  return 0;
}
