// Host evaluation of the device element code (muscade.jl_gb300/csrc/beam_math.hpp
// and bar_math.hpp, the bodies of beam_kernel and bar_kernel) for the CPU parity
// test against the oracle's nested duals.
// stdin:  kind nele nder p0 p1 p2 t   (kind: beam | bar), then per element its
//         fields (69 beam, 38 bar) and X0, X1, X2 (12 or 6 values each)
// stdout: per element R[nx] then the matrix [nx*nx] (column-major, entry i + nx j
//         = ∂R_i/∂X_j along the variation X₀ += p0 δ, X₁ += p1 δ, X₂ += p2 δ)
#include <cstdio>
#include <cstring>
#include <initializer_list>

#include "bar_math.hpp"
#include "beam_const.hpp"

int main() {
  char kind[16];
  long nele = 0;
  int nder = 1;
  double p0 = 1, p1 = 0, p2 = 0, t = 0;
  if (scanf("%15s %ld %d %lf %lf %lf %lf", kind, &nele, &nder, &p0, &p1, &p2, &t) != 7) return 2;
  const bool beam = std::strcmp(kind, "beam") == 0;
  const int nf = beam ? 69 : 38, nx = beam ? 12 : 6;
  for (long e = 0; e < nele; ++e) {
    double f[69], X0[12], X1[12], X2[12], R[12], K[144];
    for (int i = 0; i < nf; ++i)
      if (scanf("%lf", &f[i]) != 1) return 2;
    for (double* X : {X0, X1, X2})
      for (int i = 0; i < nx; ++i)
        if (scanf("%lf", &X[i]) != 1) return 2;
    if (beam) {
      mgpu::BeamConst bc;
      mgpu::beam_const_from_fields(f, bc);
      if (nder == 1)
        mgpu::beam_element<false>(bc, X0, X0, X0, nullptr, mgpu::Perturb{p0, 0, 0}, nullptr, nullptr, R, K, nullptr,
                                  nullptr);
      else
        mgpu::beam_element<true>(bc, X0, X1, X2, nullptr, mgpu::Perturb{p0, p1, p2}, nullptr, nullptr, R, K, nullptr,
                                 nullptr);
    } else {
      mgpu::BarConst bc;
      mgpu::bar_const_from_fields(f, bc);
      mgpu::bar_element(bc, nder, X0, X1, X2, nullptr, t, p0, p1, p2, nullptr, nullptr, R, K, nullptr, nullptr);
    }
    for (int i = 0; i < nx; ++i) printf("%.17g ", R[i]);
    for (int i = 0; i < nx * nx; ++i) printf("%.17g ", K[i]);
    printf("\n");
  }
  return 0;
}
