// Host evaluation of the device element code (muscade.jl_gb300/csrc/beam_math.hpp)
// for the CPU parity test against the oracle's nested duals.
// stdin:  nele mode a1 b1, then per element 69 fields and X0[12], X1[12], X2[12]
//         (mode 1: SweepX{0} R and K;  mode 3: Newmark iteration R and K + a1 C + b1 M)
// stdout: per element R[12] then K[144] (column-major, K[i + 12 j] = ∂R_i/∂X_j)
#include <cstdio>
#include <initializer_list>

#include "beam_const.hpp"

int main() {
  long nele = 0;
  int mode = 1;
  double a1 = 0, b1 = 0;
  if (scanf("%ld %d %lf %lf", &nele, &mode, &a1, &b1) != 4) return 2;
  for (long e = 0; e < nele; ++e) {
    double f[69], X0[12], X1[12], X2[12], R[12], K[144];
    for (double& v : f)
      if (scanf("%lf", &v) != 1) return 2;
    for (double* X : {X0, X1, X2})
      for (int i = 0; i < 12; ++i)
        if (scanf("%lf", &X[i]) != 1) return 2;
    mgpu::BeamConst bc;
    mgpu::beam_const_from_fields(f, bc);
    if (mode == 1)
      mgpu::beam_element<false>(bc, X0, X0, X0, nullptr, mgpu::Perturb{1, 0, 0}, nullptr, nullptr, R, K, nullptr,
                                nullptr);
    else
      mgpu::beam_element<true>(bc, X0, X1, X2, nullptr, mgpu::Perturb{1, a1, b1}, nullptr, nullptr, R, K, nullptr,
                               nullptr);
    for (double v : R) printf("%.17g ", v);
    for (double v : K) printf("%.17g ", v);
    printf("\n");
  }
  return 0;
}
