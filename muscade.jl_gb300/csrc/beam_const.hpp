// Host-side repacking of an EulerBeam3D record (the element's fields in the
// reference's declaration order, toolbox/BeamElement.jl:87-103 with the
// BeamCrossSection of :6-22) into the constants the element kernels use.
#pragma once
#include "beam_math.hpp"

namespace mgpu {

constexpr int BEAM_NFIELD = 69;

MG_HD void beam_const_from_fields(const double* f, BeamConst& c) {
  const double* rm = f + 3;
  const double* tgm = f + 18;
  const double* ya = f + 24;
  const double* yu = f + 28;
  const double* yv = f + 32;
  const double* ka = f + 36;
  const double* ku = f + 40;
  const double* kv = f + 44;
  const double L = f[48];
  const double* dL = f + 49;
  const double* mat = f + 53;
  for (int k = 0; k < 9; ++k) c.rm[k] = rm[k];
  for (int k = 0; k < 3; ++k) c.tgm[k] = tgm[k];
  c.L = L;
  // Gauss sums, added in symmetric pairs (points 1,4 and 2,3) so that odd
  // integrands such as κᵤκᵥ cancel exactly
  auto gsum = [&](auto f) { return (f(0) + f(3)) + (f(1) + f(2)); };
  const double S0 = gsum([&](int g) { return dL[g]; });
  const double Sa2 = gsum([&](int g) { return dL[g] * ka[g] * ka[g]; });
  const double Su2 = gsum([&](int g) { return dL[g] * ku[g] * ku[g]; });
  const double Sv2 = gsum([&](int g) { return dL[g] * kv[g] * kv[g]; });
  const double Suv = gsum([&](int g) { return dL[g] * ku[g] * kv[g]; });
  for (int g = 0; g < 4; ++g) {
    c.dL[g] = dL[g];
    c.ya[g] = ya[g];
    c.yu[g] = yu[g];
    c.yv[g] = yv[g];
  }
  const double EA = mat[0], EI2 = mat[1], EI3 = mat[2], GJ = mat[3];
  c.S0 = S0;
  c.ke = EA * S0;
  c.kt = GJ * Sa2;
  c.k3u = EI3 * Su2;
  c.k3uv = EI3 * Suv;
  c.k3v = EI3 * Sv2;
  c.k2u = EI2 * Su2;
  c.k2uv = EI2 * Suv;
  c.k2v = EI2 * Sv2;
  c.mu = mat[4];
  c.iota1 = mat[5];
  c.w = mat[6];
  c.Ca[0] = mat[7];
  c.Cl[0] = mat[8];
  c.Cq[0] = mat[9];
  c.Ca[1] = mat[10];
  c.Cl[1] = mat[11];
  c.Cq[1] = mat[12];
  c.Ca[2] = mat[13];
  c.Cl[2] = mat[14];
  c.Cq[2] = mat[15];
}

}  // namespace mgpu
