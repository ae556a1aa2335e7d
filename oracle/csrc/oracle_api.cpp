// Oracle (test infrastructure only): C entry points over the dual-number
// restatement, called through ctypes by the tests, by the golden-vector
// checks and by the CPU-baseline leg of bench.py.  Never linked into the
// product library.
//
// Seeding modes mirror the reference's assemblers:
//   mode 0  "diffed"      one partial per X₀,X₁,X₂ (and U) entry, like
//                         diffed_residual (src/Diagnostic.jl:929-965)
//   mode 1  SweepX{0}     δX = δ{1,Nx}(scale.X)              (src/SweepX.jl:90-96)
//   mode 2  SweepX{2}     step: δX and δr                     (src/SweepX.jl:45-59)
//   mode 3  SweepX{2}     iter: δX with a₁, b₁                (src/SweepX.jl:60-67)
// In modes 1-3 the residual and its partials are multiplied by scale.X like
// `Lλ .* scale.X`.
#include <cstdint>
#include <cstring>
#include <vector>

#include "bar.hpp"

using namespace oracle;

namespace {

template <int NO>
using OD = Dual<double, NO>;

// Element adaptor: evaluates R and its partials for one element with NX dofs.
template <int NX, int NO, class F>
void eval_one(F&& resid, int ND, const double* X, const double* U, int nU, int mode, double a1, double b1,
              const double* sX, const double* av, const double* bv, double* R, double* J, int NJ) {
  OD<NO> Xo[3][NX];
  OD<NO> Uo[3];
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < NX; ++i) Xo[d][i] = OD<NO>(d < ND ? X[d * NX + i] : 0.0);
  for (int i = 0; i < nU; ++i) Uo[i] = OD<NO>(U[i]);
  if (mode == 0) {
    int p = 0;
    for (int d = 0; d < ND; ++d)
      for (int i = 0; i < NX; ++i, ++p)
        if (p < NO) Xo[d][i].dx[p] = 1.0;
    for (int i = 0; i < nU; ++i, ++p)
      if (p < NO) Uo[i].dx[p] = 1.0;
  } else if (mode == 1) {
    for (int i = 0; i < NX; ++i) Xo[0][i].dx[i] = sX[i];
  } else {
    for (int i = 0; i < NX; ++i) {
      Xo[0][i].dx[i] = sX[i];
      Xo[1][i].dx[i] = a1 * sX[i];
      Xo[2][i].dx[i] = b1 * sX[i];
      if (mode == 2 && NX < NO) {  // δr with partial 1 in slot NX
        Xo[1][i].dx[NX < NO ? NX : 0] = av[i];
        Xo[2][i].dx[NX < NO ? NX : 0] = bv[i];
      }
    }
  }
  OD<NO> Ro[NX];
  resid(Xo, Uo, Ro);
  for (int i = 0; i < NX; ++i) {
    double s = (mode == 0) ? 1.0 : sX[i];
    R[i] = Ro[i].x * s;
    for (int j = 0; j < NJ && j < NO; ++j) J[i * NJ + j] = Ro[i].dx[j] * s;
  }
}

template <int NX, int NO, class F>
void eval_all(F&& make_resid, int n, int ND, const double* X, const double* U, int nU, int mode, double a1,
              double b1, const double* scaleX, const double* a, const double* b, double* R, double* J, int NJ,
              int nthreads) {
  std::vector<double> ones(NX, 1.0);
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t e = 0; e < n; ++e) {
    const double* sX = scaleX ? scaleX + e * NX : ones.data();
    auto resid = make_resid(e);
    eval_one<NX, NO>(resid, ND, X + e * ND * NX, U ? U + e * nU : nullptr, nU, mode, a1, b1, sX,
                     a ? a + e * NX : nullptr, b ? b + e * NX : nullptr, R + e * NX, J + e * NX * NJ, NJ);
  }
}

}  // namespace

extern "C" {

int oracle_beam_construct(int64_t n, const double* c1, const double* c2, const double* orient2, const double* mat,
                          double* ele) {
  int bad = 0;
  for (int64_t e = 0; e < n; ++e) {
    BeamMat m;
    std::memcpy(&m, mat + 16 * e, sizeof(BeamMat));
    BeamEle o;
    if (beam_construct(c1 + 3 * e, c2 + 3 * e, orient2 + 3 * e, m, o)) bad = 1;
    std::memcpy(ele + 69 * e, &o, sizeof(BeamEle));
  }
  return bad;
}

int oracle_bar_construct(int64_t n, const double* c1, const double* c2, const double* mat, double epss, double* ele) {
  for (int64_t e = 0; e < n; ++e) {
    BarMat m;
    std::memcpy(&m, mat + 9 * e, sizeof(BarMat));
    BarEle o;
    bar_construct(c1 + 3 * e, c2 + 3 * e, m, epss, o);
    std::memcpy(ele + 38 * e, &o, sizeof(BarEle));
  }
  return 0;
}

// Element results of EulerBeam3D at states X[n][12] (getresult of the
// residual's requestable values, toolbox/BeamElement.jl:151-189 with
// kinematics :177-189 and resultants :28-62): out[n][50] = ε, rₛₘ (9,
// column-major), then per Gauss point x (3), κ (3), fᵢ, mᵢ (3).
int oracle_beam_results(int64_t n, const double* ele, const double* X, double* out) {
  for (int64_t e = 0; e < n; ++e) {
    BeamEle o;
    std::memcpy(&o, ele + 69 * e, sizeof(BeamEle));
    BeamKin<double> k;
    kinematics(o, X + 12 * e, k);
    double* r = out + 50 * e;
    r[0] = k.eps;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) r[1 + i + 3 * j] = k.rsm.m[i + 3 * j];
    for (int g = 0; g < 4; ++g) {
      double* q = r + 10 + 10 * g;
      for (int i = 0; i < 3; ++i) q[i] = k.x[g].v[i];
      for (int i = 0; i < 3; ++i) q[3 + i] = k.kappa[g].v[i];
      q[6] = o.mat.EA * k.eps;
      q[7] = o.mat.GJ * k.kappa[g].v[0];
      q[8] = o.mat.EI3 * k.kappa[g].v[1];
      q[9] = o.mat.EI2 * k.kappa[g].v[2];
    }
  }
  return 0;
}

// Number of partials returned in J for a given mode.
int oracle_nj(int nx, int ND, int nU, int mode) {
  if (mode == 0) return nx * ND + nU;
  if (mode == 2) return nx + 1;
  return nx;
}

// Beam: X[n][ND][12], U[n][3] (udof only), R[n][12], J[n][12][NJ].
int oracle_beam_eval(int64_t n, const double* ele, int ND, const double* X, const double* U, int udof, int mode,
                     double a1, double b1, const double* scaleX, const double* a, const double* b, double* R,
                     double* J, int nthreads) {
  int nU = udof ? 3 : 0;
  int NJ = oracle_nj(12, ND, nU, mode);
  if (ND < 1 || ND > 3) return 2;
  if ((mode == 2 || mode == 3) && ND != 3) return 2;
  if (mode == 1 && ND != 1) return 2;
  const BeamEle* E = reinterpret_cast<const BeamEle*>(ele);
  bool ud = udof != 0;
#define BEAM_CASE(NO, NDV)                                                                                      \
  eval_all<12, NO>(                                                                                             \
      [&](int64_t e) {                                                                                          \
        return [&, e](OD<NO>(*Xo)[12], OD<NO>* Uo, OD<NO>* Ro) { beam_residual<OD<NO>, NDV>(E[e], Xo, Uo, ud, Ro); }; \
      },                                                                                                        \
      n, ND, X, U, nU, mode, a1, b1, scaleX, a, b, R, J, NJ, nthreads)
  if (mode == 1) {
    BEAM_CASE(12, 1);
  } else if (mode == 2) {
    BEAM_CASE(13, 3);
  } else if (mode == 3) {
    BEAM_CASE(12, 3);
  } else {
    if (ND == 1) { BEAM_CASE(15, 1); }
    else if (ND == 2) { BEAM_CASE(27, 2); }
    else { BEAM_CASE(39, 3); }
  }
#undef BEAM_CASE
  return 0;
}

int oracle_bar_eval(int64_t n, const double* ele, int ND, const double* X, const double* U, int udof, double t,
                    int mode, double a1, double b1, const double* scaleX, const double* a, const double* b, double* R,
                    double* J, int nthreads) {
  int nU = udof ? 3 : 0;
  int NJ = oracle_nj(6, ND, nU, mode);
  if (ND < 1 || ND > 3) return 2;
  if ((mode == 2 || mode == 3) && ND != 3) return 2;
  if (mode == 1 && ND != 1) return 2;
  const BarEle* E = reinterpret_cast<const BarEle*>(ele);
  bool ud = udof != 0;
#define BAR_CASE(NO, NDV)                                                                                         \
  eval_all<6, NO>(                                                                                                \
      [&](int64_t e) {                                                                                            \
        return [&, e](OD<NO>(*Xo)[6], OD<NO>* Uo, OD<NO>* Ro) { bar_residual<OD<NO>, NDV>(E[e], Xo, Uo, ud, t, Ro); }; \
      },                                                                                                          \
      n, ND, X, U, nU, mode, a1, b1, scaleX, a, b, R, J, NJ, nthreads)
  if (mode == 1) {
    BAR_CASE(6, 1);
  } else if (mode == 2) {
    BAR_CASE(7, 3);
  } else if (mode == 3) {
    BAR_CASE(6, 3);
  } else {
    if (ND == 1) { BAR_CASE(9, 1); }
    else if (ND == 2) { BAR_CASE(15, 2); }
    else { BAR_CASE(21, 3); }
  }
#undef BAR_CASE
  return 0;
}

// add_value! / add_∂! (src/Assemble.jl:559-608) for one element type, serial
// like the reference's loop: for each element in order, Lλ[asm1[e,i]] += R[e,i]
// and nzval[asm2[e,i+nX*j]] += J[e,i,j] (column-major entries, 0 = skip);
// J[e] is nX × NJ row-major and only its first nX columns are added.
// minus_col >= 0 also subtracts column minus_col of J from Lλ (the δr part of
// the Newmark step, add_∂!{1,:minus}).
void oracle_scatter(int64_t nele, int nX, int NJ, const int64_t* asm1, const int64_t* asm2, const double* R,
                    const double* J, int minus_col, double* Ll, double* nzval) {
  for (int64_t e = 0; e < nele; ++e) {
    const double* Re = R + e * nX;
    const double* Je = J + e * nX * NJ;
    const int64_t* a1 = asm1 + e * nX;
    const int64_t* a2 = asm2 + e * nX * nX;
    for (int i = 0; i < nX; ++i)
      if (a1[i]) Ll[a1[i] - 1] += Re[i];
    if (minus_col >= 0)
      for (int i = 0; i < nX; ++i)
        if (a1[i]) Ll[a1[i] - 1] += -Je[i * NJ + minus_col];
    for (int j = 0; j < nX; ++j)
      for (int i = 0; i < nX; ++i) {
        const int64_t q = a2[i + nX * j];
        if (q) nzval[q - 1] += Je[i * NJ + j];
      }
  }
}

// ---- rotation helpers for the golden tests (test/TestRotations.jl) ----------
double oracle_sinc1k(int k, double x) {
  switch (k) {
    case 0: return sinc1_0(x);
    case 1: return sinc1_1(x);
    case 2: return sinc1_2(x);
    case 3: return sinc1_3(x);
    case 4: return sinc1_4(x);
    default: return sinc1_5(x);
  }
}
// scac and its first four derivatives through nested duals (like scac1..scac4)
void oracle_scac_derivs(double x, double* out5) {
  using D1 = Dual<double, 1>;
  using D2 = Dual<D1, 1>;
  using D3 = Dual<D2, 1>;
  using D4 = Dual<D3, 1>;
  D1 a(x);
  a.dx[0] = 1.0;
  D2 b(a, 0);
  b.dx[0] = D1(1.0);
  D3 c(b, 0);
  c.dx[0] = D2(1.0);
  D4 d(c, 0);
  d.dx[0] = D3(1.0);
  D4 y = scac(d);
  out5[0] = y.x.x.x.x;
  out5[1] = y.x.x.x.dx[0];
  out5[2] = y.x.x.dx[0].dx[0];
  out5[3] = y.x.dx[0].dx[0].dx[0];
  out5[4] = y.dx[0].dx[0].dx[0].dx[0];
}
void oracle_rodrigues(const double* v, double* R) {
  V3<double> a;
  for (int i = 0; i < 3; ++i) a.v[i] = v[i];
  M3<double> M = Rodrigues(a);
  for (int k = 0; k < 9; ++k) R[k] = M.m[k];
}
// w = Rodrigues⁻¹(Rodrigues(v)) and ∂w/∂v (3x3 row-major)
void oracle_rodrigues_roundtrip(const double* v, double* w, double* J) {
  using D = Dual<double, 3>;
  V3<D> a;
  for (int i = 0; i < 3; ++i) {
    a.v[i] = D(v[i]);
    a.v[i].dx[i] = 1.0;
  }
  V3<D> r = Rodriguesinv(Rodrigues(a));
  for (int i = 0; i < 3; ++i) {
    w[i] = r.v[i].x;
    for (int j = 0; j < 3; ++j) J[3 * i + j] = r.v[i].dx[j];
  }
}

}  // extern "C"
