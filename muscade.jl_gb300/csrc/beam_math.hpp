// EulerBeam3D residual and exact Newton tangent, closed form over the
// corotational kinematics, for the GB300 element kernels (host-compilable too).
//
// Reference behaviour (toolbox/BeamElement.jl):
//   residual   :151-174    R = Σ_gp (fᵢ ε∂X₀ + mᵢ·κ∂X₀ + fₑ·x∂X₀ + mₑ·vₛₘ∂X₀) dL
//   kinematics :177-189,  corotated :193-208,  resultants :28-64
//   rotations  toolbox/Rotations.jl:13-182 (sinc1 branches, scac Taylor
//              branch, norm3 zeroing below 1e-14 -- all mirrored here)
//
// Formulation used here (mathematically identical to the reference):
//  * The rotation core (r₁, r₂, Δv = ½Rod⁻¹(r₂r₁ᵀ), rₛₘ = Rod(Δv) r₁ rₘ, vₛₘ)
//    depends only on the six rotation dofs; it is evaluated in truncated
//    Taylor arithmetic (tj.hpp) which yields values, gradients, Hessians and
//    the time jets needed by inertia and drag.
//  * With t,n,b the columns of rₛₘ and d = ½(u₂-u₁)+½tgₘ, the local quantities
//    are uₗ₂ = rₛₘᵀd − ½L e₁ and vₗ₂ = rₛₘᵀΔv, hence ε = 2|d|/L − 1,
//    κ = (κₐ t·Δv, κᵤ n·d + κᵥ b·Δv, κᵤ b·d − κᵥ n·Δv) and the Gauss point
//    position x = yᵤ d + (yₐ−yᵤ)(t·d) t + yᵥ Δv×t + ½(u₁+u₂) + cₘ.
//  * Σ_gp(fᵢ ε∂X₀ + mᵢ·κ∂X₀)dL is the gradient of the quadratic strain energy
//    Π; the external terms are the gradient of ψ = Σ_gp dL f_gp·x_gp +
//    Σ_gp dL mₑ·vₛₘ with the loads held fixed.  R = ∇(Π+ψ) and the tangent is
//    ∇²(Π+ψ) plus Σ_gp dL x∂X₀ᵀ δf_gp + vₛₘ∂X₀ᵀ δmₑ (load variation).
// Output layout: R[12], K[i + 12 j] = ∂R_i/∂X_j (column-major, like asm[2]).
#pragma once
#include "tj.hpp"

namespace mgpu {

// ---- special functions (toolbox/Rotations.jl) -------------------------------
// sinc1(x)=sin(x)/x and its derivatives with the reference's branch points.
MG_HD real sinc1_0(real x) {
  const real y = x * 0.31830988618379067154;  // x/π (Base.sinc of x/π)
  if (fabs(y) < 1e-3) {
    const real p2 = 9.8696044010893586188;  // π²
    const real y2 = y * y;
    return 1.0 + y2 * (-p2 / 6.0 + y2 * (p2 * p2 / 120.0));
  }
  return sin(x) / x;
}
MG_HD real sinc1_1(real x) {
  if (fabs(x) > 1e-3) {
    real s, c;
    sincos(x, &s, &c);
    return c / x - s / (x * x);
  }
  const real x2 = x * x;
  return x * (-1.0 / 3.0 + x2 / 30.0);
}
MG_HD real sinc1_2(real x) {
  if (fabs(x) > 1e-1) {
    real s, c;
    sincos(x, &s, &c);
    return -s / x - 2.0 * c / (x * x) + 2.0 * s / (x * x * x);
  }
  const real x2 = x * x;
  return -1.0 / 3.0 + x2 * (1.0 / 10.0 + x2 * (-1.0 / 168.0 + x2 * (1.0 / 6480.0)));
}
MG_HD real sinc1_3(real x) {
  if (fabs(x) > 0.4) {
    real s, c;
    sincos(x, &s, &c);
    const real x2 = x * x;
    return -c / x + 3.0 * s / x2 + 6.0 * c / (x2 * x) - 6.0 * s / (x2 * x2);
  }
  const real x2 = x * x;
  return x * (1.0 / 5.0 + x2 * (-1.0 / 42.0 + x2 * (1.0 / 1080.0 + x2 * (-1.0 / 55440.0 + x2 * (1.0 / 4717440.0)))));
}

// scac(x) = sinc1(acos x) with the reference's degree-5 Taylor branch near 1;
// f[0..3] = value and first three derivatives.
MG_HD void scac_derivs(real x, real f[4]) {
  const real dx = x - 1.0;
  if (fabs(dx) > 1e-3) {
    const real th = acos(x);
    const real q = 1.0 - x * x;
    const real sq = sqrt(q);
    const real t1 = -1.0 / sq;
    const real t2 = -x / (q * sq);
    const real t3 = -(1.0 + 2.0 * x * x) / (q * q * sq);
    const real s0 = sinc1_0(th), s1 = sinc1_1(th), s2 = sinc1_2(th), s3 = sinc1_3(th);
    f[0] = s0;
    f[1] = s1 * t1;
    f[2] = s2 * t1 * t1 + s1 * t2;
    f[3] = s3 * t1 * t1 * t1 + 3.0 * s2 * t1 * t2 + s1 * t3;
    return;
  }
  const real c1 = 1.0 / 3.0, c2 = -2.0 / 90.0, c3 = 0.0052911879917544626, c4 = -0.0016229317117234072, c5 = 0.0005625;
  f[0] = 1.0 + dx * (c1 + dx * (c2 + dx * (c3 + dx * (c4 + dx * c5))));
  f[1] = c1 + dx * (2.0 * c2 + dx * (3.0 * c3 + dx * (4.0 * c4 + dx * (5.0 * c5))));
  f[2] = 2.0 * c2 + dx * (6.0 * c3 + dx * (12.0 * c4 + dx * (20.0 * c5)));
  f[3] = 6.0 * c3 + dx * (24.0 * c4 + dx * (60.0 * c5));
}

// ---- rotations in Taylor arithmetic ----------------------------------------
// Rodrigues(v) = I + sinc1(θ) S + ½ sinc1(θ/2)² S²,  θ = norm3(v)   (Rotations.jl:131-135)
// A = sinc1(θ) and B = ½ sinc1(θ/2)² as compositions of s2 = |v|²
template <bool D, int N>
MG_HD void rod_AB(const TJ<D, N>& s2, TJ<D, N>& A, TJ<D, N>& B) {
  const real th = sqrt(s2.v);
  if (th < 1e-14) {  // norm3 returns an exact zero: sinc1 terms become constants
    A = tj_const<D, N>(1.0);
    B = tj_const<D, N>(0.5);
  } else {
    const real r = 1.0 / th;
    // θ = √s2
    const TJ<D, N> t = tj_apply(s2, th, 0.5 * r, -0.25 * r * r * r, 0.375 * r * r * r * r * r);
    A = tj_apply(t, sinc1_0(th), sinc1_1(th), sinc1_2(th), sinc1_3(th));
    const real h = 0.5 * th;
    // B(θ) = ½ s(θ/2)² with s = sinc1, composed from its derivatives in θ:
    // B′ = ½ s s′, B″ = ¼ (s′² + s s″), B‴ = ⅛ (3 s′ s″ + s s‴)
    const real s0 = sinc1_0(h), s1 = sinc1_1(h), s2d = sinc1_2(h), s3 = sinc1_3(h);
    B = tj_apply(t, 0.5 * s0 * s0, 0.5 * s0 * s1, 0.25 * fma(s1, s1, s0 * s2d), 0.125 * fma(3.0 * s1, s2d, s0 * s3));
  }
}

template <bool D, int N>
MG_HD void rodrigues(const TJ<D, N> v[3], TJ<D, N> R[9]) {
  const TJ<D, N> s2 = tj_dot3(v, v);
  TJ<D, N> A, B;
  rod_AB(s2, A, B);
  // S = spin(v): S[2,1]=v3, S[3,1]=-v2, S[1,2]=-v3, S[3,2]=v1, S[1,3]=v2, S[2,3]=-v1
  // S² = v vᵀ - |v|² I  (spin², Rotations.jl:114-122)
  const TJ<D, N> ab = v[0] * v[1], ca = v[2] * v[0], bc = v[1] * v[2];
  const TJ<D, N> aa = v[0] * v[0], bb = v[1] * v[1], cc = v[2] * v[2];
  const TJ<D, N> one = tj_const<D, N>(1.0);
  R[0] = tj_fnma(B, bb + cc, one);
  R[4] = tj_fnma(B, aa + cc, one);
  R[8] = tj_fnma(B, aa + bb, one);
  const TJ<D, N> Bab = B * ab, Bca = B * ca, Bbc = B * bc;
  const TJ<D, N> Av0 = A * v[0], Av1 = A * v[1], Av2 = A * v[2];
  R[1] = Av2 + Bab;   // [2,1]
  R[3] = Bab - Av2;   // [1,2]
  R[2] = Bca - Av1;   // [3,1]
  R[6] = Av1 + Bca;   // [1,3]
  R[5] = Av0 + Bbc;   // [3,2]
  R[7] = Bbc - Av0;   // [2,3]
}

// Products with the nodal variables vᵢ = xᵢ + εᵢ + x1ᵢ τ + yᵢ τ² (y = ½ x₂) of one
// node, in closed form: vₐ v_b, and a·vᵢ for a general three-variable a.
template <bool D>
MG_HD TJ<D, 3> tj_varprod(int a, int b, const real x[3], const real x1[3], const real y[3]) {
  TJ<D, 3> r = tj_const<D, 3>(x[a] * x[b]);
  r.g[a] = x[b];
  r.g[b] += x[a];
  r.h[a <= b ? hidx<3>(a, b) : hidx<3>(b, a)] = a == b ? 2.0 : 1.0;
  if constexpr (D) {
    r.vt = fma(x[a], x1[b], x1[a] * x[b]);
    r.vtt = fma(x[a], y[b], fma(x1[a], x1[b], y[a] * x[b]));
    r.gt[a] = x1[b];
    r.gt[b] += x1[a];
    r.gtt[a] = y[b];
    r.gtt[b] += y[a];
  }
  return r;
}
template <bool D>
MG_HD TJ<D, 3> tj_mulvar(const TJ<D, 3>& a, int i, const real x[3], const real x1[3], const real y[3]) {
  TJ<D, 3> r = tj_scale(a, x[i]);
  r.g[i] += a.v;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const int k = m <= i ? hidx<3>(m, i) : hidx<3>(i, m);
    r.h[k] = m == i ? fma(2.0, a.g[i], r.h[k]) : r.h[k] + a.g[m];
  }
  if constexpr (D) {
    r.vt = fma(a.v, x1[i], r.vt);
    r.vtt = fma(a.vt, x1[i], fma(a.v, y[i], r.vtt));
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      r.gt[m] = fma(a.g[m], x1[i], r.gt[m]);
      r.gtt[m] = fma(a.gt[m], x1[i], fma(a.g[m], y[i], r.gtt[m]));
    }
    r.gt[i] += a.vt;
    r.gtt[i] += a.vtt;
  }
  return r;
}

// Rodrigues(v) of a node's rotation dofs v = x + ε (with their time jet), over
// those three variables
template <bool D>
MG_HD void rodrigues_nodal(const double xd[3], const double x1d[3], const double x2d[3], TJ<D, 3> R[9]) {
  const real x[3] = {xd[0], xd[1], xd[2]};
  real x1[3] = {0.0, 0.0, 0.0}, y[3] = {0.0, 0.0, 0.0};
  if constexpr (D)
    for (int i = 0; i < 3; ++i) {
      x1[i] = x1d[i];
      y[i] = 0.5 * x2d[i];
    }
  TJ<D, 3> s2 = tj_const<D, 3>(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  for (int i = 0; i < 3; ++i) {
    s2.g[i] = 2.0 * x[i];
    s2.h[hidx<3>(i, i)] = 2.0;
  }
  if constexpr (D) {
    s2.vt = 2.0 * (x[0] * x1[0] + x[1] * x1[1] + x[2] * x1[2]);
    s2.vtt = x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2] + 2.0 * (x[0] * y[0] + x[1] * y[1] + x[2] * y[2]);
    for (int i = 0; i < 3; ++i) {
      s2.gt[i] = 2.0 * x1[i];
      s2.gtt[i] = 2.0 * y[i];
    }
  }
  TJ<D, 3> A, B;
  rod_AB(s2, A, B);
  const TJ<D, 3> ab = tj_varprod<D>(0, 1, x, x1, y), ca = tj_varprod<D>(2, 0, x, x1, y),
                 bc = tj_varprod<D>(1, 2, x, x1, y);
  const TJ<D, 3> aa = tj_varprod<D>(0, 0, x, x1, y), bb = tj_varprod<D>(1, 1, x, x1, y),
                 cc = tj_varprod<D>(2, 2, x, x1, y);
  const TJ<D, 3> one = tj_const<D, 3>(1.0);
  R[0] = tj_fnma(B, bb + cc, one);
  R[4] = tj_fnma(B, aa + cc, one);
  R[8] = tj_fnma(B, aa + bb, one);
  const TJ<D, 3> Bab = B * ab, Bca = B * ca, Bbc = B * bc;
  const TJ<D, 3> Av0 = tj_mulvar(A, 0, x, x1, y), Av1 = tj_mulvar(A, 1, x, x1, y), Av2 = tj_mulvar(A, 2, x, x1, y);
  R[1] = Av2 + Bab;   // [2,1]
  R[3] = Bab - Av2;   // [1,2]
  R[2] = Bca - Av1;   // [3,1]
  R[6] = Av1 + Bca;   // [1,3]
  R[5] = Av0 + Bbc;   // [3,2]
  R[7] = Bbc - Av0;   // [2,3]
}

// Rodrigues⁻¹(m) = spin⁻¹(m) / scac((tr m − 1)/2)   (Rotations.jl:105)
template <bool D>
MG_HD void rodrigues_inv(const TJ<D> m[9], TJ<D> w[3], real scale = 1.0) {
  const TJ<D> c = (m[0] + m[4] + m[8] + (-1.0)) * 0.5;
  real f[4];
  scac_derivs(c.v, f);
  const TJ<D> s = tj_apply(c, f[0], f[1], f[2], f[3]);
  const real iv = 1.0 / s.v;
  // ½ scale / s, the ½ of spin⁻¹ and the caller's scale taken into the composition
  const real q = 0.5 * scale;
  const TJ<D> is = tj_apply(s, q * iv, -q * iv * iv, q * 2.0 * iv * iv * iv, -q * 6.0 * iv * iv * iv * iv);
  w[0] = (m[5] - m[7]) * is;  // (m32 - m23)/2
  w[1] = (m[6] - m[2]) * is;  // (m13 - m31)/2
  w[2] = (m[1] - m[3]) * is;  // (m21 - m12)/2
}

// C = B Aᵀ with A over node 1's variables and B over node 2's (r₂ r₁ᵀ)
template <bool D>
MG_HD void mul_abt_nodes(const TJ<D, 3> B[9], const TJ<D, 3> A[9], TJ<D> C[9]) {
  const TJ<D> zero = tj_const<D>(0.0);  // not accumulated into (ACC = false)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const TJ<D> z = tj_cross<false>(A[j], B[i], zero);
      C[i + 3 * j] = tj_cross<true>(A[j + 6], B[i + 6], tj_cross<true>(A[j + 3], B[i + 3], z));
    }
}
// C = A B with B over node 1's variables (r_Δ r₁)
template <bool D>
MG_HD void mul_ab_node1(const TJ<D> A[9], const TJ<D, 3> B[9], TJ<D> C[9]) {
  const TJ<D> zero = tj_const<D>(0.0);  // not accumulated into (ACC = false)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const TJ<D> z = tj_mixA<false>(A[i], B[3 * j], zero);
      C[i + 3 * j] = tj_mixA<true>(A[i + 6], B[2 + 3 * j], tj_mixA<true>(A[i + 3], B[1 + 3 * j], z));
    }
}
// Σ m[i] v[i] with m over node 1's variables (a column of r₁rₘ) and v over six
template <bool D>
MG_HD TJ<D> tj_dot3_node1(const TJ<D, 3> m[3], const TJ<D> v[3]) {
  const TJ<D> zero = tj_const<D>(0.0);  // not accumulated into (ACC = false)
  return tj_mixA<true>(v[2], m[2], tj_mixA<true>(v[1], m[1], tj_mixA<false>(v[0], m[0], zero)));
}
// C = A M with M a constant matrix
template <bool D, int N>
MG_HD void mul_ac(const TJ<D, N> A[9], const double M[9], TJ<D, N> C[9]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C[i + 3 * j] = tj_fma(A[i + 6], real(M[2 + 3 * j]), tj_fma(A[i + 3], real(M[1 + 3 * j]), A[i] * real(M[3 * j])));
}

// ---- per-element constants, precomputed at create time ----------------------
struct BeamConst {
  double rm[9];   // as-meshed frame (column-major)
  double tgm[3];  // c₂ − c₁
  double L;
  // strain energy Π = ½kε ε² + ½kt θt² + ½k3v θb² + k3uv wn θb + ½k3u wn²
  //                 + ½k2v θn² − k2uv wb θn + ½k2u wb²
  double ke, kt, k3u, k3uv, k3v, k2u, k2uv, k2v;
  double S0;                                    // Σ dL
  double dL[4], ya[4], yu[4], yv[4];            // Gauss data
  double mu, iota1, w, Ca[3], Cl[3], Cq[3];     // cross section (dynamic part)
};

// Newton variation of the state: X₀ += p0 δ, X₁ += p1 δ, X₂ += p2 δ
// (SweepX{0}: 1,0,0;  Newmark: 1,a₁,b₁;  diffed K/C/M: unit vectors).
struct Perturb {
  double p0, p1, p2;
};

// rotation-dof index (0..5) of element dof j, or -1 for translations
MG_HD int rot_index(int j) { return (j >= 3 && j < 6) ? j - 3 : (j >= 9 ? j - 6 : -1); }

// Full element evaluation.
//   X0,X1,X2: element dofs and their first/second time derivatives (X1,X2 ignored if !D)
//   U: U-dof loads per unit length (nullptr if none)
//   out R[12], K[144];  rdir[12] (optional): derivative along X₁ += a δr, X₂ += b δr
//   H[36] (optional): ∂R/∂U, column-major 12x3
template <bool D>
MG_HD void beam_element(const BeamConst& c, const double* X0, const double* X1, const double* X2, const double* U,
                        Perturb pt, const double* av, const double* bv, double* R, double* K, double* rdir,
                        double* H) {
  // ---- rotation core
  // the nodal rotations depend on their own node's three dofs only
  TJ<D, 3> r1[9];
  TJ<D> rsm[9], dv[3];
  {
    TJ<D, 3> r2[9];
    TJ<D> Q[9];
    rodrigues_nodal<D>(X0 + 3, X1 + 3, X2 + 3, r1);
    rodrigues_nodal<D>(X0 + 9, X1 + 9, X2 + 9, r2);
    mul_abt_nodes(r2, r1, Q);
    rodrigues_inv(Q, dv, 0.5);  // Δv = ½ Rodrigues⁻¹(r₂r₁ᵀ)
  }
  // rₛₘ = r_Δ (r₁ rₘ): the constant frame goes into the node-1 value first
  TJ<D, 3> r1m[9];
  mul_ac(r1, c.rm, r1m);
  {
    TJ<D> rD[9];
    rodrigues(dv, rD);
    mul_ab_node1(rD, r1m, rsm);
  }
  const TJ<D>* t = rsm;      // first column
  const TJ<D>* n = rsm + 3;  // second column
  const TJ<D>* b = rsm + 6;  // third column

  // ---- translations (d = ½(u₂−u₁)+½tgₘ enters linearly)
  real d[3], dd1[3], dd2[3];
  for (int i = 0; i < 3; ++i) {
    d[i] = 0.5 * (X0[6 + i] - X0[i]) + 0.5 * c.tgm[i];
    dd1[i] = D ? 0.5 * (X1[6 + i] - X1[i]) : 0.0;
    dd2[i] = D ? 0.5 * (X2[6 + i] - X2[i]) : 0.0;
  }
  const real dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const real dh[3] = {d[0] / dn, d[1] / dn, d[2] / dn};
  const real eps = dn * 2.0 / c.L - 1.0;

  // ---- strain measures
  // (t, n, b)·Δv = rₛₘᵀΔv = (r₁rₘ)ᵀ r_ΔᵀΔv = (r₁rₘ)ᵀΔv, since Rod(Δv) leaves Δv
  // fixed (S Δv = 0): node-1 × six-variable products
  const TJ<D> th_t = tj_dot3_node1(r1m, dv), th_n = tj_dot3_node1(r1m + 3, dv), th_b = tj_dot3_node1(r1m + 6, dv);
  const TJ<D> w_n = tj_dot3(n, d);
  const TJ<D> w_b = tj_dot3(b, d);
  // frozen stresses σ = ∂Π/∂q
  const real s_e = c.ke * eps;
  const real s_t = c.kt * th_t.v;
  const real s_wn = c.k3u * w_n.v + c.k3uv * th_b.v;
  const real s_b = c.k3uv * w_n.v + c.k3v * th_b.v;
  const real s_wb = c.k2u * w_b.v - c.k2uv * th_n.v;
  const real s_n = -c.k2uv * w_b.v + c.k2v * th_n.v;

  // ---- Gauss point positions: x = yᵤ d + (yₐ−yᵤ) m + yᵥ w + ½(u₁+u₂) + cₘ
  real d2h[3];
  for (int i = 0; i < 3; ++i) d2h[i] = 0.5 * dd2[i];
  const TJ<D> td = tj_dot3_time(t, d, dd1, d2h);  // t·d with d's time jet
  TJ<D> mv[3], wv[3];  // m = (t·d) t,  w = Δv × t
  for (int i = 0; i < 3; ++i) mv[i] = td * t[i];
  wv[0] = tj_fnma(dv[2], t[1], dv[1] * t[2]);
  wv[1] = tj_fnma(dv[0], t[2], dv[2] * t[0]);
  wv[2] = tj_fnma(dv[1], t[0], dv[0] * t[1]);

  // ---- loads per Gauss point (frozen) and their sums
  real fg[4][3];
  real r0[9];
  for (int k = 0; k < 9; ++k) r0[k] = rsm[k].v;
  real xd[4][3], xdd[4][3];  // Gauss point velocity / acceleration
  real vi21 = 0.0;
  TJ<D> vsm[3];
  const bool rotinertia = D && (c.iota1 != 0.0);
  for (int g = 0; g < 4; ++g) {
    for (int i = 0; i < 3; ++i) {
      fg[g][i] = 0.0;
      xd[g][i] = 0.0;
      xdd[g][i] = 0.0;
    }
    fg[g][2] = c.w;
    if (U)
      for (int i = 0; i < 3; ++i) fg[g][i] -= U[i];
  }
  if constexpr (D) {
    for (int g = 0; g < 4; ++g) {
      const real ya = c.ya[g], yu = c.yu[g], yv = c.yv[g];
      for (int i = 0; i < 3; ++i) {
        // x = yu d + (ya-yu) m + yv w + c: time coefficients
        const real c1 = 0.5 * (X1[i] + X1[6 + i]);
        const real c2 = 0.5 * (X2[i] + X2[6 + i]);
        xd[g][i] = yu * dd1[i] + (ya - yu) * mv[i].vt + yv * wv[i].vt + c1;
        xdd[g][i] = yu * dd2[i] + 2.0 * ((ya - yu) * mv[i].vtt + yv * wv[i].vtt) + c2;
      }
      real xl1[3], xl2[3];
      for (int k = 0; k < 3; ++k) {
        xl1[k] = r0[3 * k] * xd[g][0] + r0[3 * k + 1] * xd[g][1] + r0[3 * k + 2] * xd[g][2];
        xl2[k] = r0[3 * k] * xdd[g][0] + r0[3 * k + 1] * xdd[g][1] + r0[3 * k + 2] * xdd[g][2];
      }
      real fl[3];
      for (int k = 0; k < 3; ++k) {
        real fq = c.Cq[k] * xl1[k] * xl1[k];
        if (xl1[k] < 0.0) fq = -fq;
        fl[k] = c.Ca[k] * xl2[k] + c.Cl[k] * xl1[k] + fq;
      }
      for (int i = 0; i < 3; ++i)
        fg[g][i] += c.mu * xdd[g][i] + r0[i] * fl[0] + r0[i + 3] * fl[1] + r0[i + 6] * fl[2];
    }
    if (rotinertia) {
      // vᵢ₂ = spin⁻¹(ṙᵀṙ + rᵀr̈);  the ṙᵀṙ part is symmetric and drops out
      real ndd[3], bdd[3];
      for (int i = 0; i < 3; ++i) {
        ndd[i] = 2.0 * n[i].vtt;
        bdd[i] = 2.0 * b[i].vtt;
      }
      vi21 = 0.5 * (r0[6] * ndd[0] + r0[7] * ndd[1] + r0[8] * ndd[2] - (r0[3] * bdd[0] + r0[4] * bdd[1] + r0[5] * bdd[2]));
      // vₛₘ = Rodrigues⁻¹(rₛₘ) (static part only is used)
      rodrigues_inv(rsm, vsm);
    }
  }
  // sums over Gauss points (frozen loads)
  real Au[3] = {0, 0, 0}, Aa[3] = {0, 0, 0}, Av[3] = {0, 0, 0}, A0[3] = {0, 0, 0};
  for (int g = 0; g < 4; ++g)
    for (int i = 0; i < 3; ++i) {
      const real f = c.dL[g] * fg[g][i];
      Au[i] += c.yu[g] * f;
      Aa[i] += (c.ya[g] - c.yu[g]) * f;
      Av[i] += c.yv[g] * f;
      A0[i] += f;
    }
  real me[3] = {0, 0, 0};
  if (rotinertia)
    for (int i = 0; i < 3; ++i) me[i] = c.S0 * c.iota1 * vi21 * r0[i];

  // ---- Φ_v: scalar with frozen multipliers, Taylor in the rotation dofs
  TJ<D> Phi = tj_fma(w_b, s_wb, tj_fma(w_n, s_wn, tj_fma(th_b, s_b, tj_fma(th_n, s_n, th_t * s_t))));
  {
    const TJ<D> tAa = tj_dot3(t, Aa);
    const TJ<D> tdv = tj_dot3(t, d);
    Phi = tj_fma(tdv, tAa, Phi);
    Phi = tj_fma(wv[2], Av[2], tj_fma(wv[1], Av[1], tj_fma(wv[0], Av[0], Phi)));
    if (rotinertia) Phi = tj_fma(vsm[2], me[2], tj_fma(vsm[1], me[1], tj_fma(vsm[0], me[0], Phi)));
    // P = ∂Φ/∂d (value and rotation gradient)
    TJ<D> P[3];
    for (int i = 0; i < 3; ++i)
      P[i] = tj_fma(n[i], s_wn, tj_fma(b[i], s_wb, tAa * t[i])) + (s_e * 2.0 / c.L * dh[i] + Au[i]);
    // residual
    for (int i = 0; i < 3; ++i) {
      R[i] = to_d(-0.5 * P[i].v + 0.5 * A0[i]);
      R[6 + i] = to_d(0.5 * P[i].v + 0.5 * A0[i]);
      R[3 + i] = to_d(Phi.g[i]);
      R[9 + i] = to_d(Phi.g[3 + i]);
    }
    // ---- tangent: geometric part ∇²Φ (frozen loads), scaled by p0
    const real p0 = pt.p0;
    for (int k = 0; k < 144; ++k) K[k] = 0.0;
    // rot-rot
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        const int a = i < 3 ? 3 + i : 6 + i, bb = j < 3 ? 3 + j : 6 + j;
        K[a + 12 * bb] = to_d(p0 * Phi.h[i <= j ? hidx(i, j) : hidx(j, i)]);
      }
    // rot-trans:  ∂²/∂v_j∂u₁ = −½ ∂P/∂v_j,  ∂²/∂v_j∂u₂ = +½ ∂P/∂v_j
    for (int j = 0; j < 6; ++j) {
      const int a = j < 3 ? 3 + j : 6 + j;
      for (int k = 0; k < 3; ++k) {
        const real q = 0.5 * p0 * P[k].g[j];
        K[a + 12 * k] -= to_d(q);
        K[k + 12 * a] -= to_d(q);
        K[a + 12 * (6 + k)] += to_d(q);
        K[(6 + k) + 12 * a] += to_d(q);
      }
    }
  }
  // trans-trans: σε ∂²ε/∂d² with ∂d/∂u₁ = −½, ∂d/∂u₂ = ½
  {
    const real f = pt.p0 * s_e * (2.0 / c.L) / dn;
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) {
        const real h = f * ((k == l ? 1.0 : 0.0) - dh[k] * dh[l]) * 0.25;
        K[k + 12 * l] += to_d(h);
        K[(6 + k) + 12 * (6 + l)] += to_d(h);
        K[k + 12 * (6 + l)] -= to_d(h);
        K[(6 + k) + 12 * l] -= to_d(h);
      }
  }
  // ---- material part Gᵀ D G over q = (ε, θt, θn, θb, wn, wb).  Row 0 of G (ε)
  // is zero on the rotation dofs and rows 1-3 (θ) on the translation dofs, and
  // D is symmetric: the upper triangle is summed over the rows that are nonzero
  // at its row dof (3 at a translation dof, 5 at a rotation dof), p0 taken
  // into D G, and mirrored.
  {
    real G[6][12];
    for (int q = 0; q < 6; ++q)
      for (int j = 0; j < 12; ++j) G[q][j] = 0.0;
    for (int k = 0; k < 3; ++k) {
      G[0][k] = -dh[k] / c.L;
      G[0][6 + k] = dh[k] / c.L;
      G[4][k] = -0.5 * n[k].v;
      G[4][6 + k] = 0.5 * n[k].v;
      G[5][k] = -0.5 * b[k].v;
      G[5][6 + k] = 0.5 * b[k].v;
    }
    for (int j = 0; j < 6; ++j) {
      const int a = j < 3 ? 3 + j : 6 + j;
      G[1][a] = th_t.g[j];
      G[2][a] = th_n.g[j];
      G[3][a] = th_b.g[j];
      G[4][a] = w_n.g[j];
      G[5][a] = w_b.g[j];
    }
    const real p0 = pt.p0;
    real DG[6][12];
#pragma unroll
    for (int j = 0; j < 12; ++j) {
      const bool tr = j < 3 || (j >= 6 && j < 9);
      if (tr) {
        DG[0][j] = p0 * (c.ke * G[0][j]);
        DG[1][j] = 0.0;
        DG[2][j] = p0 * (-c.k2uv * G[5][j]);
        DG[3][j] = p0 * (c.k3uv * G[4][j]);
        DG[4][j] = p0 * (c.k3u * G[4][j]);
        DG[5][j] = p0 * (c.k2u * G[5][j]);
      } else {
        DG[0][j] = 0.0;
        DG[1][j] = p0 * (c.kt * G[1][j]);
        DG[2][j] = p0 * fma(c.k2v, G[2][j], -c.k2uv * G[5][j]);
        DG[3][j] = p0 * fma(c.k3v, G[3][j], c.k3uv * G[4][j]);
        DG[4][j] = p0 * fma(c.k3uv, G[3][j], c.k3u * G[4][j]);
        DG[5][j] = p0 * fma(-c.k2uv, G[2][j], c.k2u * G[5][j]);
      }
    }
#pragma unroll
    for (int i = 0; i < 12; ++i) {
      const bool tr = i < 3 || (i >= 6 && i < 9);
#pragma unroll
      for (int j = i; j < 12; ++j) {
        real v;
        if (tr)
          v = fma(G[0][i], DG[0][j], fma(G[4][i], DG[4][j], G[5][i] * DG[5][j]));
        else
          v = fma(G[1][i], DG[1][j],
                  fma(G[2][i], DG[2][j], fma(G[3][i], DG[3][j], fma(G[4][i], DG[4][j], G[5][i] * DG[5][j]))));
        K[i + 12 * j] += to_d(v);
        if (j != i) K[j + 12 * i] += to_d(v);
      }
    }
  }

  // ---- load variation (dynamic loads) and U-derivative
  const bool need_jx = D || (H != nullptr);
  if (!need_jx) return;
  // Jx_g: ∂x_g/∂X₀ (3x12):  rot: yu*0 + (ya-yu) m.g + yv w.g ; trans: s M_g + ½ I
  // M_g = yu I + (ya-yu) t tᵀ
  const real tv[3] = {t[0].v, t[1].v, t[2].v};
  if (H) {
    for (int k = 0; k < 36; ++k) H[k] = 0.0;
  }
  // accumulate per Gauss point
  for (int g = 0; g < 4; ++g) {
    const real ya = c.ya[g], yu = c.yu[g], yv = c.yv[g], yd = ya - yu, wq = c.dL[g];
    real Jx[3][12];
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 6; ++j) {
        const int a = j < 3 ? 3 + j : 6 + j;
        Jx[i][a] = yd * mv[i].g[j] + yv * wv[i].g[j];
      }
      for (int k = 0; k < 3; ++k) {
        const real M = (i == k ? yu : 0.0) + yd * tv[i] * tv[k];
        Jx[i][k] = -0.5 * M + (i == k ? 0.5 : 0.0);
        Jx[i][6 + k] = 0.5 * M + (i == k ? 0.5 : 0.0);
      }
    }
    if (H) {
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 12; ++a) H[a + 12 * k] -= to_d(wq * Jx[k][a]);
    }
    if constexpr (D) {
      // derivatives of load with respect to x-dot, x-ddot and r₀ (local frame)
      real xl1[3];
      for (int k = 0; k < 3; ++k) xl1[k] = r0[3 * k] * xd[g][0] + r0[3 * k + 1] * xd[g][1] + r0[3 * k + 2] * xd[g][2];
      real xl2[3];
      for (int k = 0; k < 3; ++k)
        xl2[k] = r0[3 * k] * xdd[g][0] + r0[3 * k + 1] * xdd[g][1] + r0[3 * k + 2] * xdd[g][2];
      real fl[3], dfl1[3];
      for (int k = 0; k < 3; ++k) {
        real fq = c.Cq[k] * xl1[k] * xl1[k];
        if (xl1[k] < 0.0) fq = -fq;
        fl[k] = c.Ca[k] * xl2[k] + c.Cl[k] * xl1[k] + fq;
        dfl1[k] = c.Cl[k] + 2.0 * c.Cq[k] * fabs(xl1[k]);
      }
      // Ṁ, M̈ for translation columns
      real td1[3], td2[3];
      for (int i = 0; i < 3; ++i) {
        td1[i] = t[i].vt;
        td2[i] = 2.0 * t[i].vtt;
      }
      // direction loop (12 Newton directions, plus δr)
      const int ndir = rdir ? 13 : 12;
      for (int j = 0; j < ndir; ++j) {
        real dx1[3], dx2[3], dr0[9];
        for (int k = 0; k < 9; ++k) dr0[k] = 0.0;
        if (j < 12) {
          const int e = rot_index(j);
          if (e >= 0) {
            for (int i = 0; i < 3; ++i) {
              const real gx = yd * mv[i].g[e] + yv * wv[i].g[e];
              const real gtx = yd * mv[i].gt[e] + yv * wv[i].gt[e];
              const real gttx = yd * mv[i].gtt[e] + yv * wv[i].gtt[e];
              dx1[i] = gtx * pt.p0 + gx * pt.p1;
              dx2[i] = 2.0 * gttx * pt.p0 + 2.0 * gtx * pt.p1 + gx * pt.p2;
            }
            for (int k = 0; k < 9; ++k) dr0[k] = rsm[k].g[e] * pt.p0;
          } else {
            const int k = j < 3 ? j : j - 6;
            const real s = j < 3 ? -0.5 : 0.5;
            for (int i = 0; i < 3; ++i) {
              const real M = (i == k ? yu : 0.0) + yd * tv[i] * tv[k];
              const real M1 = yd * (td1[i] * tv[k] + tv[i] * td1[k]);
              const real M2 = yd * (td2[i] * tv[k] + 2.0 * td1[i] * td1[k] + tv[i] * td2[k]);
              const real I = (i == k ? 0.5 : 0.0);
              dx1[i] = s * (M1 * pt.p0 + M * pt.p1) + I * pt.p1;
              dx2[i] = s * (M2 * pt.p0 + 2.0 * M1 * pt.p1 + M * pt.p2) + I * pt.p2;
            }
          }
        } else {
          // δr: X₁ += a δr, X₂ += b δr
          for (int i = 0; i < 3; ++i) {
            dx1[i] = 0.0;
            dx2[i] = 0.0;
          }
          for (int jj = 0; jj < 12; ++jj) {
            const int e = rot_index(jj);
            for (int i = 0; i < 3; ++i) {
              real gx, gtx;
              if (e >= 0) {
                gx = yd * mv[i].g[e] + yv * wv[i].g[e];
                gtx = yd * mv[i].gt[e] + yv * wv[i].gt[e];
              } else {
                const int k = jj < 3 ? jj : jj - 6;
                const real s = jj < 3 ? -0.5 : 0.5;
                const real M = (i == k ? yu : 0.0) + yd * tv[i] * tv[k];
                const real M1 = yd * (td1[i] * tv[k] + tv[i] * td1[k]);
                gx = s * M + (i == k ? 0.5 : 0.0);
                gtx = s * M1;
              }
              dx1[i] += gx * av[jj];
              dx2[i] += 2.0 * gtx * av[jj] + gx * bv[jj];
            }
          }
        }
        // δ(local components):  δ(r₀ᵀy) = δr₀ᵀ y + r₀ᵀ δy  (δr₀ = 0 along the
        // translation directions and δr)
        const bool rotdir = j < 12 && rot_index(j) >= 0;
        real dl1[3], dl2[3];
        for (int k = 0; k < 3; ++k) {
          dl1[k] = r0[3 * k] * dx1[0] + r0[3 * k + 1] * dx1[1] + r0[3 * k + 2] * dx1[2];
          dl2[k] = r0[3 * k] * dx2[0] + r0[3 * k + 1] * dx2[1] + r0[3 * k + 2] * dx2[2];
          if (rotdir) {
            dl1[k] += dr0[3 * k] * xd[g][0] + dr0[3 * k + 1] * xd[g][1] + dr0[3 * k + 2] * xd[g][2];
            dl2[k] += dr0[3 * k] * xdd[g][0] + dr0[3 * k + 1] * xdd[g][1] + dr0[3 * k + 2] * xdd[g][2];
          }
        }
        real dfl[3];
        for (int k = 0; k < 3; ++k) dfl[k] = c.Ca[k] * dl2[k] + dfl1[k] * dl1[k];
        real df[3];
        for (int i = 0; i < 3; ++i) {
          df[i] = c.mu * dx2[i] + r0[i] * dfl[0] + r0[i + 3] * dfl[1] + r0[i + 6] * dfl[2];
          if (rotdir) df[i] += dr0[i] * fl[0] + dr0[i + 3] * fl[1] + dr0[i + 6] * fl[2];
        }
        double* col = (j < 12) ? (K + 12 * j) : rdir;
        if (j == 12 && g == 0)
          for (int a = 0; a < 12; ++a) rdir[a] = 0.0;
        const real w0 = wq * df[0], w1 = wq * df[1], w2 = wq * df[2];
        for (int a = 0; a < 12; ++a) col[a] = to_d(fma(Jx[2][a], w2, fma(Jx[1][a], w1, fma(Jx[0][a], w0, real(col[a])))));
      }
    }
  }
  if constexpr (D) {
    if (rdir == nullptr && false) return;
    if (rotinertia) {
      // rotational inertia: S0 vₛₘ∂X₀ᵀ δmₑ,  mₑ = ι₁ vᵢ₂[1] t
      const int ndir = rdir ? 13 : 12;
      for (int j = 0; j < ndir; ++j) {
        real dvi = 0.0, dt[3] = {0, 0, 0};
        if (j < 12) {
          const int e = rot_index(j);
          if (e < 0) continue;
          for (int i = 0; i < 3; ++i) {
            const real dn_ = n[i].g[e] * pt.p0, db_ = b[i].g[e] * pt.p0;
            const real dndd = 2.0 * n[i].gtt[e] * pt.p0 + 2.0 * n[i].gt[e] * pt.p1 + n[i].g[e] * pt.p2;
            const real dbdd = 2.0 * b[i].gtt[e] * pt.p0 + 2.0 * b[i].gt[e] * pt.p1 + b[i].g[e] * pt.p2;
            dvi += 0.5 * (db_ * 2.0 * n[i].vtt + r0[6 + i] * dndd - dn_ * 2.0 * b[i].vtt - r0[3 + i] * dbdd);
            dt[i] = t[i].g[e] * pt.p0;
          }
        } else {
          for (int jj = 0; jj < 12; ++jj) {
            const int e = rot_index(jj);
            if (e < 0) continue;
            for (int i = 0; i < 3; ++i) {
              const real dndd = 2.0 * n[i].gt[e] * av[jj] + n[i].g[e] * bv[jj];
              const real dbdd = 2.0 * b[i].gt[e] * av[jj] + b[i].g[e] * bv[jj];
              dvi += 0.5 * (r0[6 + i] * dndd - r0[3 + i] * dbdd);
            }
          }
        }
        real dme[3];
        for (int i = 0; i < 3; ++i) dme[i] = c.S0 * c.iota1 * (dvi * r0[i] + vi21 * dt[i]);
        double* col = (j < 12) ? (K + 12 * j) : rdir;
        for (int a2 = 0; a2 < 6; ++a2) {
          const int a = a2 < 3 ? 3 + a2 : 6 + a2;
          col[a] += to_d(vsm[0].g[a2] * dme[0] + vsm[1].g[a2] * dme[1] + vsm[2].g[a2] * dme[2]);
        }
      }
    }
  }
}

// ---- element results of one beam at a state (getresult of the residual's
// requestable values, toolbox/BeamElement.jl:151-189): the element record's
// 69 fields f, the dofs X0[12], the EI scale a (1 without an A-dof); out[50]:
// ε, rₛₘ (9, column-major), then per Gauss point x (3), κ (3), fᵢ = EA ε and
// mᵢ = (GJ κ₁, a EI₃ κ₂, a EI₂ κ₃).  The rotation core is the element's own
// (static jets; only the values are used), the rest follows kinematics
// (:177-189): uₗ₂ = rₛₘᵀ d − L/2 e₁ and vₗ₂ = rₛₘᵀΔv.
MG_HD void beam_results(const double* f, const double* X0, double a, double* out) {
  const double* rm = f + 3;
  const double* cm = f;
  const double* zgp = f + 12;
  const double* tgm = f + 18;
  const double* tge = f + 21;
  const double* ya = f + 24;
  const double* yu = f + 28;
  const double* yv = f + 32;
  const double* ka = f + 36;
  const double* ku = f + 40;
  const double* kv = f + 44;
  const double L = f[48];
  const double EA = f[53], EI2 = a * f[54], EI3 = a * f[55], GJ = f[56];
  TJ<false, 3> r1[9];
  TJ<false> dv[3], rsm[9];
  {
    TJ<false, 3> r2[9];
    TJ<false> Q[9];
    const double zero[3] = {0.0, 0.0, 0.0};
    rodrigues_nodal<false>(X0 + 3, zero, zero, r1);
    rodrigues_nodal<false>(X0 + 9, zero, zero, r2);
    mul_abt_nodes(r2, r1, Q);
    rodrigues_inv(Q, dv, 0.5);
  }
  {
    double rmc[9];
    for (int k = 0; k < 9; ++k) rmc[k] = rm[k];
    TJ<false, 3> r1m[9];
    mul_ac(r1, rmc, r1m);
    TJ<false> rD[9];
    rodrigues(dv, rD);
    mul_ab_node1(rD, r1m, rsm);
  }
  double r[9], d[3], cs[3], ul2[3], vl2[3];
  for (int k = 0; k < 9; ++k) r[k] = rsm[k].v;
  for (int i = 0; i < 3; ++i) {
    d[i] = 0.5 * (X0[6 + i] - X0[i]) + 0.5 * tgm[i];
    cs[i] = 0.5 * (X0[i] + X0[6 + i]) + cm[i];
  }
  for (int k = 0; k < 3; ++k) {
    ul2[k] = r[3 * k] * d[0] + r[3 * k + 1] * d[1] + r[3 * k + 2] * d[2];
    vl2[k] = r[3 * k] * dv[0].v + r[3 * k + 1] * dv[1].v + r[3 * k + 2] * dv[2].v;
  }
  ul2[0] -= 0.5 * L;
  const double eps = sqrt((ul2[0] + 0.5 * L) * (ul2[0] + 0.5 * L) + ul2[1] * ul2[1] + ul2[2] * ul2[2]) * 2.0 / L - 1.0;
  out[0] = eps;
  for (int k = 0; k < 9; ++k) out[1 + k] = r[k];
  for (int g = 0; g < 4; ++g) {
    double* o = out + 10 + 10 * g;
    const double k0 = ka[g] * vl2[0];
    const double k1 = ku[g] * ul2[1] + kv[g] * vl2[2];
    const double k2 = ku[g] * ul2[2] - kv[g] * vl2[1];
    const double y[3] = {ya[g] * ul2[0], yu[g] * ul2[1] + yv[g] * vl2[2], yu[g] * ul2[2] - yv[g] * vl2[1]};
    double pp[3];
    for (int i = 0; i < 3; ++i) pp[i] = tge[i] * zgp[g] + y[i];
    for (int i = 0; i < 3; ++i) o[i] = r[i] * pp[0] + r[i + 3] * pp[1] + r[i + 6] * pp[2] + cs[i];
    o[3] = k0;
    o[4] = k1;
    o[5] = k2;
    o[6] = EA * eps;
    o[7] = GJ * k0;
    o[8] = EI3 * k1;
    o[9] = EI2 * k2;
  }
}

}  // namespace mgpu
