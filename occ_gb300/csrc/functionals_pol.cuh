// Spin-polarised exchange-correlation functionals for the unrestricted (UKS)
// build, per grid point: the polarised forms of the Libxc 6.2.2 functionals
// OCC's methods name (m_method.functionals_polarized,
// include/occ/dft/dft.h:207-209; evaluated through src/dft/functional.cpp:
// 18-65 with rho = (rho_a, rho_b), sigma = (s_aa, s_ab, s_bb)), restated from
// the published papers:
//   Slater, B88, PBE exchange: the exact spin scaling
//     E_x[rho_a, rho_b] = (E_x[2 rho_a] + E_x[2 rho_b]) / 2;
//   VWN (Vosko, Wilk, Nusair, Can. J. Phys. 58, 1200 (1980)):
//     eps = eps_P + alpha_c f(z) / f''(0) (1 - z^4) + (eps_F - eps_P) f(z) z^4
//     with the Ceperley-Alder (VWN5) or RPA fits of eps_P, eps_F, alpha_c;
//     VWN3 scales the RPA spin interpolation by (eps_F - eps_P)_CA /
//     (eps_F - eps_P)_RPA;
//   PW92 (Perdew, Wang, PRB 45, 13244 (1992)) the same interpolation with its
//     three G(rs) fits (alpha_c = -G), inside PBE correlation with
//     phi(z) = ((1 + z)^(2/3) + (1 - z)^(2/3)) / 2;
//   LYP in the form of Miehlich, Savin, Stoll, Preuss, CPL 157, 200 (1989),
//     eq. 2.
// Derivatives by forward-mode dual numbers over (rho_a, rho_b, s_aa, s_ab,
// s_bb): PD<double> (FP64 value and derivatives) for the FP64 build, PD<float>
// (FP64 value, FP32 derivatives) for the tensor-core build, whose V_xc
// tolerance FP32 derivatives meet.  Thresholds (not pinned against Libxc):
// the point is zero below a total density of 1e-15; a spin channel's exchange
// is zero below 1e-15; 1 +- zeta is kept >= 2.2e-16 (DBL_EPSILON, Libxc's
// zeta threshold).
#pragma once
#include <cuda_runtime.h>

#include "functionals.cuh"

namespace occx {
namespace fnp {

constexpr int kNd = 5; // d/d rho_a, rho_b, s_aa, s_ab, s_bb

// value (FP64) and the five derivatives in D (double or float); the casts
// below are no-ops for D = double, which is the FP64 path's arithmetic
template <class D> struct PD {
  double v;
  D d[kNd];
};
using P5 = PD<double>;

template <class D> __device__ __forceinline__ PD<D> cst(double v) {
  PD<D> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = D(0);
  return r;
}
template <class D> __device__ __forceinline__ PD<D> var(double v, int k) {
  PD<D> r = cst<D>(v);
  r.d[k] = D(1);
  return r;
}
template <class D> __device__ __forceinline__ PD<D> operator+(PD<D> a, PD<D> b) {
  PD<D> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <class D> __device__ __forceinline__ PD<D> operator-(PD<D> a, PD<D> b) {
  PD<D> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <class D> __device__ __forceinline__ PD<D> operator*(PD<D> a, PD<D> b) {
  PD<D> r;
  r.v = a.v * b.v;
  const D av = static_cast<D>(a.v), bv = static_cast<D>(b.v);
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = fma(a.d[i], bv, av * b.d[i]);
  return r;
}
template <class D> __device__ __forceinline__ PD<D> operator/(PD<D> a, PD<D> b) {
  const double iv = 1.0 / b.v, q = a.v * iv;
  PD<D> r;
  r.v = q;
  const D qd = static_cast<D>(q), ivd = static_cast<D>(iv);
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = (a.d[i] - qd * b.d[i]) * ivd;
  return r;
}
template <class D> __device__ __forceinline__ PD<D> operator/(double c, PD<D> b) {
  const double iv = 1.0 / b.v, q = c * iv;
  PD<D> r;
  r.v = q;
  const D qd = static_cast<D>(q), ivd = static_cast<D>(iv);
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = -qd * b.d[i] * ivd;
  return r;
}
template <class D> __device__ __forceinline__ PD<D> operator*(double c, PD<D> a) {
  PD<D> r;
  r.v = c * a.v;
  const D cd = static_cast<D>(c);
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = cd * a.d[i];
  return r;
}
template <class D> __device__ __forceinline__ PD<D> operator+(double c, PD<D> a) {
  a.v += c;
  return a;
}
template <class D> __device__ __forceinline__ PD<D> operator-(double c, PD<D> a) {
  PD<D> r;
  r.v = c - a.v;
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = -a.d[i];
  return r;
}
template <class D> __device__ __forceinline__ PD<D> neg(PD<D> a) { return 0.0 - a; }
template <class D> __device__ __forceinline__ PD<D> chain(PD<D> a, double f, double df) {
  PD<D> r;
  r.v = f;
  const D dd = static_cast<D>(df);
#pragma unroll
  for (int i = 0; i < kNd; i++)
    r.d[i] = dd * a.d[i];
  return r;
}
template <class D> __device__ __forceinline__ PD<D> dlog(PD<D> a) {
  return chain(a, log(a.v), 1.0 / a.v);
}
template <class D> __device__ __forceinline__ PD<D> dexp(PD<D> a) {
  const double e = exp(a.v);
  return chain(a, e, e);
}
template <class D> __device__ __forceinline__ PD<D> dsqrt(PD<D> a) {
  const double s = sqrt(a.v);
  return chain(a, s, 0.5 / s);
}
template <class D> __device__ __forceinline__ PD<D> datan(PD<D> a) {
  return chain(a, atan(a.v), 1.0 / fma(a.v, a.v, 1.0));
}
template <class D> __device__ __forceinline__ PD<D> dasinh(PD<D> a) {
  return chain(a, asinh(a.v), rsqrt(fma(a.v, a.v, 1.0)));
}
// a^(k/3) from one cube root (k = 1, 2, 4, 8); zero with a zero derivative
// at a <= 0 (only reached for k >= 4, where that is the limit)
template <class D> __device__ __forceinline__ PD<D> dpow3(PD<D> a, int k) {
  if (!(a.v > 0.0))
    return cst<D>(0.0);
  const double c = cbrt(a.v);
  double ck = 1.0;
  for (int i = 0; i < k; i++)
    ck *= c;
  return chain(a, ck, (k / 3.0) * ck / a.v);
}
template <class D> __device__ __forceinline__ PD<D> dmax(PD<D> a, double lo) {
  return a.v >= lo ? a : cst<D>(lo);
}

constexpr double kPiP = 3.14159265358979323846;
constexpr double kFpp0 = 1.7099209341613657; // f''(0) = 4 / (9 (2^(1/3) - 1))

// f(z) = ((1 + z)^(4/3) + (1 - z)^(4/3) - 2) / (2^(4/3) - 2), with opz = 1 + z,
// omz = 1 - z already thresholded
template <class D> __device__ __forceinline__ PD<D> fzeta(PD<D> opz, PD<D> omz) {
  return (1.0 / 0.5198420997897464) * (dpow3(opz, 4) + dpow3(omz, 4) - cst<D>(2.0));
}

// VWN Pade form of one fit (the restricted vwn_eps)
template <class D>
__device__ __forceinline__ PD<D> vwn_fit(PD<D> rs, double A, double b, double c, double x0) {
  PD<D> x = dsqrt(rs);
  PD<D> X = x * x + b * x + cst<D>(c);
  const double X0 = x0 * x0 + b * x0 + c;
  const double Q = sqrt(4.0 * c - b * b);
  PD<D> at = datan(cst<D>(Q) / (2.0 * x + cst<D>(b)));
  PD<D> t1 = dlog(x * x / X) + (2.0 * b / Q) * at;
  PD<D> xm = x - cst<D>(x0);
  PD<D> t2 = dlog(xm * xm / X) + (2.0 * (b + 2.0 * x0) / Q) * at;
  return A * (t1 - (b * x0 / X0) * t2);
}

template <class D> struct Spin {
  PD<D> ra, rb, saa, sab, sbb, rho, rs, z, opz, omz;
};

template <class D>
__device__ __forceinline__ Spin<D> spin_vars(double ra, double rb, double saa, double sab,
                                             double sbb) {
  Spin<D> s;
  s.ra = var<D>(ra, 0);
  s.rb = var<D>(rb, 1);
  s.saa = var<D>(saa, 2);
  s.sab = var<D>(sab, 3);
  s.sbb = var<D>(sbb, 4);
  s.rho = s.ra + s.rb;
  s.rs = 0.6203504908994001 / dpow3(s.rho, 1); // (3 / (4 pi rho))^(1/3)
  s.z = (s.ra - s.rb) / s.rho;
  s.opz = dmax(1.0 + s.z, 2.220446049250313e-16);
  s.omz = dmax(1.0 - s.z, 2.220446049250313e-16);
  return s;
}

// Slater exchange of one spin channel, -cx 2^(1/3) rho_s^(4/3)
template <class D> __device__ __forceinline__ PD<D> slater_s(PD<D> rs) {
  return (-0.7385587663820224 * 1.2599210498948732) * dpow3(rs, 4);
}
// B88 of one spin channel (rho_s, sigma_ss)
template <class D> __device__ __forceinline__ PD<D> b88_s(PD<D> r, PD<D> s) {
  const double beta = 0.0042, cs = 0.9305257363491000;
  PD<D> r43 = dpow3(r, 4);
  PD<D> x2 = s / (r43 * r43);
  PD<D> x = dsqrt(x2);
  return neg(cs * r43) - beta * r43 * x2 / (1.0 + 6.0 * beta * x * dasinh(x));
}
// PBE exchange of one spin channel: E_x^PBE[2 rho_s, 4 sigma_ss] / 2
template <class D> __device__ __forceinline__ PD<D> pbe_x_s(PD<D> r, PD<D> s) {
  const double kappa = 0.8040, mu = 0.2195149727645171;
  PD<D> n = 2.0 * r;
  PD<D> kf = 3.0936677262801355 * dpow3(n, 1);
  PD<D> s2 = (4.0 * s) / (4.0 * kf * kf * n * n);
  PD<D> F = (1.0 + kappa) - kappa / (1.0 + (mu / kappa) * s2);
  return 0.5 * ((-0.7385587663820224) * dpow3(n, 4) * F);
}

// VWN energy per particle for the parameter sets of one variant
// (P, F, alpha rows of A, b, c, x0); rpa3: the VWN3 form
template <class D> __device__ __forceinline__ PD<D> vwn_pol_eps(const Spin<D> &S, int variant) {
  // Ceperley-Alder (VWN5) and RPA fits: paramagnetic, ferromagnetic, alpha_c
  const double A[3] = {0.0310907, 0.01554535, -1.0 / (6.0 * kPiP * kPiP)};
  const double bc[3] = {3.72744, 7.06042, 1.13107}, cc[3] = {12.9352, 18.0578, 13.0045},
               xc[3] = {-0.10498, -0.32500, -0.0047584};
  const double br[3] = {13.0720, 20.1231, 1.06835}, cr[3] = {42.7198, 101.578, 11.4813},
               xr[3] = {-0.409286, -0.743294, -0.228344};
  PD<D> f = fzeta(S.opz, S.omz);
  PD<D> z2 = S.z * S.z, z4 = z2 * z2;
  if (variant == 0 || variant == 1) { // 0: VWN5 (CA), 1: RPA
    const double *b = variant == 0 ? bc : br, *c = variant == 0 ? cc : cr,
                 *x0 = variant == 0 ? xc : xr;
    PD<D> eP = vwn_fit(S.rs, A[0], b[0], c[0], x0[0]);
    PD<D> eF = vwn_fit(S.rs, A[1], b[1], c[1], x0[1]);
    PD<D> ac = vwn_fit(S.rs, A[2], b[2], c[2], x0[2]);
    return eP + (1.0 / kFpp0) * ac * f * (1.0 - z4) + (eF - eP) * f * z4;
  }
  // VWN3: CA paramagnetic, RPA spin stiffness scaled by the CA / RPA
  // polarisation energies
  PD<D> eP = vwn_fit(S.rs, A[0], bc[0], cc[0], xc[0]);
  PD<D> dCA = vwn_fit(S.rs, A[1], bc[1], cc[1], xc[1]) - eP;
  PD<D> dRPA =
      vwn_fit(S.rs, A[1], br[1], cr[1], xr[1]) - vwn_fit(S.rs, A[0], br[0], cr[0], xr[0]);
  PD<D> ar = vwn_fit(S.rs, A[2], br[2], cr[2], xr[2]);
  return eP + (1.0 / kFpp0) * ar * f * (1.0 - z4) * dCA / dRPA + dCA * f * z4;
}

// PW92 G(rs) of one fit
template <class D>
__device__ __forceinline__ PD<D> pw_g(PD<D> rs, double A, double a1, double b1, double b2,
                                      double b3, double b4) {
  PD<D> srs = dsqrt(rs);
  PD<D> den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return (-2.0 * A) * (1.0 + a1 * rs) * dlog(1.0 + cst<D>(1.0) / den);
}
template <class D> __device__ __forceinline__ PD<D> pw92_pol_eps(const Spin<D> &S) {
  PD<D> e0 = pw_g(S.rs, 0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294);
  PD<D> e1 = pw_g(S.rs, 0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517);
  PD<D> ac = neg(pw_g(S.rs, 0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671));
  PD<D> f = fzeta(S.opz, S.omz);
  PD<D> z2 = S.z * S.z, z4 = z2 * z2;
  return e0 + (1.0 / kFpp0) * ac * f * (1.0 - z4) + (e1 - e0) * f * z4;
}
template <class D> __device__ __forceinline__ PD<D> pbe_c_pol(const Spin<D> &S) {
  const double beta = 0.06672455060314922, gamma = 0.031090690869654897;
  PD<D> eps = pw92_pol_eps(S);
  PD<D> phi = 0.5 * (dpow3(S.opz, 2) + dpow3(S.omz, 2));
  PD<D> phi3 = phi * phi * phi;
  PD<D> kf = 3.0936677262801355 * dpow3(S.rho, 1);
  PD<D> ks2 = (4.0 / kPiP) * kf;
  PD<D> sig = S.saa + 2.0 * S.sab + S.sbb;
  PD<D> t2 = sig / (4.0 * phi * phi * ks2 * S.rho * S.rho);
  PD<D> Af = (beta / gamma) / (dexp(neg(eps) / (gamma * phi3)) - cst<D>(1.0));
  PD<D> At2 = Af * t2;
  PD<D> H =
      gamma * phi3 * dlog(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return S.rho * (eps + H);
}
template <class D> __device__ __forceinline__ PD<D> lyp_pol(const Spin<D> &S) {
  const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
  const double cf = 2.8712340001881915; // (3/10)(3 pi^2)^(2/3)
  PD<D> rm13 = cst<D>(1.0) / dpow3(S.rho, 1);
  PD<D> den = 1.0 + d * rm13;
  PD<D> rm113 = cst<D>(1.0) / (dpow3(S.rho, 8) * S.rho); // rho^(-11/3)
  PD<D> omega = dexp(neg(c * rm13)) / den * rm113;
  PD<D> delta = c * rm13 + d * rm13 / den;
  PD<D> gg = S.saa + 2.0 * S.sab + S.sbb; // |grad rho|^2
  PD<D> rarb = S.ra * S.rb;
  PD<D> r2 = S.rho * S.rho;
  PD<D> t1 = neg(4.0 * a * rarb / (den * S.rho));
  PD<D> br = (12.699208415745595 * cf) * (dpow3(S.ra, 8) + dpow3(S.rb, 8)) + // 2^(11/3) C_F
             (47.0 / 18.0 - (7.0 / 18.0) * delta) * gg -
             (2.5 - (1.0 / 18.0) * delta) * (S.saa + S.sbb) -
             ((1.0 / 9.0) * (delta - cst<D>(11.0))) * (S.ra / S.rho * S.saa + S.rb / S.rho * S.sbb);
  PD<D> rest = neg((2.0 / 3.0) * r2 * gg) + ((2.0 / 3.0) * r2 - S.ra * S.ra) * S.sbb +
               ((2.0 / 3.0) * r2 - S.rb * S.rb) * S.saa;
  return t1 - (a * b) * omega * (rarb * br + rest);
}

} // namespace fnp

// One point of a polarised method in dual type PD<D>: the sum of the
// components (zero below the density threshold).
template <class D>
__device__ __forceinline__ fnp::PD<D> eval_pol_sum(const FuncSet &fs, double ra, double rb,
                                                   double saa, double sab, double sbb) {
  using namespace fnp;
  PD<D> tot = cst<D>(0.0);
  if (!(ra + rb >= 1e-15))
    return tot;
  const Spin<D> S = spin_vars<D>(ra, rb, saa, sab, sbb);
  const bool sa = ra >= 1e-15, sb = rb >= 1e-15;
  for (int i = 0; i < fs.n; i++) {
    PD<D> c = cst<D>(0.0);
    auto slater = [&] {
      PD<D> x = cst<D>(0.0);
      if (sa)
        x = x + slater_s(S.ra);
      if (sb)
        x = x + slater_s(S.rb);
      return x;
    };
    auto b88 = [&] {
      PD<D> x = cst<D>(0.0);
      if (sa)
        x = x + b88_s(S.ra, S.saa);
      if (sb)
        x = x + b88_s(S.rb, S.sbb);
      return x;
    };
    auto vwn = [&](int variant) { return S.rho * vwn_pol_eps(S, variant); };
    switch (fs.id[i]) {
    case kLdaX: c = slater(); break;
    case kLdaCVwn: c = vwn(0); break;
    case kLdaCVwnRpa: c = vwn(1); break;
    case kLdaCVwn3: c = vwn(2); break;
    case kGgaXPbe: {
      PD<D> x = cst<D>(0.0);
      if (sa)
        x = x + pbe_x_s(S.ra, S.saa);
      if (sb)
        x = x + pbe_x_s(S.rb, S.sbb);
      c = x;
      break;
    }
    case kGgaCPbe: c = pbe_c_pol(S); break;
    case kGgaXB88: c = b88(); break;
    case kGgaCLyp: c = lyp_pol(S); break;
    case kHybB3lyp:
      c = 0.08 * slater() + 0.72 * b88() + 0.19 * vwn(1) + 0.81 * lyp_pol(S);
      break;
    case kHybB3lyp5:
      c = 0.08 * slater() + 0.72 * b88() + 0.19 * vwn(0) + 0.81 * lyp_pol(S);
      break;
    case kHybPbeh: {
      PD<D> x = cst<D>(0.0);
      if (sa)
        x = x + pbe_x_s(S.ra, S.saa);
      if (sb)
        x = x + pbe_x_s(S.rb, S.sbb);
      c = 0.75 * x + pbe_c_pol(S);
      break;
    }
    case kHybBhandh: c = 0.5 * slater() + lyp_pol(S); break;
    case kHybBhandhlyp: c = 0.5 * b88() + lyp_pol(S); break;
    default: break; // meta-GGA components: eval_xc_mgga_pol
    }
    tot = tot + fs.coef[i] * c;
  }
  return tot;
}

// One point of a polarised method: energy per volume e and vrho[2],
// vsigma[3] (zero below the density threshold), FP64.
__device__ __forceinline__ void eval_xc_pol(const FuncSet &fs, double ra, double rb, double saa,
                                            double sab, double sbb, double &e, double *vrho,
                                            double *vsig) {
  ra = fmax(ra, 0.0);
  rb = fmax(rb, 0.0);
  saa = fmax(saa, 1e-40);
  sbb = fmax(sbb, 1e-40);
  const fnp::P5 t = eval_pol_sum<double>(fs, ra, rb, saa, sab, sbb);
  e = t.v;
  vrho[0] = t.d[0];
  vrho[1] = t.d[1];
  vsig[0] = t.d[2];
  vsig[1] = t.d[3];
  vsig[2] = t.d[4];
}

static __device__ __noinline__ void eval_xc_pol_fp64_call(const FuncSet &fs, double ra,
                                                          double rb, double saa, double sab,
                                                          double sbb, double *out6) {
  eval_xc_pol(fs, ra, rb, saa, sab, sbb, out6[0], out6 + 1, out6 + 3);
}

// The tensor-core build's evaluator: FP64 values, FP32 derivatives where both
// spin densities are >= 1e-10 (so that powers of either stay inside the FP32
// range), the FP64 evaluator elsewhere and for any point whose result is not
// finite.
__device__ __forceinline__ void eval_xc_pol_mixed(const FuncSet &fs, double ra, double rb,
                                                  double saa, double sab, double sbb, double &e,
                                                  double *vrho, double *vsig) {
  if (!(ra >= 1e-10) || !(rb >= 1e-10)) {
    double o[6];
    eval_xc_pol_fp64_call(fs, ra, rb, saa, sab, sbb, o);
    e = o[0], vrho[0] = o[1], vrho[1] = o[2], vsig[0] = o[3], vsig[1] = o[4], vsig[2] = o[5];
    return;
  }
  const fnp::PD<float> t =
      eval_pol_sum<float>(fs, ra, rb, fmax(saa, 1e-40), sab, fmax(sbb, 1e-40));
  bool fin = isfinite(t.v);
#pragma unroll
  for (int i = 0; i < fnp::kNd; i++)
    fin = fin && isfinite(t.d[i]);
  if (!fin) { // an FP32 overflow
    double o[6];
    eval_xc_pol_fp64_call(fs, ra, rb, saa, sab, sbb, o);
    e = o[0], vrho[0] = o[1], vrho[1] = o[2], vsig[0] = o[3], vsig[1] = o[4], vsig[2] = o[5];
    return;
  }
  e = t.v;
  vrho[0] = t.d[0];
  vrho[1] = t.d[1];
  vsig[0] = t.d[2];
  vsig[1] = t.d[3];
  vsig[2] = t.d[4];
}

} // namespace occx
