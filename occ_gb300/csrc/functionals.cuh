// Device exchange-correlation functionals (unpolarised), evaluated per grid
// point in FP64.  These are the Libxc 6.2.2 functionals OCC's methods use
// (share/methods/dft_methods.json via src/dft/functional.cpp:18-65), restated
// from the published papers:
//   Slater (Dirac 1930); VWN, CA and RPA fits (Vosko-Wilk-Nusair 1980);
//   B88 (Becke 1988); LYP in the Miehlich-Savin-Stoll-Preuss (1989)
//   gradient form; PBE exchange and correlation (Perdew-Burke-Ernzerhof 1996)
//   with the PW92 LDA in the digits Libxc uses inside PBE.
// For an unpolarised density Libxc's lda_c_vwn_3 reduces to the VWN
// paramagnetic Ceperley-Alder fit, the same as lda_c_vwn.
// Derivatives come from forward-mode dual numbers (value, d/drho, d/dsigma),
// so vrho and vsigma are the exact derivatives of the energy density.
#pragma once
#include <cuda_runtime.h>

namespace occx {

enum FuncId : int {
  kLdaX = 1,
  kLdaCVwn = 7,
  kLdaCVwnRpa = 8,
  kLdaCVwn3 = 30,
  kGgaXPbe = 101,
  kGgaXB88 = 106,
  kGgaCPbe = 130,
  kGgaCLyp = 131,
  kHybB3lyp = 402,
  kHybB3lyp5 = 475,
};

constexpr int kMaxFuncs = 8;
struct FuncSet {
  int n;
  int id[kMaxFuncs];
  double coef[kMaxFuncs];
};

__host__ __device__ inline bool func_is_gga(int id) {
  return id == kGgaXPbe || id == kGgaXB88 || id == kGgaCPbe || id == kGgaCLyp ||
         id == kHybB3lyp || id == kHybB3lyp5;
}
__host__ __device__ inline bool func_known(int id) {
  return id == kLdaX || id == kLdaCVwn || id == kLdaCVwnRpa || id == kLdaCVwn3 ||
         func_is_gga(id);
}

namespace fn {

struct D3 {
  double v, r, s;
};
__device__ __forceinline__ D3 mk(double v) { return {v, 0.0, 0.0}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.v + b.v, a.r + b.r, a.s + b.s}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.v - b.v, a.r - b.r, a.s - b.s}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
  return {a.v * b.v, fma(a.r, b.v, a.v * b.r), fma(a.s, b.v, a.v * b.s)};
}
__device__ __forceinline__ D3 operator/(D3 a, D3 b) {
  double iv = 1.0 / b.v, q = a.v * iv;
  return {q, (a.r - q * b.r) * iv, (a.s - q * b.s) * iv};
}
__device__ __forceinline__ D3 operator*(double c, D3 a) { return {c * a.v, c * a.r, c * a.s}; }
__device__ __forceinline__ D3 operator+(double c, D3 a) { return {c + a.v, a.r, a.s}; }
__device__ __forceinline__ D3 operator-(double c, D3 a) { return {c - a.v, -a.r, -a.s}; }
__device__ __forceinline__ D3 operator/(double c, D3 b) {
  double iv = 1.0 / b.v, q = c * iv;
  return {q, -q * b.r * iv, -q * b.s * iv};
}
__device__ __forceinline__ D3 neg(D3 a) { return {-a.v, -a.r, -a.s}; }
__device__ __forceinline__ D3 apply(D3 a, double f, double df) { return {f, df * a.r, df * a.s}; }
__device__ __forceinline__ D3 dlog(D3 a) { return apply(a, log(a.v), 1.0 / a.v); }
__device__ __forceinline__ D3 dexp(D3 a) {
  double e = exp(a.v);
  return apply(a, e, e);
}
__device__ __forceinline__ D3 dsqrt(D3 a) {
  double s = sqrt(a.v);
  return apply(a, s, 0.5 / s);
}
__device__ __forceinline__ D3 datan(D3 a) { return apply(a, atan(a.v), 1.0 / fma(a.v, a.v, 1.0)); }
__device__ __forceinline__ D3 dasinh(D3 a) { return apply(a, asinh(a.v), rsqrt(fma(a.v, a.v, 1.0))); }

constexpr double kPi = 3.14159265358979323846;

// rho^(1/3) and friends from one cube root
struct RhoPowers {
  D3 r13, r43, rm13; // rho^(1/3), rho^(4/3), rho^(-1/3)
};
__device__ __forceinline__ RhoPowers rho_powers(D3 rho) {
  double c = cbrt(rho.v);
  D3 r13 = apply(rho, c, c / (3.0 * rho.v));
  D3 r43 = rho * r13;
  D3 rm13 = apply(rho, 1.0 / c, -1.0 / (3.0 * c * rho.v));
  return {r13, r43, rm13};
}

__device__ __forceinline__ D3 slater(const RhoPowers &P) {
  const double cx = 0.7385587663820224; // (3/4)(3/pi)^(1/3)
  return -cx * P.r43;
}

__device__ __forceinline__ D3 vwn_eps(D3 rs, double A, double b, double c, double x0) {
  D3 x = dsqrt(rs);
  D3 X = x * x + b * x + mk(c);
  double X0 = x0 * x0 + b * x0 + c;
  double Q = sqrt(4.0 * c - b * b);
  D3 at = datan(mk(Q) / (2.0 * x + mk(b)));
  D3 t1 = dlog(x * x / X) + (2.0 * b / Q) * at;
  D3 xm = x - mk(x0);
  D3 t2 = dlog(xm * xm / X) + (2.0 * (b + 2.0 * x0) / Q) * at;
  return A * (t1 - (b * x0 / X0) * t2);
}

__device__ __forceinline__ D3 rs_of(const RhoPowers &P) {
  const double k = 0.6203504908994001; // (3/(4 pi))^(1/3)
  return k * P.rm13;
}

__device__ __forceinline__ D3 vwn5(D3 rho, const RhoPowers &P) {
  return rho * vwn_eps(rs_of(P), 0.0310907, 3.72744, 12.9352, -0.10498);
}
__device__ __forceinline__ D3 vwn_rpa(D3 rho, const RhoPowers &P) {
  return rho * vwn_eps(rs_of(P), 0.0310907, 13.0720, 42.7198, -0.409286);
}

__device__ __forceinline__ D3 b88(D3 rho, D3 sigma, const RhoPowers &P) {
  const double beta = 0.0042;
  const double cs = 0.9305257363491000; // (3/2)(3/(4 pi))^(1/3)
  // spin density rho/2: (rho/2)^(4/3) = rho^(4/3) / 2^(4/3)
  D3 r43s = 0.39685026299204984 * P.r43;
  D3 x2 = (0.25 * sigma) / (r43s * r43s);
  D3 x = dsqrt(x2);
  D3 per = neg(cs * r43s) - beta * r43s * x2 / (1.0 + 6.0 * beta * x * dasinh(x));
  return 2.0 * per;
}

__device__ __forceinline__ D3 lyp(D3 rho, D3 sigma, const RhoPowers &P) {
  const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
  const double cf = 2.8712340001881915; // (3/10)(3 pi^2)^(2/3)
  D3 den = 1.0 + d * P.rm13;
  D3 E = dexp(neg(c * P.rm13));
  D3 delta = c * P.rm13 + d * P.rm13 / den;
  D3 rm53 = P.rm13 / P.r43; // rho^(-5/3)
  D3 t1 = neg(a * rho / den);
  D3 t2 = neg((a * b * cf) * rho * E / den);
  D3 t3 = (a * b / 72.0) * (3.0 + 7.0 * delta) * sigma * rm53 * E / den;
  return t1 + t2 + t3;
}

__device__ __forceinline__ D3 kf2_of(const RhoPowers &P) {
  const double k = 3.0936677262801355; // (3 pi^2)^(1/3)
  D3 kf = k * P.r13;
  return kf * kf;
}

__device__ __forceinline__ D3 pbe_x(D3 rho, D3 sigma, const RhoPowers &P) {
  const double kappa = 0.8040, mu = 0.2195149727645171;
  D3 s2 = sigma / (4.0 * kf2_of(P) * rho * rho);
  D3 F = (1.0 + kappa) - kappa / (1.0 + (mu / kappa) * s2);
  return slater(P) * F;
}

__device__ __forceinline__ D3 pbe_c(D3 rho, D3 sigma, const RhoPowers &P) {
  const double beta = 0.06672455060314922;
  const double gamma = 0.031090690869654897; // (1 - ln 2) / pi^2
  const double A = 0.0310907, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382,
               b4 = 0.49294;
  D3 rs = rs_of(P);
  D3 srs = dsqrt(rs);
  D3 den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  D3 eps = (-2.0 * A) * (1.0 + a1 * rs) * dlog(1.0 + mk(1.0) / den);
  const double k = 3.0936677262801355;
  D3 kf = k * P.r13;
  D3 ks2 = (4.0 / kPi) * kf;
  D3 t2 = sigma / (4.0 * ks2 * rho * rho);
  D3 Af = (beta / gamma) / (dexp(neg(eps) / mk(gamma)) - mk(1.0));
  D3 At2 = Af * t2;
  D3 H = gamma * dlog(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return rho * (eps + H);
}

// Energy density of one component (before its mixture coefficient).
__device__ __forceinline__ D3 component(int id, D3 rho, D3 sigma, const RhoPowers &P) {
  switch (id) {
  case kLdaX:
    return slater(P);
  case kLdaCVwn:
  case kLdaCVwn3:
    return vwn5(rho, P);
  case kLdaCVwnRpa:
    return vwn_rpa(rho, P);
  case kGgaXPbe:
    return pbe_x(rho, sigma, P);
  case kGgaCPbe:
    return pbe_c(rho, sigma, P);
  case kGgaXB88:
    return b88(rho, sigma, P);
  case kGgaCLyp:
    return lyp(rho, sigma, P);
  case kHybB3lyp:
    return 0.08 * slater(P) + 0.72 * b88(rho, sigma, P) + 0.19 * vwn_rpa(rho, P) +
           0.81 * lyp(rho, sigma, P);
  case kHybB3lyp5:
    return 0.08 * slater(P) + 0.72 * b88(rho, sigma, P) + 0.19 * vwn5(rho, P) +
           0.81 * lyp(rho, sigma, P);
  }
  return mk(0.0);
}

} // namespace fn

// Sum of the method's components at one point: energy per volume e and its
// derivatives (vrho, vsigma).  Points below the density threshold give zero,
// as Libxc does.
__device__ __forceinline__ void eval_xc(const FuncSet &fs, double rho, double sigma, double &e,
                                        double &vrho, double &vsigma) {
  e = vrho = vsigma = 0.0;
  if (!(rho >= 1e-15))
    return;
  fn::D3 r{rho, 1.0, 0.0};
  fn::D3 s{fmax(sigma, 1e-40), 0.0, 1.0};
  fn::RhoPowers P = fn::rho_powers(r);
  for (int i = 0; i < fs.n; i++) {
    fn::D3 c = fn::component(fs.id[i], r, s, P);
    e += fs.coef[i] * c.v;
    vrho += fs.coef[i] * c.r;
    vsigma += fs.coef[i] * c.s;
  }
}

} // namespace occx
