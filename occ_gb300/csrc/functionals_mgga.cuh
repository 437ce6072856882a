// Meta-GGA functionals (unpolarised), FP64 per grid point: TPSS exchange and
// correlation, the Libxc 6.2.2 functionals mgga_x_tpss (id 202) and
// mgga_c_tpss (id 231) of OCC's "tpss" method (share/methods/dft_methods.json;
// evaluated through src/dft/functional.cpp:49-58 with rho, sigma, laplacian,
// tau), restated from J. Tao, J.P. Perdew, V.N. Staroverov, G.E. Scuseria,
// PRL 91, 146401 (2003):
//   exchange  e_x = -(3/4)(3/pi)^(1/3) rho^(4/3) F_x(p, z), eqs. 4-10, with
//             p = sigma / (4 (3 pi^2)^(2/3) rho^(8/3)), z = tau_W / tau,
//             alpha = (tau - tau_W) / tau_unif;
//   correlation (revPKZB, eqs. 11-14) for zeta = 0 (so C(0, 0) = 0.53):
//             eps = eps_PBE(rho, sigma) (1 + 0.53 z^2)
//                   - 1.53 z^2 max(eps_PBE(rho/2, 0; sigma/4), eps_PBE(rho, sigma)),
//             e_c = rho eps (1 + 2.8 eps z^3),
//   where eps_PBE(rho/2, 0; sigma/4) is PBE correlation of the fully
//   polarised density rho/2 (PW92 ferromagnetic fit, phi = phi(zeta = 1)).
// Neither reads the laplacian.  Derivatives by forward-mode dual numbers over
// (rho, sigma, tau).  Thresholds: as for the GGAs the point is zero below
// rho = 1e-15; tau >= 1e-20, sigma >= 1e-40, and sigma is clamped to
// 8 rho tau (z <= 1) before evaluation, as Libxc does for meta-GGAs.
#pragma once
#include <cuda_runtime.h>

#include "functionals.cuh"

namespace occx {

enum MggaId : int {
  kMggaXTpss = 202,
  kMggaCTpss = 231,
};

__host__ __device__ inline bool func_is_mgga(int id) {
  return id == kMggaXTpss || id == kMggaCTpss;
}

namespace fnm {

struct M3 { // value and d/drho, d/dsigma, d/dtau
  double v, r, s, t;
};
__device__ __forceinline__ M3 cst(double v) { return {v, 0.0, 0.0, 0.0}; }
__device__ __forceinline__ M3 operator+(M3 a, M3 b) {
  return {a.v + b.v, a.r + b.r, a.s + b.s, a.t + b.t};
}
__device__ __forceinline__ M3 operator-(M3 a, M3 b) {
  return {a.v - b.v, a.r - b.r, a.s - b.s, a.t - b.t};
}
__device__ __forceinline__ M3 operator*(M3 a, M3 b) {
  return {a.v * b.v, fma(a.r, b.v, a.v * b.r), fma(a.s, b.v, a.v * b.s),
          fma(a.t, b.v, a.v * b.t)};
}
__device__ __forceinline__ M3 operator/(M3 a, M3 b) {
  const double inv = 1.0 / b.v, q = a.v * inv;
  return {q, (a.r - q * b.r) * inv, (a.s - q * b.s) * inv, (a.t - q * b.t) * inv};
}
__device__ __forceinline__ M3 operator*(double c, M3 a) {
  return {c * a.v, c * a.r, c * a.s, c * a.t};
}
__device__ __forceinline__ M3 operator+(double c, M3 a) { return {c + a.v, a.r, a.s, a.t}; }
__device__ __forceinline__ M3 operator-(double c, M3 a) { return {c - a.v, -a.r, -a.s, -a.t}; }
__device__ __forceinline__ M3 operator/(double c, M3 b) {
  const double q = c / b.v, f = -q / b.v;
  return {q, f * b.r, f * b.s, f * b.t};
}
__device__ __forceinline__ M3 chain(M3 a, double f, double df) {
  return {f, df * a.r, df * a.s, df * a.t};
}
__device__ __forceinline__ M3 mlog(M3 a) { return chain(a, log(a.v), 1.0 / a.v); }
__device__ __forceinline__ M3 mexp(M3 a) {
  const double e = exp(a.v);
  return chain(a, e, e);
}
__device__ __forceinline__ M3 msqrt(M3 a) {
  const double s = sqrt(a.v);
  return chain(a, s, 0.5 / s);
}
__device__ __forceinline__ M3 mcbrt(M3 a) { // a > 0
  const double c = cbrt(a.v);
  return chain(a, c, c / (3.0 * a.v));
}
__device__ __forceinline__ M3 mmax(M3 a, M3 b) { return a.v >= b.v ? a : b; }

constexpr double kPiM = 3.14159265358979323846;
constexpr double kK2 = 9.570780000627305;     // (3 pi^2)^(2/3)
constexpr double kKf = 3.0936677262801355;    // (3 pi^2)^(1/3)
constexpr double kCx = 0.7385587663820224;    // (3/4)(3/pi)^(1/3)
constexpr double kRs = 0.6203504908994001;    // (3/(4 pi))^(1/3)
constexpr double kCbrt2 = 1.2599210498948732; // 2^(1/3)
// phi(zeta = 1) with 1 - zeta held at DBL_EPSILON: (2^(2/3) + eps^(2/3)) / 2
constexpr double kPhi1 = 0.79370052600243400;

struct Pow {
  M3 r13, r43, r53, r83;
};
__device__ __forceinline__ Pow powers(M3 rho) {
  Pow P;
  P.r13 = mcbrt(rho);
  P.r43 = rho * P.r13;
  P.r53 = P.r43 * P.r13;
  P.r83 = P.r53 * rho;
  return P;
}

__device__ __forceinline__ M3 tpss_x(M3 rho, M3 sigma, M3 tau, const Pow &P) {
  const double kappa = 0.804, b = 0.40, c = 1.59096, e = 1.537, mu = 0.21951;
  const double se = 1.2397580409095962; // sqrt(e)
  M3 p = sigma / ((4.0 * kK2) * P.r83);
  M3 tw = sigma / (8.0 * rho);
  M3 z = tw / tau;
  M3 alpha = (tau - tw) / ((0.3 * kK2) * P.r53);
  M3 am1 = alpha - cst(1.0);
  M3 qb = 0.45 * am1 / msqrt(1.0 + b * alpha * am1) + (2.0 / 3.0) * p;
  M3 z2 = z * z;
  M3 opz2 = 1.0 + z2;
  M3 tz2 = 0.36 * z2; // (3 z / 5)^2
  M3 p2 = p * p;
  M3 num = (cst(10.0 / 81.0) + c * z2 / (opz2 * opz2)) * p + (146.0 / 2025.0) * qb * qb -
           (73.0 / 405.0) * qb * msqrt(0.5 * tz2 + 0.5 * p2) +
           ((1.0 / kappa) * (10.0 / 81.0) * (10.0 / 81.0)) * p2 +
           (2.0 * se * (10.0 / 81.0)) * tz2 + (e * mu) * p2 * p;
  M3 den = 1.0 + se * p;
  M3 x = num / (den * den);
  M3 Fx = (1.0 + kappa) - kappa / (1.0 + (1.0 / kappa) * x);
  return (-kCx) * P.r43 * Fx;
}

// PW92 G(rs) of one fit
__device__ __forceinline__ M3 pw_g(M3 rs, double A, double a1, double b1, double b2, double b3,
                                   double b4) {
  M3 srs = msqrt(rs);
  M3 den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return (-2.0 * A) * (1.0 + a1 * rs) * mlog(1.0 + 1.0 / den);
}

// PBE correlation per particle given the LDA part eps, the spin factor phi
// (phi^3 = phi3), k_F and n, and |grad n|^2
__device__ __forceinline__ M3 pbe_h(M3 eps, double phi, M3 kf, M3 n, M3 sig) {
  const double beta = 0.06672455060314922, gamma = 0.031090690869654897;
  const double phi3 = phi * phi * phi;
  M3 ks2 = (4.0 / kPiM) * kf;
  M3 t2 = sig / ((4.0 * phi * phi) * ks2 * n * n);
  M3 A = (beta / gamma) / (mexp((-1.0 / (gamma * phi3)) * eps) - cst(1.0));
  M3 At2 = A * t2;
  return (gamma * phi3) * mlog(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
}

__device__ __forceinline__ M3 tpss_c(M3 rho, M3 sigma, M3 tau, const Pow &P) {
  // unpolarised PBE
  M3 rs = kRs / P.r13;
  M3 e0 = pw_g(rs, 0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294);
  M3 kf = kKf * P.r13;
  M3 epbe = e0 + pbe_h(e0, 1.0, kf, rho, sigma);
  // fully polarised PBE of rho/2 with |grad(rho/2)|^2 = sigma/4
  M3 rs1 = kCbrt2 * rs;
  M3 e1 = pw_g(rs1, 0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517);
  M3 kf1 = (kKf / kCbrt2) * P.r13;
  M3 epbe1 = e1 + pbe_h(e1, kPhi1, kf1, 0.5 * rho, 0.25 * sigma);
  M3 et = mmax(epbe1, epbe);
  M3 z = sigma / (8.0 * rho * tau);
  M3 z2 = z * z;
  M3 erev = epbe * (1.0 + 0.53 * z2) - 1.53 * z2 * et;
  return rho * erev * (1.0 + 2.8 * erev * z2 * z);
}

} // namespace fnm

// Sum of the method's components at one point of a meta-GGA method: energy
// per volume e and vrho, vsigma, vtau.  LDA and GGA components of the same
// method go through eval_xc's evaluators (vtau 0 for them), as OCC sums
// Results of mixed families (include/occ/dft/functional.h:441-458).
__device__ __forceinline__ void eval_xc_mgga(const FuncSet &fs, double rho, double sigma,
                                             double tau, double &e, double &vrho, double &vsigma,
                                             double &vtau) {
  e = vrho = vsigma = vtau = 0.0;
  if (!(rho >= 1e-15))
    return;
  const double sg = fmax(sigma, 1e-40);
  const double tm = fmax(tau, 1e-20);
  const double sm = fmin(sg, 8.0 * rho * tm);
  fnm::M3 r{rho, 1.0, 0.0, 0.0}, s{sm, 0.0, 1.0, 0.0}, t{tm, 0.0, 0.0, 1.0};
  const fnm::Pow P = fnm::powers(r);
  fn::D3 r3{rho, 1.0, 0.0}, s3{sg, 0.0, 1.0};
  fn::RhoPowers<fn::D3> P3 = fn::rho_powers(r3);
  for (int i = 0; i < fs.n; i++) {
    const int id = fs.id[i];
    const double c = fs.coef[i];
    if (id == kMggaXTpss || id == kMggaCTpss) {
      const fnm::M3 v = id == kMggaXTpss ? fnm::tpss_x(r, s, t, P) : fnm::tpss_c(r, s, t, P);
      e += c * v.v;
      vrho += c * v.r;
      vsigma += c * v.s;
      vtau += c * v.t;
    } else {
      const fn::D3 v = fn::component(id, r3, s3, P3);
      e += c * v.v;
      vrho += c * v.r;
      vsigma += c * v.s;
    }
  }
}

} // namespace occx
