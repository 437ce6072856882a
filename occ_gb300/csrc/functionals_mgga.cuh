// Meta-GGA functionals per grid point: TPSS exchange and
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
// (rho, sigma, tau): M3 (FP64) for the FP64 build, MF3 (FP64 value, FP32
// derivatives) for the tensor-core build; the spin-polarised form (general
// zeta, for the UKS builds) over seven variables in P7 (FP64).  Thresholds: as for the GGAs the point is zero below
// rho = 1e-15; tau >= 1e-20, sigma >= 1e-40, and sigma is clamped to
// 8 rho tau (z <= 1) before evaluation, as Libxc does for meta-GGAs.
#pragma once
#include <cuda_runtime.h>

#include "functionals.cuh"
#include "functionals_pol.cuh"

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
template <class T> __device__ __forceinline__ T cst(double v);
template <> __device__ __forceinline__ M3 cst<M3>(double v) { return {v, 0.0, 0.0, 0.0}; }
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

// ---- the polarised form's dual: d/d rho_a, rho_b, s_aa, s_ab, s_bb, tau_a,
// tau_b in D (double: the FP64 build; float: the tensor-core build)
constexpr int kN7 = 7;
template <class D> struct Q7 {
  double v;
  D d[kN7];
};
using P7 = Q7<double>;
template <class D> __device__ __forceinline__ Q7<D> cst7(double v) {
  Q7<D> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < kN7; i++)
    r.d[i] = D(0);
  return r;
}
template <> __device__ __forceinline__ P7 cst<P7>(double v) { return cst7<double>(v); }
template <> __device__ __forceinline__ Q7<float> cst<Q7<float>>(double v) {
  return cst7<float>(v);
}
template <class D> __device__ __forceinline__ Q7<D> var7(double v, int k) {
  Q7<D> r = cst7<D>(v);
  r.d[k] = D(1);
  return r;
}
template <class D> __device__ __forceinline__ Q7<D> operator+(Q7<D> a, Q7<D> b) {
  Q7<D> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < kN7; i++)
    r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <class D> __device__ __forceinline__ Q7<D> operator-(Q7<D> a, Q7<D> b) {
  Q7<D> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < kN7; i++)
    r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <class D> __device__ __forceinline__ Q7<D> operator*(Q7<D> a, Q7<D> b) {
  Q7<D> r;
  r.v = a.v * b.v;
  const D av = static_cast<D>(a.v), bv = static_cast<D>(b.v);
#pragma unroll
  for (int i = 0; i < kN7; i++)
    r.d[i] = fma(a.d[i], bv, av * b.d[i]);
  return r;
}
template <class D> __device__ __forceinline__ Q7<D> operator/(Q7<D> a, Q7<D> b) {
  const double inv = 1.0 / b.v, q = a.v * inv;
  Q7<D> r;
  r.v = q;
  const D qd = static_cast<D>(q), ivd = static_cast<D>(inv);
#pragma unroll
  for (int i = 0; i < kN7; i++)
    r.d[i] = (a.d[i] - qd * b.d[i]) * ivd;
  return r;
}
template <class D> __device__ __forceinline__ Q7<D> operator*(double c, Q7<D> a) {
  Q7<D> r;
  r.v = c * a.v;
  const D cd = static_cast<D>(c);
#pragma unroll
  for (int i = 0; i < kN7; i++)
    r.d[i] = cd * a.d[i];
  return r;
}
template <class D> __device__ __forceinline__ Q7<D> operator+(double c, Q7<D> a) {
  a.v += c;
  return a;
}
template <class D> __device__ __forceinline__ Q7<D> operator-(double c, Q7<D> a) {
  return cst7<D>(c) - a;
}
template <class D> __device__ __forceinline__ Q7<D> operator/(double c, Q7<D> b) {
  return cst7<D>(c) / b;
}
template <class D> __device__ __forceinline__ Q7<D> chain(Q7<D> a, double f, double df) {
  Q7<D> r;
  r.v = f;
  const D dd = static_cast<D>(df);
#pragma unroll
  for (int i = 0; i < kN7; i++)
    r.d[i] = dd * a.d[i];
  return r;
}
template <class D> __device__ __forceinline__ Q7<D> mlog(Q7<D> a) {
  return chain(a, log(a.v), 1.0 / a.v);
}
template <class D> __device__ __forceinline__ Q7<D> mexp(Q7<D> a) {
  const double e = exp(a.v);
  return chain(a, e, e);
}
template <class D> __device__ __forceinline__ Q7<D> msqrt(Q7<D> a) {
  const double q = sqrt(a.v);
  return chain(a, q, 0.5 / q);
}
template <class D> __device__ __forceinline__ Q7<D> mcbrt(Q7<D> a) { // a > 0
  const double c = cbrt(a.v);
  return chain(a, c, c / (3.0 * a.v));
}
template <class D> __device__ __forceinline__ Q7<D> mmax(Q7<D> a, Q7<D> b) {
  return a.v >= b.v ? a : b;
}
// a, or the constant lo where a < lo (Libxc's zeta threshold)
template <class D> __device__ __forceinline__ Q7<D> mfloor(Q7<D> a, double lo) {
  return a.v >= lo ? a : cst7<D>(lo);
}

// ---- the tensor-core path's dual: FP64 value, FP32 derivatives (the value
// carries the energy; the derivatives feed V_xc, whose tolerance FP32 meets)
struct MF3 {
  double v;
  float r, s, t;
};
template <> __device__ __forceinline__ MF3 cst<MF3>(double v) { return {v, 0.f, 0.f, 0.f}; }
__device__ __forceinline__ MF3 operator+(MF3 a, MF3 b) {
  return {a.v + b.v, a.r + b.r, a.s + b.s, a.t + b.t};
}
__device__ __forceinline__ MF3 operator-(MF3 a, MF3 b) {
  return {a.v - b.v, a.r - b.r, a.s - b.s, a.t - b.t};
}
__device__ __forceinline__ MF3 operator*(MF3 a, MF3 b) {
  const float av = static_cast<float>(a.v), bv = static_cast<float>(b.v);
  return {a.v * b.v, fmaf(a.r, bv, av * b.r), fmaf(a.s, bv, av * b.s), fmaf(a.t, bv, av * b.t)};
}
__device__ __forceinline__ MF3 operator/(MF3 a, MF3 b) {
  const double q = a.v / b.v;
  const float iv = 1.f / static_cast<float>(b.v), qf = static_cast<float>(q);
  return {q, (a.r - qf * b.r) * iv, (a.s - qf * b.s) * iv, (a.t - qf * b.t) * iv};
}
__device__ __forceinline__ MF3 operator*(double c, MF3 a) {
  const float cf = static_cast<float>(c);
  return {c * a.v, cf * a.r, cf * a.s, cf * a.t};
}
__device__ __forceinline__ MF3 operator+(double c, MF3 a) { return {c + a.v, a.r, a.s, a.t}; }
__device__ __forceinline__ MF3 operator-(double c, MF3 a) { return {c - a.v, -a.r, -a.s, -a.t}; }
__device__ __forceinline__ MF3 operator/(double c, MF3 b) {
  const double q = c / b.v;
  const float f = -static_cast<float>(q) / static_cast<float>(b.v);
  return {q, f * b.r, f * b.s, f * b.t};
}
__device__ __forceinline__ MF3 chain(MF3 a, double f, float df) {
  return {f, df * a.r, df * a.s, df * a.t};
}
__device__ __forceinline__ MF3 mlog(MF3 a) {
  return chain(a, log(a.v), 1.f / static_cast<float>(a.v));
}
__device__ __forceinline__ MF3 mexp(MF3 a) {
  const double e = exp(a.v);
  return chain(a, e, static_cast<float>(e));
}
__device__ __forceinline__ MF3 msqrt(MF3 a) {
  const double q = sqrt(a.v);
  return chain(a, q, 0.5f / static_cast<float>(q));
}
__device__ __forceinline__ MF3 mcbrt(MF3 a) { // a > 0
  const double c = cbrt(a.v);
  return chain(a, c, static_cast<float>(c / (3.0 * a.v)));
}
__device__ __forceinline__ MF3 mmax(MF3 a, MF3 b) { return a.v >= b.v ? a : b; }

constexpr double kPiM = 3.14159265358979323846;
constexpr double kK2 = 9.570780000627305;     // (3 pi^2)^(2/3)
constexpr double kKf = 3.0936677262801355;    // (3 pi^2)^(1/3)
constexpr double kCx = 0.7385587663820224;    // (3/4)(3/pi)^(1/3)
constexpr double kRs = 0.6203504908994001;    // (3/(4 pi))^(1/3)
constexpr double kCbrt2 = 1.2599210498948732; // 2^(1/3)
// phi(zeta = 1) with 1 - zeta held at DBL_EPSILON: (2^(2/3) + eps^(2/3)) / 2
constexpr double kPhi1 = 0.79370052600243400;

template <class T> struct Pow {
  T r13, r43, r53, r83;
};
template <class T> __device__ __forceinline__ Pow<T> powers(T rho) {
  Pow<T> P;
  P.r13 = mcbrt(rho);
  P.r43 = rho * P.r13;
  P.r53 = P.r43 * P.r13;
  P.r83 = P.r53 * rho;
  return P;
}

template <class T>
__device__ __forceinline__ T tpss_x(T rho, T sigma, T tau, const Pow<T> &P) {
  using M3 = T;
  const double kappa = 0.804, b = 0.40, c = 1.59096, e = 1.537, mu = 0.21951;
  const double se = 1.2397580409095962; // sqrt(e)
  M3 p = sigma / ((4.0 * kK2) * P.r83);
  M3 tw = sigma / (8.0 * rho);
  M3 z = tw / tau;
  M3 alpha = (tau - tw) / ((0.3 * kK2) * P.r53);
  M3 am1 = alpha - cst<T>(1.0);
  M3 qb = 0.45 * am1 / msqrt(1.0 + b * alpha * am1) + (2.0 / 3.0) * p;
  M3 z2 = z * z;
  M3 opz2 = 1.0 + z2;
  M3 tz2 = 0.36 * z2; // (3 z / 5)^2
  M3 p2 = p * p;
  M3 num = (cst<T>(10.0 / 81.0) + c * z2 / (opz2 * opz2)) * p + (146.0 / 2025.0) * qb * qb -
           (73.0 / 405.0) * qb * msqrt(0.5 * tz2 + 0.5 * p2) +
           ((1.0 / kappa) * (10.0 / 81.0) * (10.0 / 81.0)) * p2 +
           (2.0 * se * (10.0 / 81.0)) * tz2 + (e * mu) * p2 * p;
  M3 den = 1.0 + se * p;
  M3 x = num / (den * den);
  M3 Fx = (1.0 + kappa) - kappa / (1.0 + (1.0 / kappa) * x);
  return (-kCx) * P.r43 * Fx;
}

// PW92 G(rs) of one fit
template <class T>
__device__ __forceinline__ T pw_g(T rs, double A, double a1, double b1, double b2, double b3,
                                  double b4) {
  using M3 = T;
  M3 srs = msqrt(rs);
  M3 den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return (-2.0 * A) * (1.0 + a1 * rs) * mlog(1.0 + 1.0 / den);
}

// PBE correlation per particle given the LDA part eps, the spin factor phi
// (phi^3 = phi3), k_F and n, and |grad n|^2
template <class M3>
__device__ __forceinline__ M3 pbe_h(M3 eps, double phi, M3 kf, M3 n, M3 sig) {
  const double beta = 0.06672455060314922, gamma = 0.031090690869654897;
  const double phi3 = phi * phi * phi;
  M3 ks2 = (4.0 / kPiM) * kf;
  M3 t2 = sig / ((4.0 * phi * phi) * ks2 * n * n);
  M3 A = (beta / gamma) / (mexp((-1.0 / (gamma * phi3)) * eps) - cst<M3>(1.0));
  M3 At2 = A * t2;
  return (gamma * phi3) * mlog(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
}

template <class M3>
__device__ __forceinline__ M3 tpss_c(M3 rho, M3 sigma, M3 tau, const Pow<M3> &P) {
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

// ---- spin-polarised TPSS (the UKS builds), over Q7<double> or Q7<float>
// PBE correlation per particle of spin densities (ra, rb) with total
// |grad rho|^2 = sig: PW92's spin interpolation and phi(zeta)
template <class P7> __device__ __forceinline__ P7 pbe_eps_pol(P7 ra, P7 rb, P7 sig) {
  const double beta = 0.06672455060314922, gamma = 0.031090690869654897;
  const double fpp0 = 1.7099209341613657, eps_z = 2.220446049250313e-16;
  P7 n = ra + rb;
  P7 z = (ra - rb) / n;
  P7 opz = mfloor(1.0 + z, eps_z), omz = mfloor(1.0 - z, eps_z);
  P7 n13 = mcbrt(n);
  P7 rs = kRs / n13;
  P7 e0 = pw_g(rs, 0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294);
  P7 e1 = pw_g(rs, 0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517);
  P7 ac = cst<P7>(0.0) - pw_g(rs, 0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671);
  P7 o13 = mcbrt(opz), m13 = mcbrt(omz);
  P7 f = (1.0 / 0.5198420997897464) * (opz * o13 + omz * m13 - cst<P7>(2.0));
  P7 z2 = z * z, z4 = z2 * z2;
  P7 eps = e0 + (1.0 / fpp0) * ac * f * (1.0 - z4) + (e1 - e0) * f * z4;
  P7 phi = 0.5 * (o13 * o13 + m13 * m13);
  P7 phi3 = phi * phi * phi;
  P7 ks2 = (4.0 / kPiM) * (kKf * n13);
  P7 t2 = sig / (4.0 * phi * phi * ks2 * n * n);
  P7 A = (beta / gamma) / (mexp(cst<P7>(0.0) - eps / (gamma * phi3)) - cst<P7>(1.0));
  P7 At2 = A * t2;
  P7 H = gamma * phi3 * mlog(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return eps + H;
}

// TPSS exchange of one spin channel: E_x[2 rho_s, 4 s_ss, 2 tau_s] / 2
template <class P7> __device__ __forceinline__ P7 tpss_x_s(P7 r, P7 s, P7 t) {
  const P7 n = 2.0 * r;
  return 0.5 * tpss_x(n, 4.0 * s, 2.0 * t, powers(n));
}

// revPKZB / TPSS correlation (eqs. 11-14) of a polarised density
template <class P7>
__device__ __forceinline__ P7 tpss_c_pol(P7 ra, P7 rb, P7 saa, P7 sab, P7 sbb, P7 ta, P7 tb,
                                         bool sa, bool sb) {
  const double eps_z = 2.220446049250313e-16;
  P7 n = ra + rb;
  P7 sig = saa + 2.0 * sab + sbb;
  P7 tau = ta + tb;
  P7 z = sig / (8.0 * n * tau);
  P7 zeta = (ra - rb) / n;
  P7 opz = mfloor(1.0 + zeta, eps_z), omz = mfloor(1.0 - zeta, eps_z);
  P7 n2 = n * n;
  P7 gz2 = 4.0 * (rb * rb * saa - 2.0 * ra * rb * sab + ra * ra * sbb) / (n2 * n2);
  P7 n13 = mcbrt(n);
  P7 xi2 = gz2 / ((4.0 * kKf * kKf) * n13 * n13);
  P7 zt2 = zeta * zeta;
  P7 C0 = 0.53 + zt2 * (0.87 + zt2 * (0.50 + 2.26 * zt2));
  P7 o13 = mcbrt(opz), m13 = mcbrt(omz);
  P7 g = 1.0 + 0.5 * xi2 * (1.0 / (opz * o13) + 1.0 / (omz * m13));
  P7 g2 = g * g;
  P7 C = C0 / (g2 * g2);
  P7 epbe = pbe_eps_pol(ra, rb, sig);
  P7 sum = cst<P7>(0.0);
  if (sa)
    sum = sum + ra / n * mmax(pbe_eps_pol(ra, cst<P7>(0.0), saa), epbe);
  if (sb)
    sum = sum + rb / n * mmax(pbe_eps_pol(rb, cst<P7>(0.0), sbb), epbe);
  P7 z2 = z * z;
  P7 erev = epbe * (1.0 + C * z2) - (1.0 + C) * z2 * sum;
  return n * erev * (1.0 + 2.8 * erev * z2 * z);
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
  const fnm::Pow<fnm::M3> P = fnm::powers(r);
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

// Out-of-line entries for the mixed evaluator's rare paths (kept out of its
// register allocation).
static __device__ __noinline__ void eval_xc_mgga_fp64_call(const FuncSet &fs, double rho,
                                                           double sigma, double tau,
                                                           double *out4) {
  eval_xc_mgga(fs, rho, sigma, tau, out4[0], out4[1], out4[2], out4[3]);
}
static __device__ __noinline__ void eval_xc_mixed_call(const FuncSet &fs, double rho,
                                                       double sigma, double *out3) {
  eval_xc_mixed(fs, rho, sigma, out3[0], out3[1], out3[2]);
}

// The tensor-core path's evaluator: meta-GGA components with FP64 values and
// FP32 derivatives (MF3) on the FP64 evaluator's clamped arguments, where
// rho >= 1e-10 and p = s^2 <= 1e4 (so that the FP32 derivatives of the p^3
// term stay inside the FP32 range), the FP64 evaluator elsewhere and for any
// point whose result is not finite; LDA / GGA components through eval_xc_mixed.
__device__ __forceinline__ void eval_xc_mgga_mixed(const FuncSet &fs, double rho, double sigma,
                                                   double tau, double &e, double &vrho,
                                                   double &vsigma, double &vtau) {
  const double tm = fmax(tau, 1e-20);
  const double sm = fmin(fmax(sigma, 1e-40), 8.0 * rho * tm);
  const float rf = static_cast<float>(rho), r13 = cbrtf(rf);
  const float pf = static_cast<float>(sm) / (38.28312000250922f * rf * rf * r13 * r13);
  if (!(rho >= 1e-10) || !(pf <= 1e4f)) {
    double o[4];
    eval_xc_mgga_fp64_call(fs, rho, sigma, tau, o);
    e = o[0], vrho = o[1], vsigma = o[2], vtau = o[3];
    return;
  }
  e = vrho = vsigma = vtau = 0.0;
  bool other = false;
  for (int i = 0; i < fs.n; i++)
    other = other || !func_is_mgga(fs.id[i]);
  if (other) { // the method's LDA / GGA components, as the GGA mixed path evaluates them
    FuncSet g = fs;
    g.n = 0;
    for (int i = 0; i < fs.n; i++)
      if (!func_is_mgga(fs.id[i])) {
        g.id[g.n] = fs.id[i];
        g.coef[g.n++] = fs.coef[i];
      }
    double o[3];
    eval_xc_mixed_call(g, rho, sigma, o);
    e = o[0], vrho = o[1], vsigma = o[2];
  }
  fnm::MF3 r{rho, 1.f, 0.f, 0.f}, s{sm, 0.f, 1.f, 0.f}, t{tm, 0.f, 0.f, 1.f};
  const fnm::Pow<fnm::MF3> P = fnm::powers(r);
  for (int i = 0; i < fs.n; i++) {
    const int id = fs.id[i];
    if (id != kMggaXTpss && id != kMggaCTpss)
      continue;
    const fnm::MF3 v = id == kMggaXTpss ? fnm::tpss_x(r, s, t, P) : fnm::tpss_c(r, s, t, P);
    const double c = fs.coef[i];
    e += c * v.v;
    vrho += c * static_cast<double>(v.r);
    vsigma += c * static_cast<double>(v.s);
    vtau += c * static_cast<double>(v.t);
  }
  if (!isfinite(e) || !isfinite(vrho) || !isfinite(vsigma) || !isfinite(vtau)) {
    double o[4]; // an FP32 overflow
    eval_xc_mgga_fp64_call(fs, rho, sigma, tau, o);
    e = o[0], vrho = o[1], vsigma = o[2], vtau = o[3];
  }
}

// The meta-GGA components of a polarised method in Q7<D>, on arguments
// already clamped as Libxc clamps them (tau_s >= 1e-20, s_ss <= 8 rho_s tau_s,
// |s_ab| <= (s_aa + s_bb) / 2).
template <class D>
__device__ __forceinline__ fnm::Q7<D> mgga_pol_sum(const FuncSet &fs, double ra, double rb,
                                                   double saa, double sab, double sbb,
                                                   double ta, double tb) {
  using Q = fnm::Q7<D>;
  const Q Ra = fnm::var7<D>(ra, 0), Rb = fnm::var7<D>(rb, 1), Saa = fnm::var7<D>(saa, 2),
          Sab = fnm::var7<D>(sab, 3), Sbb = fnm::var7<D>(sbb, 4), Ta = fnm::var7<D>(ta, 5),
          Tb = fnm::var7<D>(tb, 6);
  const bool sa = ra >= 1e-15, sb = rb >= 1e-15;
  Q tot = fnm::cst7<D>(0.0);
  for (int i = 0; i < fs.n; i++) {
    if (fs.id[i] == kMggaXTpss) {
      Q x = fnm::cst7<D>(0.0);
      if (sa)
        x = x + fnm::tpss_x_s(Ra, Saa, Ta);
      if (sb)
        x = x + fnm::tpss_x_s(Rb, Sbb, Tb);
      tot = tot + fs.coef[i] * x;
    } else if (fs.id[i] == kMggaCTpss) {
      tot = tot + fs.coef[i] * fnm::tpss_c_pol(Ra, Rb, Saa, Sab, Sbb, Ta, Tb, sa, sb);
    }
  }
  return tot;
}

// Libxc's clamps of the meta-GGA arguments; false below the density threshold
__device__ __forceinline__ bool mgga_pol_clamp(double &ra, double &rb, double &saa, double &sab,
                                               double &sbb, double &ta, double &tb) {
  ra = fmax(ra, 0.0);
  rb = fmax(rb, 0.0);
  if (!(ra + rb >= 1e-15))
    return false;
  ta = fmax(ta, 1e-20);
  tb = fmax(tb, 1e-20);
  saa = fmin(fmax(saa, 1e-40), 8.0 * ra * ta);
  sbb = fmin(fmax(sbb, 1e-40), 8.0 * rb * tb);
  const double lim = 0.5 * (saa + sbb);
  sab = fmin(fmax(sab, -lim), lim);
  return true;
}

template <class D>
__device__ __forceinline__ void mgga_pol_add(const fnm::Q7<D> &t, double &e, double *vrho,
                                             double *vsig, double *vtau) {
  e += t.v;
  vrho[0] += t.d[0];
  vrho[1] += t.d[1];
  vsig[0] += t.d[2];
  vsig[1] += t.d[3];
  vsig[2] += t.d[4];
  vtau[0] = t.d[5];
  vtau[1] = t.d[6];
}

// One point of a polarised meta-GGA method: e and vrho[2], vsigma[3],
// vtau[2], FP64.  Meta-GGA components on the clamped arguments, the method's
// LDA / GGA components through eval_xc_pol on the arguments as given.
__device__ __forceinline__ void eval_xc_mgga_pol(const FuncSet &fs, double ra, double rb,
                                                 double saa, double sab, double sbb, double ta,
                                                 double tb, double &e, double *vrho,
                                                 double *vsig, double *vtau) {
  eval_xc_pol(fs, ra, rb, saa, sab, sbb, e, vrho, vsig); // its switch skips meta-GGA ids
  vtau[0] = vtau[1] = 0.0;
  if (mgga_pol_clamp(ra, rb, saa, sab, sbb, ta, tb))
    mgga_pol_add(mgga_pol_sum<double>(fs, ra, rb, saa, sab, sbb, ta, tb), e, vrho, vsig, vtau);
}

static __device__ __noinline__ void eval_xc_mgga_pol_fp64_call(const FuncSet &fs, double ra,
                                                               double rb, double saa,
                                                               double sab, double sbb,
                                                               double ta, double tb,
                                                               double *out8) {
  eval_xc_mgga_pol(fs, ra, rb, saa, sab, sbb, ta, tb, out8[0], out8 + 1, out8 + 3, out8 + 6);
}

// The tensor-core UKS build's evaluator: FP64 values with FP32 derivatives
// where both spin densities are >= 1e-10 and each channel's p = s^2 <= 1e4
// (the FP32 derivatives of TPSS exchange's p^3 term stay in range), the FP64
// evaluator elsewhere and for any point whose result is not finite.
__device__ __forceinline__ void eval_xc_mgga_pol_mixed(const FuncSet &fs, double ra, double rb,
                                                       double saa, double sab, double sbb,
                                                       double ta, double tb, double &e,
                                                       double *vrho, double *vsig,
                                                       double *vtau) {
  const double ra0 = ra, rb0 = rb, saa0 = saa, sab0 = sab, sbb0 = sbb, ta0 = ta, tb0 = tb;
  bool fast = ra >= 1e-10 && rb >= 1e-10 && mgga_pol_clamp(ra, rb, saa, sab, sbb, ta, tb);
  if (fast) { // p of each channel (exchange of 2 rho_s, 4 s_ss)
    const float a = static_cast<float>(2.0 * ra), b = static_cast<float>(2.0 * rb);
    const float a13 = cbrtf(a), b13 = cbrtf(b);
    fast = static_cast<float>(4.0 * saa) / (38.28312000250922f * a * a * a13 * a13) <= 1e4f &&
           static_cast<float>(4.0 * sbb) / (38.28312000250922f * b * b * b13 * b13) <= 1e4f;
  }
  if (fast) {
    eval_xc_pol_mixed(fs, ra0, rb0, saa0, sab0, sbb0, e, vrho, vsig);
    vtau[0] = vtau[1] = 0.0;
    mgga_pol_add(mgga_pol_sum<float>(fs, ra, rb, saa, sab, sbb, ta, tb), e, vrho, vsig, vtau);
    fast = isfinite(e) && isfinite(vrho[0]) && isfinite(vrho[1]) && isfinite(vsig[0]) &&
           isfinite(vsig[1]) && isfinite(vsig[2]) && isfinite(vtau[0]) && isfinite(vtau[1]);
  }
  if (!fast) {
    double o[8];
    eval_xc_mgga_pol_fp64_call(fs, ra0, rb0, saa0, sab0, sbb0, ta0, tb0, o);
    e = o[0], vrho[0] = o[1], vrho[1] = o[2], vsig[0] = o[3], vsig[1] = o[4], vsig[2] = o[5];
    vtau[0] = o[6], vtau[1] = o[7];
  }
}

} // namespace occx
