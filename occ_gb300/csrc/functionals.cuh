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
  kHybPbeh = 406,      // 0.75 PBE exchange + PBE correlation (PBE0's local part)
  kHybBhandh = 435,    // 0.5 Slater + LYP
  kHybBhandhlyp = 436, // 0.5 B88 + LYP
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
         id == kHybB3lyp || id == kHybB3lyp5 || id == kHybPbeh || id == kHybBhandh ||
         id == kHybBhandhlyp;
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

// ---- the mixed path's dual number: value in double-float FP32, derivatives
// in FP32.  FP32 arithmetic is tens of times the FP64 rate on this GPU; the
// value keeps about 44 bits (error-free transformations: Knuth's TwoSum,
// FMA-based TwoProduct; Dekker/Shewchuk double-float algorithms), so energy
// densities stay FP64-grade, while the derivatives feed V_xc, whose
// tolerance FP32 meets.  exp, log, cube roots, sqrt and divisions are done in
// double-float (f2_exp, f2_log, f2_cbrt below); atan and asinh (VWN, B88)
// take FP64 from the double-float argument.  The _rn intrinsics keep the compiler from fusing
// the error-free transformations into FMAs.
struct F2 {
  float h, l; // value h + l, |l| <= ulp(h) / 2
};
__host__ __device__ constexpr F2 f2c(double x) {
  return {static_cast<float>(x), static_cast<float>(x - static_cast<double>(static_cast<float>(x)))};
}
__device__ __forceinline__ F2 f2(double x) {
  const float h = static_cast<float>(x);
  return {h, static_cast<float>(x - static_cast<double>(h))};
}
__device__ __forceinline__ double to_d(F2 a) {
  return static_cast<double>(a.h) + static_cast<double>(a.l);
}
__device__ __forceinline__ F2 quick_two_sum(float a, float b) { // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
// x as a double-float by integer operations, off the FP64 pipe: the sign,
// exponent and top 23 mantissa bits as h, the remaining 29 bits as l =
// (m29 2^-29) 2^(E-23), E the exponent of x: m29 rounded to FP32 and scaled
// by two powers of two, both exact while 2^(E-23) is an FP32 normal number
// (|x| above about 1e-31), then renormalised.  For |x| below FP32's largest
// value; below about 1e-31 l is dropped (x keeps FP32 precision), and values
// below FP32's normal range give zero.
__device__ __forceinline__ F2 f2_bits(double x) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
  const int e = static_cast<int>((u >> 52) & 0x7ff);
  if (e - 1023 + 127 < 1) // below FP32's normal range (and zero)
    return {0.f, 0.f};
  const unsigned sgn = static_cast<unsigned>(u >> 32) & 0x80000000u;
  const float h = __uint_as_float(sgn | (static_cast<unsigned>(e - 1023 + 127) << 23) |
                                  static_cast<unsigned>((u >> 29) & 0x7fffffu));
  const int es = e - 1023 - 23 + 127; // biased exponent of 2^(E-23)
  const float scale = es >= 1 ? __uint_as_float(static_cast<unsigned>(es) << 23) : 0.f;
  const float l = (__uint2float_rn(static_cast<unsigned>(u & 0x1fffffffu)) * 0x1p-29f) * scale;
  return quick_two_sum(h, sgn ? -l : l);
}
__device__ __forceinline__ F2 two_sum_f(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const F2 s = two_sum_f(a.h, b.h);
  const F2 t = two_sum_f(a.l, b.l);
  F2 u = quick_two_sum(s.h, __fadd_rn(s.l, t.h));
  return quick_two_sum(u.h, __fadd_rn(u.l, t.l));
}
__device__ __forceinline__ F2 f2_neg(F2 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.h, b.h);
  const float e = fmaf(a.h, b.h, -p);
  return quick_two_sum(p, __fadd_rn(e, __fadd_rn(__fmul_rn(a.h, b.l), __fmul_rn(a.l, b.h))));
}
__device__ __forceinline__ F2 f2_div(F2 a, F2 b) {
  // two correction steps of the float quotient
  const float q1 = __fdiv_rn(a.h, b.h);
  F2 r = f2_add(a, f2_neg(f2_mul({q1, 0.f}, b)));
  const float q2 = __fdiv_rn(r.h, b.h);
  r = f2_add(r, f2_neg(f2_mul({q2, 0.f}, b)));
  const float q3 = __fdiv_rn(r.h, b.h);
  return f2_add(quick_two_sum(q1, q2), {q3, 0.f});
}
__device__ __forceinline__ F2 f2_sqrt(F2 a) { // one Newton step from the float root
  const float y = sqrtf(a.h);
  const F2 yy = f2_mul({y, 0.f}, {y, 0.f});
  const F2 r = f2_add(a, f2_neg(yy));
  return quick_two_sum(y, __fdiv_rn(r.h, __fmul_rn(2.f, y)));
}

// Double-float transcendentals from FP32 operations (the FP64 pipe is a
// small fraction of this GPU's), accurate to about 1e-14 relative:
// e^x by Cody-Waite reduction x = n ln2 + r (W.J. Cody, W. Waite, Software
// Manual for the Elementary Functions, 1980) with ln2 in three floats, e^r
// from e^(r/4) by its Taylor series (degree 11) and two squarings, then the
// exact scaling 2^n; log x by one Newton step y + x e^-y - 1 from the
// FP32 logarithm, and x^(1/3) by one Newton step from the FP32 cube root
// (each step squares the FP32 starting error, ~1e-7, to ~1e-14).
__device__ __forceinline__ F2 f2_scale(F2 a, float c) { // c a power of two
  return {a.h * c, a.l * c};
}
// e^r - 1 for |r| <= 0.35 (so that the result keeps its relative accuracy
// when it is small): from t = r / 4 and two squarings.
__device__ __forceinline__ F2 f2_expm1_small(F2 r) {
  r = f2_scale(r, 0.25f);
  // e^t - 1 for |t| <= 0.087 by Taylor, degree 11 (truncation < 1e-21); the
  // 1/k! as double-floats
  const float ih[9] = {2.755731998e-07f, 2.755731884e-06f, 2.480158764e-05f, 1.984127011e-04f,
                        1.388888923e-03f, 8.333333768e-03f, 4.166666791e-02f, 1.666666716e-01f,
                        5.000000000e-01f};
  const float il[9] = {-7.575112209e-15f, 3.793571224e-14f, -3.406996094e-13f, -2.725596875e-12f,
                        -3.363109444e-11f, -4.346172033e-10f, -1.241763470e-09f, -4.967053879e-09f,
                        0.000000000e+00f};
  F2 q = {2.505210794e-08f, 4.417623045e-16f}; // 1/11!
#pragma unroll
  for (int k = 0; k < 9; k++) // + 1/10!, ..., 1/2!
    q = f2_add(f2_mul(q, r), {ih[k], il[k]});
  q = f2_add(f2_mul(q, r), {1.f, 0.f});
  F2 em1 = f2_mul(q, r); // e^t - 1
  // (1 + u)^2 = 1 + (2u + u^2): square twice keeping the "- 1" form
#pragma unroll
  for (int k = 0; k < 2; k++)
    em1 = f2_add(f2_scale(em1, 2.f), f2_mul(em1, em1));
  return em1;
}
__device__ __forceinline__ F2 f2_exp(F2 x) {
  const float n = rintf(x.h * 1.44269504088896341f);
  const float c1 = 0.693145751953125f;             // 15 bits: n c1 exact
  const float c2h = 1.42860677e-06f, c2l = 5.4979231e-14f; // ln2 - c1 in two floats
  F2 r = two_sum_f(x.h, -n * c1);
  const float p2 = __fmul_rn(n, c2h);
  r = f2_add(r, {-p2, -fmaf(n, c2h, -p2)});
  r = f2_add(r, {-n * c2l, 0.f});
  r = f2_add(r, {x.l, 0.f});
  const F2 e = f2_add({1.f, 0.f}, f2_expm1_small(r));
  const float s = n < -126.f ? 0.f : __int_as_float((static_cast<int>(n) + 127) << 23);
  return f2_scale(e, s);
}
__device__ __forceinline__ F2 f2_log(F2 x) { // x > 0
  F2 d;
  float y0;
  if (fabsf(x.h - 1.f) < 0.25f) {
    // near 1 the result is small: d = (1 + u) e^-y0 - 1 = m + u (1 + m),
    // m = e^-y0 - 1, each term with its own relative accuracy
    const F2 u = f2_add(x, {-1.f, 0.f}); // exact (Sterbenz)
    y0 = log1pf(u.h);
    const F2 m = f2_expm1_small({-y0, 0.f});
    d = f2_add(m, f2_mul(u, f2_add({1.f, 0.f}, m)));
  } else {
    y0 = logf(x.h);
    d = f2_add(f2_mul(x, f2_exp({-y0, 0.f})), {-1.f, 0.f}); // x e^-y0 - 1, ~1e-7
  }
  // log(1 + d) = d - d^2 / 2 + O(d^3)
  return f2_add({y0, 0.f}, f2_add(d, {-0.5f * d.h * d.h, 0.f}));
}
__device__ __forceinline__ F2 f2_cbrt(F2 x) { // x > 0
  const float y0 = cbrtf(x.h);
  const F2 y3 = f2_mul(f2_mul({y0, 0.f}, {y0, 0.f}), {y0, 0.f});
  const F2 r = f2_add(x, f2_neg(y3));
  return quick_two_sum(y0, __fdiv_rn(r.h, 3.f * y0 * y0));
}

struct G {
  F2 v;
  float r, s;
};
__device__ __forceinline__ G operator+(G a, G b) { return {f2_add(a.v, b.v), a.r + b.r, a.s + b.s}; }
__device__ __forceinline__ G operator-(G a, G b) {
  return {f2_add(a.v, f2_neg(b.v)), a.r - b.r, a.s - b.s};
}
__device__ __forceinline__ G operator*(G a, G b) {
  return {f2_mul(a.v, b.v), fmaf(a.r, b.v.h, a.v.h * b.r), fmaf(a.s, b.v.h, a.v.h * b.s)};
}
__device__ __forceinline__ G operator/(G a, G b) {
  const F2 q = f2_div(a.v, b.v);
  const float iv = 1.f / b.v.h;
  return {q, (a.r - q.h * b.r) * iv, (a.s - q.h * b.s) * iv};
}
__device__ __forceinline__ G operator*(double c, G a) {
  const F2 cc = f2c(c);
  return {f2_mul(cc, a.v), cc.h * a.r, cc.h * a.s};
}
__device__ __forceinline__ G operator+(double c, G a) { return {f2_add(f2c(c), a.v), a.r, a.s}; }
__device__ __forceinline__ G operator-(double c, G a) {
  return {f2_add(f2c(c), f2_neg(a.v)), -a.r, -a.s};
}
__device__ __forceinline__ G operator/(double c, G b) {
  const F2 q = f2_div(f2c(c), b.v);
  const float iv = 1.f / b.v.h;
  return {q, -q.h * b.r * iv, -q.h * b.s * iv};
}
__device__ __forceinline__ G neg(G a) { return {f2_neg(a.v), -a.r, -a.s}; }
__device__ __forceinline__ G mkg(double v) { return {f2c(v), 0.f, 0.f}; }
__device__ __forceinline__ G gapply(G a, double f, float df) { return {f2(f), df * a.r, df * a.s}; }
__device__ __forceinline__ G dlog(G a) {
  const float d = 1.f / a.v.h;
  return {f2_log(a.v), d * a.r, d * a.s};
}
__device__ __forceinline__ G dexp(G a) {
  const F2 e = f2_exp(a.v);
  return {e, e.h * a.r, e.h * a.s};
}
__device__ __forceinline__ G dsqrt(G a) {
  const F2 s = f2_sqrt(a.v);
  const float d = 0.5f / s.h;
  return {s, d * a.r, d * a.s};
}
__device__ __forceinline__ G datan(G a) {
  return gapply(a, atan(to_d(a.v)), 1.f / fmaf(a.v.h, a.v.h, 1.f));
}
__device__ __forceinline__ G dasinh(G a) {
  return gapply(a, asinh(to_d(a.v)), rsqrtf(fmaf(a.v.h, a.v.h, 1.f)));
}

// constants of either dual type
template <class T> struct Num;
template <> struct Num<D3> {
  __device__ __forceinline__ static D3 c(double v) { return mk(v); }
};
template <> struct Num<G> {
  __device__ __forceinline__ static G c(double v) { return mkg(v); }
};

constexpr double kPi = 3.14159265358979323846;

// rho^(1/3) and friends from one cube root
template <class T> struct RhoPowers {
  T r13, r43, rm13; // rho^(1/3), rho^(4/3), rho^(-1/3)
};
__device__ __forceinline__ RhoPowers<D3> rho_powers(D3 rho) {
  double c = cbrt(rho.v);
  D3 r13 = apply(rho, c, c / (3.0 * rho.v));
  D3 r43 = rho * r13;
  D3 rm13 = apply(rho, 1.0 / c, -1.0 / (3.0 * c * rho.v));
  return {r13, r43, rm13};
}
__device__ __forceinline__ RhoPowers<G> rho_powers(G rho) {
  const F2 c = f2_cbrt(rho.v);
  const float cf = c.h, rf = rho.v.h;
  const float d13 = cf / (3.f * rf), dm13 = -1.f / (3.f * cf * rf);
  G r13 = {c, d13 * rho.r, d13 * rho.s};
  G r43 = rho * r13;
  G rm13 = {f2_div({1.f, 0.f}, c), dm13 * rho.r, dm13 * rho.s};
  return {r13, r43, rm13};
}

template <class T> __device__ __forceinline__ T slater(const RhoPowers<T> &P) {
  const double cx = 0.7385587663820224; // (3/4)(3/pi)^(1/3)
  return -cx * P.r43;
}

template <class T>
__device__ __forceinline__ T vwn_eps(T rs, double A, double b, double c, double x0) {
  using N = Num<T>;
  T x = dsqrt(rs);
  T X = x * x + b * x + N::c(c);
  double X0 = x0 * x0 + b * x0 + c;
  double Q = sqrt(4.0 * c - b * b);
  T at = datan(N::c(Q) / (2.0 * x + N::c(b)));
  T t1 = dlog(x * x / X) + (2.0 * b / Q) * at;
  T xm = x - N::c(x0);
  T t2 = dlog(xm * xm / X) + (2.0 * (b + 2.0 * x0) / Q) * at;
  return A * (t1 - (b * x0 / X0) * t2);
}

template <class T> __device__ __forceinline__ T rs_of(const RhoPowers<T> &P) {
  const double k = 0.6203504908994001; // (3/(4 pi))^(1/3)
  return k * P.rm13;
}

template <class T> __device__ __forceinline__ T vwn5(T rho, const RhoPowers<T> &P) {
  return rho * vwn_eps(rs_of(P), 0.0310907, 3.72744, 12.9352, -0.10498);
}
template <class T> __device__ __forceinline__ T vwn_rpa(T rho, const RhoPowers<T> &P) {
  return rho * vwn_eps(rs_of(P), 0.0310907, 13.0720, 42.7198, -0.409286);
}

template <class T> __device__ __forceinline__ T b88(T rho, T sigma, const RhoPowers<T> &P) {
  const double beta = 0.0042;
  const double cs = 0.9305257363491000; // (3/2)(3/(4 pi))^(1/3)
  // spin density rho/2: (rho/2)^(4/3) = rho^(4/3) / 2^(4/3)
  T r43s = 0.39685026299204984 * P.r43;
  T x2 = (0.25 * sigma) / (r43s * r43s);
  T x = dsqrt(x2);
  T per = neg(cs * r43s) - beta * r43s * x2 / (1.0 + 6.0 * beta * x * dasinh(x));
  return 2.0 * per;
}

template <class T> __device__ __forceinline__ T lyp(T rho, T sigma, const RhoPowers<T> &P) {
  const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
  const double cf = 2.8712340001881915; // (3/10)(3 pi^2)^(2/3)
  T den = 1.0 + d * P.rm13;
  T E = dexp(neg(c * P.rm13));
  T delta = c * P.rm13 + d * P.rm13 / den;
  T rm53 = P.rm13 / P.r43; // rho^(-5/3)
  T t1 = neg(a * rho / den);
  T t2 = neg((a * b * cf) * rho * E / den);
  T t3 = (a * b / 72.0) * (3.0 + 7.0 * delta) * sigma * rm53 * E / den;
  return t1 + t2 + t3;
}

template <class T> __device__ __forceinline__ T kf2_of(const RhoPowers<T> &P) {
  const double k = 3.0936677262801355; // (3 pi^2)^(1/3)
  T kf = k * P.r13;
  return kf * kf;
}

template <class T> __device__ __forceinline__ T pbe_x(T rho, T sigma, const RhoPowers<T> &P) {
  const double kappa = 0.8040, mu = 0.2195149727645171;
  T s2 = sigma / (4.0 * kf2_of(P) * rho * rho);
  T F = (1.0 + kappa) - kappa / (1.0 + (mu / kappa) * s2);
  return slater(P) * F;
}

template <class T> __device__ __forceinline__ T pbe_c(T rho, T sigma, const RhoPowers<T> &P) {
  using N = Num<T>;
  const double beta = 0.06672455060314922;
  const double gamma = 0.031090690869654897; // (1 - ln 2) / pi^2
  const double A = 0.0310907, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382,
               b4 = 0.49294;
  T rs = rs_of(P);
  T srs = dsqrt(rs);
  T den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  T eps = (-2.0 * A) * (1.0 + a1 * rs) * dlog(1.0 + N::c(1.0) / den);
  const double k = 3.0936677262801355;
  T kf = k * P.r13;
  T ks2 = (4.0 / kPi) * kf;
  T t2 = sigma / (4.0 * ks2 * rho * rho);
  T Af = (beta / gamma) / (dexp(neg(eps) / N::c(gamma)) - N::c(1.0));
  T At2 = Af * t2;
  T H = gamma * dlog(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return rho * (eps + H);
}

// Energy density of one component (before its mixture coefficient).
template <class T>
__device__ __forceinline__ T component(int id, T rho, T sigma, const RhoPowers<T> &P) {
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
  case kHybPbeh:
    return 0.75 * pbe_x(rho, sigma, P) + pbe_c(rho, sigma, P);
  case kHybBhandh:
    return 0.5 * slater(P) + lyp(rho, sigma, P);
  case kHybBhandhlyp:
    return 0.5 * b88(rho, sigma, P) + lyp(rho, sigma, P);
  }
  return Num<T>::c(0.0);
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
  fn::RhoPowers<fn::D3> P = fn::rho_powers(r);
  for (int i = 0; i < fs.n; i++) {
    fn::D3 c = fn::component(fs.id[i], r, s, P);
    e += fs.coef[i] * c.v;
    vrho += fs.coef[i] * c.r;
    vsigma += fs.coef[i] * c.s;
  }
}

// The mixed path's evaluator: double-float values and FP32 derivatives
// (fn::G) where rho >= 1e-10 and sigma >= 1e-30; FP64 (eval_xc) elsewhere,
// where intermediate powers of rho would leave the FP32 exponent range or
// sigma meets the FP64 path's clamp.
__device__ __forceinline__ void eval_xc_mixed(const FuncSet &fs, double rho, double sigma,
                                              double &e, double &vrho, double &vsigma) {
  if (!(rho >= 1e-10) || !(sigma >= 1e-30)) {
    eval_xc(fs, rho, sigma, e, vrho, vsigma);
    return;
  }
  fn::G r{fn::f2(rho), 1.f, 0.f};
  fn::G s{fn::f2(sigma), 0.f, 1.f};
  fn::RhoPowers<fn::G> P = fn::rho_powers(r);
  e = vrho = vsigma = 0.0;
  for (int i = 0; i < fs.n; i++) {
    fn::G c = fn::component(fs.id[i], r, s, P);
    e += fs.coef[i] * fn::to_d(c.v);
    vrho += fs.coef[i] * static_cast<double>(c.r);
    vsigma += fs.coef[i] * static_cast<double>(c.s);
  }
}

// The same with double-float inputs and outputs and no FP64 operation but
// VWN's atan and B88's asinh (the mixture coefficients are split by integer
// operations), where
// rho >= 1e-10 and, for a GGA (gga), sigma >= 1e-30.  Elsewhere it returns
// false without a result, and the caller evaluates the point with eval_xc on
// its FP64 inputs (a double-float sigma below FP32's range would be zero).
__device__ __forceinline__ bool eval_xc_mixed_f2(const FuncSet &fs, bool gga, fn::F2 rho,
                                                 fn::F2 sigma, fn::F2 &e, float &vrho,
                                                 float &vsigma) {
  if (!(rho.h >= 1e-10f) || (gga && !(sigma.h >= 1e-30f)))
    return false;
  fn::G r{rho, 1.f, 0.f};
  fn::G s{sigma, 0.f, 1.f};
  fn::RhoPowers<fn::G> P = fn::rho_powers(r);
  e = {0.f, 0.f};
  vrho = vsigma = 0.f;
  for (int i = 0; i < fs.n; i++) {
    const fn::F2 ci = fn::f2_bits(fs.coef[i]);
    fn::G c = fn::component(fs.id[i], r, s, P);
    e = fn::f2_add(e, fn::f2_mul(ci, c.v));
    vrho = fmaf(ci.h, c.r, vrho);
    vsigma = fmaf(ci.h, c.s, vsigma);
  }
  return true;
}

} // namespace occx
