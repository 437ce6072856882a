// CPU oracle: meta-GGA functionals -- TEST INFRASTRUCTURE ONLY.
//
// TPSS exchange and correlation, the Libxc 6.2.2 functionals mgga_x_tpss and
// mgga_c_tpss that OCC's "tpss" method names (share/methods/dft_methods.json),
// called through src/dft/functional.cpp:49-58 with rho, sigma, laplacian and
// tau.  Restated from the papers:
//   J. Tao, J.P. Perdew, V.N. Staroverov, G.E. Scuseria, PRL 91, 146401 (2003)
//     (exchange eqs. 4-10, correlation eqs. 11-14);
//   PBE correlation (PRL 77, 3865 (1996)) with the PW92 LDA in the same digits
//     as the GGA functionals of xc_oracle_functionals.cpp.
// The functional is written once, in the general spin-polarised form
// (rho_a, rho_b, s_aa, s_ab, s_bb, tau_a, tau_b); the unpolarised entry
// evaluates it at rho_a = rho_b = rho / 2, s_aa = s_ab = s_bb = sigma / 4,
// tau_a = tau_b = tau / 2.  Neither depends on the laplacian.
//
// Derivatives by the complex step (W. Squire, G. Trapp, SIAM Review 40, 110
// (1998)): f'(x) = Im f(x + i h) / h with h = 1e-25 |x| (a step relative to
// the argument: sigma can be 1e-40) is exact to rounding for the analytic
// pieces; max() and the thresholds select by the real part.
// This is independent of the dual numbers the GPU functional uses.
//
// Pinned against the reference's Libxc known answers (tests/dft_tests.cpp:
// 138-193; met to 4.3e-9), whose four points all sit on the sigma = 8 rho tau
// clamp below.  Other thresholds (not pinned against Libxc): the point is zero
// below a total density of 1e-15 (a spin channel's exchange below 1e-15);
// tau >= 1e-20; sigma >= 1e-40; as Libxc does for meta-GGAs, sigma is clamped
// to 8 rho tau (per spin channel when polarised) before evaluation, which
// keeps z = tau_W / tau <= 1; 1 +- zeta is kept >= DBL_EPSILON.
#include "xc_oracle.h"

#include <cmath>
#include <complex>

namespace {

using cd = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;
constexpr double kEpsZ = 2.220446049250313e-16;

inline cd cpow(cd z, double p) { return std::exp(p * std::log(z)); }
inline cd rmax(cd a, cd b) { return a.real() >= b.real() ? a : b; }
inline cd rmaxc(cd a, double lo) { return a.real() >= lo ? a : cd(lo, 0.0); }

// PW92 G(rs) of one fit
cd pw_g(cd rs, double A, double a1, double b1, double b2, double b3, double b4) {
  cd srs = std::sqrt(rs);
  cd den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return -2.0 * A * (1.0 + a1 * rs) * std::log(1.0 + 1.0 / den);
}

// PBE correlation energy per particle for spin densities (ra, rb) and total
// |grad rho|^2 = sig
cd pbe_c_eps(cd ra, cd rb, cd sig) {
  const double beta = 0.06672455060314922, gamma = 0.031090690869654897;
  const double fpp0 = 1.7099209341613657;
  cd n = ra + rb;
  cd z = (ra - rb) / n;
  cd opz = rmaxc(1.0 + z, kEpsZ), omz = rmaxc(1.0 - z, kEpsZ);
  cd rs = cpow(3.0 / (4.0 * kPi * n), 1.0 / 3.0);
  cd e0 = pw_g(rs, 0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294);
  cd e1 = pw_g(rs, 0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517);
  cd ac = -pw_g(rs, 0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671);
  cd f = (cpow(opz, 4.0 / 3.0) + cpow(omz, 4.0 / 3.0) - 2.0) / (std::pow(2.0, 4.0 / 3.0) - 2.0);
  cd z4 = z * z * z * z;
  cd eps = e0 + ac * f * (1.0 - z4) / fpp0 + (e1 - e0) * f * z4;
  cd phi = 0.5 * (cpow(opz, 2.0 / 3.0) + cpow(omz, 2.0 / 3.0));
  cd phi3 = phi * phi * phi;
  cd kf = cpow(3.0 * kPi * kPi * n, 1.0 / 3.0);
  cd ks2 = 4.0 * kf / kPi;
  cd t2 = sig / (4.0 * phi * phi * ks2 * n * n);
  cd A = (beta / gamma) / (std::exp(-eps / (gamma * phi3)) - 1.0);
  cd At2 = A * t2;
  cd H = gamma * phi3 * std::log(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return eps + H;
}

// TPSS exchange energy per volume of an unpolarised density (n, sigma, tau)
cd tpss_x_unpol(cd n, cd sig, cd tau) {
  const double kappa = 0.804, b = 0.40, c = 1.59096, e = 1.537, mu = 0.21951;
  const double k2 = std::pow(3.0 * kPi * kPi, 2.0 / 3.0);
  cd n13 = cpow(n, 1.0 / 3.0);
  cd n43 = n * n13, n53 = n43 * n13, n83 = n53 * n;
  cd p = sig / (4.0 * k2 * n83);
  cd tw = sig / (8.0 * n);
  cd z = tw / tau;
  cd alpha = (tau - tw) / (0.3 * k2 * n53);
  cd qb = 0.45 * (alpha - 1.0) / std::sqrt(1.0 + b * alpha * (alpha - 1.0)) + 2.0 * p / 3.0;
  cd z2 = z * z;
  cd opz2 = 1.0 + z2;
  cd tz = 0.6 * z; // 3 z / 5
  const double se = std::sqrt(e);
  cd num = (10.0 / 81.0 + c * z2 / (opz2 * opz2)) * p + (146.0 / 2025.0) * qb * qb -
           (73.0 / 405.0) * qb * std::sqrt(0.5 * tz * tz + 0.5 * p * p) +
           (1.0 / kappa) * (10.0 / 81.0) * (10.0 / 81.0) * p * p +
           2.0 * se * (10.0 / 81.0) * tz * tz + e * mu * p * p * p;
  cd den = (1.0 + se * p) * (1.0 + se * p);
  cd x = num / den;
  cd Fx = 1.0 + kappa - kappa / (1.0 + x / kappa);
  const double cx = 0.75 * std::cbrt(3.0 / kPi);
  return -cx * n43 * Fx;
}

// TPSS exchange of a polarised density: (E_x[2 rho_a] + E_x[2 rho_b]) / 2
cd tpss_x_pol(cd ra, cd rb, cd saa, cd sbb, cd ta, cd tb) {
  cd e = 0.0;
  if (ra.real() >= 1e-15)
    e += 0.5 * tpss_x_unpol(2.0 * ra, 4.0 * saa, 2.0 * ta);
  if (rb.real() >= 1e-15)
    e += 0.5 * tpss_x_unpol(2.0 * rb, 4.0 * sbb, 2.0 * tb);
  return e;
}

// TPSS correlation energy per volume (revPKZB, eqs. 11-14)
cd tpss_c_pol(cd ra, cd rb, cd saa, cd sab, cd sbb, cd ta, cd tb) {
  const double d = 2.8;
  cd n = ra + rb;
  cd sig = saa + 2.0 * sab + sbb;
  cd tau = ta + tb;
  cd z = sig / (8.0 * n * tau); // tau_W / tau of the total density
  cd zeta = (ra - rb) / n;
  cd opz = rmaxc(1.0 + zeta, kEpsZ), omz = rmaxc(1.0 - zeta, kEpsZ);
  cd n2 = n * n;
  cd gz2 = 4.0 * (rb * rb * saa - 2.0 * ra * rb * sab + ra * ra * sbb) / (n2 * n2); // |grad zeta|^2
  cd xi2 = gz2 / (4.0 * cpow(3.0 * kPi * kPi * n, 2.0 / 3.0));
  cd zt2 = zeta * zeta;
  cd C0 = 0.53 + 0.87 * zt2 + 0.50 * zt2 * zt2 + 2.26 * zt2 * zt2 * zt2;
  cd g = 1.0 + 0.5 * xi2 * (cpow(opz, -4.0 / 3.0) + cpow(omz, -4.0 / 3.0));
  cd C = C0 / (g * g * g * g);
  cd epbe = pbe_c_eps(ra, rb, sig);
  cd sum = 0.0;
  if (ra.real() >= 1e-15)
    sum += ra / n * rmax(pbe_c_eps(ra, cd(0.0), saa), epbe);
  if (rb.real() >= 1e-15)
    sum += rb / n * rmax(pbe_c_eps(rb, cd(0.0), sbb), epbe);
  cd z2 = z * z;
  cd erev = epbe * (1.0 + C * z2) - (1.0 + C) * z2 * sum;
  return n * erev * (1.0 + d * erev * z2 * z);
}

cd mgga_component(int id, cd ra, cd rb, cd saa, cd sab, cd sbb, cd ta, cd tb) {
  switch (id) {
  case ORC_MGGA_X_TPSS:
    return tpss_x_pol(ra, rb, saa, sbb, ta, tb);
  case ORC_MGGA_C_TPSS:
    return tpss_c_pol(ra, rb, saa, sab, sbb, ta, tb);
  }
  return 0.0;
}

constexpr double kH = 1e-25; // relative complex step
inline double step(double x) { return kH * std::fmax(std::fabs(x), 1e-280); }

} // namespace

extern "C" int oracle_functional_is_mgga(int id) {
  return (id == ORC_MGGA_X_TPSS || id == ORC_MGGA_C_TPSS) ? 1 : 0;
}

extern "C" int oracle_functional_mgga(int id, long n, const double *rho, const double *sigma,
                                      const double *tau, double *exc, double *vrho,
                                      double *vsigma, double *vtau) {
  if (!oracle_functional_is_mgga(id))
    return -1;
  for (long i = 0; i < n; i++) {
    exc[i] = vrho[i] = vsigma[i] = vtau[i] = 0.0;
    const double r = rho[i];
    if (!(r >= 1e-15))
      continue;
    const double t = std::fmax(tau[i], 1e-20);
    const double s = std::fmin(std::fmax(sigma[i], 1e-40), 8.0 * r * t);
    auto f = [&](cd R, cd S, cd T) {
      return mgga_component(id, 0.5 * R, 0.5 * R, 0.25 * S, 0.25 * S, 0.25 * S, 0.5 * T, 0.5 * T);
    };
    const double hr = step(r), hs = step(s), ht = step(t);
    const cd fr = f(cd(r, hr), s, t);
    const cd fs = f(r, cd(s, hs), t);
    const cd ft = f(r, s, cd(t, ht));
    exc[i] = fr.real() / r;
    vrho[i] = fr.imag() / hr;
    vsigma[i] = fs.imag() / hs;
    vtau[i] = ft.imag() / ht;
  }
  return 0;
}

extern "C" int oracle_functional_mgga_polarized(int id, long n, const double *ra,
                                                const double *rb, const double *saa,
                                                const double *sab, const double *sbb,
                                                const double *ta, const double *tb, double *exc,
                                                double *vr, double *vs, double *vt) {
  if (!oracle_functional_is_mgga(id))
    return -1;
  for (long i = 0; i < n; i++) {
    double x[7];
    x[0] = std::fmax(ra[i], 0.0);
    x[1] = std::fmax(rb[i], 0.0);
    x[5] = std::fmax(ta[i], 1e-20);
    x[6] = std::fmax(tb[i], 1e-20);
    x[2] = std::fmin(std::fmax(saa[i], 1e-40), 8.0 * x[0] * x[5]);
    x[4] = std::fmin(std::fmax(sbb[i], 1e-40), 8.0 * x[1] * x[6]);
    x[3] = sab[i];
    const double lim = 0.5 * (x[2] + x[4]);
    x[3] = std::fmin(std::fmax(x[3], -lim), lim);
    exc[i] = 0.0;
    for (int k = 0; k < 2; k++)
      vr[2 * i + k] = vt[2 * i + k] = 0.0;
    for (int k = 0; k < 3; k++)
      vs[3 * i + k] = 0.0;
    const double nt = x[0] + x[1];
    if (!(nt >= 1e-15))
      continue;
    double d[7];
    double e = 0.0;
    for (int k = 0; k < 7; k++) {
      const double h = step(x[k]);
      cd y[7];
      for (int j = 0; j < 7; j++)
        y[j] = cd(x[j], j == k ? h : 0.0);
      const cd v = mgga_component(id, y[0], y[1], y[2], y[3], y[4], y[5], y[6]);
      e = v.real();
      d[k] = v.imag() / h;
    }
    exc[i] = e / nt;
    vr[2 * i] = d[0];
    vr[2 * i + 1] = d[1];
    vs[3 * i] = d[2];
    vs[3 * i + 1] = d[3];
    vs[3 * i + 2] = d[4];
    vt[2 * i] = d[5];
    vt[2 * i + 1] = d[6];
  }
  return 0;
}
