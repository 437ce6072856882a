// CPU oracle: exchange-correlation functionals (unpolarised) -- TEST
// INFRASTRUCTURE ONLY.
//
// Restates the Libxc 6.2.2 functionals that OCC's methods name
// (share/methods/dft_methods.json; called through src/dft/functional.cpp:18-65)
// from the published papers.  Derivatives are taken by forward-mode dual
// numbers, so vrho/vsigma are exact derivatives of the energy density written
// here.
//
//   Slater exchange           P.A.M. Dirac, Proc. Camb. Phil. Soc. 26, 376 (1930)
//   VWN (CA and RPA fits)     Vosko, Wilk, Nusair, Can. J. Phys. 58, 1200 (1980)
//   B88 exchange              A.D. Becke, Phys. Rev. A 38, 3098 (1988)
//   LYP correlation           Lee, Yang, Parr, PRB 37, 785 (1988), in the
//                             density-gradient form of Miehlich, Savin, Stoll,
//                             Preuss, CPL 157, 200 (1989)
//   PBE exchange/correlation  Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996),
//                             with the PW92 LDA (Perdew, Wang, PRB 45, 13244
//                             (1992)) in the more-digits variant Libxc uses
//                             inside PBE.
//
// Libxc's lda_c_vwn_3 differs from lda_c_vwn only in its spin interpolation;
// for an unpolarised density both reduce to the VWN paramagnetic fit to the
// Ceperley-Alder data, which is what this file evaluates for id 30.
// Libxc zeroes every output where rho is below the functional's density
// threshold; we use 1e-15 for all functionals (not pinned against Libxc).
#include "xc_oracle.h"

#include <cmath>

namespace {

struct Dual {
  double v, dr, ds; // value, d/drho, d/dsigma
  Dual(double x = 0, double a = 0, double b = 0) : v(x), dr(a), ds(b) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.dr + b.dr, a.ds + b.ds}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.dr - b.dr, a.ds - b.ds}; }
inline Dual operator-(Dual a) { return {-a.v, -a.dr, -a.ds}; }
inline Dual operator*(Dual a, Dual b) {
  return {a.v * b.v, a.dr * b.v + a.v * b.dr, a.ds * b.v + a.v * b.ds};
}
inline Dual operator/(Dual a, Dual b) {
  double inv = 1.0 / b.v;
  double q = a.v * inv;
  return {q, (a.dr - q * b.dr) * inv, (a.ds - q * b.ds) * inv};
}
inline Dual operator*(double s, Dual a) { return {s * a.v, s * a.dr, s * a.ds}; }
inline Dual operator+(double s, Dual a) { return {s + a.v, a.dr, a.ds}; }
inline Dual operator-(double s, Dual a) { return {s - a.v, -a.dr, -a.ds}; }
inline Dual chain(Dual a, double f, double df) { return {f, df * a.dr, df * a.ds}; }
inline Dual dlog(Dual a) { return chain(a, std::log(a.v), 1.0 / a.v); }
inline Dual dexp(Dual a) {
  double e = std::exp(a.v);
  return chain(a, e, e);
}
inline Dual dsqrt(Dual a) {
  double s = std::sqrt(a.v);
  return chain(a, s, 0.5 / s);
}
inline Dual dpow(Dual a, double p) {
  double f = std::pow(a.v, p);
  return chain(a, f, p * f / a.v);
}
inline Dual datan(Dual a) { return chain(a, std::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
inline Dual dasinh(Dual a) {
  return chain(a, std::asinh(a.v), 1.0 / std::sqrt(1.0 + a.v * a.v));
}

const double kPi = 3.14159265358979323846;

// --- LDA pieces -----------------------------------------------------------
Dual slater(Dual rho) {
  const double cx = 0.75 * std::cbrt(3.0 / kPi);
  return -cx * dpow(rho, 4.0 / 3.0);
}

Dual rs_of(Dual rho) { return dpow((3.0 / (4.0 * kPi)) / rho, 1.0 / 3.0); }

// VWN interpolation formula, energy per particle as a function of rs.
Dual vwn_eps(Dual rs, double A, double b, double c, double x0) {
  Dual x = dsqrt(rs);
  Dual X = x * x + b * x + Dual(c);
  double X0 = x0 * x0 + b * x0 + c;
  double Q = std::sqrt(4.0 * c - b * b);
  Dual at = datan(Dual(Q) / (2.0 * x + Dual(b)));
  Dual t1 = dlog(x * x / X) + (2.0 * b / Q) * at;
  Dual xm = x - Dual(x0);
  Dual t2 = dlog(xm * xm / X) + (2.0 * (b + 2.0 * x0) / Q) * at;
  return A * (t1 - (b * x0 / X0) * t2);
}

Dual vwn5(Dual rho) { return rho * vwn_eps(rs_of(rho), 0.0310907, 3.72744, 12.9352, -0.10498); }
Dual vwn_rpa(Dual rho) { return rho * vwn_eps(rs_of(rho), 0.0310907, 13.0720, 42.7198, -0.409286); }

// PW92 correlation energy per particle, unpolarised, Libxc's "mod" digits.
Dual pw92_eps(Dual rs) {
  const double A = 0.0310907, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382,
               b4 = 0.49294;
  Dual srs = dsqrt(rs);
  Dual den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return -2.0 * A * (1.0 + a1 * rs) * dlog(1.0 + Dual(1.0) / den);
}

// --- GGA pieces -----------------------------------------------------------
Dual b88(Dual rho, Dual sigma) {
  const double beta = 0.0042;
  const double cs = 1.5 * std::cbrt(3.0 / (4.0 * kPi));
  Dual rs_ = 0.5 * rho;    // spin density
  Dual ss = 0.25 * sigma;  // |grad rho_s|^2
  Dual r43 = dpow(rs_, 4.0 / 3.0);
  Dual x2 = ss / (r43 * r43);
  Dual x = dsqrt(x2);
  Dual per_spin = -cs * r43 - beta * r43 * x2 / (1.0 + 6.0 * beta * x * dasinh(x));
  return 2.0 * per_spin;
}

Dual lyp(Dual rho, Dual sigma) {
  const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
  const double cf = 0.3 * std::pow(3.0 * kPi * kPi, 2.0 / 3.0);
  Dual rm13 = dpow(rho, -1.0 / 3.0);
  Dual den = 1.0 + d * rm13;
  Dual E = dexp(-c * rm13);
  Dual delta = c * rm13 + d * rm13 / den;
  Dual t1 = -a * rho / den;
  Dual t2 = -(a * b * cf) * rho * E / den;
  Dual t3 = (a * b / 72.0) * (3.0 + 7.0 * delta) * sigma * dpow(rho, -5.0 / 3.0) * E / den;
  return t1 + t2 + t3;
}

Dual pbe_x(Dual rho, Dual sigma) {
  const double kappa = 0.8040, mu = 0.2195149727645171;
  Dual kf = dpow(3.0 * kPi * kPi * rho, 1.0 / 3.0);
  Dual s2 = sigma / (4.0 * kf * kf * rho * rho);
  Dual F = (1.0 + kappa) - kappa / (1.0 + (mu / kappa) * s2);
  return slater(rho) * F;
}

Dual pbe_c(Dual rho, Dual sigma) {
  const double beta = 0.06672455060314922;
  const double gamma = (1.0 - std::log(2.0)) / (kPi * kPi);
  Dual rs = rs_of(rho);
  Dual eps = pw92_eps(rs);
  Dual kf = dpow(3.0 * kPi * kPi * rho, 1.0 / 3.0);
  Dual ks2 = (4.0 / kPi) * kf;
  Dual t2 = sigma / (4.0 * ks2 * rho * rho);
  Dual A = (beta / gamma) / (dexp(-eps / Dual(gamma)) - Dual(1.0));
  Dual At2 = A * t2;
  Dual H = gamma * dlog(1.0 + (beta / gamma) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return rho * (eps + H);
}

bool is_gga(int id) {
  switch (id) {
  case ORC_GGA_X_PBE:
  case ORC_GGA_X_B88:
  case ORC_GGA_C_PBE:
  case ORC_GGA_C_LYP:
  case ORC_HYB_GGA_XC_B3LYP:
  case ORC_HYB_GGA_XC_B3LYP5:
    return true;
  default:
    return false;
  }
}

bool known(int id) {
  switch (id) {
  case ORC_LDA_X:
  case ORC_LDA_C_VWN:
  case ORC_LDA_C_VWN_RPA:
  case ORC_LDA_C_VWN_3:
    return true;
  default:
    return is_gga(id);
  }
}

Dual energy_density(int id, Dual rho, Dual sigma) {
  switch (id) {
  case ORC_LDA_X:
    return slater(rho);
  case ORC_LDA_C_VWN:
  case ORC_LDA_C_VWN_3:
    return vwn5(rho);
  case ORC_LDA_C_VWN_RPA:
    return vwn_rpa(rho);
  case ORC_GGA_X_PBE:
    return pbe_x(rho, sigma);
  case ORC_GGA_C_PBE:
    return pbe_c(rho, sigma);
  case ORC_GGA_X_B88:
    return b88(rho, sigma);
  case ORC_GGA_C_LYP:
    return lyp(rho, sigma);
  case ORC_HYB_GGA_XC_B3LYP: // Libxc mixture: 0.08 S + 0.72 B88 + 0.19 VWN(RPA) + 0.81 LYP
    return 0.08 * slater(rho) + 0.72 * b88(rho, sigma) + 0.19 * vwn_rpa(rho) +
           0.81 * lyp(rho, sigma);
  case ORC_HYB_GGA_XC_B3LYP5: // same mixture with the VWN5 fit
    return 0.08 * slater(rho) + 0.72 * b88(rho, sigma) + 0.19 * vwn5(rho) +
           0.81 * lyp(rho, sigma);
  }
  return Dual(0.0);
}

} // namespace

extern "C" int oracle_functional_is_gga(int id) { return is_gga(id) ? 1 : 0; }

extern "C" int oracle_functional(int id, long n, const double *rho,
                                 const double *sigma, double *exc, double *vrho,
                                 double *vsigma) {
  if (!known(id))
    return -1;
  const bool gga = is_gga(id);
  const double dens_threshold = 1e-15;
  for (long i = 0; i < n; i++) {
    double r = rho[i];
    if (!(r >= dens_threshold)) {
      exc[i] = 0.0;
      vrho[i] = 0.0;
      if (gga && vsigma)
        vsigma[i] = 0.0;
      continue;
    }
    double s = gga ? std::fmax(sigma[i], 1e-40) : 0.0;
    Dual e = energy_density(id, Dual(r, 1.0, 0.0), Dual(s, 0.0, 1.0));
    exc[i] = e.v / r;
    vrho[i] = e.dr;
    if (gga && vsigma)
      vsigma[i] = e.ds;
  }
  return 0;
}
