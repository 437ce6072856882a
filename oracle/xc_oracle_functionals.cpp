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
  case ORC_HYB_GGA_XC_PBEH:
  case ORC_HYB_GGA_XC_BHANDH:
  case ORC_HYB_GGA_XC_BHANDHLYP:
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
  // Libxc's hybrid mixtures of OCC's pbeh, bhandh and bhandhlyp (their
  // Hartree-Fock share is outside the XC build)
  case ORC_HYB_GGA_XC_PBEH: // 0.75 PBE exchange + PBE correlation
    return 0.75 * pbe_x(rho, sigma) + pbe_c(rho, sigma);
  case ORC_HYB_GGA_XC_BHANDH: // 0.5 Slater + LYP
    return 0.5 * slater(rho) + lyp(rho, sigma);
  case ORC_HYB_GGA_XC_BHANDHLYP: // 0.5 B88 + LYP
    return 0.5 * b88(rho, sigma) + lyp(rho, sigma);
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

// ---------------------------------------------------------------------------
// Spin-polarised forms (the UKS build, m_method.functionals_polarized,
// include/occ/dft/dft.h:207-209), restated from the same papers:
//   exchange (Slater, B88, PBE) by the exact spin scaling
//     E_x[rho_a, rho_b] = (E_x[2 rho_a] + E_x[2 rho_b]) / 2;
//   VWN: eps = eps_P + alpha_c f(z)/f''(0) (1 - z^4) + (eps_F - eps_P) f(z) z^4
//     (VWN 1980, CA and RPA fits; VWN3 scales the RPA spin stiffness by the
//     CA / RPA polarisation energies);
//   PW92: the same interpolation with alpha_c = -G(rs) of its third fit, in
//     PBE correlation with phi(z) = ((1+z)^(2/3) + (1-z)^(2/3)) / 2;
//   LYP: Miehlich, Savin, Stoll, Preuss, CPL 157, 200 (1989), eq. 2.
// Derivatives by the complex step, dE/dx = Im E(x + i h) / h with h = 1e-30
// (W. Squire, G. Trapp, SIAM Review 40, 110 (1998)), exact to rounding for
// these analytic forms and independent of dual-number code.
#include <complex>

namespace {

using Cx = std::complex<double>;
const double kEps = 2.220446049250313e-16;

Cx c13(Cx x) { return std::pow(x, 1.0 / 3.0); }
Cx p43(Cx x) { return std::pow(x, 4.0 / 3.0); }

Cx vwn_fit_c(Cx rs, double A, double b, double c, double x0) {
  Cx x = std::sqrt(rs);
  Cx X = x * x + b * x + c;
  double X0 = x0 * x0 + b * x0 + c;
  double Q = std::sqrt(4.0 * c - b * b);
  Cx at = std::atan(Q / (2.0 * x + b));
  Cx t1 = std::log(x * x / X) + (2.0 * b / Q) * at;
  Cx t2 = std::log((x - x0) * (x - x0) / X) + (2.0 * (b + 2.0 * x0) / Q) * at;
  return A * (t1 - (b * x0 / X0) * t2);
}

Cx pw_g_c(Cx rs, double A, double a1, double b1, double b2, double b3, double b4) {
  Cx srs = std::sqrt(rs);
  Cx den = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return -2.0 * A * (1.0 + a1 * rs) * std::log(1.0 + 1.0 / den);
}

struct PolPoint {
  Cx ra, rb, saa, sab, sbb;
  bool sa, sb; // spin channel above the density threshold
};

Cx slater_c(Cx r) { return -0.75 * std::cbrt(3.0 / kPi) * std::cbrt(2.0) * p43(r); }
Cx b88_c(Cx r, Cx s) {
  const double beta = 0.0042, cs = 1.5 * std::cbrt(3.0 / (4.0 * kPi));
  Cx r43 = p43(r);
  Cx x = std::sqrt(s) / r43;
  return -cs * r43 - beta * r43 * x * x / (1.0 + 6.0 * beta * x * std::asinh(x));
}
Cx pbe_x_c(Cx r, Cx s) { // E_x^PBE[2 r, 4 s] / 2
  const double kappa = 0.8040, mu = 0.2195149727645171;
  Cx n = 2.0 * r;
  Cx kf = c13(3.0 * kPi * kPi * n);
  Cx s2 = 4.0 * s / (4.0 * kf * kf * n * n);
  Cx F = (1.0 + kappa) - kappa / (1.0 + (mu / kappa) * s2);
  return 0.5 * (-0.75 * std::cbrt(3.0 / kPi) * p43(n) * F);
}

Cx pol_energy(int id, const PolPoint &P) {
  Cx rho = P.ra + P.rb;
  Cx z = (P.ra - P.rb) / rho;
  Cx opz = 1.0 + z, omz = 1.0 - z;
  if (opz.real() < kEps)
    opz = kEps;
  if (omz.real() < kEps)
    omz = kEps;
  const double fpp = 4.0 / (9.0 * (std::cbrt(2.0) - 1.0));
  Cx f = (p43(opz) + p43(omz) - 2.0) / (std::pow(2.0, 4.0 / 3.0) - 2.0);
  Cx z4 = z * z * z * z;
  Cx rs = c13(3.0 / (4.0 * kPi * rho));
  auto X = [&](Cx (*fx)(Cx, Cx)) {
    Cx e = 0.0;
    if (P.sa)
      e += fx(P.ra, P.saa);
    if (P.sb)
      e += fx(P.rb, P.sbb);
    return e;
  };
  auto slater = [&] {
    Cx e = 0.0;
    if (P.sa)
      e += slater_c(P.ra);
    if (P.sb)
      e += slater_c(P.rb);
    return e;
  };
  const double Avwn[3] = {0.0310907, 0.01554535, -1.0 / (6.0 * kPi * kPi)};
  const double bca[3] = {3.72744, 7.06042, 1.13107}, cca[3] = {12.9352, 18.0578, 13.0045},
               xca[3] = {-0.10498, -0.32500, -0.0047584};
  const double brp[3] = {13.0720, 20.1231, 1.06835}, crp[3] = {42.7198, 101.578, 11.4813},
               xrp[3] = {-0.409286, -0.743294, -0.228344};
  auto vwn = [&](int variant) {
    if (variant < 2) {
      const double *b = variant == 0 ? bca : brp, *c = variant == 0 ? cca : crp,
                   *x0 = variant == 0 ? xca : xrp;
      Cx eP = vwn_fit_c(rs, Avwn[0], b[0], c[0], x0[0]);
      Cx eF = vwn_fit_c(rs, Avwn[1], b[1], c[1], x0[1]);
      Cx ac = vwn_fit_c(rs, Avwn[2], b[2], c[2], x0[2]);
      return rho * (eP + ac * f / fpp * (1.0 - z4) + (eF - eP) * f * z4);
    }
    Cx eP = vwn_fit_c(rs, Avwn[0], bca[0], cca[0], xca[0]);
    Cx dca = vwn_fit_c(rs, Avwn[1], bca[1], cca[1], xca[1]) - eP;
    Cx drpa = vwn_fit_c(rs, Avwn[1], brp[1], crp[1], xrp[1]) -
              vwn_fit_c(rs, Avwn[0], brp[0], crp[0], xrp[0]);
    Cx ar = vwn_fit_c(rs, Avwn[2], brp[2], crp[2], xrp[2]);
    return rho * (eP + ar * f / fpp * (1.0 - z4) * dca / drpa + dca * f * z4);
  };
  auto lyp = [&] {
    const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
    const double cf = 0.3 * std::pow(3.0 * kPi * kPi, 2.0 / 3.0);
    Cx rm13 = 1.0 / c13(rho);
    Cx den = 1.0 + d * rm13;
    Cx omega = std::exp(-c * rm13) / den * std::pow(rho, -11.0 / 3.0);
    Cx delta = c * rm13 + d * rm13 / den;
    Cx gg = P.saa + 2.0 * P.sab + P.sbb;
    Cx ab = P.ra * P.rb;
    auto p83 = [](Cx x) { return x.real() > 0.0 ? std::pow(x, 8.0 / 3.0) : Cx(0.0); };
    Cx br = std::pow(2.0, 11.0 / 3.0) * cf * (p83(P.ra) + p83(P.rb)) +
            (47.0 / 18.0 - 7.0 / 18.0 * delta) * gg - (2.5 - delta / 18.0) * (P.saa + P.sbb) -
            (delta - 11.0) / 9.0 * (P.ra / rho * P.saa + P.rb / rho * P.sbb);
    Cx rest = -2.0 / 3.0 * rho * rho * gg + (2.0 / 3.0 * rho * rho - P.ra * P.ra) * P.sbb +
              (2.0 / 3.0 * rho * rho - P.rb * P.rb) * P.saa;
    return -4.0 * a / den * ab / rho - a * b * omega * (ab * br + rest);
  };
  auto pbe_c = [&] {
    const double beta = 0.06672455060314922, gamma = (1.0 - std::log(2.0)) / (kPi * kPi);
    Cx e0 = pw_g_c(rs, 0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294);
    Cx e1 = pw_g_c(rs, 0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517);
    Cx ac = -pw_g_c(rs, 0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671);
    Cx eps = e0 + ac * f / fpp * (1.0 - z4) + (e1 - e0) * f * z4;
    Cx phi = 0.5 * (std::pow(opz, 2.0 / 3.0) + std::pow(omz, 2.0 / 3.0));
    Cx phi3 = phi * phi * phi;
    Cx kf = c13(3.0 * kPi * kPi * rho);
    Cx ks2 = 4.0 / kPi * kf;
    Cx t2 = (P.saa + 2.0 * P.sab + P.sbb) / (4.0 * phi * phi * ks2 * rho * rho);
    Cx A = beta / gamma / (std::exp(-eps / (gamma * phi3)) - 1.0);
    Cx At2 = A * t2;
    Cx H = gamma * phi3 * std::log(1.0 + beta / gamma * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
    return rho * (eps + H);
  };
  switch (id) {
  case ORC_LDA_X: return slater();
  case ORC_LDA_C_VWN: return vwn(0);
  case ORC_LDA_C_VWN_RPA: return vwn(1);
  case ORC_LDA_C_VWN_3: return vwn(2);
  case ORC_GGA_X_PBE: return X(pbe_x_c);
  case ORC_GGA_C_PBE: return pbe_c();
  case ORC_GGA_X_B88: return X(b88_c);
  case ORC_GGA_C_LYP: return lyp();
  case ORC_HYB_GGA_XC_B3LYP:
    return 0.08 * slater() + 0.72 * X(b88_c) + 0.19 * vwn(1) + 0.81 * lyp();
  case ORC_HYB_GGA_XC_B3LYP5:
    return 0.08 * slater() + 0.72 * X(b88_c) + 0.19 * vwn(0) + 0.81 * lyp();
  case ORC_HYB_GGA_XC_PBEH:
    return 0.75 * X(pbe_x_c) + pbe_c();
  case ORC_HYB_GGA_XC_BHANDH:
    return 0.5 * slater() + lyp();
  case ORC_HYB_GGA_XC_BHANDHLYP:
    return 0.5 * X(b88_c) + lyp();
  }
  return 0.0;
}

} // namespace

// Polarised evaluation at n points: rho_a, rho_b, s_aa, s_ab, s_bb in;
// exc (per particle), vrho_a, vrho_b, vs_aa, vs_ab, vs_bb out (the sigma
// arrays and outputs may be NULL for an LDA).
extern "C" int oracle_functional_polarized(int id, long n, const double *ra, const double *rb,
                                           const double *saa, const double *sab,
                                           const double *sbb, double *exc, double *vra,
                                           double *vrb, double *vsaa, double *vsab,
                                           double *vsbb) {
  if (!known(id))
    return -1;
  const bool gga = is_gga(id);
  const double h = 1e-30;
  for (long i = 0; i < n; i++) {
    const double a = std::fmax(ra[i], 0.0), b = std::fmax(rb[i], 0.0);
    double x[5] = {a, b, gga ? std::fmax(saa[i], 1e-40) : 0.0, gga ? sab[i] : 0.0,
                   gga ? std::fmax(sbb[i], 1e-40) : 0.0};
    double out[6] = {0, 0, 0, 0, 0, 0};
    if (a + b >= 1e-15) {
      for (int k = -1; k < (gga ? 5 : 2); k++) {
        PolPoint P{x[0], x[1], x[2], x[3], x[4], a >= 1e-15, b >= 1e-15};
        Cx *v[5] = {&P.ra, &P.rb, &P.saa, &P.sab, &P.sbb};
        if (k >= 0)
          *v[k] += Cx(0.0, h);
        Cx e = pol_energy(id, P);
        if (k < 0)
          out[0] = e.real() / (a + b);
        else
          out[1 + k] = e.imag() / h;
      }
    }
    exc[i] = out[0];
    vra[i] = out[1];
    vrb[i] = out[2];
    if (gga) {
      if (vsaa)
        vsaa[i] = out[3];
      if (vsab)
        vsab[i] = out[4];
      if (vsbb)
        vsbb[i] = out[5];
    }
  }
  return 0;
}
