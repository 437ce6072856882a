// Basis normalisation, solid-harmonic transforms and host shell evaluation.
#include "gto_eval.h"
#include "xc_host.hpp"

#include <cmath>
#include <mutex>
#include <stdexcept>

namespace occx {

namespace {
const double kPi = 3.14159265358979323846;

// src/gto/shell.cpp:20-23: integral of r^n exp(-alpha r^2) over r in [0, inf).
double gint(int n, double alpha) {
  double n1_2 = 0.5 * (n + 1);
  return std::tgamma(n1_2) / (2.0 * std::pow(alpha, n1_2));
}

double fact(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; i++)
    r *= i;
  return r;
}
double choose(int n, int k) {
  if (k < 0 || k > n)
    return 0.0;
  return fact(n) / (fact(k) * fact(n - k));
}
} // namespace

void normalize_shell(int l, int nprim, const double *exps, double *coefs) {
  // primitive normalisation: gto_norm (src/gto/shell.cpp:35-50)
  for (int i = 0; i < nprim; i++)
    coefs[i] *= 1.0 / std::sqrt(gint(2 * l + 2, 2.0 * exps[i]));
  // contraction normalisation (src/gto/shell.cpp:52-64)
  double s = 0.0;
  for (int i = 0; i < nprim; i++)
    for (int j = 0; j < nprim; j++)
      s += coefs[i] * gint(2 * l + 2, exps[i] + exps[j]) * coefs[j];
  double f = 1.0 / std::sqrt(s);
  for (int i = 0; i < nprim; i++)
    coefs[i] *= f;
}

double common_fac(int l, bool pure) {
  if (l == 0)
    return 0.282094791773878143;
  if (l == 1)
    return 0.488602511902919921;
  return pure ? std::sqrt((2 * l + 1) / (4 * kPi)) : 1.0;
}

// Real solid harmonics S_lm (Helgaker, Jorgensen, Olsen, Molecular
// Electronic-Structure Theory, eq. 6.4.47): for m >= 0 the cosine-type and for
// m < 0 the sine-type combinations, listed m = -l..l (CCA order).
const std::vector<double> &spherical_transform(int l) {
  static std::vector<double> tables[kMaxL + 1];
  static std::once_flag once;
  std::call_once(once, [] {
    for (int L = 0; L <= kMaxL; L++) {
      int nc = ncart_of(L);
      std::vector<double> T((2 * L + 1) * nc, 0.0);
      for (int m = -L; m <= L; m++) {
        int am = m < 0 ? -m : m;
        double N = std::sqrt(2.0 * fact(L + am) * fact(L - am) / (m == 0 ? 2.0 : 1.0)) /
                   (std::pow(2.0, am) * fact(L));
        // v runs over integers (m >= 0) or half-integers (m < 0); k = 2v
        int k_lo = m < 0 ? 1 : 0;
        for (int t = 0; t <= (L - am) / 2; t++)
          for (int u = 0; u <= t; u++)
            for (int k = k_lo; k <= am; k += 2) {
              double sign = ((t + (k - k_lo) / 2) & 1) ? -1.0 : 1.0;
              double c = sign * std::pow(0.25, t) * choose(L, t) * choose(L - t, am + t) *
                         choose(t, u) * choose(am, k);
              int ex = 2 * t + am - 2 * u - k, ey = 2 * u + k, ez = L - 2 * t - am;
              // CCA index of x^ex y^ey z^ez
              int idx = 0;
              for (int a = L; a > ex; a--)
                idx += L - a + 1;
              idx += L - ex - ey;
              (void)ez;
              T[(m + L) * nc + idx] += N * c;
            }
      }
      tables[L] = T;
    }
  });
  if (l < 0 || l > kMaxL)
    throw std::runtime_error("angular momentum above 4 is not supported");
  return tables[l];
}

void Basis::finalise() {
  first_bf.resize(shells.size());
  nbf = 0;
  lmax = 0;
  for (size_t s = 0; s < shells.size(); s++) {
    first_bf[s] = nbf;
    nbf += shell_size(static_cast<int>(s));
    lmax = std::max(lmax, shells[s].l);
  }
}

void eval_shell_values(const Shell &sh, bool pure, long n, const double *xyz, double *out) {
  const int l = sh.l, nc = ncart_of(l);
  const int nf = pure ? 2 * l + 1 : nc;
  const double fac = common_fac(l, pure);
  const std::vector<double> &T = spherical_transform(l);
  double cart[ncart_of(kMaxL)];
  for (long p = 0; p < n; p++) {
    double x = xyz[3 * p] - sh.origin[0], y = xyz[3 * p + 1] - sh.origin[1],
           z = xyz[3 * p + 2] - sh.origin[2];
    double r2 = x * x + y * y + z * z, R = 0.0;
    for (size_t k = 0; k < sh.exps.size(); k++)
      R += sh.coefs[k] * std::exp(-sh.exps[k] * r2);
    cart_eval<double>(l, x, y, z, R, 0.0, cart, nullptr, nullptr, nullptr);
    for (int f = 0; f < nf; f++) {
      double v;
      if (pure) {
        v = 0.0;
        for (int c = 0; c < nc; c++)
          v += T[f * nc + c] * cart[c];
      } else {
        v = cart[f];
      }
      out[f * n + p] = v * fac;
    }
  }
}

} // namespace occx
