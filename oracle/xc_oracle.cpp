// CPU oracle for the restricted Kohn-Sham XC build -- TEST INFRASTRUCTURE
// ONLY (see xc_oracle.h).  Every step cites the reference code it restates.
#include "gemm.h"
#include "xc_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = 3.14159265358979323846;

// src/gto/gto.cpp:7-16
double common_fac(int l, bool pure) {
  if (l == 0)
    return 0.282094791773878143;
  if (l == 1)
    return 0.488602511902919921;
  return pure ? std::sqrt((2 * l + 1) / (4 * kPi)) : 1.0;
}

double factorial(int n) {
  double r = 1;
  for (int i = 2; i <= n; i++)
    r *= i;
  return r;
}
double binom(int n, int k) {
  if (k < 0 || k > n)
    return 0.0;
  return factorial(n) / (factorial(k) * factorial(n - k));
}

int ncart(int l) { return (l + 1) * (l + 2) / 2; }
// Position of x^a y^b z^(l-a-b) in CCA order (xx, xy, xz, yy, yz, zz, ...).
int cart_index(int l, int a, int b) {
  int idx = 0;
  for (int aa = l; aa > a; aa--)
    idx += l - aa + 1;
  return idx + (l - a - b);
}

// Real solid harmonics in CCA order m = -l..l as combinations of Cartesian
// monomials (Helgaker, Jorgensen, Olsen, Molecular Electronic-Structure
// Theory, eqs. 6.4.47-6.4.50).  This is the convention gau2grid's
// GG_SPHERICAL_CCA transform follows (src/3rdparty/gau2grid).
std::vector<double> spherical_transform(int l) {
  int nc = ncart(l), ns = 2 * l + 1;
  std::vector<double> T(ns * nc, 0.0);
  for (int m = -l; m <= l; m++) {
    int am = std::abs(m);
    double N = 1.0 / (std::pow(2.0, am) * factorial(l)) *
               std::sqrt(2.0 * factorial(l + am) * factorial(l - am) / (m == 0 ? 2.0 : 1.0));
    int v2_lo = (m < 0) ? 1 : 0;
    int v2_hi = (m < 0) ? 2 * ((am - 1) / 2) + 1 : 2 * (am / 2);
    for (int t = 0; t <= (l - am) / 2; t++)
      for (int u = 0; u <= t; u++)
        for (int v2 = v2_lo; v2 <= v2_hi; v2 += 2) {
          int sgn_exp = t + (v2 - v2_lo) / 2;
          double C = ((sgn_exp % 2) ? -1.0 : 1.0) * std::pow(0.25, t) * binom(l, t) *
                     binom(l - t, am + t) * binom(t, u) * binom(am, v2);
          int ex = 2 * t + am - 2 * u - v2;
          int ey = 2 * u + v2;
          int ez = l - 2 * t - am;
          if (ex < 0 || ey < 0 || ez < 0)
            continue;
          T[(m + l) * nc + cart_index(l, ex, ey)] += N * C;
        }
  }
  return T;
}

inline double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; i++)
    r *= x;
  return r;
}

// d^k/dx^k of x^a (k = 0, 1, 2), 0 where the power runs out.
inline double dpow(double x, int a, int k) {
  if (k == 0)
    return ipow(x, a);
  if (k == 1)
    return a > 0 ? a * ipow(x, a - 1) : 0.0;
  return a > 1 ? a * (a - 1) * ipow(x, a - 2) : 0.0;
}

// Collocation of one shell at points; out[comp][func][p], comp 0 = value,
// 1..3 = d/dx, d/dy, d/dz and, for deriv 2, 4..9 = d2/dxx, dxy, dxz, dyy,
// dyz, dzz (the order of OCC's GTOValues).  Restates what src/gto/gto.cpp
// :212-287 obtains from gau2grid (contracted Cartesian Gaussians, CCA order,
// optional spherical transform) including the common_fac scaling.  With the
// radial part R(s), s = r^2, dR = 2 R'(s) and d2R = 4 R''(s), the second
// derivatives of M(x, y, z) R are M_ij R + (M_i x_j + M_j x_i) dR
// + M (x_i x_j d2R + delta_ij dR).
void collocate(int l, bool pure, int nprim, const double *exps, const double *coefs,
               const double *A, long n, const double *xyz, long stride, int deriv,
               double *out, long out_stride) {
  const int nc = ncart(l);
  const int nf = pure ? 2 * l + 1 : nc;
  std::vector<double> T;
  if (pure)
    T = spherical_transform(l);
  const double fac = common_fac(l, pure);
  // the shell's Cartesian components in CCA order, hoisted out of the point loop
  struct Comp {
    int a, b, c, i;
  };
  std::vector<Comp> comps;
  for (int a = l; a >= 0; a--)
    for (int b = l - a; b >= 0; b--)
      comps.push_back({a, b, l - a - b, cart_index(l, a, b)});
  std::vector<double> cart(10 * nc);
  static const int hi[6] = {0, 0, 0, 1, 1, 2}, hj[6] = {0, 1, 2, 1, 2, 2};
  const int ncomp = deriv > 1 ? 10 : (deriv ? 4 : 1);
  double xp[8], yp[8], zp[8]; // powers 0..l (l <= 6), built by repeated products
  for (long p = 0; p < n; p++) {
    double x = xyz[3 * p] - A[0], y = xyz[3 * p + 1] - A[1], z = xyz[3 * p + 2] - A[2];
    double r2 = x * x + y * y + z * z;
    double R = 0.0, dR = 0.0, d2R = 0.0;
    for (int k = 0; k < nprim; k++) {
      double e = coefs[k] * std::exp(-exps[k] * r2);
      R += e;
      if (deriv) {
        dR += -2.0 * exps[k] * e;
        if (deriv > 1)
          d2R += 4.0 * exps[k] * exps[k] * e;
      }
    }
    xp[0] = yp[0] = zp[0] = 1.0;
    for (int k = 1; k <= l; k++) {
      xp[k] = xp[k - 1] * x;
      yp[k] = yp[k - 1] * y;
      zp[k] = zp[k - 1] * z;
    }
    const double r[3] = {x, y, z};
    for (const Comp &cp : comps) {
      const int a = cp.a, b = cp.b, c = cp.c, i = cp.i;
      double mono = xp[a] * yp[b] * zp[c];
      cart[i] = mono * R;
      if (deriv) {
        double gx = (a > 0 ? a * xp[a - 1] * yp[b] * zp[c] : 0.0);
        double gy = (b > 0 ? b * xp[a] * yp[b - 1] * zp[c] : 0.0);
        double gz = (c > 0 ? c * xp[a] * yp[b] * zp[c - 1] : 0.0);
        cart[nc + i] = gx * R + mono * x * dR;
        cart[2 * nc + i] = gy * R + mono * y * dR;
        cart[3 * nc + i] = gz * R + mono * z * dR;
        if (deriv > 1) {
          const double M1[3] = {gx, gy, gz};
          const int pw[3] = {a, b, c};
          for (int q = 0; q < 6; q++) {
            const int u = hi[q], v = hj[q];
            int k[3] = {0, 0, 0};
            k[u]++;
            k[v]++;
            const double Mij = dpow(x, pw[0], k[0]) * dpow(y, pw[1], k[1]) * dpow(z, pw[2], k[2]);
            cart[(4 + q) * nc + i] = Mij * R + (M1[u] * r[v] + M1[v] * r[u]) * dR +
                                     mono * (r[u] * r[v] * d2R + (u == v ? dR : 0.0));
          }
        }
      }
    }
    for (int q = 0; q < ncomp; q++)
      for (int f = 0; f < nf; f++) {
        double v;
        if (pure) {
          v = 0.0;
          for (int i = 0; i < nc; i++)
            v += T[f * nc + i] * cart[q * nc + i];
        } else {
          v = cart[q * nc + f];
        }
        out[(q * nf + f) * out_stride + p] = v * fac;
      }
  }
}

struct Basis {
  int nsh;
  const int *l, *nprim, *off;
  const double *exps, *coefs, *origin;
  bool pure;
  std::vector<int> first_bf;
  int nbf;
  int size(int s) const { return pure ? 2 * l[s] + 1 : ncart(l[s]); }
};

// src/gto/gto.cpp:18-67: first radius (0.5 .. 30 Bohr in 0.1 steps, along
// +x from the shell centre) where max |phi| drops below the threshold.
void decay_cutoff(const Basis &bs, double threshold, double *ext) {
  const double max_radius = 30.0, increment = 0.1, min_radius = 0.5;
  const int npts = static_cast<int>((max_radius - min_radius) / increment) + 1;
  const double step = (max_radius - min_radius) / (npts - 1); // Eigen LinSpaced
  std::vector<double> xyz(3 * npts);
  for (int s = 0; s < bs.nsh; s++) {
    const double *A = bs.origin + 3 * s;
    for (int i = 0; i < npts; i++) {
      double xi = (i == npts - 1) ? max_radius : min_radius + i * step;
      xyz[3 * i] = xi + A[0];
      xyz[3 * i + 1] = 0.0 + A[1];
      xyz[3 * i + 2] = 0.0 + A[2];
    }
    int nf = bs.size(s);
    std::vector<double> vals(nf * npts);
    collocate(bs.l[s], bs.pure, bs.nprim[s], bs.exps + bs.off[s], bs.coefs + bs.off[s], A,
              npts, xyz.data(), 3, 0, vals.data(), npts);
    for (int i = 0; i < npts; i++) {
      ext[s] = i * increment + min_radius;
      double v = 0.0;
      for (int f = 0; f < nf; f++)
        v = std::max(v, std::fabs(vals[f * npts + i]));
      if (v < threshold)
        break;
    }
  }
}

// src/numint/spatial_grid_hierarchy.cpp:7-31 (bit dilation, 21 bits/axis)
inline uint64_t dilate3(uint64_t x) {
  x &= 0x1fffff;
  x = (x | (x << 32)) & 0x1f00000000ffffULL;
  x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
  x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
  x = (x | (x << 2)) & 0x1249249249249249ULL;
  return x;
}

struct Leaf {
  long off, cnt;
  double c[3], r;
};

// src/numint/spatial_grid_hierarchy.cpp:40-147
std::vector<Leaf> morton_leaves(long n, const double *pts, long target, long min_leaf,
                                long max_leaf, std::vector<long> &perm) {
  std::vector<Leaf> leaves;
  perm.assign(n, 0);
  if (n == 0)
    return leaves;
  double lo[3], hi[3], ext[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = hi[d] = pts[d];
  }
  for (long i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      lo[d] = std::min(lo[d], pts[3 * i + d]);
      hi[d] = std::max(hi[d], pts[3 * i + d]);
    }
  for (int d = 0; d < 3; d++) {
    ext[d] = hi[d] - lo[d];
    if (ext[d] < 1e-10)
      ext[d] = 1.0;
  }
  const uint64_t scale = (1ULL << 21) - 1;
  std::vector<std::pair<uint64_t, long>> codes(n);
  for (long i = 0; i < n; i++) {
    uint64_t q[3];
    for (int d = 0; d < 3; d++) {
      double u = (pts[3 * i + d] - lo[d]) / ext[d];
      u = std::min(std::max(u, 0.0), 1.0);
      q[d] = static_cast<uint64_t>(u * scale);
    }
    codes[i] = {dilate3(q[0]) | (dilate3(q[1]) << 1) | (dilate3(q[2]) << 2), i};
  }
  std::sort(codes.begin(), codes.end());
  for (long i = 0; i < n; i++)
    perm[i] = codes[i].second;
  long off = 0;
  while (off < n) {
    long rem = n - off, cnt;
    if (rem <= max_leaf)
      cnt = rem;
    else if (rem < 2 * min_leaf)
      cnt = rem / 2;
    else
      cnt = std::min(target, rem);
    Leaf lf;
    lf.off = off;
    lf.cnt = cnt;
    double c[3] = {0, 0, 0};
    for (long i = off; i < off + cnt; i++)
      for (int d = 0; d < 3; d++)
        c[d] += pts[3 * perm[i] + d];
    for (int d = 0; d < 3; d++)
      lf.c[d] = c[d] / cnt;
    double r = 0.0;
    for (long i = off; i < off + cnt; i++) {
      double dx = pts[3 * perm[i]] - lf.c[0], dy = pts[3 * perm[i] + 1] - lf.c[1],
             dz = pts[3 * perm[i] + 2] - lf.c[2];
      r = std::max(r, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    lf.r = r;
    leaves.push_back(lf);
    off += cnt;
  }
  return leaves;
}

double g_last_flops = 0.0;  // 4 sum n_b m_b^2 over the leaves the last build processed
double g_total_flops = 0.0; // the same over all leaves of the last build

} // namespace

extern "C" double oracle_last_flops() { return g_last_flops; }
extern "C" double oracle_total_flops() { return g_total_flops; }

extern "C" int oracle_collocation(int l, int pure, int nprim, const double *exps,
                                  const double *coefs, const double *origin, long n,
                                  const double *xyz, int deriv, double *out) {
  collocate(l, pure != 0, nprim, exps, coefs, origin, n, xyz, 3, deriv, out, n);
  return 0;
}

extern "C" void oracle_decay_cutoff(int nsh, const int *sh_l, const int *sh_nprim,
                                    const int *sh_off, const double *exps,
                                    const double *coefs, const double *sh_origin, int pure,
                                    double threshold, double *extents) {
  Basis bs{nsh, sh_l, sh_nprim, sh_off, exps, coefs, sh_origin, pure != 0, {}, 0};
  decay_cutoff(bs, threshold, extents);
}

extern "C" long oracle_morton_leaves(long n, const double *points, long target,
                                     long min_leaf, long max_leaf, long *perm,
                                     long *leaf_off, long *leaf_cnt, double *centres,
                                     double *radii) {
  std::vector<double> xyz(3 * n);
  for (long i = 0; i < n; i++)
    for (int d = 0; d < 3; d++)
      xyz[3 * i + d] = points[3 * i + d];
  std::vector<long> p;
  auto leaves = morton_leaves(n, xyz.data(), target, min_leaf, max_leaf, p);
  if (perm)
    std::memcpy(perm, p.data(), sizeof(long) * n);
  for (size_t i = 0; i < leaves.size(); i++) {
    if (leaf_off)
      leaf_off[i] = leaves[i].off;
    if (leaf_cnt)
      leaf_cnt[i] = leaves[i].cnt;
    if (centres)
      for (int d = 0; d < 3; d++)
        centres[3 * i + d] = leaves[i].c[d];
    if (radii)
      radii[i] = leaves[i].r;
  }
  return static_cast<long>(leaves.size());
}

// include/occ/dft/dft.h:192-388 (screened path), src/dft/dft_kernels.cpp:9-70,
// src/gto/density.cpp:8-43, src/dft/xc_potential_matrix.cpp:9-41.
extern "C" int oracle_xc_build(int nsh, const int *sh_l, const int *sh_nprim,
                               const int *sh_off, const double *exps, const double *coefs,
                               const double *sh_origin, int pure, long npts,
                               const double *points, const double *weights, const double *D,
                               int nfunc, const int *func_ids, const double *func_coefs,
                               double screen_threshold, double density_threshold,
                               long leaf_target, long leaf_min, long leaf_max, int nthreads,
                               long leaf_stride, double *V, double *exc_out,
                               double *nelec_out) {
  Basis bs{nsh, sh_l, sh_nprim, sh_off, exps, coefs, sh_origin, pure != 0, {}, 0};
  bs.first_bf.resize(nsh);
  int nbf = 0;
  for (int s = 0; s < nsh; s++) {
    bs.first_bf[s] = nbf;
    nbf += bs.size(s);
  }
  bs.nbf = nbf;
  int deriv = 0; // OCC's density_derivative(): 0 LDA, 1 GGA, 2 meta-GGA
  for (int f = 0; f < nfunc; f++) {
    if (oracle_functional_is_mgga(func_ids[f]))
      deriv = 2;
    else
      deriv = std::max(deriv, oracle_functional_is_gga(func_ids[f]));
  }
  std::vector<double> ext(nsh);
  decay_cutoff(bs, screen_threshold, ext.data());
  std::vector<long> perm;
  auto leaves = morton_leaves(npts, points, leaf_target, leaf_min, leaf_max, perm);
  long nleaves = static_cast<long>(leaves.size());
  const long stride = leaf_stride > 1 ? leaf_stride : 1;

  // D2 = 2 D (dft.h:205)
  std::vector<double> D2(static_cast<size_t>(nbf) * nbf);
  for (size_t i = 0; i < D2.size(); i++)
    D2[i] = 2.0 * D[i];

#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
  (void)nthreads;
#endif
  std::vector<std::vector<double>> Vloc(nt);
  std::vector<double> eloc(nt, 0.0), nloc(nt, 0.0), floc(nt, 0.0);
  g_total_flops = 0.0;
  for (const Leaf &lf : leaves) {
    double m = 0.0;
    for (int s = 0; s < nsh; s++) {
      const double *A = sh_origin + 3 * s;
      double dx = A[0] - lf.c[0], dy = A[1] - lf.c[1], dz = A[2] - lf.c[2];
      if (std::sqrt(dx * dx + dy * dy + dz * dz) - ext[s] < lf.r)
        m += bs.size(s);
    }
    g_total_flops += 4.0 * lf.cnt * m * m;
  }

#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    std::vector<double> &K = Vloc[tid];
    K.assign(static_cast<size_t>(nbf) * nbf, 0.0);
    std::vector<double> xyz, w, phi, Dloc, Dphi, rho, sigma, exc, vrho, vsig, e1, v1, s1, Y,
        Kb, tau, vtau, t1;
    std::vector<int> sig, loc0;
#pragma omp for schedule(dynamic, 4)
    for (long li = 0; li < nleaves; li++) {
      if (li % stride != 0)
        continue;
      const Leaf &lf = leaves[li];
      const long n = lf.cnt;
      if (n == 0)
        continue;
      sig.clear();
      for (int s = 0; s < nsh; s++) {
        const double *A = sh_origin + 3 * s;
        double dx = A[0] - lf.c[0], dy = A[1] - lf.c[1], dz = A[2] - lf.c[2];
        double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (dist - ext[s] < lf.r)
          sig.push_back(s);
      }
      if (sig.empty())
        continue;
      loc0.assign(sig.size(), 0);
      int m = 0;
      for (size_t k = 0; k < sig.size(); k++) {
        loc0[k] = m;
        m += bs.size(sig[k]);
      }
      floc[tid] += 4.0 * n * static_cast<double>(m) * m;
      xyz.resize(3 * n);
      w.resize(n);
      for (long i = 0; i < n; i++) {
        long o = perm[lf.off + i];
        for (int d = 0; d < 3; d++)
          xyz[3 * i + d] = points[3 * o + d];
        w[i] = weights[o];
      }
      // gather D_local (dft.h:340-348)
      Dloc.assign(static_cast<size_t>(m) * m, 0.0);
      for (size_t a = 0; a < sig.size(); a++)
        for (size_t b = 0; b < sig.size(); b++) {
          int la = bs.size(sig[a]), lb = bs.size(sig[b]);
          for (int j = 0; j < lb; j++)
            for (int i = 0; i < la; i++)
              Dloc[(loc0[b] + j) * static_cast<size_t>(m) + loc0[a] + i] =
                  D2[(bs.first_bf[sig[b]] + j) * static_cast<size_t>(nbf) + bs.first_bf[sig[a]] + i];
        }
      // collocation: phi[comp][m][n]
      const int ncomp = deriv ? 4 : 1;
      phi.assign(static_cast<size_t>(ncomp) * m * n, 0.0);
      {
        std::vector<double> tmp;
        for (size_t k = 0; k < sig.size(); k++) {
          int s = sig[k], nf = bs.size(s);
          tmp.assign(static_cast<size_t>(ncomp) * nf * n, 0.0);
          collocate(sh_l[s], bs.pure, sh_nprim[s], exps + sh_off[s], coefs + sh_off[s],
                    sh_origin + 3 * s, n, xyz.data(), 3, deriv ? 1 : 0, tmp.data(), n);
          for (int q = 0; q < ncomp; q++)
            for (int f = 0; f < nf; f++)
              std::memcpy(&phi[(static_cast<size_t>(q) * m + loc0[k] + f) * n],
                          &tmp[(static_cast<size_t>(q) * nf + f) * n], sizeof(double) * n);
        }
      }
      // density (src/gto/density.cpp:33-43): Dphi = phi * D, rho = rowsum(phi o Dphi)
      Dphi.assign(static_cast<size_t>(m) * n, 0.0);
      oracle_gemm::gemm_nn(n, m, m, phi.data(), n, Dloc.data(), m, Dphi.data(), n);
      rho.assign(4 * n, 0.0);
      for (int j = 0; j < m; j++) {
        const double *dp = &Dphi[static_cast<size_t>(j) * n];
        const double *ph = &phi[static_cast<size_t>(j) * n];
        for (long p = 0; p < n; p++)
          rho[p] += ph[p] * dp[p];
        if (deriv)
          for (int q = 1; q < 4; q++) {
            const double *g = &phi[(static_cast<size_t>(q) * m + j) * n];
            for (long p = 0; p < n; p++)
              rho[q * n + p] += 2.0 * g[p] * dp[p];
          }
      }
      // meta-GGA: tau = 0.5 sum_k (d_k phi) D2 (d_k phi) (src/gto/density.cpp:
      // 73-101); the laplacian is not formed, as no functional here reads it
      if (deriv == 2) {
        tau.assign(n, 0.0);
        for (int q = 1; q < 4; q++) {
          std::fill(Dphi.begin(), Dphi.end(), 0.0);
          oracle_gemm::gemm_nn(n, m, m, &phi[static_cast<size_t>(q) * m * n], n, Dloc.data(), m,
                               Dphi.data(), n);
          for (int j = 0; j < m; j++) {
            const double *dp = &Dphi[static_cast<size_t>(j) * n];
            const double *g = &phi[(static_cast<size_t>(q) * m + j) * n];
            for (long p = 0; p < n; p++)
              tau[p] += g[p] * dp[p];
          }
        }
        for (long p = 0; p < n; p++)
          tau[p] *= 0.5;
      }
      // totals and block skip (src/dft/dft_kernels.cpp:27-40)
      double maxrho = -1e300;
      for (long p = 0; p < n; p++) {
        nloc[tid] += rho[p] * w[p];
        maxrho = std::max(maxrho, rho[p]);
      }
      if (maxrho < density_threshold)
        continue;
      // functional (src/dft/functional.cpp:18-65, summed over components)
      sigma.assign(n, 0.0);
      if (deriv)
        for (long p = 0; p < n; p++)
          sigma[p] = rho[n + p] * rho[n + p] + rho[2 * n + p] * rho[2 * n + p] +
                     rho[3 * n + p] * rho[3 * n + p];
      exc.assign(n, 0.0);
      vrho.assign(n, 0.0);
      vsig.assign(n, 0.0);
      e1.resize(n);
      v1.resize(n);
      s1.resize(n);
      vtau.assign(n, 0.0);
      t1.assign(n, 0.0);
      for (int f = 0; f < nfunc; f++) {
        std::fill(s1.begin(), s1.end(), 0.0);
        std::fill(t1.begin(), t1.end(), 0.0);
        if (oracle_functional_is_mgga(func_ids[f]))
          oracle_functional_mgga(func_ids[f], n, rho.data(), sigma.data(), tau.data(), e1.data(),
                                 v1.data(), s1.data(), t1.data());
        else
          oracle_functional(func_ids[f], n, rho.data(), sigma.data(), e1.data(), v1.data(),
                            s1.data());
        double c = func_coefs ? func_coefs[f] : 1.0;
        for (long p = 0; p < n; p++) {
          exc[p] += c * e1[p];
          vrho[p] += c * v1[p];
          vsig[p] += c * s1[p];
          vtau[p] += c * t1[p];
        }
      }
      // weight_by (include/occ/dft/functional.h:460-470)
      for (long p = 0; p < n; p++) {
        exc[p] *= w[p];
        vrho[p] *= w[p];
        vsig[p] *= w[p];
        vtau[p] *= w[p];
      }
      for (long p = 0; p < n; p++)
        eloc[tid] += rho[p] * exc[p];
      // V block (src/dft/xc_potential_matrix.cpp:9-41)
      Y.assign(static_cast<size_t>(m) * n, 0.0);
      for (int j = 0; j < m; j++) {
        const double *ph = &phi[static_cast<size_t>(j) * n];
        double *y = &Y[static_cast<size_t>(j) * n];
        if (!deriv) {
          for (long p = 0; p < n; p++)
            y[p] = ph[p] * vrho[p];
        } else {
          const double *gx = &phi[(static_cast<size_t>(1) * m + j) * n];
          const double *gy = &phi[(static_cast<size_t>(2) * m + j) * n];
          const double *gz = &phi[(static_cast<size_t>(3) * m + j) * n];
          for (long p = 0; p < n; p++)
            y[p] = 0.5 * ph[p] * vrho[p] + 2.0 * gx[p] * (rho[n + p] * vsig[p]) +
                   2.0 * gy[p] * (rho[2 * n + p] * vsig[p]) +
                   2.0 * gz[p] * (rho[3 * n + p] * vsig[p]);
        }
      }
      Kb.assign(static_cast<size_t>(m) * m, 0.0);
      oracle_gemm::gemm_tn(m, m, n, phi.data(), n, Y.data(), n, Kb.data(), m);
      if (deriv) { // V = K + K^T
        for (int j = 0; j < m; j++)
          for (int i = 0; i < j; i++) {
            double s = Kb[static_cast<size_t>(j) * m + i] + Kb[static_cast<size_t>(i) * m + j];
            Kb[static_cast<size_t>(j) * m + i] = s;
            Kb[static_cast<size_t>(i) * m + j] = s;
          }
        for (int i = 0; i < m; i++)
          Kb[static_cast<size_t>(i) * m + i] *= 2.0;
      }
      if (deriv == 2) // V += sum_k (d_k phi)^T diag(0.5 w vtau) (d_k phi)
        for (int q = 1; q < 4; q++) {
          const double *g = &phi[static_cast<size_t>(q) * m * n];
          for (int j = 0; j < m; j++)
            for (long p = 0; p < n; p++)
              Y[static_cast<size_t>(j) * n + p] = (0.5 * vtau[p]) * g[static_cast<size_t>(j) * n + p];
          oracle_gemm::gemm_tn(m, m, n, g, n, Y.data(), n, Kb.data(), m);
        }
      // scatter (dft.h:361-369)
      for (size_t a = 0; a < sig.size(); a++)
        for (size_t b = 0; b < sig.size(); b++) {
          int la = bs.size(sig[a]), lb = bs.size(sig[b]);
          for (int j = 0; j < lb; j++)
            for (int i = 0; i < la; i++)
              K[(bs.first_bf[sig[b]] + j) * static_cast<size_t>(nbf) + bs.first_bf[sig[a]] + i] +=
                  Kb[(loc0[b] + j) * static_cast<size_t>(m) + loc0[a] + i];
        }
    }
  }
  // reduction (dft.h:374-380)
  std::memset(V, 0, sizeof(double) * nbf * nbf);
  double E = 0.0, Ne = 0.0;
  g_last_flops = 0.0;
  for (int t = 0; t < nt; t++)
    g_last_flops += floc[t];
  for (int t = 0; t < nt; t++) {
    for (size_t i = 0; i < static_cast<size_t>(nbf) * nbf; i++)
      V[i] += Vloc[t][i];
    E += eloc[t];
    Ne += nloc[t];
  }
  *exc_out = E;
  if (nelec_out)
    *nelec_out = Ne;
  return 0;
}

// The restricted XC nuclear gradient, screened path: include/occ/dft/dft.h
// :599-749 (leaf loop, D2 = 2 D gathered per leaf, AO second derivatives for
// a GGA) with src/dft/dft_gradient_kernels.cpp:472-595 per leaf:
//   LDA: Vx = phi_x^T (w vrho phi)
//   GGA: aow = 0.5 w vrho phi + 2 w vsigma grad rho . grad phi,
//        Vx = phi_x^T aow + (phi^T aow_x)^T, aow_x = 0.5 w vrho phi_x
//             + 2 w vsigma grad rho . grad phi_x          (y, z alike)
//   gradient(:, atom(mu)) -= V(mu, nu) * 2 D2(mu, nu), |2 D2| >= 1e-12.
// Grid weights are held fixed (no weight derivatives), as there.
extern "C" int oracle_xc_gradient(int nsh, const int *sh_l, const int *sh_nprim,
                                  const int *sh_off, const double *exps, const double *coefs,
                                  const double *sh_origin, const int *sh_atom, int natoms,
                                  int pure, long npts, const double *points,
                                  const double *weights, const double *D, int nfunc,
                                  const int *func_ids, const double *func_coefs,
                                  double screen_threshold, double density_threshold,
                                  long leaf_target, long leaf_min, long leaf_max, int nthreads,
                                  double *grad) {
  Basis bs{nsh, sh_l, sh_nprim, sh_off, exps, coefs, sh_origin, pure != 0, {}, 0};
  bs.first_bf.resize(nsh);
  int nbf = 0;
  for (int s = 0; s < nsh; s++) {
    bs.first_bf[s] = nbf;
    nbf += bs.size(s);
  }
  int deriv = 0; // 0 LDA, 1 GGA, 2 meta-GGA
  for (int f = 0; f < nfunc; f++) {
    if (oracle_functional_is_mgga(func_ids[f]))
      deriv = 2;
    else
      deriv = std::max(deriv, oracle_functional_is_gga(func_ids[f]));
  }
  const int ncomp = deriv ? 10 : 4;
  std::vector<double> ext(nsh);
  decay_cutoff(bs, screen_threshold, ext.data());
  std::vector<long> perm;
  auto leaves = morton_leaves(npts, points, leaf_target, leaf_min, leaf_max, perm);
  const long nleaves = static_cast<long>(leaves.size());
  std::vector<double> D2(static_cast<size_t>(nbf) * nbf);
  for (size_t i = 0; i < D2.size(); i++)
    D2[i] = 2.0 * D[i];
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
  (void)nthreads;
#endif
  std::vector<std::vector<double>> gloc(nt, std::vector<double>(3 * natoms, 0.0));
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    std::vector<double> &G = gloc[tid];
    std::vector<double> xyz, w, phi, Dloc, Dphi, rho, sigma, e1, v1, s1, vrho, vsig, aow,
        Vx, Vy, Vz, tmp, tau, vtau, t1;
    std::vector<int> sig, loc0, bf_atom;
#pragma omp for schedule(dynamic, 4)
    for (long li = 0; li < nleaves; li++) {
      const Leaf &lf = leaves[li];
      const long n = lf.cnt;
      if (n == 0)
        continue;
      sig.clear();
      for (int s = 0; s < nsh; s++) {
        const double *A = sh_origin + 3 * s;
        double dx = A[0] - lf.c[0], dy = A[1] - lf.c[1], dz = A[2] - lf.c[2];
        if (std::sqrt(dx * dx + dy * dy + dz * dz) - ext[s] < lf.r)
          sig.push_back(s);
      }
      if (sig.empty())
        continue;
      loc0.assign(sig.size(), 0);
      bf_atom.clear();
      int m = 0;
      for (size_t k = 0; k < sig.size(); k++) {
        loc0[k] = m;
        for (int f = 0; f < bs.size(sig[k]); f++)
          bf_atom.push_back(sh_atom[sig[k]]);
        m += bs.size(sig[k]);
      }
      xyz.resize(3 * n);
      w.resize(n);
      for (long i = 0; i < n; i++) {
        long o = perm[lf.off + i];
        for (int d = 0; d < 3; d++)
          xyz[3 * i + d] = points[3 * o + d];
        w[i] = weights[o];
      }
      Dloc.assign(static_cast<size_t>(m) * m, 0.0);
      for (size_t a = 0; a < sig.size(); a++)
        for (size_t b = 0; b < sig.size(); b++) {
          int la = bs.size(sig[a]), lb = bs.size(sig[b]);
          for (int j = 0; j < lb; j++)
            for (int i = 0; i < la; i++)
              Dloc[(loc0[b] + j) * static_cast<size_t>(m) + loc0[a] + i] =
                  D2[(bs.first_bf[sig[b]] + j) * static_cast<size_t>(nbf) + bs.first_bf[sig[a]] + i];
        }
      phi.assign(static_cast<size_t>(ncomp) * m * n, 0.0);
      for (size_t k = 0; k < sig.size(); k++) {
        int s = sig[k], nf = bs.size(s);
        tmp.assign(static_cast<size_t>(ncomp) * nf * n, 0.0);
        collocate(sh_l[s], bs.pure, sh_nprim[s], exps + sh_off[s], coefs + sh_off[s],
                  sh_origin + 3 * s, n, xyz.data(), 3, deriv ? 2 : 1, tmp.data(), n);
        for (int q = 0; q < ncomp; q++)
          for (int f = 0; f < nf; f++)
            std::memcpy(&phi[(static_cast<size_t>(q) * m + loc0[k] + f) * n],
                        &tmp[(static_cast<size_t>(q) * nf + f) * n], sizeof(double) * n);
      }
      auto P = [&](int q, int j) { return &phi[(static_cast<size_t>(q) * m + j) * n]; };
      // density (src/gto/density.cpp:33-43) with D2
      Dphi.assign(static_cast<size_t>(m) * n, 0.0);
      for (int j = 0; j < m; j++)
        for (int k = 0; k < m; k++) {
          double d = Dloc[static_cast<size_t>(j) * m + k];
          if (d == 0.0)
            continue;
          for (long p = 0; p < n; p++)
            Dphi[static_cast<size_t>(j) * n + p] += P(0, k)[p] * d;
        }
      rho.assign(4 * n, 0.0);
      for (int j = 0; j < m; j++)
        for (long p = 0; p < n; p++) {
          const double dp = Dphi[static_cast<size_t>(j) * n + p];
          rho[p] += P(0, j)[p] * dp;
          for (int q = 1; q < 4; q++)
            rho[q * n + p] += 2.0 * P(q, j)[p] * dp;
        }
      if (deriv == 2) { // tau = 0.5 sum_k (d_k phi) D2 (d_k phi)
        tau.assign(n, 0.0);
        for (int q = 1; q < 4; q++) {
          std::fill(Dphi.begin(), Dphi.end(), 0.0);
          for (int j = 0; j < m; j++)
            for (int k = 0; k < m; k++) {
              double d = Dloc[static_cast<size_t>(j) * m + k];
              if (d == 0.0)
                continue;
              for (long p = 0; p < n; p++)
                Dphi[static_cast<size_t>(j) * n + p] += P(q, k)[p] * d;
            }
          for (int j = 0; j < m; j++)
            for (long p = 0; p < n; p++)
              tau[p] += P(q, j)[p] * Dphi[static_cast<size_t>(j) * n + p];
        }
        for (long p = 0; p < n; p++)
          tau[p] *= 0.5;
      }
      double maxrho = -1e300;
      for (long p = 0; p < n; p++)
        maxrho = std::max(maxrho, rho[p]);
      if (maxrho < density_threshold)
        continue;
      sigma.assign(n, 0.0);
      for (long p = 0; p < n; p++)
        sigma[p] = rho[n + p] * rho[n + p] + rho[2 * n + p] * rho[2 * n + p] +
                   rho[3 * n + p] * rho[3 * n + p];
      vrho.assign(n, 0.0);
      vsig.assign(n, 0.0);
      e1.resize(n);
      v1.resize(n);
      s1.resize(n);
      vtau.assign(n, 0.0);
      t1.assign(n, 0.0);
      for (int f = 0; f < nfunc; f++) {
        std::fill(s1.begin(), s1.end(), 0.0);
        std::fill(t1.begin(), t1.end(), 0.0);
        if (oracle_functional_is_mgga(func_ids[f]))
          oracle_functional_mgga(func_ids[f], n, rho.data(), sigma.data(), tau.data(), e1.data(),
                                 v1.data(), s1.data(), t1.data());
        else
          oracle_functional(func_ids[f], n, rho.data(), sigma.data(), e1.data(), v1.data(),
                            s1.data());
        double c = func_coefs ? func_coefs[f] : 1.0;
        for (long p = 0; p < n; p++) {
          vrho[p] += c * v1[p];
          vsig[p] += c * s1[p];
          vtau[p] += c * t1[p];
        }
      }
      for (long p = 0; p < n; p++) {
        vrho[p] *= w[p];
        vsig[p] *= w[p];
        vtau[p] *= w[p];
      }
      Vx.assign(static_cast<size_t>(m) * m, 0.0);
      Vy.assign(static_cast<size_t>(m) * m, 0.0);
      Vz.assign(static_cast<size_t>(m) * m, 0.0);
      double *VV[3] = {Vx.data(), Vy.data(), Vz.data()};
      aow.assign(static_cast<size_t>(m) * n, 0.0);
      if (!deriv) { // accumulate_gradient_contribution_R<0>
        for (int nu = 0; nu < m; nu++)
          for (long p = 0; p < n; p++)
            aow[static_cast<size_t>(nu) * n + p] = P(0, nu)[p] * vrho[p];
        for (int c = 0; c < 3; c++)
          for (int nu = 0; nu < m; nu++)
            for (int mu = 0; mu < m; mu++) {
              double acc = 0.0;
              for (long p = 0; p < n; p++)
                acc += P(1 + c, mu)[p] * aow[static_cast<size_t>(nu) * n + p];
              VV[c][static_cast<size_t>(nu) * m + mu] += acc;
            }
      } else { // accumulate_gradient_contribution_R<1>
        for (int nu = 0; nu < m; nu++)
          for (long p = 0; p < n; p++)
            aow[static_cast<size_t>(nu) * n + p] =
                0.5 * vrho[p] * P(0, nu)[p] +
                2.0 * vsig[p] * (rho[n + p] * P(1, nu)[p] + rho[2 * n + p] * P(2, nu)[p] +
                                 rho[3 * n + p] * P(3, nu)[p]);
        for (int c = 0; c < 3; c++)
          for (int nu = 0; nu < m; nu++)
            for (int mu = 0; mu < m; mu++) {
              double acc = 0.0;
              for (long p = 0; p < n; p++)
                acc += P(1 + c, mu)[p] * aow[static_cast<size_t>(nu) * n + p];
              VV[c][static_cast<size_t>(nu) * m + mu] += acc;
            }
        // second-derivative planes (xx, xy, xz, yy, yz, zz) for d/dc of grad phi
        static const int hq[3][3] = {{4, 5, 6}, {5, 7, 8}, {6, 8, 9}};
        std::vector<double> aowc(static_cast<size_t>(m) * n);
        for (int c = 0; c < 3; c++) {
          for (int mu = 0; mu < m; mu++)
            for (long p = 0; p < n; p++)
              aowc[static_cast<size_t>(mu) * n + p] =
                  0.5 * vrho[p] * P(1 + c, mu)[p] +
                  2.0 * vsig[p] *
                      (rho[n + p] * P(hq[c][0], mu)[p] + rho[2 * n + p] * P(hq[c][1], mu)[p] +
                       rho[3 * n + p] * P(hq[c][2], mu)[p]);
          // V_c += (phi^T aow_c)^T: V_c(mu, nu) += sum_p aow_c(p, mu) phi(p, nu)
          for (int nu = 0; nu < m; nu++)
            for (int mu = 0; mu < m; mu++) {
              double acc = 0.0;
              for (long p = 0; p < n; p++)
                acc += aowc[static_cast<size_t>(mu) * n + p] * P(0, nu)[p];
              VV[c][static_cast<size_t>(nu) * m + mu] += acc;
            }
        }
      }
      // meta-GGA (accumulate_gradient_contribution_R<2>, dft_gradient_kernels.cpp:
      // 151-172): V_c(mu, nu) += sum_k sum_p d_c d_k phi_mu (0.5 w vtau) d_k phi_nu
      if (deriv == 2) {
        static const int hq2[3][3] = {{4, 5, 6}, {5, 7, 8}, {6, 8, 9}};
        for (int c = 0; c < 3; c++)
          for (int nu = 0; nu < m; nu++)
            for (int mu = 0; mu < m; mu++) {
              double acc = 0.0;
              for (int k = 0; k < 3; k++)
                for (long p = 0; p < n; p++)
                  acc += P(hq2[c][k], mu)[p] * (0.5 * vtau[p]) * P(1 + k, nu)[p];
              VV[c][static_cast<size_t>(nu) * m + mu] += acc;
            }
      }
      // distribute to atoms (dft_gradient_kernels.cpp:535-547)
      for (int mu = 0; mu < m; mu++) {
        const int atom = bf_atom[mu];
        for (int nu = 0; nu < m; nu++) {
          const double Dval = 2.0 * Dloc[static_cast<size_t>(nu) * m + mu];
          if (std::abs(Dval) < 1e-12)
            continue;
          for (int c = 0; c < 3; c++)
            G[3 * atom + c] -= VV[c][static_cast<size_t>(nu) * m + mu] * Dval;
        }
      }
    }
  }
  std::memset(grad, 0, sizeof(double) * 3 * natoms);
  for (int t = 0; t < nt; t++)
    for (int i = 0; i < 3 * natoms; i++)
      grad[i] += gloc[t][i];
  return 0;
}

// The unrestricted build, screened path: include/occ/dft/dft.h:192-388 with
// nspin = 2 (D2 = 2 D per spin block, dft.h:205, 336-348), the unrestricted
// density (src/gto/density.cpp:44-70), set_params for two spins
// (include/occ/dft/dft_kernels.h:16-60), the block skip on the largest rho_a
// or rho_b (src/dft/dft_kernels.cpp:18-40) and the per-spin potential
// (src/dft/xc_potential_matrix.cpp:61-105):
//   V_s = phi^T (w vrho_s phi) + k + k^T,  k = phi^T G_s,
//   G_a = (2 w vs_aa grad rho_a + w vs_ab grad rho_b) . grad phi.
extern "C" int oracle_xc_build_unrestricted(
    int nsh, const int *sh_l, const int *sh_nprim, const int *sh_off, const double *exps,
    const double *coefs, const double *sh_origin, int pure, long npts, const double *points,
    const double *weights, const double *D, int nfunc, const int *func_ids,
    const double *func_coefs, double screen_threshold, double density_threshold,
    long leaf_target, long leaf_min, long leaf_max, int nthreads, double *V, double *exc_out,
    double *nelec2) {
  Basis bs{nsh, sh_l, sh_nprim, sh_off, exps, coefs, sh_origin, pure != 0, {}, 0};
  bs.first_bf.resize(nsh);
  int nbf = 0;
  for (int s = 0; s < nsh; s++) {
    bs.first_bf[s] = nbf;
    nbf += bs.size(s);
  }
  bs.nbf = nbf;
  int deriv = 0; // 0 LDA, 1 GGA, 2 meta-GGA
  for (int f = 0; f < nfunc; f++) {
    if (oracle_functional_is_mgga(func_ids[f]))
      deriv = 2;
    else
      deriv = std::max(deriv, oracle_functional_is_gga(func_ids[f]));
  }
  std::vector<double> ext(nsh);
  decay_cutoff(bs, screen_threshold, ext.data());
  std::vector<long> perm;
  auto leaves = morton_leaves(npts, points, leaf_target, leaf_min, leaf_max, perm);
  const long nleaves = static_cast<long>(leaves.size());
  const size_t ld = 2 * static_cast<size_t>(nbf); // rows of OCC's 2 nbf x nbf D and V

#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
  (void)nthreads;
#endif
  std::vector<std::vector<double>> Vloc(nt);
  std::vector<double> eloc(nt, 0.0), naloc(nt, 0.0), nbloc(nt, 0.0);
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    std::vector<double> &K = Vloc[tid];
    K.assign(ld * nbf, 0.0);
    std::vector<double> xyz, w, phi, Dloc, Dphi, rho[2], exc, e1, vr[2], v1[2], vs[3], s1[3],
        G, Kb, kt, tau[2], vt[2], mr, ms, mt;
    std::vector<int> sig, loc0;
#pragma omp for schedule(dynamic, 4)
    for (long li = 0; li < nleaves; li++) {
      const Leaf &lf = leaves[li];
      const long n = lf.cnt;
      if (n == 0)
        continue;
      sig.clear();
      for (int s = 0; s < nsh; s++) {
        const double *A = sh_origin + 3 * s;
        double dx = A[0] - lf.c[0], dy = A[1] - lf.c[1], dz = A[2] - lf.c[2];
        if (std::sqrt(dx * dx + dy * dy + dz * dz) - ext[s] < lf.r)
          sig.push_back(s);
      }
      if (sig.empty())
        continue;
      loc0.assign(sig.size(), 0);
      int m = 0;
      for (size_t k = 0; k < sig.size(); k++) {
        loc0[k] = m;
        m += bs.size(sig[k]);
      }
      xyz.resize(3 * n);
      w.resize(n);
      for (long i = 0; i < n; i++) {
        long o = perm[lf.off + i];
        for (int d = 0; d < 3; d++)
          xyz[3 * i + d] = points[3 * o + d];
        w[i] = weights[o];
      }
      const int ncomp = deriv ? 4 : 1;
      phi.assign(static_cast<size_t>(ncomp) * m * n, 0.0);
      {
        std::vector<double> tmp;
        for (size_t k = 0; k < sig.size(); k++) {
          int s = sig[k], nf = bs.size(s);
          tmp.assign(static_cast<size_t>(ncomp) * nf * n, 0.0);
          collocate(sh_l[s], bs.pure, sh_nprim[s], exps + sh_off[s], coefs + sh_off[s],
                    sh_origin + 3 * s, n, xyz.data(), 3, deriv ? 1 : 0, tmp.data(), n);
          for (int q = 0; q < ncomp; q++)
            for (int f = 0; f < nf; f++)
              std::memcpy(&phi[(static_cast<size_t>(q) * m + loc0[k] + f) * n],
                          &tmp[(static_cast<size_t>(q) * nf + f) * n], sizeof(double) * n);
        }
      }
      // per spin: D2_s local block, Dphi = phi D2_s, rho_s and grad rho_s
      double maxrho = -1e300;
      for (int sp = 0; sp < 2; sp++) {
        Dloc.assign(static_cast<size_t>(m) * m, 0.0);
        for (size_t a = 0; a < sig.size(); a++)
          for (size_t b = 0; b < sig.size(); b++) {
            int la = bs.size(sig[a]), lb = bs.size(sig[b]);
            for (int j = 0; j < lb; j++)
              for (int i = 0; i < la; i++)
                Dloc[(loc0[b] + j) * static_cast<size_t>(m) + loc0[a] + i] =
                    2.0 * D[(bs.first_bf[sig[b]] + j) * ld + sp * static_cast<size_t>(nbf) +
                            bs.first_bf[sig[a]] + i];
          }
        Dphi.assign(static_cast<size_t>(m) * n, 0.0);
        for (int j = 0; j < m; j++)
          for (int k = 0; k < m; k++) {
            double d = Dloc[static_cast<size_t>(j) * m + k];
            if (d == 0.0)
              continue;
            const double *ph = &phi[static_cast<size_t>(k) * n];
            double *out = &Dphi[static_cast<size_t>(j) * n];
            for (long p = 0; p < n; p++)
              out[p] += ph[p] * d;
          }
        rho[sp].assign(4 * n, 0.0);
        for (int j = 0; j < m; j++) {
          const double *dp = &Dphi[static_cast<size_t>(j) * n];
          for (long p = 0; p < n; p++)
            rho[sp][p] += phi[static_cast<size_t>(j) * n + p] * dp[p];
          if (deriv)
            for (int q = 1; q < 4; q++)
              for (long p = 0; p < n; p++)
                rho[sp][q * n + p] += 2.0 * phi[(static_cast<size_t>(q) * m + j) * n + p] * dp[p];
        }
        for (long p = 0; p < n; p++) {
          (sp == 0 ? naloc : nbloc)[tid] += rho[sp][p] * w[p];
          maxrho = std::max(maxrho, rho[sp][p]);
        }
        // meta-GGA: tau_s = 0.5 sum_k (d_k phi) D2_s (d_k phi) (src/gto/density.cpp:
        // 104-166)
        if (deriv == 2) {
          tau[sp].assign(n, 0.0);
          for (int q = 1; q < 4; q++) {
            std::fill(Dphi.begin(), Dphi.end(), 0.0);
            for (int j = 0; j < m; j++)
              for (int k = 0; k < m; k++) {
                double d = Dloc[static_cast<size_t>(j) * m + k];
                if (d == 0.0)
                  continue;
                const double *g = &phi[(static_cast<size_t>(q) * m + k) * n];
                double *out = &Dphi[static_cast<size_t>(j) * n];
                for (long p = 0; p < n; p++)
                  out[p] += g[p] * d;
              }
            for (int j = 0; j < m; j++) {
              const double *g = &phi[(static_cast<size_t>(q) * m + j) * n];
              const double *dp = &Dphi[static_cast<size_t>(j) * n];
              for (long p = 0; p < n; p++)
                tau[sp][p] += g[p] * dp[p];
            }
          }
          for (long p = 0; p < n; p++)
            tau[sp][p] *= 0.5;
        }
      }
      if (maxrho < density_threshold)
        continue;
      // polarised functional, summed over components, weighted
      std::vector<double> saa(n, 0.0), sab(n, 0.0), sbb(n, 0.0);
      if (deriv)
        for (long p = 0; p < n; p++)
          for (int q = 1; q < 4; q++) {
            saa[p] += rho[0][q * n + p] * rho[0][q * n + p];
            sab[p] += rho[0][q * n + p] * rho[1][q * n + p];
            sbb[p] += rho[1][q * n + p] * rho[1][q * n + p];
          }
      exc.assign(n, 0.0);
      e1.resize(n);
      for (int sp = 0; sp < 2; sp++) {
        vr[sp].assign(n, 0.0);
        v1[sp].resize(n);
      }
      for (int k = 0; k < 3; k++) {
        vs[k].assign(n, 0.0);
        s1[k].assign(n, 0.0);
      }
      for (int sp = 0; sp < 2; sp++)
        vt[sp].assign(n, 0.0);
      for (int f = 0; f < nfunc; f++) {
        double c = func_coefs ? func_coefs[f] : 1.0;
        if (oracle_functional_is_mgga(func_ids[f])) {
          mr.resize(2 * n);
          ms.resize(3 * n);
          mt.resize(2 * n);
          oracle_functional_mgga_polarized(func_ids[f], n, rho[0].data(), rho[1].data(),
                                           saa.data(), sab.data(), sbb.data(), tau[0].data(),
                                           tau[1].data(), e1.data(), mr.data(), ms.data(),
                                           mt.data());
          for (long p = 0; p < n; p++) {
            exc[p] += c * e1[p];
            for (int sp = 0; sp < 2; sp++) {
              vr[sp][p] += c * mr[2 * p + sp];
              vt[sp][p] += c * mt[2 * p + sp];
            }
            for (int k = 0; k < 3; k++)
              vs[k][p] += c * ms[3 * p + k];
          }
          continue;
        }
        oracle_functional_polarized(func_ids[f], n, rho[0].data(), rho[1].data(), saa.data(),
                                    sab.data(), sbb.data(), e1.data(), v1[0].data(),
                                    v1[1].data(), s1[0].data(), s1[1].data(), s1[2].data());
        for (long p = 0; p < n; p++) {
          exc[p] += c * e1[p];
          vr[0][p] += c * v1[0][p];
          vr[1][p] += c * v1[1][p];
          for (int k = 0; k < 3; k++)
            vs[k][p] += c * s1[k][p];
        }
      }
      for (long p = 0; p < n; p++) {
        exc[p] *= w[p];
        vr[0][p] *= w[p];
        vr[1][p] *= w[p];
        for (int k = 0; k < 3; k++)
          vs[k][p] *= w[p];
        vt[0][p] *= w[p];
        vt[1][p] *= w[p];
        eloc[tid] += exc[p] * (rho[0][p] + rho[1][p]);
      }
      for (int sp = 0; sp < 2; sp++) {
        const int ot = 1 - sp;
        const std::vector<double> &vss = vs[sp == 0 ? 0 : 2];
        Kb.assign(static_cast<size_t>(m) * m, 0.0);
        for (int j = 0; j < m; j++)
          for (int i = 0; i < m; i++) {
            double acc = 0.0;
            for (long p = 0; p < n; p++)
              acc += phi[static_cast<size_t>(i) * n + p] * phi[static_cast<size_t>(j) * n + p] *
                     vr[sp][p];
            Kb[static_cast<size_t>(j) * m + i] = acc;
          }
        if (deriv) {
          G.assign(static_cast<size_t>(m) * n, 0.0);
          for (int j = 0; j < m; j++)
            for (long p = 0; p < n; p++) {
              double g = 0.0;
              for (int q = 1; q < 4; q++)
                g += phi[(static_cast<size_t>(q) * m + j) * n + p] *
                     (2.0 * vss[p] * rho[sp][q * n + p] + vs[1][p] * rho[ot][q * n + p]);
              G[static_cast<size_t>(j) * n + p] = g;
            }
          kt.assign(static_cast<size_t>(m) * m, 0.0);
          for (int j = 0; j < m; j++)
            for (int i = 0; i < m; i++) {
              double acc = 0.0;
              for (long p = 0; p < n; p++)
                acc += phi[static_cast<size_t>(i) * n + p] * G[static_cast<size_t>(j) * n + p];
              kt[static_cast<size_t>(j) * m + i] = acc;
            }
          for (int j = 0; j < m; j++)
            for (int i = 0; i < m; i++)
              Kb[static_cast<size_t>(j) * m + i] +=
                  kt[static_cast<size_t>(j) * m + i] + kt[static_cast<size_t>(i) * m + j];
        }
        if (deriv == 2) // V_s += sum_k (d_k phi)^T diag(0.5 w vtau_s) (d_k phi)
          for (int q = 1; q < 4; q++)
            for (int j = 0; j < m; j++) {
              const double *b = &phi[(static_cast<size_t>(q) * m + j) * n];
              for (int i = 0; i < m; i++) {
                const double *a = &phi[(static_cast<size_t>(q) * m + i) * n];
                double acc = 0.0;
                for (long p = 0; p < n; p++)
                  acc += a[p] * (0.5 * vt[sp][p]) * b[p];
                Kb[static_cast<size_t>(j) * m + i] += acc;
              }
            }
        for (size_t a = 0; a < sig.size(); a++)
          for (size_t b = 0; b < sig.size(); b++) {
            int la = bs.size(sig[a]), lb = bs.size(sig[b]);
            for (int j = 0; j < lb; j++)
              for (int i = 0; i < la; i++)
                K[(bs.first_bf[sig[b]] + j) * ld + sp * static_cast<size_t>(nbf) +
                  bs.first_bf[sig[a]] + i] += Kb[(loc0[b] + j) * static_cast<size_t>(m) + loc0[a] + i];
          }
      }
    }
  }
  std::memset(V, 0, sizeof(double) * ld * nbf);
  double E = 0.0, Na = 0.0, Nb = 0.0;
  for (int t = 0; t < nt; t++) {
    for (size_t i = 0; i < ld * nbf; i++)
      V[i] += Vloc[t][i];
    E += eloc[t];
    Na += naloc[t];
    Nb += nbloc[t];
  }
  *exc_out = E;
  if (nelec2) {
    nelec2[0] = Na;
    nelec2[1] = Nb;
  }
  return 0;
}

// VV10 non-local correlation, restated from src/dft/nonlocal_correlation.cpp:
// vv10_kernel (:37-110) over the points in the given (grid) order -- as the
// reference writes it, each point i sums its partners j < i only, with half
// of its own r = 0 term -- and vv10 (:331-388): the density with the whole
// basis (no screening) on the NLC grid, E = sum exc rho, V = k + k^T with
// k = phi^T (0.5 vrho phi + 2 vsigma grad rho . grad phi).
extern "C" void oracle_vv10_kernel(long n, const double *points, const double *weights,
                                   const double *rho, const double *sigma, double b, double C,
                                   int nthreads, double *exc, double *vrho, double *vsigma) {
  const double pi = 3.14159265358979323846, pi4_3 = 4.0 * pi / 3.0;
  const double kappa_factor = b * 1.5 * pi * std::pow(9.0 * pi, -1.0 / 6.0);
  const double beta = std::pow(3.0 / (b * b), 0.75) / 32.0;
  std::vector<double> rw(n), tmp(n), om(n), dom_r(n), dom_g(n), kap(n), dkap(n), F(n, 0.0),
      U(n, 0.0), W(n, 0.0);
  for (long i = 0; i < n; i++) {
    rw[i] = rho[i] * weights[i];
    double t = sigma[i] / (rho[i] * rho[i]);
    t = C * t * t;
    tmp[i] = t;
    om[i] = std::sqrt(t + pi4_3 * rho[i]);
    dom_r[i] = (0.5 * pi4_3 * rho[i] - 2.0 * t) / om[i];
    dom_g[i] = t * rho[i] / (sigma[i] * om[i]);
    kap[i] = kappa_factor * std::pow(rho[i], 1.0 / 6.0);
    dkap[i] = kap[i] / 6.0;
  }
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
  (void)nthreads;
#endif
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
  for (long i = 0; i < n; i++) {
    if (rho[i] < 1e-8)
      continue;
    const double k = kap[i];
    double f = rw[i] / (2 * k * k * k);
    double u = f * (1.0 / k + 1.0 / (2 * k));
    double w = 0.0;
    for (long j = 0; j < i; j++) {
      if (rho[j] < 1e-8)
        continue;
      const double dx = points[3 * i] - points[3 * j], dy = points[3 * i + 1] - points[3 * j + 1],
                   dz = points[3 * i + 2] - points[3 * j + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      const double gi = r2 * om[i] + kap[i];
      const double gj = r2 * om[j] + kap[j];
      double t = 2 * rw[j] / (gi * gj * (gi + gj));
      f += t;
      t *= 1.0 / gi + 1.0 / (gi + gj);
      u += t;
      w += t * r2;
    }
    F[i] = f * -1.5;
    U[i] = u;
    W[i] = w;
  }
  for (long i = 0; i < n; i++) {
    exc[i] = (beta + 0.5 * F[i]) * weights[i];
    vrho[i] = (beta + F[i] + 1.5 * (U[i] * dkap[i] + W[i] * dom_r[i])) * weights[i];
    vsigma[i] = (1.5 * W[i] * dom_g[i]) * weights[i];
  }
}

extern "C" int oracle_nlc_vv10(int nsh, const int *sh_l, const int *sh_nprim, const int *sh_off,
                               const double *exps, const double *coefs, const double *sh_origin,
                               int pure, long npts, const double *points, const double *weights,
                               const double *D, double b, double C, int nthreads, double *V,
                               double *energy) {
  Basis bs{nsh, sh_l, sh_nprim, sh_off, exps, coefs, sh_origin, pure != 0, {}, 0};
  bs.first_bf.resize(nsh);
  int nbf = 0;
  for (int s = 0; s < nsh; s++) {
    bs.first_bf[s] = nbf;
    nbf += bs.size(s);
  }
  bs.nbf = nbf;
  const long n = npts;
  // phi, grad phi of every AO at every point: [comp][nbf][n]
  std::vector<double> phi(static_cast<size_t>(4) * nbf * n, 0.0);
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
#endif
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
  for (int s = 0; s < nsh; s++) {
    int nf = bs.size(s);
    std::vector<double> tmp(static_cast<size_t>(4) * nf * n);
    collocate(sh_l[s], bs.pure, sh_nprim[s], exps + sh_off[s], coefs + sh_off[s],
              sh_origin + 3 * s, n, points, 3, 1, tmp.data(), n);
    for (int q = 0; q < 4; q++)
      for (int f = 0; f < nf; f++)
        std::memcpy(&phi[(static_cast<size_t>(q) * nbf + bs.first_bf[s] + f) * n],
                    &tmp[(static_cast<size_t>(q) * nf + f) * n], sizeof(double) * n);
  }
  // density with D2 = 2 D (src/gto/density.cpp:33-43)
  std::vector<double> rho(4 * n, 0.0);
#pragma omp parallel for num_threads(nt) schedule(static)
  for (long p = 0; p < n; p++) {
    for (int j = 0; j < nbf; j++) {
      double x = 0.0;
      for (int k = 0; k < nbf; k++)
        x += phi[static_cast<size_t>(k) * n + p] * 2.0 * D[static_cast<size_t>(j) * nbf + k];
      rho[p] += phi[static_cast<size_t>(j) * n + p] * x;
      for (int q = 1; q < 4; q++)
        rho[q * n + p] += 2.0 * phi[(static_cast<size_t>(q) * nbf + j) * n + p] * x;
    }
  }
  std::vector<double> sigma(n), exc(n), vr(n), vs(n);
  for (long p = 0; p < n; p++)
    sigma[p] = rho[n + p] * rho[n + p] + rho[2 * n + p] * rho[2 * n + p] +
               rho[3 * n + p] * rho[3 * n + p];
  oracle_vv10_kernel(n, points, weights, rho.data(), sigma.data(), b, C, nthreads, exc.data(),
                     vr.data(), vs.data());
  double e = 0.0;
  for (long p = 0; p < n; p++)
    e += exc[p] * rho[p];
  *energy = e;
  if (V) {
    // Y = 0.5 vrho phi + 2 vsigma grad rho . grad phi; k = phi^T Y; V = k + k^T
    std::vector<double> Y(static_cast<size_t>(nbf) * n), K(static_cast<size_t>(nbf) * nbf);
    for (int j = 0; j < nbf; j++)
      for (long p = 0; p < n; p++) {
        double y = 0.5 * vr[p] * phi[static_cast<size_t>(j) * n + p];
        for (int q = 1; q < 4; q++)
          y += 2.0 * vs[p] * rho[q * n + p] * phi[(static_cast<size_t>(q) * nbf + j) * n + p];
        Y[static_cast<size_t>(j) * n + p] = y;
      }
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int j = 0; j < nbf; j++)
      for (int i = 0; i < nbf; i++) {
        double acc = 0.0;
        for (long p = 0; p < n; p++)
          acc += phi[static_cast<size_t>(i) * n + p] * Y[static_cast<size_t>(j) * n + p];
        K[static_cast<size_t>(j) * nbf + i] = acc;
      }
    for (int j = 0; j < nbf; j++)
      for (int i = 0; i < nbf; i++)
        V[static_cast<size_t>(j) * nbf + i] =
            K[static_cast<size_t>(j) * nbf + i] + K[static_cast<size_t>(i) * nbf + j];
  }
  return 0;
}

// The unrestricted XC nuclear gradient (include/occ/dft/dft.h:599-749 with
// accumulate_gradient_contribution_U<0,1,2>, src/dft/dft_gradient_kernels.cpp:
// 175-470, and the distribution of :549-575), screened path, grid fixed.
// D is OCC's unrestricted mo.D (2 nbf x nbf, alpha block above beta); with
// D2 = 2 mo.D and Da, Db its blocks, per spin s
//   V_c,s(mu, nu) = sum_p d_c phi_mu Y_s,nu + Z_c,s,mu phi_nu
//                   [+ sum_k d_c d_k phi_mu (0.5 w vtau_s) d_k phi_nu]
//   Y_s = 0.5 w vrho_s phi + w (2 vsigma_ss grad rho_s + vsigma_ab grad rho_s') . grad phi
//   Z_c,s = 0.5 w vrho_s d_c phi + w (2 vsigma_ss grad rho_s + vsigma_ab grad rho_s')
//           . grad d_c phi
// (for an LDA, Y_s = w vrho_s phi and Z = 0: the same sum), and
//   g_A,c -= sum_{mu on A, nu} 2 (V_c,a Da + V_c,b Db)(mu, nu),
// skipping |Da + Db| < 1e-12.
extern "C" int oracle_xc_gradient_unrestricted(
    int nsh, const int *sh_l, const int *sh_nprim, const int *sh_off, const double *exps,
    const double *coefs, const double *sh_origin, const int *sh_atom, int natoms, int pure,
    long npts, const double *points, const double *weights, const double *D, int nfunc,
    const int *func_ids, const double *func_coefs, double screen_threshold,
    double density_threshold, long leaf_target, long leaf_min, long leaf_max, int nthreads,
    double *grad) {
  Basis bs{nsh, sh_l, sh_nprim, sh_off, exps, coefs, sh_origin, pure != 0, {}, 0};
  bs.first_bf.resize(nsh);
  int nbf = 0;
  for (int s = 0; s < nsh; s++) {
    bs.first_bf[s] = nbf;
    nbf += bs.size(s);
  }
  bs.nbf = nbf;
  int deriv = 0;
  for (int f = 0; f < nfunc; f++) {
    if (oracle_functional_is_mgga(func_ids[f]))
      deriv = 2;
    else
      deriv = std::max(deriv, oracle_functional_is_gga(func_ids[f]));
  }
  const int ncomp = deriv ? 10 : 4;
  std::vector<double> ext(nsh);
  decay_cutoff(bs, screen_threshold, ext.data());
  std::vector<long> perm;
  auto leaves = morton_leaves(npts, points, leaf_target, leaf_min, leaf_max, perm);
  const long nleaves = static_cast<long>(leaves.size());
  const size_t ld = 2 * static_cast<size_t>(nbf);
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
  (void)nthreads;
#endif
  std::vector<std::vector<double>> gloc(nt, std::vector<double>(3 * natoms, 0.0));
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    std::vector<double> &G = gloc[tid];
    std::vector<double> xyz, w, phi, Dloc[2], Dphi, rho[2], tau[2], tmp, e1, mr, ms, mt;
    std::vector<double> vr[2], vs[3], vt[2], v1[2], s1[3], aow, V[2][3];
    std::vector<int> sig, loc0, bf_atom;
#pragma omp for schedule(dynamic, 4)
    for (long li = 0; li < nleaves; li++) {
      const Leaf &lf = leaves[li];
      const long n = lf.cnt;
      if (n == 0)
        continue;
      sig.clear();
      for (int s = 0; s < nsh; s++) {
        const double *A = sh_origin + 3 * s;
        double dx = A[0] - lf.c[0], dy = A[1] - lf.c[1], dz = A[2] - lf.c[2];
        if (std::sqrt(dx * dx + dy * dy + dz * dz) - ext[s] < lf.r)
          sig.push_back(s);
      }
      if (sig.empty())
        continue;
      loc0.assign(sig.size(), 0);
      bf_atom.clear();
      int m = 0;
      for (size_t k = 0; k < sig.size(); k++) {
        loc0[k] = m;
        for (int f = 0; f < bs.size(sig[k]); f++)
          bf_atom.push_back(sh_atom[sig[k]]);
        m += bs.size(sig[k]);
      }
      xyz.resize(3 * n);
      w.resize(n);
      for (long i = 0; i < n; i++) {
        long o = perm[lf.off + i];
        for (int d = 0; d < 3; d++)
          xyz[3 * i + d] = points[3 * o + d];
        w[i] = weights[o];
      }
      phi.assign(static_cast<size_t>(ncomp) * m * n, 0.0);
      for (size_t k = 0; k < sig.size(); k++) {
        int s = sig[k], nf = bs.size(s);
        tmp.assign(static_cast<size_t>(ncomp) * nf * n, 0.0);
        collocate(sh_l[s], bs.pure, sh_nprim[s], exps + sh_off[s], coefs + sh_off[s],
                  sh_origin + 3 * s, n, xyz.data(), 3, deriv ? 2 : 1, tmp.data(), n);
        for (int q = 0; q < ncomp; q++)
          for (int f = 0; f < nf; f++)
            std::memcpy(&phi[(static_cast<size_t>(q) * m + loc0[k] + f) * n],
                        &tmp[(static_cast<size_t>(q) * nf + f) * n], sizeof(double) * n);
      }
      auto P = [&](int q, int j) { return &phi[(static_cast<size_t>(q) * m + j) * n]; };
      // per spin: D2_s local block, rho_s, grad rho_s, tau_s
      double maxrho = -1e300;
      for (int sp = 0; sp < 2; sp++) {
        Dloc[sp].assign(static_cast<size_t>(m) * m, 0.0);
        for (size_t a = 0; a < sig.size(); a++)
          for (size_t b = 0; b < sig.size(); b++) {
            int la = bs.size(sig[a]), lb = bs.size(sig[b]);
            for (int j = 0; j < lb; j++)
              for (int i = 0; i < la; i++)
                Dloc[sp][(loc0[b] + j) * static_cast<size_t>(m) + loc0[a] + i] =
                    2.0 * D[(bs.first_bf[sig[b]] + j) * ld + sp * static_cast<size_t>(nbf) +
                            bs.first_bf[sig[a]] + i];
          }
        rho[sp].assign(4 * n, 0.0);
        for (int q = 0; q < (deriv == 2 ? 4 : 1); q++) {
          Dphi.assign(static_cast<size_t>(m) * n, 0.0);
          for (int j = 0; j < m; j++)
            for (int k = 0; k < m; k++) {
              double d = Dloc[sp][static_cast<size_t>(j) * m + k];
              if (d == 0.0)
                continue;
              for (long p = 0; p < n; p++)
                Dphi[static_cast<size_t>(j) * n + p] += P(q, k)[p] * d;
            }
          if (q == 0) {
            for (int j = 0; j < m; j++)
              for (long p = 0; p < n; p++) {
                const double dp = Dphi[static_cast<size_t>(j) * n + p];
                rho[sp][p] += P(0, j)[p] * dp;
                for (int c = 1; c < 4; c++)
                  rho[sp][c * n + p] += 2.0 * P(c, j)[p] * dp;
              }
            if (deriv == 2)
              tau[sp].assign(n, 0.0);
          } else {
            for (int j = 0; j < m; j++)
              for (long p = 0; p < n; p++)
                tau[sp][p] += 0.5 * P(q, j)[p] * Dphi[static_cast<size_t>(j) * n + p];
          }
        }
        for (long p = 0; p < n; p++)
          maxrho = std::max(maxrho, rho[sp][p]);
      }
      if (maxrho < density_threshold)
        continue;
      std::vector<double> saa(n, 0.0), sab(n, 0.0), sbb(n, 0.0);
      for (long p = 0; p < n; p++)
        for (int c = 1; c < 4; c++) {
          saa[p] += rho[0][c * n + p] * rho[0][c * n + p];
          sab[p] += rho[0][c * n + p] * rho[1][c * n + p];
          sbb[p] += rho[1][c * n + p] * rho[1][c * n + p];
        }
      e1.resize(n);
      for (int sp = 0; sp < 2; sp++) {
        vr[sp].assign(n, 0.0);
        vt[sp].assign(n, 0.0);
        v1[sp].resize(n);
      }
      for (int k = 0; k < 3; k++) {
        vs[k].assign(n, 0.0);
        s1[k].assign(n, 0.0);
      }
      for (int f = 0; f < nfunc; f++) {
        const double c = func_coefs ? func_coefs[f] : 1.0;
        if (oracle_functional_is_mgga(func_ids[f])) {
          mr.resize(2 * n);
          ms.resize(3 * n);
          mt.resize(2 * n);
          oracle_functional_mgga_polarized(func_ids[f], n, rho[0].data(), rho[1].data(),
                                           saa.data(), sab.data(), sbb.data(), tau[0].data(),
                                           tau[1].data(), e1.data(), mr.data(), ms.data(),
                                           mt.data());
          for (long p = 0; p < n; p++) {
            for (int sp = 0; sp < 2; sp++) {
              vr[sp][p] += c * mr[2 * p + sp];
              vt[sp][p] += c * mt[2 * p + sp];
            }
            for (int k = 0; k < 3; k++)
              vs[k][p] += c * ms[3 * p + k];
          }
          continue;
        }
        oracle_functional_polarized(func_ids[f], n, rho[0].data(), rho[1].data(), saa.data(),
                                    sab.data(), sbb.data(), e1.data(), v1[0].data(),
                                    v1[1].data(), s1[0].data(), s1[1].data(), s1[2].data());
        for (long p = 0; p < n; p++) {
          vr[0][p] += c * v1[0][p];
          vr[1][p] += c * v1[1][p];
          for (int k = 0; k < 3; k++)
            vs[k][p] += c * s1[k][p];
        }
      }
      for (long p = 0; p < n; p++) {
        for (int sp = 0; sp < 2; sp++) {
          vr[sp][p] *= w[p];
          vt[sp][p] *= w[p];
        }
        for (int k = 0; k < 3; k++)
          vs[k][p] *= w[p];
      }
      static const int hq[3][3] = {{4, 5, 6}, {5, 7, 8}, {6, 8, 9}};
      for (int sp = 0; sp < 2; sp++) {
        const int ot = 1 - sp;
        const std::vector<double> &vss = vs[sp == 0 ? 0 : 2];
        for (int c = 0; c < 3; c++)
          V[sp][c].assign(static_cast<size_t>(m) * m, 0.0);
        aow.assign(static_cast<size_t>(m) * n, 0.0);
        // grad-rho coefficient of this spin: 2 vsigma_ss grad rho_s + vsigma_ab grad rho_s'
        auto gc = [&](int c, long p) {
          return 2.0 * vss[p] * rho[sp][(1 + c) * n + p] + vs[1][p] * rho[ot][(1 + c) * n + p];
        };
        if (!deriv) { // accumulate_gradient_contribution_U<0>
          for (int nu = 0; nu < m; nu++)
            for (long p = 0; p < n; p++)
              aow[static_cast<size_t>(nu) * n + p] = P(0, nu)[p] * vr[sp][p];
          for (int c = 0; c < 3; c++)
            for (int nu = 0; nu < m; nu++)
              for (int mu = 0; mu < m; mu++) {
                double acc = 0.0;
                for (long p = 0; p < n; p++)
                  acc += P(1 + c, mu)[p] * aow[static_cast<size_t>(nu) * n + p];
                V[sp][c][static_cast<size_t>(nu) * m + mu] += acc;
              }
        } else { // U<1>, and the GGA part of U<2>
          for (int nu = 0; nu < m; nu++)
            for (long p = 0; p < n; p++)
              aow[static_cast<size_t>(nu) * n + p] =
                  0.5 * vr[sp][p] * P(0, nu)[p] + gc(0, p) * P(1, nu)[p] +
                  gc(1, p) * P(2, nu)[p] + gc(2, p) * P(3, nu)[p];
          for (int c = 0; c < 3; c++)
            for (int nu = 0; nu < m; nu++)
              for (int mu = 0; mu < m; mu++) {
                double acc = 0.0;
                for (long p = 0; p < n; p++)
                  acc += P(1 + c, mu)[p] * aow[static_cast<size_t>(nu) * n + p];
                V[sp][c][static_cast<size_t>(nu) * m + mu] += acc;
              }
          for (int c = 0; c < 3; c++)
            for (int nu = 0; nu < m; nu++)
              for (int mu = 0; mu < m; mu++) {
                double acc = 0.0;
                for (long p = 0; p < n; p++) {
                  const double z = 0.5 * vr[sp][p] * P(1 + c, mu)[p] +
                                   gc(0, p) * P(hq[c][0], mu)[p] +
                                   gc(1, p) * P(hq[c][1], mu)[p] + gc(2, p) * P(hq[c][2], mu)[p];
                  acc += z * P(0, nu)[p];
                }
                V[sp][c][static_cast<size_t>(nu) * m + mu] += acc;
              }
          if (deriv == 2) // the tau terms of U<2>
            for (int c = 0; c < 3; c++)
              for (int nu = 0; nu < m; nu++)
                for (int mu = 0; mu < m; mu++) {
                  double acc = 0.0;
                  for (int k = 0; k < 3; k++)
                    for (long p = 0; p < n; p++)
                      acc += P(hq[c][k], mu)[p] * (0.5 * vt[sp][p]) * P(1 + k, nu)[p];
                  V[sp][c][static_cast<size_t>(nu) * m + mu] += acc;
                }
        }
      }
      // distribution (dft_gradient_kernels.cpp:549-575)
      for (int mu = 0; mu < m; mu++) {
        const int atom = bf_atom[mu];
        for (int nu = 0; nu < m; nu++) {
          const size_t e = static_cast<size_t>(nu) * m + mu;
          const double da = Dloc[0][e], db = Dloc[1][e];
          if (std::abs(da + db) < 1e-12)
            continue;
          for (int c = 0; c < 3; c++)
            G[3 * atom + c] -= 2.0 * (V[0][c][e] * da + V[1][c][e] * db);
        }
      }
    }
  }
  std::memset(grad, 0, sizeof(double) * 3 * natoms);
  for (int t = 0; t < nt; t++)
    for (int i = 0; i < 3 * natoms; i++)
      grad[i] += gloc[t][i];
  return 0;
}
