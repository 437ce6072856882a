// Molecular integration grid (set-up, once per molecule): LMG radial grids,
// NWChem angular pruning, Lebedev angular rules and Becke partitioning with
// the Treutler-Ahlrichs radius adjustment.  Restates
// src/numint/grid_utils.cpp and src/numint/molecular_grid.cpp.
#include "lebedev_table.h"
#include "xc_host.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <set>
#include <stdexcept>
#include <tuple>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace occx {

namespace {
const double kPi = 3.14159265358979323846;
const double kAngstromToBohr = 1.0 / 0.52917721067; // include/occ/core/units.h:7-8

// src/numint/grid_utils.cpp:16-19
const int kLevels[] = {1,    6,    14,   26,   38,   50,   74,   86,   110,  146,  170,
                       194,  230,  266,  302,  350,  434,  590,  770,  974,  1202, 1454,
                       1730, 2030, 2354, 2702, 3074, 3470, 3890, 4334, 4802, 5294, 5810};
const int kNumLevels = sizeof(kLevels) / sizeof(kLevels[0]);

// Bragg radii in Angstrom, H..Ar (src/numint/grid_utils.cpp:23-41); the
// elements beyond Ar are outside what this build's workloads use.
const double kBragg[] = {0.35, 1.40, 1.45, 1.05, 0.85, 0.70, 0.65, 0.60, 0.50,
                         1.50, 1.80, 1.50, 1.25, 1.10, 1.00, 1.00, 1.00, 1.80};

int level_at_or_above(int n) {
  for (int i = 0; i < kNumLevels; i++)
    if (kLevels[i] >= n)
      return kLevels[i];
  throw std::runtime_error("Requested number of angular points exceeds 5810");
}
int level_below(int n) {
  if (n <= kLevels[0])
    return kLevels[0];
  for (int i = kNumLevels - 1; i >= 0; i--)
    if (kLevels[i] < n)
      return kLevels[i];
  return kLevels[0];
}

double bragg_radius(int Z) {
  if (Z < 1 || Z > static_cast<int>(sizeof(kBragg) / sizeof(kBragg[0])))
    throw std::runtime_error("element outside the supported range (H..Ar)");
  return kBragg[Z - 1] * kAngstromToBohr;
}

// --- LMG radial grid: Lindh, Malmqvist, Gagliardi, TCA 106, 178 (2001) ---
// src/numint/grid_utils.cpp:411-514.  The searches are the reference's
// step-halving walks, reproduced operation for operation (including their
// behaviour for angular momenta that an atom's basis lacks, whose minimum
// exponent is DBL_MAX).
double lmg_inner(double max_error, double alpha_inner) {
  int m = 0;
  double d = 1.9;
  double r = d - std::log(1.0 / max_error);
  r = r * 2.0 / (m + 3.0);
  r = std::exp(r) / alpha_inner;
  return std::sqrt(r);
}

double lmg_outer(double max_error, double alpha_outer, int l, double guess) {
  int m = 2 * l;
  double r = guess, r_old = 1.0e50, step = 0.5, sign, sign_old, f = 1.0e50;
  sign = (f > max_error) ? 1.0 : -1.0;
  while (std::fabs(r_old - r) > 1e-14) {
    double c = std::tgamma((m + 3.0) / 2.0);
    double a = std::pow(alpha_outer * r * r, (m + 1.0) / 2.0);
    double e = std::exp(-alpha_outer * r * r);
    f = c * a * e;
    sign_old = sign;
    sign = (f > max_error) ? 1.0 : -1.0;
    if (r < 0.0)
      sign = 1.0;
    if (sign != sign_old)
      step *= 0.1;
    r_old = r;
    r += sign * step;
  }
  return r;
}

double lmg_h(double max_error, int l, double guess) {
  int m = 2 * l;
  double h = guess, h_old = 1.0e50, step = 0.1 * guess, sign, sign_old, f = 1.0e50;
  sign = (f > max_error) ? -1.0 : 1.0;
  while (std::fabs(h_old - h) > 1e-14) {
    double c0 = 4.0 * std::sqrt(2.0) * kPi;
    double cm = std::tgamma(3.0 / 2.0) / std::tgamma((m + 3.0) / 2.0);
    double p0 = 1.0 / h;
    double e0 = std::exp(-kPi * kPi / (2.0 * h));
    double pm = std::pow(kPi / h, m / 2.0);
    double rd0 = c0 * p0 * e0;
    f = cm * pm * rd0;
    sign_old = sign;
    sign = (f > max_error) ? -1.0 : 1.0;
    if (h < 0.0)
      sign = 1.0;
    if (sign != sign_old)
      step *= 0.1;
    h_old = h;
    h += sign * step;
  }
  return h;
}

void lmg_radial(int Z, double precision, double alpha_max, int l_max,
                const std::vector<double> &alpha_min, std::vector<double> &r,
                std::vector<double> &w) {
  double r_inner = lmg_inner(precision, 2.0 * alpha_max);
  double h = std::numeric_limits<float>::max();
  double r_outer = 0.0;
  double br = bragg_radius(Z);
  for (int i = 0; i <= l_max; i++) {
    if (alpha_min[i] > 0.0) {
      r_outer = std::max(r_outer, lmg_outer(precision, alpha_min[i], i, 4.0 * br));
      h = std::min(h, lmg_h(precision, i, 0.1 * (r_outer - r_inner)));
    }
  }
  double c = r_inner / (std::exp(h) - 1.0);
  int n = static_cast<int>(std::log(1.0 + (r_outer / c)) / h);
  r.resize(n);
  w.resize(n);
  for (int i = 0; i < n; i++) {
    r[i] = c * (std::exp((i + 1) * h) - 1.0);
    w[i] = (r[i] + c) * h * r[i] * r[i];
  }
}

// src/numint/grid_utils.cpp:234-274
std::vector<int> prune_nwchem(int Z, int max_angular, const std::vector<double> &radii) {
  std::vector<int> out(radii.size());
  int lev[5];
  if (max_angular < 50) {
    std::fill(out.begin(), out.end(), max_angular);
    return out;
  } else if (max_angular == 50) {
    int l50[5] = {5, 6, 6, 6, 5};
    std::copy(l50, l50 + 5, lev);
  } else {
    int i;
    for (i = 6; i < kNumLevels; i++)
      if (kLevels[i] == max_angular)
        break;
    lev[0] = 5;
    lev[1] = 6;
    lev[2] = i - 1;
    lev[3] = i;
    lev[4] = i - 1;
  }
  double alphas[4] = {0.1, 0.4, 0.8, 2.5};
  if (Z <= 2) {
    double a[4] = {0.25, 0.5, 1.0, 4.5};
    std::copy(a, a + 4, alphas);
  } else if (Z <= 10) {
    double a[4] = {0.16666667, 0.5, 0.9, 3.5};
    std::copy(a, a + 4, alphas);
  }
  double radius = bragg_radius(Z);
  for (size_t i = 0; i < radii.size(); i++) {
    double scale = radii[i] / radius;
    int place = 0;
    while (place < 4 && !(alphas[place] > scale))
      place++;
    out[i] = kLevels[lev[place]];
  }
  return out;
}

struct AtomGrid {
  std::vector<double> xyz, w;
};

// src/numint/grid_utils.cpp:576-758 (LMG + NWChem path)
AtomGrid atom_grid(int Z, const GridSettings &gs, double alpha_max, int l_max,
                   const std::vector<double> &alpha_min) {
  std::vector<double> r, wr;
  if (alpha_max <= 0.0 || l_max <= 0 || alpha_min.empty()) {
    std::vector<double> def(4, 0.1);
    lmg_radial(Z, gs.radial_precision, 20.0, 3, def, r, wr);
  } else {
    lmg_radial(Z, gs.radial_precision, alpha_max, l_max, alpha_min, r, wr);
  }
  for (auto &x : wr)
    x *= 4.0 * kPi;
  int max_angular = gs.max_angular_points;
  if (gs.reduced_first_row_element_grid && Z < 3)
    max_angular = level_below(max_angular);
  std::vector<int> nang;
  if (gs.pruning_scheme == 1)
    nang = prune_nwchem(Z, max_angular, r);
  else
    nang.assign(r.size(), max_angular);
  AtomGrid g;
  std::vector<double> leb;
  for (size_t i = 0; i < r.size(); i++) {
    int n = level_at_or_above(nang[i]);
    if (lebedev_rule(n, leb) != n)
      throw std::runtime_error("Lebedev rule not available: " + std::to_string(n));
    for (int k = 0; k < n; k++) {
      g.xyz.push_back(leb[4 * k] * r[i]);
      g.xyz.push_back(leb[4 * k + 1] * r[i]);
      g.xyz.push_back(leb[4 * k + 2] * r[i]);
      g.w.push_back(leb[4 * k + 3] * wr[i]);
    }
  }
  return g;
}

} // namespace

int lebedev_rule(int npoints, std::vector<double> &out) {
  using namespace lebedev_table;
  const Rule *rule = nullptr;
  for (int i = 0; i < kNumRules; i++)
    if (kRules[i].npoints == npoints)
      rule = &kRules[i];
  if (!rule)
    return 0;
  out.clear();
  for (int o = 0; o < rule->norbits; o++) {
    const Orbit &ob = rule->orbits[o];
    double g[3];
    switch (ob.kind) {
    case 0: g[0] = 1.0; g[1] = 0.0; g[2] = 0.0; break;
    case 1: g[0] = 0.0; g[1] = g[2] = std::sqrt(0.5); break;
    case 2: g[0] = g[1] = g[2] = std::sqrt(1.0 / 3.0); break;
    case 3: g[0] = g[1] = ob.p0; g[2] = std::sqrt(1.0 - 2.0 * ob.p0 * ob.p0); break;
    case 4: g[0] = ob.p0; g[1] = std::sqrt(1.0 - ob.p0 * ob.p0); g[2] = 0.0; break;
    default: g[0] = ob.p0; g[1] = ob.p1; g[2] = std::sqrt(1.0 - ob.p0 * ob.p0 - ob.p1 * ob.p1); break;
    }
    // all distinct images under coordinate permutations and sign changes
    std::set<std::tuple<double, double, double>> seen;
    const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    for (const auto &p : perms)
      for (int s = 0; s < 8; s++) {
        double v[3];
        for (int d = 0; d < 3; d++) {
          v[d] = g[p[d]];
          if ((s >> d) & 1)
            v[d] = -v[d];
          v[d] += 0.0; // fold -0 into +0
        }
        auto key = std::make_tuple(v[0], v[1], v[2]);
        if (seen.insert(key).second) {
          out.push_back(v[0]);
          out.push_back(v[1]);
          out.push_back(v[2]);
          out.push_back(ob.w);
        }
      }
  }
  return static_cast<int>(out.size() / 4);
}

MolecularGrid build_molecular_grid(const std::vector<int> &Z, const std::vector<double> &xyz,
                                   const Basis &basis, const GridSettings &gs_in, int nthreads,
                                   const PartitionFn *partition) {
  GridSettings gs = gs_in;
  // src/numint/molecular_grid.cpp:142-181 (ensure_settings)
  if (gs.max_angular_points < gs.min_angular_points)
    gs.max_angular_points = gs.min_angular_points + 1;
  gs.max_angular_points = level_at_or_above(gs.max_angular_points);
  gs.min_angular_points = level_at_or_above(gs.min_angular_points);

  const size_t natom = Z.size();
  // src/numint/molecular_grid.cpp:183-247: per-atom exponent ranges; the
  // angular-momentum range is the whole basis' l_max for every atom.
  const int lmax = basis.lmax;
  std::vector<double> amax(natom, 0.0);
  std::vector<std::vector<double>> amin(natom, std::vector<double>(lmax + 1, DBL_MAX));
  for (const auto &sh : basis.shells) {
    for (double e : sh.exps) {
      amin[sh.atom][sh.l] = std::min(amin[sh.atom][sh.l], e);
      amax[sh.atom] = std::max(amax[sh.atom], e);
    }
  }
  // one grid per element, generated from the first atom of that element
  std::vector<int> uniq(Z.begin(), Z.end());
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  std::vector<AtomGrid> egrid(uniq.size());
  for (size_t u = 0; u < uniq.size(); u++) {
    size_t first = 0;
    while (Z[first] != uniq[u])
      first++;
    egrid[u] = atom_grid(uniq[u], gs, amax[first], lmax, amin[first]);
  }
  std::vector<double> radii(natom), dist(natom * natom, 0.0);
  for (size_t i = 0; i < natom; i++)
    radii[i] = bragg_radius(Z[i]);
  for (size_t i = 0; i < natom; i++)
    for (size_t j = i + 1; j < natom; j++) {
      double dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1],
             dz = xyz[3 * i + 2] - xyz[3 * j + 2];
      dist[i * natom + j] = dist[j * natom + i] = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  // Treutler-Ahlrichs radius adjustment factors a_ij
  // (src/numint/grid_utils.cpp:125-137)
  std::vector<double> aij(natom * natom, 0.0);
  std::vector<char> adj(natom * natom, 0);
  for (size_t i = 0; i < natom; i++)
    for (size_t j = 0; j < i; j++) {
      double ri = radii[i], rj = radii[j];
      if (std::fabs(ri - rj) > 1e-14) {
        double xi = gs.treutler_alrichs_adjustment ? std::sqrt(ri / rj) : ri / rj;
        double u = (xi - 1) / (xi + 1);
        aij[i * natom + j] = u / (u * u - 1.0);
        adj[i * natom + j] = 1;
      }
    }

  MolecularGrid mg;
  long total = 0;
  std::vector<size_t> which(natom);
  for (size_t a = 0; a < natom; a++) {
    which[a] = std::lower_bound(uniq.begin(), uniq.end(), Z[a]) - uniq.begin();
    mg.atom_offset.push_back(total);
    mg.atom_count.push_back(static_cast<long>(egrid[which[a]].w.size()));
    total += static_cast<long>(egrid[which[a]].w.size());
  }
  mg.xyz.resize(3 * total);
  mg.w.resize(total);

  if (partition && *partition) {
    // positions, owners and radial x angular weights here; the partition elsewhere
    std::vector<int> owner(total);
    std::vector<double> wra(total), inv_dist(natom * natom, 0.0), adj_ab(natom * natom, 0.0);
    for (size_t a = 0; a < natom; a++) {
      const AtomGrid &g = egrid[which[a]];
      for (long k = 0; k < mg.atom_count[a]; k++) {
        const long gp = mg.atom_offset[a] + k;
        for (int dd = 0; dd < 3; dd++)
          mg.xyz[3 * gp + dd] = g.xyz[3 * k + dd] + xyz[3 * a + dd];
        owner[gp] = static_cast<int>(a);
        wra[gp] = g.w[k];
      }
    }
    for (size_t i = 0; i < natom; i++)
      for (size_t j = 0; j < natom; j++) {
        if (i != j)
          inv_dist[i * natom + j] = 1.0 / dist[i * natom + j];
        const size_t hi = std::max(i, j), lo = std::min(i, j);
        if (hi != lo && adj[hi * natom + lo])
          adj_ab[i * natom + j] = aij[hi * natom + lo];
      }
    PartitionInput in;
    in.natom = static_cast<int>(natom);
    in.atom_xyz = xyz.data();
    in.inv_dist = inv_dist.data();
    in.adj_ab = adj_ab.data();
    in.npts = total;
    in.xyz = mg.xyz.data();
    in.owner = owner.data();
    in.wra = wra.data();
    (*partition)(in, mg.w.data());
    return mg;
  }

#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
  (void)nthreads;
#endif
  // Becke partition weights (src/numint/grid_utils.cpp:149-200 and
  // src/numint/molecular_grid.cpp:46-82), one point at a time.
#pragma omp parallel num_threads(nt)
  {
    std::vector<double> d(natom), W(natom);
#pragma omp for schedule(dynamic, 256)
    for (long gp = 0; gp < total; gp++) {
      size_t a = std::upper_bound(mg.atom_offset.begin(), mg.atom_offset.end(), gp) -
                 mg.atom_offset.begin() - 1;
      const AtomGrid &g = egrid[which[a]];
      long k = gp - mg.atom_offset[a];
      double p[3] = {g.xyz[3 * k] + xyz[3 * a], g.xyz[3 * k + 1] + xyz[3 * a + 1],
                     g.xyz[3 * k + 2] + xyz[3 * a + 2]};
      for (size_t i = 0; i < natom; i++) {
        double dx = p[0] - xyz[3 * i], dy = p[1] - xyz[3 * i + 1], dz = p[2] - xyz[3 * i + 2];
        d[i] = std::sqrt(dx * dx + dy * dy + dz * dz);
        W[i] = 1.0;
      }
      for (size_t i = 0; i < natom; i++)
        for (size_t j = 0; j < i; j++) {
          double v = (d[i] - d[j]) / dist[i * natom + j];
          if (adj[i * natom + j])
            v += aij[i * natom + j] * (1 - v * v);
          for (int it = 0; it < 3; it++)
            v = (3 - v * v) * v * 0.5;
          if (std::fabs(1.0 - v) < 1e-14) {
            W[i] = 0.0;
          } else {
            W[i] *= 0.5 * (1.0 - v);
            W[j] *= 0.5 * (1.0 + v);
          }
        }
      double sum = 0.0;
      for (size_t i = 0; i < natom; i++)
        sum += W[i];
      for (int dd = 0; dd < 3; dd++)
        mg.xyz[3 * gp + dd] = p[dd];
      mg.w[gp] = g.w[k] * (W[a] / sum);
    }
  }
  return mg;
}

} // namespace occx
