// Per-molecule build plan: Morton-ordered leaves with bounding spheres
// (src/numint/spatial_grid_hierarchy.cpp:35-147), shell decay radii
// (src/gto/gto.cpp:18-67) and the per-leaf significant-shell lists of the
// screened XC build (include/occ/dft/dft.h:303-320).
#include "xc_host.hpp"

#include <algorithm>
#include <cmath>
#include <utility>

namespace occx {

namespace {
inline uint64_t spread3(uint64_t x) {
  x &= 0x1fffff;
  x = (x | (x << 32)) & 0x1f00000000ffffULL;
  x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
  x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
  x = (x | (x << 2)) & 0x1249249249249249ULL;
  return x;
}
} // namespace

std::vector<double> decay_cutoff(const Basis &basis, double threshold) {
  const double max_radius = 30.0, increment = 0.1, min_radius = 0.5;
  const int npts = static_cast<int>((max_radius - min_radius) / increment) + 1;
  const double step = (max_radius - min_radius) / (npts - 1);
  std::vector<double> ext(basis.shells.size(), 0.0);
  std::vector<double> xyz(3 * npts), vals;
  for (size_t s = 0; s < basis.shells.size(); s++) {
    const Shell &sh = basis.shells[s];
    for (int i = 0; i < npts; i++) {
      double x = (i == npts - 1) ? max_radius : min_radius + i * step;
      xyz[3 * i] = x + sh.origin[0];
      xyz[3 * i + 1] = sh.origin[1];
      xyz[3 * i + 2] = sh.origin[2];
    }
    int nf = basis.shell_size(static_cast<int>(s));
    vals.assign(static_cast<size_t>(nf) * npts, 0.0);
    eval_shell_values(sh, basis.pure, npts, xyz.data(), vals.data());
    for (int i = 0; i < npts; i++) {
      ext[s] = i * increment + min_radius;
      double v = 0.0;
      for (int f = 0; f < nf; f++)
        v = std::max(v, std::fabs(vals[static_cast<size_t>(f) * npts + i]));
      if (v < threshold)
        break;
    }
  }
  return ext;
}

void morton_leaves(const MolecularGrid &grid, const BuildSettings &bs, Plan &plan) {
  const long n = grid.npts();
  plan.npts = n;
  plan.perm.assign(n, 0);
  plan.pts4.assign(4 * n, 0.0);
  plan.leaf_off.clear();
  plan.leaf_cnt.clear();
  plan.leaf_centre.clear();
  plan.leaf_radius.clear();
  if (n == 0)
    return;
  double lo[3], hi[3], ext[3];
  for (int d = 0; d < 3; d++)
    lo[d] = hi[d] = grid.xyz[d];
  for (long i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      lo[d] = std::min(lo[d], grid.xyz[3 * i + d]);
      hi[d] = std::max(hi[d], grid.xyz[3 * i + d]);
    }
  for (int d = 0; d < 3; d++) {
    ext[d] = hi[d] - lo[d];
    if (ext[d] < 1e-10)
      ext[d] = 1.0;
  }
  const uint64_t scale = (1ULL << 21) - 1;
  std::vector<std::pair<uint64_t, long>> key(n);
  for (long i = 0; i < n; i++) {
    uint64_t q[3];
    for (int d = 0; d < 3; d++) {
      double u = (grid.xyz[3 * i + d] - lo[d]) / ext[d];
      u = std::min(std::max(u, 0.0), 1.0);
      q[d] = static_cast<uint64_t>(u * scale);
    }
    key[i] = {spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2), i};
  }
  std::sort(key.begin(), key.end());
  for (long i = 0; i < n; i++) {
    long o = key[i].second;
    plan.perm[i] = o;
    for (int d = 0; d < 3; d++)
      plan.pts4[4 * i + d] = grid.xyz[3 * o + d];
    plan.pts4[4 * i + 3] = grid.w[o];
  }
  long off = 0;
  while (off < n) {
    long rem = n - off, cnt;
    if (rem <= bs.leaf_max)
      cnt = rem;
    else if (rem < 2 * bs.leaf_min)
      cnt = rem / 2;
    else
      cnt = std::min(bs.leaf_target, rem);
    double c[3] = {0, 0, 0};
    for (long i = off; i < off + cnt; i++)
      for (int d = 0; d < 3; d++)
        c[d] += plan.pts4[4 * i + d];
    for (int d = 0; d < 3; d++)
      c[d] /= static_cast<double>(cnt);
    double r = 0.0;
    for (long i = off; i < off + cnt; i++) {
      double dx = plan.pts4[4 * i] - c[0], dy = plan.pts4[4 * i + 1] - c[1],
             dz = plan.pts4[4 * i + 2] - c[2];
      r = std::max(r, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    plan.leaf_off.push_back(off);
    plan.leaf_cnt.push_back(cnt);
    plan.leaf_centre.insert(plan.leaf_centre.end(), c, c + 3);
    plan.leaf_radius.push_back(r);
    off += cnt;
  }
}

void atom_batch_leaves(const MolecularGrid &grid, long batch, Plan &plan) {
  const long n = grid.npts();
  plan.npts = n;
  plan.perm.resize(n);
  plan.pts4.assign(4 * n, 0.0);
  plan.leaf_off.clear();
  plan.leaf_cnt.clear();
  plan.leaf_centre.clear();
  plan.leaf_radius.clear();
  for (long i = 0; i < n; i++) {
    plan.perm[i] = i;
    for (int d = 0; d < 3; d++)
      plan.pts4[4 * i + d] = grid.xyz[3 * i + d];
    plan.pts4[4 * i + 3] = grid.w[i];
  }
  for (size_t a = 0; a < grid.atom_offset.size(); a++) {
    const long a0 = grid.atom_offset[a], na = grid.atom_count[a];
    for (long b0 = 0; b0 < na; b0 += batch) {
      const long off = a0 + b0, cnt = std::min(batch, na - b0);
      double c[3] = {0, 0, 0};
      for (long i = off; i < off + cnt; i++)
        for (int d = 0; d < 3; d++)
          c[d] += grid.xyz[3 * i + d];
      for (int d = 0; d < 3; d++)
        c[d] /= static_cast<double>(cnt);
      double r = 0.0;
      for (long i = off; i < off + cnt; i++) {
        const double dx = grid.xyz[3 * i] - c[0], dy = grid.xyz[3 * i + 1] - c[1],
                     dz = grid.xyz[3 * i + 2] - c[2];
        r = std::max(r, std::sqrt(dx * dx + dy * dy + dz * dz));
      }
      plan.leaf_off.push_back(off);
      plan.leaf_cnt.push_back(cnt);
      plan.leaf_centre.insert(plan.leaf_centre.end(), c, c + 3);
      plan.leaf_radius.push_back(r);
    }
  }
}

void screen_leaves(const Basis &basis, const BuildSettings &bs, Plan &plan) {
  const long nl = plan.nleaves();
  const int nsh = static_cast<int>(basis.shells.size());
  plan.extents = decay_cutoff(basis, bs.xc_screening_threshold);
  plan.leaf_sh_ptr.assign(nl + 1, 0);
  plan.leaf_sh.clear();
  plan.leaf_nbf.assign(nl, 0);
  for (long b = 0; b < nl; b++) {
    const double *c = &plan.leaf_centre[3 * b];
    int m = 0;
    for (int s = 0; s < nsh; s++) {
      const double *A = basis.shells[s].origin;
      double dx = A[0] - c[0], dy = A[1] - c[1], dz = A[2] - c[2];
      double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (dist - plan.extents[s] < plan.leaf_radius[b]) {
        plan.leaf_sh.push_back(s);
        m += basis.shell_size(s);
      }
    }
    plan.leaf_sh_ptr[b + 1] = static_cast<long>(plan.leaf_sh.size());
    plan.leaf_nbf[b] = m;
  }
}

} // namespace occx
