// Host-side data model of the GB300 XC build: basis, molecular grid and the
// per-build plan (Morton-ordered point blocks with their screened shells).
// Everything here is set-up work done once per molecule; the per-iteration
// build runs on the device (xc_device.cuh).
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace occx {

// One contracted shell as OCC's gto::Shell holds it after
// Shell::incorporate_shell_norm (src/gto/shell.cpp:180-186): coefficients
// already carry the primitive and contraction normalisation.
struct Shell {
  int l = 0;
  int atom = 0;
  double origin[3] = {0, 0, 0}; // Bohr
  std::vector<double> exps;
  std::vector<double> coefs;
};

struct Basis {
  std::vector<Shell> shells;
  bool pure = true;
  std::vector<int> first_bf;
  int nbf = 0;
  int lmax = 0;
  int shell_size(int s) const {
    int l = shells[s].l;
    return pure ? 2 * l + 1 : (l + 1) * (l + 2) / 2;
  }
  void finalise();
};

// src/gto/shell.cpp:20-64, 180-186
void normalize_shell(int l, int nprim, const double *exps, double *coefs);
// src/gto/gto.cpp:7-16
double common_fac(int l, bool pure);
// Real solid harmonic transform, CCA order; T[(m+l)*ncart + cart].
const std::vector<double> &spherical_transform(int l);

// Mirrors occ::numint::GridSettings (include/occ/numint/grid_settings.h:81-95).
struct GridSettings {
  int max_angular_points = 302;
  int min_angular_points = 110;
  int radial_points = 50;
  double radial_precision = 1e-12;
  bool reduced_first_row_element_grid = true;
  bool treutler_alrichs_adjustment = true;
  int pruning_scheme = 1; // 0 none, 1 NWChem
};

// Molecular grid in OCC's layout: atom blocks concatenated in atom order
// (src/numint/molecular_grid_points.cpp:15-50).
struct MolecularGrid {
  std::vector<double> xyz; // 3 per point
  std::vector<double> w;
  std::vector<long> atom_offset, atom_count;
  long npts() const { return static_cast<long>(w.size()); }
};

int lebedev_rule(int npoints, std::vector<double> &xyzw); // returns count or 0

// The Becke partition step (src/numint/grid_utils.cpp:149-200,
// src/numint/molecular_grid.cpp:46-82) as data: atoms, the pair tables, and
// per point its position, owning atom and radial x angular weight.  inv_dist
// is 1/|R_i - R_j| (0 on the diagonal); adj_ab[i * natom + j] is the
// Treutler-Ahlrichs a_ij of the ordered pair (max(i, j), min(i, j)), 0 where
// the radii are equal.  A partition function writes w[p] = wra[p] *
// P_owner(p) / sum_i P_i(p).
struct PartitionInput {
  int natom = 0;
  const double *atom_xyz = nullptr;
  const double *inv_dist = nullptr;
  const double *adj_ab = nullptr;
  long npts = 0;
  const double *xyz = nullptr;
  const int *owner = nullptr;
  const double *wra = nullptr;
};
using PartitionFn = std::function<void(const PartitionInput &, double *w)>;

// partition: nullptr for the host loop (OpenMP over nthreads), else e.g. the
// device kernel of xc_grid.cu.
MolecularGrid build_molecular_grid(const std::vector<int> &Z, const std::vector<double> &xyz,
                                   const Basis &basis, const GridSettings &gs, int nthreads,
                                   const PartitionFn *partition = nullptr);

// Per-build settings (include/occ/dft/dft.h:760-761, spatial_grid_hierarchy.h:26-30).
struct BuildSettings {
  double xc_screening_threshold = 1e-10;
  double density_threshold = 1e-10;
  long leaf_target = 128, leaf_min = 32, leaf_max = 256;
};

// The plan: Morton-sorted points cut into leaves (the reference's blocking),
// and for each leaf the significant shells in ascending order with their
// local AO layout.
struct Plan {
  long npts = 0;
  std::vector<double> pts4;     // x, y, z, w per sorted point
  std::vector<long> perm;       // sorted -> original point index
  std::vector<long> leaf_off, leaf_cnt;
  std::vector<double> leaf_centre, leaf_radius;
  std::vector<double> extents; // per shell decay radius
  std::vector<long> leaf_sh_ptr; // CSR over leaves
  std::vector<int> leaf_sh;      // significant shells
  std::vector<int> leaf_nbf;     // m_b, local AO count
  long nleaves() const { return static_cast<long>(leaf_off.size()); }
};

std::vector<double> decay_cutoff(const Basis &basis, double threshold);
void morton_leaves(const MolecularGrid &grid, const BuildSettings &bs, Plan &plan);
void screen_leaves(const Basis &basis, const BuildSettings &bs, Plan &plan);
// Batches of `batch` consecutive points of each atom block, in the grid's
// own order (the seminumerical exchange's batching,
// src/qm/seminumerical_exchange.cpp:726-752), with their centroids and
// bounding radii; perm is the identity.
void atom_batch_leaves(const MolecularGrid &grid, long batch, Plan &plan);

// Host evaluation of one shell (values only) at n points; out[f*n + p].
void eval_shell_values(const Shell &sh, bool pure, long n, const double *xyz, double *out);

} // namespace occx
