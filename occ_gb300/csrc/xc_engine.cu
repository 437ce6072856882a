// Engine and C ABI of the GB300 XC build (include/occ_xc.h).
//
// occ_xc_molecule_create does OCC's set-up (grid, leaves, screening) once on
// the host and uploads the result; occ_xc_compute_vxc runs the per-iteration
// build on the device.  All device memory of a molecule is allocated at
// creation so that a build allocates nothing.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/occ_xc.h"
#include "host/gto_eval.h"
#include "host/xc_host.hpp"
#include "functionals_mgga.cuh"
#include "xc_device.cuh"
#include "xc_engine.hpp"

namespace occx {

void fill_sph_table(double *out) {
  for (int l = 0; l <= kMaxL; l++) {
    const std::vector<double> &T = spherical_transform(l);
    std::copy(T.begin(), T.end(), out + sph_offset(l));
  }
}

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess)
    throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// OCC method names -> functional components (share/methods/dft_methods.json,
// src/dft/dft_method.cpp:14-37, 161-227).  Component scale factors are not
// applied, as in OCC's DensityFunctional::evaluate.
FuncSet parse_method(const std::string &method_in) {
  std::string method;
  for (char c : method_in)
    method.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(c))));
  std::istringstream ss(method);
  std::string tok;
  FuncSet fs{};
  auto add = [&](int id) {
    if (fs.n >= kMaxFuncs)
      throw MethodError("too many functional components");
    fs.id[fs.n] = id;
    fs.coef[fs.n] = 1.0;
    fs.n++;
  };
  while (ss >> tok) {
    if (!tok.empty() && tok[0] == 'u')
      throw MethodError("unrestricted (spin-polarised) XC is not supported: " + tok);
    if (tok == "lda" || tok == "svwn" || tok == "lsda") {
      add(kLdaX);
      add(kLdaCVwn3);
    } else if (tok == "svwn5") {
      add(kLdaX);
      add(kLdaCVwn);
    } else if (tok == "pbe" || tok == "pbepbe" || tok == "pbe0" || tok == "pbe1pbe") {
      add(kGgaXPbe);
      add(kGgaCPbe);
    } else if (tok == "blyp") {
      add(kGgaXB88);
      add(kGgaCLyp);
    } else if (tok == "bpbe") {
      add(kGgaXB88);
      add(kGgaCPbe);
    } else if (tok == "b3lyp") {
      add(kHybB3lyp);
    } else if (tok == "b3lyp5") {
      add(kHybB3lyp5);
    } else if (tok == "pbeh" || tok == "hyb_gga_xc_pbeh") {
      add(kHybPbeh);
    } else if (tok == "bhandh" || tok == "hyb_gga_xc_bhandh") {
      add(kHybBhandh);
    } else if (tok == "bhandhlyp" || tok == "hyb_gga_xc_bhandhlyp") {
      add(kHybBhandhlyp);
    } else if (tok == "vwn5") {
      add(kLdaCVwn);
    } else if (tok == "tpss") {
      add(kMggaXTpss);
      add(kMggaCTpss);
    } else if (tok == "mgga_x_tpss" || tok == "xc_mgga_x_tpss") {
      add(kMggaXTpss);
    } else if (tok == "mgga_c_tpss" || tok == "xc_mgga_c_tpss") {
      add(kMggaCTpss);
    } else if (tok == "lda_x" || tok == "xc_lda_x") {
      add(kLdaX);
    } else if (tok == "lda_c_vwn" || tok == "xc_lda_c_vwn") {
      add(kLdaCVwn);
    } else if (tok == "lda_c_vwn_rpa" || tok == "xc_lda_c_vwn_rpa") {
      add(kLdaCVwnRpa);
    } else if (tok == "lda_c_vwn_3" || tok == "xc_lda_c_vwn_3") {
      add(kLdaCVwn3);
    } else if (tok == "gga_x_pbe" || tok == "xc_gga_x_pbe") {
      add(kGgaXPbe);
    } else if (tok == "gga_c_pbe" || tok == "xc_gga_c_pbe") {
      add(kGgaCPbe);
    } else if (tok == "gga_x_b88" || tok == "xc_gga_x_b88") {
      add(kGgaXB88);
    } else if (tok == "gga_c_lyp" || tok == "xc_gga_c_lyp") {
      add(kGgaCLyp);
    } else {
      throw MethodError("unknown or unsupported functional: " + tok);
    }
  }
  if (fs.n == 0)
    throw MethodError("empty method string");
  return fs;
}

void require_not_mgga(int deriv, const char *what) {
  if (deriv == 2)
    throw ArgError(std::string(what) + ": not available for meta-GGA functionals "
                   "(the restricted FP64 build is)");
}

Molecule::~Molecule() {
  for (void *p : allocations)
    cudaFree(p);
  free_mixed(mixed);
  free_grad_mixed(gmixed);
  free_meta_mixed(mmixed);
}

void *Molecule::alloc(size_t bytes) {
  void *p = nullptr;
  cuda_check(cudaMalloc(&p, std::max<size_t>(bytes, 16)), "cudaMalloc");
  allocations.push_back(p);
  device_bytes += static_cast<double>(bytes);
  return p;
}

static size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

void Molecule::build_plan() {
  // on the molecule's GPU; OCC_XC_PLAN=host selects the host restatement
  // (host/plan.cpp), which gives the same plan (tests compare the two)
  const char *sel = std::getenv("OCC_XC_PLAN");
  if (atom_batch > 0) {
    atom_batch_leaves(grid, atom_batch, plan);
    screen_leaves(basis, bs, plan);
  } else if (sel && std::strcmp(sel, "host") == 0) {
    morton_leaves(grid, bs, plan);
    screen_leaves(basis, bs, plan);
  } else {
    device_plan(device, grid, basis, bs, plan);
  }
  const int ncomp = deriv ? 4 : 1;
  leaves.clear();
  leaf_sh.clear();
  leaf_ao.clear();
  slabs.clear();
  tiles.clear();
  ws_elems = 0;
  flops = 0.0;
  for (long b = 0; b < plan.nleaves(); b++) {
    const int m = plan.leaf_nbf[b];
    if (m == 0)
      continue; // no significant shell: the leaf contributes nothing (dft.h:321-322)
    DevLeaf L{};
    L.off = static_cast<int>(plan.leaf_off[b]);
    L.cnt = static_cast<int>(plan.leaf_cnt[b]);
    L.sh_begin = static_cast<int>(leaf_sh.size());
    L.ao_begin = static_cast<int>(leaf_ao.size());
    for (long k = plan.leaf_sh_ptr[b]; k < plan.leaf_sh_ptr[b + 1]; k++) {
      int s = plan.leaf_sh[k];
      leaf_sh.push_back(s);
      for (int f = 0; f < basis.shell_size(s); f++)
        leaf_ao.push_back(basis.first_bf[s] + f);
    }
    L.sh_end = static_cast<int>(leaf_sh.size());
    L.nbf = m;
    L.mpad = static_cast<int>(round_up(m, kAoTile));
    L.npad = static_cast<int>(round_up(L.cnt, kPtTile));
    L.ws_off = static_cast<long long>(ws_elems);
    ws_elems += static_cast<size_t>(ncomp) * L.mpad * L.npad;
    const int li = static_cast<int>(leaves.size());
    for (int p0 = 0; p0 < L.npad; p0 += kPtTile)
      slabs.push_back({li, p0});
    for (int i0 = 0; i0 < L.mpad; i0 += kAoTile)
      for (int j0 = 0; j0 < L.mpad; j0 += kAoTile)
        tiles.push_back({li, i0, j0, 0});
    flops += 4.0 * L.cnt * static_cast<double>(m) * m;
    leaves.push_back(L);
  }
  // longest slabs (cost m^2) first, so that the launch does not end on a
  // tail of a few long CTAs
  std::stable_sort(slabs.begin(), slabs.end(), [&](const SlabItem &a, const SlabItem &b) {
    return leaves[a.leaf].mpad > leaves[b.leaf].mpad;
  });
  std::stable_sort(tiles.begin(), tiles.end(), [&](const TileItem &a, const TileItem &b) {
    return leaves[a.leaf].npad > leaves[b.leaf].npad; // tile cost: its K = npad points
  });
}

void Molecule::upload() {
  size_t bytes = 0;
  std::vector<DevShell> sh(basis.shells.size());
  std::vector<double2> prims;
  for (size_t s = 0; s < basis.shells.size(); s++) {
    const Shell &S = basis.shells[s];
    DevShell &d = sh[s];
    for (int k = 0; k < 3; k++)
      d.A[k] = S.origin[k];
    d.fac = common_fac(S.l, basis.pure);
    d.l = S.l;
    d.nprim = static_cast<int>(S.exps.size());
    d.prim_off = static_cast<int>(prims.size());
    d.nfunc = basis.shell_size(static_cast<int>(s));
    for (size_t k = 0; k < S.exps.size(); k++)
      prims.push_back(make_double2(S.exps[k], S.coefs[k]));
  }
  std::vector<Pt4> pts(plan.npts);
  for (long i = 0; i < plan.npts; i++)
    pts[i] = make_pt4(plan.pts4[4 * i], plan.pts4[4 * i + 1], plan.pts4[4 * i + 2],
                          plan.pts4[4 * i + 3]);
  d_pts = dev_upload(pts, bytes);
  allocations.push_back(d_pts);
  d_shells = dev_upload(sh, bytes);
  allocations.push_back(d_shells);
  d_prims = dev_upload(prims, bytes);
  allocations.push_back(d_prims);
  d_leaves = dev_upload(leaves, bytes);
  allocations.push_back(d_leaves);
  d_leaf_sh = dev_upload(leaf_sh, bytes);
  allocations.push_back(d_leaf_sh);
  d_leaf_ao = dev_upload(leaf_ao, bytes);
  allocations.push_back(d_leaf_ao);
  d_slabs = dev_upload(slabs, bytes);
  allocations.push_back(d_slabs);
  d_tiles = dev_upload(tiles, bytes);
  allocations.push_back(d_tiles);
  device_bytes += static_cast<double>(bytes);

  const size_t N = static_cast<size_t>(std::max<long>(plan.npts, 1));
  const size_t nl = std::max<size_t>(leaves.size(), 1);
  d_rho = static_cast<double *>(alloc(rho_components(deriv) * N * sizeof(double)));
  d_coef = static_cast<double *>(alloc(coef_components(deriv) * N * sizeof(double)));
  d_epart = static_cast<double *>(alloc(2 * nl * sizeof(double)));
  d_out2 = static_cast<double *>(alloc(2 * sizeof(double)));
  const size_t nbf2 = static_cast<size_t>(basis.nbf) * basis.nbf;
  d_D = static_cast<double *>(alloc(std::max<size_t>(nbf2, 1) * sizeof(double)));
  d_V = static_cast<double *>(alloc(std::max<size_t>(nbf2, 1) * sizeof(double)));
  cuda_check(cudaMemset(d_rho, 0, rho_components(deriv) * N * sizeof(double)), "cudaMemset");
}

MolDev Molecule::dev() const {
  MolDev m;
  m.pts = d_pts;
  m.shells = d_shells;
  m.prims = d_prims;
  m.leaves = d_leaves;
  m.leaf_sh = d_leaf_sh;
  m.leaf_ao = d_leaf_ao;
  m.nleaves = static_cast<int>(leaves.size());
  m.npts = static_cast<int>(plan.npts);
  m.nbf = basis.nbf;
  m.pure = basis.pure ? 1 : 0;
  return m;
}

// One restricted XC build on device buffers (the FP64 sequence).
void Molecule::ensure_fp64_ws() {
  if (!d_ws)
    d_ws = static_cast<double *>(alloc(std::max<size_t>(ws_elems, 1) * sizeof(double)));
}

void Molecule::prepare(int precision) {
  if (precision == OCC_XC_MIXED && deriv == 2)
    prepare_mgga_mixed();
  else if (precision == OCC_XC_MIXED)
    ensure_mixed_ws();
  else
    ensure_fp64_ws();
}

void Molecule::build_fp64(const double *dD, double *dV, double *dout2, cudaStream_t st,
                          double *ws, bool ws_holds_ao) {
  bool skip_colloc = ws && ws_holds_ao;
  if (!ws) {
    ensure_fp64_ws();
    ws = d_ws;
    skip_colloc = fp64_ao_valid; // the private workspace keeps the AO values
  }
  const MolDev m = dev();
  const size_t nbf2 = static_cast<size_t>(basis.nbf) * basis.nbf;
  Context &c = *ctx;
  cuda_check(cudaMemsetAsync(dV, 0, nbf2 * sizeof(double), st), "cudaMemsetAsync");
  if (!skip_colloc)
    c.launch("colloc_f64", st, [&] { launch_colloc_f64(m, deriv, ws, st); });
  c.launch("rho_f64", st, [&] {
    launch_rho_f64(m, deriv, dD, ws, d_slabs, static_cast<int>(slabs.size()), d_rho, st);
  });
  if (deriv == 2)
    c.launch("tau_f64", st, [&] {
      launch_tau_f64(m, dD, ws, d_slabs, static_cast<int>(slabs.size()), d_rho, st);
    });
  c.launch("func", st, [&] {
    launch_func(m, deriv, fs, bs.density_threshold, d_rho, d_coef, d_epart, st);
  });
  c.launch("vxc_f64", st, [&] {
    launch_vxc_f64(m, deriv, ws, d_coef, d_tiles, static_cast<int>(tiles.size()), dV, st);
  });
  c.launch("reduce", st, [&] { launch_reduce(d_epart, m.nleaves, dout2, st); });
  cuda_check(cudaGetLastError(), "kernel launch");
  if (ws == d_ws)
    fp64_ao_valid = true;
}

void Molecule::build(int precision, const double *dD, double *dV, double *dout2,
                     cudaStream_t st) {
  if (precision == OCC_XC_MIXED)
    build_mixed(dD, dV, dout2, st);
  else
    build_fp64(dD, dV, dout2, st);
}

cudaEvent_t KernelProfiler::get() {
  if (pool.empty()) {
    cudaEvent_t e;
    cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    return e;
  }
  cudaEvent_t e = pool.back();
  pool.pop_back();
  return e;
}

void KernelProfiler::begin(const char *name, cudaStream_t st) {
  Rec r{name, get(), get()};
  cuda_check(cudaEventRecord(r.a, st), "cudaEventRecord");
  pending.push_back(r);
}

void KernelProfiler::end(cudaStream_t st) {
  cuda_check(cudaEventRecord(pending.back().b, st), "cudaEventRecord");
}

void KernelProfiler::collect() {
  for (Rec &r : pending) {
    cuda_check(cudaEventSynchronize(r.b), "cudaEventSynchronize");
    float ms = 0.f;
    cuda_check(cudaEventElapsedTime(&ms, r.a, r.b), "cudaEventElapsedTime");
    Total *t = nullptr;
    for (Total &x : totals)
      if (x.name == r.name)
        t = &x;
    if (!t) {
      totals.push_back(Total{r.name, 0.0, 0});
      t = &totals.back();
    }
    t->ms += ms;
    t->launches++;
    pool.push_back(r.a);
    pool.push_back(r.b);
  }
  pending.clear();
}

KernelProfiler::~KernelProfiler() {
  for (Rec &r : pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : pool)
    cudaEventDestroy(e);
}

Context::Context(int dev) : device(dev) {
  cuda_check(cudaSetDevice(dev), "cudaSetDevice");
  cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  upload_sph_table();
  upload_sph_table_mixed();
  upload_sph_table_grad();
}
Context::~Context() {
  if (stream)
    cudaStreamDestroy(stream);
}


Basis make_basis(int natoms, const double *xyz, int nshells, const int *shell_l,
                 const int *shell_atom, const int *shell_nprim, const double *exponents,
                 const double *coefficients, int pure) {
  Basis basis;
  basis.pure = pure != 0;
  size_t off = 0;
  for (int s = 0; s < nshells; s++) {
    if (shell_l[s] < 0 || shell_l[s] > kMaxL)
      throw ArgError("shell angular momentum must be in 0..4");
    if (shell_atom[s] < 0 || shell_atom[s] >= natoms || shell_nprim[s] <= 0)
      throw ArgError("bad shell atom index or primitive count");
    Shell sh;
    sh.l = shell_l[s];
    sh.atom = shell_atom[s];
    for (int k = 0; k < 3; k++)
      sh.origin[k] = xyz[3 * sh.atom + k];
    sh.exps.assign(exponents + off, exponents + off + shell_nprim[s]);
    sh.coefs.assign(coefficients + off, coefficients + off + shell_nprim[s]);
    off += shell_nprim[s];
    basis.shells.push_back(sh);
  }
  basis.finalise();
  return basis;
}

GridSettings grid_settings_from(const occ_xc_grid_settings *grid) {
  GridSettings gs;
  if (grid) {
    gs.max_angular_points = grid->max_angular_points;
    gs.min_angular_points = grid->min_angular_points;
    gs.radial_points = grid->radial_points;
    gs.radial_precision = grid->radial_precision;
    gs.reduced_first_row_element_grid = grid->reduced_first_row_element_grid != 0;
    gs.treutler_alrichs_adjustment = grid->treutler_alrichs_adjustment != 0;
    gs.pruning_scheme = grid->pruning_scheme;
  }
  return gs;
}


void check_build_settings(const BuildSettings &b) {
  if (b.leaf_max > 1024 || b.leaf_target <= 0 || b.leaf_min <= 0 || b.leaf_target > b.leaf_max ||
      2 * b.leaf_min > b.leaf_max)
    throw ArgError("leaf sizes must satisfy 0 < target <= max <= 1024, 2 min <= max");
  if (!(b.xc_screening_threshold >= 0.0) || !(b.density_threshold >= 0.0))
    throw ArgError("thresholds must be non-negative");
}

std::unique_ptr<Molecule> molecule_host(Context *ctx, const MoleculeArgs &a) {
  if (a.natoms <= 0 || a.nshells <= 0 || !a.Z || !a.xyz || !a.shell_l || !a.shell_atom ||
      !a.shell_nprim || !a.exponents || !a.coefficients || !a.method)
    throw ArgError("molecule: missing or empty input");
  auto M = std::make_unique<Molecule>();
  M->ctx = ctx;
  M->device = ctx->device;
  M->fs = parse_method(a.method);
  M->deriv = 0;
  for (int i = 0; i < M->fs.n; i++)
    M->deriv = std::max(M->deriv, func_is_mgga(M->fs.id[i]) ? 2
                                  : func_is_gga(M->fs.id[i]) ? 1
                                                             : 0);
  M->Z.assign(a.Z, a.Z + a.natoms);
  M->xyz.assign(a.xyz, a.xyz + 3 * a.natoms);
  M->basis = make_basis(a.natoms, a.xyz, a.nshells, a.shell_l, a.shell_atom,
                                a.shell_nprim, a.exponents, a.coefficients, a.pure);
  M->gs = grid_settings_from(a.grid);
  if (a.build) {
    M->bs.xc_screening_threshold = a.build->xc_screening_threshold;
    M->bs.density_threshold = a.build->density_threshold;
    M->bs.leaf_target = a.build->leaf_target;
    M->bs.leaf_min = a.build->leaf_min;
    M->bs.leaf_max = a.build->leaf_max;
    check_build_settings(M->bs);
  }
  // the Becke partition on the molecule's device when it fits there
  PartitionFn part;
  if (device_partition_fits(ctx->device, a.natoms))
    part = [dev = ctx->device](const PartitionInput &in, double *w) {
      device_partition(dev, in, w);
    };
  M->grid = build_molecular_grid(M->Z, M->xyz, M->basis, M->gs, 0, part ? &part : nullptr);
  M->build_plan();
  return M;
}

void replan(Molecule &M, const BuildSettings &b) {
  check_build_settings(b);
  const bool had = !M.allocations.empty();
  if (had)
    M.release_device();
  M.bs = b;
  M.build_plan();
  if (had)
    M.materialise();
}

void Molecule::materialise() {
  upload();
  prepare_mixed();
}

void Molecule::release_device() {
  for (void *p : allocations)
    cudaFree(p);
  allocations.clear();
  free_mixed(mixed);
  mixed = nullptr;
  device_bytes = 0.0;
  d_pts = nullptr;
  d_shells = nullptr;
  d_prims = nullptr;
  d_leaves = nullptr;
  d_leaf_sh = d_leaf_ao = nullptr;
  d_slabs = nullptr;
  d_tiles = nullptr;
  d_ws = d_rho = d_coef = d_epart = d_out2 = d_D = d_V = nullptr;
  fp64_ao_valid = false;
  ggroups.clear();
  d_gleaves = nullptr;
  d_gslabs = nullptr;
  d_ao_atom = nullptr;
  d_gws = d_grad = nullptr;
  grad_bytes = 0.0;
  d_rho_b = d_coef_b = d_epart_u = d_Dab = d_Vab = d_Duks = d_Vuks = d_out3 = nullptr;
  d_uks_tabs = nullptr;
  d_uks_tabs_meta = nullptr;
  nlc.reset();
  free_grad_mixed(gmixed);
  gmixed = nullptr;
  free_meta_mixed(mmixed);
  mmixed = nullptr;
}

// Device bytes that materialise() allocates -- the resident state, without the
// per-build workspaces (an upper bound: every array rounded up to 256 bytes,
// plus the mixed path's launch lists).
double Molecule::estimate_resident_bytes() const {
  auto r = [](double b) { return std::ceil(std::max(b, 16.0) / 256.0) * 256.0; };
  const double N = static_cast<double>(std::max<long>(plan.npts, 1));
  const double nl = static_cast<double>(std::max<size_t>(leaves.size(), 1));
  const double nbf2 = static_cast<double>(basis.nbf) * basis.nbf;
  double nprim = 0;
  for (const Shell &sh : basis.shells)
    nprim += static_cast<double>(sh.exps.size());
  const double nsh = static_cast<double>(basis.shells.size());
  double b = r(N * sizeof(Pt4)) + r(nsh * sizeof(DevShell)) + r(nprim * sizeof(double2)) +
             r(nl * sizeof(DevLeaf)) + r(leaf_sh.size() * 4.0) + r(leaf_ao.size() * 4.0) +
             r(slabs.size() * sizeof(SlabItem)) + r(tiles.size() * sizeof(TileItem));
  b += r(rho_components(deriv) * N * 8.0) + r(coef_components(deriv) * N * 8.0) + r(2 * nl * 8.0) + r(16.0) + 2 * r(nbf2 * 8.0);
  double blocks = 0, items = 0;
  for (const DevLeaf &L : leaves) {
    const double nb = std::ceil(L.cnt / 128.0);
    blocks += nb;
    items += nb * std::ceil(std::ceil(L.nbf / 32.0) * 32.0 / 128.0);
  }
  b += r(nprim * 16.0) + r(2 * nsh * 16.0) + r(16.0);
  b += r(blocks * 32.0) + r(blocks * 4.0) + r(items * 8.0) + r(nl * 8.0) + r(4096.0) + r(16.0);
  return b;
}

size_t Molecule::fp64_workspace_bytes() const {
  return std::max<size_t>(ws_elems, 1) * sizeof(double);
}

} // namespace occx

using namespace occx;


extern "C" {

void occ_xc_default_grid_settings(occ_xc_grid_settings *o) {
  GridSettings g;
  o->max_angular_points = g.max_angular_points;
  o->min_angular_points = g.min_angular_points;
  o->radial_points = g.radial_points;
  o->radial_precision = g.radial_precision;
  o->reduced_first_row_element_grid = g.reduced_first_row_element_grid;
  o->treutler_alrichs_adjustment = g.treutler_alrichs_adjustment;
  o->pruning_scheme = g.pruning_scheme;
}

void occ_xc_default_build_settings(occ_xc_build_settings *o) {
  BuildSettings b;
  o->xc_screening_threshold = b.xc_screening_threshold;
  o->density_threshold = b.density_threshold;
  o->leaf_target = static_cast<int>(b.leaf_target);
  o->leaf_min = static_cast<int>(b.leaf_min);
  o->leaf_max = static_cast<int>(b.leaf_max);
}

int occ_xc_normalize_shell(int l, int nprim, const double *exps, double *coefs) {
  if (l < 0 || l > kMaxL || nprim <= 0 || !exps || !coefs)
    return OCC_XC_ERR_ARG;
  normalize_shell(l, nprim, exps, coefs);
  return OCC_XC_OK;
}

} // extern "C"

namespace {
// occ_xc_molecular_grid[_device]: the count alone needs no partition weights.
int molecular_grid_impl(occ_xc_context *ctx, int natoms, const int *Z, const double *xyz,
                        int nshells, const int *shell_l, const int *shell_atom,
                        const int *shell_nprim, const double *exponents,
                        const double *coefficients, int pure, const occ_xc_grid_settings *grid,
                        long *npoints, double *points, double *weights) {
  if (natoms <= 0 || nshells <= 0 || !Z || !xyz || !shell_l || !shell_atom || !shell_nprim ||
      !exponents || !coefficients || !npoints)
    return OCC_XC_ERR_ARG;
  auto run = [&] {
    Basis basis = make_basis(natoms, xyz, nshells, shell_l, shell_atom, shell_nprim, exponents,
                             coefficients, pure);
    GridSettings gs = grid_settings_from(grid);
    const bool fill = points && weights;
    PartitionFn part;
    if (!fill)
      part = [](const PartitionInput &, double *) {};
    else if (ctx)
      part = [dev = ctx->impl->device](const PartitionInput &in, double *w) {
        device_partition(dev, in, w);
      };
    MolecularGrid mg = build_molecular_grid(std::vector<int>(Z, Z + natoms),
                                            std::vector<double>(xyz, xyz + 3 * natoms), basis, gs,
                                            0, part ? &part : nullptr);
    if (fill) {
      if (*npoints < mg.npts())
        throw ArgError("point buffers smaller than the grid");
      std::memcpy(points, mg.xyz.data(), mg.xyz.size() * sizeof(double));
      std::memcpy(weights, mg.w.data(), mg.w.size() * sizeof(double));
    }
    *npoints = mg.npts();
  };
  if (ctx) {
    if (!device_partition_fits(ctx->impl->device, natoms))
      return OCC_XC_ERR_ARG;
    std::lock_guard<std::mutex> lock(ctx->mu);
    return guarded(ctx, run);
  }
  try {
    run();
    return OCC_XC_OK;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "occ_xc_molecular_grid: %s\n", e.what());
    return OCC_XC_ERR_ARG;
  }
}
} // namespace

extern "C" {

int occ_xc_molecular_grid(int natoms, const int *Z, const double *xyz, int nshells,
                          const int *shell_l, const int *shell_atom, const int *shell_nprim,
                          const double *exponents, const double *coefficients, int pure,
                          const occ_xc_grid_settings *grid, long *npoints, double *points,
                          double *weights) {
  return molecular_grid_impl(nullptr, natoms, Z, xyz, nshells, shell_l, shell_atom, shell_nprim,
                             exponents, coefficients, pure, grid, npoints, points, weights);
}

int occ_xc_molecular_grid_device(occ_xc_context *ctx, int natoms, const int *Z,
                                 const double *xyz, int nshells, const int *shell_l,
                                 const int *shell_atom, const int *shell_nprim,
                                 const double *exponents, const double *coefficients, int pure,
                                 const occ_xc_grid_settings *grid, long *npoints, double *points,
                                 double *weights) {
  if (!ctx)
    return OCC_XC_ERR_ARG;
  return molecular_grid_impl(ctx, natoms, Z, xyz, nshells, shell_l, shell_atom, shell_nprim,
                             exponents, coefficients, pure, grid, npoints, points, weights);
}

int occ_xc_lebedev(int n, double *xyzw) {
  if (!xyzw)
    return 0;
  std::vector<double> v;
  const int got = lebedev_rule(n, v);
  if (got != n)
    return 0;
  std::memcpy(xyzw, v.data(), v.size() * sizeof(double));
  return n;
}

int occ_xc_context_create(int device, occ_xc_context **out) {
  if (!out)
    return OCC_XC_ERR_ARG;
  *out = nullptr;
  auto ctx = std::make_unique<occ_xc_context>();
  int rc = guarded(ctx.get(), [&] { ctx->impl = std::make_unique<Context>(device); });
  if (rc != OCC_XC_OK) {
    std::fprintf(stderr, "occ_xc_context_create: %s\n", ctx->err.c_str());
    return rc;
  }
  *out = ctx.release();
  return OCC_XC_OK;
}

void occ_xc_context_destroy(occ_xc_context *ctx) { delete ctx; }

const char *occ_xc_last_error(const occ_xc_context *ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

int occ_xc_molecule_create(occ_xc_context *ctx, int natoms, const int *Z, const double *xyz,
                           int nshells, const int *shell_l, const int *shell_atom,
                           const int *shell_nprim, const double *exponents,
                           const double *coefficients, int pure, const char *method,
                           const occ_xc_grid_settings *grid, const occ_xc_build_settings *build,
                           occ_xc_molecule **out) {
  if (!ctx || !out)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  *out = nullptr;
  auto mol = std::make_unique<occ_xc_molecule>();
  mol->ctx = ctx;
  int rc = guarded(ctx, [&] {
    MoleculeArgs a{natoms, Z, xyz, nshells, shell_l, shell_atom, shell_nprim, exponents,
                   coefficients, pure, method, grid, build};
    cuda_check(cudaSetDevice(ctx->impl->device), "cudaSetDevice");
    auto M = molecule_host(ctx->impl.get(), a);
    M->materialise();
    mol->impl = std::move(M);
  });
  if (rc == OCC_XC_OK)
    *out = mol.release();
  return rc;
}

void occ_xc_molecule_destroy(occ_xc_molecule *mol) {
  if (!mol)
    return;
  // the molecule may outlive its context (e.g. at process exit): use its own
  // device ordinal, never the context
  if (mol->impl)
    cudaSetDevice(mol->impl->device);
  delete mol;
}

int occ_xc_molecule_info_get(const occ_xc_molecule *mol, occ_xc_molecule_info *o) {
  if (!mol || !o)
    return OCC_XC_ERR_ARG;
  const Molecule &M = *mol->impl;
  o->nbf = M.basis.nbf;
  o->natoms = static_cast<int>(M.Z.size());
  o->nshells = static_cast<int>(M.basis.shells.size());
  o->deriv = M.deriv;
  o->npoints = M.plan.npts;
  o->nleaves = static_cast<long>(M.leaves.size());
  o->flops_per_build = M.flops;
  o->device_bytes = M.device_bytes;
  o->workspace_bytes = static_cast<double>(M.fp64_workspace_bytes());
  o->mixed_workspace_bytes = M.mixed ? static_cast<double>(M.mixed_workspace_bytes()) : 0.0;
  o->resident_bytes = M.estimate_resident_bytes();
  return OCC_XC_OK;
}

int occ_xc_molecule_grid(const occ_xc_molecule *mol, double *points, double *weights) {
  if (!mol || !points || !weights)
    return OCC_XC_ERR_ARG;
  const Molecule &M = *mol->impl;
  std::memcpy(points, M.grid.xyz.data(), M.grid.xyz.size() * sizeof(double));
  std::memcpy(weights, M.grid.w.data(), M.grid.w.size() * sizeof(double));
  return OCC_XC_OK;
}

int occ_xc_compute_vxc_device(occ_xc_context *ctx, occ_xc_molecule *mol, const double *d_D,
                              int precision, double *d_V, double *d_exc2, void *stream) {
  if (!ctx || !mol || !d_D || !d_V || !d_exc2)
    return OCC_XC_ERR_ARG;
  if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->impl->stream;
    mol->impl->build(precision, d_D, d_V, d_exc2, st);
  });
}

int occ_xc_compute_vxc(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D,
                       int precision, double *V, double *exc, double *nelec_out) {
  if (!ctx || !mol || !D || !V || !exc)
    return OCC_XC_ERR_ARG;
  if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    Molecule &M = *mol->impl;
    cudaStream_t st = ctx->impl->stream;
    const size_t nbf2 = static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
    cuda_check(cudaMemcpyAsync(M.d_D, D, nbf2 * sizeof(double), cudaMemcpyHostToDevice, st),
               "cudaMemcpyAsync H2D");
    M.build(precision, M.d_D, M.d_V, M.d_out2, st);
    double out2[2];
    cuda_check(cudaMemcpyAsync(V, M.d_V, nbf2 * sizeof(double), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaMemcpyAsync(out2, M.d_out2, sizeof(out2), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (precision == OCC_XC_MIXED && mixed_error_flag(M, st))
      throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
    *exc = out2[0];
    if (nelec_out)
      *nelec_out = out2[1];
  });
}

} // extern "C"

extern "C" {

int occ_xc_molecule_leaves(const occ_xc_molecule *mol, int *npoints, int *nbf_local) {
  if (!mol || !npoints || !nbf_local)
    return OCC_XC_ERR_ARG;
  const Molecule &M = *mol->impl;
  for (size_t i = 0; i < M.leaves.size(); i++) {
    npoints[i] = M.leaves[i].cnt;
    nbf_local[i] = M.leaves[i].nbf;
  }
  return OCC_XC_OK;
}

int occ_xc_profile_enable(occ_xc_context *ctx, int on) {
  if (!ctx)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->impl->prof.on = on != 0;
  return OCC_XC_OK;
}

int occ_xc_profile_reset(occ_xc_context *ctx) {
  if (!ctx)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    ctx->impl->prof.collect();
    ctx->impl->prof.totals.clear();
  });
}

int occ_xc_profile_count(occ_xc_context *ctx) {
  if (!ctx)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  int rc = guarded(ctx, [&] { ctx->impl->prof.collect(); });
  return rc == OCC_XC_OK ? static_cast<int>(ctx->impl->prof.totals.size()) : rc;
}

int occ_xc_profile_entry(occ_xc_context *ctx, int i, const char **name, double *total_ms,
                         long *launches) {
  if (!ctx || !name || !total_ms || !launches)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  auto &t = ctx->impl->prof.totals;
  if (i < 0 || i >= static_cast<int>(t.size()))
    return OCC_XC_ERR_ARG;
  *name = t[i].name.c_str();
  *total_ms = t[i].ms;
  *launches = t[i].launches;
  return OCC_XC_OK;
}

long occ_xc_launch_count(const occ_xc_context *ctx) { return ctx ? ctx->impl->launches : -1; }

} // extern "C"
