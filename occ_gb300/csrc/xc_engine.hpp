// Engine internals shared by the C ABI and the precision-specific build paths.
#pragma once
#include <algorithm>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda.h>

#include "../../include/occ_xc.h"
#include "host/xc_host.hpp"
#include "xc_device.cuh"

namespace occx {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct MethodError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct ArgError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct TimeoutError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void cuda_check(cudaError_t e, const char *what);

// Makes `device` current for the lifetime of the guard and puts the caller's
// current device back on every exit path.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int device) {
    cuda_check(cudaGetDevice(&prev), "cudaGetDevice");
    if (prev != device)
      cuda_check(cudaSetDevice(device), "cudaSetDevice");
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
      cudaSetDevice(prev);
  }
};

// cudaMalloc of max(size, 1) elements and a copy of h; adds the bytes to `bytes`.
template <typename T> T *dev_upload(const std::vector<T> &h, size_t &bytes) {
  T *d = nullptr;
  size_t n = std::max<size_t>(h.size(), 1);
  cuda_check(cudaMalloc(&d, n * sizeof(T)), "cudaMalloc");
  if (!h.empty())
    cuda_check(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice),
               "cudaMemcpy H2D");
  bytes += n * sizeof(T);
  return d;
}
void fill_sph_table(double *out);
void upload_sph_table_grad();
// Components of the FP64 path's per-point density array (rho, grad rho and,
// for a meta-GGA, the three tau sums) and of its V_xc coefficient array.
inline int rho_components(int deriv) { return deriv == 2 ? 7 : deriv ? 4 : 1; }
inline int coef_components(int deriv) { return deriv == 2 ? 5 : deriv ? 4 : 1; }
// Entry points that have no meta-GGA form throw ArgError for one.
void require_not_mgga(int deriv, const char *what);
// the unrestricted build's polarised functional stage and its sums (xc_uks.cu)
// (mixed: the tensor-core build's evaluators, FP32 derivatives)
void launch_func_pol(const MolDev &m, int deriv, const FuncSet &fs, double thr,
                     const double *rho_a, const double *rho_b, double *coef_a, double *coef_b,
                     double *epart3, cudaStream_t st, bool mixed = false);
void launch_reduce3(const double *epart3, int n, double *out3, cudaStream_t st);
// Becke partition weights on `device` (xc_grid.cu); fits: the kernel's
// shared memory holds natom atoms.
bool device_partition_fits(int device, int natom);
void device_partition(int device, const PartitionInput &in, double *w);
// The build plan (Morton order, leaves, screening) on the GPU (xc_plan.cu);
// the same plan as host/plan.cpp's morton_leaves + screen_leaves.
void device_plan(int device, const MolecularGrid &grid, const Basis &basis,
                 const BuildSettings &bs, Plan &plan);
FuncSet parse_method(const std::string &method);
// occ_xc_grid_settings -> GridSettings (defaults for NULL)
GridSettings grid_settings_from(const occ_xc_grid_settings *grid);
void upload_sph_table_mixed();
struct MixedState;
void free_mixed(MixedState *S);
struct Molecule;
// 1 if a bounded wait in the mixed-precision kernels gave up (synchronises st)
int mixed_error_flag(Molecule &M, cudaStream_t st);
void set_wait_limit(int device, uint32_t polls);

// Per-kernel device timing with CUDA events on the launching stream, the
// device analogue of OCC's timing categories (include/occ/core/timings.h).
// Off by default; when on, every kernel launch of a build is bracketed.
struct KernelProfiler {
  struct Rec {
    const char *name;
    cudaEvent_t a, b;
  };
  struct Total {
    std::string name;
    double ms = 0.0;
    long launches = 0;
  };
  bool on = false;
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  std::vector<Total> totals;
  cudaEvent_t get();
  void begin(const char *name, cudaStream_t st);
  void end(cudaStream_t st);
  void collect();
  ~KernelProfiler();
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  KernelProfiler prof;
  long launches = 0; // kernels launched by the library on this context
  int max_ctas = 0;  // CTAs of the persistent tensor-core kernels (0: one per SM)
  explicit Context(int dev);
  ~Context();
  // bracket one kernel launch (profiling) and count it
  template <typename F> void launch(const char *name, cudaStream_t st, F &&f) {
    if (prof.on)
      prof.begin(name, st);
    f();
    if (prof.on)
      prof.end(st);
    launches++;
  }
};

// Tensor maps of a workspace region as rows of 128 FP32: boxes of 32 points
// x 32 rows and of 32 points x 128 rows (one copy for a whole 128-row tile).
struct WsMaps {
  CUtensorMap rows32, rows128;
};
struct MixedState; // device state of the mixed-precision path (xc_mixed.cu)
struct GradMixed;  // the tensor-core XC gradient's workspace and plan (xc_mixed.cu)
void free_grad_mixed(GradMixed *g);
struct MetaMixed;  // the tensor-core meta-GGA build's workspace and plan (xc_mixed.cu)
void free_meta_mixed(MetaMixed *g);

// Default cap of the XC gradient's workspace per leaf group (bytes).
constexpr size_t kGradWsCapDefault = size_t(8) << 30;

// The molecule arguments of occ_xc_molecule_create.
struct MoleculeArgs {
  int natoms;
  const int *Z;
  const double *xyz;
  int nshells;
  const int *shell_l, *shell_atom, *shell_nprim;
  const double *exponents, *coefficients;
  int pure;
  const char *method;
  const occ_xc_grid_settings *grid;
  const occ_xc_build_settings *build;
};

struct Molecule {
  Context *ctx = nullptr;
  int device = 0;
  // host model
  std::vector<int> Z;
  std::vector<double> xyz;
  Basis basis;
  GridSettings gs;
  BuildSettings bs;
  FuncSet fs{};
  int deriv = 0; // OCC's density_derivative(): 0 LDA, 1 GGA, 2 meta-GGA
  int vxc_n = 256; // tuning: N of the mixed path's V_xc tile
  int ctas = 0;    // tuning: CTAs of its persistent kernels (0: the context's setting)
  long atom_batch = 0; // > 0: leaves are batches of this many points per atom block in
                       // grid order (atom_batch_leaves), not Morton leaves
  MolecularGrid grid;
  Plan plan;
  // device plan
  std::vector<DevLeaf> leaves;
  std::vector<int> leaf_sh, leaf_ao;
  std::vector<SlabItem> slabs;
  std::vector<TileItem> tiles;
  size_t ws_elems = 0;
  double flops = 0.0;
  double device_bytes = 0.0;
  std::vector<void *> allocations;
  Pt4 *d_pts = nullptr;
  DevShell *d_shells = nullptr;
  double2 *d_prims = nullptr;
  DevLeaf *d_leaves = nullptr;
  int *d_leaf_sh = nullptr, *d_leaf_ao = nullptr;
  SlabItem *d_slabs = nullptr;
  TileItem *d_tiles = nullptr;
  double *d_ws = nullptr, *d_rho = nullptr, *d_coef = nullptr, *d_epart = nullptr;
  double *d_out2 = nullptr, *d_D = nullptr, *d_V = nullptr;
  MixedState *mixed = nullptr;
  bool fp64_ao_valid = false; // d_ws holds this molecule's AO values (no collocation)
  // XC nuclear gradient: leaves with 4 (LDA) or 10 (GGA) AO planes, grouped
  // under a workspace cap; allocated on the molecule's first gradient
  struct GradGroup {
    int leaf0, nleaf, slab0, nslab;
  };
  std::vector<GradGroup> ggroups;
  DevLeaf *d_gleaves = nullptr;
  SlabItem *d_gslabs = nullptr;
  int *d_ao_atom = nullptr;
  double *d_gws = nullptr, *d_grad = nullptr;
  size_t grad_ws_cap_bytes = kGradWsCapDefault;
  // unrestricted (UKS) build: beta density and coefficients, per-spin D / V
  // blocks, OCC-layout D / V of the host entry point (first UKS build)
  double *d_rho_b = nullptr, *d_coef_b = nullptr, *d_epart_u = nullptr, *d_Dab = nullptr,
         *d_Vab = nullptr, *d_Duks = nullptr, *d_Vuks = nullptr, *d_out3 = nullptr;
  // VV10: the molecule on OCC's NLC grid (first VV10 call) and, on that
  // molecule, its sorted -> grid-order map and the pair kernel's buffers
  std::unique_ptr<Molecule> nlc;
  GradMixed *gmixed = nullptr;
  MetaMixed *mmixed = nullptr;
  int *d_nlc_perm = nullptr;
  void *d_nlc_pts = nullptr, *d_nlc_pts32 = nullptr;
  double *d_nlc_fuw = nullptr, *d_nlc_epart = nullptr;
  double grad_bytes = 0.0; // device bytes of the gradient's state

  ~Molecule();
  void *alloc(size_t bytes);
  void build_plan();
  void upload();
  void prepare_mixed();
  void materialise();    // upload() + prepare_mixed(): the resident device state
  void release_device(); // frees all device state (back to the host-only molecule)
  double estimate_resident_bytes() const; // what materialise() allocates (upper bound)
  // Per-build workspaces.  A molecule built on its own allocates a private
  // one per precision on first use; batches and the server lend it a region
  // of a shared one instead.
  size_t fp64_workspace_bytes() const;
  size_t mixed_workspace_bytes() const;
  void ensure_fp64_ws();
  void ensure_mixed_ws();
  void prepare(int precision); // the private workspace of `precision` (before a capture)
  MolDev dev() const;
  void build(int precision, const double *dD, double *dV, double *dout2, cudaStream_t st);
  // ws: an FP64 workspace of fp64_workspace_bytes() (nullptr: the private one);
  // ws_holds_ao: ws already holds this molecule's AO values
  void build_fp64(const double *dD, double *dV, double *dout2, cudaStream_t st,
                  double *ws = nullptr, bool ws_holds_ao = false);
  void build_mixed(const double *dD, double *dV, double *dout2, cudaStream_t st);
  // the meta-GGA build with its tau contractions on the tensor cores
  void prepare_mgga_mixed();
  void build_mixed_mgga(const double *dD, double *dV, double *dout2, cudaStream_t st);
  void prepare_gradient();
  void prepare_uks();
  void prepare_gradient_mixed();
  // the same gradient with the contractions on the tensor cores (3xTF32)
  void xc_gradient_mixed(const double *dD, double *dgrad, double *dout2, cudaStream_t st);
  void xc_gradient_mixed_mgga(const double *dD, double *dgrad, double *dout2, cudaStream_t st);
  void xc_gradient_uks_mixed_mgga(const double *dD, double *dgrad, double *dout3, cudaStream_t st);
  void grad_tables(GradMixed &g);
  void prepare_nlc();
  // VV10 energy (dE, one double) and, if dV, its V (nbf x nbf) for mo.D = dD;
  // precision OCC_XC_FP64 or OCC_XC_MIXED (FP32 pair sums)
  void nlc_vv10(const double *dD, double b, double C, int precision, double *dV, double *dE,
                cudaStream_t st);
  // UKS build (FP64): dD, dV 2 nbf x nbf in OCC's layout; dout3 = {E_xc,
  // integrated rho_a, integrated rho_b}
  void build_fp64_uks(const double *dD, double *dV, double *dout3, cudaStream_t st);
  // the same with the density and potential contractions on the tensor cores
  void build_mixed_uks(const double *dD, double *dV, double *dout3, cudaStream_t st);
  void *d_uks_tabs = nullptr; // the mixed plan's table with the beta rho / coef arrays
  void *d_uks_tabs_meta = nullptr; // the same for the meta-GGA plan
  void build_mixed_uks_mgga(const double *dD, double *dV, double *dout3, cudaStream_t st);
  void release_gradient(); // frees the gradient's device state
  // dE_xc/dR (3 per atom, grid fixed) for mo.D = dD; dout2 = {E_xc, density}
  void xc_gradient(const double *dD, double *dgrad, double *dout2, cudaStream_t st);
  // the same for OCC's unrestricted mo.D (2 nbf x nbf); dout3 = {E_xc, rho_a, rho_b}
  void xc_gradient_uks(const double *dD, double *dgrad, double *dout3, cudaStream_t st);
  // ... with the contractions on the tensor cores (LDA / GGA)
  void xc_gradient_uks_mixed(const double *dD, double *dgrad, double *dout3, cudaStream_t st);
};

// Host part of a molecule: basis, molecular grid, Morton leaves and screening
// (no device memory); materialise() uploads it.
std::unique_ptr<Molecule> molecule_host(Context *ctx, const MoleculeArgs &a);
void check_build_settings(const BuildSettings &b);
// New leaves and screening under `b` (the grid is kept); device state is
// rebuilt if the molecule had any.
void replan(Molecule &M, const BuildSettings &b);

// Staging for launch lists built per call (the server's batched builds):
// one device region and one pinned host region, grown on demand.
struct ListArena {
  void *d = nullptr, *h = nullptr;
  size_t cap = 0;
  void reserve(size_t bytes);
  ~ListArena();
};
// One mixed-precision build of each molecule in `mols` (each at most once)
// through shared launches, reading and writing the molecules' own D, V and
// {E_xc, density} buffers, with their workspaces laid out one after the
// other from d_ws.  Lists go through `arena`; *d_err is the
// bounded-wait flag.  Asynchronous on st; the arena may be reused once st has
// passed this call.
void mixed_build_group(Context &c, const std::vector<Molecule *> &mols, ListArena &arena,
                       char *d_ws, int *d_err, cudaStream_t st);
// Bytes of the shared workspace mixed_build_group needs for `mols` (d_ws).
size_t group_workspace_bytes(const std::vector<Molecule *> &mols);
// The same over workspaces that persist in a pool (the server's sessions):
// ws[i] is molecule i's region (mixed_workspace_bytes, 512-byte aligned from
// pool), ao_valid[i] says it already holds the molecule's AO values, and
// pool_map is encode_ws_map of the whole pool.
void mixed_build_in_pool(Context &c, const std::vector<Molecule *> &mols,
                         const std::vector<char *> &ws, const std::vector<int> &ao_valid,
                         const char *pool, const WsMaps &pool_map, ListArena &arena,
                         int *d_err, cudaStream_t st);
void encode_ws_map(WsMaps &map, const void *base, size_t bytes);

} // namespace occx

// The opaque handles of include/occ_xc.h.
struct occ_xc_context {
  std::unique_ptr<occx::Context> impl;
  std::string err;
  std::mutex mu;
};
struct occ_xc_molecule {
  std::unique_ptr<occx::Molecule> impl;
  occ_xc_context *ctx;
};

namespace occx {
// Runs f, mapping the engine's exceptions to OCC_XC_ERR_* codes with the
// message kept in the context.
template <typename F> int guarded(occ_xc_context *ctx, F &&f) {
  try {
    f();
    return OCC_XC_OK;
  } catch (const MethodError &e) {
    if (ctx)
      ctx->err = e.what();
    return OCC_XC_ERR_METHOD;
  } catch (const CudaError &e) {
    if (ctx)
      ctx->err = e.what();
    return OCC_XC_ERR_CUDA;
  } catch (const ArgError &e) {
    if (ctx)
      ctx->err = e.what();
    return OCC_XC_ERR_ARG;
  } catch (const TimeoutError &e) {
    if (ctx)
      ctx->err = e.what();
    return OCC_XC_ERR_TIMEOUT;
  } catch (const std::bad_alloc &) {
    if (ctx)
      ctx->err = "host allocation failed";
    return OCC_XC_ERR_NOMEM;
  } catch (const std::exception &e) {
    if (ctx)
      ctx->err = e.what();
    return OCC_XC_ERR_INTERNAL;
  }
}
} // namespace occx
