// Engine internals shared by the C ABI and the precision-specific build paths.
#pragma once
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

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
FuncSet parse_method(const std::string &method);
void upload_sph_table_mixed();
struct MixedState;
void free_mixed(MixedState *S);
struct Molecule;
// 1 if a bounded wait in the mixed-precision kernels gave up (synchronises st)
int mixed_error_flag(Molecule &M, cudaStream_t st);

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

struct MixedState; // device state of the mixed-precision path (xc_mixed.cu)

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
  int deriv = 0;
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

  ~Molecule();
  void *alloc(size_t bytes);
  void build_plan();
  void upload();
  void prepare_mixed();
  MolDev dev() const;
  void build(int precision, const double *dD, double *dV, double *dout2, cudaStream_t st);
  void build_fp64(const double *dD, double *dV, double *dout2, cudaStream_t st);
  void build_mixed(const double *dD, double *dV, double *dout2, cudaStream_t st);
};

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
