// Autotuner of a molecule's build: Morton leaf size, the V_xc tensor-core tile
// and the persistent CTA count, chosen by timing real builds of the molecule
// on the device.
//
// OCC fixes its leaves at 128 points (min 32, max 256,
// include/occ/numint/spatial_grid_hierarchy.h:26-30) for a CPU cache; on the
// GPU the best size depends on the basis and the geometry (larger leaves
// give fewer, wider blocks and fewer V_xc atomics, smaller ones fewer
// screened-in AOs per point).  The search is coordinate-wise: leaf target
// over {64, 128, 256, 512} with OCC's min/max ratios, then the tile N over
// {128, 256}, then the CTA count over {SMs, SMs / 2}.  A leaf size changes
// which shells pass the per-leaf screening, so a candidate is kept only if
// its E_xc stays within tol_exc of the build at OCC's defaults.  Results are
// cached per molecule fingerprint in the text file named by
// OCC_XC_TUNE_CACHE (if set), so later runs apply them without timing.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "xc_engine.hpp"

namespace occx {
namespace {

struct Candidate {
  BuildSettings bs;
  int vxc_n = 256;
  int ctas = 0;
};

std::string fingerprint(const Molecule &M, int precision) {
  // geometry, basis size, grid size and method: enough to tell molecules apart
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    h ^= v;
    h *= 1099511628211ull;
  };
  for (int z : M.Z)
    mix(static_cast<uint64_t>(z));
  for (double x : M.xyz)
    mix(static_cast<uint64_t>(std::llround(x * 1e6)));
  mix(static_cast<uint64_t>(M.basis.nbf));
  mix(static_cast<uint64_t>(M.grid.npts()));
  for (int i = 0; i < M.fs.n; i++) {
    mix(static_cast<uint64_t>(M.fs.id[i]));
    mix(static_cast<uint64_t>(std::llround(M.fs.coef[i] * 1e9)));
  }
  std::ostringstream os;
  os << std::hex << h << "-p" << precision;
  return os.str();
}

bool cache_lookup(const std::string &key, Candidate &c) {
  const char *path = std::getenv("OCC_XC_TUNE_CACHE");
  if (!path)
    return false;
  std::ifstream f(path);
  std::string k;
  Candidate r;
  bool found = false;
  while (f >> k >> r.bs.leaf_target >> r.bs.leaf_min >> r.bs.leaf_max >> r.vxc_n >> r.ctas) {
    if (k == key) {
      c.bs.leaf_target = r.bs.leaf_target;
      c.bs.leaf_min = r.bs.leaf_min;
      c.bs.leaf_max = r.bs.leaf_max;
      c.vxc_n = r.vxc_n;
      c.ctas = r.ctas;
      found = true; // the last entry for a key wins
    }
  }
  return found;
}

void cache_store(const std::string &key, const Candidate &c) {
  const char *path = std::getenv("OCC_XC_TUNE_CACHE");
  if (!path)
    return;
  std::ofstream f(path, std::ios::app);
  f << key << ' ' << c.bs.leaf_target << ' ' << c.bs.leaf_min << ' ' << c.bs.leaf_max << ' '
    << c.vxc_n << ' ' << c.ctas << '\n';
}

void apply(Molecule &M, const Candidate &c) {
  const bool tile = c.vxc_n != M.vxc_n;
  M.vxc_n = c.vxc_n;
  M.ctas = c.ctas;
  if (c.bs.leaf_target != M.bs.leaf_target || c.bs.leaf_min != M.bs.leaf_min ||
      c.bs.leaf_max != M.bs.leaf_max) {
    replan(M, c.bs); // rebuilds the device state with the new tile too
  } else if (tile && !M.allocations.empty()) {
    // the tile lives in the molecule's table and its single-build plan
    M.release_device();
    M.materialise();
  }
}

// Mean ms per build over `reps` builds after `warm` untimed ones; E_xc out.
double time_builds(Molecule &M, int precision, cudaStream_t st, int warm, int reps,
                   double *exc) {
  M.prepare(precision);
  for (int i = 0; i < warm; i++)
    M.build(precision, M.d_D, M.d_V, M.d_out2, st);
  cudaEvent_t a, b;
  cuda_check(cudaEventCreate(&a), "cudaEventCreate");
  cuda_check(cudaEventCreate(&b), "cudaEventCreate");
  cuda_check(cudaEventRecord(a, st), "cudaEventRecord");
  for (int i = 0; i < reps; i++)
    M.build(precision, M.d_D, M.d_V, M.d_out2, st);
  cuda_check(cudaEventRecord(b, st), "cudaEventRecord");
  double out2[2];
  cuda_check(cudaMemcpyAsync(out2, M.d_out2, sizeof(out2), cudaMemcpyDeviceToHost, st), "D2H");
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  float ms = 0.f;
  cuda_check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (precision == OCC_XC_MIXED && mixed_error_flag(M, st))
    throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
  *exc = out2[0];
  return ms / reps;
}

} // namespace
} // namespace occx

using namespace occx;

extern "C" int occ_xc_molecule_set_build_settings(occ_xc_context *ctx, occ_xc_molecule *mol,
                                                  const occ_xc_build_settings *b) {
  if (!ctx || !mol || !b)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  try {
    cuda_check(cudaSetDevice(ctx->impl->device), "cudaSetDevice");
    BuildSettings s;
    s.xc_screening_threshold = b->xc_screening_threshold;
    s.density_threshold = b->density_threshold;
    s.leaf_target = b->leaf_target;
    s.leaf_min = b->leaf_min;
    s.leaf_max = b->leaf_max;
    replan(*mol->impl, s);
    return OCC_XC_OK;
  } catch (const ArgError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_ARG;
  } catch (const CudaError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_CUDA;
  } catch (const std::exception &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_INTERNAL;
  }
}

extern "C" int occ_xc_molecule_autotune(occ_xc_context *ctx, occ_xc_molecule *mol,
                                        int precision, const double *D, double tol_exc,
                                        int apply_best, occ_xc_tune_result *out) {
  if (!ctx || !mol || !D || !out || (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  try {
    cuda_check(cudaSetDevice(ctx->impl->device), "cudaSetDevice");
    Molecule &M = *mol->impl;
    cudaStream_t st = ctx->impl->stream;
    const size_t n2 = static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
    const std::vector<double> Dh(D, D + n2);
    auto load_D = [&] {
      cuda_check(cudaMemcpyAsync(M.d_D, Dh.data(), n2 * sizeof(double), cudaMemcpyHostToDevice,
                                 st), "H2D");
    };
    Candidate orig;
    orig.bs = M.bs;
    orig.vxc_n = M.vxc_n;
    orig.ctas = M.ctas;
    const std::string key = fingerprint(M, precision);
    *out = occ_xc_tune_result{};
    Candidate best;
    if (cache_lookup(key, best)) {
      best.bs.xc_screening_threshold = M.bs.xc_screening_threshold;
      best.bs.density_threshold = M.bs.density_threshold;
      apply(M, apply_best ? best : orig);
      out->leaf_target = best.bs.leaf_target;
      out->leaf_min = best.bs.leaf_min;
      out->leaf_max = best.bs.leaf_max;
      out->vxc_tile_n = best.vxc_n;
      out->persistent_ctas = best.ctas;
      out->from_cache = 1;
      return OCC_XC_OK;
    }
    int sms = 0;
    cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->impl->device),
               "attribute");
    // reference point: OCC's default leaves, full tile, one CTA per SM
    Candidate def;
    def.bs = M.bs;
    def.bs.leaf_target = 128;
    def.bs.leaf_min = 32;
    def.bs.leaf_max = 256;
    def.vxc_n = 256;
    def.ctas = 0;
    int ncand = 0;
    double e_def = 0.0, max_de = 0.0;
    auto evaluate = [&](const Candidate &c, double *exc) {
      apply(M, c);
      load_D();
      ncand++;
      return time_builds(M, precision, st, 2, 5, exc);
    };
    double best_ms = evaluate(def, &e_def);
    best = def;
    out->default_ms_per_build = best_ms;
    auto consider = [&](const Candidate &c) {
      double e = 0.0;
      const double ms = evaluate(c, &e);
      const double de = std::fabs(e - e_def);
      if (de > tol_exc)
        return; // screening at this leaf size moves E_xc too far
      max_de = std::max(max_de, de);
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    };
    for (int target : {64, 256, 512}) {
      Candidate c = def;
      c.bs.leaf_target = target;
      c.bs.leaf_min = std::max(8, target / 4);
      c.bs.leaf_max = std::min(1024, 2 * target);
      consider(c);
    }
    if (precision == OCC_XC_MIXED) {
      Candidate c = best;
      c.vxc_n = 128;
      consider(c);
      c = best;
      c.ctas = std::max(1, sms / 2);
      consider(c);
    }
    cache_store(key, best);
    apply(M, apply_best ? best : orig);
    load_D();
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    out->leaf_target = best.bs.leaf_target;
    out->leaf_min = best.bs.leaf_min;
    out->leaf_max = best.bs.leaf_max;
    out->vxc_tile_n = best.vxc_n;
    out->persistent_ctas = best.ctas;
    out->ms_per_build = best_ms;
    out->max_dexc = max_de;
    out->candidates = ncand;
    out->from_cache = 0;
    return OCC_XC_OK;
  } catch (const TimeoutError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_TIMEOUT;
  } catch (const ArgError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_ARG;
  } catch (const CudaError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_CUDA;
  } catch (const std::exception &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_INTERNAL;
  }
}

extern "C" int occ_xc_molecule_apply_tuning(occ_xc_context *ctx, occ_xc_molecule *mol,
                                            const occ_xc_tune_result *t) {
  if (!ctx || !mol || !t || (t->vxc_tile_n != 64 && t->vxc_tile_n != 128 && t->vxc_tile_n != 256) ||
      t->persistent_ctas < 0)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  try {
    cuda_check(cudaSetDevice(ctx->impl->device), "cudaSetDevice");
    Molecule &M = *mol->impl;
    Candidate c;
    c.bs = M.bs;
    c.bs.leaf_target = t->leaf_target;
    c.bs.leaf_min = t->leaf_min;
    c.bs.leaf_max = t->leaf_max;
    c.vxc_n = t->vxc_tile_n;
    c.ctas = t->persistent_ctas;
    apply(M, c);
    return OCC_XC_OK;
  } catch (const ArgError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_ARG;
  } catch (const CudaError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_CUDA;
  } catch (const std::exception &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_INTERNAL;
  }
}
