// An FP64 XC build that allocates nothing, for callers that cannot allocate
// device memory.
//
// Who needs it: code embedded in a host application that owns all of the
// GPU's memory through its own pool (a cudaMalloc there fails, or carves
// memory out of the pool behind the host's back), and code that runs where
// an allocation is not allowed at all, such as a latency-bound loop that
// must never block in the allocator.  Such a caller creates its molecules
// once, at set-up, and then calls occ_xc_compute_vxc_noalloc with its own
// input and output buffers.
//
// The build is the FP64 kernel sequence of Molecule::build_fp64, but its
// scratch (AO values, densities, functional coefficients, per-leaf energy
// partials) lives in one file-scope __device__ array of kNoAllocScratchBytes
// instead of the molecule's own workspace:
//  - every GPU on which the entry point has run holds that array until the
//    process exits.  Under CUDA's lazy module loading (the default) the
//    module that holds the array loads, and its 64 MiB are taken, on the
//    first call on a device, when the host looks up the array's address: a
//    caller whose pool takes the GPU's memory makes that first call at
//    set-up, before the pool grows;
//  - the host obtains the array's device address with cudaGetSymbolAddress,
//    once per device, with that device current (the call makes the
//    context's device current and restores the caller's device before it
//    returns), the first time the entry point runs on that device; make that
//    first call before any stream capture;
//  - every call shares the array: calls whose work overlaps on the GPU race
//    on it and give wrong results, so a caller serialises them (one stream,
//    or events between streams);
//  - the array keeps the previous call's contents; every scratch word a call
//    reads it has first written in the same call, and V, the only buffer
//    accumulated with atomics, is the caller's output and is cleared by the
//    call itself.
#include <cstring>
#include <mutex>

#include "../../include/occ_xc.h"
#include "xc_engine.hpp"

namespace occx {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20; // 64 MiB
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchBytes / sizeof(double)];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double *g_scratch_ptr[kMaxDevices] = {};

// Device address of the static scratch on `device` (which must be current).
double *noalloc_scratch(int device) {
  if (device < 0 || device >= kMaxDevices)
    throw ArgError("device ordinal out of range for the static scratch table");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[device]) {
    void *p = nullptr;
    cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
    g_scratch_ptr[device] = static_cast<double *>(p);
  }
  return g_scratch_ptr[device];
}

size_t align_elems(size_t n) { return (n + 31) / 32 * 32; } // 256-byte boundaries

} // namespace
} // namespace occx

using namespace occx;

extern "C" int occ_xc_compute_vxc_noalloc(occ_xc_context *ctx, occ_xc_molecule *mol,
                                          const double *d_D, double *d_V, double *d_exc2,
                                          void *stream) {
  if (!ctx || !mol || !d_D || !d_V || !d_exc2)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  try {
    if (mol->ctx != ctx) {
      ctx->err = "occ_xc_compute_vxc_noalloc: the molecule was created on another context";
      return OCC_XC_ERR_ARG;
    }
    Context &c = *ctx->impl;
    Molecule &M = *mol->impl;
    const size_t N = static_cast<size_t>(M.plan.npts);
    const size_t nl = M.leaves.size();
    const size_t nrho = rho_components(M.deriv) * N, ncoef = coef_components(M.deriv) * N;
    const size_t need = align_elems(M.ws_elems) + align_elems(nrho) + align_elems(ncoef) +
                        align_elems(2 * nl);
    if (need * sizeof(double) > kNoAllocScratchBytes) {
      ctx->err = "occ_xc_compute_vxc_noalloc: this molecule needs " +
                 std::to_string(need * sizeof(double)) +
                 " bytes of scratch, more than the static maximum of " +
                 std::to_string(kNoAllocScratchBytes) + " bytes; use occ_xc_compute_vxc_device";
      return OCC_XC_ERR_ARG;
    }
    DeviceGuard on_device(c.device);
    double *ws = noalloc_scratch(c.device);
    double *rho = ws + align_elems(M.ws_elems);
    double *coef = rho + align_elems(nrho);
    double *epart = coef + align_elems(ncoef);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c.stream;
    const MolDev m = M.dev();
    const size_t nbf2 = static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
    cuda_check(cudaMemsetAsync(d_V, 0, nbf2 * sizeof(double), st), "cudaMemsetAsync");
    // the launches of Molecule::build_fp64, counted and profiled the same way
    const int nslabs = static_cast<int>(M.slabs.size()), ntiles = static_cast<int>(M.tiles.size());
    c.launch("colloc_f64", st, [&] { launch_colloc_f64(m, M.deriv, ws, st); });
    c.launch("rho_f64", st,
             [&] { launch_rho_f64(m, M.deriv, d_D, ws, M.d_slabs, nslabs, rho, st); });
    if (M.deriv == 2)
      c.launch("tau_f64", st, [&] { launch_tau_f64(m, d_D, ws, M.d_slabs, nslabs, rho, st); });
    c.launch("func", st, [&] {
      launch_func(m, M.deriv, M.fs, M.bs.density_threshold, rho, coef, epart, st);
    });
    c.launch("vxc_f64", st,
             [&] { launch_vxc_f64(m, M.deriv, ws, coef, M.d_tiles, ntiles, d_V, st); });
    c.launch("reduce", st, [&] { launch_reduce(epart, m.nleaves, d_exc2, st); });
    cuda_check(cudaGetLastError(), "kernel launch");
    return OCC_XC_OK;
  } catch (const CudaError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_CUDA;
  } catch (const std::exception &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_ARG;
  }
}
