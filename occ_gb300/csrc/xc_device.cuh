// Device-side data layout of the XC build and the kernel launchers.
//
// HBM layout per molecule (resident across SCF iterations):
//   pts    Pt4[npts]     Morton-sorted x, y, z, w
//   shells DevShell[nsh]     centre, l, primitive range, AO count, common_fac
//   prims  double2[nprim]    (exponent, normalised coefficient)
//   leaves DevLeaf[nleaves]  point range, significant-shell range, local AO
//                            count m and its padded sizes, workspace offset
//   leaf_sh int[]            significant shells per leaf, ascending
//   leaf_ao int[]            local -> global AO index per leaf
// Per build (workspace, reusable):
//   phi    [comp][mpad][npad] per leaf, FP64 (plain) or FP32 pairs (mixed)
//   rho    [4][npts]          rho, d/dx, d/dy, d/dz at sorted points
//   coef   [4][npts]          0.5 w vrho and 2 w vsigma grad(rho)
//   epart  [nleaves]          per-leaf E_xc and electron-count partials
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "functionals.cuh"

namespace occx {

struct alignas(32) Pt4 {
  double x, y, z, w;
};
__host__ __device__ inline Pt4 make_pt4(double x, double y, double z, double w) {
  return Pt4{x, y, z, w};
}

struct DevShell {
  double A[3];
  double fac;
  int l, nprim, prim_off, nfunc;
};

struct DevLeaf {
  int off, cnt;           // sorted point range
  int sh_begin, sh_end;   // into leaf_sh
  int ao_begin, nbf;      // into leaf_ao; m = nbf
  int mpad, npad;         // AO rows padded to the AO tile, points to the point tile
  long long ws_off;       // workspace offset (elements) of this leaf's phi block
};

// Work items of the contraction kernels.
struct SlabItem {
  int leaf, p0;
};
struct TileItem {
  int leaf, i0, j0, pad;
};

constexpr int kAoTile = 64;   // AO tile of the FP64 contractions
constexpr int kPtTile = 64;   // point tile (rows) of the FP64 density contraction
constexpr int kKChunk = 16;   // reduction chunk staged through shared memory

struct MolDev {
  const Pt4 *pts;
  const DevShell *shells;
  const double2 *prims;
  const DevLeaf *leaves;
  const int *leaf_sh;
  const int *leaf_ao;
  int nleaves, npts, nbf, pure;
};

void upload_sph_table();

// FP64 plain path
void launch_colloc_f64(const MolDev &m, int deriv, double *ws, cudaStream_t st);
void launch_rho_f64(const MolDev &m, int deriv, const double *D, const double *ws,
                    const SlabItem *slabs, int nslabs, double *rho, cudaStream_t st);
// meta-GGA: the three (d_k phi) D2 (d_k phi) sums into rho components 4-6
void launch_tau_f64(const MolDev &m, const double *D, const double *ws, const SlabItem *slabs,
                    int nslabs, double *rho, cudaStream_t st);
void launch_func(const MolDev &m, int deriv, const FuncSet &fs, double dens_thr, const double *rho,
                 double *coef, double *epart, cudaStream_t st);
void launch_vxc_f64(const MolDev &m, int deriv, const double *ws, const double *coef,
                    const TileItem *tiles, int ntiles, double *V, cudaStream_t st);
void launch_reduce(const double *epart, int nleaves, double *out2, cudaStream_t st);

} // namespace occx
