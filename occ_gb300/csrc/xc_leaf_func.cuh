// The functional stage of one Morton leaf, shared by the FP64 and the mixed
// paths: include/occ/dft/dft.h:339-352 with src/dft/dft_kernels.cpp:27-70.
// One CTA per leaf (256 threads, or NT); a leaf may hold any number of
// points (threads stride over them).  The leaf is skipped when max rho < thr
// (dft_kernels.cpp:37-40); coefficients are those of the V_xc contraction
// (src/dft/xc_potential_matrix.cpp:19-41): coef0 = 0.5 w vrho and, for a GGA,
// coef1..3 = 2 w vsigma grad rho.  epart2 receives {sum w e_xc rho, sum w rho}.
#pragma once
#include "functionals.cuh"
#include "functionals_mgga.cuh"
#include "xc_device.cuh"

namespace occx {

// Sum / maximum over the NT threads of the CTA (sh: NT / 32 doubles).
template <int NT = 256> __device__ __forceinline__ double leaf_sum256(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < NT / 32; i++)
    s += sh[i];
  __syncthreads();
  return s;
}

template <int NT = 256> __device__ __forceinline__ double leaf_max256(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = sh[0];
  for (int i = 1; i < NT / 32; i++)
    s = fmax(s, sh[i]);
  __syncthreads();
  return s;
}

// MIXED: the mixed path's evaluator (double-float values, FP32 derivatives).
// NT: threads of the CTA (they stride over the leaf's points).
template <bool DERIV, bool MIXED = false, int NT = 256>
__device__ __forceinline__ void leaf_functional(const DevLeaf &L, const Pt4 *__restrict__ pts,
                                                size_t N, const FuncSet &fs, double thr,
                                                const double *__restrict__ rho,
                                                double *__restrict__ coef, double *epart2,
                                                double *sh) {
  double mx = -1e300;
  for (int p = threadIdx.x; p < L.cnt; p += NT)
    mx = fmax(mx, rho[static_cast<size_t>(L.off) + p]);
  mx = leaf_max256<NT>(mx, sh);
  const bool skip = mx < thr;
  double nel = 0.0, ew = 0.0;
  for (int p = threadIdx.x; p < L.cnt; p += NT) {
    const size_t idx = static_cast<size_t>(L.off) + p;
    const double r = rho[idx];
    const double w = pts[idx].w;
    nel += w * r;
    double gx = 0, gy = 0, gz = 0, sigma = 0;
    if (DERIV) {
      gx = rho[N + idx];
      gy = rho[2 * N + idx];
      gz = rho[3 * N + idx];
      sigma = gx * gx + gy * gy + gz * gz;
    }
    double e = 0, vr = 0, vs = 0;
    if (!skip) {
      if (MIXED)
        eval_xc_mixed(fs, r, sigma, e, vr, vs);
      else
        eval_xc(fs, r, sigma, e, vr, vs);
    }
    coef[idx] = 0.5 * w * vr;
    if (DERIV) {
      const double f = 2.0 * w * vs;
      coef[N + idx] = f * gx;
      coef[2 * N + idx] = f * gy;
      coef[3 * N + idx] = f * gz;
    }
    ew += w * e;
  }
  nel = leaf_sum256<NT>(nel, sh);
  ew = leaf_sum256<NT>(ew, sh);
  if (threadIdx.x == 0) {
    epart2[0] = ew;
    epart2[1] = nel;
  }
}

// The meta-GGA functional stage (MIXED: FP32 derivatives, eval_xc_mgga_mixed): rho components 0-3 as for a GGA and
// 4-6 the three (d_k phi) D2 (d_k phi) sums, tau = half their sum
// (src/gto/density.cpp:86-100, include/occ/dft/dft_kernels.h:49-58).
// Coefficients 0-3 as for a GGA and coef4 = 0.25 w vtau (the V kernel's
// K + K^T then carries src/dft/xc_potential_matrix.cpp:43-58's 0.5 w vtau).
template <bool MIXED = false>
__device__ __forceinline__ void leaf_functional_mgga(const DevLeaf &L,
                                                     const Pt4 *__restrict__ pts, size_t N,
                                                     const FuncSet &fs, double thr,
                                                     const double *__restrict__ rho,
                                                     double *__restrict__ coef, double *epart2,
                                                     double *sh) {
  double mx = -1e300;
  for (int p = threadIdx.x; p < L.cnt; p += 256)
    mx = fmax(mx, rho[static_cast<size_t>(L.off) + p]);
  mx = leaf_max256(mx, sh);
  const bool skip = mx < thr;
  double nel = 0.0, ew = 0.0;
  for (int p = threadIdx.x; p < L.cnt; p += 256) {
    const size_t idx = static_cast<size_t>(L.off) + p;
    const double r = rho[idx];
    const double w = pts[idx].w;
    nel += w * r;
    const double gx = rho[N + idx], gy = rho[2 * N + idx], gz = rho[3 * N + idx];
    const double sigma = gx * gx + gy * gy + gz * gz;
    const double tau = 0.5 * (rho[4 * N + idx] + rho[5 * N + idx] + rho[6 * N + idx]);
    double e = 0, vr = 0, vs = 0, vt = 0;
    if (!skip) {
      if (MIXED)
        eval_xc_mgga_mixed(fs, r, sigma, tau, e, vr, vs, vt);
      else
        eval_xc_mgga(fs, r, sigma, tau, e, vr, vs, vt);
    }
    coef[idx] = 0.5 * w * vr;
    const double f = 2.0 * w * vs;
    coef[N + idx] = f * gx;
    coef[2 * N + idx] = f * gy;
    coef[3 * N + idx] = f * gz;
    coef[4 * N + idx] = 0.25 * w * vt;
    ew += w * e;
  }
  nel = leaf_sum256(nel, sh);
  ew = leaf_sum256(ew, sh);
  if (threadIdx.x == 0) {
    epart2[0] = ew;
    epart2[1] = nel;
  }
}

} // namespace occx
