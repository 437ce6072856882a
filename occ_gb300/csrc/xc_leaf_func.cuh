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

// The barrier of the NT threads that run a leaf's functional: the whole CTA
// (BAR = 0), or named barrier BAR shared by threads 0 .. NT - 1 only.
template <int NT, int BAR> __device__ __forceinline__ void leaf_bar() {
  if constexpr (BAR == 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"n"(BAR), "n"(NT) : "memory");
}

// Sum / maximum over the NT threads 0 .. NT - 1 (sh: NT / 32 doubles).
template <int NT = 256, int BAR = 0>
__device__ __forceinline__ double leaf_sum256(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  leaf_bar<NT, BAR>();
  double s = 0.0;
  for (int i = 0; i < NT / 32; i++)
    s += sh[i];
  leaf_bar<NT, BAR>();
  return s;
}

template <int NT = 256, int BAR = 0>
__device__ __forceinline__ double leaf_max256(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  leaf_bar<NT, BAR>();
  double s = sh[0];
  for (int i = 1; i < NT / 32; i++)
    s = fmax(s, sh[i]);
  leaf_bar<NT, BAR>();
  return s;
}

// MIXED: the mixed path's evaluator (double-float values, FP32 derivatives).
// NT: threads 0 .. NT - 1 stride over the leaf's points; BAR: their barrier
// (leaf_bar).
template <bool DERIV, bool MIXED = false, int NT = 256, int BAR = 0>
__device__ __forceinline__ void leaf_functional(const DevLeaf &L, const Pt4 *__restrict__ pts,
                                                size_t N, const FuncSet &fs, double thr,
                                                const double *__restrict__ rho,
                                                double *__restrict__ coef, double *epart2,
                                                double *sh) {
  double mx = -1e300;
  for (int p = threadIdx.x; p < L.cnt; p += NT)
    mx = fmax(mx, rho[static_cast<size_t>(L.off) + p]);
  mx = leaf_max256<NT, BAR>(mx, sh);
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
  nel = leaf_sum256<NT, BAR>(nel, sh);
  ew = leaf_sum256<NT, BAR>(ew, sh);
  if (threadIdx.x == 0) {
    epart2[0] = ew;
    epart2[1] = nel;
  }
}

// Sum over threads 0 .. NT - 1 of a double-float (sh: NT / 32 float2).
template <int NT, int BAR>
__device__ __forceinline__ fn::F2 leaf_sum_f2(fn::F2 v, float2 *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const fn::F2 w{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
    v = fn::f2_add(v, w);
  }
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = make_float2(v.h, v.l);
  leaf_bar<NT, BAR>();
  fn::F2 s{0.f, 0.f};
  for (int i = 0; i < NT / 32; i++)
    s = fn::f2_add(s, fn::F2{sh[i].x, sh[i].y});
  leaf_bar<NT, BAR>();
  return s;
}

// Maximum over threads 0 .. NT - 1 of FP64 bit patterns as signed integers:
// the maximum of the values when any is non-negative, and a negative value
// when all are (sh: NT / 32 long longs).
template <int NT, int BAR>
__device__ __forceinline__ long long leaf_max_bits(long long v, long long *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  leaf_bar<NT, BAR>();
  long long s = sh[0];
  for (int i = 1; i < NT / 32; i++)
    s = max(s, sh[i]);
  leaf_bar<NT, BAR>();
  return s;
}

// The tensor-core build's functional stage in double-float arithmetic, with
// no FP64 operation per point but VWN's atan and B88's asinh where
// rho >= 1e-10 and sigma >= 1e-30 (the
// FP64 inputs are split by integer operations, fn::f2_bits;
// eval_xc_mixed_f2; the FP64 evaluator elsewhere): the skip, weights and
// coefficients of leaf_functional<.., MIXED>, the coefficients as FP32
// handed to store(p, c) for p < npad (zero past the leaf's points), E and
// the electron count summed in double-float and written as FP64 partials.
// sh: NT / 32 eight-byte words.
template <bool DERIV, int NT, int BAR, class Store>
__device__ __forceinline__ void leaf_functional_f2(const DevLeaf &L, const Pt4 *__restrict__ pts,
                                                   size_t N, const FuncSet &fs, double thr,
                                                   const double *__restrict__ rho, Store store,
                                                   int npad, double *epart2, double *sh) {
  long long mb = -0x7fffffffffffffffLL - 1;
  for (int p = threadIdx.x; p < L.cnt; p += NT)
    mb = max(mb, __double_as_longlong(rho[static_cast<size_t>(L.off) + p]));
  mb = leaf_max_bits<NT, BAR>(mb, reinterpret_cast<long long *>(sh));
  const bool skip = __longlong_as_double(mb) < thr;
  fn::F2 nel{0.f, 0.f}, ew{0.f, 0.f};
  for (int p = threadIdx.x; p < npad; p += NT) {
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p < L.cnt) {
      const size_t idx = static_cast<size_t>(L.off) + p;
      const fn::F2 r = fn::f2_bits(rho[idx]);
      const fn::F2 w = fn::f2_bits(pts[idx].w);
      nel = fn::f2_add(nel, fn::f2_mul(w, r));
      fn::F2 gx{0.f, 0.f}, gy{0.f, 0.f}, gz{0.f, 0.f}, sigma{0.f, 0.f};
      if (DERIV) {
        gx = fn::f2_bits(rho[N + idx]);
        gy = fn::f2_bits(rho[2 * N + idx]);
        gz = fn::f2_bits(rho[3 * N + idx]);
        sigma = fn::f2_add(fn::f2_add(fn::f2_mul(gx, gx), fn::f2_mul(gy, gy)), fn::f2_mul(gz, gz));
      }
      if (!skip) {
        fn::F2 e;
        float vr, vs;
        if (!eval_xc_mixed_f2(fs, DERIV, r, sigma, e, vr, vs)) {
          // low density or gradient: FP64 on the FP64 inputs
          double sd = 0.0, ed, vrd, vsd;
          if (DERIV) {
            const double dx = rho[N + idx], dy = rho[2 * N + idx], dz = rho[3 * N + idx];
            sd = dx * dx + dy * dy + dz * dz;
          }
          eval_xc(fs, rho[idx], sd, ed, vrd, vsd);
          e = fn::f2(ed);
          vr = static_cast<float>(vrd);
          vs = static_cast<float>(vsd);
        }
        c.x = 0.5f * w.h * vr;
        if (DERIV) {
          const float f = 2.f * w.h * vs;
          c.y = f * gx.h;
          c.z = f * gy.h;
          c.w = f * gz.h;
        }
        ew = fn::f2_add(ew, fn::f2_mul(w, e));
      }
    }
    store(p, c);
  }
  float2 *shf = reinterpret_cast<float2 *>(sh);
  nel = leaf_sum_f2<NT, BAR>(nel, shf);
  ew = leaf_sum_f2<NT, BAR>(ew, shf);
  if (threadIdx.x == 0) {
    epart2[0] = fn::to_d(ew);
    epart2[1] = fn::to_d(nel);
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
