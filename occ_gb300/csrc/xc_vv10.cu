// VV10 non-local correlation on the device (FP64, or FP32 pair sums): OCC's
// NonLocalCorrelationFunctional (src/dft/nonlocal_correlation.cpp), the
// energy and potential that DFT::post_scf_nlc_correction
// (include/occ/dft/dft.h:476-483) adds for the "-V" methods.
//
// The functional lives on its own coarse grid (set_integration_grid,
// nonlocal_correlation.cpp:17-31: GridSettings{110, 50, 50, 1e-7, false},
// whose fifth initialiser lands in int_acc, so the H/He grid stays reduced),
// built here as a second molecule over the same basis (the Becke partition
// on the GPU), with near-dense screening (1e-14) where OCC evaluates every
// AO at every point.  Per build:
//   k_colloc_f64, k_rho_f64   rho, grad rho on that grid (Morton order)
//   k_vv10_prep               per point, in the grid's own order: position,
//                             omega0 = sqrt(C (|grad rho|^2 / rho^2)^2 +
//                             4 pi rho / 3), kappa = b 3 pi / 2 (9 pi)^(-1/6)
//                             rho^(1/6), rho w
//   k_vv10_pairs              for every point i, the sums over partners
//                             j < i (the reference's loop, :68-92, taken in
//                             the same order)
//                               t = 2 rho_j w_j / (g_i g_j (g_i + g_j)),
//                               g = r^2 omega0 + kappa,
//                             F_i = -1.5 (rho_i w_i / (2 k^3) + sum t),
//                             U_i, W_i as the reference accumulates them;
//                             tiles of 128 points staged in shared memory,
//                             the longest rows of the triangle first;
//                             OCC_XC_MIXED: k_vv10_pairs32, the same sums in
//                             FP32 (double-float coordinate differences,
//                             one approximate reciprocal, Kahan sums flushed
//                             to FP64 per tile), the triangle spread over
//                             CTAs of 16 partner tiles each
//   k_vv10_final              exc, vrho, vsigma (:97-108), E partials, and
//                             the V coefficients 0.5 vrho, 2 vsigma grad rho
//   k_vxc_f64                 V = k + k^T (:373-386), the build's own kernel
#include <algorithm>
#include <vector>

#include "xc_device.cuh"
#include "xc_engine.hpp"
#include "xc_leaf_func.cuh"

namespace occx {

namespace {

constexpr int kVvTile = 128;
constexpr double kVvRhoMin = 1e-8; // nonlocal_correlation.cpp:73, 80

struct VvPoint {
  double x, y, z, om; // position, omega0
  double kap, rw2, rho, active; // kappa, 2 rho w, rho, 1 if rho >= 1e-8
};

struct VvConst {
  double b, C, kappa_factor, beta;
};

// The mixed-precision pair kernel's point: coordinates as (hi, lo) float
// pairs, so that a difference of two is as accurate as FP32 allows however
// far the points are from the origin; omega0, kappa and 2 rho w in FP32.
struct VvPoint32 {
  float xh, xl, yh, yl, zh, zl, om, kap, rw2, active;
};

// Per sorted point s (original index perm[s]): the kernel's inputs in the
// grid's own order.
__global__ void k_vv10_prep(MolDev m, VvConst K, const int *__restrict__ perm,
                            const double *__restrict__ rho, VvPoint *__restrict__ pts) {
  const long s = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= m.npts)
    return;
  const size_t N = static_cast<size_t>(m.npts);
  const Pt4 P = m.pts[s];
  const double r = rho[s];
  const double gx = rho[N + s], gy = rho[2 * N + s], gz = rho[3 * N + s];
  const double sig = gx * gx + gy * gy + gz * gz;
  double t = sig / (r * r);
  t = K.C * t * t;
  VvPoint q;
  q.x = P.x;
  q.y = P.y;
  q.z = P.z;
  q.om = sqrt(t + (4.0 * 3.14159265358979323846 / 3.0) * r);
  q.kap = K.kappa_factor * pow(r, 1.0 / 6.0);
  q.rw2 = 2.0 * r * P.w;
  q.rho = r;
  q.active = r >= kVvRhoMin ? 1.0 : 0.0;
  pts[perm[s]] = q;
}

__device__ __forceinline__ void f32_pair(double v, float &h, float &l) {
  h = static_cast<float>(v);
  l = static_cast<float>(v - static_cast<double>(h));
}

__global__ void k_vv10_prep32(long n, const VvPoint *__restrict__ p,
                              VvPoint32 *__restrict__ q) {
  const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const VvPoint P = p[i];
  VvPoint32 Q;
  f32_pair(P.x, Q.xh, Q.xl);
  f32_pair(P.y, Q.yh, Q.yl);
  f32_pair(P.z, Q.zh, Q.zl);
  // a point below the density cut takes part as an exact zero (finite
  // omega0 and kappa, no weight), so that the pair loop needs no branch
  const bool act = P.active != 0.0;
  Q.om = act ? static_cast<float>(P.om) : 1.0f;
  Q.kap = act ? static_cast<float>(P.kap) : 1.0f;
  Q.rw2 = act ? static_cast<float>(P.rw2) : 0.0f;
  Q.active = act ? 1.0f : 0.0f;
  q[i] = Q;
}

// s + c += v (Kahan); the _rn intrinsics keep the compensation from being
// contracted or reassociated
__device__ __forceinline__ void kahan(float &s, float &c, float v) {
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Tile b (of 128 points i) against tiles 0..b (partners j < i).  Blocks run
// the longest rows first.
__global__ void __launch_bounds__(kVvTile)
    k_vv10_pairs(long n, const VvPoint *__restrict__ pts, double *__restrict__ FUW) {
  __shared__ double sx[kVvTile], sy[kVvTile], sz[kVvTile], som[kVvTile], skap[kVvTile],
      srw[kVvTile], sact[kVvTile];
  const long ntiles = (n + kVvTile - 1) / kVvTile;
  const long b = ntiles - 1 - blockIdx.x;
  const long i = b * kVvTile + threadIdx.x;
  const bool iv = i < n;
  VvPoint P{};
  if (iv)
    P = pts[i];
  const bool act = iv && P.active != 0.0;
  double f = 0.0, u = 0.0, w = 0.0;
  if (act) {
    const double k = P.kap;
    f = 0.5 * P.rw2 / (2 * k * k * k);
    u = f * (1.0 / k + 1.0 / (2 * k));
  }
  for (long jt = 0; jt <= b; jt++) {
    const long j0 = jt * kVvTile;
    const long jl = j0 + threadIdx.x;
    if (jl < n) {
      const VvPoint Q = pts[jl];
      sx[threadIdx.x] = Q.x;
      sy[threadIdx.x] = Q.y;
      sz[threadIdx.x] = Q.z;
      som[threadIdx.x] = Q.om;
      skap[threadIdx.x] = Q.kap;
      srw[threadIdx.x] = Q.rw2;
      sact[threadIdx.x] = Q.active;
    } else {
      sact[threadIdx.x] = 0.0;
    }
    __syncthreads();
    if (act) {
      const int jmax = (jt == b) ? static_cast<int>(threadIdx.x) : kVvTile;
      for (int jj = 0; jj < jmax; jj++) {
        if (sact[jj] == 0.0)
          continue;
        const double dx = P.x - sx[jj], dy = P.y - sy[jj], dz = P.z - sz[jj];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double gi = r2 * P.om + P.kap;
        const double gj = r2 * som[jj] + skap[jj];
        const double s = gi + gj;
        const double inv = 1.0 / (gi * gj * s);
        double t = srw[jj] * inv;
        f += t;
        t *= (s + gi) * gj * inv; // 1/g_i + 1/(g_i + g_j)
        u += t;
        w = fma(t, r2, w);
      }
    }
    __syncthreads();
  }
  if (iv) {
    FUW[3 * i] = act ? -1.5 * f : 0.0;
    FUW[3 * i + 1] = act ? u : 0.0;
    FUW[3 * i + 2] = act ? w : 0.0;
  }
}

// The pair sums alone (no self term) in FP32.  Block (x, y): rows of tile
// b = ntiles - 1 - x against partner tiles [16 y, 16 y + 15] (clipped to
// b), so that the triangle spreads over many CTAs; two Kahan-compensated
// accumulator sets per thread (even and odd partners), flushed to FP64 per
// partner tile, and one FP64 atomic add per row and sum at the end (FUW
// zeroed before).
constexpr int kVvChunk = 16; // partner tiles per CTA

// 1/x to about one ulp in one instruction (the pair sums' other roundings
// are of the same size)
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void vv_pair32(const VvPoint32 &P, const VvPoint32 &Q, float &fs,
                                          float &fc, float &us, float &uc, float &ws, float &wc) {
  const float dx = __fadd_rn(__fsub_rn(P.xh, Q.xh), __fsub_rn(P.xl, Q.xl));
  const float dy = __fadd_rn(__fsub_rn(P.yh, Q.yh), __fsub_rn(P.yl, Q.yl));
  const float dz = __fadd_rn(__fsub_rn(P.zh, Q.zh), __fsub_rn(P.zl, Q.zl));
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float gi = fmaf(r2, P.om, P.kap);
  const float gj = fmaf(r2, Q.om, Q.kap);
  const float sg = gi + gj;
  const float inv = rcp_approx(gi * gj * sg);
  const float t = Q.rw2 * inv;
  kahan(fs, fc, t);
  const float t2 = t * ((sg + gi) * gj * inv); // t (1/g_i + 1/(g_i + g_j))
  kahan(us, uc, t2);
  kahan(ws, wc, t2 * r2);
}

__global__ void __launch_bounds__(kVvTile)
    k_vv10_pairs32(long n, const VvPoint32 *__restrict__ pts, double *__restrict__ FUW) {
  __shared__ VvPoint32 sp[kVvTile];
  const long ntiles = (n + kVvTile - 1) / kVvTile;
  const long b = ntiles - 1 - blockIdx.x;
  const long jt0 = static_cast<long>(blockIdx.y) * kVvChunk;
  if (jt0 > b)
    return; // the whole CTA: beyond this row tile's triangle
  const long jt1 = min(jt0 + kVvChunk - 1, b);
  const long i = b * kVvTile + threadIdx.x;
  const bool iv = i < n;
  VvPoint32 P{};
  if (iv)
    P = pts[i];
  const bool act = iv && P.active != 0.0f;
  double F = 0.0, U = 0.0, W = 0.0;
  for (long jt = jt0; jt <= jt1; jt++) {
    const long jl = jt * kVvTile + threadIdx.x;
    if (jl < n) {
      sp[threadIdx.x] = pts[jl];
    } else {
      VvPoint32 z{};
      z.om = z.kap = 1.0f;
      sp[threadIdx.x] = z;
    }
    __syncthreads();
    if (act) {
      float a[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, c[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      const int jmax = (jt == b) ? static_cast<int>(threadIdx.x) : kVvTile;
      int jj = 0;
      for (; jj + 1 < jmax; jj += 2) {
        vv_pair32(P, sp[jj], a[0], a[1], a[2], a[3], a[4], a[5]);
        vv_pair32(P, sp[jj + 1], c[0], c[1], c[2], c[3], c[4], c[5]);
      }
      if (jj < jmax)
        vv_pair32(P, sp[jj], a[0], a[1], a[2], a[3], a[4], a[5]);
      F += (static_cast<double>(a[0]) - a[1]) + (static_cast<double>(c[0]) - c[1]);
      U += (static_cast<double>(a[2]) - a[3]) + (static_cast<double>(c[2]) - c[3]);
      W += (static_cast<double>(a[4]) - a[5]) + (static_cast<double>(c[4]) - c[5]);
    }
    __syncthreads();
  }
  if (act) {
    atomicAdd(&FUW[3 * i], F);
    atomicAdd(&FUW[3 * i + 1], U);
    atomicAdd(&FUW[3 * i + 2], W);
  }
}

// pair_only: FUW holds the pair sums alone; the self term (rho w / (2 k^3)
// in f, f (1/k + 1/(2k)) in u) and the -1.5 are applied here.
__global__ void __launch_bounds__(256)
    k_vv10_final(MolDev m, VvConst K, const int *__restrict__ perm,
                 const double *__restrict__ rho, const double *__restrict__ FUW, bool pair_only,
                 double *__restrict__ coef, double *__restrict__ epart) {
  __shared__ double sh[8];
  const long s = static_cast<long>(blockIdx.x) * 256 + threadIdx.x;
  const size_t N = static_cast<size_t>(m.npts);
  double e = 0.0;
  if (s < m.npts) {
    const double r = rho[s];
    const double gx = rho[N + s], gy = rho[2 * N + s], gz = rho[3 * N + s];
    const double sig = gx * gx + gy * gy + gz * gz;
    const double w = m.pts[s].w;
    double t = sig / (r * r);
    t = K.C * t * t;
    const double pi4_3 = 4.0 * 3.14159265358979323846 / 3.0;
    const double om = sqrt(t + pi4_3 * r);
    const double dom_r = (0.5 * pi4_3 * r - 2.0 * t) / om;
    const double dom_g = t * r / (sig * om);
    const double dkap = K.kappa_factor * pow(r, 1.0 / 6.0) / 6.0;
    const int o = perm[s];
    double F = FUW[3 * o], U = FUW[3 * o + 1], W = FUW[3 * o + 2];
    if (pair_only) {
      if (r >= kVvRhoMin) {
        const double k = K.kappa_factor * pow(r, 1.0 / 6.0);
        const double fself = r * w / (2 * k * k * k);
        F = -1.5 * (fself + F);
        U = fself * (1.0 / k + 1.0 / (2 * k)) + U;
      } else {
        F = U = W = 0.0;
      }
    }
    const double exc = (K.beta + 0.5 * F) * w;
    const double vr = (K.beta + F + 1.5 * (U * dkap + W * dom_r)) * w;
    const double vs = (1.5 * W * dom_g) * w;
    e = exc * r;
    coef[s] = 0.5 * vr;
    coef[N + s] = 2.0 * vs * gx;
    coef[2 * N + s] = 2.0 * vs * gy;
    coef[3 * N + s] = 2.0 * vs * gz;
  }
  e = leaf_sum256(e, sh);
  if (threadIdx.x == 0)
    epart[blockIdx.x] = e;
}

__global__ void __launch_bounds__(256) k_vv10_sum(const double *__restrict__ epart, int n,
                                                  double *__restrict__ out) {
  __shared__ double sh[8];
  double e = 0.0;
  for (int i = threadIdx.x; i < n; i += 256)
    e += epart[i];
  e = leaf_sum256(e, sh);
  if (threadIdx.x == 0)
    out[0] = e;
}

} // namespace

// OCC's NLC grid settings (nonlocal_correlation.h:35-37 as compiled).
static GridSettings nlc_grid_settings() {
  GridSettings g;
  g.max_angular_points = 110;
  g.min_angular_points = 50;
  g.radial_points = 50;
  g.radial_precision = 1e-7;
  return g;
}

void Molecule::prepare_nlc() {
  if (nlc)
    return;
  if (!d_pts)
    throw ArgError("the molecule has no device state");
  auto N = std::make_unique<Molecule>();
  N->ctx = ctx;
  N->device = device;
  N->Z = Z;
  N->xyz = xyz;
  N->basis = basis;
  N->fs = fs;
  N->deriv = 1;
  N->gs = nlc_grid_settings();
  N->bs = bs;
  N->bs.xc_screening_threshold = 1e-14;
  PartitionFn part;
  if (device_partition_fits(device, static_cast<int>(Z.size())))
    part = [dev = device](const PartitionInput &in, double *w) { device_partition(dev, in, w); };
  N->grid = build_molecular_grid(N->Z, N->xyz, N->basis, N->gs, 0, part ? &part : nullptr);
  N->build_plan();
  N->upload();
  const size_t n = static_cast<size_t>(std::max<long>(N->plan.npts, 1));
  std::vector<int> perm(n, 0);
  for (long s = 0; s < N->plan.npts; s++)
    perm[s] = static_cast<int>(N->plan.perm[s]);
  size_t bytes = 0;
  N->d_nlc_perm = dev_upload(perm, bytes);
  N->allocations.push_back(N->d_nlc_perm);
  N->device_bytes += static_cast<double>(bytes);
  N->d_nlc_pts = N->alloc(n * sizeof(VvPoint));
  N->d_nlc_pts32 = N->alloc(n * sizeof(VvPoint32));
  N->d_nlc_fuw = static_cast<double *>(N->alloc(3 * n * sizeof(double)));
  N->d_nlc_epart = static_cast<double *>(N->alloc(((n + 255) / 256) * sizeof(double)));
  nlc = std::move(N);
}

void Molecule::nlc_vv10(const double *dD, double b, double C, int precision, double *dV,
                        double *dE, cudaStream_t st) {
  prepare_nlc();
  Molecule &N = *nlc;
  N.ensure_fp64_ws();
  const MolDev m = N.dev();
  const double pi = 3.14159265358979323846;
  VvConst K{b, C, b * 1.5 * pi * std::pow(9.0 * pi, -1.0 / 6.0),
            std::pow(3.0 / (b * b), 0.75) / 32.0};
  Context &c = *ctx;
  const long n = N.plan.npts;
  const int blocks = static_cast<int>((n + 255) / 256);
  if (!N.fp64_ao_valid)
    c.launch("colloc_f64", st, [&] { launch_colloc_f64(m, 1, N.d_ws, st); });
  N.fp64_ao_valid = true;
  c.launch("rho_f64", st, [&] {
    launch_rho_f64(m, 1, dD, N.d_ws, N.d_slabs, static_cast<int>(N.slabs.size()), N.d_rho, st);
  });
  c.launch("vv10_prep", st, [&] {
    k_vv10_prep<<<blocks, 256, 0, st>>>(m, K, N.d_nlc_perm, N.d_rho,
                                        static_cast<VvPoint *>(N.d_nlc_pts));
  });
  const int tiles = static_cast<int>((n + kVvTile - 1) / kVvTile);
  const bool mixed = precision == OCC_XC_MIXED;
  if (mixed) {
    c.launch("vv10_prep32", st, [&] {
      k_vv10_prep32<<<blocks, 256, 0, st>>>(n, static_cast<const VvPoint *>(N.d_nlc_pts),
                                            static_cast<VvPoint32 *>(N.d_nlc_pts32));
    });
    cuda_check(cudaMemsetAsync(N.d_nlc_fuw, 0, 3 * static_cast<size_t>(std::max<long>(n, 1)) *
                                                  sizeof(double), st),
               "cudaMemsetAsync");
    c.launch("vv10_pairs32", st, [&] {
      if (tiles > 0)
        k_vv10_pairs32<<<dim3(tiles, (tiles + kVvChunk - 1) / kVvChunk), kVvTile, 0, st>>>(
            n, static_cast<const VvPoint32 *>(N.d_nlc_pts32), N.d_nlc_fuw);
    });
  } else {
    c.launch("vv10_pairs", st, [&] {
      if (tiles > 0)
        k_vv10_pairs<<<tiles, kVvTile, 0, st>>>(n, static_cast<const VvPoint *>(N.d_nlc_pts),
                                                N.d_nlc_fuw);
    });
  }
  c.launch("vv10_final", st, [&] {
    k_vv10_final<<<blocks, 256, 0, st>>>(m, K, N.d_nlc_perm, N.d_rho, N.d_nlc_fuw, mixed,
                                         N.d_coef, N.d_nlc_epart);
  });
  c.launch("reduce", st, [&] { k_vv10_sum<<<1, 256, 0, st>>>(N.d_nlc_epart, blocks, dE); });
  if (dV) {
    const size_t nbf2 = static_cast<size_t>(basis.nbf) * basis.nbf;
    cuda_check(cudaMemsetAsync(dV, 0, nbf2 * sizeof(double), st), "cudaMemsetAsync");
    c.launch("vxc_f64", st, [&] {
      launch_vxc_f64(m, 1, N.d_ws, N.d_coef, N.d_tiles, static_cast<int>(N.tiles.size()), dV, st);
    });
  }
  cuda_check(cudaGetLastError(), "kernel launch");
}

} // namespace occx

using namespace occx;

extern "C" {

int occ_xc_nlc_vv10(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D, double b,
                    double C, int precision, double *energy, double *V) {
  if (!ctx || !mol || !D || !energy || !(b > 0.0) || !(C >= 0.0))
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
    M.nlc_vv10(M.d_D, b, C, precision, V ? M.d_V : nullptr, M.d_out2, st);
    if (V)
      cuda_check(cudaMemcpyAsync(V, M.d_V, nbf2 * sizeof(double), cudaMemcpyDeviceToHost, st),
                 "cudaMemcpyAsync D2H");
    double e = 0.0;
    cuda_check(cudaMemcpyAsync(&e, M.d_out2, sizeof(double), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    *energy = e;
  });
}

int occ_xc_nlc_grid_points(const occ_xc_molecule *mol, long *npoints) {
  if (!mol || !npoints)
    return OCC_XC_ERR_ARG;
  const Molecule &M = *mol->impl;
  *npoints = M.nlc ? M.nlc->grid.npts() : -1;
  return OCC_XC_OK;
}

int occ_xc_nlc_grid(const occ_xc_molecule *mol, double *points, double *weights) {
  if (!mol || !points || !weights)
    return OCC_XC_ERR_ARG;
  const Molecule &M = *mol->impl;
  if (!M.nlc)
    return OCC_XC_ERR_ARG;
  std::copy(M.nlc->grid.xyz.begin(), M.nlc->grid.xyz.end(), points);
  std::copy(M.nlc->grid.w.begin(), M.nlc->grid.w.end(), weights);
  return OCC_XC_OK;
}

} // extern "C"
