// Seminumerical exchange (COSX, the ESP form) on the GPU: OCC's
// SemiNumericalExchange with set_use_esp(true)
// (src/qm/seminumerical_exchange.cpp:233-250 set-up, :517-529 restricted
// build, :714-855 the grid sweep), on the grid of GridSettings::for_sgx(n)
// (src/numint/grid_settings.cpp:59-68).
//
// Set-up (once per molecule and grid): a second molecule over the same basis
// on the exchange grid (for_sgx(n): n angular points on every shell, LMG
// radial precision 1e-5, no pruning, no reduced H / He grid), cut into the
// reference's batches (128 consecutive points of each atom block, in grid
// order), its AO values, the numerical overlap S_num = sum_g w_g phi phi^T
// (the FP64 V_xc kernel with coefficient w / 2), the analytic overlap S
// (McMurchie-Davidson, host) and the overlap projector Q = S_num^-1 S
// (Cholesky solve, host); the significant shell pairs p >= q (a shared
// origin or an overlap block of norm >= 1e-12) with their primitive-pair
// tables (exponent sum, centre, prefactor, Hermite expansion coefficients
// E^{ij}_t per axis) and the centre and extent of their most diffuse
// primitive pair.
//
// Per call, for mo.D:
//   k_cosx_d2q    D2q = Q (2 D), row-major
//   k_cosx_mask   shell pair (p, q) kept when max |D2q| over its two blocks
//                 reaches 1e-6 (the reference's density screen)
//   per group of batches (a workspace cap bounds F and G, both AO-major:
//   row lambda, one column per point of the group):
//   k_cosx_f      F[lambda, g] = w_g sum_sigma phi_sigma(g) D2q[sigma, lambda]
//   k_cosx_g      G[nu, g] -= sum_mu F[mu, g] V_g(mu, nu) (and the transposed
//                 block for p != q), V_g(mu, nu) = int phi_mu phi_nu / |r - g|
//                 by McMurchie-Davidson over the Boys function, one thread
//                 per grid point, the kept pairs that pass the batch's
//                 geometric screen (|P - c| - extent < radius + 1 Bohr) split
//                 into slices over the blocks of a batch
//   k_cosx_k      K'[mu, lambda] -= sum_g phi_mu(g) G[lambda, g]
//   k_cosx_sym    K = (K' + K'^T) / 4
// All in FP64, except under OCC_XC_MIXED the ESP integrals (E coefficients,
// Boys function, R_tuv), F and their contraction, in FP32; G is summed in
// FP64 either way.  Shells up to d.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/occ_xc.h"
#include "host/xc_host.hpp"
#include "xc_device.cuh"
#include "xc_engine.hpp"

namespace occx {
namespace {

constexpr int kCosxLmax = 2;                   // shells up to d
constexpr int kCosxNc = 6;                     // Cartesian components of a d shell
constexpr double kCosxDensityThreshold = 1e-6; // seminumerical_exchange.cpp:789
constexpr double kCosxMargin = 1.0;            // cosx::Settings::margin (Bohr)
constexpr int kCosxAoTile = 16;                // AOs lambda per block of the F and K kernels
constexpr int kCosxTargetBlocks = 152 * 32;    // G kernel: blocks to aim for (32 per SM)
constexpr int kCosxMaxSlices = 64;             // G kernel: most pair slices per leaf
constexpr double kCosxLogThreshold = 27.631021115928547; // -ln(1e-12): pair extents
constexpr double kCosxPairOverlap = 1e-12;     // IntegralEngine::compute_shellpairs
constexpr double kPi = 3.14159265358979323846;

// Cartesian powers of the components of a shell (CCA order), packed a | b<<4 | c<<8.
__constant__ int c_cx_comp[3][kCosxNc];
// Real solid-harmonic transforms (m = -l..l) of l = 0..2, T[f][i], and the
// identity for Cartesian shells.
__constant__ double c_cx_T[3][5][kCosxNc];
__constant__ float c_cx_Tf[3][5][kCosxNc]; // the same in FP32 (the mixed precision)
template <typename R> __device__ __forceinline__ R sph_t(int l, int f, int i);
template <> __device__ __forceinline__ double sph_t<double>(int l, int f, int i) {
  return c_cx_T[l][f][i];
}
template <> __device__ __forceinline__ float sph_t<float>(int l, int f, int i) {
  return c_cx_Tf[l][f][i];
}

struct CxPair {
  double Pc[3], ext;        // centre and extent of the most diffuse primitive pair
  int bf_p, bf_q, np, nq;   // first AO and AO count of each shell
  int la, lb, prim0, nprim; // angular momenta, primitive-pair range
};
struct CxPrim {
  double pexp, P[3], pref; // a + b, centre, c_a c_b 2 pi / p fac_a fac_b
  int e_off;               // E tables: 3 axes x (la+1)(lb+1)(la+lb+1)
  int pad;
};
// The same in FP32 for the mixed precision: the centre as an unevaluated sum
// hi + lo of two floats, so that P - C keeps the FP32 relative precision of
// the difference, not of the coordinates (GB300 runs FP64 at 1/64 of the FP32
// rate: the FP32 path does no FP64 arithmetic per primitive pair).
struct CxPrimF {
  float pexp, pref, Ph[3], Pl[3];
  int e_off, pad;
};
struct CxPtF {
  float h[3], l[3];
};

__device__ __forceinline__ void pc_diff(const CxPrim &Q, const Pt4 &C, double &x, double &y,
                                        double &z) {
  x = Q.P[0] - C.x;
  y = Q.P[1] - C.y;
  z = Q.P[2] - C.z;
}
__device__ __forceinline__ void pc_diff(const CxPrimF &Q, const CxPtF &C, float &x, float &y,
                                        float &z) {
  x = (Q.Ph[0] - C.h[0]) + (Q.Pl[0] - C.l[0]);
  y = (Q.Ph[1] - C.h[1]) + (Q.Pl[1] - C.l[1]);
  z = (Q.Ph[2] - C.h[2]) + (Q.Pl[2] - C.l[2]);
}
__device__ __forceinline__ Pt4 cx_point(const Pt4 &C, double) { return C; }
__device__ __forceinline__ CxPtF cx_point(const Pt4 &C, float) {
  CxPtF r;
  const double c[3] = {C.x, C.y, C.z};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    r.h[d] = static_cast<float>(c[d]);
    r.l[d] = static_cast<float>(c[d] - static_cast<double>(r.h[d]));
  }
  return r;
}
// FP32 to FP64 by integer operations (exact for normal numbers; zero and
// FP32 subnormals, below 1.2e-38, give a signed zero), off the FP64 pipe.
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned hi = e == 0 ? (u & 0x80000000u)
                             : (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  const unsigned lo = e == 0 ? 0u : u << 29;
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}
template <typename Rt> struct CxPrimOf { using type = CxPrim; };
template <> struct CxPrimOf<float> { using type = CxPrimF; };

// Index of R_tuv (t + u + v <= 4) in a packed array: by shell of degree s,
// then t descending, then u descending.
__host__ __device__ constexpr int r_index(int t, int u, int v) {
  return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 +
         ((u + v) * (u + v + 1)) / 2 + v;
}

// 1 / (2 i + 1), i = 0 .. kBoysTable - 1: the Boys series and recursions
// multiply by these instead of dividing (GB300's FP64 divisions are slow).
constexpr int kBoysTable = 64; // the series runs below T = 5: under 40 terms
__constant__ double c_inv_odd[kBoysTable];
__constant__ float c_inv_odd_f[kBoysTable];
template <typename R> __device__ __forceinline__ R inv_odd(int i);
template <> __device__ __forceinline__ double inv_odd<double>(int i) { return c_inv_odd[i]; }
template <> __device__ __forceinline__ float inv_odd<float>(int i) { return c_inv_odd_f[i]; }
__device__ __forceinline__ double r_exp(double x) { return exp(x); }
__device__ __forceinline__ float r_exp(float x) { return expf(x); }
__device__ __forceinline__ double r_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float r_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double r_erf(double x) { return erf(x); }
__device__ __forceinline__ float r_erf(float x) { return erff(x); }

// F_n(T), n = 0..NMAX: for T < 5 the series
// F_n(T) = e^-T sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)) at n = NMAX and
// downward recursion F_{n-1} = (2T F_n + e^-T) / (2n - 1); from there
// F_0 = (pi / T)^{1/2} erf(sqrt T) / 2 (erf(sqrt T) taken as 1 beyond T = 36
// in FP64 and T = 18 in FP32, where it is 1 to the working precision) and
// upward recursion F_{n+1} = ((2n+1) F_n - e^-T) / (2T), whose cancellation
// at T >= 5 up to F_4 stays within a few ulps; divisions by odd numbers through
// the reciprocal table.
// R: double (the FP64 path) or float (the mixed path; the series stops at
// 1e-8 of the sum).
template <typename R, int NMAX> __device__ __forceinline__ void boys_t(R T, R (&F)[NMAX + 1]) {
  static_assert(NMAX <= 4, "upward recursion from T = 5 is checked for n <= 4 (shells up to d)");
  const R et = r_exp(-T);
  const R t2 = R(2) * T;
  if (T < R(5)) {
    R term = inv_odd<R>(NMAX), sum = term;
    const R stop = sizeof(R) == 8 ? R(1e-17) : R(1e-8);
    for (int k = 1; k < kBoysTable - NMAX; k++) {
      term *= t2 * inv_odd<R>(NMAX + k);
      sum += term;
      if (term < stop * sum)
        break;
    }
    F[NMAX] = et * sum;
#pragma unroll
    for (int n = NMAX; n > 0; n--)
      F[n - 1] = (t2 * F[n] + et) * inv_odd<R>(n - 1);
  } else {
    F[0] = R(0.5) * r_sqrt(R(kPi) / T);
    if (T < (sizeof(R) == 8 ? R(36) : R(18)))
      F[0] *= r_erf(r_sqrt(T));
    const R it2 = R(1) / t2;
#pragma unroll
    for (int n = 0; n < NMAX; n++)
      F[n + 1] = (R(2 * n + 1) * F[n] - et) * it2;
  }
}

// R_tuv^(0), t + u + v <= L (compile time, all in registers), for exponent p
// and PC = P - C (McMurchie-Davidson recursion from R^(n)_000 = (-2p)^n F_n,
// level by level).
template <typename Rt, int L>
__device__ __forceinline__ void hermite_r_t(Rt p, Rt X, Rt Y, Rt Z,
                                            Rt (&R)[(L + 1) * (L + 2) * (L + 3) / 6]) {
  constexpr int NR = (L + 1) * (L + 2) * (L + 3) / 6;
  Rt F[L + 1];
  boys_t<Rt, L>(p * (X * X + Y * Y + Z * Z), F);
  Rt up[NR], cur[NR];
  Rt m2p[L + 1];
  m2p[0] = Rt(1);
#pragma unroll
  for (int n = 1; n <= L; n++)
    m2p[n] = m2p[n - 1] * (Rt(-2) * p);
#pragma unroll
  for (int n = L; n >= 0; n--) {
#pragma unroll
    for (int sdeg = 0; sdeg <= L - n; sdeg++)
#pragma unroll
      for (int t = sdeg; t >= 0; t--)
#pragma unroll
        for (int u = sdeg - t; u >= 0; u--) {
          const int v = sdeg - t - u;
          Rt val;
          if (sdeg == 0)
            val = m2p[n] * F[n];
          else if (t > 0)
            val = (t > 1 ? Rt(t - 1) * up[r_index(t > 1 ? t - 2 : 0, u, v)] : Rt(0)) +
                  X * up[r_index(t - 1, u, v)];
          else if (u > 0)
            val = (u > 1 ? Rt(u - 1) * up[r_index(t, u > 1 ? u - 2 : 0, v)] : Rt(0)) +
                  Y * up[r_index(t, u - 1, v)];
          else
            val = (v > 1 ? Rt(v - 1) * up[r_index(t, u, v > 1 ? v - 2 : 0)] : Rt(0)) +
                  Z * up[r_index(t, u, v - 1)];
          cur[r_index(t, u, v)] = val;
        }
#pragma unroll
    for (int i = 0; i < NR; i++)
      up[i] = cur[i];
  }
#pragma unroll
  for (int i = 0; i < NR; i++)
    R[i] = up[i];
}

// Cartesian power of component i (CCA order) of a shell of angular momentum
// l along axis (0 x, 1 y, 2 z).
__host__ __device__ constexpr int cca_pow(int l, int i, int axis) {
  int k = 0;
  for (int a = l; a >= 0; a--)
    for (int b = l - a; b >= 0; b--) {
      if (k == i)
        return axis == 0 ? a : (axis == 1 ? b : l - a - b);
      k++;
    }
  return 0;
}

// D2q = Q (2 D): Q, D column-major nbf x nbf; out row-major.  16 x 16 tiles.
__global__ void k_cosx_d2q(int nbf, const double *__restrict__ Q, const double *__restrict__ D,
                           size_t ldd, double *__restrict__ D2q) {
  __shared__ double Qs[16][17], Ds[16][17];
  const int lam = blockIdx.x * 16 + threadIdx.x, sig = blockIdx.y * 16 + threadIdx.y;
  double acc = 0.0;
  for (int k0 = 0; k0 < nbf; k0 += 16) {
    const int kq = k0 + threadIdx.x, kd = k0 + threadIdx.y;
    Qs[threadIdx.y][threadIdx.x] = (sig < nbf && kq < nbf) ? Q[static_cast<size_t>(kq) * nbf + sig] : 0.0;
    Ds[threadIdx.y][threadIdx.x] = (kd < nbf && lam < nbf) ? D[lam * ldd + kd] : 0.0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; k++)
      acc = fma(Qs[threadIdx.y][k], Ds[k][threadIdx.x], acc);
    __syncthreads();
  }
  if (sig < nbf && lam < nbf)
    D2q[static_cast<size_t>(sig) * nbf + lam] = 2.0 * acc;
}

__global__ void k_cosx_mask(int npairs, int nbf, const CxPair *__restrict__ pairs,
                            const double *__restrict__ D2q, int *__restrict__ mask) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npairs)
    return;
  const CxPair P = pairs[k];
  double mx = 0.0;
  for (int i = 0; i < P.np; i++)
    for (int j = 0; j < P.nq; j++) {
      mx = fmax(mx, fabs(D2q[static_cast<size_t>(P.bf_p + i) * nbf + P.bf_q + j]));
      mx = fmax(mx, fabs(D2q[static_cast<size_t>(P.bf_q + j) * nbf + P.bf_p + i]));
    }
  mask[k] = mx >= kCosxDensityThreshold ? 1 : 0;
}

// F[lambda, g] = w_g sum_sigma phi_sigma(g) D2q[sigma, lambda] for the
// points of leaf l0 + blockIdx.x (g counted from the group's first point off0,
// row stride ld) and the kCosxAoTile AOs lambda of blockIdx.y; a thread per
// point.
__global__ void __launch_bounds__(128) k_cosx_f(MolDev m, const double *__restrict__ ws, int l0,
                                                int off0, size_t ld,
                                                const double *__restrict__ D2q,
                                                double *__restrict__ F) {
  const DevLeaf L = m.leaves[l0 + blockIdx.x];
  const int lam0 = blockIdx.y * kCosxAoTile;
  const int nl = min(kCosxAoTile, m.nbf - lam0);
  const double *phi = ws + L.ws_off;
  const int *g = m.leaf_ao + L.ao_begin;
  const size_t nbf = static_cast<size_t>(m.nbf);
  for (int p = threadIdx.x; p < L.cnt; p += blockDim.x) {
    double acc[kCosxAoTile];
#pragma unroll
    for (int j = 0; j < kCosxAoTile; j++)
      acc[j] = 0.0;
    for (int s = 0; s < L.nbf; s++) {
      const double ph = phi[static_cast<size_t>(s) * L.npad + p];
      const double *d = D2q + static_cast<size_t>(g[s]) * nbf + lam0;
#pragma unroll
      for (int j = 0; j < kCosxAoTile; j++)
        if (j < nl)
          acc[j] = fma(ph, d[j], acc[j]);
    }
    const double w = m.pts[L.off + p].w;
    const size_t col = static_cast<size_t>(L.off - off0 + p);
#pragma unroll
    for (int j = 0; j < kCosxAoTile; j++)
      if (j < nl)
        F[(lam0 + j) * ld + col] = w * acc[j];
  }
}

// Double-float operands of the mixed precision's F and K: x = hi + lo, hi the
// FP32 rounding of x and lo that of the rest (about 48 significant bits).
__device__ __forceinline__ float2 split_hl(double x) {
  const float h = static_cast<float>(x);
  return make_float2(h, static_cast<float>(x - static_cast<double>(h)));
}
__global__ void k_cosx_split(size_t n, const double *__restrict__ x, float2 *__restrict__ y) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    y[i] = split_hl(x[i]);
}
// sh + sl += a b for double-float a and b in FP32 arithmetic (GB300's FP32
// rate is 64 times its FP64 rate): the product's rounding error (an FMA) and
// its cross terms, and the sum's rounding error (Knuth's TwoSum, rounded
// intrinsics so that nothing is contracted), go to sl.  Relative to the sum
// of |a b| the result holds about 1e-14.
__device__ __forceinline__ void df_fma(float2 a, float2 b, float &sh, float &sl) {
  const float p = __fmul_rn(a.x, b.x);
  const float e = fmaf(a.x, b.y, fmaf(a.y, b.x, fmaf(a.x, b.x, -p)));
  const float t = __fadd_rn(sh, p);
  const float v = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, v)), __fsub_rn(p, v));
  sl = __fadd_rn(sl, __fadd_rn(err, e));
  sh = t;
}

// k_cosx_f in the mixed precision: double-float phi (the workspace split into
// phi_hl) and D2q (D2q_hl), F stored in FP32.
__global__ void __launch_bounds__(128) k_cosx_f_df(MolDev m, const float2 *__restrict__ phi_hl,
                                                   int l0, int off0, size_t ld,
                                                   const float2 *__restrict__ D2q_hl,
                                                   float *__restrict__ F) {
  const DevLeaf L = m.leaves[l0 + blockIdx.x];
  const int lam0 = blockIdx.y * kCosxAoTile;
  const int nl = min(kCosxAoTile, m.nbf - lam0);
  const float2 *phi = phi_hl + L.ws_off;
  const int *g = m.leaf_ao + L.ao_begin;
  const size_t nbf = static_cast<size_t>(m.nbf);
  for (int p = threadIdx.x; p < L.cnt; p += blockDim.x) {
    float sh[kCosxAoTile], sl[kCosxAoTile];
#pragma unroll
    for (int j = 0; j < kCosxAoTile; j++)
      sh[j] = sl[j] = 0.f;
    for (int s = 0; s < L.nbf; s++) {
      const float2 a = phi[static_cast<size_t>(s) * L.npad + p];
      const float2 *d = D2q_hl + static_cast<size_t>(g[s]) * nbf + lam0;
#pragma unroll
      for (int j = 0; j < kCosxAoTile; j++)
        if (j < nl)
          df_fma(a, d[j], sh[j], sl[j]);
    }
    const float w = static_cast<float>(m.pts[L.off + p].w);
    const size_t col = static_cast<size_t>(L.off - off0 + p);
#pragma unroll
    for (int j = 0; j < kCosxAoTile; j++)
      if (j < nl)
        F[(lam0 + j) * ld + col] = w * (sh[j] + sl[j]);
  }
}

// One kept shell pair (angular momenta LA, LB at compile time, so that the
// Hermite integrals, the ESP block and the transforms stay in registers) at
// one point C: V_g(mu, nu) = sum over primitive pairs of pref sum_tuv
// E^x_t E^y_u E^z_v R_tuv, then G[:, q] -= F[:, p] V and, for p != q,
// G[:, p] -= F[:, q] V^T, through the shells' solid-harmonic transforms
// when pure.
template <typename Rt, int LA, int LB, typename Prim, typename Pt>
__device__ __forceinline__ void cosx_pair(const CxPair &P, const Prim *__restrict__ prims,
                                          const Rt *__restrict__ etab, const Pt &C, bool pure,
                                          const Rt *__restrict__ Fg, double *__restrict__ Gg,
                                          size_t ld) {
  constexpr int NCA = (LA + 1) * (LA + 2) / 2, NCB = (LB + 1) * (LB + 2) / 2;
  constexpr int L2 = LA + LB, NA = LA + 1, NB = LB + 1, NT = L2 + 1;
  constexpr int NR = (L2 + 1) * (L2 + 2) * (L2 + 3) / 6;
  Rt V[NCA][NCB];
#pragma unroll
  for (int i = 0; i < NCA; i++)
#pragma unroll
    for (int j = 0; j < NCB; j++)
      V[i][j] = Rt(0);
  for (int r = 0; r < P.nprim; r++) {
    const Prim Q = prims[P.prim0 + r];
    Rt R[NR], X, Y, Z;
    pc_diff(Q, C, X, Y, Z);
    hermite_r_t<Rt, L2>(Q.pexp, X, Y, Z, R);
    const Rt *Ex = etab + Q.e_off, *Ey = Ex + NA * NB * NT, *Ez = Ey + NA * NB * NT;
#pragma unroll
    for (int i = 0; i < NCA; i++) {
      const int ax = cca_pow(LA, i, 0), ay = cca_pow(LA, i, 1), az = cca_pow(LA, i, 2);
#pragma unroll
      for (int j = 0; j < NCB; j++) {
        const int bx = cca_pow(LB, j, 0), by = cca_pow(LB, j, 1), bz = cca_pow(LB, j, 2);
        const Rt *ex = Ex + (ax * NB + bx) * NT, *ey = Ey + (ay * NB + by) * NT,
                 *ez = Ez + (az * NB + bz) * NT;
        Rt acc = Rt(0);
        // compile-time trip counts (L2) with the exponent bounds as guards,
        // so that every R index is a constant and R stays in registers
#pragma unroll
        for (int t = 0; t <= L2; t++)
#pragma unroll
          for (int u = 0; u <= L2 - t; u++) {
            if (t > ax + bx || u > ay + by)
              continue;
            const Rt exy = ex[t] * ey[u];
#pragma unroll
            for (int v = 0; v <= L2 - t - u; v++)
              if (v <= az + bz)
                acc = fma(exy * ez[v], R[r_index(t, u, v)], acc);
          }
        V[i][j] = fma(Q.pref, acc, V[i][j]);
      }
    }
  }
  // the shells' functions: NFA / NFB of them, pure (2l + 1) or Cartesian;
  // the contraction with F in the ESP integrals' precision (F is stored in
  // it), G accumulated in FP64
  const int nfa = pure ? 2 * LA + 1 : NCA, nfb = pure ? 2 * LB + 1 : NCB;
  auto ta = [&](int f, int i) {
    return pure ? sph_t<Rt>(LA, f < 5 ? f : 4, i) : (f == i ? Rt(1) : Rt(0));
  };
  auto tb = [&](int h, int j) {
    return pure ? sph_t<Rt>(LB, h < 5 ? h : 4, j) : (h == j ? Rt(1) : Rt(0));
  };
  Rt Fc[NCA], Gc[NCB];
#pragma unroll
  for (int i = 0; i < NCA; i++) {
    Rt s = Rt(0);
#pragma unroll
    for (int f = 0; f < NCA; f++)
      if (f < nfa)
        s = fma(Fg[(P.bf_p + f) * ld], ta(f, i), s);
    Fc[i] = s;
  }
#pragma unroll
  for (int j = 0; j < NCB; j++) {
    Rt s = Rt(0);
#pragma unroll
    for (int i = 0; i < NCA; i++)
      s = fma(Fc[i], V[i][j], s);
    Gc[j] = s;
  }
#pragma unroll
  for (int h = 0; h < NCB; h++)
    if (h < nfb) {
      Rt s = Rt(0);
#pragma unroll
      for (int j = 0; j < NCB; j++)
        s = fma(tb(h, j), Gc[j], s);
      atomicAdd(Gg + (P.bf_q + h) * ld, to_f64(-s));
    }
  if (P.bf_p != P.bf_q) {
    Rt Fq[NCB], Gp[NCA];
#pragma unroll
    for (int j = 0; j < NCB; j++) {
      Rt s = Rt(0);
#pragma unroll
      for (int h = 0; h < NCB; h++)
        if (h < nfb)
          s = fma(Fg[(P.bf_q + h) * ld], tb(h, j), s);
      Fq[j] = s;
    }
#pragma unroll
    for (int i = 0; i < NCA; i++) {
      Rt s = Rt(0);
#pragma unroll
      for (int j = 0; j < NCB; j++)
        s = fma(V[i][j], Fq[j], s);
      Gp[i] = s;
    }
#pragma unroll
    for (int f = 0; f < NCA; f++)
      if (f < nfa) {
        Rt s = Rt(0);
#pragma unroll
        for (int i = 0; i < NCA; i++)
          s = fma(ta(f, i), Gp[i], s);
        atomicAdd(Gg + (P.bf_p + f) * ld, to_f64(-s));
      }
  }
}

// G for one leaf's points and one slice of the shell pairs (pairs k with
// k = blockIdx.y mod gridDim.y), a thread per point.  The block screens 128
// candidate pairs at a time, once for all its points (the density mask and
// the batch's geometric screen, seminumerical_exchange.cpp:789-799), and
// compacts the survivors into shared memory in pair order; every thread then
// runs them at its point.  F and G are AO-major (row lambda, column the
// group's point, row stride ld); the slices of a leaf add into G by atomics.
// In FP32 the bounds give 128 registers and four blocks per SM (a 144-byte
// spill; faster than 168 registers and three blocks: 3.35 -> 2.72 ms a call
// at 8 waters with 16 target blocks per SM, against 8, and 2.53 ms with 32);
// the FP64 form needs the full register file.
template <typename Rt>
__global__ void __launch_bounds__(128, sizeof(Rt) == 4 ? 4 : 1)
    k_cosx_g(MolDev m, int l0, int off0, int npairs, const CxPair *__restrict__ pairs,
             const typename CxPrimOf<Rt>::type *__restrict__ prims, const Rt *__restrict__ etab,
             const int *__restrict__ mask, const double4 *__restrict__ lgeo, int pure, size_t ld,
             const Rt *__restrict__ F, double *__restrict__ G) {
  __shared__ CxPair list[128];
  __shared__ int wcount[4];
  const DevLeaf L = m.leaves[l0 + blockIdx.x];
  const double4 geo = lgeo[l0 + blockIdx.x];
  const int nslice = gridDim.y, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c0 = blockIdx.y; c0 < npairs; c0 += 128 * nslice) {
    const int k = c0 + threadIdx.x * nslice;
    bool keep = false;
    CxPair P;
    if (k < npairs && mask[k]) {
      P = pairs[k];
      const double dx = P.Pc[0] - geo.x, dy = P.Pc[1] - geo.y, dz = P.Pc[2] - geo.z;
      keep = sqrt(dx * dx + dy * dy + dz * dz) - P.ext < geo.w + kCosxMargin;
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, keep);
    if (lane == 0)
      wcount[warp] = __popc(ballot);
    __syncthreads();
    int base = 0, n = 0;
#pragma unroll
    for (int w = 0; w < 4; w++) {
      base += w < warp ? wcount[w] : 0;
      n += wcount[w];
    }
    if (keep)
      list[base + __popc(ballot & ((1u << lane) - 1u))] = P;
    __syncthreads();
    for (int p = threadIdx.x; p < L.cnt; p += blockDim.x) {
      const auto C = cx_point(m.pts[L.off + p], Rt(0));
      const size_t g = static_cast<size_t>(L.off - off0 + p);
      const Rt *Fg = F + g;
      double *Gg = G + g;
      for (int e = 0; e < n; e++) {
        const CxPair &Q = list[e];
        switch (Q.la * 3 + Q.lb) { // shells up to d (kCosxLmax)
        case 0: cosx_pair<Rt, 0, 0>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        case 1: cosx_pair<Rt, 0, 1>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        case 2: cosx_pair<Rt, 0, 2>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        case 3: cosx_pair<Rt, 1, 0>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        case 4: cosx_pair<Rt, 1, 1>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        case 5: cosx_pair<Rt, 1, 2>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        case 6: cosx_pair<Rt, 2, 0>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        case 7: cosx_pair<Rt, 2, 1>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        default: cosx_pair<Rt, 2, 2>(Q, prims, etab, C, pure, Fg, Gg, ld); break;
        }
      }
    }
    __syncthreads();
  }
}

// K'[mu, lambda] -= sum_g phi_mu(g) G[lambda, g], mu over the leaf's AOs and
// the kCosxAoTile AOs lambda of blockIdx.y: the leaf's G columns staged in
// shared memory, 128 points at a time; thread (mu group, lambda).
__global__ void __launch_bounds__(128) k_cosx_k(MolDev m, const double *__restrict__ ws, int l0,
                                                int off0, size_t ld,
                                                const double *__restrict__ G,
                                                double *__restrict__ Kp) {
  __shared__ double Gs[kCosxAoTile][129]; // padded: the 16 rows in distinct banks
  const DevLeaf L = m.leaves[l0 + blockIdx.x];
  const int lam0 = blockIdx.y * kCosxAoTile;
  const int nl = min(kCosxAoTile, m.nbf - lam0);
  const double *phi = ws + L.ws_off;
  const int *g = m.leaf_ao + L.ao_begin;
  const size_t nbf = static_cast<size_t>(m.nbf);
  const size_t col0 = static_cast<size_t>(L.off - off0);
  constexpr int kGroups = 128 / kCosxAoTile;
  const int j = threadIdx.x % kCosxAoTile, sg = threadIdx.x / kCosxAoTile;
  for (int pc = 0; pc < L.cnt; pc += 128) {
    const int np = min(128, L.cnt - pc);
    for (int e = threadIdx.x; e < kCosxAoTile * 128; e += blockDim.x) {
      const int r = e / 128, p = e % 128;
      Gs[r][p] = r < nl && p < np ? G[(lam0 + r) * ld + col0 + pc + p] : 0.0;
    }
    __syncthreads();
    for (int s = sg; s < L.nbf; s += kGroups) {
      const double *ph = phi + static_cast<size_t>(s) * L.npad + pc;
      double acc = 0.0;
      for (int p = 0; p < np; p++)
        acc = fma(ph[p], Gs[j][p], acc);
      if (j < nl)
        atomicAdd(&Kp[static_cast<size_t>(g[s]) * nbf + lam0 + j], -acc);
    }
    __syncthreads();
  }
}

// k_cosx_k in the mixed precision: double-float phi and G (G split as it is
// staged), K' summed in FP64.
__global__ void __launch_bounds__(128) k_cosx_k_df(MolDev m, const float2 *__restrict__ phi_hl,
                                                   int l0, int off0, size_t ld,
                                                   const double *__restrict__ G,
                                                   double *__restrict__ Kp) {
  __shared__ float2 Gs[kCosxAoTile][129]; // padded: the 16 rows in distinct banks
  const DevLeaf L = m.leaves[l0 + blockIdx.x];
  const int lam0 = blockIdx.y * kCosxAoTile;
  const int nl = min(kCosxAoTile, m.nbf - lam0);
  const float2 *phi = phi_hl + L.ws_off;
  const int *g = m.leaf_ao + L.ao_begin;
  const size_t nbf = static_cast<size_t>(m.nbf);
  const size_t col0 = static_cast<size_t>(L.off - off0);
  constexpr int kGroups = 128 / kCosxAoTile;
  const int j = threadIdx.x % kCosxAoTile, sg = threadIdx.x / kCosxAoTile;
  for (int pc = 0; pc < L.cnt; pc += 128) {
    const int np = min(128, L.cnt - pc);
    for (int e = threadIdx.x; e < kCosxAoTile * 128; e += blockDim.x) {
      const int r = e / 128, p = e % 128;
      Gs[r][p] = r < nl && p < np ? split_hl(G[(lam0 + r) * ld + col0 + pc + p])
                                  : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int s = sg; s < L.nbf; s += kGroups) {
      const float2 *ph = phi + static_cast<size_t>(s) * L.npad + pc;
      float sh = 0.f, sl = 0.f;
      for (int p = 0; p < np; p++)
        df_fma(ph[p], Gs[j][p], sh, sl);
      if (j < nl)
        atomicAdd(&Kp[static_cast<size_t>(g[s]) * nbf + lam0 + j], -(to_f64(sh) + to_f64(sl)));
    }
    __syncthreads();
  }
}

// K = scale (K' + K'^T) into column-major K with leading dimension ldk.
__global__ void k_cosx_sym(int nbf, const double *__restrict__ Kp, double *__restrict__ K,
                           size_t ldk, double scale) {
  const size_t n2 = static_cast<size_t>(nbf) * nbf;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n2;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t i = e / nbf, j = e % nbf;
    K[i * ldk + j] = scale * (Kp[e] + Kp[j * nbf + i]);
  }
}

__global__ void k_cosx_halfw(long n, const Pt4 *__restrict__ pts, double *__restrict__ coef) {
  const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n)
    coef[i] = 0.5 * pts[i].w;
}

// Hermite expansion coefficients E^{ij}_t (t = 0..i+j) of x^i e^{-a x^2}
// times x^j e^{-b x^2}, centres Qx = A - B apart (Helgaker et al., ch. 9).
void hermite_table(int la, int lb, double a, double b, double Qx, std::vector<double> &out) {
  const double p = a + b, q = a * b / p;
  const int nt = la + lb + 1;
  // E[i][j][t]
  std::vector<double> E(static_cast<size_t>(la + 1) * (lb + 1) * (nt + 1), 0.0);
  auto at = [&](int i, int j, int t) -> double & {
    return E[(static_cast<size_t>(i) * (lb + 1) + j) * (nt + 1) + t];
  };
  auto get = [&](int i, int j, int t) {
    if (t < 0 || t > i + j)
      return 0.0;
    return at(i, j, t);
  };
  for (int i = 0; i <= la; i++)
    for (int j = 0; j <= lb; j++)
      for (int t = 0; t <= i + j; t++) {
        double v;
        if (i == 0 && j == 0)
          v = std::exp(-q * Qx * Qx);
        else if (j == 0)
          v = get(i - 1, j, t - 1) / (2 * p) - q * Qx / a * get(i - 1, j, t) +
              (t + 1) * get(i - 1, j, t + 1);
        else
          v = get(i, j - 1, t - 1) / (2 * p) + q * Qx / b * get(i, j - 1, t) +
              (t + 1) * get(i, j - 1, t + 1);
        at(i, j, t) = v;
      }
  for (int i = 0; i <= la; i++)
    for (int j = 0; j <= lb; j++)
      for (int t = 0; t < nt; t++)
        out.push_back(get(i, j, t));
}

std::vector<int> cart_powers(int l) {
  std::vector<int> c;
  for (int a = l; a >= 0; a--)
    for (int b = l - a; b >= 0; b--)
      c.push_back(a | (b << 4) | ((l - a - b) << 8));
  return c;
}

// The analytic overlap of the basis' functions (host, McMurchie-Davidson).
std::vector<double> overlap_matrix(const Basis &B) {
  const int n = B.nbf;
  std::vector<double> S(static_cast<size_t>(n) * n, 0.0);
  std::vector<double> et;
  for (size_t s1 = 0; s1 < B.shells.size(); s1++)
    for (size_t s2 = 0; s2 < B.shells.size(); s2++) {
      const Shell &A = B.shells[s1], &Bs = B.shells[s2];
      const auto ca = cart_powers(A.l), cb = cart_powers(Bs.l);
      std::vector<double> Sc(ca.size() * cb.size(), 0.0);
      for (size_t x = 0; x < A.exps.size(); x++)
        for (size_t y = 0; y < Bs.exps.size(); y++) {
          const double a = A.exps[x], b = Bs.exps[y], p = a + b;
          std::vector<double> E[3];
          for (int d = 0; d < 3; d++)
            hermite_table(A.l, Bs.l, a, b, A.origin[d] - Bs.origin[d], E[d]);
          const int nb = Bs.l + 1, nt = A.l + Bs.l + 1;
          const double pref = A.coefs[x] * Bs.coefs[y] * std::pow(kPi / p, 1.5);
          for (size_t i = 0; i < ca.size(); i++)
            for (size_t j = 0; j < cb.size(); j++) {
              const int pa[3] = {ca[i] & 15, (ca[i] >> 4) & 15, ca[i] >> 8};
              const int pb[3] = {cb[j] & 15, (cb[j] >> 4) & 15, cb[j] >> 8};
              double e = pref;
              for (int d = 0; d < 3; d++)
                e *= E[d][(pa[d] * nb + pb[d]) * nt];
              Sc[i * cb.size() + j] += e;
            }
        }
      const double fac = common_fac(A.l, B.pure) * common_fac(Bs.l, B.pure);
      const int na = B.shell_size(static_cast<int>(s1)), nbb = B.shell_size(static_cast<int>(s2));
      const std::vector<double> *Ta = B.pure ? &spherical_transform(A.l) : nullptr;
      const std::vector<double> *Tb = B.pure ? &spherical_transform(Bs.l) : nullptr;
      for (int f = 0; f < na; f++)
        for (int h = 0; h < nbb; h++) {
          double v = 0.0;
          for (size_t i = 0; i < ca.size(); i++)
            for (size_t j = 0; j < cb.size(); j++) {
              const double ta = Ta ? (*Ta)[f * ca.size() + i] : (static_cast<size_t>(f) == i);
              const double tb = Tb ? (*Tb)[h * cb.size() + j] : (static_cast<size_t>(h) == j);
              v += ta * Sc[i * cb.size() + j] * tb;
            }
          const size_t r = B.first_bf[s1] + f, c = B.first_bf[s2] + h;
          S[c * n + r] = fac * v; // column-major
        }
    }
  return S;
}

// X = A^-1 B for symmetric positive definite A (column-major n x n): Cholesky.
std::vector<double> spd_solve(std::vector<double> A, const std::vector<double> &B, int n) {
  auto a = [&](int i, int j) -> double & { return A[static_cast<size_t>(j) * n + i]; };
  for (int j = 0; j < n; j++) {
    double d = a(j, j);
    for (int k = 0; k < j; k++)
      d -= a(j, k) * a(j, k);
    if (!(d > 0.0))
      throw ArgError("COSX: the numerical overlap matrix is not positive definite");
    a(j, j) = std::sqrt(d);
    for (int i = j + 1; i < n; i++) {
      double s = a(i, j);
      for (int k = 0; k < j; k++)
        s -= a(i, k) * a(j, k);
      a(i, j) = s / a(j, j);
    }
  }
  std::vector<double> X = B;
  for (int c = 0; c < n; c++) {
    double *x = &X[static_cast<size_t>(c) * n];
    for (int i = 0; i < n; i++) {
      double s = x[i];
      for (int k = 0; k < i; k++)
        s -= a(i, k) * x[k];
      x[i] = s / a(i, i);
    }
    for (int i = n - 1; i >= 0; i--) {
      double s = x[i];
      for (int k = i + 1; k < n; k++)
        s -= a(k, i) * x[k];
      x[i] = s / a(i, i);
    }
  }
  return X;
}

} // namespace

struct CosxState {
  std::unique_ptr<Molecule> N;
  int nbf = 0, npairs = 0;
  int precision = OCC_XC_FP64; // OCC_XC_MIXED: the ESP integrals in FP32
  std::vector<int> group_leaf0, group_nleaf, group_off0, group_npts;
  size_t group_pts_max = 0;
  double *d_Q = nullptr, *d_D = nullptr, *d_D2q = nullptr, *d_Kp = nullptr, *d_K = nullptr;
  double *d_F = nullptr, *d_G = nullptr, *d_etab = nullptr;
  float *d_etab_f = nullptr; // the E coefficients in FP32 (the mixed precision)
  float2 *d_phi_hl = nullptr, *d_D2q_hl = nullptr; // double-float phi and D2q (mixed)
  CxPair *d_pairs = nullptr;
  CxPrim *d_prims = nullptr;
  CxPrimF *d_prims_f = nullptr;
  int *d_mask = nullptr;
  double4 *d_lgeo = nullptr;
  std::vector<void *> allocations;
  ~CosxState() {
    for (void *p : allocations)
      cudaFree(p);
  }
  template <typename T> T *alloc(size_t n) {
    void *p = nullptr;
    cuda_check(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
    allocations.push_back(p);
    return static_cast<T *>(p);
  }
};

namespace {

// GridSettings::for_sgx(n) (src/numint/grid_settings.cpp:59-68)
GridSettings sgx_grid_settings(int angular) {
  GridSettings g;
  g.max_angular_points = angular;
  g.min_angular_points = angular;
  g.radial_precision = 1e-5;
  g.pruning_scheme = 0;
  g.reduced_first_row_element_grid = false;
  return g;
}

void upload_cosx_tables() {
  int comp[3][kCosxNc] = {};
  double T[3][5][kCosxNc] = {};
  for (int l = 0; l <= kCosxLmax; l++) {
    const auto c = cart_powers(l);
    for (size_t i = 0; i < c.size(); i++)
      comp[l][i] = c[i];
    const auto &t = spherical_transform(l);
    const int nc = static_cast<int>(c.size());
    for (int f = 0; f < 2 * l + 1; f++)
      for (int i = 0; i < nc; i++)
        T[l][f][i] = t[f * nc + i];
  }
  cuda_check(cudaMemcpyToSymbol(c_cx_comp, comp, sizeof(comp)), "cudaMemcpyToSymbol");
  cuda_check(cudaMemcpyToSymbol(c_cx_T, T, sizeof(T)), "cudaMemcpyToSymbol");
  float Tf[3][5][kCosxNc];
  for (int l = 0; l < 3; l++)
    for (int f = 0; f < 5; f++)
      for (int i = 0; i < kCosxNc; i++)
        Tf[l][f][i] = static_cast<float>(T[l][f][i]);
  cuda_check(cudaMemcpyToSymbol(c_cx_Tf, Tf, sizeof(Tf)), "cudaMemcpyToSymbol");
  double inv[kBoysTable];
  for (int i = 0; i < kBoysTable; i++)
    inv[i] = 1.0 / (2 * i + 1);
  cuda_check(cudaMemcpyToSymbol(c_inv_odd, inv, sizeof(inv)), "cudaMemcpyToSymbol");
  float invf[kBoysTable];
  for (int i = 0; i < kBoysTable; i++)
    invf[i] = static_cast<float>(inv[i]);
  cuda_check(cudaMemcpyToSymbol(c_inv_odd_f, invf, sizeof(invf)), "cudaMemcpyToSymbol");
}

} // namespace

std::unique_ptr<CosxState> cosx_create(Molecule &M, const GridSettings &gs, size_t ws_cap_bytes) {
  for (const Shell &s : M.basis.shells)
    if (s.l > kCosxLmax)
      throw ArgError("COSX: shells up to d are supported");
  DeviceGuard on_device(M.device);
  upload_cosx_tables();
  auto S = std::make_unique<CosxState>();
  S->nbf = M.basis.nbf;
  const int nbf = S->nbf;
  // the molecule on the SGX grid, AO values only
  auto N = std::make_unique<Molecule>();
  N->ctx = M.ctx;
  N->device = M.device;
  N->Z = M.Z;
  N->xyz = M.xyz;
  N->basis = M.basis;
  N->fs = M.fs;
  N->deriv = 0;
  N->gs = gs;
  N->bs = M.bs;
  N->bs.xc_screening_threshold = 1e-14;
  N->atom_batch = 128; // the reference's batches (seminumerical_exchange.cpp:726-752)
  PartitionFn part;
  if (device_partition_fits(M.device, static_cast<int>(M.Z.size())))
    part = [dev = M.device](const PartitionInput &in, double *w) { device_partition(dev, in, w); };
  N->grid = build_molecular_grid(N->Z, N->xyz, N->basis, N->gs, 0, part ? &part : nullptr);
  N->build_plan();
  N->upload();
  N->ensure_fp64_ws();
  cudaStream_t st = M.ctx->stream;
  const MolDev m = N->dev();
  launch_colloc_f64(m, 0, N->d_ws, st);
  N->fp64_ao_valid = true;
  S->d_phi_hl = S->alloc<float2>(N->ws_elems);
  k_cosx_split<<<1024, 256, 0, st>>>(N->ws_elems, N->d_ws, S->d_phi_hl);
  // S_num = phi^T diag(w) phi: the V_xc kernel with coefficient w / 2
  const long npts = N->plan.npts;
  k_cosx_halfw<<<static_cast<int>((npts + 255) / 256), 256, 0, st>>>(npts, N->d_pts, N->d_coef);
  double *d_Sn = S->alloc<double>(static_cast<size_t>(nbf) * nbf);
  cuda_check(cudaMemsetAsync(d_Sn, 0, static_cast<size_t>(nbf) * nbf * sizeof(double), st),
             "cudaMemsetAsync");
  launch_vxc_f64(m, 0, N->d_ws, N->d_coef, N->d_tiles, static_cast<int>(N->tiles.size()), d_Sn,
                 st);
  cuda_check(cudaGetLastError(), "kernel launch");
  std::vector<double> Sn(static_cast<size_t>(nbf) * nbf);
  cuda_check(cudaMemcpyAsync(Sn.data(), d_Sn, Sn.size() * sizeof(double), cudaMemcpyDeviceToHost,
                             st),
             "cudaMemcpyAsync D2H");
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  // Q = S_num^-1 S
  const std::vector<double> Sa = overlap_matrix(M.basis);
  const std::vector<double> Q = spd_solve(Sn, Sa, nbf);
  S->d_Q = S->alloc<double>(Q.size());
  cuda_check(cudaMemcpy(S->d_Q, Q.data(), Q.size() * sizeof(double), cudaMemcpyHostToDevice),
             "cudaMemcpy H2D");
  // shell pairs p >= q and their primitive pairs
  std::vector<CxPair> pairs;
  std::vector<CxPrim> prims;
  std::vector<double> et;
  const Basis &B = M.basis;
  for (size_t p = 0; p < B.shells.size(); p++)
    for (size_t q = 0; q <= p; q++) {
      const Shell &A = B.shells[p], &Bq = B.shells[q];
      // the engine's significant pairs: a shared origin, or an overlap block
      // of Frobenius norm >= 1e-12
      const bool same = A.origin[0] == Bq.origin[0] && A.origin[1] == Bq.origin[1] &&
                        A.origin[2] == Bq.origin[2];
      if (!same) {
        double f2 = 0.0;
        for (int i = 0; i < B.shell_size(static_cast<int>(p)); i++)
          for (int j = 0; j < B.shell_size(static_cast<int>(q)); j++) {
            const double v = Sa[static_cast<size_t>(B.first_bf[q] + j) * nbf + B.first_bf[p] + i];
            f2 += v * v;
          }
        if (!(std::sqrt(f2) >= kCosxPairOverlap))
          continue;
      }
      CxPair P{};
      double pmin = 1e300;
      P.bf_p = B.first_bf[p];
      P.bf_q = B.first_bf[q];
      P.np = B.shell_size(static_cast<int>(p));
      P.nq = B.shell_size(static_cast<int>(q));
      P.la = A.l;
      P.lb = Bq.l;
      P.prim0 = static_cast<int>(prims.size());
      const double fac = common_fac(A.l, B.pure) * common_fac(Bq.l, B.pure);
      for (size_t x = 0; x < A.exps.size(); x++)
        for (size_t y = 0; y < Bq.exps.size(); y++) {
          CxPrim r{};
          const double a = A.exps[x], b = Bq.exps[y];
          r.pexp = a + b;
          for (int d = 0; d < 3; d++)
            r.P[d] = (a * A.origin[d] + b * Bq.origin[d]) / r.pexp;
          if (r.pexp < pmin) { // the first most diffuse pair (esp.cpp:84-96)
            pmin = r.pexp;
            for (int d = 0; d < 3; d++)
              P.Pc[d] = r.P[d];
          }
          r.pref = A.coefs[x] * Bq.coefs[y] * 2.0 * kPi / r.pexp * fac;
          r.e_off = static_cast<int>(et.size());
          for (int d = 0; d < 3; d++)
            hermite_table(A.l, Bq.l, a, b, A.origin[d] - Bq.origin[d], et);
          prims.push_back(r);
        }
      P.nprim = static_cast<int>(prims.size()) - P.prim0;
      P.ext = std::sqrt(kCosxLogThreshold / pmin);
      pairs.push_back(P);
    }
  S->npairs = static_cast<int>(pairs.size());
  size_t bytes = 0;
  S->d_pairs = dev_upload(pairs, bytes);
  S->allocations.push_back(S->d_pairs);
  S->d_prims = dev_upload(prims, bytes);
  S->allocations.push_back(S->d_prims);
  std::vector<CxPrimF> primsf(prims.size());
  for (size_t i = 0; i < prims.size(); i++) {
    CxPrimF &f = primsf[i];
    f.pexp = static_cast<float>(prims[i].pexp);
    f.pref = static_cast<float>(prims[i].pref);
    for (int d = 0; d < 3; d++) {
      f.Ph[d] = static_cast<float>(prims[i].P[d]);
      f.Pl[d] = static_cast<float>(prims[i].P[d] - static_cast<double>(f.Ph[d]));
    }
    f.e_off = prims[i].e_off;
    f.pad = 0;
  }
  S->d_prims_f = dev_upload(primsf, bytes);
  S->allocations.push_back(S->d_prims_f);
  S->d_etab = dev_upload(et, bytes);
  S->allocations.push_back(S->d_etab);
  const std::vector<float> etf(et.begin(), et.end());
  S->d_etab_f = dev_upload(etf, bytes);
  S->allocations.push_back(S->d_etab_f);
  S->d_mask = S->alloc<int>(pairs.size());
  // bounding spheres of the leaves kept by the plan (those with AOs)
  std::vector<double4> lgeo;
  for (long b = 0; b < N->plan.nleaves(); b++)
    if (N->plan.leaf_nbf[b] > 0)
      lgeo.push_back(make_double4(N->plan.leaf_centre[3 * b], N->plan.leaf_centre[3 * b + 1],
                                  N->plan.leaf_centre[3 * b + 2], N->plan.leaf_radius[b]));
  if (lgeo.size() != N->leaves.size())
    throw std::runtime_error("COSX: leaf geometry does not match the plan");
  S->d_lgeo = dev_upload(lgeo, bytes);
  S->allocations.push_back(S->d_lgeo);
  S->d_D = S->alloc<double>(2 * static_cast<size_t>(nbf) * nbf); // room for a UHF D
  S->d_D2q = S->alloc<double>(static_cast<size_t>(nbf) * nbf);
  S->d_D2q_hl = S->alloc<float2>(static_cast<size_t>(nbf) * nbf);
  S->d_Kp = S->alloc<double>(static_cast<size_t>(nbf) * nbf);
  S->d_K = S->alloc<double>(2 * static_cast<size_t>(nbf) * nbf);
  // leaf groups whose point-major F and G fit the cap
  const size_t per_pt = 2 * static_cast<size_t>(nbf) * sizeof(double);
  const size_t cap_pts = std::max<size_t>(ws_cap_bytes / std::max<size_t>(per_pt, 1), 256);
  const auto &Ls = N->leaves;
  size_t i = 0;
  while (i < Ls.size()) {
    const size_t l0 = i;
    const int off0 = Ls[i].off;
    size_t pts = 0;
    while (i < Ls.size() && (pts + Ls[i].cnt <= cap_pts || i == l0)) {
      pts = static_cast<size_t>(Ls[i].off + Ls[i].cnt - off0);
      i++;
    }
    S->group_leaf0.push_back(static_cast<int>(l0));
    S->group_nleaf.push_back(static_cast<int>(i - l0));
    S->group_off0.push_back(off0);
    S->group_npts.push_back(static_cast<int>(pts));
    S->group_pts_max = std::max(S->group_pts_max, pts);
  }
  S->d_F = S->alloc<double>(S->group_pts_max * nbf);
  S->d_G = S->alloc<double>(S->group_pts_max * nbf);
  S->N = std::move(N);
  return S;
}

// K of one density block: dD column-major with leading dimension ldd (nbf for
// a restricted D, 2 nbf for a spin block of an unrestricted one), K = scale
// (K' + K'^T) into dK with leading dimension ldk.
void cosx_exchange(Context &c, CosxState &S, const double *dD, size_t ldd, double *dK, size_t ldk,
                   double scale, cudaStream_t st) {
  const int nbf = S.nbf;
  const size_t n2 = static_cast<size_t>(nbf) * nbf;
  Molecule &N = *S.N;
  const MolDev m = N.dev();
  c.launch("cosx_d2q", st, [&] {
    k_cosx_d2q<<<dim3((nbf + 15) / 16, (nbf + 15) / 16), dim3(16, 16), 0, st>>>(nbf, S.d_Q, dD, ldd,
                                                                              S.d_D2q);
  });
  const bool mixed = S.precision == OCC_XC_MIXED;
  if (mixed)
    c.launch("cosx_split", st, [&] {
      const int g = static_cast<int>(std::min<size_t>((n2 + 255) / 256, 1024));
      k_cosx_split<<<g, 256, 0, st>>>(n2, S.d_D2q, S.d_D2q_hl);
    });
  c.launch("cosx_mask", st, [&] {
    k_cosx_mask<<<(S.npairs + 127) / 128, 128, 0, st>>>(S.npairs, nbf, S.d_pairs, S.d_D2q,
                                                        S.d_mask);
  });
  cuda_check(cudaMemsetAsync(S.d_Kp, 0, n2 * sizeof(double), st), "cudaMemsetAsync");
  for (size_t gi = 0; gi < S.group_leaf0.size(); gi++) {
    const int l0 = S.group_leaf0[gi], nl = S.group_nleaf[gi], off0 = S.group_off0[gi];
    const size_t ld = static_cast<size_t>(S.group_npts[gi]);
    const dim3 gf(nl, (nbf + kCosxAoTile - 1) / kCosxAoTile);
    // pair slices: enough blocks to fill the SMs a few times over
    const int nslice = std::max(1, std::min(kCosxMaxSlices, (kCosxTargetBlocks + nl - 1) / nl));
    const dim3 gg(nl, nslice);
    cuda_check(cudaMemsetAsync(S.d_G, 0, ld * nbf * sizeof(double), st), "cudaMemsetAsync");
    float *Ff = reinterpret_cast<float *>(S.d_F); // the mixed precision's F (half the buffer)
    c.launch("cosx_f", st, [&] {
      if (mixed)
        k_cosx_f_df<<<gf, 128, 0, st>>>(m, S.d_phi_hl, l0, off0, ld, S.d_D2q_hl, Ff);
      else
        k_cosx_f<<<gf, 128, 0, st>>>(m, N.d_ws, l0, off0, ld, S.d_D2q, S.d_F);
    });
    c.launch("cosx_g", st, [&] {
      if (mixed)
        k_cosx_g<float><<<gg, 128, 0, st>>>(m, l0, off0, S.npairs, S.d_pairs, S.d_prims_f,
                                            S.d_etab_f, S.d_mask, S.d_lgeo, N.basis.pure ? 1 : 0,
                                            ld, Ff, S.d_G);
      else
        k_cosx_g<double><<<gg, 128, 0, st>>>(m, l0, off0, S.npairs, S.d_pairs, S.d_prims,
                                             S.d_etab, S.d_mask, S.d_lgeo, N.basis.pure ? 1 : 0,
                                             ld, S.d_F, S.d_G);
    });
    c.launch("cosx_k", st, [&] {
      if (mixed)
        k_cosx_k_df<<<gf, 128, 0, st>>>(m, S.d_phi_hl, l0, off0, ld, S.d_G, S.d_Kp);
      else
        k_cosx_k<<<gf, 128, 0, st>>>(m, N.d_ws, l0, off0, ld, S.d_G, S.d_Kp);
    });
  }
  c.launch("cosx_sym", st, [&] {
    const int g = static_cast<int>(std::min<size_t>((n2 + 255) / 256, 1024));
    k_cosx_sym<<<g, 256, 0, st>>>(nbf, S.d_Kp, dK, ldk, scale);
  });
  cuda_check(cudaGetLastError(), "kernel launch");
}

} // namespace occx

using namespace occx;

struct occ_xc_cosx {
  std::unique_ptr<CosxState> impl;
  occ_xc_context *ctx;
};

extern "C" {

int occ_xc_cosx_create(occ_xc_context *ctx, occ_xc_molecule *mol,
                       const occ_xc_grid_settings *grid, occ_xc_cosx **out) {
  if (!ctx || !mol || !out || mol->ctx != ctx)
    return OCC_XC_ERR_ARG;
  if (grid && (grid->max_angular_points <= 0 || grid->min_angular_points <= 0 ||
               !(grid->radial_precision > 0.0)))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    auto cx = std::make_unique<occ_xc_cosx>();
    cx->ctx = ctx;
    cx->impl = cosx_create(*mol->impl, grid ? grid_settings_from(grid) : sgx_grid_settings(50),
                           size_t(2) << 30);
    *out = cx.release();
  });
}

void occ_xc_cosx_destroy(occ_xc_cosx *cx) { delete cx; }

int occ_xc_cosx_set_precision(occ_xc_cosx *cx, int precision) {
  if (!cx || (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED))
    return OCC_XC_ERR_ARG;
  cx->impl->precision = precision;
  return OCC_XC_OK;
}

int occ_xc_cosx_grid_points(const occ_xc_cosx *cx, long *npoints) {
  if (!cx || !npoints)
    return OCC_XC_ERR_ARG;
  *npoints = cx->impl->N->plan.npts;
  return OCC_XC_OK;
}

// Restricted: K = 1/4 (K' + K'^T) of D2q = Q (2 D) (seminumerical_exchange.cpp:
// 517-529).  Unrestricted (D and K 2 nbf x nbf, the alpha block above the
// beta one): per spin K_s = 1/2 (K'_s + K'_s^T) of Q (2 D_s) (:616-648).
static void cosx_any(Context &c, CosxState &S, const double *dD, double *dK, bool uhf,
                     cudaStream_t st) {
  const size_t n = static_cast<size_t>(S.nbf);
  if (!uhf) {
    cosx_exchange(c, S, dD, n, dK, n, 0.25, st);
    return;
  }
  cosx_exchange(c, S, dD, 2 * n, dK, 2 * n, 0.5, st);
  cosx_exchange(c, S, dD + n, 2 * n, dK + n, 2 * n, 0.5, st);
}

static int cosx_host(occ_xc_context *ctx, occ_xc_cosx *cx, const double *D, double *K, bool uhf) {
  if (!ctx || !cx || !D || !K || cx->ctx != ctx)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    DeviceGuard on_device(ctx->impl->device);
    CosxState &S = *cx->impl;
    cudaStream_t st = ctx->impl->stream;
    const size_t n2 = static_cast<size_t>(S.nbf) * S.nbf * (uhf ? 2 : 1);
    cuda_check(cudaMemcpyAsync(S.d_D, D, n2 * sizeof(double), cudaMemcpyHostToDevice, st),
               "cudaMemcpyAsync H2D");
    cosx_any(*ctx->impl, S, S.d_D, S.d_K, uhf, st);
    cuda_check(cudaMemcpyAsync(K, S.d_K, n2 * sizeof(double), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  });
}

static int cosx_device(occ_xc_context *ctx, occ_xc_cosx *cx, const double *d_D, double *d_K,
                       void *stream, bool uhf) {
  if (!ctx || !cx || !d_D || !d_K || cx->ctx != ctx)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    DeviceGuard on_device(ctx->impl->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->impl->stream;
    cosx_any(*ctx->impl, *cx->impl, d_D, d_K, uhf, st);
  });
}

int occ_xc_cosx_exchange(occ_xc_context *ctx, occ_xc_cosx *cx, const double *D, double *K) {
  return cosx_host(ctx, cx, D, K, false);
}

int occ_xc_cosx_exchange_device(occ_xc_context *ctx, occ_xc_cosx *cx, const double *d_D,
                                double *d_K, void *stream) {
  return cosx_device(ctx, cx, d_D, d_K, stream, false);
}

int occ_xc_cosx_exchange_unrestricted(occ_xc_context *ctx, occ_xc_cosx *cx, const double *D,
                                      double *K) {
  return cosx_host(ctx, cx, D, K, true);
}

int occ_xc_cosx_exchange_unrestricted_device(occ_xc_context *ctx, occ_xc_cosx *cx,
                                             const double *d_D, double *d_K, void *stream) {
  return cosx_device(ctx, cx, d_D, d_K, stream, true);
}

} // extern "C"
