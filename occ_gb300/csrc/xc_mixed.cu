// Mixed-precision XC build on the tcgen05 tensor cores.
//
// Both contractions run as TF32 MMAs with FP32 accumulators in tensor memory
// (TMEM).  The TMEM accumulation truncates (rounds toward zero) at every MMA,
// which biases long sums of same-signed terms; the density contraction is
// therefore done on an exact grid (see k_rho_mixed) so that its result is
// unbiased, while the potential contraction uses 3xTF32.  Collocation runs in
// FP32 with FP64 displacements and compensated exponents/coefficients; the
// functional, the per-leaf energy partials, the cross-block accumulation of
// V_xc (FP64 atomics) and the final sums are FP64.
//
// Work unit: a "block" = up to 128 points of one Morton leaf (a 256-point
// leaf is two blocks sharing the leaf's significant-AO list).  Per block:
//   k_colloc_f32   phi, grad phi (FP32) -> ws32[block][comp][mp][128], and a
//                  power-of-two bound of each point's |phi| row
//   k_rho_mixed    X = phi D2 (M = 128 points, N <= 128 AOs per pass, K = m in
//                  segments of <= 512), epilogue rho = rowsum(phi o X),
//                  grad rho = 2 rowsum(grad phi o X)   (src/gto/density.cpp:33-43)
//   k_func         FP64 functional per leaf (shared with the FP64 path)
//                  and, in the same launch, Y = 0.5 w vrho phi + 2 w vsigma
//                  grad rho . grad phi per block (ymix_block)
//   k_vxc_tma      K = phi^T Y (M = 128 AOs, N <= 256, K = the points of up to
//                  two blocks of a leaf), operands by TMA, V += K + K^T with
//                  FP64 atomics   (src/dft/xc_potential_matrix.cpp:19-41)
//   k_reduce       fixed-order FP64 sum of the per-leaf partials
#include <algorithm>
#include <cstring>
#include <type_traits>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "../../include/occ_xc.h"
#include "host/gto_eval.h"
#include "umma.cuh"
#include "xc_leaf_func.cuh"
#include "xc_engine.hpp"

namespace occx {

// Solid-harmonic transform for the FP32 collocation, factored per row f as
// T[f][k] = n_f t[f][k] with t small integers (exact in FP32) and the row
// scale n_f kept as a (hi, lo) float pair: rounding a factor such as sqrt(3)
// to one float would scale every AO of that kind the same way, a bias that
// does not average out over the grid.
constexpr int kSphRows = (kMaxL + 1) * (kMaxL + 1); // sum over l of 2l + 1
__constant__ float c_spht[kSphTableSize];
__constant__ float2 c_sphn[kSphRows];

void fill_sph_table(double *out);

void upload_sph_table_mixed() {
  double h[kSphTableSize];
  float t[kSphTableSize];
  float2 n[kSphRows];
  fill_sph_table(h);
  int row = 0;
  for (int l = 0; l <= kMaxL; l++) {
    const int nc = ncart_of(l);
    for (int f = 0; f < 2 * l + 1; f++, row++) {
      const double *T = h + sph_offset(l) + f * nc;
      double mn = 1e300;
      for (int k = 0; k < nc; k++)
        if (T[k] != 0.0)
          mn = std::min(mn, std::fabs(T[k]));
      int q = 1;
      for (; q <= 16; q++) {
        bool ok = true;
        for (int k = 0; k < nc; k++) {
          const double r = T[k] / (mn / q);
          ok = ok && std::fabs(r - std::nearbyint(r)) < 1e-9;
        }
        if (ok)
          break;
      }
      if (q > 16)
        throw std::runtime_error("solid-harmonic row does not factor into integers");
      const double scale = mn / q;
      for (int k = 0; k < nc; k++)
        t[sph_offset(l) + f * nc + k] = static_cast<float>(std::nearbyint(T[k] / scale));
      const float hi = static_cast<float>(scale);
      n[row] = make_float2(hi, static_cast<float>(scale - hi));
    }
  }
  cuda_check(cudaMemcpyToSymbol(c_spht, t, sizeof(t)), "cudaMemcpyToSymbol");
  cuda_check(cudaMemcpyToSymbol(c_sphn, n, sizeof(n)), "cudaMemcpyToSymbol");
}

namespace {

constexpr int kBlockPts = 128;  // points per block (M of the density GEMM)
constexpr int kKc = 32;         // K chunk: one 128-byte swizzle row of TF32
constexpr int kMaxN = 256;      // N per pass of the 3xTF32 GEMM
constexpr int kExactN = 128;    // N per pass of the exact-grid GEMM
constexpr int kExactKSeg = 512; // K per exact accumulation (keeps integer sums < 2^24)
constexpr uint32_t kStageBytes = 96 * 1024;
// 3xTF32 stage: A hi/lo (128 x 32) and B hi/lo (up to 256 x 32)
constexpr uint32_t kOffAhi = 0, kOffAlo = 16 * 1024, kOffBhi = 32 * 1024, kOffBlo = 64 * 1024;
// exact-grid stage: A slices 1..3 (128 x 32) and B slices 1..3 (up to 128 x 32)
constexpr uint32_t kOffA1 = 0, kOffA2 = 16 * 1024, kOffA3 = 32 * 1024;
constexpr uint32_t kOffB1 = 48 * 1024, kOffB2 = 64 * 1024, kOffB3 = 80 * 1024;
constexpr uint32_t kWaitIter = 1u << 24; // bounded mbarrier waits
// The bound of the persistent kernels' pipeline waits (polls), read once per
// CTA.  occ_xc_set_wait_limit lowers it so that a test can make a wait run
// out; the final drains (bulk copies and MMAs in flight, before a CTA frees
// its TMEM and leaves) keep kWaitIter.
__device__ uint32_t g_wait_limit = kWaitIter;
constexpr uint32_t kRhoStageA = 3 * 16384; // exact-grid A slices of one K chunk (128 x 32 each)
constexpr int kErrTimeout = 1;
// AO planes of a block, [plane][mp][128] FP32 each: phi, d/dx, d/dy, d/dz
// (k_colloc_f32), Y (the V_xc operand, per build), then three planes' worth
// of the exact-grid slices of phi as the density GEMM's A operand: per K
// chunk of 64 AOs, three 128 x 64 BF16 K-major tiles in the 128-byte-swizzled
// layout of shared memory (k_colloc_f32), so that k_rho_mixed stages them
// with one bulk copy.  Everything but Y depends only on the grid and the
// basis and stays valid across builds of a molecule whose workspace is its
// own.
constexpr int kPlanes = 8;
constexpr int kPlaneYHi = 4, kPlaneASlices = 5;

struct MBlock {
  int mol;          // molecule (row of the MixTab table)
  int leaf;         // index into that molecule's leaves
  int p0;           // first point of the block within the leaf
  int cnt;          // points in the block (<= 128)
  int mp;           // significant AOs of the leaf, padded to 32
  int lblock;       // index of the block within its molecule (row scales)
  long long ws_off; // float offset of the block's [kPlanes][mp][128] planes in the molecule's ws
};
// A V_xc work item: AO rows i0 .. i0 + 127 of nblk consecutive blocks of one
// leaf (index block0 into the launch's block list); K runs over all their points.
struct VItem {
  int block0, nblk, i0;
};
// A leaf of the functional stage and its blocks (block0 .. block0 + nblk - 1).
struct LeafItem {
  int mol, leaf, block0, nblk;
};

// Everything the mixed kernels need of one molecule; a launch covers a table
// of these (one molecule for a single build, many for a batched build).
struct MixTab {
  MolDev m;
  FuncSet fs;
  double dens_thr;
  const float4 *prim32; // primitives (alpha hi, alpha lo, c hi, c lo)
  const float4 *shA;    // shell centres (hi xyz, lo xyz)
  float *ws;            // AO planes [block][kPlanes][mp][128]
  float *rowscale;      // power-of-two bound of each block row of phi
  float2 *dhl;          // D2 as (hi, lo) floats
  float *colb;          // column bounds of D2
  double *rho, *coef, *epart;
  const double *D;      // this build's density (mo.D)
  double *V;            // V_xc (A with V = A + A^T, then symmetrised)
  double *out2;         // {E_xc, integrated density}
  int vxc_n;            // N of the V_xc tile (64, 128 or 256)
  long long ws_row0;    // row of ws in the launch's tensor map (rows of 128 floats)
  int ao_valid;         // ws already holds this molecule's AO values: no collocation
};

// Per-launch replacement of a one-molecule table's D / V / out2 (so that a
// single build can read and write caller-owned buffers without a table update).
struct Override {
  const double *D;
  double *V, *out2;
};
__device__ __forceinline__ const double *t_D(const MixTab &T, const Override &o) {
  return o.D ? o.D : T.D;
}
__device__ __forceinline__ double *t_V(const MixTab &T, const Override &o) {
  return o.V ? o.V : T.V;
}
__device__ __forceinline__ double *t_out(const MixTab &T, const Override &o) {
  return o.out2 ? o.out2 : T.out2;
}

// Shared state of a CTA's two-stage shared-memory pipeline.
struct Pipe {
  uint8_t *stage[2];
  uint64_t *bar; // 2 mbarriers, one per stage
  uint32_t uses[2];
  uint32_t tmem;
  uint32_t ncols;
  bool ok;
};

__device__ __forceinline__ void pipe_wait_stage(Pipe &P, int s, int *err) {
  if (P.uses[s] > 0 && P.ok) {
    if (!umma::mbar_wait(&P.bar[s], (P.uses[s] - 1) & 1u, kWaitIter)) {
      P.ok = false;
      atomicExch(err, kErrTimeout);
    }
  }
}

__device__ __forceinline__ void pipe_drain(Pipe &P, int *err) {
  for (int s = 0; s < 2; s++)
    pipe_wait_stage(P, s, err);
}

// Barriers and TMEM (warp 0 allocates ncols columns, a power of two >= 32).
__device__ __forceinline__ void pipe_init(Pipe &P, uint8_t *smem, uint64_t *bars,
                                          uint32_t *tmem_slot, uint32_t ncols) {
  P.stage[0] = smem;
  P.stage[1] = smem + kStageBytes;
  P.bar = bars;
  P.uses[0] = P.uses[1] = 0;
  P.ok = true;
  P.ncols = ncols;
  if (threadIdx.x == 0) {
    umma::mbar_init(&bars[0], 1);
    umma::mbar_init(&bars[1], 1);
    umma::fence_proxy_async();
  }
  if (threadIdx.x < 32)
    umma::tmem_alloc(tmem_slot, ncols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  P.tmem = *tmem_slot;
}

__device__ __forceinline__ void pipe_finish(Pipe &P) {
  umma::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32)
    umma::tmem_dealloc(P.tmem, P.ncols);
}

// 3xTF32 MMAs of one K chunk into TMEM columns [tmem, tmem + N).
__device__ __forceinline__ void issue_tf32x3(const Pipe &P, int s, int N, bool first) {
  const uint32_t base = umma::smem_u32(P.stage[s]);
  const uint32_t idesc = umma::idesc_tf32(128, N);
  umma::fence_after_sync();
#pragma unroll
  for (int kk = 0; kk < kKc / 8; kk++) {
    const uint32_t o = kk * 32;
    const uint64_t ahi = umma::desc_kmajor_sw128(base + kOffAhi + o);
    const uint64_t alo = umma::desc_kmajor_sw128(base + kOffAlo + o);
    const uint64_t bhi = umma::desc_kmajor_sw128(base + kOffBhi + o);
    const uint64_t blo = umma::desc_kmajor_sw128(base + kOffBlo + o);
    umma::mma_tf32(P.tmem, alo, bhi, idesc, (first && kk == 0) ? 0u : 1u);
    umma::mma_tf32(P.tmem, ahi, blo, idesc, 1u);
    umma::mma_tf32(P.tmem, ahi, bhi, idesc, 1u);
  }
}

// Exact-grid MMAs of one K chunk: acc0 += A1 B1 (exact), acc1 += A1 B2 +
// A2 B1 (exact), acc2 += A2 B2 + A1 B3 + A3 B1 + A2 B3 + A3 B2 (tail, at most
// 2^-15 of the result, so its truncation is negligible), at TMEM columns
// tmem, tmem + 128, tmem + 256.  Only A3 B3 (about 2^-32 of the row bounds)
// is dropped.
__device__ __forceinline__ void issue_exact(const Pipe &P, int s, int N, bool first) {
  const uint32_t base = umma::smem_u32(P.stage[s]);
  const uint32_t idesc = umma::idesc_tf32(128, N);
  const uint32_t d0 = P.tmem, d1 = P.tmem + kExactN, d2 = P.tmem + 2 * kExactN;
  umma::fence_after_sync();
#pragma unroll
  for (int kk = 0; kk < kKc / 8; kk++) {
    const uint32_t o = kk * 32;
    const uint64_t a1 = umma::desc_kmajor_sw128(base + kOffA1 + o);
    const uint64_t a2 = umma::desc_kmajor_sw128(base + kOffA2 + o);
    const uint64_t a3 = umma::desc_kmajor_sw128(base + kOffA3 + o);
    const uint64_t b1 = umma::desc_kmajor_sw128(base + kOffB1 + o);
    const uint64_t b2 = umma::desc_kmajor_sw128(base + kOffB2 + o);
    const uint64_t b3 = umma::desc_kmajor_sw128(base + kOffB3 + o);
    const uint32_t acc = (first && kk == 0) ? 0u : 1u;
    umma::mma_tf32(d0, a1, b1, idesc, acc);
    umma::mma_tf32(d1, a1, b2, idesc, acc);
    umma::mma_tf32(d1, a2, b1, idesc, 1u);
    umma::mma_tf32(d2, a2, b3, idesc, acc);
    umma::mma_tf32(d2, a3, b2, idesc, 1u);
    umma::mma_tf32(d2, a2, b2, idesc, 1u);
    umma::mma_tf32(d2, a1, b3, idesc, 1u);
    umma::mma_tf32(d2, a3, b1, idesc, 1u);
  }
}

// One GEMM pass over nchunks K chunks: producers fill a stage (all threads),
// thread 0 issues the MMAs and commits them to the stage's barrier.
template <bool EXACT, class FA, class FB>
__device__ __forceinline__ void gemm_pass(Pipe &P, int N, int nchunks, FA &&fa, FB &&fb,
                                          int *err) {
  for (int c = 0; c < nchunks; c++) {
    const int s = c & 1;
    pipe_wait_stage(P, s, err);
    if (P.ok) {
      fa(c, P.stage[s]);
      fb(c, P.stage[s]);
    }
    umma::fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0 && P.ok) {
      if (EXACT)
        issue_exact(P, s, N, c == 0);
      else
        issue_tf32x3(P, s, N, c == 0);
      umma::commit(&P.bar[s]);
    }
    P.uses[s]++;
  }
  pipe_drain(P, err);
  umma::fence_after_sync();
}

// Store 4 consecutive FP32 values as TF32 hi/lo into row r, 16-byte chunk c.
__device__ __forceinline__ void store4(uint8_t *hi_tile, uint8_t *lo_tile, int r, int c, float a,
                                       float b, float cc, float d) {
  uint32_t h0, l0, h1, l1, h2, l2, h3, l3;
  umma::split_tf32(a, h0, l0);
  umma::split_tf32(b, h1, l1);
  umma::split_tf32(cc, h2, l2);
  umma::split_tf32(d, h3, l3);
  const uint32_t off = umma::sw128_offset(r, c);
  *reinterpret_cast<uint4 *>(hi_tile + off) = make_uint4(h0, h1, h2, h3);
  *reinterpret_cast<uint4 *>(lo_tile + off) = make_uint4(l0, l1, l2, l3);
}

// x = a1 + a2 + a3 relative to a power-of-two row bound s >= |row|:
// a1 on the grid s 2^-7 and a2 on the grid s 2^-15 (each at most 8
// significant bits, so products of slices of two rows are exact and their
// sums are exact integers on a common grid while below 2^24 units), a3 the
// TF32-rounded tail (|a3| <= s 2^-16).
// `tail` (optional) is a correction below the float precision of x (the
// FP64 residual of a value rounded to float) folded into a3.
__device__ __forceinline__ void slice3(float x, float s, float inv_s, uint32_t &a1, uint32_t &a2,
                                       uint32_t &a3, float tail = 0.f) {
  const float q = x * inv_s;
  const float i1 = rintf(q * 128.f);
  const float r1 = q - i1 * (1.f / 128.f);
  const float i2 = rintf(r1 * 32768.f);
  const float r2 = r1 - i2 * (1.f / 32768.f);
  a1 = __float_as_uint(i1 * (1.f / 128.f) * s);
  a2 = __float_as_uint(i2 * (1.f / 32768.f) * s);
  uint32_t t;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(fmaf(r2, s, tail)));
  a3 = t;
}

__device__ __forceinline__ void store4_exact(uint8_t *t1, uint8_t *t2, uint8_t *t3, int r, int c,
                                             const float (&v)[4], float s, float inv_s,
                                             const float (&tail)[4] = {0.f, 0.f, 0.f, 0.f}) {
  uint32_t a1[4], a2[4], a3[4];
#pragma unroll
  for (int e = 0; e < 4; e++)
    slice3(v[e], s, inv_s, a1[e], a2[e], a3[e], tail[e]);
  const uint32_t off = umma::sw128_offset(r, c);
  *reinterpret_cast<uint4 *>(t1 + off) = make_uint4(a1[0], a1[1], a1[2], a1[3]);
  *reinterpret_cast<uint4 *>(t2 + off) = make_uint4(a2[0], a2[1], a2[2], a2[3]);
  *reinterpret_cast<uint4 *>(t3 + off) = make_uint4(a3[0], a3[1], a3[2], a3[3]);
}

// The density GEMM's operands: the same three slices in BF16.  a1 and a2 hold
// at most 8 significant bits and are exact in BF16; the tail a3 is rounded to
// the nearest BF16 (|error| <= 2^-25 s).  A K chunk of the density GEMM is 64
// AOs: one 128-byte row of BF16, the same bytes as 32 TF32 values, so the
// tiles keep the TF32 path's 128-byte-swizzled layout and descriptors.
constexpr int kKcR = 64;
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi); // .x (low half) = lo
  return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ void slice3f(float x, float s, float inv_s, float &a1, float &a2,
                                        float &a3, float tail) {
  const float q = x * inv_s;
  const float i1 = rintf(q * 128.f);
  const float r1 = q - i1 * (1.f / 128.f);
  const float i2 = rintf(r1 * 32768.f);
  const float r2 = r1 - i2 * (1.f / 32768.f);
  a1 = i1 * (1.f / 128.f) * s;
  a2 = i2 * (1.f / 32768.f) * s;
  a3 = fmaf(r2, s, tail);
}
// Eight consecutive K values of row r (16-byte chunk c) of the three BF16
// slice tiles.
__device__ __forceinline__ void store8_exact_bf16(uint8_t *t1, uint8_t *t2, uint8_t *t3, int r,
                                                  int c, const float (&v)[8], float s,
                                                  float inv_s, const float (&tail)[8]) {
  float a1[8], a2[8], a3[8];
#pragma unroll
  for (int e = 0; e < 8; e++)
    slice3f(v[e], s, inv_s, a1[e], a2[e], a3[e], tail[e]);
  const uint32_t off = umma::sw128_offset(r, c);
  *reinterpret_cast<uint4 *>(t1 + off) =
      make_uint4(bf16x2_bits(a1[0], a1[1]), bf16x2_bits(a1[2], a1[3]), bf16x2_bits(a1[4], a1[5]),
                 bf16x2_bits(a1[6], a1[7]));
  *reinterpret_cast<uint4 *>(t2 + off) =
      make_uint4(bf16x2_bits(a2[0], a2[1]), bf16x2_bits(a2[2], a2[3]), bf16x2_bits(a2[4], a2[5]),
                 bf16x2_bits(a2[6], a2[7]));
  *reinterpret_cast<uint4 *>(t3 + off) =
      make_uint4(bf16x2_bits(a3[0], a3[1]), bf16x2_bits(a3[2], a3[3]), bf16x2_bits(a3[4], a3[5]),
                 bf16x2_bits(a3[6], a3[7]));
}

// Power of two >= |v| (1 for zero rows).
__device__ __forceinline__ float pow2_bound(float v) {
  if (!(v > 0.f))
    return 1.f;
  int e;
  frexpf(v, &e); // v = f 2^e, 0.5 <= f < 1
  return ldexpf(1.f, e);
}

// One step of a compensated dot product (Ogita, Rump, Oishi, SIAM J. Sci.
// Comput. 26, 1955 (2005), Dot2): the product's rounding error from an FMA
// and the sum's from TwoSum go to the running correction c.  The _rn
// intrinsics are never contracted into FMAs, which would break the
// error-free transformations.
__device__ __forceinline__ void dot2_step(float a, float b, float &s, float &c) {
  const float p = __fmul_rn(a, b);
  const float pe = fmaf(a, b, -p);
  const float t = __fadd_rn(s, p);
  const float bp = __fsub_rn(t, s);
  const float se = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  s = t;
  c = __fadd_rn(c, __fadd_rn(se, pe));
}

// s + e = a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// e^(-t) for t >= 0 in FP32 without a systematic error: Cody-Waite argument
// reduction (W.J. Cody, W. Waite, Software Manual for the Elementary
// Functions, 1980), -t = n ln2 + r with |r| <= ln2/2 and ln2 split into a
// 15-bit head (n * head is exact) and a tail, then the degree-8 Taylor
// polynomial of e^r (truncation below 2e-10, of either sign with r) and an
// exact scaling by 2^n.  Measured on GB300, the library expf has a one-sided
// mean relative error of about +6e-9, which summed over a grid biases the
// density; this routine's rounding errors are unbiased.
__device__ __forceinline__ float exp_neg(float t) {
  const float x = -t;
  const float n = rintf(x * 1.44269504088896341f);
  float r = fmaf(-n, 0.693145751953125f, x);  // exact (Sterbenz)
  r = fmaf(-n, 1.42860682030941723e-06f, r);  // ln2 - head
  float p = 2.48015873015873016e-05f;         // 1/8!
  p = fmaf(p, r, 1.98412698412698413e-04f);   // 1/7!
  p = fmaf(p, r, 1.38888888888888889e-03f);   // 1/6!
  p = fmaf(p, r, 8.33333333333333333e-03f);   // 1/5!
  p = fmaf(p, r, 4.16666666666666667e-02f);   // 1/4!
  p = fmaf(p, r, 1.66666666666666667e-01f);   // 1/3!
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  // exact scaling by 2^n, -126 <= n <= 0, through the exponent field
  return n < -126.f ? 0.f : p * __int_as_float((static_cast<int>(n) + 127) << 23);
}

// Difference of two double-float numbers (ah + al) - (bh + bl) as a
// double-float (hi, lo), from FP32 operations only (TwoSum on the heads).
__device__ __forceinline__ void df_sub(float ah, float al, float bh, float bl, float &h,
                                       float &l) {
  float s, e;
  two_sum(ah, -bh, s, e);
  e = __fadd_rn(e, __fsub_rn(al, bl));
  h = __fadd_rn(s, e);
  l = __fsub_rn(e, __fsub_rn(h, s));
}

// ---------------------------------------------------------------------------
// FP32 collocation of one block: ws32[comp][mp][128]
// x = hi + lo with hi = x rounded to the nearest TF32 and lo = (x - hi)
// rounded to the nearest TF32: both exact TF32 values, so the tensor core
// drops no bits and the split error has no sign bias (the 3xTF32 operands).
__device__ __forceinline__ void tf32_split(float x, float &hi, float &lo) {
  uint32_t h, l;
  umma::split_tf32(x, h, l);
  hi = __uint_as_float(h);
  lo = __uint_as_float(l);
}

// The exact-grid BF16 slices of one point's row of an AO plane (phi or a
// derivative, [mp][128]) as the density GEMM's A operand: per K chunk of 64
// AOs one 48 KB image of the three swizzled 128 x 64 tiles, AOs at and beyond
// mp zero.  ceil(mp / 64) images take at most the three planes' room.
__device__ __forceinline__ void write_a_slices(uint8_t *as, const float *plane0, int mp, int p,
                                               float sA, float isA) {
  const float zero8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int c = 0; c < (mp + kKcR - 1) / kKcR; c++) {
    uint8_t *tile = as + static_cast<size_t>(c) * kRhoStageA;
#pragma unroll 2
    for (int q = 0; q < kKcR / 8; q++) {
      float v[8];
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const int f = c * kKcR + q * 8 + e;
        v[e] = f < mp ? plane0[static_cast<size_t>(f) * kBlockPts + p] : 0.f;
      }
      store8_exact_bf16(tile, tile + 16384, tile + 32768, p, q, v, sA, isA, zero8);
    }
  }
}

template <int L>
__device__ __forceinline__ float colloc_shell_f32(const DevShell &sh, bool pure, float x, float y,
                                                  float z, float R, float dR, bool valid,
                                                  float *out, size_t plane) {
  // common_fac is folded into the contraction coefficients (prim32)
  constexpr int NC = ncart_of(L);
  constexpr int NF = 2 * L + 1 > NC ? 2 * L + 1 : NC;
  float cv[NC], cx[NC], cy[NC], cz[NC];
  cart_eval_l<L, float>(x, y, z, R, dR, cv, cx, cy, cz);
  float v[NF], gx[NF], gy[NF], gz[NF];
  if (!pure || L == 0) {
#pragma unroll
    for (int c = 0; c < NC; c++) {
      v[c] = cv[c];
      gx[c] = cx[c];
      gy[c] = cy[c];
      gz[c] = cz[c];
    }
  } else {
    const float *Tm = c_spht + sph_offset(L);
    const float2 *Nm = c_sphn + L * L;
#pragma unroll
    for (int f = 0; f < 2 * L + 1; f++) {
      float a = 0.f, b = 0.f, c = 0.f, d = 0.f;
#pragma unroll
      for (int k = 0; k < NC; k++) {
        const float t = Tm[f * NC + k];
        a = fmaf(t, cv[k], a);
        b = fmaf(t, cx[k], b);
        c = fmaf(t, cy[k], c);
        d = fmaf(t, cz[k], d);
      }
      const float2 n = Nm[f];
      v[f] = fmaf(n.x, a, n.y * a);
      gx[f] = fmaf(n.x, b, n.y * b);
      gy[f] = fmaf(n.x, c, n.y * c);
      gz[f] = fmaf(n.x, d, n.y * d);
    }
  }
  float vmax = 0.f;
  const int nf = pure ? 2 * L + 1 : NC;
#pragma unroll
  for (int f = 0; f < NF; f++) { // compile-time bound keeps v[] in registers
    if (f < nf) {
      const size_t o = static_cast<size_t>(f) * kBlockPts;
      const float val = valid ? v[f] : 0.f;
      vmax = fmaxf(vmax, fabsf(val));
      out[o] = val;
      out[plane + o] = valid ? gx[f] : 0.f;
      out[2 * plane + o] = valid ? gy[f] : 0.f;
      out[3 * plane + o] = valid ? gz[f] : 0.f;
    }
  }
  return vmax;
}

// Exponents and coefficients as (hi, lo) float pairs: rounding alpha or c to
// one float would bias every point a primitive touches the same way, an error
// that does not average out over the grid.
__global__ void __launch_bounds__(128, 3) k_colloc_f32(const MixTab *__restrict__ tabs,
                                                    const MBlock *__restrict__ blocks) {
  const MBlock B = blocks[blockIdx.x];
  const MixTab &T = tabs[B.mol];
  if (T.ao_valid)
    return;
  const MolDev m = T.m;
  const float4 *__restrict__ prim32 = T.prim32;
  const float4 *__restrict__ shA = T.shA;
  float *__restrict__ ws = T.ws;
  const DevLeaf L = m.leaves[B.leaf];
  const int p = threadIdx.x;
  const bool valid = p < B.cnt;
  const size_t plane = static_cast<size_t>(B.mp) * kBlockPts;
  float *base = ws + B.ws_off;
  const Pt4 P = valid ? m.pts[L.off + B.p0 + p] : make_pt4(0.0, 0.0, 0.0, 0.0);
  // the point as double-float coordinates (once per point)
  const float pxh = static_cast<float>(P.x), pyh = static_cast<float>(P.y),
              pzh = static_cast<float>(P.z);
  const float pxl = static_cast<float>(P.x - pxh), pyl = static_cast<float>(P.y - pyh),
              pzl = static_cast<float>(P.z - pzh);
  float vmax = 0.f;
  int loc = 0;
  for (int k = L.sh_begin; k < L.sh_end; k++) {
    const int si = m.leaf_sh[k];
    const DevShell sh = m.shells[si];
    // Displacement as a double-float (hi, lo) pair; r^2 and alpha r^2 as
    // double-float pairs.  All points of a radial shell of an atom's grid lie
    // at the same distance from that atom, so a rounding of r^2 or alpha r^2
    // would be shared by every point of the shell and would not average out.
    const float4 ah = shA[2 * si], al = shA[2 * si + 1]; // centre (hi xyz, lo xyz)
    float x, y, z, xl, yl, zl;
    df_sub(pxh, pxl, ah.x, al.x, x, xl);
    df_sub(pyh, pyl, ah.y, al.y, y, yl);
    df_sub(pzh, pzl, ah.z, al.z, z, zl);
    float r2h, r2l;
    {
      const float p1 = __fmul_rn(x, x), p2 = __fmul_rn(y, y), p3 = __fmul_rn(z, z);
      const float q = (fmaf(x, x, -p1) + fmaf(y, y, -p2) + fmaf(z, z, -p3)) +
                      2.f * (x * xl + y * yl + z * zl);
      float s12, e12, e3;
      two_sum(p1, p2, s12, e12);
      two_sum(s12, p3, r2h, e3);
      r2l = (e12 + e3) + q;
    }
    float R = 0.f, dR = 0.f;
    for (int q = 0; q < sh.nprim; q++) {
      const float4 pc = prim32[sh.prim_off + q]; // alpha hi, alpha lo, c hi, c lo
      const float th = __fmul_rn(pc.x, r2h);
      const float tl = fmaf(pc.x, r2h, -th) + fmaf(pc.x, r2l, pc.y * r2h);
      const float e0 = exp_neg(th);
      const float ex = fmaf(-e0, tl, e0); // e^(-th - tl) to first order in tl
      const float e = fmaf(pc.z, ex, pc.w * ex);
      R += e;
      dR = fmaf(-2.f * pc.x, e, fmaf(-2.f * pc.y, e, dR));
    }
    float *out = base + static_cast<size_t>(loc) * kBlockPts + p;
    float v;
    switch (sh.l) {
    case 0: v = colloc_shell_f32<0>(sh, m.pure, x, y, z, R, dR, valid, out, plane); break;
    case 1: v = colloc_shell_f32<1>(sh, m.pure, x, y, z, R, dR, valid, out, plane); break;
    case 2: v = colloc_shell_f32<2>(sh, m.pure, x, y, z, R, dR, valid, out, plane); break;
    case 3: v = colloc_shell_f32<3>(sh, m.pure, x, y, z, R, dR, valid, out, plane); break;
    default: v = colloc_shell_f32<4>(sh, m.pure, x, y, z, R, dR, valid, out, plane); break;
    }
    vmax = fmaxf(vmax, v);
    loc += sh.nfunc;
  }
  for (int f = loc; f < B.mp; f++) {
    const size_t o = static_cast<size_t>(f) * kBlockPts + p;
    base[o] = 0.f;
    base[plane + o] = 0.f;
    base[2 * plane + o] = 0.f;
    base[3 * plane + o] = 0.f;
  }
  const float sA = pow2_bound(vmax), isA = 1.f / sA;
  T.rowscale[static_cast<size_t>(B.lblock) * kBlockPts + p] = sA;
  // the A operand of k_rho_mixed: this point's row of phi on the exact grid
  // (scale sA) in BF16, chunk by chunk of 64 AOs (the last one zero-padded),
  // at its swizzled place in the three tiles
  write_a_slices(reinterpret_cast<uint8_t *>(base + kPlaneASlices * plane), base, B.mp, p, sA,
                 isA);
}

constexpr uint32_t kSmemMain = 2 * kStageBytes;

constexpr int kMaxMapSmem = 1024; // block AO maps up to this size live in shared memory

struct alignas(16) SmemTail {
  uint64_t bars[2];
  uint32_t tmem_slot;
  int next; // work item fetched from the queue, broadcast to the CTA
  float coef[4][kBlockPts];
  float red[2][4][kBlockPts];
  int gmap[kMaxMapSmem];
  float bscale[kExactN]; // exact-split scales of the current pass's B rows
};
constexpr uint32_t kSmemTotal = kSmemMain + sizeof(SmemTail) + 1024;

__device__ __forceinline__ uint8_t *aligned_smem(uint8_t *raw) {
  const uint32_t a = umma::smem_u32(raw);
  return raw + ((1024u - (a & 1023u)) & 1023u);
}

// Per build: D2 = 2 D as (hi, lo) float pairs and, per column j, a power of
// two bounding |D2[k][j]| over all k (the column scale of the exact split).
// Grid: (max nbf, molecules).
__global__ void __launch_bounds__(256) k_prep_density(const MixTab *__restrict__ tabs,
                                                      Override ov, int *queue) {
  __shared__ float red[256];
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < 2)
    queue[threadIdx.x] = 0; // work queues of k_rho_mixed and k_vxc_tma
  const MixTab &T = tabs[blockIdx.y];
  const int nbf = T.m.nbf;
  const int j = blockIdx.x;
  if (j >= nbf)
    return;
  const double *__restrict__ D = t_D(T, ov);
  double *__restrict__ V = t_V(T, ov);
  float2 *__restrict__ dhl = T.dhl;
  float *__restrict__ colb = T.colb;
  float mx = 0.f;
  for (int k = threadIdx.x; k < nbf; k += 256) {
    const size_t o = static_cast<size_t>(j) * nbf + k;
    V[o] = 0.0; // V_xc is accumulated with atomics later in the build
    const double d = 2.0 * D[o];
    const float hi = static_cast<float>(d);
    dhl[o] = make_float2(hi, static_cast<float>(d - static_cast<double>(hi)));
    mx = fmaxf(mx, fabsf(hi));
  }
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    colb[j] = pow2_bound(red[0]);
}

// V holds A after the contractions, with V_xc = A + A^T: the final FP64
// symmetrisation, each unordered pair (r, c) read and written by one thread.
// Grid: (x, molecules).
__global__ void __launch_bounds__(256) k_symmetrize(const MixTab *__restrict__ tabs,
                                                    Override ov) {
  const MixTab &T = tabs[blockIdx.y];
  double *__restrict__ V = t_V(T, ov);
  const size_t n = static_cast<size_t>(T.m.nbf);
  for (size_t q = static_cast<size_t>(blockIdx.x) * 256 + threadIdx.x; q < n * n;
       q += static_cast<size_t>(gridDim.x) * 256) {
    const size_t c = q / n, r = q % n; // element (r, c), column-major
    if (r < c) {
      const double v = V[q] + V[r * n + c];
      V[q] = v;
      V[r * n + c] = v;
    } else if (r == c) {
      V[q] = 2.0 * V[q];
    }
  }
}

// ---- density: X = phi D2 on tcgen05, rho = rowsum(phi o X) ----------------
// (src/gto/density.cpp:33-43).  X is computed on an exact grid: phi rows
// scaled by a power of two s_p, D2 columns by t_j, both operands split into
// slices a1 (grid 2^-7), a2 (grid 2^-15), a3 (TF32 tail); acc0 = a1 b1 and
// acc1 = a1 b2 + a2 b1 are exact integer sums while a K segment holds at most
// 512 AOs, acc2 collects the tail products (at most 2^-15 of the result).
// One CTA per SM, persistent over blocks (most AOs first) from a global
// queue, with a ring of block indices in shared memory and these roles:
//   warp 12      block fetch, and per K chunk of 64 AOs one bulk copy of the
//                block's precomputed BF16 A slices (k_colloc_f32)
//   warps 4-11   B producers: D2 (hi, lo) gathered through the block's AO map
//                for 64 columns j x 64 AOs k, sliced with t_j, into the stage
//   warp 13      MMA issuer: eight BF16 MMAs per K step of 16 into acc0..acc2
//                of one of two TMEM buffers (3 x 64 columns each)
//   warp 14      epilogue loader: per 16 columns of a pass, bulk copies of
//                phi (and grad phi) of those AOs into a ring of two slots
//   warps 0-3    epilogue, one point per thread: X = acc0 + acc1 + acc2 and
//                compensated FP32 dot products with phi and grad phi read
//                from shared memory; rho and grad rho (FP64) when the block
//                is done
// The epilogue once read phi straight from global memory after each TMEM
// load, with only four warps to hide that latency; staging it through the
// loader takes the loads off its path.
// Every wait is bounded; on expiry the error flag is set and all roles leave.
constexpr int kRing = 4;                                   // depth of the work-item rings
constexpr int kRhoN = 64;                                  // columns j per pass
constexpr uint32_t kRhoStageB = 3 * (kRhoN * 128);        // B slices (64 x 64 BF16 each)
constexpr uint32_t kRhoStage = kRhoStageA + kRhoStageB;   // 72 KB
constexpr int kRhoStages = 2;
constexpr int kRhoThreads = 512; // + the scheduler warp (15)
constexpr int kRhoProd = 256;  // B producer threads (warps 4-11)
constexpr int kRhoEpi = 128;   // epilogue threads (warps 0-3)
constexpr int kRhoMap = 1024;  // AO maps up to this size are staged in shared memory
constexpr int kEpiCols = 16;   // columns per epilogue slot
constexpr int kEpiSlots = 2;
constexpr uint32_t kEpiPlaneBytes = kEpiCols * kBlockPts * 4;      // 8 KB
constexpr uint32_t kEpiSlotBytes = 4 * kEpiPlaneBytes;             // phi and grad phi
constexpr uint32_t kEpiBytes = kEpiSlots * kEpiSlotBytes;          // 64 KB

// What every role needs of a block, resolved once by the scheduler warp.
struct RhoInfo {
  int bi; // block index; -1: the queue is exhausted
  int mp, cnt, nbf_leaf, nbf;
  const float *ws;   // the block's AO planes
  const int *amap;   // the leaf's AO map
  const float2 *dhl; // D2 as (hi, lo)
  const float *colb; // D2's column bounds
  double *rho;       // the density components
  long long idx0;    // the block's first point in the molecule's grid
  long long np;      // the molecule's points
};

struct alignas(16) RhoSmem {
  uint64_t full[kRhoStages], empty[kRhoStages]; // per stage: B written, MMAs done
  uint64_t afull[kRhoStages];                     // per stage: the A bulk copy landed
  uint64_t efull[kEpiSlots], eempty[kEpiSlots];   // per epilogue slot: landed, read
  uint64_t tfull[2], tempty[2];
  uint64_t ifull[kRing], iempty[kRing];
  uint64_t done;
  uint32_t tmem_slot;
  RhoInfo info[kRing];
  int gmap[kRhoMap]; // the producers' current AO map
};
constexpr uint32_t kRhoSmem = kRhoStages * kRhoStage + kEpiBytes + sizeof(RhoSmem) + 1024;
static_assert(kRhoSmem <= 232448, "density kernel exceeds the shared memory of a CTA");

__device__ __forceinline__ void bar_named(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
// AND of v over the n threads of named barrier id (a barrier among them too).
__device__ __forceinline__ bool bar_all(int id, int n, bool v) {
  uint32_t r;
  asm volatile("{\n\t.reg .pred p, q;\n\t"
               "setp.ne.u32 p, %1, 0;\n\t"
               "barrier.red.and.pred q, %2, %3, p;\n\t"
               "selp.u32 %0, 1, 0, q;\n\t}"
               : "=r"(r)
               : "r"(static_cast<uint32_t>(v)), "r"(id), "r"(n)
               : "memory");
  return r != 0;
}

// TAU (meta-GGA): the same GEMM with the A slices of d_k phi (k = tk, built
// by k_meta_ops at plane kPlaneTauA + 3 (tk - 1)), contracted with d_k phi:
// sum_j d_k phi_j (d_k phi D2)_j into rho component 3 + tk.
constexpr int kPlaneTauA = kPlanes; // planes 8-16
template <bool DERIV, bool TAU = false>
__global__ void __launch_bounds__(kRhoThreads, 1)
    k_rho_mixed(const MixTab *__restrict__ tabs, const MBlock *__restrict__ blocks,
                const int *__restrict__ order, int nblocks, int *queue, int *err, int tk = 0) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = aligned_smem(smem_raw);
  uint8_t *ebuf = smem + kRhoStages * kRhoStage; // epilogue slots
  RhoSmem *sm = reinterpret_cast<RhoSmem *>(ebuf + kEpiBytes);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // AO planes the epilogue reads: phi (and its gradient), or d_k phi (TAU)
  constexpr int kEpiPlanes = (DERIV && !TAU) ? 4 : 1;
  if (t == 0) {
    for (int s = 0; s < kRhoStages; s++) {
      umma::mbar_init(&sm->full[s], kRhoProd);
      umma::mbar_init(&sm->afull[s], 1);
      umma::mbar_init(&sm->empty[s], 1);
    }
    for (int e = 0; e < kEpiSlots; e++) {
      umma::mbar_init(&sm->efull[e], 1);
      umma::mbar_init(&sm->eempty[e], kRhoEpi);
    }
    for (int b = 0; b < 2; b++) {
      umma::mbar_init(&sm->tfull[b], 1);
      umma::mbar_init(&sm->tempty[b], kRhoEpi);
    }
    for (int r = 0; r < kRing; r++) {
      umma::mbar_init(&sm->ifull[r], 1);
      umma::mbar_init(&sm->iempty[r], 3 + kRhoProd + kRhoEpi);
    }
    umma::mbar_init(&sm->done, 1);
    umma::fence_proxy_async();
  }
  if (warp == 0)
    umma::tmem_alloc(&sm->tmem_slot, 512);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = sm->tmem_slot;
  bool ok = true;
  const uint32_t wait_limit = g_wait_limit;
  auto wait = [&](uint64_t *bar, uint32_t parity) {
    if (ok && !umma::mbar_wait(bar, parity, wait_limit)) {
      ok = false;
      atomicExch(err, kErrTimeout);
    }
    return ok;
  };
  // groups that share named barriers take every decision to stop together
  const bool epi = warp < 4, prod = warp >= 4 && warp < 12;
  auto agree = [&] {
    if (epi)
      ok = bar_all(1, kRhoEpi, ok);
    else if (prod)
      ok = bar_all(2, kRhoProd, ok);
    return ok;
  };
  // consumer side of the block ring: the next block's resolved description
  // (false at the end of the queue or on a timed-out wait)
  auto next_block = [&](int k, RhoInfo &w) {
    const int slot = k % kRing;
    wait(&sm->ifull[slot], (k / kRing) & 1);
    if (!agree())
      return false;
    w = sm->info[slot];
    umma::mbar_arrive(&sm->iempty[slot]);
    return w.bi >= 0;
  };
  auto segs = [](int mp) { return (mp + kExactKSeg - 1) / kExactKSeg; };
  auto seg_chunks = [](int mp, int k0) { return (min(kExactKSeg, mp - k0) + kKcR - 1) / kKcR; };

  if (warp == 15) {
    // ---- scheduler (lane 0): blocks from the global queue, resolved into the
    // ring up to kRing ahead of the slowest role ----
    if (lane == 0) {
      for (int k = 0;; k++) {
        const int slot = k % kRing;
        if (k >= kRing && !wait(&sm->iempty[slot], ((k / kRing) - 1) & 1))
          break;
        const int qi = atomicAdd(&queue[0], 1);
        RhoInfo w;
        w.bi = qi < nblocks ? order[qi] : -1;
        if (w.bi >= 0) {
          const MBlock B = blocks[w.bi];
          const MixTab &T = tabs[B.mol];
          const DevLeaf L = T.m.leaves[B.leaf];
          w.mp = B.mp;
          w.cnt = B.cnt;
          w.nbf_leaf = L.nbf;
          w.nbf = T.m.nbf;
          w.ws = T.ws + B.ws_off;
          w.amap = T.m.leaf_ao + L.ao_begin;
          w.dhl = T.dhl;
          w.colb = T.colb;
          w.rho = T.rho;
          w.idx0 = static_cast<long long>(L.off) + B.p0;
          w.np = T.m.npts;
        }
        sm->info[slot] = w;
        umma::mbar_arrive(&sm->ifull[slot]);
        if (w.bi < 0)
          break;
      }
    }
  } else if (warp == 12) {
    // ---- A slices (lane 0) ----
    if (lane == 0) {
      uint32_t g = 0;
      RhoInfo B;
      for (int k = 0; ok; k++) {
        if (!next_block(k, B))
          break;
        const int aplane = TAU ? kPlaneTauA + 3 * (tk - 1) : kPlaneASlices;
        const uint8_t *as = reinterpret_cast<const uint8_t *>(
            B.ws + static_cast<size_t>(aplane) * B.mp * kBlockPts);
        for (int n0 = 0; n0 < B.mp && ok; n0 += kRhoN)
          for (int k0 = 0; k0 < B.mp && ok; k0 += kExactKSeg)
            for (int c = 0; c < seg_chunks(B.mp, k0); c++, g++) {
              const int s = g % kRhoStages;
              const uint32_t use = g / kRhoStages;
              if (use > 0 && !wait(&sm->empty[s], (use - 1) & 1))
                break;
              umma::mbar_arrive_expect_tx(&sm->afull[s], kRhoStageA);
              umma::bulk_load(smem + s * kRhoStage,
                              as + static_cast<size_t>(k0 / kKcR + c) * kRhoStageA, kRhoStageA,
                              &sm->afull[s]);
            }
        if (!ok)
          break;
      }
      for (uint32_t q = (g >= kRhoStages ? g - kRhoStages : 0); q < g; q++)
        umma::mbar_wait(&sm->afull[q % kRhoStages], (q / kRhoStages) & 1, kWaitIter);
    }
  } else if (prod) {
    // ---- B producers ----
    const int pt = t - 128;
    const int jr = pt & 63;        // row j of the B tile this thread fills
    const int qb = pt >> 6;        // first 16-byte chunk (0..3); then qb + 4
    uint32_t g = 0;
    RhoInfo B;
    for (int k = 0; ok; k++) {
      if (!next_block(k, B))
        break;
      const int *gsrc = B.amap;
      const int lnbf = B.nbf_leaf;
      const bool gsh = lnbf <= kRhoMap;
      if (gsh) {
        bar_named(2, kRhoProd);
        for (int q = pt; q < lnbf; q += kRhoProd)
          sm->gmap[q] = gsrc[q];
        bar_named(2, kRhoProd);
      }
      const int *gm = gsh ? sm->gmap : gsrc;
      const float2 *__restrict__ dhl = B.dhl;
      const size_t nbf = static_cast<size_t>(B.nbf);
      for (int n0 = 0; n0 < B.mp && ok; n0 += kRhoN) {
        const int lj = n0 + jr;
        const bool jv = lj < lnbf;
        const size_t gj = jv ? static_cast<size_t>(gm[lj]) : 0;
        const float sB = jv ? B.colb[gj] : 1.f, isB = 1.f / sB;
        // the pass's K chunks of 64 AOs in the order of the segments and
        // chunks the loader and the MMA issuer walk; each chunk's gathers
        // are issued one chunk ahead, so that their latency overlaps the
        // wait for the stage and the slicing of the previous chunk
        const int nq = (B.mp + kKcR - 1) / kKcR;
        auto fetch = [&](int q, float2(&d)[2][8]) {
#pragma unroll
          for (int r = 0; r < 2; r++)
#pragma unroll
            for (int e = 0; e < 8; e++) {
              const int lk = q * kKcR + (qb + 4 * r) * 8 + e;
              d[r][e] = (jv && lk < lnbf) ? dhl[static_cast<size_t>(gm[lk]) * nbf + gj]
                                          : make_float2(0.f, 0.f);
            }
        };
        float2 cur[2][8], nxt[2][8];
        fetch(0, cur);
        for (int q = 0; q < nq && ok; q++, g++) {
          if (q + 1 < nq)
            fetch(q + 1, nxt);
          const int s = g % kRhoStages;
          const uint32_t use = g / kRhoStages;
          if (use > 0 && !wait(&sm->empty[s], (use - 1) & 1))
            break;
          uint8_t *st = smem + s * kRhoStage + kRhoStageA;
#pragma unroll
          for (int r = 0; r < 2; r++) {
            float v[8], lo[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
              v[e] = cur[r][e].x;
              lo[e] = cur[r][e].y;
            }
            store8_exact_bf16(st, st + kRhoN * 128, st + 2 * kRhoN * 128, jr, qb + 4 * r, v,
                              sB, isB, lo);
          }
          umma::fence_proxy_async();
          umma::mbar_arrive(&sm->full[s]);
#pragma unroll
          for (int r = 0; r < 2; r++)
#pragma unroll
            for (int e = 0; e < 8; e++)
              cur[r][e] = nxt[r][e];
        }
      }
    }
  } else if (warp == 13) {
    // ---- MMA issuer (lane 0) ----
    if (lane == 0) {
      uint32_t g = 0, sc = 0; // chunks, segments
      bool issued = false;
      RhoInfo B;
      for (int k = 0; ok; k++) {
        if (!next_block(k, B))
          break;
        const int mp = B.mp;
        for (int n0 = 0; n0 < mp && ok; n0 += kRhoN) {
          const int N = min(kRhoN, mp - n0);
          const uint32_t idesc = umma::idesc_bf16(128, N);
          for (int k0 = 0; k0 < mp && ok; k0 += kExactKSeg, sc++) {
            const uint32_t buf = sc & 1, ub = sc >> 1;
            if (ub > 0 && !wait(&sm->tempty[buf], (ub - 1) & 1))
              break;
            umma::fence_after_sync();
            const uint32_t d0 = tmem + buf * 256, d1 = d0 + kRhoN, d2 = d0 + 2 * kRhoN;
            const int nch = seg_chunks(mp, k0);
            for (int c = 0; c < nch && ok; c++, g++) {
              const int s = g % kRhoStages;
              if (!wait(&sm->afull[s], (g / kRhoStages) & 1) ||
                  !wait(&sm->full[s], (g / kRhoStages) & 1))
                break;
              umma::fence_after_sync();
              const uint32_t base = umma::smem_u32(smem + s * kRhoStage);
#pragma unroll
              for (int kk = 0; kk < 4; kk++) { // K = 16 AOs (32 bytes of a row) per MMA
                const uint32_t o = kk * 32;
                const uint64_t a1 = umma::desc_kmajor_sw128(base + o);
                const uint64_t a2 = umma::desc_kmajor_sw128(base + 16384 + o);
                const uint64_t a3 = umma::desc_kmajor_sw128(base + 32768 + o);
                const uint64_t b1 = umma::desc_kmajor_sw128(base + kRhoStageA + o);
                const uint64_t b2 = umma::desc_kmajor_sw128(base + kRhoStageA + kRhoN * 128 + o);
                const uint64_t b3 =
                    umma::desc_kmajor_sw128(base + kRhoStageA + 2 * kRhoN * 128 + o);
                const uint32_t acc = (c == 0 && kk == 0) ? 0u : 1u;
                umma::mma_bf16(d0, a1, b1, idesc, acc);
                umma::mma_bf16(d1, a1, b2, idesc, acc);
                umma::mma_bf16(d1, a2, b1, idesc, 1u);
                umma::mma_bf16(d2, a2, b3, idesc, acc);
                umma::mma_bf16(d2, a3, b2, idesc, 1u);
                umma::mma_bf16(d2, a2, b2, idesc, 1u);
                umma::mma_bf16(d2, a1, b3, idesc, 1u);
                umma::mma_bf16(d2, a3, b1, idesc, 1u);
              }
              umma::commit(&sm->empty[s]);
              issued = true;
            }
            umma::commit(&sm->tfull[buf]);
          }
        }
      }
      if (issued) {
        umma::commit(&sm->done);
        umma::mbar_wait(&sm->done, 0, kWaitIter);
      }
    }
  } else if (warp == 14) {
    // ---- epilogue loader (lane 0): the AO values of each 16 columns of a
    // pass into a slot, in the order the epilogue consumes them ----
    if (lane == 0) {
      uint32_t e = 0; // slots filled
      RhoInfo B;
      for (int k = 0; ok; k++) {
        if (!next_block(k, B))
          break;
        const size_t plane = static_cast<size_t>(B.mp) * kBlockPts;
        const float *src = B.ws + (TAU ? tk * plane : 0);
        for (int n0 = 0; n0 < B.mp && ok; n0 += kRhoN) {
          const int N = min(kRhoN, B.mp - n0);
          for (int k0 = 0; k0 < B.mp && ok; k0 += kExactKSeg)
            for (int c0 = 0; c0 < N && ok; c0 += kEpiCols, e++) {
              const int slot = e % kEpiSlots;
              const uint32_t use = e / kEpiSlots;
              if (use > 0 && !wait(&sm->eempty[slot], (use - 1) & 1))
                break;
              umma::mbar_arrive_expect_tx(&sm->efull[slot], kEpiPlanes * kEpiPlaneBytes);
              for (int c = 0; c < kEpiPlanes; c++)
                umma::bulk_load(ebuf + slot * kEpiSlotBytes + c * kEpiPlaneBytes,
                                src + c * plane + static_cast<size_t>(n0 + c0) * kBlockPts,
                                kEpiPlaneBytes, &sm->efull[slot]);
            }
        }
      }
      // copies still in flight land before the CTA leaves
      for (uint32_t q = (e >= kEpiSlots ? e - kEpiSlots : 0); q < e; q++)
        umma::mbar_wait(&sm->efull[q % kEpiSlots], (q / kEpiSlots) & 1, kWaitIter);
    }
  } else if (epi) {
    // ---- epilogue: thread t holds point t of the block ----
    const int quad = warp;
    const int p = t;
    uint32_t sc = 0, e = 0; // segments, epilogue slots consumed
    RhoInfo B;
    for (int k = 0; ok; k++) {
      if (!next_block(k, B))
        break;
      float acc[4] = {0.f, 0.f, 0.f, 0.f}, cmp[4] = {0.f, 0.f, 0.f, 0.f};
      for (int n0 = 0; n0 < B.mp && ok; n0 += kRhoN) {
        const int N = min(kRhoN, B.mp - n0);
        for (int k0 = 0; k0 < B.mp && ok; k0 += kExactKSeg, sc++) {
          const uint32_t buf = sc & 1, ub = sc >> 1;
          wait(&sm->tfull[buf], ub & 1);
          if (!agree())
            break;
          umma::fence_after_sync();
          const uint32_t lanebase = tmem + (static_cast<uint32_t>(quad * 32) << 16) + buf * 256;
          for (int c0 = 0; c0 < N; c0 += kEpiCols, e++) {
            const int slot = e % kEpiSlots;
            wait(&sm->efull[slot], (e / kEpiSlots) & 1);
            if (!agree())
              break;
            const float *eph =
                reinterpret_cast<const float *>(ebuf + slot * kEpiSlotBytes) + p;
            uint32_t r0[16], r1[16], r2[16];
            umma::tmem_ld16(lanebase + c0, r0);
            umma::tmem_ld16(lanebase + kRhoN + c0, r1);
            umma::tmem_ld16(lanebase + 2 * kRhoN + c0, r2);
            umma::tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < kEpiCols; i++) {
              const float x = __fadd_rn(__uint_as_float(r0[i]),
                                        __fadd_rn(__uint_as_float(r1[i]), __uint_as_float(r2[i])));
              const int o = i * kBlockPts;
              // rho (the energy's direct input) with compensation; its
              // gradient, which enters through sigma, by plain FP32 FMAs
              dot2_step(eph[o], x, acc[0], cmp[0]);
              if (DERIV && !TAU) {
                acc[1] = fmaf(eph[kEpiCols * kBlockPts + o], x, acc[1]);
                acc[2] = fmaf(eph[2 * kEpiCols * kBlockPts + o], x, acc[2]);
                acc[3] = fmaf(eph[3 * kEpiCols * kBlockPts + o], x, acc[3]);
              }
            }
            // the slot's next fill is a bulk copy (async proxy): order this
            // thread's generic-proxy reads of it before that write (without
            // the fence a build now and then read a refilled slot)
            umma::fence_proxy_async();
            umma::mbar_arrive(&sm->eempty[slot]);
          }
          umma::fence_before_sync();
          umma::mbar_arrive(&sm->tempty[buf]);
        }
      }
      if (ok && p < B.cnt) {
        const size_t idx = static_cast<size_t>(B.idx0) + p;
        const size_t Np = static_cast<size_t>(B.np);
        if (TAU) {
          B.rho[(3 + tk) * Np + idx] = static_cast<double>(acc[0]) + static_cast<double>(cmp[0]);
          continue;
        }
        B.rho[idx] = static_cast<double>(acc[0]) + static_cast<double>(cmp[0]);
        if (DERIV)
          for (int c = 1; c < 4; c++)
            B.rho[c * Np + idx] = 2.0 * (static_cast<double>(acc[c]) + static_cast<double>(cmp[c]));
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0)
    umma::tmem_dealloc(tmem, 512);
}

// ---- V_xc: K = phi^T Y on tcgen05, operands staged by TMA ------------------
// One CTA per SM, persistent over V items (AO rows i0 .. i0 + 127 of the
// blocks of one leaf; K = their points) fetched from a global queue by a
// scheduler warp (kVxcSchedWarp), which resolves each item (sizes, workspace rows, AO
// map, output) and hands it to the roles through a ring in shared memory,
// up to four items ahead:
//   warp 8       TMA producer: per K chunk of 32 points the FP32 A rows
//                (phi, or the pair's A plane) and B rows (Y, or the pair's B
//                plane) into the hi slots, with the 128-byte swizzle: one
//                32 x 128 box per whole 128-row tile, 32 x 32 boxes for the
//                rest (the copies issued by the one producer thread bound
//                this kernel: the 128-row boxes took it from 1.02 to 0.90 ms
//                at 32 waters)
//   warps 10-13  the TF32 split: every word split in place into hi and,
//                beside it, lo (elementwise, so the swizzle does not
//                matter); then the stage goes to the MMA issuer.  Half the
//                operand bytes of pre-split hi / lo planes.
//   warp 9       MMA issuer: hi*hi + hi*lo + lo*hi ("3xTF32") into one of two
//                TMEM accumulators of 256 columns
//   warps 0-7    epilogue (two warps per TMEM lane quarter, each half of the
//                columns): TMEM -> FP64 atomics, coalesced along the rows,
//                into A with V_xc = A + A^T.  (Forming K^T beside K to add
//                each unordered pair once halves the atomics but measured
//                slower: 1.07 ms with it for leaves of at most 128 AOs,
//                1.22 ms with paired 128 x 128 tiles.)
// Stages and accumulators are double-buffered, so loads, MMAs and atomics of
// consecutive chunks and passes overlap.  Every wait is bounded; on expiry
// the error flag is set and all roles leave.
constexpr int kItemBlocks = 2;   // blocks of a leaf accumulated in one V item
constexpr int kVxcEpi = 256;     // epilogue threads (warps 0-7)
constexpr int kVxcConvWarps = 4;                 // split warps (10 .. 10 + kVxcConvWarps - 1)
constexpr int kVxcConv = 32 * kVxcConvWarps;      // split threads
constexpr int kVxcSchedWarp = 10 + kVxcConvWarps; // the scheduler warp
constexpr int kVxcThreads = 32 * (kVxcSchedWarp + 1); // + TMA warp 8, MMA warp 9
// The stages share 192 KB: two of 96 KB for tiles of up to 256 columns
// (k_vxc_tma<2>), or three of 64 KB for tiles of up to 128 columns
// (k_vxc_tma<3>), which keeps one more chunk in flight.
constexpr uint32_t kVxcStageArea = 2 * kStageBytes;
template <int NS> struct VxcStage {
  static constexpr uint32_t bytes = kVxcStageArea / NS;
  static constexpr int max_n = NS == 2 ? 256 : 128;
  static constexpr uint32_t off_blo = kOffBhi + static_cast<uint32_t>(max_n) * 128u;
};
static_assert(VxcStage<3>::off_blo + 128 * 128 <= VxcStage<3>::bytes, "three-stage layout");
static_assert(VxcStage<2>::off_blo + 256 * 128 <= VxcStage<2>::bytes, "two-stage layout");

// What every role needs of a V item, resolved once by the scheduler warp
// (the chain of dependent global loads would otherwise stall each role at
// every item).
struct VxcInfo {
  int it; // item index; -1: the queue is exhausted
  int mp, rows_a, nblk, i0, nbf_leaf, vxc_n, nbf;
  int r0[kItemBlocks]; // first row of each block in the tensor map
  const int *amap;     // the leaf's AO map
  double *V;           // accumulation target (A with V_xc = A + A^T)
};

struct alignas(16) VxcSmem {
  uint64_t full[3], empty[3];   // per stage: TMA landed, MMAs done
  uint64_t conv[3];             // per stage: TF32 split done
  uint64_t tfull[2], tempty[2]; // per accumulator: ready, drained
  uint64_t ifull[kRing], iempty[kRing];
  uint64_t done;                // the MMA thread's final commit
  uint32_t tmem_slot;
  VxcInfo info[kRing];
};
constexpr uint32_t kVxcSmem = kVxcStageArea + sizeof(VxcSmem) + 1024;

// Operand planes of k_vxc_tma: K = sum over npairs (1..3) of (A pair)^T
// (B pair), each operand an FP32 plane of the blocks, split into TF32 hi / lo
// in shared memory.  The builds: one pair (phi, Y) (the meta-GGA build adds
// (d_k phi, t_k)); the XC gradient: two pairs (d_c phi, Y) and (Z_c, phi);
// the meta-GGA gradient's tau term three pairs (2 d_c d_k phi, t_k).  Scalar
// fields, selected without indexing, so that the parameters stay in the
// constant bank.
struct VxcPlanes {
  int a0, b0, a1, b1, a2, b2;
  int npairs;
};
// phi (plane 0) and Y (written by the functional stage)
constexpr VxcPlanes kVxcSplitPlanes{0, kPlaneYHi, 0, 0, 0, 0, 1};

// Split n16 16-byte words at hi in place into TF32 hi and their remainders
// (TF32) at lo, by the split threads (ct = 0 .. kVxcConv - 1).
__device__ __forceinline__ void split_words(uint8_t *hi, uint8_t *lo, int n16, int ct) {
  float4 *h4 = reinterpret_cast<float4 *>(hi);
  float4 *l4 = reinterpret_cast<float4 *>(lo);
#pragma unroll 4
  for (int q = ct; q < n16; q += kVxcConv) {
    const float4 v = h4[q];
    float4 h, l;
    tf32_split(v.x, h.x, l.x);
    tf32_split(v.y, h.y, l.y);
    tf32_split(v.z, h.z, l.z);
    tf32_split(v.w, h.w, l.w);
    h4[q] = h;
    l4[q] = l;
  }
}

// The FP64 value of FP32 bits by integer operations (rebias the exponent,
// widen the mantissa), off the FP64 pipe, which GB300 has little of and
// which the epilogue's conversions would otherwise occupy.  Zero and FP32
// subnormals (below 1.2e-38) give a signed zero; the accumulators hold
// neither infinities nor NaNs.
__device__ __forceinline__ double f32_bits_to_f64(uint32_t u) {
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t hi = (u & 0x80000000u) | (e ? (((e + 896u) << 20) | ((u & 0x7fffffu) >> 3)) : 0u);
  const uint32_t lo = e ? (u << 29) : 0u;
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

template <int NS>
__global__ void __launch_bounds__(kVxcThreads, 1)
    k_vxc_tma(const MixTab *__restrict__ tabs, const MBlock *__restrict__ blocks,
              const VItem *__restrict__ items, int nitems, Override ov, int *queue, int *err,
              const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap tmap128,
              VxcPlanes pl) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = aligned_smem(smem_raw);
  using SG = VxcStage<NS>;
  VxcSmem *sm = reinterpret_cast<VxcSmem *>(smem + kVxcStageArea);
  auto stage = [&](int s) { return smem + static_cast<uint32_t>(s) * SG::bytes; };
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  if (t == 0) {
    for (int s = 0; s < NS; s++) {
      umma::mbar_init(&sm->full[s], 1);
      umma::mbar_init(&sm->empty[s], 1);
      umma::mbar_init(&sm->conv[s], kVxcConv);
    }
    for (int s = 0; s < 2; s++) {
      umma::mbar_init(&sm->tfull[s], 1);
      umma::mbar_init(&sm->tempty[s], kVxcEpi);
    }
    for (int r = 0; r < kRing; r++) {
      umma::mbar_init(&sm->ifull[r], 1);
      // consumers: the TMA thread, the MMA thread, the epilogue, the split
      umma::mbar_init(&sm->iempty[r], 2 + kVxcEpi + kVxcConv);
    }
    umma::mbar_init(&sm->done, 1);
    umma::fence_proxy_async();
    umma::tma_prefetch_desc(&tmap);
    umma::tma_prefetch_desc(&tmap128);
  }
  if (warp == 0)
    umma::tmem_alloc(&sm->tmem_slot, 512);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = sm->tmem_slot;
  bool ok = true;
  const uint32_t wait_limit = g_wait_limit;
  auto wait = [&](uint64_t *bar, uint32_t parity) {
    if (ok && !umma::mbar_wait(bar, parity, wait_limit)) {
      ok = false;
      atomicExch(err, kErrTimeout);
    }
    return ok;
  };
  // the epilogue and split warps work warp by warp, with no barrier between
  // warps (the epilogue shares each step's column AOs by shuffles, the split
  // warps each release their share of a stage): the threads of a warp, which issue
  // warp-collective TMEM loads, take every decision to stop together
  const bool epi = warp < 8, cv = warp >= 10 && warp < kVxcSchedWarp;
  auto agree = [&] {
    if (epi || cv)
      ok = __all_sync(0xffffffffu, ok);
    return ok;
  };
  // consumer side of the item ring: the next item's resolved description
  // (false at the end of the queue or on a timed-out wait)
  auto next_item = [&](int k, VxcInfo &w) {
    const int slot = k % kRing;
    wait(&sm->ifull[slot], (k / kRing) & 1);
    if (!agree())
      return false;
    w = sm->info[slot];
    umma::mbar_arrive(&sm->iempty[slot]);
    return w.it >= 0;
  };

  if (warp == kVxcSchedWarp) {
    // ---- scheduler (lane 0): items from the global queue, resolved into the
    // ring up to kRing ahead of the slowest role ----
    if (lane == 0) {
      for (int k = 0;; k++) {
        const int slot = k % kRing;
        if (k >= kRing && !wait(&sm->iempty[slot], ((k / kRing) - 1) & 1))
          break;
        const int it = atomicAdd(&queue[1], 1);
        VxcInfo w;
        w.it = it < nitems ? it : -1;
        if (w.it >= 0) {
          const VItem I = items[it];
          const MBlock B0 = blocks[I.block0];
          const MixTab &T = tabs[B0.mol];
          const DevLeaf L = T.m.leaves[B0.leaf];
          w.mp = B0.mp;
          w.nblk = I.nblk;
          w.i0 = I.i0;
          w.rows_a = min(128, B0.mp - I.i0); // a multiple of 32
          w.nbf_leaf = L.nbf;
          w.vxc_n = T.vxc_n;
          w.nbf = T.m.nbf;
          w.r0[0] = static_cast<int>(T.ws_row0 + B0.ws_off / kBlockPts);
          w.r0[1] = I.nblk > 1
                        ? static_cast<int>(T.ws_row0 + blocks[I.block0 + 1].ws_off / kBlockPts)
                        : 0;
          w.amap = T.m.leaf_ao + L.ao_begin;
          w.V = t_V(T, ov);
        }
        sm->info[slot] = w;
        umma::mbar_arrive(&sm->ifull[slot]);
        if (w.it < 0)
          break;
      }
    }
  } else if (warp == 8) {
    // ---- TMA producer (lane 0) ----
    if (lane == 0) {
      uint32_t g = 0; // chunks issued
      VxcInfo W;
      for (int k = 0; ok; k++) {
        if (!next_item(k, W))
          break;
        const int NT = W.vxc_n, mp = W.mp;
        for (int n0 = 0; n0 < mp && ok; n0 += NT) {
          const int N = min(NT, mp - n0);
          for (int pr = 0; pr < pl.npairs && ok; pr++)
          for (int b = 0; b < W.nblk && ok; b++) {
            const int r0 = b ? W.r0[1] : W.r0[0];
            for (int c = 0; c < kBlockPts / kKc; c++, g++) {
              const int s = static_cast<int>(g % NS);
              if (g >= NS && !wait(&sm->empty[s], ((g / NS) - 1) & 1))
                break;
              umma::mbar_arrive_expect_tx(&sm->full[s],
                                          static_cast<uint32_t>(W.rows_a + N) * 128u);
              uint8_t *st = stage(s);
              const int ah = pr == 0 ? pl.a0 : (pr == 1 ? pl.a1 : pl.a2);
              const int bh = pr == 0 ? pl.b0 : (pr == 1 ? pl.b1 : pl.b2);
              // whole 128-row tiles in one copy each, the rest 32 rows at a time
              for (int r = 0; r < W.rows_a;) {
                const bool big = W.rows_a - r >= 128;
                umma::tma_load_2d(st + kOffAhi + r * 128, big ? &tmap128 : &tmap, c * kKc,
                                  r0 + ah * mp + W.i0 + r, &sm->full[s]);
                r += big ? 128 : 32;
              }
              for (int r = 0; r < N;) {
                const bool big = N - r >= 128;
                umma::tma_load_2d(st + kOffBhi + r * 128, big ? &tmap128 : &tmap, c * kKc,
                                  r0 + bh * mp + n0 + r, &sm->full[s]);
                r += big ? 128 : 32;
              }
            }
          }
        }
      }
      // loads still in flight land before the CTA leaves
      for (uint32_t q = (g >= NS ? g - NS : 0); q < g; q++)
        umma::mbar_wait(&sm->full[q % NS], (q / NS) & 1, kWaitIter);
    }
  } else if (warp == 9) {
    // ---- MMA issuer (lane 0) ----
    if (lane == 0) {
      uint32_t g = 0, pc = 0; // chunks consumed, passes
      bool issued = false;
      VxcInfo W;
      for (int k = 0; ok; k++) {
        if (!next_item(k, W))
          break;
        const int NT = W.vxc_n;
        for (int n0 = 0; n0 < W.mp && ok; n0 += NT, pc++) {
          const int N = min(NT, W.mp - n0);
          const uint32_t buf = pc & 1, ub = pc >> 1;
          if (ub > 0 && !wait(&sm->tempty[buf], (ub - 1) & 1))
            break;
          umma::fence_after_sync();
          const uint32_t d = tmem + buf * 256;
          const uint32_t idesc = umma::idesc_tf32(128, N);
          const int nch = pl.npairs * W.nblk * (kBlockPts / kKc);
          for (int c = 0; c < nch && ok; c++, g++) {
            const int s = static_cast<int>(g % NS);
            if (!wait(&sm->conv[s], (g / NS) & 1))
              break;
            umma::fence_after_sync();
            const uint32_t base = umma::smem_u32(stage(s));
#pragma unroll
            for (int kk = 0; kk < kKc / 8; kk++) {
              const uint32_t o = kk * 32;
              const uint64_t ahi = umma::desc_kmajor_sw128(base + kOffAhi + o);
              const uint64_t alo = umma::desc_kmajor_sw128(base + kOffAlo + o);
              const uint64_t bhi = umma::desc_kmajor_sw128(base + kOffBhi + o);
              const uint64_t blo = umma::desc_kmajor_sw128(base + SG::off_blo + o);
              const uint32_t acc = (c == 0 && kk == 0) ? 0u : 1u;
              umma::mma_tf32(d, alo, bhi, idesc, acc);
              umma::mma_tf32(d, ahi, blo, idesc, 1u);
              umma::mma_tf32(d, ahi, bhi, idesc, 1u);
            }
            umma::commit(&sm->empty[s]);
            issued = true;
          }
          umma::commit(&sm->tfull[buf]);
        }
      }
      if (issued) { // every MMA done before TMEM is released
        umma::commit(&sm->done);
        umma::mbar_wait(&sm->done, 0, kWaitIter);
      }
    }
  } else if (cv) {
    // ---- TF32 split (warps 10 .. kVxcSchedWarp - 1) ----
    {
      const int ct = t - 10 * 32;
      uint32_t g = 0; // chunks split
      VxcInfo W;
      for (int k = 0; ok; k++) {
        if (!next_item(k, W))
          break;
        const int NT = W.vxc_n;
        for (int n0 = 0; n0 < W.mp && ok; n0 += NT) {
          const int N = min(NT, W.mp - n0);
          const int nch = pl.npairs * W.nblk * (kBlockPts / kKc);
          for (int c = 0; c < nch; c++, g++) {
            const int s = static_cast<int>(g % NS);
            wait(&sm->full[s], (g / NS) & 1);
            if (!agree())
              break;
            uint8_t *st = stage(s);
            split_words(st + kOffAhi, st + kOffAlo, W.rows_a * 8, ct);
            split_words(st + kOffBhi, st + SG::off_blo, N * 8, ct);
            umma::fence_proxy_async(); // generic-proxy writes, read by the MMAs
            umma::mbar_arrive(&sm->conv[s]);
          }
        }
      }
    }
  } else if (epi) {
    // ---- epilogue (warps 0-7) ----
    const int quad = warp & 3, half = warp >> 2;
    const int i = quad * 32 + lane; // row of the tile
    uint32_t pc = 0;
    VxcInfo W;
    for (int k = 0; ok; k++) {
      if (!next_item(k, W))
        break;
      const int *__restrict__ g = W.amap;
      double *__restrict__ V = W.V;
      const size_t nbf = static_cast<size_t>(W.nbf);
      const int NT = W.vxc_n;
      const int li = W.i0 + i;
      const bool iv = li < W.nbf_leaf;
      const size_t gi = iv ? static_cast<size_t>(g[li]) : 0;
      for (int n0 = 0; n0 < W.mp && ok; n0 += NT, pc++) {
        const int N = min(NT, W.mp - n0);
        const uint32_t buf = pc & 1, ub = pc >> 1;
        wait(&sm->tfull[buf], ub & 1);
        if (!agree())
          break;
        umma::fence_after_sync();
        const uint32_t lanebase = tmem + (static_cast<uint32_t>(quad * 32) << 16) + buf * 256;
        const int cols = N / 2; // a multiple of 16
        for (int c0 = half * cols; c0 < (half + 1) * cols; c0 += 16) {
          uint32_t r[16];
          umma::tmem_ld16(lanebase + c0, r);
          // the chunk's 16 column AOs, one load per lane, shared by shuffles
          const int ljl = n0 + c0 + (lane & 15);
          const int gl = ljl < W.nbf_leaf ? g[ljl] : 0;
          umma::tmem_wait_ld();
#pragma unroll
          for (int e = 0; e < 16; e++) {
            const int lj = n0 + c0 + e;
            const size_t gj = static_cast<size_t>(__shfl_sync(0xffffffffu, gl, e));
            // V accumulates A with V_xc = A + A^T (k_symmetrize): K[i][j]
            // goes to A[gi][gj], so a warp's lanes (consecutive rows i)
            // update consecutive addresses of one column
            if (iv && lj < W.nbf_leaf)
              atomicAdd(&V[gj * nbf + gi], f32_bits_to_f64(r[e]));
          }
        }
        umma::fence_before_sync();
        umma::mbar_arrive(&sm->tempty[buf]);
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0)
    umma::tmem_dealloc(tmem, 512);
}

constexpr int kYmixBatch = 4; // ymix_stream: iterations whose loads are issued together

// Y of one block from the coefficients cf[0 .. 127] (FP32) into the Y hi
// plane as FP32 (k_vxc_tma splits it in shared memory), by the NS threads
// tid = 0 .. NS - 1.
template <bool DERIV>
__device__ __forceinline__ void ymix_stream(const MixTab &T, const MBlock &B,
                                            const float4 *__restrict__ cf, int tid, int NS) {
  // Every load of kYmixBatch iterations is issued before the first store:
  // Y shares its base with the planes it is formed from, so the compiler
  // would otherwise keep one iteration's loads in flight per thread, too few
  // with the four CTAs an SM of the functional stage.
  constexpr int U = kYmixBatch, NC = DERIV ? 4 : 1;
  const size_t plane = static_cast<size_t>(B.mp) * (kBlockPts / 4); // in float4
  const int n4 = B.mp * (kBlockPts / 4);
  const float4 *__restrict__ src = reinterpret_cast<const float4 *>(T.ws + B.ws_off);
  float4 *__restrict__ dst = reinterpret_cast<float4 *>(T.ws + B.ws_off) + kPlaneYHi * plane;
  for (int q0 = tid; q0 < n4; q0 += NS * U) {
    float4 v[U][NC];
#pragma unroll
    for (int u = 0; u < U; u++)
      if (q0 + u * NS < n4)
#pragma unroll
        for (int c = 0; c < NC; c++)
          v[u][c] = src[c * plane + q0 + u * NS];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * NS;
      if (q >= n4)
        break;
      const int p = (q % (kBlockPts / 4)) * 4;
      const float4 c0 = cf[p], c1 = cf[p + 1], c2 = cf[p + 2], c3 = cf[p + 3];
      const float4 a = v[u][0];
      float4 y;
      y.x = a.x * c0.x;
      y.y = a.y * c1.x;
      y.z = a.z * c2.x;
      y.w = a.w * c3.x;
      if (DERIV) {
        const float4 gx = v[u][DERIV ? 1 : 0], gy = v[u][DERIV ? 2 : 0], gz = v[u][DERIV ? 3 : 0];
        y.x = fmaf(gz.x, c0.w, fmaf(gy.x, c0.z, fmaf(gx.x, c0.y, y.x)));
        y.y = fmaf(gz.y, c1.w, fmaf(gy.y, c1.z, fmaf(gx.y, c1.y, y.y)));
        y.z = fmaf(gz.z, c2.w, fmaf(gy.z, c2.z, fmaf(gx.z, c2.y, y.z)));
        y.w = fmaf(gz.w, c3.w, fmaf(gy.w, c3.z, fmaf(gx.w, c3.y, y.w)));
      }
      dst[q] = y;
    }
  }
}

// The B operand of k_vxc_tma for one block:
// Y = 0.5 w vrho phi + 2 w vsigma grad rho . grad phi (FP32) into the Y plane
// (split into TF32 hi / lo by k_vxc_tma); streams 4 planes in, 1 out.  Run by
// a whole CTA; cf holds 128 float4.
template <bool DERIV>
__device__ __forceinline__ void ymix_block(const MixTab &T, const MBlock &B, float4 *cf) {
  if (threadIdx.x < kBlockPts) {
    const int p = threadIdx.x;
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p < B.cnt) {
      const size_t N = static_cast<size_t>(T.m.npts);
      const size_t idx = static_cast<size_t>(T.m.leaves[B.leaf].off) + B.p0 + p;
      c.x = static_cast<float>(T.coef[idx]);
      if (DERIV) {
        c.y = static_cast<float>(T.coef[N + idx]);
        c.z = static_cast<float>(T.coef[2 * N + idx]);
        c.w = static_cast<float>(T.coef[3 * N + idx]);
      }
    }
    cf[p] = c;
  }
  __syncthreads();
  ymix_stream<DERIV>(T, B, cf, threadIdx.x, blockDim.x);
  __syncthreads(); // cf is reused by the next block
}

// Functional per leaf (one CTA per leaf item), the batched counterpart of the
// FP64 path's k_func: block skip, FP64 functional, weights, coefficients and
// the per-leaf energy / electron-count partials.
__device__ __forceinline__ double bsum256(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < 8; i++)
    s += sh[i];
  __syncthreads();
  return s;
}

// ... followed by the V_xc operand Y of each of the leaf's blocks (ymix_block):
// the latency-bound functional of some CTAs overlaps the HBM-bound Y
// streaming of the others on the SM.  128 threads, one per point of a full
// block (a CTA of 256 left half of its threads idle in the functional, with
// eight active warps an SM).
constexpr int kFuncThreads = 128;
template <bool DERIV>
__global__ void __launch_bounds__(kFuncThreads, 4) k_func_b(const MixTab *__restrict__ tabs,
                                                         const MBlock *__restrict__ blocks,
                                                         const LeafItem *__restrict__ litems) {
  __shared__ double sh[kFuncThreads / 32];
  __shared__ float4 cf[kBlockPts];
  const LeafItem li = litems[blockIdx.x];
  const MixTab &T = tabs[li.mol];
  leaf_functional<DERIV, true, kFuncThreads>(T.m.leaves[li.leaf], T.m.pts,
                                             static_cast<size_t>(T.m.npts), T.fs, T.dens_thr,
                                             T.rho, T.coef, T.epart + 2 * li.leaf, sh);
  __syncthreads(); // the leaf's coefficients are written
  for (int b = 0; b < li.nblk; b++)
    ymix_block<DERIV>(T, blocks[li.block0 + b], cf);
}

constexpr int kLeafMaxPts = 1024; // leaf_max's bound (check_build_settings)

// The build's functional stage (one CTA per leaf item, four per SM): the
// functional in double-float arithmetic (leaf_functional_f2, no FP64
// operation per point but VWN's atan and B88's asinh) with the coefficients
// as FP32 into shared memory, then
// the V_xc operand Y of each of the leaf's blocks from them (ymix_stream, one
// FP32 plane: k_vxc_tma forms hi and lo).  The FP64 coefficient
// array is not written.
template <bool DERIV>
__global__ void __launch_bounds__(kFuncThreads, 4) k_func_f2(const MixTab *__restrict__ tabs,
                                                          const MBlock *__restrict__ blocks,
                                                          const LeafItem *__restrict__ litems) {
  __shared__ double red[kFuncThreads / 32];
  __shared__ float4 cf[kLeafMaxPts];
  const LeafItem li = litems[blockIdx.x];
  const MixTab &T = tabs[li.mol];
  const int nblk = min(li.nblk, kLeafMaxPts / kBlockPts);
  leaf_functional_f2<DERIV, kFuncThreads, 0>(
      T.m.leaves[li.leaf], T.m.pts, static_cast<size_t>(T.m.npts), T.fs, T.dens_thr, T.rho,
      [&](int p, float4 c) { cf[p] = c; }, nblk * kBlockPts, T.epart + 2 * li.leaf, red);
  __syncthreads(); // cf is complete
  for (int q = 0; q < nblk; q++)
    ymix_stream<DERIV>(T, blocks[li.block0 + q], &cf[q * kBlockPts], threadIdx.x,
                       kFuncThreads);
}

// Fixed-order FP64 sums of the per-leaf partials, one CTA per molecule.
__global__ void __launch_bounds__(256) k_reduce_b(const MixTab *__restrict__ tabs, Override ov) {
  __shared__ double sh[8];
  const MixTab &T = tabs[blockIdx.x];
  const int n = T.m.nleaves;
  double e = 0.0, ne = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) {
    e += T.epart[2 * i];
    ne += T.epart[2 * i + 1];
  }
  e = bsum256(e, sh);
  ne = bsum256(ne, sh);
  if (threadIdx.x == 0) {
    double *o = t_out(T, ov);
    o[0] = e;
    o[1] = ne;
  }
}

// Self-test: C[128][N] = A[128][K] B[N][K]^T with the 3xTF32 pipeline
// (exact = 0) or the exact-grid pipeline (exact = 1, N <= 128, K <= 512).
__global__ void __launch_bounds__(256, 1) k_selftest_gemm(const float *__restrict__ A,
                                                          const float *__restrict__ Bm,
                                                          float *__restrict__ Cm, int N, int K,
                                                          int exact, int *err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = aligned_smem(smem_raw);
  SmemTail *tail = reinterpret_cast<SmemTail *>(smem + kSmemMain);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int quad = warp & 3, half = warp >> 2;
  Pipe P;
  pipe_init(P, smem, tail->bars, &tail->tmem_slot, exact ? 512 : kMaxN);
  const int row = quad * 32 + lane;
  const int cols = N / 2;
  if (!exact) {
    auto fa = [&](int c, uint8_t *st) {
      const int r = t & 127, kh = t >> 7;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float *s = A + static_cast<size_t>(r) * K + c * kKc + kh * 16 + 4 * q;
        store4(st + kOffAhi, st + kOffAlo, r, kh * 4 + q, s[0], s[1], s[2], s[3]);
      }
    };
    auto fb = [&](int c, uint8_t *st) {
      if (t >= N)
        return;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const float *s = Bm + static_cast<size_t>(t) * K + c * kKc + 4 * q;
        store4(st + kOffBhi, st + kOffBlo, t, q, s[0], s[1], s[2], s[3]);
      }
    };
    gemm_pass<false>(P, N, K / kKc, fa, fb, err);
    for (int c0 = half * cols; c0 < (half + 1) * cols; c0 += 16) {
      uint32_t r[16];
      umma::tmem_ld16(P.tmem + (static_cast<uint32_t>(quad * 32) << 16) + c0, r);
      umma::tmem_wait_ld();
#pragma unroll
      for (int i = 0; i < 16; i++)
        Cm[static_cast<size_t>(row) * N + c0 + i] = __uint_as_float(r[i]);
    }
  } else {
    // row bounds of A (row t & 127) and B (row t < N)
    float ma = 0.f, mb = 0.f;
    for (int k = 0; k < K; k++) {
      ma = fmaxf(ma, fabsf(A[static_cast<size_t>(t & 127) * K + k]));
      if (t < N)
        mb = fmaxf(mb, fabsf(Bm[static_cast<size_t>(t) * K + k]));
    }
    const float sA = pow2_bound(ma), isA = 1.f / sA, sB = pow2_bound(mb), isB = 1.f / sB;
    auto fa = [&](int c, uint8_t *st) {
      const int r = t & 127, kh = t >> 7;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float *s = A + static_cast<size_t>(r) * K + c * kKc + kh * 16 + 4 * q;
        const float v[4] = {s[0], s[1], s[2], s[3]};
        store4_exact(st + kOffA1, st + kOffA2, st + kOffA3, r, kh * 4 + q, v, sA, isA);
      }
    };
    auto fb = [&](int c, uint8_t *st) {
      if (t >= N)
        return;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const float *s = Bm + static_cast<size_t>(t) * K + c * kKc + 4 * q;
        const float v[4] = {s[0], s[1], s[2], s[3]};
        store4_exact(st + kOffB1, st + kOffB2, st + kOffB3, t, q, v, sB, isB);
      }
    };
    gemm_pass<true>(P, N, K / kKc, fa, fb, err);
    const uint32_t lanebase = P.tmem + (static_cast<uint32_t>(quad * 32) << 16);
    for (int c0 = half * cols; c0 < (half + 1) * cols; c0 += 16) {
      uint32_t r0[16], r1[16], r2[16];
      umma::tmem_ld16(lanebase + c0, r0);
      umma::tmem_ld16(lanebase + kExactN + c0, r1);
      umma::tmem_ld16(lanebase + 2 * kExactN + c0, r2);
      umma::tmem_wait_ld();
#pragma unroll
      for (int i = 0; i < 16; i++)
        Cm[static_cast<size_t>(row) * N + c0 + i] =
            __fadd_rn(__uint_as_float(r0[i]),
                      __fadd_rn(__uint_as_float(r1[i]), __uint_as_float(r2[i])));
    }
  }
  pipe_finish(P);
}

size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

void set_smem_attributes() {
  cuda_check(cudaFuncSetAttribute(k_rho_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kRhoSmem), "cudaFuncSetAttribute");
  cuda_check(cudaFuncSetAttribute(k_rho_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kRhoSmem), "cudaFuncSetAttribute");
  cuda_check(cudaFuncSetAttribute(k_rho_mixed<true, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, kRhoSmem),
             "cudaFuncSetAttribute");
  cuda_check(cudaFuncSetAttribute(k_vxc_tma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kVxcSmem), "cudaFuncSetAttribute");
  cuda_check(cudaFuncSetAttribute(k_vxc_tma<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kVxcSmem), "cudaFuncSetAttribute");
  cuda_check(cudaFuncSetAttribute(k_selftest_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kSmemTotal), "cudaFuncSetAttribute");
}

} // namespace

// Work lists and molecule table of one launch sequence: a single molecule,
// or a batch whose blocks, items and leaves all go into the same launches.
struct LaunchPlan {
  std::vector<MBlock> blocks;
  std::vector<VItem> items;
  std::vector<LeafItem> litems;
  std::vector<MixTab> tabs;
  std::vector<int> order; // k_rho_mixed's block order
  MBlock *d_blocks = nullptr;
  int *d_order = nullptr;
  int *d_queue = nullptr; // the two work-queue counters
  VItem *d_items = nullptr;
  LeafItem *d_litems = nullptr;
  MixTab *d_tabs = nullptr;
  int maxnbf = 0, deriv = 0;
  WsMaps tmap;            // the workspace as rows of 128 floats (k_vxc_tma)
  // the workspace already holds these molecules' AO values (phi, its gradient,
  // its TF32 split, row scales): collocation is skipped
  bool ao_valid = false;
  bool ao_cacheable = false; // the workspace belongs to this plan alone
  std::vector<void *> owned;
  ~LaunchPlan() {
    for (void *p : owned)
      cudaFree(p);
  }
};

// k_vxc_tma with the stage count that the widest V tile of the launch
// allows: three stages when every molecule's tile N is at most 128.
int plan_max_n(const LaunchPlan &P) {
  int m = 0;
  for (const MixTab &t : P.tabs)
    m = std::max(m, t.vxc_n);
  return m;
}
template <class... A> void launch_vxc(const LaunchPlan &P, int grid, cudaStream_t st, A... args) {
  if (plan_max_n(P) <= VxcStage<3>::max_n)
    k_vxc_tma<3><<<grid, kVxcThreads, kVxcSmem, st>>>(args...);
  else
    k_vxc_tma<2><<<grid, kVxcThreads, kVxcSmem, st>>>(args...);
}

// Per-molecule resident state of the mixed path.  The per-build workspace
// (AO planes, row scales, D2 hi/lo, column bounds) is bound separately: a
// private one for builds of the molecule alone, or a region of a batch's or
// the server's shared workspace.
struct MixedState {
  std::vector<MBlock> blocks; // this molecule's blocks (mol = 0)
  size_t ws_floats = 0;
  float4 *d_prim32 = nullptr;
  float4 *d_shA = nullptr; // shell centres as (hi xyz, lo xyz) float pairs
  int *d_err = nullptr;
  MixTab tab{};            // resident fields; workspace fields null
  char *d_private = nullptr;           // private workspace, allocated on first use
  std::unique_ptr<LaunchPlan> single;  // the one-molecule plan over it
};

// Layout of one molecule's mixed workspace (offsets from its base, 256-byte
// aligned).
struct WsLayout {
  size_t ws, rowscale, dhl, colb, total;
};
WsLayout ws_layout(const Molecule &M, int planes = kPlanes) {
  WsLayout L{};
  size_t off = 0;
  auto put = [&](size_t bytes) {
    const size_t o = off;
    off = (off + std::max<size_t>(bytes, 16) + 511) / 512 * 512; // whole tensor-map rows
    return o;
  };
  const size_t nbf = static_cast<size_t>(M.basis.nbf);
  size_t ws_floats = 0, nblocks = 0; // as prepare_mixed lays the blocks out
  for (const DevLeaf &Lf : M.leaves) {
    const size_t nb = (Lf.cnt + kBlockPts - 1) / kBlockPts;
    const size_t mp = (Lf.nbf + kKc - 1) / kKc * kKc;
    nblocks += nb;
    ws_floats += nb * planes * mp * kBlockPts;
  }
  L.ws = put(ws_floats * sizeof(float));
  L.rowscale = put(nblocks * kBlockPts * sizeof(float));
  L.dhl = put(nbf * nbf * sizeof(float2));
  L.colb = put(nbf * sizeof(float));
  L.total = off;
  return L;
}
// The molecule's workspace at `base` inside a region that starts at map_base
// (the region the launch's tensor map covers).
MixTab bind_ws(const Molecule &M, char *base, const char *map_base, int planes = kPlanes) {
  const WsLayout L = ws_layout(M, planes);
  MixTab T = M.mixed->tab;
  T.ws = reinterpret_cast<float *>(base + L.ws);
  T.ws_row0 = static_cast<long long>((base + L.ws) - map_base) / (kBlockPts * sizeof(float));
  T.ao_valid = 0;
  T.rowscale = reinterpret_cast<float *>(base + L.rowscale);
  T.dhl = reinterpret_cast<float2 *>(base + L.dhl);
  T.colb = reinterpret_cast<float *>(base + L.colb);
  return T;
}

namespace {

template <typename T> T *plan_upload(LaunchPlan &P, const std::vector<T> &v) {
  T *d = nullptr;
  cuda_check(cudaMalloc(&d, std::max<size_t>(v.size(), 1) * sizeof(T)), "cudaMalloc");
  P.owned.push_back(d);
  if (!v.empty())
    cuda_check(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice),
               "cudaMemcpy H2D");
  return d;
}

// Concatenate the molecules' work lists.  Items are interleaved so that CTAs
// running at the same time come from distant parts of the Morton order (and of
// the batch) and update different V_xc elements.
void make_plan_lists(LaunchPlan &P, const std::vector<Molecule *> &mols,
                     const std::vector<MixTab> &tabs, bool meta_plan = false) {
  P.tabs = tabs;
  P.deriv = mols.empty() ? 0 : mols[0]->deriv;
  if (!meta_plan)
    require_not_mgga(P.deriv, "batched mixed precision");
  std::vector<VItem> items;
  for (size_t mi = 0; mi < mols.size(); mi++) {
    Molecule &M = *mols[mi];
    if (M.deriv != P.deriv)
      throw ArgError("a launch plan holds molecules of one functional family (LDA or GGA)");
    P.maxnbf = std::max(P.maxnbf, M.basis.nbf);
    const int base = static_cast<int>(P.blocks.size());
    for (const MBlock &b0 : M.mixed->blocks) {
      MBlock b = b0;
      b.mol = static_cast<int>(mi);
      P.blocks.push_back(b);
    }
    // the blocks of a leaf are consecutive: V items over groups of up to
    // kItemBlocks of them, one leaf item over all of them
    const std::vector<MBlock> &mb = M.mixed->blocks;
    for (size_t b = 0; b < mb.size();) {
      size_t e = b;
      while (e < mb.size() && mb[e].leaf == mb[b].leaf)
        e++;
      P.litems.push_back({static_cast<int>(mi), mb[b].leaf, base + static_cast<int>(b),
                          static_cast<int>(e - b)});
      for (size_t g = b; g < e; g += kItemBlocks) {
        const int nb = static_cast<int>(std::min<size_t>(kItemBlocks, e - g));
        const int blk = base + static_cast<int>(g);
        for (int i0 = 0; i0 < mb[b].mp; i0 += 128)
          items.push_back({blk, nb, i0});
      }
      b = e;
    }
  }
  // interleave (CTAs running together then work on distant parts of the
  // Morton order and touch different V elements), then order by decreasing
  // cost so that the dynamic queue ends with small items (greedy balance)
  const size_t n = items.size(), lanes = 152, stride = (n + lanes - 1) / lanes;
  for (size_t r = 0; r < stride; r++)
    for (size_t q = 0; q < lanes; q++)
      if (q * stride + r < n)
        P.items.push_back(items[q * stride + r]);
  auto vcost = [&](const VItem &v) {
    const MBlock &b = P.blocks[v.block0];
    return static_cast<long>(std::min(128, b.mp - v.i0)) * b.mp * v.nblk;
  };
  std::stable_sort(P.items.begin(), P.items.end(),
                   [&](const VItem &a, const VItem &b) { return vcost(a) > vcost(b); });
  const size_t nb = P.blocks.size(), bstride = (nb + lanes - 1) / lanes;
  for (size_t r = 0; r < bstride; r++)
    for (size_t q = 0; q < lanes; q++)
      if (q * bstride + r < nb)
        P.order.push_back(static_cast<int>(q * bstride + r));
  std::stable_sort(P.order.begin(), P.order.end(),
                   [&](int a, int b) { return P.blocks[a].mp > P.blocks[b].mp; });
}

// Lists in their own device allocations (a plan that lives with its molecule
// or batch).
void make_plan(LaunchPlan &P, const std::vector<Molecule *> &mols, const std::vector<MixTab> &tabs) {
  make_plan_lists(P, mols, tabs);
  P.d_blocks = plan_upload(P, P.blocks);
  P.d_order = plan_upload(P, P.order);
  P.d_queue = plan_upload(P, std::vector<int>(2, 0));
  P.d_items = plan_upload(P, P.items);
  P.d_litems = plan_upload(P, P.litems);
  P.d_tabs = plan_upload(P, P.tabs);
}

int num_sms(int device) {
  int n = 0;
  cuda_check(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device), "attribute");
  return n;
}

// The mixed launch sequence of a plan (seven kernels whatever the molecule count,
// and the collocation on a workspace's first build).
void run_plan(LaunchPlan &P, Context &c, Override ov, int *err, cudaStream_t st, int max_ctas) {
  const int nmol = static_cast<int>(P.tabs.size());
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int nl = static_cast<int>(P.litems.size());
  if (nmol == 0)
    return;
  const int ctas = max_ctas > 0 ? max_ctas : num_sms(c.device);
  c.launch("prep_density", st, [&] {
    k_prep_density<<<dim3(P.maxnbf, nmol), 256, 0, st>>>(P.d_tabs, ov, P.d_queue);
  });
  if (nb > 0) {
    if (!P.ao_valid)
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    c.launch("rho_mixed", st, [&] {
      const int g = std::min(nb, ctas);
      if (P.deriv)
        k_rho_mixed<true><<<g, kRhoThreads, kRhoSmem, st>>>(P.d_tabs, P.d_blocks, P.d_order, nb,
                                                      P.d_queue, err);
      else
        k_rho_mixed<false><<<g, kRhoThreads, kRhoSmem, st>>>(P.d_tabs, P.d_blocks, P.d_order, nb,
                                                       P.d_queue, err);
    });
  }
  if (nl > 0)
    c.launch("func", st, [&] {
      if (P.deriv)
        k_func_f2<true><<<nl, kFuncThreads, 0, st>>>(P.d_tabs, P.d_blocks, P.d_litems);
      else
        k_func_f2<false><<<nl, kFuncThreads, 0, st>>>(P.d_tabs, P.d_blocks, P.d_litems);
    });
  if (ni > 0)
    c.launch("vxc_mixed", st, [&] {
      const int g = std::min(ni, ctas);
      launch_vxc(P, g, st, P.d_tabs, P.d_blocks, P.d_items, ni, ov, P.d_queue, err, P.tmap.rows32,
                 P.tmap.rows128, kVxcSplitPlanes);
    });
  c.launch("symmetrize", st, [&] {
    const size_t n2 = static_cast<size_t>(P.maxnbf) * P.maxnbf;
    const int gx = static_cast<int>(std::min<size_t>((n2 + 255) / 256, 1024));
    k_symmetrize<<<dim3(gx, nmol), 256, 0, st>>>(P.d_tabs, ov);
  });
  c.launch("reduce", st, [&] { k_reduce_b<<<nmol, 256, 0, st>>>(P.d_tabs, ov); });
  cuda_check(cudaGetLastError(), "kernel launch");
  if (P.ao_cacheable)
    P.ao_valid = true;
}

} // namespace

void Molecule::prepare_mixed() {
  MixedState *S = new MixedState();
  mixed = S;
  int lblock = 0;
  for (size_t li = 0; li < leaves.size(); li++) {
    const DevLeaf &L = leaves[li];
    const int mp = static_cast<int>(round_up(L.nbf, kKc));
    for (int p0 = 0; p0 < L.cnt; p0 += kBlockPts) {
      MBlock B;
      B.mol = 0;
      B.leaf = static_cast<int>(li);
      B.p0 = p0;
      B.cnt = std::min(kBlockPts, L.cnt - p0);
      B.mp = mp;
      B.lblock = lblock++;
      B.ws_off = static_cast<long long>(S->ws_floats);
      S->ws_floats += static_cast<size_t>(kPlanes) * mp * kBlockPts;
      S->blocks.push_back(B);
    }
  }
  // primitives as (alpha hi, alpha lo, c hi, c lo) float pairs, with OCC's
  // common_fac folded into c in FP64
  std::vector<float4> prim32, shA;
  for (const Shell &sh : basis.shells) {
    const double fac = common_fac(sh.l, basis.pure);
    for (size_t k = 0; k < sh.exps.size(); k++) {
      const double c = sh.coefs[k] * fac;
      const float ah = static_cast<float>(sh.exps[k]);
      const float ch = static_cast<float>(c);
      prim32.push_back(make_float4(ah, static_cast<float>(sh.exps[k] - ah), ch,
                                   static_cast<float>(c - ch)));
    }
    float h[3], l[3];
    for (int d = 0; d < 3; d++) {
      h[d] = static_cast<float>(sh.origin[d]);
      l[d] = static_cast<float>(sh.origin[d] - h[d]);
    }
    shA.push_back(make_float4(h[0], h[1], h[2], 0.f));
    shA.push_back(make_float4(l[0], l[1], l[2], 0.f));
  }
  auto up = [&](auto &vec, auto *&dptr) {
    using T = typename std::remove_reference<decltype(vec)>::type::value_type;
    dptr = static_cast<T *>(alloc(std::max<size_t>(vec.size(), 1) * sizeof(T)));
    if (!vec.empty())
      cuda_check(cudaMemcpy(dptr, vec.data(), vec.size() * sizeof(T), cudaMemcpyHostToDevice),
                 "cudaMemcpy H2D");
  };
  up(prim32, S->d_prim32);
  up(shA, S->d_shA);
  S->d_err = static_cast<int *>(alloc(sizeof(int)));
  cuda_check(cudaMemset(S->d_err, 0, sizeof(int)), "cudaMemset");
  MixTab &T = S->tab;
  T.m = dev();
  T.fs = fs;
  T.dens_thr = bs.density_threshold;
  T.prim32 = S->d_prim32;
  T.shA = S->d_shA;
  T.ws = nullptr;
  T.rowscale = nullptr;
  T.dhl = nullptr;
  T.colb = nullptr;
  T.rho = d_rho;
  T.coef = d_coef;
  T.epart = d_epart;
  T.D = d_D;
  T.V = d_V;
  T.out2 = d_out2;
  T.vxc_n = vxc_n;
  set_smem_attributes();
}

size_t Molecule::mixed_workspace_bytes() const { return ws_layout(*this).total; }

// Tensor map of a workspace region: rows of 128 FP32 (512 bytes), boxes of
// 32 x 32 with the 128-byte swizzle that the UMMA descriptors expect.
static void encode_ws_map_box(CUtensorMap &map, const void *base, size_t bytes,
                              uint32_t box_rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cuda_check(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                cudaEnableDefault, &q),
               "cudaGetDriverEntryPointByVersion");
    if (q != cudaDriverEntryPointSuccess || !fn)
      throw CudaError("cuTensorMapEncodeTiled is not available from the driver");
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t rows = std::max<cuuint64_t>(bytes / (kBlockPts * sizeof(float)), 1);
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(kBlockPts), rows};
  const cuuint64_t strides[1] = {kBlockPts * sizeof(float)};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(kKc), box_rows};
  const cuuint32_t estr[2] = {1u, 1u};
  const CUresult r = encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base),
                            dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw CudaError("cuTensorMapEncodeTiled failed (" + std::to_string(static_cast<int>(r)) + ")");
}

void encode_ws_map(WsMaps &map, const void *base, size_t bytes) {
  encode_ws_map_box(map.rows32, base, bytes, 32u);
  encode_ws_map_box(map.rows128, base, bytes, 128u);
}

void Molecule::ensure_mixed_ws() {
  MixedState *S = mixed;
  if (S->d_private)
    return;
  const size_t bytes = ws_layout(*this).total;
  S->d_private = static_cast<char *>(alloc(bytes));
  auto P = std::make_unique<LaunchPlan>();
  make_plan(*P, {this}, {bind_ws(*this, S->d_private, S->d_private)});
  P->ao_cacheable = true;
  encode_ws_map(P->tmap, S->d_private, bytes);
  S->single = std::move(P);
}

void Molecule::build_mixed(const double *dD, double *dV, double *dout2, cudaStream_t st) {
  if (deriv == 2) {
    build_mixed_mgga(dD, dV, dout2, st);
    return;
  }
  ensure_mixed_ws();
  run_plan(*mixed->single, *ctx, Override{dD, dV, dout2}, mixed->d_err, st,
           ctas > 0 ? ctas : ctx->max_ctas);
}

int mixed_error_flag(Molecule &M, cudaStream_t st) {
  if (!M.mixed)
    return 0;
  int h = 0;
  cuda_check(cudaMemcpyAsync(&h, M.mixed->d_err, sizeof(int), cudaMemcpyDeviceToHost, st),
             "cudaMemcpyAsync D2H");
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (h) // reported once; the next build starts clean
    cuda_check(cudaMemsetAsync(M.mixed->d_err, 0, sizeof(int), st), "cudaMemsetAsync");
  return h;
}

void set_wait_limit(int device, uint32_t polls) {
  int prev = 0;
  cuda_check(cudaGetDevice(&prev), "cudaGetDevice");
  cuda_check(cudaSetDevice(device), "cudaSetDevice");
  const cudaError_t e = cudaMemcpyToSymbol(g_wait_limit, &polls, sizeof(polls));
  cudaSetDevice(prev);
  cuda_check(e, "cudaMemcpyToSymbol");
}

void free_mixed(MixedState *S) { delete S; }

void ListArena::reserve(size_t bytes) {
  if (bytes <= cap)
    return;
  const size_t n = std::max(bytes, 2 * cap);
  if (d)
    cudaFree(d);
  if (h)
    cudaFreeHost(h);
  d = h = nullptr;
  cap = 0;
  cuda_check(cudaMalloc(&d, n), "cudaMalloc");
  cuda_check(cudaMallocHost(&h, n), "cudaMallocHost");
  cap = n;
}
ListArena::~ListArena() {
  if (d)
    cudaFree(d);
  if (h)
    cudaFreeHost(h);
}

// One launch sequence per functional family over molecules whose workspaces
// are already bound (tabs[i] for mols[i]) inside the region `map` covers.
void mixed_build_bound(Context &c, const std::vector<Molecule *> &mols,
                       const std::vector<MixTab> &bound, const WsMaps &map,
                       ListArena &arena, int *d_err, cudaStream_t st) {
  LaunchPlan P[2];
  std::vector<Molecule *> group[2];
  std::vector<MixTab> tabs[2];
  for (size_t i = 0; i < mols.size(); i++) {
    for (size_t j = 0; j < i; j++)
      if (mols[j] == mols[i])
        throw ArgError("a molecule may appear only once in a group build");
    const int g = mols[i]->deriv ? 1 : 0;
    group[g].push_back(mols[i]);
    tabs[g].push_back(bound[i]);
  }
  for (int g = 0; g < 2; g++)
    P[g].tmap = map;
  // pack both plans' lists into the arena: one pinned staging area, one copy
  size_t off = 0;
  auto place = [&](size_t bytes) {
    const size_t o = off;
    off = round_up(off + std::max<size_t>(bytes, 16), 256);
    return o;
  };
  struct Slot {
    size_t tabs, blocks, order, queue, items, litems;
  } slot[2]{};
  for (int g = 0; g < 2; g++) {
    if (group[g].empty())
      continue;
    make_plan_lists(P[g], group[g], tabs[g]);
    slot[g].tabs = place(P[g].tabs.size() * sizeof(MixTab));
    slot[g].blocks = place(P[g].blocks.size() * sizeof(MBlock));
    slot[g].order = place(P[g].order.size() * sizeof(int));
    slot[g].queue = place(2 * sizeof(int));
    slot[g].items = place(P[g].items.size() * sizeof(VItem));
    slot[g].litems = place(P[g].litems.size() * sizeof(LeafItem));
  }
  if (off == 0)
    return;
  arena.reserve(off);
  char *h = static_cast<char *>(arena.h);
  char *d = static_cast<char *>(arena.d);
  auto put = [&](size_t o, const void *src, size_t bytes) {
    if (bytes)
      std::memcpy(h + o, src, bytes);
  };
  for (int g = 0; g < 2; g++) {
    if (group[g].empty())
      continue;
    LaunchPlan &L = P[g];
    const int zero[2] = {0, 0};
    put(slot[g].tabs, L.tabs.data(), L.tabs.size() * sizeof(MixTab));
    put(slot[g].blocks, L.blocks.data(), L.blocks.size() * sizeof(MBlock));
    put(slot[g].order, L.order.data(), L.order.size() * sizeof(int));
    put(slot[g].queue, zero, sizeof(zero));
    put(slot[g].items, L.items.data(), L.items.size() * sizeof(VItem));
    put(slot[g].litems, L.litems.data(), L.litems.size() * sizeof(LeafItem));
    L.d_tabs = reinterpret_cast<MixTab *>(d + slot[g].tabs);
    L.d_blocks = reinterpret_cast<MBlock *>(d + slot[g].blocks);
    L.d_order = reinterpret_cast<int *>(d + slot[g].order);
    L.d_queue = reinterpret_cast<int *>(d + slot[g].queue);
    L.d_items = reinterpret_cast<VItem *>(d + slot[g].items);
    L.d_litems = reinterpret_cast<LeafItem *>(d + slot[g].litems);
  }
  cuda_check(cudaMemcpyAsync(d, h, off, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync H2D");
  for (int g = 0; g < 2; g++)
    if (!group[g].empty())
      run_plan(P[g], c, Override{nullptr, nullptr, nullptr}, d_err, st, c.max_ctas);
}

void mixed_build_group(Context &c, const std::vector<Molecule *> &mols, ListArena &arena,
                       char *d_ws, int *d_err, cudaStream_t st) {
  std::vector<MixTab> tabs;
  size_t wsoff = 0;
  for (Molecule *M : mols) {
    tabs.push_back(bind_ws(*M, d_ws + wsoff, d_ws));
    wsoff += M->mixed_workspace_bytes();
  }
  WsMaps map;
  encode_ws_map(map, d_ws, std::max<size_t>(wsoff, 512));
  mixed_build_bound(c, mols, tabs, map, arena, d_err, st);
}

void mixed_build_in_pool(Context &c, const std::vector<Molecule *> &mols,
                         const std::vector<char *> &ws, const std::vector<int> &ao_valid,
                         const char *pool, const WsMaps &pool_map, ListArena &arena,
                         int *d_err, cudaStream_t st) {
  std::vector<MixTab> tabs;
  for (size_t i = 0; i < mols.size(); i++) {
    MixTab T = bind_ws(*mols[i], ws[i], pool);
    T.ao_valid = ao_valid[i];
    tabs.push_back(T);
  }
  mixed_build_bound(c, mols, tabs, pool_map, arena, d_err, st);
}

size_t group_workspace_bytes(const std::vector<Molecule *> &mols) {
  size_t b = 0;
  for (const Molecule *M : mols)
    b += M->mixed_workspace_bytes();
  return b;
}

// ---- batches ---------------------------------------------------------------
// A batch owns one D, V and {E_xc, density} buffer per molecule and one
// shared mixed workspace.  Its molecules are split, in order, into
// sub-batches whose workspaces fit the cap; each sub-batch is one launch
// sequence per functional family (LDA, GGA) and the sub-batches run one
// after the other over the same workspace.
struct SubBatch {
  LaunchPlan plan[2];
};
struct Batch {
  std::vector<Molecule *> mols;
  std::vector<double *> dD, dV, dE;
  std::vector<std::unique_ptr<SubBatch>> subs;
  char *d_ws = nullptr;      // mixed workspace of the largest sub-batch
  size_t ws_bytes = 0;
  double *d_ws64 = nullptr;  // FP64 workspace (molecules built one at a time), on first use
  int *d_err = nullptr;
  bool fp64_only = false;    // holds a meta-GGA molecule: no tensor-core plans
  Context *ctx = nullptr;
  ~Batch() {
    for (double *p : dD)
      cudaFree(p);
    for (double *p : dV)
      cudaFree(p);
    for (double *p : dE)
      cudaFree(p);
    cudaFree(d_ws);
    cudaFree(d_ws64);
    cudaFree(d_err);
  }
};

Batch *batch_create(Context *ctx, const std::vector<Molecule *> &mols, double ws_cap) {
  auto B = std::make_unique<Batch>();
  B->ctx = ctx;
  B->mols = mols;
  for (size_t i = 0; i < mols.size(); i++)
    for (size_t j = 0; j < i; j++)
      if (mols[j] == mols[i])
        throw ArgError("a molecule may appear only once in a batch (its buffers are shared)");
  if (ws_cap <= 0) {
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    ws_cap = 0.5 * static_cast<double>(fr);
  }
  for (Molecule *M : mols) {
    const size_t n2 = std::max<size_t>(static_cast<size_t>(M->basis.nbf) * M->basis.nbf, 1);
    double *d = nullptr, *v = nullptr, *e = nullptr;
    cuda_check(cudaMalloc(&d, n2 * sizeof(double)), "cudaMalloc");
    B->dD.push_back(d);
    cuda_check(cudaMalloc(&v, n2 * sizeof(double)), "cudaMalloc");
    B->dV.push_back(v);
    cuda_check(cudaMalloc(&e, 2 * sizeof(double)), "cudaMalloc");
    B->dE.push_back(e);
  }
  for (Molecule *M : mols)
    B->fp64_only = B->fp64_only || M->deriv == 2;
  if (B->fp64_only) { // meta-GGA: FP64 builds only, no tensor-core workspace or plans
    cuda_check(cudaMalloc(&B->d_ws, 256), "cudaMalloc");
    cuda_check(cudaMalloc(&B->d_err, sizeof(int)), "cudaMalloc");
    cuda_check(cudaMemset(B->d_err, 0, sizeof(int)), "cudaMemset");
    return B.release();
  }
  // partition in order under the cap (a molecule above the cap goes alone)
  std::vector<std::vector<size_t>> parts;
  size_t cur = 0;
  for (size_t i = 0; i < mols.size(); i++) {
    const size_t w = mols[i]->mixed_workspace_bytes();
    if (parts.empty() || (cur + w > ws_cap && !parts.back().empty())) {
      parts.emplace_back();
      cur = 0;
    }
    parts.back().push_back(i);
    cur += w;
    B->ws_bytes = std::max(B->ws_bytes, cur);
  }
  cuda_check(cudaMalloc(&B->d_ws, std::max<size_t>(B->ws_bytes, 256)), "cudaMalloc");
  for (const auto &part : parts) {
    auto sb = std::make_unique<SubBatch>();
    std::vector<Molecule *> group[2];
    std::vector<MixTab> tabs[2];
    size_t off = 0;
    for (size_t i : part) {
      Molecule *M = mols[i];
      MixTab T = bind_ws(*M, B->d_ws + off, B->d_ws);
      off += M->mixed_workspace_bytes();
      T.D = B->dD[i];
      T.V = B->dV[i];
      T.out2 = B->dE[i];
      const int g = M->deriv ? 1 : 0;
      group[g].push_back(M);
      tabs[g].push_back(T);
    }
    for (int g = 0; g < 2; g++)
      if (!group[g].empty()) {
        make_plan(sb->plan[g], group[g], tabs[g]);
        sb->plan[g].ao_cacheable = parts.size() == 1; // else sub-batches share the space
        encode_ws_map(sb->plan[g].tmap, B->d_ws, std::max<size_t>(B->ws_bytes, 256));
      }
    B->subs.push_back(std::move(sb));
  }
  cuda_check(cudaMalloc(&B->d_err, sizeof(int)), "cudaMalloc");
  cuda_check(cudaMemset(B->d_err, 0, sizeof(int)), "cudaMemset");
  return B.release();
}

// Workspaces a build of `precision` needs (allocated outside any capture).
void batch_prepare(Batch &B, int precision) {
  if (precision == OCC_XC_FP64 && !B.d_ws64) {
    size_t w = 1;
    for (Molecule *M : B.mols)
      w = std::max(w, M->fp64_workspace_bytes());
    cuda_check(cudaMalloc(&B.d_ws64, w), "cudaMalloc");
  }
}

void batch_build(Batch &B, int precision, cudaStream_t st) {
  if (precision == OCC_XC_MIXED && B.fp64_only)
    throw ArgError("a batch with a meta-GGA molecule builds in FP64 only (OCC_XC_FP64)");
  if (precision == OCC_XC_MIXED) {
    for (auto &sb : B.subs)
      for (LaunchPlan &P : sb->plan)
        run_plan(P, *B.ctx, Override{nullptr, nullptr, nullptr}, B.d_err, st, B.ctx->max_ctas);
  } else {
    if (!B.d_ws64)
      throw ArgError("FP64 batch workspace missing (batch_prepare not called)");
    for (size_t i = 0; i < B.mols.size(); i++)
      B.mols[i]->build_fp64(B.dD[i], B.dV[i], B.dE[i], st, B.d_ws64);
  }
}

void batch_destroy(Batch *B) { delete B; }
void batch_buffers(Batch &B, int i, double **d, double **v, double **e) {
  *d = B.dD.at(i);
  *v = B.dV.at(i);
  *e = B.dE.at(i);
}
int batch_size(const Batch &B) { return static_cast<int>(B.mols.size()); }
int batch_error_flag(Batch &B, cudaStream_t st) {
  int h = 0;
  cuda_check(cudaMemcpyAsync(&h, B.d_err, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (h) // reported once; the next build starts clean
    cuda_check(cudaMemsetAsync(B.d_err, 0, sizeof(int), st), "cudaMemsetAsync");
  return h;
}

} // namespace occx

using namespace occx;

// C = A B^T for A[128][K], B[N][K] (row-major FP32, host buffers): one tile of
// the mixed path's tcgen05 pipeline, for testing it in isolation.  exact = 0:
// 3xTF32, N a multiple of 32 up to 256, K a multiple of 32.  exact = 1: the
// exact-grid split, N a multiple of 32 up to 128, K a multiple of 32 up to 512.
extern "C" int occ_xc_selftest_tf32_gemm(occ_xc_context *ctx, int exact, int N, int K,
                                         const float *A, const float *Bm, float *Cm) {
  const int nmax = exact ? kExactN : kMaxN;
  if (!ctx || !A || !Bm || !Cm || N <= 0 || N > nmax || N % 32 || K <= 0 || K % kKc ||
      (exact && K > kExactKSeg))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int *dErr = nullptr;
  int rc = OCC_XC_OK;
  try {
    cudaStream_t st = ctx->impl->stream;
    set_smem_attributes();
    cuda_check(cudaMalloc(&dA, sizeof(float) * 128 * K), "cudaMalloc");
    cuda_check(cudaMalloc(&dB, sizeof(float) * N * K), "cudaMalloc");
    cuda_check(cudaMalloc(&dC, sizeof(float) * 128 * N), "cudaMalloc");
    cuda_check(cudaMalloc(&dErr, sizeof(int)), "cudaMalloc");
    cuda_check(cudaMemcpy(dA, A, sizeof(float) * 128 * K, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(dB, Bm, sizeof(float) * N * K, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemset(dErr, 0, sizeof(int)), "memset");
    k_selftest_gemm<<<1, 256, kSmemTotal, st>>>(dA, dB, dC, N, K, exact, dErr);
    cuda_check(cudaGetLastError(), "launch");
    cuda_check(cudaStreamSynchronize(st), "sync");
    int herr = 0;
    cuda_check(cudaMemcpy(&herr, dErr, sizeof(int), cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(Cm, dC, sizeof(float) * 128 * N, cudaMemcpyDeviceToHost), "D2H");
    if (herr) {
      ctx->err = "tcgen05 pipeline wait timed out";
      rc = OCC_XC_ERR_TIMEOUT;
    }
  } catch (const std::exception &e) {
    ctx->err = e.what();
    rc = OCC_XC_ERR_CUDA;
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dErr);
  return rc;
}

// ---- batches and CUDA graphs (C ABI) ----------------------------------------
struct occ_xc_batch {
  occx::Batch *impl;
  occ_xc_context *ctx;
};
struct occ_xc_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int device = 0;
  cudaStream_t stream = nullptr; // the context's stream: where a NULL-stream launch goes
};

namespace {
template <typename F> int api_guard(occ_xc_context *ctx, F &&f) {
  try {
    f();
    return OCC_XC_OK;
  } catch (const MethodError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_METHOD;
  } catch (const ArgError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_ARG;
  } catch (const TimeoutError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_TIMEOUT;
  } catch (const CudaError &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_CUDA;
  } catch (const std::exception &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_INTERNAL;
  }
}

// Capture what `body` launches on a private stream into an instantiated graph.
template <typename F> occ_xc_graph *capture(Context &c, F &&body) {
  auto G = std::make_unique<occ_xc_graph>();
  G->device = c.device;
  G->stream = c.stream;
  cudaStream_t st;
  cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
  const bool prof = c.prof.on;
  c.prof.on = false; // no profiling events inside a graph
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    try {
      body(st);
    } catch (...) {
      cudaGraph_t g;
      cudaStreamEndCapture(st, &g);
      if (g)
        cudaGraphDestroy(g);
      cudaStreamDestroy(st);
      c.prof.on = prof;
      throw;
    }
    e = cudaStreamEndCapture(st, &G->graph);
  }
  c.prof.on = prof;
  cudaStreamDestroy(st);
  cuda_check(e, "stream capture");
  cuda_check(cudaGraphInstantiate(&G->exec, G->graph, 0), "cudaGraphInstantiate");
  return G.release();
}
} // namespace

extern "C" {

int occ_xc_batch_create_capped(occ_xc_context *ctx, int nmol, occ_xc_molecule *const *mols,
                               double workspace_cap_bytes, occ_xc_batch **out) {
  if (!ctx || !out || nmol <= 0 || !mols)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  *out = nullptr;
  return api_guard(ctx, [&] {
    std::vector<Molecule *> ms;
    for (int i = 0; i < nmol; i++) {
      if (!mols[i] || mols[i]->ctx != ctx)
        throw ArgError("every molecule of a batch must belong to the batch's context");
      ms.push_back(mols[i]->impl.get());
    }
    cuda_check(cudaSetDevice(ctx->impl->device), "cudaSetDevice");
    auto b = std::make_unique<occ_xc_batch>();
    b->ctx = ctx;
    b->impl = batch_create(ctx->impl.get(), ms, workspace_cap_bytes);
    *out = b.release();
  });
}

int occ_xc_batch_create(occ_xc_context *ctx, int nmol, occ_xc_molecule *const *mols,
                        occ_xc_batch **out) {
  return occ_xc_batch_create_capped(ctx, nmol, mols, 0.0, out);
}

void occ_xc_batch_destroy(occ_xc_batch *b) {
  if (!b)
    return;
  batch_destroy(b->impl);
  delete b;
}

int occ_xc_batch_buffers(occ_xc_batch *b, int i, double **d_D, double **d_V, double **d_exc2) {
  if (!b || !d_D || !d_V || !d_exc2 || i < 0 || i >= batch_size(*b->impl))
    return OCC_XC_ERR_ARG;
  batch_buffers(*b->impl, i, d_D, d_V, d_exc2);
  return OCC_XC_OK;
}

int occ_xc_batch_compute(occ_xc_context *ctx, occ_xc_batch *b, int precision, void *stream) {
  if (!ctx || !b || (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->impl->stream;
    batch_prepare(*b->impl, precision);
    batch_build(*b->impl, precision, st);
  });
}

int occ_xc_batch_check(occ_xc_context *ctx, occ_xc_batch *b, void *stream) {
  if (!ctx || !b)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->impl->stream;
    if (batch_error_flag(*b->impl, st))
      throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
  });
}

int occ_xc_graph_capture(occ_xc_context *ctx, occ_xc_molecule *mol, int precision, int niter,
                         const double *const *d_D, double *const *d_V,
                         double *const *d_exc2, occ_xc_graph **out) {
  if (!ctx || !mol || !out || niter <= 0 || !d_D || !d_V || !d_exc2 ||
      (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  *out = nullptr;
  return api_guard(ctx, [&] {
    cuda_check(cudaSetDevice(ctx->impl->device), "cudaSetDevice");
    mol->impl->prepare(precision); // workspaces are allocated outside the capture
    *out = capture(*ctx->impl, [&](cudaStream_t st) {
      for (int k = 0; k < niter; k++)
        mol->impl->build(precision, d_D[k], d_V[k], d_exc2[k], st);
    });
  });
}

int occ_xc_batch_graph_capture(occ_xc_context *ctx, occ_xc_batch *b, int precision,
                               occ_xc_graph **out) {
  if (!ctx || !b || !out || (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  *out = nullptr;
  return api_guard(ctx, [&] {
    cuda_check(cudaSetDevice(ctx->impl->device), "cudaSetDevice");
    batch_prepare(*b->impl, precision);
    *out = capture(*ctx->impl, [&](cudaStream_t st) { batch_build(*b->impl, precision, st); });
  });
}

int occ_xc_graph_launch(occ_xc_graph *g, void *stream) {
  if (!g || !g->exec)
    return OCC_XC_ERR_ARG;
  cudaError_t e = cudaGraphLaunch(g->exec, stream ? static_cast<cudaStream_t>(stream) : g->stream);
  return e == cudaSuccess ? OCC_XC_OK : OCC_XC_ERR_CUDA;
}

void occ_xc_graph_destroy(occ_xc_graph *g) {
  if (!g)
    return;
  cudaSetDevice(g->device);
  if (g->exec)
    cudaGraphExecDestroy(g->exec);
  if (g->graph)
    cudaGraphDestroy(g->graph);
  delete g;
}

int occ_xc_set_persistent_ctas(occ_xc_context *ctx, int ctas) {
  if (!ctx || ctas < 0)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->impl->max_ctas = ctas;
  return OCC_XC_OK;
}

int occ_xc_set_wait_limit(occ_xc_context *ctx, unsigned int polls) {
  if (!ctx)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  try {
    set_wait_limit(ctx->impl->device, polls);
  } catch (const std::exception &e) {
    ctx->err = e.what();
    return OCC_XC_ERR_CUDA;
  }
  return OCC_XC_OK;
}

} // extern "C"

extern "C" int occ_xc_batch_compute_host(occ_xc_context *ctx, occ_xc_batch *b, int precision,
                                         const double *const *D, double *const *V, double *exc,
                                         double *nelec) {
  if (!ctx || !b || !D || !V || !exc || (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    Batch &B = *b->impl;
    cudaStream_t st = ctx->impl->stream;
    for (size_t i = 0; i < B.mols.size(); i++) {
      const size_t n2 = static_cast<size_t>(B.mols[i]->basis.nbf) * B.mols[i]->basis.nbf;
      cuda_check(cudaMemcpyAsync(B.dD[i], D[i], n2 * sizeof(double), cudaMemcpyHostToDevice, st),
                 "H2D");
    }
    batch_prepare(B, precision);
    batch_build(B, precision, st);
    std::vector<double> e2(2 * B.mols.size());
    for (size_t i = 0; i < B.mols.size(); i++) {
      const size_t n2 = static_cast<size_t>(B.mols[i]->basis.nbf) * B.mols[i]->basis.nbf;
      cuda_check(cudaMemcpyAsync(V[i], B.dV[i], n2 * sizeof(double), cudaMemcpyDeviceToHost, st),
                 "D2H");
      cuda_check(cudaMemcpyAsync(&e2[2 * i], B.dE[i], 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                 st), "D2H");
    }
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (precision == OCC_XC_MIXED && batch_error_flag(B, st))
      throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
    for (size_t i = 0; i < B.mols.size(); i++) {
      exc[i] = e2[2 * i];
      if (nelec)
        nelec[i] = e2[2 * i + 1];
    }
  });
}

extern "C" int occ_xc_batch_set_density(occ_xc_context *ctx, occ_xc_batch *b, int i,
                                        const double *D) {
  if (!ctx || !b || !D || i < 0 || i >= batch_size(*b->impl))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    Batch &B = *b->impl;
    const size_t n2 = static_cast<size_t>(B.mols[i]->basis.nbf) * B.mols[i]->basis.nbf;
    cudaStream_t st = ctx->impl->stream;
    cuda_check(cudaMemcpyAsync(B.dD[i], D, n2 * sizeof(double), cudaMemcpyHostToDevice, st),
               "H2D");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  });
}

extern "C" int occ_xc_batch_get_result(occ_xc_context *ctx, occ_xc_batch *b, int i, double *V,
                                       double *exc2) {
  if (!ctx || !b || !V || !exc2 || i < 0 || i >= batch_size(*b->impl))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    Batch &B = *b->impl;
    const size_t n2 = static_cast<size_t>(B.mols[i]->basis.nbf) * B.mols[i]->basis.nbf;
    cudaStream_t st = ctx->impl->stream;
    cuda_check(cudaMemcpyAsync(V, B.dV[i], n2 * sizeof(double), cudaMemcpyDeviceToHost, st),
               "D2H");
    cuda_check(cudaMemcpyAsync(exc2, B.dE[i], 2 * sizeof(double), cudaMemcpyDeviceToHost, st),
               "D2H");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  });
}

namespace occx {
namespace {
// f2: the build's evaluator (eval_xc_mixed_f2 on inputs split by
// fn::f2_bits) instead of eval_xc_mixed.
__global__ void k_selftest_func(FuncSet fs, int n, const double *rho, const double *sigma,
                                double *out64, double *outm, int f2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  double e, vr, vs;
  eval_xc(fs, rho[i], sigma[i], e, vr, vs);
  out64[3 * i] = e;
  out64[3 * i + 1] = vr;
  out64[3 * i + 2] = vs;
  if (f2) {
    bool gga = false;
    for (int k = 0; k < fs.n; k++)
      gga = gga || func_is_gga(fs.id[k]);
    fn::F2 ef;
    float vrf, vsf;
    if (eval_xc_mixed_f2(fs, gga, fn::f2_bits(rho[i]), fn::f2_bits(sigma[i]), ef, vrf, vsf)) {
      e = fn::to_d(ef);
      vr = vrf;
      vs = vsf;
    } // else: FP64 on the FP64 inputs, e, vr, vs as above
  } else {
    eval_xc_mixed(fs, rho[i], sigma[i], e, vr, vs);
  }
  outm[3 * i] = e;
  outm[3 * i + 1] = vr;
  outm[3 * i + 2] = vs;
}
__global__ void k_selftest_pol(FuncSet fs, int n, const double *in5, double *out64,
                               double *outm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const double ra = in5[i], rb = in5[n + i], saa = in5[2 * n + i], sab = in5[3 * n + i],
               sbb = in5[4 * n + i];
  eval_xc_pol(fs, ra, rb, saa, sab, sbb, out64[6 * i], out64 + 6 * i + 1, out64 + 6 * i + 3);
  eval_xc_pol_mixed(fs, ra, rb, saa, sab, sbb, outm[6 * i], outm + 6 * i + 1, outm + 6 * i + 3);
}
__global__ void k_selftest_mgga(FuncSet fs, int n, const double *rho, const double *sigma,
                                const double *tau, double *out64, double *outm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  double e, vr, vs, vt;
  eval_xc_mgga(fs, rho[i], sigma[i], tau[i], e, vr, vs, vt);
  out64[4 * i] = e;
  out64[4 * i + 1] = vr;
  out64[4 * i + 2] = vs;
  out64[4 * i + 3] = vt;
  eval_xc_mgga_mixed(fs, rho[i], sigma[i], tau[i], e, vr, vs, vt);
  outm[4 * i] = e;
  outm[4 * i + 1] = vr;
  outm[4 * i + 2] = vs;
  outm[4 * i + 3] = vt;
}
} // namespace
} // namespace occx

// The polarised evaluators (FP64 and the tensor-core build's) at n points:
// in5 = rho_a, rho_b, s_aa, s_ab, s_bb (n each); out64 / outm receive e,
// vrho_a, vrho_b, vs_aa, vs_ab, vs_bb per point.  For testing.
extern "C" int occ_xc_selftest_functional_pol(occ_xc_context *ctx, const char *method, int n,
                                              const double *in5, double *out64, double *outm) {
  if (!ctx || !method || n <= 0 || !in5 || !out64 || !outm)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    const FuncSet fs = parse_method(method);
    cudaStream_t st = ctx->impl->stream;
    double *d = nullptr;
    cuda_check(cudaMalloc(&d, static_cast<size_t>(n) * 17 * sizeof(double)), "cudaMalloc");
    try {
      cuda_check(cudaMemcpyAsync(d, in5, 5 * static_cast<size_t>(n) * sizeof(double),
                                 cudaMemcpyHostToDevice, st), "H2D");
      k_selftest_pol<<<(n + 127) / 128, 128, 0, st>>>(fs, n, d, d + 5 * n, d + 11 * n);
      cuda_check(cudaGetLastError(), "kernel launch");
      cuda_check(cudaMemcpyAsync(out64, d + 5 * n, 6 * static_cast<size_t>(n) * sizeof(double),
                                 cudaMemcpyDeviceToHost, st), "D2H");
      cuda_check(cudaMemcpyAsync(outm, d + 11 * n, 6 * static_cast<size_t>(n) * sizeof(double),
                                 cudaMemcpyDeviceToHost, st), "D2H");
      cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    } catch (...) {
      cudaFree(d);
      throw;
    }
    cudaFree(d);
  });
}

// The meta-GGA evaluators (FP64 and the tensor-core path's) at n points
// (host arrays; out64 / outm receive e, vrho, vsigma, vtau per point), for
// testing.
extern "C" int occ_xc_selftest_functional_mgga(occ_xc_context *ctx, const char *method, int n,
                                               const double *rho, const double *sigma,
                                               const double *tau, double *out64, double *outm) {
  if (!ctx || !method || n <= 0 || !rho || !sigma || !tau || !out64 || !outm)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    const FuncSet fs = parse_method(method);
    cudaStream_t st = ctx->impl->stream;
    double *d = nullptr;
    const size_t bytes = static_cast<size_t>(n) * 11 * sizeof(double);
    cuda_check(cudaMalloc(&d, bytes), "cudaMalloc");
    try {
      const double *src[3] = {rho, sigma, tau};
      for (int k = 0; k < 3; k++)
        cuda_check(cudaMemcpyAsync(d + k * n, src[k], n * sizeof(double), cudaMemcpyHostToDevice,
                                   st),
                   "H2D");
      k_selftest_mgga<<<(n + 127) / 128, 128, 0, st>>>(fs, n, d, d + n, d + 2 * n, d + 3 * n,
                                                       d + 7 * n);
      cuda_check(cudaGetLastError(), "kernel launch");
      cuda_check(cudaMemcpyAsync(out64, d + 3 * n, 4 * n * sizeof(double),
                                 cudaMemcpyDeviceToHost, st), "D2H");
      cuda_check(cudaMemcpyAsync(outm, d + 7 * n, 4 * n * sizeof(double), cudaMemcpyDeviceToHost,
                                 st), "D2H");
      cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    } catch (...) {
      cudaFree(d);
      throw;
    }
    cudaFree(d);
  });
}

namespace {
int selftest_functional(occ_xc_context *ctx, const char *method, int n, const double *rho,
                        const double *sigma, double *out64, double *outm, int f2);
}

// The FP64 and the mixed-path functional evaluators at n points (host
// arrays; out64 / outm receive e, vrho, vsigma per point), for testing:
// eval_xc_mixed (the gradient's and the unrestricted builds' functional
// stage) and, with _f2, eval_xc_mixed_f2 (the restricted build's).
extern "C" int occ_xc_selftest_functional(occ_xc_context *ctx, const char *method, int n,
                                          const double *rho, const double *sigma,
                                          double *out64, double *outm) {
  return selftest_functional(ctx, method, n, rho, sigma, out64, outm, 0);
}
extern "C" int occ_xc_selftest_functional_f2(occ_xc_context *ctx, const char *method, int n,
                                             const double *rho, const double *sigma,
                                             double *out64, double *outm) {
  return selftest_functional(ctx, method, n, rho, sigma, out64, outm, 1);
}

namespace {
int selftest_functional(occ_xc_context *ctx, const char *method, int n, const double *rho,
                        const double *sigma, double *out64, double *outm, int f2) {
  if (!ctx || !method || n <= 0 || !rho || !sigma || !out64 || !outm)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return api_guard(ctx, [&] {
    const FuncSet fs = parse_method(method);
    cudaStream_t st = ctx->impl->stream;
    double *d = nullptr;
    const size_t bytes = static_cast<size_t>(n) * 8 * sizeof(double);
    cuda_check(cudaMalloc(&d, bytes), "cudaMalloc");
    try {
      cuda_check(cudaMemcpyAsync(d, rho, n * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
      cuda_check(cudaMemcpyAsync(d + n, sigma, n * sizeof(double), cudaMemcpyHostToDevice, st),
                 "H2D");
      k_selftest_func<<<(n + 127) / 128, 128, 0, st>>>(fs, n, d, d + n, d + 2 * n, d + 5 * n,
                                                       f2);
      cuda_check(cudaGetLastError(), "kernel launch");
      cuda_check(cudaMemcpyAsync(out64, d + 2 * n, 3 * n * sizeof(double),
                                 cudaMemcpyDeviceToHost, st), "D2H");
      cuda_check(cudaMemcpyAsync(outm, d + 5 * n, 3 * n * sizeof(double), cudaMemcpyDeviceToHost,
                                 st), "D2H");
      cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    } catch (...) {
      cudaFree(d);
      throw;
    }
    cudaFree(d);
  });
}
} // namespace

// ---- XC nuclear gradient on the tensor cores ------------------------------
// DFT::compute_xc_gradient (include/occ/dft/dft.h:599-749) as
//   G_c(mu, nu) = sum_p d_c phi_mu Y_nu + Z_c,mu phi_nu   (c = x, y, z)
//   g_A,c = - sum_{mu on A} sum_nu 4 D(mu, nu) G_c(mu, nu), |4 D| < 1e-12 skipped
// (src/dft/dft_gradient_kernels.cpp:472-595): the three G_c are the V_xc
// kernel's K with two operand pairs each, accumulated over the leaves into
// nbf x nbf FP64 matrices, then contracted with D.  The blocks carry, beside
// the build's eight planes, the FP32 planes of
//   Z_c = 0.5 w vrho d_c phi + 2 w vsigma grad rho . grad d_c phi
// (k_grad_ops, with the AO second derivatives in FP32); the pairs
// (d_c phi, Y) and (Z_c, phi) are read as FP32 planes (d_c phi and phi the
// collocation's, Y written unsplit by the functional stage) and split into
// TF32 hi / lo by the V_xc kernel.
namespace occx {

constexpr int kPlaneZ = kPlanes; // Z_c as FP32: planes 8 + c (d_c phi: the collocation's 1 + c)
constexpr int kPlanesGrad = kPlaneZ + 3;
// the meta-GGA plan's planes (its build and gradient share one workspace):
// after the tau density's A slices (kPlaneTauA, 9 planes)
constexpr int kPlaneMetaT = kPlaneTauA + 9; // t_k = c_tau d_k phi (FP32): planes 17 + (k-1)
constexpr int kPlaneMetaZ = kPlaneMetaT + 3; // Z_c (FP32, the gradient): planes 20 + c
constexpr int kPlaneMetaH = kPlaneMetaZ + 3; // 2 d_c d_k phi (FP32): xx, xy, xz, yy, yz, zz
constexpr int kPlanesMeta = kPlaneMetaH + 6;
// index of d_c d_k among xx, xy, xz, yy, yz, zz
__host__ __device__ constexpr int hess_index(int c, int k) {
  return c <= k ? (c == 0 ? k : (c == 1 ? 2 + k : 5)) : hess_index(k, c);
}

namespace {

// sum_k cg_k d_c d_k of the Cartesian functions of one shell (CCA order), for
// c = x, y, z, from
// d_ij (M R) = M_ij R + (M_i x_j + M_j x_i) dR + M (delta_ij dR + x_i x_j d2R)
template <int L>
__device__ __forceinline__ void cart_hess_dot_f32(float x, float y, float z, float R, float dR,
                                                  float d2R, const float *cg, float (*hz)[3]) {
  float px[L + 1], py[L + 1], pz[L + 1];
  px[0] = py[0] = pz[0] = 1.f;
#pragma unroll
  for (int i = 1; i <= L; i++) {
    px[i] = px[i - 1] * x;
    py[i] = py[i - 1] * y;
    pz[i] = pz[i - 1] * z;
  }
  const float r[3] = {x, y, z};
  int k = 0;
#pragma unroll
  for (int a = L; a >= 0; a--) {
#pragma unroll
    for (int b = L - a; b >= 0; b--) {
      const int c = L - a - b;
      const int e[3] = {a, b, c};
      const float *pp[3] = {px, py, pz};
      const float M = px[a] * py[b] * pz[c];
      float Mi[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const int o1 = (i + 1) % 3, o2 = (i + 2) % 3;
        Mi[i] = e[i] > 0 ? e[i] * pp[i][e[i] > 0 ? e[i] - 1 : 0] * pp[o1][e[o1]] * pp[o2][e[o2]]
                         : 0.f;
      }
      float H[3][3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = i; j < 3; j++) {
          float Mij;
          if (i == j) {
            const int o1 = (i + 1) % 3, o2 = (i + 2) % 3;
            Mij = e[i] > 1 ? e[i] * (e[i] - 1) * pp[i][e[i] > 1 ? e[i] - 2 : 0] * pp[o1][e[o1]] *
                                 pp[o2][e[o2]]
                           : 0.f;
          } else {
            const int l3 = 3 - i - j;
            Mij = (e[i] > 0 && e[j] > 0)
                      ? e[i] * e[j] * pp[i][e[i] > 0 ? e[i] - 1 : 0] *
                            pp[j][e[j] > 0 ? e[j] - 1 : 0] * pp[l3][e[l3]]
                      : 0.f;
          }
          const float h = Mij * R + (Mi[i] * r[j] + Mi[j] * r[i]) * dR +
                          M * ((i == j ? dR : 0.f) + r[i] * r[j] * d2R);
          H[i][j] = h;
          H[j][i] = h;
        }
      }
#pragma unroll
      for (int cc = 0; cc < 3; cc++)
        hz[k][cc] = fmaf(cg[0], H[cc][0], fmaf(cg[1], H[cc][1], cg[2] * H[cc][2]));
      k++;
    }
  }
}

// The six second derivatives (xx, xy, xz, yy, yz, zz) of the Cartesian
// functions of one shell (CCA order), by the same formula as
// cart_hess_dot_f32.
template <int L>
__device__ __forceinline__ void cart_hess6_f32(float x, float y, float z, float R, float dR,
                                               float d2R, float (*h6)[6]) {
  float px[L + 1], py[L + 1], pz[L + 1];
  px[0] = py[0] = pz[0] = 1.f;
#pragma unroll
  for (int i = 1; i <= L; i++) {
    px[i] = px[i - 1] * x;
    py[i] = py[i - 1] * y;
    pz[i] = pz[i - 1] * z;
  }
  const float r[3] = {x, y, z};
  int k = 0;
#pragma unroll
  for (int a = L; a >= 0; a--) {
#pragma unroll
    for (int b = L - a; b >= 0; b--) {
      const int c = L - a - b;
      const int e[3] = {a, b, c};
      const float *pp[3] = {px, py, pz};
      const float M = px[a] * py[b] * pz[c];
      float Mi[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const int o1 = (i + 1) % 3, o2 = (i + 2) % 3;
        Mi[i] = e[i] > 0 ? e[i] * pp[i][e[i] > 0 ? e[i] - 1 : 0] * pp[o1][e[o1]] * pp[o2][e[o2]]
                         : 0.f;
      }
#pragma unroll
      for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = i; j < 3; j++) {
          float Mij;
          if (i == j) {
            const int o1 = (i + 1) % 3, o2 = (i + 2) % 3;
            Mij = e[i] > 1 ? e[i] * (e[i] - 1) * pp[i][e[i] > 1 ? e[i] - 2 : 0] * pp[o1][e[o1]] *
                                 pp[o2][e[o2]]
                           : 0.f;
          } else {
            const int l3 = 3 - i - j;
            Mij = (e[i] > 0 && e[j] > 0)
                      ? e[i] * e[j] * pp[i][e[i] > 0 ? e[i] - 1 : 0] *
                            pp[j][e[j] > 0 ? e[j] - 1 : 0] * pp[l3][e[l3]]
                      : 0.f;
          }
          h6[k][hess_index(i, j)] = Mij * R + (Mi[i] * r[j] + Mi[j] * r[i]) * dR +
                                    M * ((i == j ? dR : 0.f) + r[i] * r[j] * d2R);
        }
      }
      k++;
    }
  }
}

// The meta-GGA gradient's operand planes of one shell: Z_c (as grad_ops_shell
// forms it) into kPlaneMetaZ + c and twice the AO Hessian into kPlaneMetaH.
template <int L>
__device__ __forceinline__ void grad_ops_shell_meta(bool pure, float x, float y, float z,
                                                    float R, float dR, float d2R, bool valid,
                                                    float c0, const float *cg, float *out,
                                                    size_t plane) {
  constexpr int NC = ncart_of(L);
  constexpr int NF = 2 * L + 1 > NC ? 2 * L + 1 : NC;
  float h6[NC][6];
  cart_hess6_f32<L>(x, y, z, R, dR, d2R, h6);
  const int nf = pure ? 2 * L + 1 : NC;
#pragma unroll
  for (int f = 0; f < NF; f++) {
    if (f >= nf)
      continue;
    float hf[6];
    if (!pure || L == 0) {
#pragma unroll
      for (int q = 0; q < 6; q++)
        hf[q] = h6[f < NC ? f : 0][q];
    } else {
      const float *Tm = c_spht + sph_offset(L) + f * NC;
      const float2 n = c_sphn[L * L + f];
#pragma unroll
      for (int q = 0; q < 6; q++) {
        float a = 0.f;
#pragma unroll
        for (int kk = 0; kk < NC; kk++)
          a = fmaf(Tm[kk], h6[kk][q], a);
        hf[q] = fmaf(n.x, a, n.y * a);
      }
    }
    const size_t o = static_cast<size_t>(f) * kBlockPts;
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
      const float dphi = out[(1 + cc) * plane + o];
      const float zh = fmaf(cg[0], hf[hess_index(cc, 0)],
                            fmaf(cg[1], hf[hess_index(cc, 1)], cg[2] * hf[hess_index(cc, 2)]));
      out[(kPlaneMetaZ + cc) * plane + o] = valid ? fmaf(c0, dphi, zh) : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 6; q++)
      out[(kPlaneMetaH + q) * plane + o] = valid ? 2.f * hf[q] : 0.f;
  }
}

template <int L>
__device__ __forceinline__ void grad_ops_shell(bool pure, float x, float y, float z, float R,
                                               float dR, float d2R, bool valid, float c0,
                                               const float *cg, float *out, size_t plane) {
  constexpr int NC = ncart_of(L);
  constexpr int NF = 2 * L + 1 > NC ? 2 * L + 1 : NC;
  float hz[NC][3];
  cart_hess_dot_f32<L>(x, y, z, R, dR, d2R, cg, hz);
  const int nf = pure ? 2 * L + 1 : NC;
#pragma unroll
  for (int f = 0; f < NF; f++) { // compile-time bound keeps hz in registers
    if (f >= nf)
      continue;
    float zh[3];
    if (!pure || L == 0) {
#pragma unroll
      for (int cc = 0; cc < 3; cc++)
        zh[cc] = hz[f < NC ? f : 0][cc];
    } else {
      const float *Tm = c_spht + sph_offset(L) + f * NC;
      const float2 n = c_sphn[L * L + f];
#pragma unroll
      for (int cc = 0; cc < 3; cc++) {
        float a = 0.f;
#pragma unroll
        for (int kk = 0; kk < NC; kk++)
          a = fmaf(Tm[kk], hz[kk][cc], a);
        zh[cc] = fmaf(n.x, a, n.y * a);
      }
    }
    const size_t o = static_cast<size_t>(f) * kBlockPts;
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
      const float dphi = out[(1 + cc) * plane + o];
      const float zc = fmaf(c0, dphi, zh[cc]);
      out[(kPlaneZ + cc) * plane + o] = valid ? zc : 0.f;
    }
  }
}

// One CTA of 128 threads (one point each) per block, after the functional
// stage: the gradient operand planes from the collocation's d_c phi, the
// functional's coefficients and the AO second derivatives.
template <bool META = false>
__global__ void __launch_bounds__(128) k_grad_ops(const MixTab *__restrict__ tabs,
                                                 const MBlock *__restrict__ blocks, int deriv) {
  const MBlock B = blocks[blockIdx.x];
  const MixTab &T = tabs[B.mol];
  const MolDev m = T.m;
  const float4 *__restrict__ prim32 = T.prim32;
  const float4 *__restrict__ shA = T.shA;
  const DevLeaf L = m.leaves[B.leaf];
  const int p = threadIdx.x;
  const bool valid = p < B.cnt;
  const size_t plane = static_cast<size_t>(B.mp) * kBlockPts;
  float *base = T.ws + B.ws_off;
  const size_t N = static_cast<size_t>(m.npts);
  const size_t gp = static_cast<size_t>(L.off) + B.p0 + (valid ? p : 0);
  const float c0 = valid ? static_cast<float>(T.coef[gp]) : 0.f;
  float cg[3] = {0.f, 0.f, 0.f};
  if (deriv && valid)
#pragma unroll
    for (int k = 0; k < 3; k++)
      cg[k] = static_cast<float>(T.coef[(k + 1) * N + gp]);
  const Pt4 P = valid ? m.pts[gp] : make_pt4(0.0, 0.0, 0.0, 0.0);
  const float pxh = static_cast<float>(P.x), pyh = static_cast<float>(P.y),
              pzh = static_cast<float>(P.z);
  const float pxl = static_cast<float>(P.x - pxh), pyl = static_cast<float>(P.y - pyh),
              pzl = static_cast<float>(P.z - pzh);
  int loc = 0;
  for (int k = L.sh_begin; k < L.sh_end; k++) {
    const int si = m.leaf_sh[k];
    const DevShell sh = m.shells[si];
    const float4 ah = shA[2 * si], al = shA[2 * si + 1];
    float x, y, z, xl, yl, zl;
    df_sub(pxh, pxl, ah.x, al.x, x, xl);
    df_sub(pyh, pyl, ah.y, al.y, y, yl);
    df_sub(pzh, pzl, ah.z, al.z, z, zl);
    // r^2 and alpha r^2 as double-float pairs, as the collocation forms them
    float r2h, r2l;
    {
      const float p1 = __fmul_rn(x, x), p2 = __fmul_rn(y, y), p3 = __fmul_rn(z, z);
      const float q = (fmaf(x, x, -p1) + fmaf(y, y, -p2) + fmaf(z, z, -p3)) +
                      2.f * (x * xl + y * yl + z * zl);
      float s12, e12, e3;
      two_sum(p1, p2, s12, e12);
      two_sum(s12, p3, r2h, e3);
      r2l = (e12 + e3) + q;
    }
    float R = 0.f, dR = 0.f, d2R = 0.f;
    for (int q = 0; q < sh.nprim; q++) {
      const float4 pc = prim32[sh.prim_off + q]; // alpha hi, alpha lo, c hi, c lo
      const float th = __fmul_rn(pc.x, r2h);
      const float tl = fmaf(pc.x, r2h, -th) + fmaf(pc.x, r2l, pc.y * r2h);
      const float e0 = exp_neg(th);
      const float ex = fmaf(-e0, tl, e0);
      const float e = fmaf(pc.z, ex, pc.w * ex);
      const float a = pc.x + pc.y;
      R += e;
      dR = fmaf(-2.f * a, e, dR);
      d2R = fmaf(4.f * a * a, e, d2R);
    }
    float *out = base + static_cast<size_t>(loc) * kBlockPts + p;
    if (META) {
      switch (sh.l) {
      case 0: grad_ops_shell_meta<0>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      case 1: grad_ops_shell_meta<1>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      case 2: grad_ops_shell_meta<2>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      case 3: grad_ops_shell_meta<3>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      default: grad_ops_shell_meta<4>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      }
    } else {
      switch (sh.l) {
      case 0: grad_ops_shell<0>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      case 1: grad_ops_shell<1>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      case 2: grad_ops_shell<2>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      case 3: grad_ops_shell<3>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      default: grad_ops_shell<4>(m.pure, x, y, z, R, dR, d2R, valid, c0, cg, out, plane); break;
      }
    }
    loc += sh.nfunc;
  }
  for (int f = loc; f < B.mp; f++) {
    const size_t o = static_cast<size_t>(f) * kBlockPts + p;
    if (META) {
#pragma unroll
      for (int q = kPlaneMetaZ; q < kPlanesMeta; q++)
        base[q * plane + o] = 0.f;
    } else {
#pragma unroll
      for (int q = kPlaneZ; q < kPlanesGrad; q++)
        base[q * plane + o] = 0.f;
    }
  }
}

// g[atom(mu)][c] -= sum_nu 4 D(mu, nu) G_c(mu, nu), |4 D| < 1e-12 skipped
// (dft_gradient_kernels.cpp:535-547).  One CTA per row mu.
__global__ void __launch_bounds__(256) k_grad_contract(const double *__restrict__ D,
                                                       const double *__restrict__ G, int nbf,
                                                       const int *__restrict__ ao_atom,
                                                       double *__restrict__ grad,
                                                       const double *__restrict__ Dot) {
  __shared__ double sh[8];
  const int mu = blockIdx.x;
  const size_t n2 = static_cast<size_t>(nbf) * nbf;
  double s[3] = {0.0, 0.0, 0.0};
  for (int nu = threadIdx.x; nu < nbf; nu += 256) {
    const size_t o = static_cast<size_t>(nu) * nbf + mu;
    const double d4 = 4.0 * D[o];
    // the reference's skip: |4 D| restricted, |2 (D_a + D_b)| unrestricted
    if (fabs(Dot ? 2.0 * (D[o] + Dot[o]) : d4) < 1e-12)
      continue;
#pragma unroll
    for (int c = 0; c < 3; c++)
      s[c] = fma(d4, G[c * n2 + o], s[c]);
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double t = leaf_sum256(s[c], sh);
    if (threadIdx.x == 0)
      atomicAdd(&grad[3 * ao_atom[mu] + c], -t);
  }
}

} // namespace

struct GradMixed {
  char *ws = nullptr;
  size_t bytes = 0;
  LaunchPlan plan;
  double *G = nullptr;
  int *ao_atom = nullptr;
  void *d_tab_b = nullptr; // the plan's table with the beta rho / coef arrays (UKS)
};

void free_grad_mixed(GradMixed *g) { delete g; }

void Molecule::prepare_gradient_mixed() {
  if (gmixed)
    return;
  if (!mixed)
    throw ArgError("the molecule has no device state");
  auto g = std::make_unique<GradMixed>();
  if (deriv == 2) {
    // the meta-GGA plan's workspace carries the gradient's planes too
    prepare_mgga_mixed();
    grad_tables(*g);
    gmixed = g.release();
    return;
  }
  const WsLayout Lw = ws_layout(*this, kPlanesGrad);
  g->bytes = Lw.total;
  g->ws = static_cast<char *>(alloc(g->bytes));
  LaunchPlan &P = g->plan;
  make_plan_lists(P, {this}, {bind_ws(*this, g->ws, g->ws, kPlanesGrad)});
  long long off = 0; // the blocks' offsets for kPlanesGrad planes (same order as prepare_mixed)
  for (MBlock &B : P.blocks) {
    B.ws_off = off;
    off += static_cast<long long>(kPlanesGrad) * B.mp * kBlockPts;
  }
  P.d_blocks = plan_upload(P, P.blocks);
  P.d_order = plan_upload(P, P.order);
  P.d_queue = plan_upload(P, std::vector<int>(2, 0));
  P.d_items = plan_upload(P, P.items);
  P.d_litems = plan_upload(P, P.litems);
  P.d_tabs = plan_upload(P, P.tabs);
  encode_ws_map(P.tmap, g->ws, g->bytes);
  P.ao_cacheable = true;
  grad_tables(*g);
  gmixed = g.release();
}

// The three G_c matrices and the AO -> atom map of a tensor-core gradient.
void Molecule::grad_tables(GradMixed &g) {
  const size_t nbf2 = std::max<size_t>(static_cast<size_t>(basis.nbf) * basis.nbf, 1);
  g.G = static_cast<double *>(alloc(3 * nbf2 * sizeof(double)));
  std::vector<int> ao_atom(std::max(basis.nbf, 1));
  for (size_t s = 0; s < basis.shells.size(); s++)
    for (int f = 0; f < basis.shell_size(static_cast<int>(s)); f++)
      ao_atom[basis.first_bf[s] + f] = basis.shells[s].atom;
  g.ao_atom = static_cast<int *>(alloc(ao_atom.size() * sizeof(int)));
  cuda_check(cudaMemcpy(g.ao_atom, ao_atom.data(), ao_atom.size() * sizeof(int),
                        cudaMemcpyHostToDevice),
             "cudaMemcpy H2D");
}

void Molecule::xc_gradient_mixed(const double *dD, double *dgrad, double *dout2,
                                 cudaStream_t st) {
  prepare_gradient_mixed();
  if (deriv == 2) {
    xc_gradient_mixed_mgga(dD, dgrad, dout2, st);
    return;
  }
  GradMixed &g = *gmixed;
  LaunchPlan &P = g.plan;
  Context &c = *ctx;
  int *err = mixed->d_err;
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int nl = static_cast<int>(P.litems.size());
  const int sms = this->ctas > 0 ? this->ctas
                                 : (ctx->max_ctas > 0 ? ctx->max_ctas : num_sms(device));
  const size_t nbf2 = static_cast<size_t>(basis.nbf) * basis.nbf;
  Override ov{dD, nullptr, dout2};
  c.launch("prep_density", st, [&] {
    k_prep_density<<<dim3(P.maxnbf, 1), 256, 0, st>>>(P.d_tabs, ov, P.d_queue);
  });
  if (nb > 0) {
    if (!P.ao_valid)
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    c.launch("rho_mixed", st, [&] {
      const int gg = std::min(nb, sms);
      if (P.deriv)
        k_rho_mixed<true><<<gg, kRhoThreads, kRhoSmem, st>>>(P.d_tabs, P.d_blocks, P.d_order, nb,
                                                       P.d_queue, err);
      else
        k_rho_mixed<false><<<gg, kRhoThreads, kRhoSmem, st>>>(P.d_tabs, P.d_blocks, P.d_order, nb,
                                                        P.d_queue, err);
    });
  }
  if (nl > 0)
    c.launch("func", st, [&] {
      if (P.deriv)
        k_func_b<true><<<nl, kFuncThreads, 0, st>>>(P.d_tabs, P.d_blocks, P.d_litems);
      else
        k_func_b<false><<<nl, kFuncThreads, 0, st>>>(P.d_tabs, P.d_blocks, P.d_litems);
    });
  if (nb > 0)
    c.launch("grad_ops", st, [&] {
      k_grad_ops<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks, P.deriv);
    });
  cuda_check(cudaMemsetAsync(g.G, 0, 3 * nbf2 * sizeof(double), st), "cudaMemsetAsync");
  for (int cc = 0; cc < 3 && ni > 0; cc++) {
    cuda_check(cudaMemsetAsync(P.d_queue + 1, 0, sizeof(int), st), "cudaMemsetAsync");
    // (d_c phi, Y) and (Z_c, phi), FP32 planes split by the kernel
    const VxcPlanes pl{1 + cc, kPlaneYHi, kPlaneZ + cc, 0, 0, 0, 2};
    Override ovc{dD, g.G + cc * nbf2, dout2};
    c.launch("grad_vxc", st, [&] {
      launch_vxc(P, std::min(ni, sms), st,
          P.d_tabs, P.d_blocks, P.d_items, ni, ovc, P.d_queue, err, P.tmap.rows32, P.tmap.rows128,
          pl);
    });
  }
  cuda_check(cudaMemsetAsync(dgrad, 0, 3 * Z.size() * sizeof(double), st), "cudaMemsetAsync");
  c.launch("grad_contract", st, [&] {
    if (basis.nbf > 0)
      k_grad_contract<<<basis.nbf, 256, 0, st>>>(dD, g.G, basis.nbf, g.ao_atom, dgrad, nullptr);
  });
  c.launch("reduce", st, [&] { k_reduce_b<<<1, 256, 0, st>>>(P.d_tabs, ov); });
  cuda_check(cudaGetLastError(), "kernel launch");
  P.ao_valid = true;
}

} // namespace occx

// ---- unrestricted (UKS) build on the tensor cores -------------------------
// compute_K_dft<deriv, Unrestricted> (include/occ/dft/dft.h:192-388): the
// mixed density kernel once per spin (k_prep_density splits D2_s before each),
// the polarised FP64 functional (k_func_pol), then per spin the V_xc operand
// Y_s (k_ymix) and the V_xc kernel into A_s, V_s = A_s + A_s^T.  The AO planes
// are the restricted build's, in the molecule's private workspace.
namespace occx {
namespace {
template <bool DERIV>
__global__ void __launch_bounds__(256) k_ymix(const MixTab *__restrict__ tabs,
                                             const MBlock *__restrict__ blocks) {
  __shared__ float4 cf[kBlockPts];
  const MBlock B = blocks[blockIdx.x];
  ymix_block<DERIV>(tabs[B.mol], B, cf);
}
} // namespace

void Molecule::build_mixed_uks(const double *dD, double *dV, double *dout3, cudaStream_t st) {
  if (deriv == 2) {
    build_mixed_uks_mgga(dD, dV, dout3, st);
    return;
  }
  ensure_mixed_ws();
  prepare_uks();
  LaunchPlan &P = *mixed->single;
  if (!d_uks_tabs) {
    MixTab tb = P.tabs[0];
    tb.rho = d_rho_b;
    tb.coef = d_coef_b;
    d_uks_tabs = alloc(sizeof(MixTab));
    cuda_check(cudaMemcpy(d_uks_tabs, &tb, sizeof(MixTab), cudaMemcpyHostToDevice),
               "cudaMemcpy H2D");
  }
  const MixTab *tabs[2] = {P.d_tabs, static_cast<const MixTab *>(d_uks_tabs)};
  Context &c = *ctx;
  int *err = mixed->d_err;
  const size_t nbf = static_cast<size_t>(basis.nbf), nbf2 = nbf * nbf;
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int sms = this->ctas > 0 ? this->ctas
                                 : (ctx->max_ctas > 0 ? ctx->max_ctas : num_sms(device));
  // OCC's 2 nbf x nbf -> two contiguous nbf x nbf blocks
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(d_Dab + s * nbf2, nbf * sizeof(double), dD + s * nbf,
                                 2 * nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaMemsetAsync(d_Vab, 0, 2 * nbf2 * sizeof(double), st), "cudaMemsetAsync");
  Override ov[2] = {{d_Dab, d_Vab, nullptr}, {d_Dab + nbf2, d_Vab + nbf2, nullptr}};
  for (int s = 0; s < 2; s++) {
    c.launch("prep_density", st, [&] {
      k_prep_density<<<dim3(P.maxnbf, 1), 256, 0, st>>>(tabs[s], ov[s], P.d_queue);
    });
    if (nb == 0)
      continue;
    if (s == 0 && !P.ao_valid)
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    c.launch("rho_mixed", st, [&] {
      const int g = std::min(nb, sms);
      if (P.deriv)
        k_rho_mixed<true><<<g, kRhoThreads, kRhoSmem, st>>>(tabs[s], P.d_blocks, P.d_order, nb,
                                                      P.d_queue, err);
      else
        k_rho_mixed<false><<<g, kRhoThreads, kRhoSmem, st>>>(tabs[s], P.d_blocks, P.d_order, nb,
                                                       P.d_queue, err);
    });
  }
  const MolDev m = dev();
  c.launch("func_pol", st, [&] {
    launch_func_pol(m, deriv, fs, bs.density_threshold, d_rho, d_rho_b, d_coef, d_coef_b,
                    d_epart_u, st, true);
  });
  for (int s = 0; s < 2 && nb > 0; s++) {
    c.launch("ymix", st, [&] {
      if (P.deriv)
        k_ymix<true><<<nb, 256, 0, st>>>(tabs[s], P.d_blocks);
      else
        k_ymix<false><<<nb, 256, 0, st>>>(tabs[s], P.d_blocks);
    });
    if (ni > 0) {
      cuda_check(cudaMemsetAsync(P.d_queue + 1, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch("vxc_mixed", st, [&] {
        launch_vxc(P, std::min(ni, sms), st,
            tabs[s], P.d_blocks, P.d_items, ni, ov[s], P.d_queue, err, P.tmap.rows32,
            P.tmap.rows128, kVxcSplitPlanes);
      });
    }
    c.launch("symmetrize", st, [&] {
      const int gx = static_cast<int>(std::min<size_t>((nbf2 + 255) / 256, 1024));
      k_symmetrize<<<dim3(std::max(gx, 1), 1), 256, 0, st>>>(tabs[s], ov[s]);
    });
  }
  c.launch("reduce", st, [&] { launch_reduce3(d_epart_u, m.nleaves, dout3, st); });
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(dV + s * nbf, 2 * nbf * sizeof(double), d_Vab + s * nbf2,
                                 nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaGetLastError(), "kernel launch");
  if (P.ao_cacheable)
    P.ao_valid = true;
}

} // namespace occx

// ---- meta-GGA build on the tensor cores -----------------------------------
// compute_K_dft<2, Restricted> (include/occ/dft/dft.h:192-388) with
//   tau = 0.5 sum_k (d_k phi) D2 (d_k phi)          (src/gto/density.cpp:86-100)
//   V  += sum_k (d_k phi)^T diag(0.5 w vtau) (d_k phi)
//                                        (src/dft/xc_potential_matrix.cpp:43-58)
// The blocks carry, beside the build's eight planes, the exact-split A
// slices of d_k phi (three per k, planes 8-16: the A operand of
// k_rho_mixed's tau mode) and, as FP32 planes, t_k = c_tau d_k phi with
// c_tau = 0.25 w vtau (17-19); the XC gradient adds Z_c (20-22) and twice the
// AO Hessian (23-28: xx, xy, xz, yy, yz, zz).  The tau term of V is the V_xc
// kernel's K with operand pairs (d_k phi, t_k), packed two a launch with the
// GGA pair (phi, Y) into the same A that k_symmetrize turns into A + A^T, all
// read as FP32 planes and split into TF32 hi / lo by the kernel.  The
// functional is
// the FP64 meta-GGA evaluator, fused with the operand planes (two CTAs an SM:
// one's FP64 functional overlaps the other's HBM-bound planes).  Measured
// alternatives: a double-float (FP32-pipe) TPSS needed 255 registers a thread
// and ran slower (5.7 against 4.7 ms for the stage), and so did the functional
// and the planes as two kernels (2.95 + 2.17 ms).
namespace occx {

// The V_xc launches of a meta build: four operand pairs, two a launch (the
// kernel's cost is partly per launch), FP32 planes split by the kernel:
//   (phi, Y) + (d_x phi, t_x),  (d_y phi, t_y) + (d_z phi, t_z)
constexpr VxcPlanes kMetaVxcPlanes[2] = {{0, kPlaneYHi, 1, kPlaneMetaT, 0, 0, 2},
                                         {2, kPlaneMetaT + 1, 3, kPlaneMetaT + 2, 0, 0, 2}};

struct MetaMixed {
  char *ws = nullptr;
  size_t bytes = 0;
  LaunchPlan plan;
};

void free_meta_mixed(MetaMixed *g) { delete g; }

namespace {

// Per block (one thread per point), after k_colloc_f32: for k = x, y, z the
// A slices of d_k phi on the exact grid of the point's own power-of-two
// bound.
__global__ void __launch_bounds__(kBlockPts) k_meta_ops(const MixTab *__restrict__ tabs,
                                                        const MBlock *__restrict__ blocks) {
  const MBlock B = blocks[blockIdx.x];
  const MixTab &T = tabs[B.mol];
  const int p = threadIdx.x;
  const size_t plane = static_cast<size_t>(B.mp) * kBlockPts;
  float *base = T.ws + B.ws_off;
  for (int k = 1; k <= 3; k++) {
    const float *g = base + k * plane;
    float vmax = 0.f;
    for (int f = 0; f < B.mp; f++)
      vmax = fmaxf(vmax, fabsf(g[static_cast<size_t>(f) * kBlockPts + p]));
    const float sA = pow2_bound(vmax), isA = 1.f / sA;
    write_a_slices(reinterpret_cast<uint8_t *>(base + (kPlaneTauA + 3 * (k - 1)) * plane), g,
                   B.mp, p, sA, isA);
  }
}

// The tau term's operands t_k = c_tau d_k phi (k = x, y, z) of one block into
// the planes from kPlaneMetaT on, by the NS threads tid = 0 .. NS - 1; as in
// ymix_stream the loads of kYmixBatch iterations go out before their stores.
__device__ __forceinline__ void tau_stream(const MixTab &T, const MBlock &B,
                                           const float *__restrict__ ct, int tid, int NS) {
  constexpr int U = kYmixBatch;
  const size_t plane = static_cast<size_t>(B.mp) * (kBlockPts / 4); // in float4
  const int n4 = B.mp * (kBlockPts / 4);
  const float4 *__restrict__ src = reinterpret_cast<const float4 *>(T.ws + B.ws_off);
  float4 *__restrict__ dst = reinterpret_cast<float4 *>(T.ws + B.ws_off) + kPlaneMetaT * plane;
  for (int q0 = tid; q0 < n4; q0 += NS * U) {
    float4 v[U][3];
#pragma unroll
    for (int u = 0; u < U; u++)
      if (q0 + u * NS < n4)
#pragma unroll
        for (int k = 0; k < 3; k++)
          v[u][k] = src[(k + 1) * plane + q0 + u * NS];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * NS;
      if (q >= n4)
        break;
      const int p = (q % (kBlockPts / 4)) * 4;
      const float c0 = ct[p], c1 = ct[p + 1], c2 = ct[p + 2], c3 = ct[p + 3];
#pragma unroll
      for (int k = 0; k < 3; k++)
        dst[k * plane + q] = make_float4(v[u][k].x * c0, v[u][k].y * c1, v[u][k].z * c2,
                                         v[u][k].w * c3);
    }
  }
}

// The meta-GGA functional per leaf (eval_xc_mgga_mixed), then per block the GGA operand Y
// (ymix_block) and the tau term's operands t_k = c_tau d_k phi, as FP32 planes.
__global__ void __launch_bounds__(256, 2) k_func_b_mgga(const MixTab *__restrict__ tabs,
                                                        const MBlock *__restrict__ blocks,
                                                        const LeafItem *__restrict__ litems) {
  __shared__ double sh[8];
  __shared__ float4 cf[kBlockPts];
  __shared__ float ct[kBlockPts];
  const LeafItem li = litems[blockIdx.x];
  const MixTab &T = tabs[li.mol];
  leaf_functional_mgga<true>(T.m.leaves[li.leaf], T.m.pts, static_cast<size_t>(T.m.npts), T.fs,
                             T.dens_thr, T.rho, T.coef, T.epart + 2 * li.leaf, sh);
  __syncthreads(); // the leaf's coefficients are written
  const size_t N = static_cast<size_t>(T.m.npts);
  for (int b = 0; b < li.nblk; b++) {
    const MBlock B = blocks[li.block0 + b];
    ymix_block<true>(T, B, cf);
    if (threadIdx.x < kBlockPts) {
      const int p = threadIdx.x;
      const size_t idx = static_cast<size_t>(T.m.leaves[B.leaf].off) + B.p0 + p;
      ct[p] = p < B.cnt ? static_cast<float>(T.coef[4 * N + idx]) : 0.f;
    }
    __syncthreads();
    tau_stream(T, B, ct, threadIdx.x, blockDim.x);
    __syncthreads(); // ct is reused by the next block
  }
}

// Per block, for one spin's table (the UKS build): the GGA operand Y
// (ymix_block) and the tau term's operands t_k = c_tau d_k phi, as FP32 planes.
__global__ void __launch_bounds__(256) k_ymix_mgga(const MixTab *__restrict__ tabs,
                                                   const MBlock *__restrict__ blocks) {
  __shared__ float4 cf[kBlockPts];
  __shared__ float ct[kBlockPts];
  const MBlock B = blocks[blockIdx.x];
  const MixTab &T = tabs[B.mol];
  const size_t N = static_cast<size_t>(T.m.npts);
  if (threadIdx.x < kBlockPts) {
    const int p = threadIdx.x;
    const size_t idx = static_cast<size_t>(T.m.leaves[B.leaf].off) + B.p0 + p;
    ct[p] = p < B.cnt ? static_cast<float>(T.coef[4 * N + idx]) : 0.f;
  }
  ymix_block<true>(T, B, cf); // synchronises after filling cf (and so ct)
  tau_stream(T, B, ct, threadIdx.x, blockDim.x);
}

} // namespace

void Molecule::prepare_mgga_mixed() {
  if (mmixed)
    return;
  if (!mixed)
    throw ArgError("the molecule has no device state");
  auto g = std::make_unique<MetaMixed>();
  const WsLayout Lw = ws_layout(*this, kPlanesMeta);
  g->bytes = Lw.total;
  g->ws = static_cast<char *>(alloc(g->bytes));
  LaunchPlan &P = g->plan;
  make_plan_lists(P, {this}, {bind_ws(*this, g->ws, g->ws, kPlanesMeta)}, true);
  long long off = 0; // the blocks' offsets for kPlanesMeta planes (same order as prepare_mixed)
  for (MBlock &B : P.blocks) {
    B.ws_off = off;
    off += static_cast<long long>(kPlanesMeta) * B.mp * kBlockPts;
  }
  P.d_blocks = plan_upload(P, P.blocks);
  P.d_order = plan_upload(P, P.order);
  P.d_queue = plan_upload(P, std::vector<int>(2, 0));
  P.d_items = plan_upload(P, P.items);
  P.d_litems = plan_upload(P, P.litems);
  P.d_tabs = plan_upload(P, P.tabs);
  encode_ws_map(P.tmap, g->ws, g->bytes);
  P.ao_cacheable = true;
  mmixed = g.release();
}

void Molecule::build_mixed_mgga(const double *dD, double *dV, double *dout2, cudaStream_t st) {
  prepare_mgga_mixed();
  LaunchPlan &P = mmixed->plan;
  Context &c = *ctx;
  int *err = mixed->d_err;
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int nl = static_cast<int>(P.litems.size());
  const int sms = this->ctas > 0 ? this->ctas
                                 : (ctx->max_ctas > 0 ? ctx->max_ctas : num_sms(device));
  Override ov{dD, dV, dout2};
  c.launch("prep_density", st, [&] {
    k_prep_density<<<dim3(P.maxnbf, 1), 256, 0, st>>>(P.d_tabs, ov, P.d_queue);
  });
  if (nb > 0) {
    if (!P.ao_valid) {
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
      c.launch("meta_ops", st, [&] {
        k_meta_ops<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    }
    const int gg = std::min(nb, sms);
    c.launch("rho_mixed", st, [&] {
      k_rho_mixed<true><<<gg, kRhoThreads, kRhoSmem, st>>>(P.d_tabs, P.d_blocks, P.d_order, nb,
                                                     P.d_queue, err);
    });
    for (int k = 1; k <= 3; k++) {
      cuda_check(cudaMemsetAsync(P.d_queue, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch("tau_mixed", st, [&] {
        k_rho_mixed<true, true><<<gg, kRhoThreads, kRhoSmem, st>>>(
            P.d_tabs, P.d_blocks, P.d_order, nb, P.d_queue, err, k);
      });
    }
  }
  if (nl > 0)
    c.launch("func", st, [&] {
      k_func_b_mgga<<<nl, 256, 0, st>>>(P.d_tabs, P.d_blocks, P.d_litems);
    });
  if (ni > 0) {
    const VxcPlanes *pls = kMetaVxcPlanes;
    for (int v = 0; v < 2; v++) {
      if (v > 0)
        cuda_check(cudaMemsetAsync(P.d_queue + 1, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch(v == 0 ? "vxc_mixed" : "vxc_tau_mixed", st, [&] {
        launch_vxc(P, std::min(ni, sms), st,
            P.d_tabs, P.d_blocks, P.d_items, ni, ov, P.d_queue, err, P.tmap.rows32,
            P.tmap.rows128, pls[v]);
      });
    }
  }
  c.launch("symmetrize", st, [&] {
    const size_t n2 = static_cast<size_t>(P.maxnbf) * P.maxnbf;
    const int gx = static_cast<int>(std::min<size_t>((n2 + 255) / 256, 1024));
    k_symmetrize<<<dim3(std::max(gx, 1), 1), 256, 0, st>>>(P.d_tabs, ov);
  });
  c.launch("reduce", st, [&] { k_reduce_b<<<1, 256, 0, st>>>(P.d_tabs, ov); });
  cuda_check(cudaGetLastError(), "kernel launch");
  P.ao_valid = true;
}

// The meta-GGA XC gradient on the tensor cores (accumulate_gradient_contribution_R<2>,
// src/dft/dft_gradient_kernels.cpp:124-172, 472-595): the meta build's density,
// tau and functional stages on the meta plan, the operand planes Z_c and 2 d_c d_k phi
// (k_grad_ops<true>), then per direction two V_xc-kernel launches into G_c,
//   (d_c phi, Y) + (Z_c, phi)   and   sum_k (2 d_c d_k phi, t_k),  t_k = 0.25 w vtau d_k phi,
// the second the reference's tau term sum_p d_c d_k phi_mu (0.5 w vtau) d_k phi_nu; then
// g_A,c = - sum_{mu on A} sum_nu 4 D(mu, nu) G_c(mu, nu) (k_grad_contract).
void Molecule::xc_gradient_mixed_mgga(const double *dD, double *dgrad, double *dout2,
                                      cudaStream_t st) {
  GradMixed &g = *gmixed;
  LaunchPlan &P = mmixed->plan;
  Context &c = *ctx;
  int *err = mixed->d_err;
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int nl = static_cast<int>(P.litems.size());
  const int sms = this->ctas > 0 ? this->ctas
                                 : (ctx->max_ctas > 0 ? ctx->max_ctas : num_sms(device));
  const size_t nbf2 = static_cast<size_t>(basis.nbf) * basis.nbf;
  Override ov{dD, nullptr, dout2};
  c.launch("prep_density", st, [&] {
    k_prep_density<<<dim3(P.maxnbf, 1), 256, 0, st>>>(P.d_tabs, ov, P.d_queue);
  });
  if (nb > 0) {
    if (!P.ao_valid) {
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
      c.launch("meta_ops", st, [&] {
        k_meta_ops<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    }
    const int gg = std::min(nb, sms);
    c.launch("rho_mixed", st, [&] {
      k_rho_mixed<true><<<gg, kRhoThreads, kRhoSmem, st>>>(P.d_tabs, P.d_blocks, P.d_order, nb,
                                                     P.d_queue, err);
    });
    for (int k = 1; k <= 3; k++) {
      cuda_check(cudaMemsetAsync(P.d_queue, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch("tau_mixed", st, [&] {
        k_rho_mixed<true, true><<<gg, kRhoThreads, kRhoSmem, st>>>(
            P.d_tabs, P.d_blocks, P.d_order, nb, P.d_queue, err, k);
      });
    }
  }
  if (nl > 0)
    c.launch("func", st, [&] {
      k_func_b_mgga<<<nl, 256, 0, st>>>(P.d_tabs, P.d_blocks, P.d_litems);
    });
  if (nb > 0)
    c.launch("grad_ops", st, [&] {
      k_grad_ops<true><<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks, 1);
    });
  cuda_check(cudaMemsetAsync(g.G, 0, 3 * nbf2 * sizeof(double), st), "cudaMemsetAsync");
  for (int cc = 0; cc < 3 && ni > 0; cc++) {
    const Override ovc{dD, g.G + cc * nbf2, dout2};
    const VxcPlanes pls[2] = {
        {1 + cc, kPlaneYHi, kPlaneMetaZ + cc, 0, 0, 0, 2},
        {kPlaneMetaH + hess_index(cc, 0), kPlaneMetaT, kPlaneMetaH + hess_index(cc, 1),
         kPlaneMetaT + 1, kPlaneMetaH + hess_index(cc, 2), kPlaneMetaT + 2, 3}};
    for (int v = 0; v < 2; v++) {
      cuda_check(cudaMemsetAsync(P.d_queue + 1, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch(v == 0 ? "grad_vxc" : "grad_vxc_tau", st, [&] {
        launch_vxc(P, std::min(ni, sms), st, P.d_tabs, P.d_blocks, P.d_items, ni, ovc, P.d_queue,
                   err, P.tmap.rows32, P.tmap.rows128, pls[v]);
      });
    }
  }
  cuda_check(cudaMemsetAsync(dgrad, 0, 3 * Z.size() * sizeof(double), st), "cudaMemsetAsync");
  c.launch("grad_contract", st, [&] {
    if (basis.nbf > 0)
      k_grad_contract<<<basis.nbf, 256, 0, st>>>(dD, g.G, basis.nbf, g.ao_atom, dgrad, nullptr);
  });
  c.launch("reduce", st, [&] { k_reduce_b<<<1, 256, 0, st>>>(P.d_tabs, ov); });
  cuda_check(cudaGetLastError(), "kernel launch");
  P.ao_valid = true;
}

// compute_K_dft<2, Unrestricted> on the tensor cores: the meta plan's blocks
// per spin (a second table points rho / coef at the beta arrays), the FP64
// polarised meta-GGA functional (k_func_pol_mgga), then per spin the operand
// planes and the three V_xc launches of the restricted meta build.
void Molecule::build_mixed_uks_mgga(const double *dD, double *dV, double *dout3,
                                    cudaStream_t st) {
  prepare_mgga_mixed();
  prepare_uks();
  LaunchPlan &P = mmixed->plan;
  if (!d_uks_tabs_meta) {
    MixTab tb = P.tabs[0];
    tb.rho = d_rho_b;
    tb.coef = d_coef_b;
    d_uks_tabs_meta = alloc(sizeof(MixTab));
    cuda_check(cudaMemcpy(d_uks_tabs_meta, &tb, sizeof(MixTab), cudaMemcpyHostToDevice),
               "cudaMemcpy H2D");
  }
  const MixTab *tabs[2] = {P.d_tabs, static_cast<const MixTab *>(d_uks_tabs_meta)};
  Context &c = *ctx;
  int *err = mixed->d_err;
  const size_t nbf = static_cast<size_t>(basis.nbf), nbf2 = nbf * nbf;
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int sms = this->ctas > 0 ? this->ctas
                                 : (ctx->max_ctas > 0 ? ctx->max_ctas : num_sms(device));
  const int gg = std::min(std::max(nb, 1), sms);
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(d_Dab + s * nbf2, nbf * sizeof(double), dD + s * nbf,
                                 2 * nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaMemsetAsync(d_Vab, 0, 2 * nbf2 * sizeof(double), st), "cudaMemsetAsync");
  Override ov[2] = {{d_Dab, d_Vab, nullptr}, {d_Dab + nbf2, d_Vab + nbf2, nullptr}};
  for (int s = 0; s < 2; s++) {
    c.launch("prep_density", st, [&] {
      k_prep_density<<<dim3(P.maxnbf, 1), 256, 0, st>>>(tabs[s], ov[s], P.d_queue);
    });
    if (nb == 0)
      continue;
    if (s == 0 && !P.ao_valid) {
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
      c.launch("meta_ops", st, [&] {
        k_meta_ops<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    }
    c.launch("rho_mixed", st, [&] {
      k_rho_mixed<true><<<gg, kRhoThreads, kRhoSmem, st>>>(tabs[s], P.d_blocks, P.d_order, nb,
                                                     P.d_queue, err);
    });
    for (int k = 1; k <= 3; k++) {
      cuda_check(cudaMemsetAsync(P.d_queue, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch("tau_mixed", st, [&] {
        k_rho_mixed<true, true><<<gg, kRhoThreads, kRhoSmem, st>>>(
            tabs[s], P.d_blocks, P.d_order, nb, P.d_queue, err, k);
      });
    }
  }
  const MolDev m = dev();
  c.launch("func_pol", st, [&] {
    launch_func_pol(m, deriv, fs, bs.density_threshold, d_rho, d_rho_b, d_coef, d_coef_b,
                    d_epart_u, st, true);
  });
  const VxcPlanes *pls = kMetaVxcPlanes;
  for (int s = 0; s < 2 && nb > 0; s++) {
    c.launch("ymix", st, [&] { k_ymix_mgga<<<nb, 256, 0, st>>>(tabs[s], P.d_blocks); });
    for (int v = 0; v < 2 && ni > 0; v++) {
      cuda_check(cudaMemsetAsync(P.d_queue + 1, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch(v == 0 ? "vxc_mixed" : "vxc_tau_mixed", st, [&] {
        launch_vxc(P, std::min(ni, sms), st,
            tabs[s], P.d_blocks, P.d_items, ni, ov[s], P.d_queue, err, P.tmap.rows32,
            P.tmap.rows128, pls[v]);
      });
    }
    c.launch("symmetrize", st, [&] {
      const int gx = static_cast<int>(std::min<size_t>((nbf2 + 255) / 256, 1024));
      k_symmetrize<<<dim3(std::max(gx, 1), 1), 256, 0, st>>>(tabs[s], ov[s]);
    });
  }
  c.launch("reduce", st, [&] { launch_reduce3(d_epart_u, m.nleaves, dout3, st); });
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(dV + s * nbf, 2 * nbf * sizeof(double), d_Vab + s * nbf2,
                                 nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaGetLastError(), "kernel launch");
  P.ao_valid = true;
}

// The unrestricted meta-GGA XC gradient on the tensor cores
// (accumulate_gradient_contribution_U<2>, src/dft/dft_gradient_kernels.cpp:
// 175-470): per spin the meta plan's density and tau, the polarised functional
// once, then per spin the operand planes (Y_s and t_k,s by k_ymix_mgga, Z_c,s
// and the AO Hessian by k_grad_ops<true>), the two G_c launches per direction
// of the restricted meta gradient and the contraction with that spin's block
// and the reference's |D_a + D_b| skip rule.
void Molecule::xc_gradient_uks_mixed_mgga(const double *dD, double *dgrad, double *dout3,
                                          cudaStream_t st) {
  prepare_gradient_mixed();
  prepare_uks();
  LaunchPlan &P = mmixed->plan;
  GradMixed &g = *gmixed;
  if (!d_uks_tabs_meta) {
    MixTab tb = P.tabs[0];
    tb.rho = d_rho_b;
    tb.coef = d_coef_b;
    d_uks_tabs_meta = alloc(sizeof(MixTab));
    cuda_check(cudaMemcpy(d_uks_tabs_meta, &tb, sizeof(MixTab), cudaMemcpyHostToDevice),
               "cudaMemcpy H2D");
  }
  const MixTab *tabs[2] = {P.d_tabs, static_cast<const MixTab *>(d_uks_tabs_meta)};
  Context &c = *ctx;
  int *err = mixed->d_err;
  const size_t nbf = static_cast<size_t>(basis.nbf), nbf2 = nbf * nbf;
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int sms = this->ctas > 0 ? this->ctas
                                 : (ctx->max_ctas > 0 ? ctx->max_ctas : num_sms(device));
  const int gg = std::min(std::max(nb, 1), sms);
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(d_Dab + s * nbf2, nbf * sizeof(double), dD + s * nbf,
                                 2 * nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaMemsetAsync(dgrad, 0, 3 * Z.size() * sizeof(double), st), "cudaMemsetAsync");
  for (int s = 0; s < 2; s++) {
    const Override ov{d_Dab + s * nbf2, nullptr, nullptr};
    c.launch("prep_density", st, [&] {
      k_prep_density<<<dim3(P.maxnbf, 1), 256, 0, st>>>(tabs[s], ov, P.d_queue);
    });
    if (nb == 0)
      continue;
    if (s == 0 && !P.ao_valid) {
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
      c.launch("meta_ops", st, [&] {
        k_meta_ops<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    }
    c.launch("rho_mixed", st, [&] {
      k_rho_mixed<true><<<gg, kRhoThreads, kRhoSmem, st>>>(tabs[s], P.d_blocks, P.d_order, nb,
                                                     P.d_queue, err);
    });
    for (int k = 1; k <= 3; k++) {
      cuda_check(cudaMemsetAsync(P.d_queue, 0, sizeof(int), st), "cudaMemsetAsync");
      c.launch("tau_mixed", st, [&] {
        k_rho_mixed<true, true><<<gg, kRhoThreads, kRhoSmem, st>>>(
            tabs[s], P.d_blocks, P.d_order, nb, P.d_queue, err, k);
      });
    }
  }
  const MolDev m = dev();
  c.launch("func_pol", st, [&] {
    launch_func_pol(m, deriv, fs, bs.density_threshold, d_rho, d_rho_b, d_coef, d_coef_b,
                    d_epart_u, st, true);
  });
  for (int s = 0; s < 2 && nb > 0; s++) {
    const double *Ds = d_Dab + s * nbf2, *Do = d_Dab + (1 - s) * nbf2;
    c.launch("ymix", st, [&] { k_ymix_mgga<<<nb, 256, 0, st>>>(tabs[s], P.d_blocks); });
    c.launch("grad_ops", st, [&] {
      k_grad_ops<true><<<nb, kBlockPts, 0, st>>>(tabs[s], P.d_blocks, 1);
    });
    cuda_check(cudaMemsetAsync(g.G, 0, 3 * nbf2 * sizeof(double), st), "cudaMemsetAsync");
    for (int cc = 0; cc < 3 && ni > 0; cc++) {
      const Override ovc{Ds, g.G + cc * nbf2, nullptr};
      const VxcPlanes pls[2] = {
          {1 + cc, kPlaneYHi, kPlaneMetaZ + cc, 0, 0, 0, 2},
          {kPlaneMetaH + hess_index(cc, 0), kPlaneMetaT, kPlaneMetaH + hess_index(cc, 1),
           kPlaneMetaT + 1, kPlaneMetaH + hess_index(cc, 2), kPlaneMetaT + 2, 3}};
      for (int v = 0; v < 2; v++) {
        cuda_check(cudaMemsetAsync(P.d_queue + 1, 0, sizeof(int), st), "cudaMemsetAsync");
        c.launch(v == 0 ? "grad_vxc" : "grad_vxc_tau", st, [&] {
          launch_vxc(P, std::min(ni, sms), st, tabs[s], P.d_blocks, P.d_items, ni, ovc,
                     P.d_queue, err, P.tmap.rows32, P.tmap.rows128, pls[v]);
        });
      }
    }
    c.launch("grad_contract", st, [&] {
      k_grad_contract<<<basis.nbf, 256, 0, st>>>(Ds, g.G, basis.nbf, g.ao_atom, dgrad, Do);
    });
  }
  c.launch("reduce", st, [&] { launch_reduce3(d_epart_u, m.nleaves, dout3, st); });
  cuda_check(cudaGetLastError(), "kernel launch");
  P.ao_valid = true;
}

} // namespace occx

// The unrestricted XC gradient on the tensor cores: the gradient plan per spin
// (a second table points rho / coef at the beta arrays), the polarised
// functional with FP32 derivatives, then per spin the operand planes (k_ymix,
// k_grad_ops with that spin's coefficients), the three G_c launches and the
// contraction with that spin's mo.D block, g -= 4 D_s G_c,s (the reference's
// 2 Da V_c,a with D2 = 2 mo.D), skipping |Da + Db| < 1e-12.  dout3 = {E_xc,
// integrated rho_a, integrated rho_b}.
namespace occx {

void Molecule::xc_gradient_uks_mixed(const double *dD, double *dgrad, double *dout3,
                                     cudaStream_t st) {
  if (deriv == 2) {
    xc_gradient_uks_mixed_mgga(dD, dgrad, dout3, st);
    return;
  }
  prepare_gradient_mixed();
  prepare_uks();
  GradMixed &g = *gmixed;
  LaunchPlan &P = g.plan;
  if (!g.d_tab_b) {
    MixTab tb = P.tabs[0];
    tb.rho = d_rho_b;
    tb.coef = d_coef_b;
    g.d_tab_b = alloc(sizeof(MixTab));
    cuda_check(cudaMemcpy(g.d_tab_b, &tb, sizeof(MixTab), cudaMemcpyHostToDevice),
               "cudaMemcpy H2D");
  }
  const MixTab *tabs[2] = {P.d_tabs, static_cast<const MixTab *>(g.d_tab_b)};
  Context &c = *ctx;
  int *err = mixed->d_err;
  const size_t nbf = static_cast<size_t>(basis.nbf), nbf2 = nbf * nbf;
  const int nb = static_cast<int>(P.blocks.size());
  const int ni = static_cast<int>(P.items.size());
  const int sms = this->ctas > 0 ? this->ctas
                                 : (ctx->max_ctas > 0 ? ctx->max_ctas : num_sms(device));
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(d_Dab + s * nbf2, nbf * sizeof(double), dD + s * nbf,
                                 2 * nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaMemsetAsync(dgrad, 0, 3 * Z.size() * sizeof(double), st), "cudaMemsetAsync");
  for (int s = 0; s < 2; s++) {
    const Override ov{d_Dab + s * nbf2, nullptr, nullptr};
    c.launch("prep_density", st, [&] {
      k_prep_density<<<dim3(P.maxnbf, 1), 256, 0, st>>>(tabs[s], ov, P.d_queue);
    });
    if (nb == 0)
      continue;
    if (s == 0 && !P.ao_valid)
      c.launch("colloc_f32", st, [&] {
        k_colloc_f32<<<nb, kBlockPts, 0, st>>>(P.d_tabs, P.d_blocks);
      });
    c.launch("rho_mixed", st, [&] {
      const int gg = std::min(nb, sms);
      if (P.deriv)
        k_rho_mixed<true><<<gg, kRhoThreads, kRhoSmem, st>>>(tabs[s], P.d_blocks, P.d_order, nb,
                                                       P.d_queue, err);
      else
        k_rho_mixed<false><<<gg, kRhoThreads, kRhoSmem, st>>>(tabs[s], P.d_blocks, P.d_order,
                                                        nb, P.d_queue, err);
    });
  }
  const MolDev m = dev();
  c.launch("func_pol", st, [&] {
    launch_func_pol(m, deriv, fs, bs.density_threshold, d_rho, d_rho_b, d_coef, d_coef_b,
                    d_epart_u, st, true);
  });
  for (int s = 0; s < 2 && nb > 0; s++) {
    const double *Ds = d_Dab + s * nbf2, *Do = d_Dab + (1 - s) * nbf2;
    c.launch("ymix", st, [&] {
      if (P.deriv)
        k_ymix<true><<<nb, 256, 0, st>>>(tabs[s], P.d_blocks);
      else
        k_ymix<false><<<nb, 256, 0, st>>>(tabs[s], P.d_blocks);
    });
    c.launch("grad_ops", st, [&] {
      k_grad_ops<<<nb, kBlockPts, 0, st>>>(tabs[s], P.d_blocks, P.deriv);
    });
    cuda_check(cudaMemsetAsync(g.G, 0, 3 * nbf2 * sizeof(double), st), "cudaMemsetAsync");
    for (int cc = 0; cc < 3 && ni > 0; cc++) {
      cuda_check(cudaMemsetAsync(P.d_queue + 1, 0, sizeof(int), st), "cudaMemsetAsync");
      const VxcPlanes pl{1 + cc, kPlaneYHi, kPlaneZ + cc, 0, 0, 0, 2};
      const Override ovc{Ds, g.G + cc * nbf2, nullptr};
      c.launch("grad_vxc", st, [&] {
        launch_vxc(P, std::min(ni, sms), st,
            tabs[s], P.d_blocks, P.d_items, ni, ovc, P.d_queue, err, P.tmap.rows32,
            P.tmap.rows128, pl);
      });
    }
    c.launch("grad_contract", st, [&] {
      k_grad_contract<<<basis.nbf, 256, 0, st>>>(Ds, g.G, basis.nbf, g.ao_atom, dgrad, Do);
    });
  }
  c.launch("reduce", st, [&] { launch_reduce3(d_epart_u, m.nleaves, dout3, st); });
  cuda_check(cudaGetLastError(), "kernel launch");
  P.ao_valid = true;
}

} // namespace occx
