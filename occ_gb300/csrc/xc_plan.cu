// The build plan on the GPU: Morton order of the grid points, leaf bounding
// spheres and per-leaf shell screening (src/numint/spatial_grid_hierarchy.cpp
// :40-147, src/gto/gto.cpp:18-67 for the decay radii, include/occ/dft/dft.h
// :303-320 for the screening), the set-up work that dominates opening a new
// molecule once its grid's Becke partition runs on the GPU (xc_grid.cu).
//
// The results are those of the host restatement (host/plan.cpp):
//  - Morton keys: 21 bits per axis from (x - lo) / extent * (2^21 - 1),
//    truncated, interleaved (x lowest); sorted by key, ties by original index
//    (a stable LSD radix sort of (key, index) pairs gives std::sort's order
//    of the pairs);
//  - leaves: the same splitting rule (target, minimum, maximum), centres as
//    the running sum of the leaf's points in order divided by the count,
//    radii as the largest distance to the centre;
//  - screening: shell s is significant for leaf b when
//    |A_s - c_b| - r_s < R_b, shells in ascending order.
// Shell decay radii stay on the host (one short radial scan per shell).
#include <algorithm>
#include <vector>

#include "host/xc_host.hpp"
#include "xc_engine.hpp"

namespace occx {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;                          // keys per thread per tile
constexpr int kSortTile = kSortThreads * kSortItems;    // 4096
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kKeyBits = 63;                            // 3 x 21 Morton bits

__device__ __forceinline__ uint64_t spread3_dev(uint64_t x) {
  x &= 0x1fffff;
  x = (x | (x << 32)) & 0x1f00000000ffffULL;
  x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
  x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
  x = (x | (x << 2)) & 0x1249249249249249ULL;
  return x;
}

// Morton key and original index of every point.
__global__ void k_morton_keys(long n, const double *__restrict__ xyz, double lo0, double lo1,
                             double lo2, double ex0, double ex1, double ex2,
                             uint64_t *__restrict__ keys, int *__restrict__ idx) {
  const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const double lo[3] = {lo0, lo1, lo2}, ex[3] = {ex0, ex1, ex2};
  const double scale = static_cast<double>((1ULL << 21) - 1);
  uint64_t q[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double u = __ddiv_rn(__dsub_rn(xyz[3 * i + d], lo[d]), ex[d]);
    u = fmin(fmax(u, 0.0), 1.0);
    q[d] = static_cast<uint64_t>(__dmul_rn(u, scale));
  }
  keys[i] = spread3_dev(q[0]) | (spread3_dev(q[1]) << 1) | (spread3_dev(q[2]) << 2);
  idx[i] = static_cast<int>(i);
}

// Digit histogram of each tile, digit-major: counts[d * ntiles + tile].
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(long n, int shift,
                                                             const uint64_t *__restrict__ keys,
                                                             unsigned *__restrict__ counts,
                                                             int ntiles) {
  __shared__ unsigned h[kRadix];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long base = static_cast<long>(blockIdx.x) * kSortTile;
  for (int r = 0; r < kSortItems; r++) {
    const long i = base + r * kSortThreads + threadIdx.x;
    if (i < n)
      atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  counts[static_cast<size_t>(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive prefix sum of the digit-major counts in place (one CTA).
__global__ void __launch_bounds__(1024) k_radix_scan(unsigned *__restrict__ counts, long len) {
  __shared__ unsigned part[1024];
  const long per = (len + 1023) / 1024;
  const long b = threadIdx.x * per, e = min(len, b + per);
  unsigned s = 0;
  for (long i = b; i < e; i++)
    s += counts[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned run = 0;
    for (int t = 0; t < 1024; t++) {
      const unsigned v = part[t];
      part[t] = run;
      run += v;
    }
  }
  __syncthreads();
  unsigned run = part[threadIdx.x];
  for (long i = b; i < e; i++) {
    const unsigned v = counts[i];
    counts[i] = run;
    run += v;
  }
}

// Stable scatter of one tile by the current digit: rounds of 256 keys in
// index order; inside a round, lanes of a warp with equal digits are ranked
// by match_any, warps by a prefix over per-warp digit counts.
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(
    long n, int shift, const uint64_t *__restrict__ kin, const int *__restrict__ vin,
    uint64_t *__restrict__ kout, int *__restrict__ vout, const unsigned *__restrict__ offsets,
    int ntiles) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ unsigned s_off[kRadix];
  __shared__ unsigned s_tot[kRadix];
  __shared__ unsigned s_w[kWarps][kRadix];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  s_off[t] = offsets[static_cast<size_t>(t) * ntiles + blockIdx.x];
  const unsigned lt = (1u << lane) - 1u;
  const long base = static_cast<long>(blockIdx.x) * kSortTile;
  for (int r = 0; r < kSortItems; r++) {
    const long i = base + r * kSortThreads + t;
    const bool valid = i < n;
    const uint64_t key = valid ? kin[i] : 0;
    const int val = valid ? vin[i] : 0;
    const unsigned d = valid ? static_cast<unsigned>((key >> shift) & (kRadix - 1)) : kRadix;
#pragma unroll
    for (int w = 0; w < kWarps; w++)
      s_w[w][t] = 0;
    __syncthreads();
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & lt);
    if (valid && rank == 0)
      s_w[warp][d] = __popc(peers);
    __syncthreads();
    {
      unsigned run = 0;
#pragma unroll
      for (int w = 0; w < kWarps; w++) {
        const unsigned c = s_w[w][t];
        s_w[w][t] = run;
        run += c;
      }
      s_tot[t] = run;
    }
    __syncthreads();
    if (valid) {
      const unsigned pos = s_off[d] + s_w[warp][d] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    s_off[t] += s_tot[t];
    __syncthreads();
  }
}

// Sorted points as (x, y, z, w).
__global__ void k_gather_pts4(long n, const int *__restrict__ perm, const double *__restrict__ xyz,
                              const double *__restrict__ w, double *__restrict__ pts4) {
  const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const long o = perm[i];
  pts4[4 * i] = xyz[3 * o];
  pts4[4 * i + 1] = xyz[3 * o + 1];
  pts4[4 * i + 2] = xyz[3 * o + 2];
  pts4[4 * i + 3] = w[o];
}

// Centre (running sum in point order / count) and radius of each leaf.
__global__ void k_leaf_spheres(int nleaves, const long *__restrict__ off,
                               const long *__restrict__ cnt, const double *__restrict__ pts4,
                               double *__restrict__ centre, double *__restrict__ radius) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaves)
    return;
  const long o = off[b], c = cnt[b];
  double s[3] = {0.0, 0.0, 0.0};
  for (long i = o; i < o + c; i++)
#pragma unroll
    for (int d = 0; d < 3; d++)
      s[d] = __dadd_rn(s[d], pts4[4 * i + d]);
#pragma unroll
  for (int d = 0; d < 3; d++)
    s[d] = __ddiv_rn(s[d], static_cast<double>(c));
  double r = 0.0;
  for (long i = o; i < o + c; i++) {
    const double dx = __dsub_rn(pts4[4 * i], s[0]), dy = __dsub_rn(pts4[4 * i + 1], s[1]),
                 dz = __dsub_rn(pts4[4 * i + 2], s[2]);
    r = fmax(r, __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                     __dmul_rn(dz, dz))));
  }
#pragma unroll
  for (int d = 0; d < 3; d++)
    centre[3 * b + d] = s[d];
  radius[b] = r;
}

// Significant shells of each leaf: a counting pass (shells and AOs), then a
// pass that writes the ascending shell list at the leaf's offset.
__device__ __forceinline__ bool shell_near(const double *A, double ext, const double *c,
                                           double rad) {
  const double dx = __dsub_rn(A[0], c[0]), dy = __dsub_rn(A[1], c[1]),
               dz = __dsub_rn(A[2], c[2]);
  const double dist =
      __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
  return __dsub_rn(dist, ext) < rad;
}

__global__ void k_screen_count(int nleaves, int nsh, const double *__restrict__ sh_xyz,
                               const double *__restrict__ ext, const int *__restrict__ sh_size,
                               const double *__restrict__ centre, const double *__restrict__ radius,
                               int *__restrict__ nsig, int *__restrict__ nao) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaves)
    return;
  int ns = 0, m = 0;
  for (int s = 0; s < nsh; s++)
    if (shell_near(sh_xyz + 3 * s, ext[s], centre + 3 * b, radius[b])) {
      ns++;
      m += sh_size[s];
    }
  nsig[b] = ns;
  nao[b] = m;
}

__global__ void k_screen_fill(int nleaves, int nsh, const double *__restrict__ sh_xyz,
                              const double *__restrict__ ext, const double *__restrict__ centre,
                              const double *__restrict__ radius, const long *__restrict__ ptr,
                              int *__restrict__ list) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaves)
    return;
  long k = ptr[b];
  for (int s = 0; s < nsh; s++)
    if (shell_near(sh_xyz + 3 * s, ext[s], centre + 3 * b, radius[b]))
      list[k++] = s;
}

// One stream and one device region for the whole plan; freed on every path.
struct PlanScratch {
  cudaStream_t st = nullptr;
  void *p = nullptr;
  void *list = nullptr;
  ~PlanScratch() {
    if (st) {
      cudaStreamSynchronize(st);
      if (p)
        cudaFreeAsync(p, st);
      if (list)
        cudaFreeAsync(list, st);
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  }
};

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

} // namespace

void device_plan(int device, const MolecularGrid &grid, const Basis &basis,
                 const BuildSettings &bs, Plan &plan) {
  const long n = grid.npts();
  if (n >= (1L << 31) - kSortTile)
    throw ArgError("grid too large for the device plan (2^31 points)");
  int prev = -1;
  cuda_check(cudaGetDevice(&prev), "cudaGetDevice");
  cuda_check(cudaSetDevice(device), "cudaSetDevice");
  struct Restore {
    int dev;
    ~Restore() {
      if (dev >= 0)
        cudaSetDevice(dev);
    }
  } restore{prev};

  plan = Plan{};
  plan.npts = n;
  plan.extents = decay_cutoff(basis, bs.xc_screening_threshold);
  if (n == 0)
    return;

  // bounding box (src/numint/spatial_grid_hierarchy.cpp:40-60)
  double lo[3], hi[3], ext[3];
  for (int d = 0; d < 3; d++)
    lo[d] = hi[d] = grid.xyz[d];
  for (long i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      lo[d] = std::min(lo[d], grid.xyz[3 * i + d]);
      hi[d] = std::max(hi[d], grid.xyz[3 * i + d]);
    }
  for (int d = 0; d < 3; d++) {
    ext[d] = hi[d] - lo[d];
    if (ext[d] < 1e-10)
      ext[d] = 1.0;
  }

  // leaves (the splitting rule of spatial_grid_hierarchy.cpp:94-124)
  long off = 0;
  while (off < n) {
    const long rem = n - off;
    long cnt;
    if (rem <= bs.leaf_max)
      cnt = rem;
    else if (rem < 2 * bs.leaf_min)
      cnt = rem / 2;
    else
      cnt = std::min(bs.leaf_target, rem);
    plan.leaf_off.push_back(off);
    plan.leaf_cnt.push_back(cnt);
    off += cnt;
  }
  const int nl = static_cast<int>(plan.leaf_off.size());
  const int nsh = static_cast<int>(basis.shells.size());
  const int ntiles = static_cast<int>((n + kSortTile - 1) / kSortTile);
  const size_t ncount = static_cast<size_t>(kRadix) * ntiles;

  // one region: xyz, w, two (key, index) buffers, counts, pts4, leaves, shells
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += align256(bytes);
    return at;
  };
  const size_t nsh1 = static_cast<size_t>(std::max(nsh, 1));
  const size_t o_xyz = take(3 * n * 8), o_w = take(n * 8), o_k0 = take(n * 8),
               o_k1 = take(n * 8), o_v0 = take(n * 4), o_v1 = take(n * 4),
               o_cnt = take(ncount * 4), o_pts = take(4 * n * 8), o_loff = take(nl * 8),
               o_lcnt = take(nl * 8), o_cen = take(3 * nl * 8), o_rad = take(nl * 8),
               o_shx = take(3 * nsh1 * 8), o_ext = take(nsh1 * 8), o_shs = take(nsh1 * 4),
               o_ns = take(nl * 4), o_na = take(nl * 4), o_ptr = take((nl + 1) * 8);
  PlanScratch S;
  cuda_check(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaMallocAsync(&S.p, o, S.st), "cudaMallocAsync");
  char *b = static_cast<char *>(S.p);
  cudaStream_t st = S.st;
  auto up = [&](size_t at, const void *src, size_t bytes) {
    cuda_check(cudaMemcpyAsync(b + at, src, bytes, cudaMemcpyHostToDevice, st), "H2D");
  };
  auto down = [&](void *dst, const void *src, size_t bytes) {
    cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st), "D2H");
  };
  up(o_xyz, grid.xyz.data(), 3 * n * 8);
  up(o_w, grid.w.data(), n * 8);

  // Morton keys and the radix sort (eight passes of eight bits)
  uint64_t *k0 = reinterpret_cast<uint64_t *>(b + o_k0);
  uint64_t *k1 = reinterpret_cast<uint64_t *>(b + o_k1);
  int *v0 = reinterpret_cast<int *>(b + o_v0), *v1 = reinterpret_cast<int *>(b + o_v1);
  unsigned *counts = reinterpret_cast<unsigned *>(b + o_cnt);
  const int g256 = static_cast<int>((n + 255) / 256);
  k_morton_keys<<<g256, 256, 0, st>>>(n, reinterpret_cast<const double *>(b + o_xyz), lo[0],
                                      lo[1], lo[2], ext[0], ext[1], ext[2], k0, v0);
  for (int shift = 0; shift < kKeyBits; shift += kRadixBits) {
    k_radix_hist<<<ntiles, kSortThreads, 0, st>>>(n, shift, k0, counts, ntiles);
    k_radix_scan<<<1, 1024, 0, st>>>(counts, static_cast<long>(ncount));
    k_radix_scatter<<<ntiles, kSortThreads, 0, st>>>(n, shift, k0, v0, k1, v1, counts, ntiles);
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  double *pts4 = reinterpret_cast<double *>(b + o_pts);
  k_gather_pts4<<<g256, 256, 0, st>>>(n, v0, reinterpret_cast<const double *>(b + o_xyz),
                                      reinterpret_cast<const double *>(b + o_w), pts4);

  // leaf spheres
  up(o_loff, plan.leaf_off.data(), nl * 8);
  up(o_lcnt, plan.leaf_cnt.data(), nl * 8);
  const int gl = (nl + 127) / 128;
  k_leaf_spheres<<<gl, 128, 0, st>>>(nl, reinterpret_cast<const long *>(b + o_loff),
                                     reinterpret_cast<const long *>(b + o_lcnt), pts4,
                                     reinterpret_cast<double *>(b + o_cen),
                                     reinterpret_cast<double *>(b + o_rad));

  // screening
  std::vector<double> shx(3 * nsh1, 0.0);
  std::vector<int> shs(nsh1, 0);
  for (int s = 0; s < nsh; s++) {
    for (int d = 0; d < 3; d++)
      shx[3 * s + d] = basis.shells[s].origin[d];
    shs[s] = basis.shell_size(s);
  }
  up(o_shx, shx.data(), shx.size() * 8);
  if (nsh > 0)
    up(o_ext, plan.extents.data(), nsh * 8);
  up(o_shs, shs.data(), shs.size() * 4);
  k_screen_count<<<gl, 128, 0, st>>>(nl, nsh, reinterpret_cast<const double *>(b + o_shx),
                                     reinterpret_cast<const double *>(b + o_ext),
                                     reinterpret_cast<const int *>(b + o_shs),
                                     reinterpret_cast<const double *>(b + o_cen),
                                     reinterpret_cast<const double *>(b + o_rad),
                                     reinterpret_cast<int *>(b + o_ns),
                                     reinterpret_cast<int *>(b + o_na));
  cuda_check(cudaGetLastError(), "plan kernel launch");
  std::vector<int> nsig(nl);
  plan.leaf_nbf.assign(nl, 0);
  down(nsig.data(), b + o_ns, nl * 4);
  down(plan.leaf_nbf.data(), b + o_na, nl * 4);
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  plan.leaf_sh_ptr.assign(nl + 1, 0);
  for (int l = 0; l < nl; l++)
    plan.leaf_sh_ptr[l + 1] = plan.leaf_sh_ptr[l] + nsig[l];
  const long nlist = plan.leaf_sh_ptr[nl];
  plan.leaf_sh.assign(nlist, 0);
  if (nlist > 0) {
    cuda_check(cudaMallocAsync(&S.list, nlist * 4, st), "cudaMallocAsync");
    up(o_ptr, plan.leaf_sh_ptr.data(), (nl + 1) * 8);
    k_screen_fill<<<gl, 128, 0, st>>>(nl, nsh, reinterpret_cast<const double *>(b + o_shx),
                                      reinterpret_cast<const double *>(b + o_ext),
                                      reinterpret_cast<const double *>(b + o_cen),
                                      reinterpret_cast<const double *>(b + o_rad),
                                      reinterpret_cast<const long *>(b + o_ptr),
                                      static_cast<int *>(S.list));
    cuda_check(cudaGetLastError(), "plan kernel launch");
    down(plan.leaf_sh.data(), S.list, nlist * 4);
  }
  // results to the host
  plan.pts4.assign(4 * n, 0.0);
  plan.leaf_centre.assign(3 * nl, 0.0);
  plan.leaf_radius.assign(nl, 0.0);
  std::vector<int> perm32(n);
  down(plan.pts4.data(), pts4, 4 * n * 8);
  down(perm32.data(), v0, n * 4);
  down(plan.leaf_centre.data(), b + o_cen, 3 * nl * 8);
  down(plan.leaf_radius.data(), b + o_rad, nl * 8);
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  plan.perm.assign(perm32.begin(), perm32.end());
}

} // namespace occx
