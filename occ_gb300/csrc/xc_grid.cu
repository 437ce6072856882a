// Becke partition weights of the molecular grid on the device
// (src/numint/grid_utils.cpp:149-200 with the Treutler-Ahlrichs adjustment of
// :125-137, applied per point as src/numint/molecular_grid.cpp:46-82 does).
//
// For a point p owned by atom a, OCC computes for every atom k the cell
// function P_k = prod_{j != k} s_kj with, for the ordered pair (i > j),
//   mu = (d_i - d_j) / R_ij,  nu = mu + a_ij (1 - mu^2),  v = f(f(f(nu))),
//   f(x) = (3 - x^2) x / 2,  W_i *= (1 - v) / 2,  W_j *= (1 + v) / 2,
// except that |1 - v| < 1e-14 sets W_i = 0 and leaves W_j, and the weight is
// w_ra(p) P_a / sum_k P_k.  That is O(natom^2) FP64 work per point, the
// dominant cost of creating a molecule on the host (6.5 s for 32 waters on
// eight cores).
//
// Here one warp takes one point:
//   1. distances to all atoms into shared memory (FP64 and FP32 copies);
//   2. every P_k in FP32 (lanes over k, all lanes stepping through j
//      together so that the pair tables are read coalesced), with the
//      factors written in the cancellation-free form
//        1 - f3(nu) = E(1 - nu),  E: e <- e^2 (3 - e) / 2 three times,
//        1 - nu = (1 - mu')(1 + sigma a (1 + mu')),  mu' = (d_k - d_j) / R,
//      sigma = -1 for k > j, +1 for k < j, so that even factors near zero
//      keep FP32's relative precision;
//   3. the atoms with P_k >= 1e-20 max_k P_k (and the owner) again in FP64
//      with OCC's formula and its 1e-14 rule, the warp's lanes splitting j;
//      dropped atoms change the sum by less than natom 1e-20 relative;
//   4. w = w_ra P_a / sum.
// The FP64 products of step 3 are taken in a different order than OCC's
// sequential loop (rounding differences of ~1e-16 relative).
#include <algorithm>
#include <mutex>
#include <vector>

#include "host/xc_host.hpp"
#include "xc_engine.hpp"

namespace occx {

namespace {

constexpr int kBeckeWarps = 4;
constexpr float kBeckeKeep = 1e-20f; // relative to the largest P_k

__device__ __forceinline__ float becke_e3(float e) {
#pragma unroll
  for (int it = 0; it < 3; it++)
    e = e * e * (1.5f - 0.5f * e);
  return e;
}

__device__ __forceinline__ double warp_prod_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v *= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Shared memory: atom coordinates (3 natom FP64), then per warp d (natom
// FP64), d32 (natom FP32), p32 (natom FP32) and the list of kept atoms
// (natom int).
__global__ void __launch_bounds__(kBeckeWarps * 32)
    k_becke(int natom, const double *__restrict__ atom_xyz, const double *__restrict__ inv_dist,
            const double *__restrict__ adj_ab, const float *__restrict__ inv_dist32,
            const float *__restrict__ sadj32, long npts, const double *__restrict__ xyz,
            const int *__restrict__ owner, const double *__restrict__ wra,
            double *__restrict__ w) {
  extern __shared__ double sh[];
  double *ax = sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per warp: d (natom FP64), then d32 (natom FP32) and p32 (natom FP32); the
  // list of kept atoms is written over d32 once step 2 no longer reads it
  double *d = sh + 3 * natom + static_cast<size_t>(warp) * natom * 2;
  float *d32 = reinterpret_cast<float *>(d + natom);
  float *p32 = d32 + natom;
  int *kept = reinterpret_cast<int *>(d32);
  for (int i = threadIdx.x; i < 3 * natom; i += blockDim.x)
    ax[i] = atom_xyz[i];
  __syncthreads();
  const long nw = static_cast<long>(gridDim.x) * kBeckeWarps;
  for (long p = static_cast<long>(blockIdx.x) * kBeckeWarps + warp; p < npts; p += nw) {
    const double px = xyz[3 * p], py = xyz[3 * p + 1], pz = xyz[3 * p + 2];
    for (int i = lane; i < natom; i += 32) {
      const double dx = px - ax[3 * i], dy = py - ax[3 * i + 1], dz = pz - ax[3 * i + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      d[i] = r;
      d32[i] = static_cast<float>(r);
    }
    __syncwarp();
    const int a = owner[p];
    // step 2: P_k in FP32
    float pmax = 0.0f;
    for (int k0 = 0; k0 < natom; k0 += 32) {
      const int k = k0 + lane;
      const bool kv = k < natom;
      const int kk = kv ? k : 0;
      const float dk = d32[kk];
      float P = 1.0f;
      for (int j = 0; j < natom; j++) {
        const float ir = inv_dist32[static_cast<size_t>(j) * natom + kk];
        const float sa = sadj32[static_cast<size_t>(j) * natom + kk];
        const float mu = (dk - d32[j]) * ir;
        const float e0 = (1.0f - mu) * (1.0f + sa * (1.0f + mu));
        const float f = 0.5f * becke_e3(e0);
        P = (j == kk) ? P : P * f;
      }
      if (kv) {
        p32[k] = P;
        pmax = fmaxf(pmax, P);
      }
    }
    pmax = warp_max_f(pmax);
    __syncwarp();
    // the kept atoms, in ascending order
    int nkept = 0;
    for (int k0 = 0; k0 < natom; k0 += 32) {
      const int k = k0 + lane;
      const bool keep = k < natom && (p32[k] >= kBeckeKeep * pmax || k == a);
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      __syncwarp();
      if (keep)
        kept[nkept + __popc(m & ((1u << lane) - 1u))] = k;
      nkept += __popc(m);
    }
    __syncwarp();
    // step 3: FP64 cell functions of the kept atoms, the warp splitting j
    double sum = 0.0, pa = 0.0;
    for (int q = 0; q < nkept; q++) {
      const int k = kept[q];
      const double dk = d[k];
      double P = 1.0;
      for (int j = lane; j < natom; j += 32) {
        if (j == k)
          continue;
        const size_t t = static_cast<size_t>(j) * natom + k;
        // the ordered pair (max(j, k), min(j, k)) as OCC forms it
        double v = (k > j ? dk - d[j] : d[j] - dk) * inv_dist[t];
        v = fma(adj_ab[t], 1.0 - v * v, v);
#pragma unroll
        for (int it = 0; it < 3; it++)
          v = (3.0 - v * v) * v * 0.5;
        const bool sat = fabs(1.0 - v) < 1e-14;
        if (k > j)
          P = sat ? 0.0 : P * (0.5 * (1.0 - v));
        else if (!sat)
          P *= 0.5 * (1.0 + v);
      }
      P = warp_prod_d(P);
      sum += P;
      if (k == a)
        pa = P;
    }
    if (lane == 0)
      w[p] = wra[p] * (pa / sum);
    __syncwarp();
  }
}

struct DevBuf {
  void *p = nullptr;
  cudaStream_t st;
  explicit DevBuf(cudaStream_t s) : st(s) {}
  ~DevBuf() {
    if (p)
      cudaFreeAsync(p, st);
  }
};

} // namespace

constexpr int kMaxBeckeDevices = 64;

size_t becke_smem_bytes(int natom) {
  // atom coordinates + per warp d (FP64) and two FP32 / int arrays
  return static_cast<size_t>(natom) * (3 * sizeof(double) + kBeckeWarps * 2 * sizeof(double));
}

bool device_partition_fits(int device, int natom) {
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) !=
      cudaSuccess)
    return false;
  return natom > 0 && becke_smem_bytes(natom) <= static_cast<size_t>(optin);
}

void device_partition(int device, const PartitionInput &in, double *w_out) {
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
  cudaStream_t st;
  cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  } sg{st};
  const size_t na = static_cast<size_t>(in.natom), n = static_cast<size_t>(in.npts);
  std::vector<float> ir32(na * na), sa32(na * na);
  for (size_t j = 0; j < na; j++)
    for (size_t k = 0; k < na; k++) {
      const size_t t = j * na + k;
      ir32[t] = static_cast<float>(in.inv_dist[t]);
      sa32[t] = static_cast<float>(k > j ? -in.adj_ab[t] : in.adj_ab[t]);
    }
  // one device region: atoms, the four tables, points, owners, wra, w
  const size_t off_ax = 0;
  const size_t off_ir = off_ax + 3 * na * 8;
  const size_t off_ad = off_ir + na * na * 8;
  const size_t off_ir32 = off_ad + na * na * 8;
  const size_t off_sa32 = off_ir32 + ((na * na * 4 + 7) / 8) * 8;
  const size_t off_xyz = off_sa32 + ((na * na * 4 + 7) / 8) * 8;
  const size_t off_own = off_xyz + 3 * n * 8;
  const size_t off_wra = off_own + ((n * 4 + 7) / 8) * 8;
  const size_t off_w = off_wra + n * 8;
  const size_t total = off_w + n * 8;
  DevBuf buf(st);
  cuda_check(cudaMallocAsync(&buf.p, total, st), "cudaMallocAsync");
  char *b = static_cast<char *>(buf.p);
  auto up = [&](size_t off, const void *src, size_t bytes) {
    cuda_check(cudaMemcpyAsync(b + off, src, bytes, cudaMemcpyHostToDevice, st),
               "cudaMemcpyAsync H2D");
  };
  up(off_ax, in.atom_xyz, 3 * na * 8);
  up(off_ir, in.inv_dist, na * na * 8);
  up(off_ad, in.adj_ab, na * na * 8);
  up(off_ir32, ir32.data(), na * na * 4);
  up(off_sa32, sa32.data(), na * na * 4);
  up(off_xyz, in.xyz, 3 * n * 8);
  up(off_own, in.owner, n * 4);
  up(off_wra, in.wra, n * 8);
  const size_t smem = becke_smem_bytes(in.natom);
  {
    // the kernel's shared-memory ceiling is a property of the function on
    // this device, shared by every thread that builds a grid: raise it once,
    // to the device's opt-in maximum, so that concurrent callers with smaller
    // molecules never lower it under a larger one's launch
    static std::mutex mu;
    static bool raised[kMaxBeckeDevices] = {};
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= kMaxBeckeDevices)
      throw ArgError("device ordinal out of range for the grid kernel");
    if (!raised[device]) {
      int optin = 0;
      cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device),
                 "cudaDeviceGetAttribute");
      cuda_check(cudaFuncSetAttribute(k_becke, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      optin),
                 "cudaFuncSetAttribute");
      raised[device] = true;
    }
  }
  int sms = 0;
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device),
             "cudaDeviceGetAttribute");
  int per_sm = 0;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_becke, kBeckeWarps * 32,
                                                           smem),
             "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  const long want = (static_cast<long>(n) + kBeckeWarps - 1) / kBeckeWarps;
  const int grid = static_cast<int>(std::max<long>(
      1, std::min<long>(want, static_cast<long>(sms) * std::max(per_sm, 1) * 8)));
  if (n > 0)
    k_becke<<<grid, kBeckeWarps * 32, smem, st>>>(
        in.natom, reinterpret_cast<const double *>(b + off_ax),
        reinterpret_cast<const double *>(b + off_ir), reinterpret_cast<const double *>(b + off_ad),
        reinterpret_cast<const float *>(b + off_ir32),
        reinterpret_cast<const float *>(b + off_sa32), static_cast<long>(n),
        reinterpret_cast<const double *>(b + off_xyz), reinterpret_cast<const int *>(b + off_own),
        reinterpret_cast<const double *>(b + off_wra), reinterpret_cast<double *>(b + off_w));
  cuda_check(cudaGetLastError(), "k_becke launch");
  cuda_check(cudaMemcpyAsync(w_out, b + off_w, n * 8, cudaMemcpyDeviceToHost, st),
             "cudaMemcpyAsync D2H");
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
}

} // namespace occx
