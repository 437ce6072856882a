// FP64 ("plain") XC build kernels for sm_103a.
//
// GB300 executes FP64 on the SM's DFMA pipe only (tcgen05 has no f64 kind),
// so the contractions here are register-tiled SIMT DFMA kernels whose bound
// is the FP64 pipe; the collocation and functional kernels are per-point
// elementwise work.  The sequence per build restates
// include/occ/dft/dft.h:279-380 leaf by leaf:
//   k_colloc_f64  phi, grad phi for the leaf's significant shells
//                 (src/gto/gto.cpp:212-287)
//   k_rho_f64     X = phi D2 (64-point x 64-AO tiles, D gathered from the
//                 global matrix), rho = rowsum(phi o X), grad rho =
//                 2 rowsum(grad phi o X)      (src/gto/density.cpp:33-43)
//   k_func        functional, block skip, weights, E_xc partials
//                 (src/dft/dft_kernels.cpp:27-62)
//   k_vxc_f64     K = phi^T Y per 64x64 AO tile, Y = 0.5 w vrho phi +
//                 2 w vsigma grad rho . grad phi, V += K + K^T scattered
//                 into the global matrix      (src/dft/xc_potential_matrix.cpp:19-41)
//   k_reduce      fixed-order sum of the per-leaf partials (dft.h:374-380)
#include "host/gto_eval.h"
#include "xc_device.cuh"
#include "xc_leaf_func.cuh"

namespace occx {

__constant__ double c_sph[kSphTableSize];

// One shell at one point: values (and gradients) of its nfunc AOs, scaled.
template <int L, bool DERIV, typename T>
__device__ __forceinline__ void shell_values(const T *sph, bool pure, T x, T y, T z, T R, T dR,
                                             T fac, T *v, T *gx, T *gy, T *gz) {
  constexpr int NC = ncart_of(L);
  T cv[NC], cx[DERIV ? NC : 1], cy[DERIV ? NC : 1], cz[DERIV ? NC : 1];
  cart_eval_l<L, T>(x, y, z, R, dR, cv, DERIV ? cx : nullptr, DERIV ? cy : nullptr,
                    DERIV ? cz : nullptr);
  if (L < 2 && !pure) {
#pragma unroll
    for (int c = 0; c < NC; c++) {
      v[c] = cv[c] * fac;
      if (DERIV) {
        gx[c] = cx[c] * fac;
        gy[c] = cy[c] * fac;
        gz[c] = cz[c] * fac;
      }
    }
    return;
  }
  if (!pure) {
#pragma unroll
    for (int c = 0; c < NC; c++) {
      v[c] = cv[c] * fac;
      if (DERIV) {
        gx[c] = cx[c] * fac;
        gy[c] = cy[c] * fac;
        gz[c] = cz[c] * fac;
      }
    }
    return;
  }
  const T *Tm = sph + sph_offset(L);
#pragma unroll
  for (int f = 0; f < 2 * L + 1; f++) {
    T a = 0, b = 0, c = 0, d = 0;
#pragma unroll
    for (int k = 0; k < NC; k++) {
      T t = Tm[f * NC + k];
      a += t * cv[k];
      if (DERIV) {
        b += t * cx[k];
        c += t * cy[k];
        d += t * cz[k];
      }
    }
    v[f] = a * fac;
    if (DERIV) {
      gx[f] = b * fac;
      gy[f] = c * fac;
      gz[f] = d * fac;
    }
  }
}

template <int L, bool DERIV>
__device__ __forceinline__ void colloc_store_f64(const DevShell &sh, bool pure, double x, double y,
                                                 double z, double R, double dR, bool valid,
                                                 double *out, size_t plane, int npad) {
  constexpr int NF = 2 * L + 1 > ncart_of(L) ? 2 * L + 1 : ncart_of(L);
  double v[NF], gx[DERIV ? NF : 1], gy[DERIV ? NF : 1], gz[DERIV ? NF : 1];
  shell_values<L, DERIV, double>(c_sph, pure, x, y, z, R, dR, sh.fac, v, gx, gy, gz);
  for (int f = 0; f < sh.nfunc; f++) {
    size_t o = static_cast<size_t>(f) * npad;
    out[o] = valid ? v[f] : 0.0;
    if (DERIV) {
      out[plane + o] = valid ? gx[f] : 0.0;
      out[2 * plane + o] = valid ? gy[f] : 0.0;
      out[3 * plane + o] = valid ? gz[f] : 0.0;
    }
  }
}

template <bool DERIV>
__global__ void __launch_bounds__(128) k_colloc_f64(MolDev m, double *__restrict__ ws) {
  const DevLeaf L = m.leaves[blockIdx.x];
  double *base = ws + L.ws_off;
  const size_t plane = static_cast<size_t>(L.mpad) * L.npad;
  for (int p = threadIdx.x; p < L.npad; p += blockDim.x) {
    const bool valid = p < L.cnt;
    const Pt4 P = valid ? m.pts[L.off + p] : make_pt4(0.0, 0.0, 0.0, 0.0);
    int loc = 0;
    for (int k = L.sh_begin; k < L.sh_end; k++) {
      const DevShell sh = m.shells[m.leaf_sh[k]];
      const double x = P.x - sh.A[0], y = P.y - sh.A[1], z = P.z - sh.A[2];
      const double r2 = x * x + y * y + z * z;
      double R = 0.0, dR = 0.0;
      for (int q = 0; q < sh.nprim; q++) {
        const double2 ec = m.prims[sh.prim_off + q];
        const double e = ec.y * exp(-ec.x * r2);
        R += e;
        dR -= 2.0 * ec.x * e;
      }
      double *out = base + static_cast<size_t>(loc) * L.npad + p;
      switch (sh.l) {
      case 0: colloc_store_f64<0, DERIV>(sh, m.pure, x, y, z, R, dR, valid, out, plane, L.npad); break;
      case 1: colloc_store_f64<1, DERIV>(sh, m.pure, x, y, z, R, dR, valid, out, plane, L.npad); break;
      case 2: colloc_store_f64<2, DERIV>(sh, m.pure, x, y, z, R, dR, valid, out, plane, L.npad); break;
      case 3: colloc_store_f64<3, DERIV>(sh, m.pure, x, y, z, R, dR, valid, out, plane, L.npad); break;
      default: colloc_store_f64<4, DERIV>(sh, m.pure, x, y, z, R, dR, valid, out, plane, L.npad); break;
      }
      loc += sh.nfunc;
    }
    for (int f = loc; f < L.mpad; f++) {
      size_t o = static_cast<size_t>(f) * L.npad + p;
      base[o] = 0.0;
      if (DERIV) {
        base[plane + o] = 0.0;
        base[2 * plane + o] = 0.0;
        base[3 * plane + o] = 0.0;
      }
    }
  }
}

// acc[i][j] += sum_kk A[kk][ta + 16 i] B[kk][tb + 16 j] over one staged
// chunk, i < NI and j < NJ: the 16-row groups of a tile that lie wholly past
// the leaf's points or AOs are not computed, which keeps the executed FLOPs
// near the useful ones (0.91 of them for the 32-water cluster, against 0.80
// and 0.69 for whole 64 x 64 tiles) for leaves whose sizes are not
// multiples of 64.
template <int NI, int NJ, int LDA, int LDB>
__device__ __forceinline__ void mac_chunk(const double (*As)[LDA], const double (*Bs)[LDB],
                                          double (&acc)[4][4], int ta, int tb) {
#pragma unroll
  for (int kk = 0; kk < kKChunk; kk++) {
    double a[NI], b[NJ];
#pragma unroll
    for (int i = 0; i < NI; i++)
      a[i] = As[kk][ta + 16 * i];
#pragma unroll
    for (int j = 0; j < NJ; j++)
      b[j] = Bs[kk][tb + 16 * j];
#pragma unroll
    for (int i = 0; i < NI; i++)
#pragma unroll
      for (int j = 0; j < NJ; j++)
        acc[i][j] = fma(a[i], b[j], acc[i][j]);
  }
}
// ni, nj: 16-row groups to compute (1..4), uniform over the CTA
template <int LDA, int LDB>
__device__ __forceinline__ void mac_chunk_n(const double (*As)[LDA], const double (*Bs)[LDB],
                                            double (&acc)[4][4], int ta, int tb, int ni, int nj) {
#define OCCX_MAC_CASE(I, J)                                                                        \
  case (I - 1) * 4 + (J - 1):                                                                      \
    mac_chunk<I, J>(As, Bs, acc, ta, tb);                                                          \
    break;
  switch ((ni - 1) * 4 + (nj - 1)) {
    OCCX_MAC_CASE(1, 1) OCCX_MAC_CASE(1, 2) OCCX_MAC_CASE(1, 3) OCCX_MAC_CASE(1, 4)
    OCCX_MAC_CASE(2, 1) OCCX_MAC_CASE(2, 2) OCCX_MAC_CASE(2, 3) OCCX_MAC_CASE(2, 4)
    OCCX_MAC_CASE(3, 1) OCCX_MAC_CASE(3, 2) OCCX_MAC_CASE(3, 3) OCCX_MAC_CASE(3, 4)
    OCCX_MAC_CASE(4, 1) OCCX_MAC_CASE(4, 2) OCCX_MAC_CASE(4, 3)
  default:
    mac_chunk<4, 4>(As, Bs, acc, ta, tb);
  }
#undef OCCX_MAC_CASE
}
// 16-row groups of a 64-wide tile starting at t0 that hold any of n rows
__device__ __forceinline__ int groups16(int n, int t0) {
  return max(1, min(4, (n - t0 + 15) / 16));
}

// rho for one 64-point slab of one leaf.  Thread (tx, ty): points
// p0 + tx + 16 i, AOs j0 + ty + 16 jj.
// TAU (meta-GGA, grid.y = 3): the same GEMM on the derivative plane
// k = 1 + blockIdx.y, (d_k phi) D2 (d_k phi) into rho component 4 + blockIdx.y
// (tau = half their sum, src/gto/density.cpp:86-100).
template <bool DERIV, bool TAU = false>
__global__ void __launch_bounds__(256, 2) k_rho_f64(MolDev m, const double *__restrict__ D,
                                                 const double *__restrict__ ws,
                                                 const SlabItem *__restrict__ slabs,
                                                 double *__restrict__ rho) {
  constexpr int NC = (DERIV && !TAU) ? 4 : 1;
  __shared__ double As[kKChunk][kPtTile];
  __shared__ double Bs[kKChunk][kAoTile];
  __shared__ double red[16][NC][kPtTile];
  const SlabItem it = slabs[blockIdx.x];
  const DevLeaf L = m.leaves[it.leaf];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const size_t plane = static_cast<size_t>(L.mpad) * L.npad;
  const double *phi = ws + L.ws_off + (TAU ? (1 + blockIdx.y) * plane : 0);
  const int *g = m.leaf_ao + L.ao_begin;
  const size_t nbf = static_cast<size_t>(m.nbf);
  double part[NC][4];
#pragma unroll
  for (int c = 0; c < NC; c++)
#pragma unroll
    for (int i = 0; i < 4; i++)
      part[c][i] = 0.0;

  // the 16-point groups of the slab and 16-AO groups of the tile past the
  // leaf's points and AOs are not computed
  const int gi = groups16(L.cnt, it.p0);
  for (int j0 = 0; j0 < L.mpad; j0 += kAoTile) {
    const int gj = groups16(L.nbf, j0);
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++)
        acc[i][j] = 0.0;
    // AOs at and beyond nbf contribute zeros: the reduction stops at the
    // first chunk boundary past them
    const int kend = (L.nbf + kKChunk - 1) / kKChunk * kKChunk;
    for (int k0 = 0; k0 < kend; k0 += kKChunk) {
#pragma unroll
      for (int r = 0; r < 4; r++) {
        int idx = threadIdx.x + r * 256;
        int kk = idx >> 6, pp = idx & 63;
        As[kk][pp] = phi[static_cast<size_t>(k0 + kk) * L.npad + it.p0 + pp];
        int kb = idx & 15, jb = idx >> 4;
        int k = k0 + kb, j = j0 + jb;
        double dv = 0.0;
        if (k < L.nbf && j < L.nbf)
          dv = 2.0 * D[static_cast<size_t>(g[j]) * nbf + g[k]];
        Bs[kb][jb] = dv;
      }
      __syncthreads();
      mac_chunk_n<kPtTile, kAoTile>(As, Bs, acc, tx, ty, gi, gj);
      __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const size_t row = static_cast<size_t>(j0 + ty + 16 * j) * L.npad + it.p0;
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const size_t o = row + tx + 16 * i;
        part[0][i] = fma(phi[o], acc[i][j], part[0][i]);
        if (DERIV && !TAU) {
          part[1][i] = fma(phi[plane + o], acc[i][j], part[1][i]);
          part[2][i] = fma(phi[2 * plane + o], acc[i][j], part[2][i]);
          part[3][i] = fma(phi[3 * plane + o], acc[i][j], part[3][i]);
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < NC; c++)
#pragma unroll
    for (int i = 0; i < 4; i++)
      red[ty][c][tx + 16 * i] = part[c][i];
  __syncthreads();
  for (int q = threadIdx.x; q < NC * kPtTile; q += 256) {
    const int c = q / kPtTile, p = q % kPtTile;
    double s = 0.0;
    for (int t = 0; t < 16; t++)
      s += red[t][c][p];
    const int lp = it.p0 + p;
    if (lp >= L.cnt)
      continue;
    if (TAU)
      rho[static_cast<size_t>(4 + blockIdx.y) * m.npts + L.off + lp] = s;
    else
      rho[static_cast<size_t>(c) * m.npts + L.off + lp] = (c == 0) ? s : 2.0 * s;
  }
}

__device__ __forceinline__ double block_sum_256(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (blockDim.x >> 5); i++)
      s += sh[i];
  __syncthreads();
  return s;
}


// One CTA per leaf (<= 256 points).
template <bool DERIV>
__global__ void __launch_bounds__(256) k_func(MolDev m, FuncSet fs, double thr,
                                              const double *__restrict__ rho,
                                              double *__restrict__ coef,
                                              double *__restrict__ epart) {
  __shared__ double sh[8];
  leaf_functional<DERIV>(m.leaves[blockIdx.x], m.pts, static_cast<size_t>(m.npts), fs, thr, rho,
                         coef, epart + 2 * blockIdx.x, sh);
}

__global__ void __launch_bounds__(256) k_func_mgga(MolDev m, FuncSet fs, double thr,
                                                   const double *__restrict__ rho,
                                                   double *__restrict__ coef,
                                                   double *__restrict__ epart) {
  __shared__ double sh[8];
  leaf_functional_mgga(m.leaves[blockIdx.x], m.pts, static_cast<size_t>(m.npts), fs, thr, rho,
                       coef, epart + 2 * blockIdx.x, sh);
}

// K = phi_I^T Y_J for one 64x64 AO tile of one leaf; V += K + K^T.
// Thread (tx, ty): K rows i0 + ty + 16 a, columns j0 + tx + 16 b.
// META adds sum_k (d_k phi_I)^T diag(c_tau) (d_k phi_J) with c_tau =
// 0.25 w vtau (coefficient component 4), so that K + K^T carries the
// tau term of src/dft/xc_potential_matrix.cpp:43-58 once.
template <bool DERIV, bool META = false>
__global__ void __launch_bounds__(256) k_vxc_f64(MolDev m, const double *__restrict__ ws,
                                                 const double *__restrict__ coef,
                                                 const TileItem *__restrict__ tiles,
                                                 double *__restrict__ V) {
  __shared__ double As[kKChunk][kAoTile + 1];
  __shared__ double Bs[kKChunk][kAoTile + 1];
  const TileItem it = tiles[blockIdx.x];
  const DevLeaf L = m.leaves[it.leaf];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const double *phi = ws + L.ws_off;
  const size_t plane = static_cast<size_t>(L.mpad) * L.npad;
  const size_t N = static_cast<size_t>(m.npts);
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
      acc[a][b] = 0.0;
  constexpr int NSEG = META ? 4 : 1;
  // the 16-AO groups of the tile past the leaf's AOs are not computed
  const int gi = groups16(L.nbf, it.i0), gj = groups16(L.nbf, it.j0);
  for (int seg = 0; seg < NSEG; seg++)
  for (int p0 = 0; p0 < (L.cnt + kKChunk - 1) / kKChunk * kKChunk; p0 += kKChunk) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = threadIdx.x + r * 256;
      const int pp = idx & 15, aa = idx >> 4;
      const int p = p0 + pp;
      const double *a = phi + seg * plane; // seg 0: phi; 1..3: d_k phi
      As[pp][aa] = a[static_cast<size_t>(it.i0 + aa) * L.npad + p];
      const size_t o = static_cast<size_t>(it.j0 + aa) * L.npad + p;
      double y = 0.0;
      if (p < L.cnt) {
        const size_t gi = static_cast<size_t>(L.off) + p;
        if (seg == 0) {
          y = coef[gi] * phi[o];
          if (DERIV)
            y += coef[N + gi] * phi[plane + o] + coef[2 * N + gi] * phi[2 * plane + o] +
                 coef[3 * N + gi] * phi[3 * plane + o];
        } else {
          y = coef[4 * N + gi] * a[o];
        }
      }
      Bs[pp][aa] = y;
    }
    __syncthreads();
    mac_chunk_n<kAoTile + 1, kAoTile + 1>(As, Bs, acc, ty, tx, gi, gj);
    __syncthreads();
  }
  const int *g = m.leaf_ao + L.ao_begin;
  const size_t nbf = static_cast<size_t>(m.nbf);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int li = it.i0 + ty + 16 * i;
    if (li >= L.nbf)
      continue;
    const size_t gi = g[li];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int lj = it.j0 + tx + 16 * j;
      if (lj >= L.nbf)
        continue;
      const size_t gj = g[lj];
      atomicAdd(&V[gj * nbf + gi], acc[i][j]);
      atomicAdd(&V[gi * nbf + gj], acc[i][j]);
    }
  }
}

__global__ void __launch_bounds__(256) k_reduce(const double *__restrict__ epart, int n,
                                                double *__restrict__ out2) {
  __shared__ double sh[8];
  double e = 0.0, ne = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) {
    e += epart[2 * i];
    ne += epart[2 * i + 1];
  }
  e = block_sum_256(e, sh);
  ne = block_sum_256(ne, sh);
  if (threadIdx.x == 0) {
    out2[0] = e;
    out2[1] = ne;
  }
}

void fill_sph_table(double *out);

void upload_sph_table() {
  double h[kSphTableSize];
  fill_sph_table(h);
  cudaMemcpyToSymbol(c_sph, h, sizeof(h));
}

void launch_colloc_f64(const MolDev &m, int deriv, double *ws, cudaStream_t st) {
  if (m.nleaves == 0)
    return;
  if (deriv)
    k_colloc_f64<true><<<m.nleaves, 128, 0, st>>>(m, ws);
  else
    k_colloc_f64<false><<<m.nleaves, 128, 0, st>>>(m, ws);
}

void launch_rho_f64(const MolDev &m, int deriv, const double *D, const double *ws,
                    const SlabItem *slabs, int nslabs, double *rho, cudaStream_t st) {
  if (nslabs == 0)
    return;
  if (deriv)
    k_rho_f64<true><<<nslabs, 256, 0, st>>>(m, D, ws, slabs, rho);
  else
    k_rho_f64<false><<<nslabs, 256, 0, st>>>(m, D, ws, slabs, rho);
}

void launch_tau_f64(const MolDev &m, const double *D, const double *ws, const SlabItem *slabs,
                    int nslabs, double *rho, cudaStream_t st) {
  if (nslabs == 0)
    return;
  k_rho_f64<true, true><<<dim3(nslabs, 3), 256, 0, st>>>(m, D, ws, slabs, rho);
}

void launch_func(const MolDev &m, int deriv, const FuncSet &fs, double thr, const double *rho,
                 double *coef, double *epart, cudaStream_t st) {
  if (m.nleaves == 0)
    return;
  if (deriv == 2)
    k_func_mgga<<<m.nleaves, 256, 0, st>>>(m, fs, thr, rho, coef, epart);
  else if (deriv)
    k_func<true><<<m.nleaves, 256, 0, st>>>(m, fs, thr, rho, coef, epart);
  else
    k_func<false><<<m.nleaves, 256, 0, st>>>(m, fs, thr, rho, coef, epart);
}

void launch_vxc_f64(const MolDev &m, int deriv, const double *ws, const double *coef,
                    const TileItem *tiles, int ntiles, double *V, cudaStream_t st) {
  if (ntiles == 0)
    return;
  if (deriv == 2)
    k_vxc_f64<true, true><<<ntiles, 256, 0, st>>>(m, ws, coef, tiles, V);
  else if (deriv)
    k_vxc_f64<true><<<ntiles, 256, 0, st>>>(m, ws, coef, tiles, V);
  else
    k_vxc_f64<false><<<ntiles, 256, 0, st>>>(m, ws, coef, tiles, V);
}

void launch_reduce(const double *epart, int nleaves, double *out2, cudaStream_t st) {
  k_reduce<<<1, 256, 0, st>>>(epart, nleaves, out2);
}

} // namespace occx
