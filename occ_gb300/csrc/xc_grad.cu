// XC nuclear gradient, dE_xc/dR_A with the grid held fixed (OCC's
// DFT::compute_xc_gradient, include/occ/dft/dft.h:599-749, with the kernels
// of src/dft/dft_gradient_kernels.cpp:472-595), restricted, FP64.
//
// OCC forms per leaf and Cartesian direction c the matrix
//   V_c(mu, nu) = sum_p d_c phi_mu Y_nu + Z_c,mu phi_nu
//   Y  = 0.5 w vrho phi + 2 w vsigma grad rho . grad phi
//   Z_c = 0.5 w vrho d_c phi + 2 w vsigma grad rho . grad d_c phi
// (for an LDA Y = w vrho phi and Z = 0, which is the same sum), and
// subtracts V_c(mu, nu) * 4 D(mu, nu) from the gradient of mu's atom,
// skipping |4 D| < 1e-12 (dft_gradient_kernels.cpp:535-547).  The sum over nu
// is taken first here:
//   g_A,c -= sum_{mu on A} sum_p [ d_c phi_mu W_mu + Z_c,mu X_mu ]
//   X_mu = sum_nu 4D(mu, nu) phi_nu,   W_mu = sum_nu 4D(mu, nu) Y_nu
// two m x m x 64-point DFMA contractions per slab instead of three m x m
// products per direction, then per-point work; the result is the same sum
// reassociated.
//
// Per build of the gradient, leaf group by leaf group (a group's workspace is
// capped so that any molecule fits):
//   k_colloc2_f64  phi, grad phi and, for a GGA, the six second derivatives
//                  (gau2grid's deriv-2 collocation, src/gto/gto.cpp:212-287)
//   k_rho_f64      rho, grad rho (the build's own kernel)
//   k_func         0.5 w vrho, 2 w vsigma grad rho (the build's own kernel)
//   k_grad_f64     X, W per 64-point slab and 64-AO tile; per-AO sums over
//                  the slab reduced over runs of AOs on one atom, then one
//                  atomic add per atom and direction
// and for a meta-GGA the tau density (the build's k_rho_f64 tau mode) and the
// tau term (k_grad_f64's TAU mode, one derivative plane k per grid row).
#include <algorithm>

#include "host/gto_eval.h"
#include "xc_device.cuh"
#include "xc_engine.hpp"
#include "xc_leaf_func.cuh"

namespace occx {

namespace {

__constant__ double c_sph2[kSphTableSize];

constexpr double kGradDensitySkip = 1e-12;          // |4 D| below this is skipped

// n-th falling factorial of a (n <= 2).
__device__ __forceinline__ double ffac(int a, int n) {
  return n == 0 ? 1.0 : (n == 1 ? double(a) : double(a) * double(a - 1));
}

// d^(nx,ny,nz) of x^a y^b z^c from the power tables.
template <int L>
__device__ __forceinline__ double dmono(const double *px, const double *py, const double *pz, int a,
                                        int b, int c, int nx, int ny, int nz) {
  if (a < nx || b < ny || c < nz)
    return 0.0;
  return ffac(a, nx) * ffac(b, ny) * ffac(c, nz) * px[a - nx] * py[b - ny] * pz[c - nz];
}

// Component q of the Cartesian functions of one shell at one point:
// q = 0 value, 1..3 d/dx, d/dy, d/dz, 4..9 xx, xy, xz, yy, yz, zz.  With
// R(r^2) the contracted radial part, dR = sum -2 a c e and d2R = sum 4 a^2 c e:
//   d_i (M R)    = M_i R + M x_i dR
//   d_ij (M R)   = M_ij R + (M_i x_j + M_j x_i) dR + M (delta_ij dR + x_i x_j d2R)
template <int L>
__device__ __forceinline__ void cart_component(int q, double x, double y, double z, double R,
                                               double dR, double d2R, double *out) {
  double px[L + 1], py[L + 1], pz[L + 1];
  px[0] = py[0] = pz[0] = 1.0;
#pragma unroll
  for (int i = 1; i <= L; i++) {
    px[i] = px[i - 1] * x;
    py[i] = py[i - 1] * y;
    pz[i] = pz[i - 1] * z;
  }
  const int ai = q == 0 ? -1 : (q <= 3 ? q - 1 : (q <= 6 ? 0 : (q <= 8 ? 1 : 2)));
  const int aj = q <= 3 ? -1 : (q == 4 ? 0 : (q == 5 ? 1 : (q == 6 ? 2 : (q == 7 ? 1 : 2))));
  const double r[3] = {x, y, z};
  int k = 0;
#pragma unroll
  for (int a = L; a >= 0; a--) {
#pragma unroll
    for (int b = L - a; b >= 0; b--) {
      const int c = L - a - b;
      const double M = px[a] * py[b] * pz[c];
      double v;
      if (ai < 0) {
        v = M * R;
      } else if (aj < 0) {
        const double Mi = dmono<L>(px, py, pz, a, b, c, ai == 0, ai == 1, ai == 2);
        v = Mi * R + M * r[ai] * dR;
      } else {
        const double Mi = dmono<L>(px, py, pz, a, b, c, ai == 0, ai == 1, ai == 2);
        const double Mj = dmono<L>(px, py, pz, a, b, c, aj == 0, aj == 1, aj == 2);
        const double Mij = dmono<L>(px, py, pz, a, b, c, (ai == 0) + (aj == 0),
                                    (ai == 1) + (aj == 1), (ai == 2) + (aj == 2));
        v = Mij * R + (Mi * r[aj] + Mj * r[ai]) * dR +
            M * ((ai == aj ? dR : 0.0) + r[ai] * r[aj] * d2R);
      }
      out[k++] = v;
    }
  }
}

template <int L, int NQ>
__device__ __forceinline__ void colloc2_store(const DevShell &sh, bool pure, double x, double y,
                                              double z, double R, double dR, double d2R,
                                              bool valid, double *out, size_t plane, int npad) {
  constexpr int NC = ncart_of(L);
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    double cv[NC];
    cart_component<L>(q, x, y, z, R, dR, d2R, cv);
    double *o = out + q * plane;
    if (pure) { // the transform of src/gto/gto.cpp (for l = 1 OCC's (y, z, x) order)
      const double *Tm = c_sph2 + sph_offset(L);
#pragma unroll
      for (int f = 0; f < 2 * L + 1; f++) {
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < NC; c++)
          s += Tm[f * NC + c] * cv[c];
        o[static_cast<size_t>(f) * npad] = valid ? s * sh.fac : 0.0;
      }
    } else {
#pragma unroll
      for (int f = 0; f < NC; f++)
        o[static_cast<size_t>(f) * npad] = valid ? cv[f] * sh.fac : 0.0;
    }
  }
}

// One CTA per leaf of the group; NQ planes (4: LDA, 10: GGA).
template <int NQ>
__global__ void __launch_bounds__(128) k_colloc2_f64(MolDev m, double *__restrict__ ws) {
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
      double R = 0.0, dR = 0.0, d2R = 0.0;
      for (int q = 0; q < sh.nprim; q++) {
        const double2 ec = m.prims[sh.prim_off + q];
        const double e = ec.y * exp(-ec.x * r2);
        R += e;
        dR -= 2.0 * ec.x * e;
        d2R += 4.0 * ec.x * ec.x * e;
      }
      double *out = base + static_cast<size_t>(loc) * L.npad + p;
      switch (sh.l) {
      case 0: colloc2_store<0, NQ>(sh, m.pure, x, y, z, R, dR, d2R, valid, out, plane, L.npad); break;
      case 1: colloc2_store<1, NQ>(sh, m.pure, x, y, z, R, dR, d2R, valid, out, plane, L.npad); break;
      case 2: colloc2_store<2, NQ>(sh, m.pure, x, y, z, R, dR, d2R, valid, out, plane, L.npad); break;
      case 3: colloc2_store<3, NQ>(sh, m.pure, x, y, z, R, dR, d2R, valid, out, plane, L.npad); break;
      default: colloc2_store<4, NQ>(sh, m.pure, x, y, z, R, dR, d2R, valid, out, plane, L.npad); break;
      }
      loc += sh.nfunc;
    }
    for (int f = loc; f < L.mpad; f++)
#pragma unroll
      for (int q = 0; q < NQ; q++)
        base[q * plane + static_cast<size_t>(f) * L.npad + p] = 0.0;
  }
}

// Hessian plane of (c, k): xx 4, xy 5, xz 6, yy 7, yz 8, zz 9.
__device__ __forceinline__ int hplane(int c, int k) {
  const int lo = c < k ? c : k, hi = c < k ? k : c;
  return lo == 0 ? 4 + hi : (lo == 1 ? 6 + hi : 9);
}

// One 64-point slab of one leaf.  Thread (tx, ty): points p0 + tx + 16 i,
// AOs mu = i0 + ty + 16 j of the current 64-AO tile.
// TAU (meta-GGA, grid.y = 3, k = blockIdx.y): the tau term of
// accumulate_gradient_contribution_R<2> (src/dft/dft_gradient_kernels.cpp:
// 151-172), V_c(mu, nu) += sum_p d_c d_k phi_mu (0.5 w vtau) d_k phi_nu, as
//   g_A,c -= sum_{mu on A} sum_p d_c d_k phi_mu (0.5 w vtau) T_k,mu,
//   T_k,mu = sum_nu 4D(mu, nu) d_k phi_nu  (the same GEMM on plane 1 + k).
template <bool GGA, bool TAU = false>
__global__ void __launch_bounds__(256) k_grad_f64(MolDev m, const double *__restrict__ D,
                                                  const double *__restrict__ ws,
                                                  const double *__restrict__ coef,
                                                  const SlabItem *__restrict__ slabs,
                                                  const int *__restrict__ ao_atom,
                                                  double *__restrict__ grad,
                                                  const double *__restrict__ Dot) {
  __shared__ double Ps[kKChunk][kPtTile];
  __shared__ double Ys[GGA ? kKChunk : 1][kPtTile];
  __shared__ double Ds[kKChunk][kAoTile];
  __shared__ double gs[3][kAoTile];
  const SlabItem it = slabs[blockIdx.x];
  const DevLeaf L = m.leaves[it.leaf];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const double *phi = ws + L.ws_off;
  const size_t plane = static_cast<size_t>(L.mpad) * L.npad;
  const size_t N = static_cast<size_t>(m.npts);
  const int *g = m.leaf_ao + L.ao_begin;
  const size_t nbf = static_cast<size_t>(m.nbf);
  const int kd = TAU ? static_cast<int>(blockIdx.y) : 0;
  const double *pha = phi + (TAU ? (1 + kd) * plane : 0); // the GEMM's AO operand

  // functional coefficients of this thread's points (zero past the leaf)
  double c0[4], cg[GGA ? 3 : 1][4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int lp = it.p0 + tx + 16 * i;
    const bool ok = lp < L.cnt;
    const size_t gp = static_cast<size_t>(L.off) + (ok ? lp : 0);
    c0[i] = ok ? (TAU ? 2.0 * coef[4 * N + gp] : coef[gp]) : 0.0; // TAU: 0.5 w vtau
    if (GGA)
#pragma unroll
      for (int k = 0; k < 3; k++)
        cg[k][i] = ok ? coef[(k + 1) * N + gp] : 0.0;
  }

  for (int i0 = 0; i0 < L.mpad; i0 += kAoTile) {
    double X[4][4], W[GGA ? 4 : 1][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
        X[i][j] = 0.0;
        if (GGA)
          W[i][j] = 0.0;
      }
    for (int k0 = 0; k0 < (L.nbf + kKChunk - 1) / kKChunk * kKChunk; k0 += kKChunk) {
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const int idx = threadIdx.x + r * 256;
        const int kk = idx >> 6, pp = idx & 63;
        const size_t o = static_cast<size_t>(k0 + kk) * L.npad + it.p0 + pp;
        const double f = pha[o];
        Ps[kk][pp] = f;
        if (GGA) {
          const int lp = it.p0 + pp;
          double y = 0.0;
          if (lp < L.cnt) {
            const size_t gp = static_cast<size_t>(L.off) + lp;
            y = coef[gp] * f + coef[N + gp] * phi[plane + o] +
                coef[2 * N + gp] * phi[2 * plane + o] + coef[3 * N + gp] * phi[3 * plane + o];
          }
          Ys[kk][pp] = y;
        }
        const int kb = idx & 15, jb = idx >> 4;
        const int nu = k0 + kb, mu = i0 + jb;
        double dv = 0.0;
        if (nu < L.nbf && mu < L.nbf) {
          const size_t e = static_cast<size_t>(g[nu]) * nbf + g[mu];
          dv = 4.0 * D[e];
          // the reference's skip: |4 D| restricted, |2 (D_a + D_b)| unrestricted
          if (fabs(Dot ? 2.0 * (D[e] + Dot[e]) : dv) < kGradDensitySkip)
            dv = 0.0;
        }
        Ds[kb][jb] = dv;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kKChunk; kk++) {
        double a[4], y[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          a[i] = Ps[kk][tx + 16 * i];
          if (GGA)
            y[i] = Ys[kk][tx + 16 * i];
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
          b[j] = Ds[kk][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            X[i][j] = fma(a[i], b[j], X[i][j]);
            if (GGA)
              W[i][j] = fma(y[i], b[j], W[i][j]);
          }
      }
      __syncthreads();
    }
    // per AO: sum over this thread's points of d_c phi W + Z_c X
    double s[4][3];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const size_t row = static_cast<size_t>(i0 + ty + 16 * j) * L.npad + it.p0;
#pragma unroll
      for (int c = 0; c < 3; c++)
        s[j][c] = 0.0;
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const size_t o = row + tx + 16 * i;
        double dphi[3];
#pragma unroll
        for (int c = 0; c < 3; c++)
          dphi[c] = phi[(c + 1) * plane + o];
        if (TAU) {
#pragma unroll
          for (int c = 0; c < 3; c++)
            s[j][c] = fma(c0[i] * phi[hplane(c, kd) * plane + o], X[i][j], s[j][c]);
        } else if (GGA) {
          double h[6];
#pragma unroll
          for (int q = 0; q < 6; q++)
            h[q] = phi[(4 + q) * plane + o];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            double z = c0[i] * dphi[c];
#pragma unroll
            for (int k = 0; k < 3; k++)
              z = fma(cg[k][i], h[hplane(c, k) - 4], z);
            s[j][c] = fma(dphi[c], W[i][j], fma(z, X[i][j], s[j][c]));
          }
        } else {
#pragma unroll
          for (int c = 0; c < 3; c++)
            s[j][c] = fma(2.0 * c0[i] * dphi[c], X[i][j], s[j][c]);
        }
      }
    }
    // reduce over the 16 point lanes (tx) of each half-warp
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        double v = s[j][c];
#pragma unroll
        for (int o = 8; o > 0; o >>= 1)
          v += __shfl_xor_sync(0xffffffffu, v, o);
        if (tx == 0)
          gs[c][ty + 16 * j] = v;
      }
    __syncthreads();
    // runs of AOs on one atom: one atomic add per run and direction
    if (threadIdx.x < 3) {
      const int c = threadIdx.x;
      const int mu_end = min(kAoTile, L.nbf - i0);
      int cur = -1;
      double run = 0.0;
      for (int u = 0; u < mu_end; u++) {
        const int atom = ao_atom[g[i0 + u]];
        if (atom != cur) {
          if (cur >= 0)
            atomicAdd(&grad[3 * cur + c], -run);
          cur = atom;
          run = 0.0;
        }
        run += gs[c][u];
      }
      if (cur >= 0)
        atomicAdd(&grad[3 * cur + c], -run);
    }
    __syncthreads();
  }
}

} // namespace

void upload_sph_table_grad() {
  double h[kSphTableSize];
  fill_sph_table(h);
  cuda_check(cudaMemcpyToSymbol(c_sph2, h, sizeof(h)), "cudaMemcpyToSymbol");
}

// Gradient leaves (the build's leaves, workspace offsets for 4 or 10 planes,
// relative to their group), their slabs, leaf groups under the workspace cap,
// and the AO -> atom map.  Allocated on the first gradient of a molecule.
void Molecule::prepare_gradient() {
  if (d_gws)
    return;
  if (!d_pts)
    throw ArgError("the molecule has no device state");
  const double bytes_before = device_bytes;
  const int nq = deriv ? 10 : 4;
  const size_t cap = std::max<size_t>(grad_ws_cap_bytes / sizeof(double), 1);
  // leaves by descending cost (m^2 n): groups of similar leaves, and within a
  // launch the longest slabs first, so that no launch ends on a tail of a
  // few long CTAs
  std::vector<int> order(leaves.size());
  for (size_t i = 0; i < order.size(); i++)
    order[i] = static_cast<int>(i);
  auto cost = [&](int i) {
    return static_cast<double>(leaves[i].mpad) * leaves[i].mpad * leaves[i].npad;
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(a) > cost(b); });
  std::vector<DevLeaf> gl(leaves.size());
  std::vector<SlabItem> gsl;
  ggroups.clear();
  size_t off = 0, max_ws = 0;
  GradGroup cur{0, 0, 0, 0};
  for (size_t k = 0; k < order.size(); k++) {
    gl[k] = leaves[order[k]];
    const size_t e = static_cast<size_t>(nq) * gl[k].mpad * gl[k].npad;
    if (cur.nleaf > 0 && off + e > cap) {
      ggroups.push_back(cur);
      cur = GradGroup{static_cast<int>(k), 0, static_cast<int>(gsl.size()), 0};
      off = 0;
    }
    gl[k].ws_off = static_cast<long long>(off);
    off += e;
    max_ws = std::max(max_ws, off);
    for (int p0 = 0; p0 < gl[k].npad; p0 += kPtTile) {
      gsl.push_back({cur.nleaf, p0});
      cur.nslab++;
    }
    cur.nleaf++;
  }
  if (cur.nleaf > 0)
    ggroups.push_back(cur);
  std::vector<int> ao_atom(std::max(basis.nbf, 1));
  for (size_t s = 0; s < basis.shells.size(); s++)
    for (int f = 0; f < basis.shell_size(static_cast<int>(s)); f++)
      ao_atom[basis.first_bf[s] + f] = basis.shells[s].atom;
  size_t bytes = 0;
  d_gleaves = dev_upload(gl, bytes);
  allocations.push_back(d_gleaves);
  d_gslabs = dev_upload(gsl, bytes);
  allocations.push_back(d_gslabs);
  d_ao_atom = dev_upload(ao_atom, bytes);
  allocations.push_back(d_ao_atom);
  device_bytes += static_cast<double>(bytes);
  d_grad = static_cast<double *>(alloc(std::max<size_t>(3 * Z.size(), 1) * sizeof(double)));
  d_gws = static_cast<double *>(alloc(std::max<size_t>(max_ws, 1) * sizeof(double)));
  grad_bytes = device_bytes - bytes_before;
}

void Molecule::release_gradient() {
  for (void *p : {static_cast<void *>(d_gleaves), static_cast<void *>(d_gslabs),
                  static_cast<void *>(d_ao_atom), static_cast<void *>(d_gws),
                  static_cast<void *>(d_grad)}) {
    if (!p)
      continue;
    auto it = std::find(allocations.begin(), allocations.end(), p);
    if (it != allocations.end()) {
      allocations.erase(it);
      cudaFree(p);
    }
  }
  ggroups.clear();
  d_gleaves = nullptr;
  d_gslabs = nullptr;
  d_ao_atom = nullptr;
  d_gws = d_grad = nullptr;
  device_bytes -= grad_bytes;
  grad_bytes = 0.0;
}

void Molecule::xc_gradient(const double *dD, double *dgrad, double *dout2, cudaStream_t st) {
  prepare_gradient();
  Context &c = *ctx;
  cuda_check(cudaMemsetAsync(dgrad, 0, 3 * Z.size() * sizeof(double), st), "cudaMemsetAsync");
  for (const GradGroup &G : ggroups) {
    MolDev m = dev();
    m.leaves = d_gleaves + G.leaf0;
    m.nleaves = G.nleaf;
    const SlabItem *sl = d_gslabs + G.slab0;
    c.launch("colloc2_f64", st, [&] {
      if (deriv)
        k_colloc2_f64<10><<<G.nleaf, 128, 0, st>>>(m, d_gws);
      else
        k_colloc2_f64<4><<<G.nleaf, 128, 0, st>>>(m, d_gws);
    });
    c.launch("rho_f64", st, [&] { launch_rho_f64(m, deriv, dD, d_gws, sl, G.nslab, d_rho, st); });
    if (deriv == 2)
      c.launch("tau_f64", st, [&] { launch_tau_f64(m, dD, d_gws, sl, G.nslab, d_rho, st); });
    c.launch("func", st, [&] {
      launch_func(m, deriv, fs, bs.density_threshold, d_rho, d_coef, d_epart + 2 * G.leaf0, st);
    });
    c.launch("grad_f64", st, [&] {
      if (deriv)
        k_grad_f64<true><<<G.nslab, 256, 0, st>>>(m, dD, d_gws, d_coef, sl, d_ao_atom, dgrad,
                                                  nullptr);
      else
        k_grad_f64<false><<<G.nslab, 256, 0, st>>>(m, dD, d_gws, d_coef, sl, d_ao_atom, dgrad,
                                                   nullptr);
    });
    if (deriv == 2)
      c.launch("grad_tau_f64", st, [&] {
        k_grad_f64<false, true><<<dim3(G.nslab, 3), 256, 0, st>>>(m, dD, d_gws, d_coef, sl,
                                                                  d_ao_atom, dgrad, nullptr);
      });
  }
  c.launch("reduce", st, [&] {
    launch_reduce(d_epart, static_cast<int>(leaves.size()), dout2, st);
  });
  cuda_check(cudaGetLastError(), "kernel launch");
}

// The unrestricted gradient (dft.h:599-749 with accumulate_gradient_
// contribution_U, src/dft/dft_gradient_kernels.cpp:175-470, distributed as
// :549-575, g -= 2 (V_c,a Da + V_c,b Db) with D2 = 2 mo.D): per spin the
// restricted kernels with that spin's mo.D block and coefficients (the UKS
// build's: 0.5 w vrho_s, w (2 vsigma_ss grad rho_s + vsigma_ab grad rho_s'),
// 0.25 w vtau_s), so that 4 D_s V_c,s is the reference's 2 Da V_c,a; elements
// skipped where |Da + Db| < 1e-12.  dD: OCC's 2 nbf x nbf; dout3 = {E_xc,
// integrated rho_a, integrated rho_b}.
void Molecule::xc_gradient_uks(const double *dD, double *dgrad, double *dout3,
                               cudaStream_t st) {
  prepare_gradient();
  prepare_uks();
  Context &c = *ctx;
  const size_t nbf = static_cast<size_t>(basis.nbf), nbf2 = nbf * nbf;
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(d_Dab + s * nbf2, nbf * sizeof(double), dD + s * nbf,
                                 2 * nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaMemsetAsync(dgrad, 0, 3 * Z.size() * sizeof(double), st), "cudaMemsetAsync");
  double *rho[2] = {d_rho, d_rho_b}, *coef[2] = {d_coef, d_coef_b};
  for (const GradGroup &G : ggroups) {
    MolDev m = dev();
    m.leaves = d_gleaves + G.leaf0;
    m.nleaves = G.nleaf;
    const SlabItem *sl = d_gslabs + G.slab0;
    c.launch("colloc2_f64", st, [&] {
      if (deriv)
        k_colloc2_f64<10><<<G.nleaf, 128, 0, st>>>(m, d_gws);
      else
        k_colloc2_f64<4><<<G.nleaf, 128, 0, st>>>(m, d_gws);
    });
    for (int s = 0; s < 2; s++) {
      const double *Ds = d_Dab + s * nbf2;
      c.launch("rho_f64", st, [&] { launch_rho_f64(m, deriv, Ds, d_gws, sl, G.nslab, rho[s], st); });
      if (deriv == 2)
        c.launch("tau_f64", st, [&] { launch_tau_f64(m, Ds, d_gws, sl, G.nslab, rho[s], st); });
    }
    c.launch("func_pol", st, [&] {
      launch_func_pol(m, deriv, fs, bs.density_threshold, d_rho, d_rho_b, d_coef, d_coef_b,
                      d_epart_u + 3 * G.leaf0, st);
    });
    for (int s = 0; s < 2; s++) {
      const double *Ds = d_Dab + s * nbf2, *Do = d_Dab + (1 - s) * nbf2;
      c.launch("grad_f64", st, [&] {
        if (deriv)
          k_grad_f64<true><<<G.nslab, 256, 0, st>>>(m, Ds, d_gws, coef[s], sl, d_ao_atom, dgrad,
                                                    Do);
        else
          k_grad_f64<false><<<G.nslab, 256, 0, st>>>(m, Ds, d_gws, coef[s], sl, d_ao_atom, dgrad,
                                                     Do);
      });
      if (deriv == 2)
        c.launch("grad_tau_f64", st, [&] {
          k_grad_f64<false, true><<<dim3(G.nslab, 3), 256, 0, st>>>(m, Ds, d_gws, coef[s], sl,
                                                                    d_ao_atom, dgrad, Do);
        });
    }
  }
  c.launch("reduce", st, [&] {
    launch_reduce3(d_epart_u, static_cast<int>(leaves.size()), dout3, st);
  });
  cuda_check(cudaGetLastError(), "kernel launch");
}

} // namespace occx

using namespace occx;

extern "C" {

int occ_xc_compute_xc_gradient(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D,
                               int precision, double *grad, double *exc) {
  if (!ctx || !mol || !D || !grad)
    return OCC_XC_ERR_ARG;
  if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    Molecule &M = *mol->impl;
    cudaStream_t st = ctx->impl->stream;
    const size_t nbf2 = static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
    double *dgrad;
    if (precision == OCC_XC_MIXED) {
      M.prepare_gradient_mixed();
      if (!M.d_grad)
        M.d_grad = static_cast<double *>(M.alloc(std::max<size_t>(3 * M.Z.size(), 1) *
                                                 sizeof(double)));
    } else {
      M.prepare_gradient();
    }
    dgrad = M.d_grad;
    cuda_check(cudaMemcpyAsync(M.d_D, D, nbf2 * sizeof(double), cudaMemcpyHostToDevice, st),
               "cudaMemcpyAsync H2D");
    if (precision == OCC_XC_MIXED)
      M.xc_gradient_mixed(M.d_D, dgrad, M.d_out2, st);
    else
      M.xc_gradient(M.d_D, dgrad, M.d_out2, st);
    double out2[2];
    cuda_check(cudaMemcpyAsync(grad, dgrad, 3 * M.Z.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaMemcpyAsync(out2, M.d_out2, sizeof(out2), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (precision == OCC_XC_MIXED && mixed_error_flag(M, st))
      throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
    if (exc)
      *exc = out2[0];
  });
}

int occ_xc_molecule_set_gradient_workspace_cap(occ_xc_context *ctx, occ_xc_molecule *mol,
                                              double bytes) {
  if (!ctx || !mol || !(bytes >= 0.0))
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    Molecule &M = *mol->impl;
    M.grad_ws_cap_bytes = bytes > 0.0 ? static_cast<size_t>(bytes) : kGradWsCapDefault;
    M.release_gradient();
  });
}

int occ_xc_compute_xc_gradient_device(occ_xc_context *ctx, occ_xc_molecule *mol,
                                      const double *d_D, int precision, double *d_grad,
                                      double *d_exc2, void *stream) {
  if (!ctx || !mol || !d_D || !d_grad)
    return OCC_XC_ERR_ARG;
  if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    Molecule &M = *mol->impl;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->impl->stream;
    if (precision == OCC_XC_MIXED)
      M.xc_gradient_mixed(d_D, d_grad, d_exc2 ? d_exc2 : M.d_out2, st);
    else
      M.xc_gradient(d_D, d_grad, d_exc2 ? d_exc2 : M.d_out2, st);
  });
}

int occ_xc_compute_xc_gradient_unrestricted(occ_xc_context *ctx, occ_xc_molecule *mol,
                                            const double *D, int precision, double *grad,
                                            double *exc) {
  if (!ctx || !mol || !D || !grad)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
      throw ArgError("precision must be OCC_XC_FP64 or OCC_XC_MIXED");
    Molecule &M = *mol->impl;
    cudaStream_t st = ctx->impl->stream;
    if (precision == OCC_XC_MIXED) {
      M.prepare_gradient_mixed();
      if (!M.d_grad)
        M.d_grad = static_cast<double *>(M.alloc(std::max<size_t>(3 * M.Z.size(), 1) *
                                                 sizeof(double)));
    } else {
      M.prepare_gradient();
    }
    M.prepare_uks();
    const size_t n2 = 2 * static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
    cuda_check(cudaMemcpyAsync(M.d_Duks, D, n2 * sizeof(double), cudaMemcpyHostToDevice, st),
               "cudaMemcpyAsync H2D");
    if (precision == OCC_XC_MIXED)
      M.xc_gradient_uks_mixed(M.d_Duks, M.d_grad, M.d_out3, st);
    else
      M.xc_gradient_uks(M.d_Duks, M.d_grad, M.d_out3, st);
    double out3[3];
    cuda_check(cudaMemcpyAsync(grad, M.d_grad, 3 * M.Z.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaMemcpyAsync(out3, M.d_out3, sizeof(out3), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (precision == OCC_XC_MIXED && mixed_error_flag(M, st))
      throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
    if (exc)
      *exc = out3[0];
  });
}

int occ_xc_compute_xc_gradient_unrestricted_device(occ_xc_context *ctx, occ_xc_molecule *mol,
                                                   const double *d_D, int precision,
                                                   double *d_grad, double *d_exc3,
                                                   void *stream) {
  if (!ctx || !mol || !d_D || !d_grad)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
      throw ArgError("precision must be OCC_XC_FP64 or OCC_XC_MIXED");
    Molecule &M = *mol->impl;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->impl->stream;
    if (precision == OCC_XC_MIXED)
      M.xc_gradient_uks_mixed(d_D, d_grad, d_exc3 ? d_exc3 : M.d_out3, st);
    else
      M.xc_gradient_uks(d_D, d_grad, d_exc3 ? d_exc3 : M.d_out3, st);
  });
}

} // extern "C"
