// Unrestricted (UKS) XC build, FP64: DFT::compute_vxc for
// SpinorbitalKind::Unrestricted (include/occ/dft/dft.h:395-429 ->
// compute_K_dft<deriv, Unrestricted>, dft.h:192-388).
//
// OCC's mo.D is 2 nbf x nbf (the alpha block above the beta block, each
// 0.5 C_s C_s^T, src/qm/orb.h:68-83); the build forms D2 = 2 D, so that
// rho_s = rowsum(phi o phi D2_s) (src/gto/density.cpp:44-70), evaluates the
// polarised functional on (rho_a, rho_b, s_aa, s_ab, s_bb)
// (include/occ/dft/dft_kernels.h:16-60), skips a leaf whose largest rho_a or
// rho_b is below the density threshold (src/dft/dft_kernels.cpp:37-40), and
// forms per spin (src/dft/xc_potential_matrix.cpp:61-105)
//   V_a = phi^T (w vrho_a phi) + phi^T G_a + G_a^T phi,
//   G_a = w (2 vs_aa grad rho_a + vs_ab grad rho_b) . grad phi
// (and a <-> b with vs_bb), E_xc = sum w e.  Here each spin's V is the FP64
// path's K + K^T with Y = 0.5 w vrho_s phi + c_s . grad phi, so the density
// and potential kernels of the restricted build run once per spin on the
// same resident AO values; only the functional stage is new (k_func_pol,
// FP64 here; with FP32 derivatives in the tensor-core build).  A meta-GGA adds
// per spin the tau densities (k_rho_f64's tau mode), the polarised TPSS
// (k_func_pol_mgga, eval_xc_mgga_pol) and the tau segments of k_vxc_f64.
// The tensor-core forms (Molecule::build_mixed_uks and build_mixed_uks_mgga,
// xc_mixed.cu) run the mixed density and potential kernels once per spin in
// the same way.
#include "functionals_mgga.cuh"
#include "functionals_pol.cuh"
#include "xc_device.cuh"
#include "xc_engine.hpp"
#include "xc_leaf_func.cuh"

namespace occx {

namespace {

// One CTA of 256 threads per leaf.  epart3 receives {sum w e, sum w rho_a,
// sum w rho_b} (the densities also for a skipped leaf, as OCC's totals).
// MIXED: the tensor-core build's evaluator (FP32 derivatives).
template <bool DERIV, bool MIXED>
__global__ void __launch_bounds__(256)
    k_func_pol(MolDev m, FuncSet fs, double thr, const double *__restrict__ rho_a,
               const double *__restrict__ rho_b, double *__restrict__ coef_a,
               double *__restrict__ coef_b, double *__restrict__ epart3) {
  __shared__ double sh[8];
  const DevLeaf L = m.leaves[blockIdx.x];
  const size_t N = static_cast<size_t>(m.npts);
  double mx = -1e300;
  for (int p = threadIdx.x; p < L.cnt; p += 256) {
    const size_t idx = static_cast<size_t>(L.off) + p;
    mx = fmax(mx, fmax(rho_a[idx], rho_b[idx]));
  }
  mx = leaf_max256(mx, sh);
  const bool skip = mx < thr;
  double na = 0.0, nb = 0.0, ew = 0.0;
  for (int p = threadIdx.x; p < L.cnt; p += 256) {
    const size_t idx = static_cast<size_t>(L.off) + p;
    const double ra = rho_a[idx], rb = rho_b[idx];
    const double w = m.pts[idx].w;
    na += w * ra;
    nb += w * rb;
    double ga[3] = {0, 0, 0}, gb[3] = {0, 0, 0};
    double saa = 0.0, sab = 0.0, sbb = 0.0;
    if (DERIV) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        ga[c] = rho_a[(c + 1) * N + idx];
        gb[c] = rho_b[(c + 1) * N + idx];
      }
      saa = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
      sab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
      sbb = gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2];
    }
    double e = 0.0, vr[2] = {0.0, 0.0}, vs[3] = {0.0, 0.0, 0.0};
    if (!skip) {
      if (MIXED)
        eval_xc_pol_mixed(fs, ra, rb, saa, sab, sbb, e, vr, vs);
      else
        eval_xc_pol(fs, ra, rb, saa, sab, sbb, e, vr, vs);
    }
    coef_a[idx] = 0.5 * w * vr[0];
    coef_b[idx] = 0.5 * w * vr[1];
    if (DERIV) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        coef_a[(c + 1) * N + idx] = w * (2.0 * vs[0] * ga[c] + vs[1] * gb[c]);
        coef_b[(c + 1) * N + idx] = w * (2.0 * vs[2] * gb[c] + vs[1] * ga[c]);
      }
    }
    ew += w * e;
  }
  ew = leaf_sum256(ew, sh);
  na = leaf_sum256(na, sh);
  nb = leaf_sum256(nb, sh);
  if (threadIdx.x == 0) {
    epart3[3 * blockIdx.x] = ew;
    epart3[3 * blockIdx.x + 1] = na;
    epart3[3 * blockIdx.x + 2] = nb;
  }
}

// The meta-GGA form (compute_K_dft<2, Unrestricted>): rho components 4-6 of
// each spin hold its (d_k phi) D2_s (d_k phi) sums, tau_s = half their sum
// (src/gto/density.cpp:104-166); coef4 of each spin = 0.25 w vtau_s, so that
// the V kernel's K + K^T carries xc_potential_matrix.cpp:110-136's 0.5 w vtau_s.
template <bool MIXED>
__global__ void __launch_bounds__(256)
    k_func_pol_mgga(MolDev m, FuncSet fs, double thr, const double *__restrict__ rho_a,
                    const double *__restrict__ rho_b, double *__restrict__ coef_a,
                    double *__restrict__ coef_b, double *__restrict__ epart3) {
  __shared__ double sh[8];
  const DevLeaf L = m.leaves[blockIdx.x];
  const size_t N = static_cast<size_t>(m.npts);
  double mx = -1e300;
  for (int p = threadIdx.x; p < L.cnt; p += 256) {
    const size_t idx = static_cast<size_t>(L.off) + p;
    mx = fmax(mx, fmax(rho_a[idx], rho_b[idx]));
  }
  mx = leaf_max256(mx, sh);
  const bool skip = mx < thr;
  double na = 0.0, nb = 0.0, ew = 0.0;
  for (int p = threadIdx.x; p < L.cnt; p += 256) {
    const size_t idx = static_cast<size_t>(L.off) + p;
    const double ra = rho_a[idx], rb = rho_b[idx];
    const double w = m.pts[idx].w;
    na += w * ra;
    nb += w * rb;
    double ga[3], gb[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      ga[c] = rho_a[(c + 1) * N + idx];
      gb[c] = rho_b[(c + 1) * N + idx];
    }
    const double saa = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
    const double sab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
    const double sbb = gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2];
    const double ta = 0.5 * (rho_a[4 * N + idx] + rho_a[5 * N + idx] + rho_a[6 * N + idx]);
    const double tb = 0.5 * (rho_b[4 * N + idx] + rho_b[5 * N + idx] + rho_b[6 * N + idx]);
    double e = 0.0, vr[2] = {0.0, 0.0}, vs[3] = {0.0, 0.0, 0.0}, vt[2] = {0.0, 0.0};
    if (!skip) {
      if (MIXED)
        eval_xc_mgga_pol_mixed(fs, ra, rb, saa, sab, sbb, ta, tb, e, vr, vs, vt);
      else
        eval_xc_mgga_pol(fs, ra, rb, saa, sab, sbb, ta, tb, e, vr, vs, vt);
    }
    coef_a[idx] = 0.5 * w * vr[0];
    coef_b[idx] = 0.5 * w * vr[1];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      coef_a[(c + 1) * N + idx] = w * (2.0 * vs[0] * ga[c] + vs[1] * gb[c]);
      coef_b[(c + 1) * N + idx] = w * (2.0 * vs[2] * gb[c] + vs[1] * ga[c]);
    }
    coef_a[4 * N + idx] = 0.25 * w * vt[0];
    coef_b[4 * N + idx] = 0.25 * w * vt[1];
    ew += w * e;
  }
  ew = leaf_sum256(ew, sh);
  na = leaf_sum256(na, sh);
  nb = leaf_sum256(nb, sh);
  if (threadIdx.x == 0) {
    epart3[3 * blockIdx.x] = ew;
    epart3[3 * blockIdx.x + 1] = na;
    epart3[3 * blockIdx.x + 2] = nb;
  }
}

// out3 = column sums of epart3 (fixed order per thread, then the block)
__global__ void __launch_bounds__(256) k_reduce3(const double *__restrict__ epart3, int n,
                                                 double *__restrict__ out3) {
  __shared__ double sh[8];
  double s[3] = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += 256)
#pragma unroll
    for (int k = 0; k < 3; k++)
      s[k] += epart3[3 * i + k];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double t = leaf_sum256(s[k], sh);
    if (threadIdx.x == 0)
      out3[k] = t;
  }
}

} // namespace

void launch_func_pol(const MolDev &m, int deriv, const FuncSet &fs, double thr,
                     const double *rho_a, const double *rho_b, double *coef_a, double *coef_b,
                     double *epart3, cudaStream_t st, bool mixed) {
  if (m.nleaves == 0)
    return;
  const dim3 g(m.nleaves);
  if (deriv == 2 && mixed)
    k_func_pol_mgga<true><<<g, 256, 0, st>>>(m, fs, thr, rho_a, rho_b, coef_a, coef_b, epart3);
  else if (deriv == 2)
    k_func_pol_mgga<false><<<g, 256, 0, st>>>(m, fs, thr, rho_a, rho_b, coef_a, coef_b, epart3);
  else if (deriv && mixed)
    k_func_pol<true, true><<<g, 256, 0, st>>>(m, fs, thr, rho_a, rho_b, coef_a, coef_b, epart3);
  else if (deriv)
    k_func_pol<true, false><<<g, 256, 0, st>>>(m, fs, thr, rho_a, rho_b, coef_a, coef_b, epart3);
  else if (mixed)
    k_func_pol<false, true><<<g, 256, 0, st>>>(m, fs, thr, rho_a, rho_b, coef_a, coef_b, epart3);
  else
    k_func_pol<false, false><<<g, 256, 0, st>>>(m, fs, thr, rho_a, rho_b, coef_a, coef_b,
                                                epart3);
}

void launch_reduce3(const double *epart3, int n, double *out3, cudaStream_t st) {
  k_reduce3<<<1, 256, 0, st>>>(epart3, n, out3);
}

void Molecule::prepare_uks() {
  if (d_rho_b)
    return;
  if (!d_pts)
    throw ArgError("the molecule has no device state");
  const size_t N = static_cast<size_t>(std::max<long>(plan.npts, 1));
  const size_t nl = std::max<size_t>(leaves.size(), 1);
  const size_t nbf2 = std::max<size_t>(static_cast<size_t>(basis.nbf) * basis.nbf, 1);
  d_rho_b = static_cast<double *>(alloc(rho_components(deriv) * N * sizeof(double)));
  d_coef_b = static_cast<double *>(alloc(coef_components(deriv) * N * sizeof(double)));
  d_epart_u = static_cast<double *>(alloc(3 * nl * sizeof(double)));
  d_Dab = static_cast<double *>(alloc(2 * nbf2 * sizeof(double)));
  d_Vab = static_cast<double *>(alloc(2 * nbf2 * sizeof(double)));
  d_Duks = static_cast<double *>(alloc(2 * nbf2 * sizeof(double)));
  d_Vuks = static_cast<double *>(alloc(2 * nbf2 * sizeof(double)));
  d_out3 = static_cast<double *>(alloc(4 * sizeof(double)));
  cuda_check(cudaMemset(d_rho_b, 0, rho_components(deriv) * N * sizeof(double)), "cudaMemset");
}

void Molecule::build_fp64_uks(const double *dD, double *dV, double *dout3, cudaStream_t st) {
  prepare_uks();
  ensure_fp64_ws();
  const MolDev m = dev();
  const size_t nbf = static_cast<size_t>(basis.nbf), nbf2 = nbf * nbf;
  Context &c = *ctx;
  // OCC's 2 nbf x nbf (column-major) -> two contiguous nbf x nbf blocks
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(d_Dab + s * nbf2, nbf * sizeof(double), dD + s * nbf,
                                 2 * nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaMemsetAsync(d_Vab, 0, 2 * nbf2 * sizeof(double), st), "cudaMemsetAsync");
  if (!fp64_ao_valid)
    c.launch("colloc_f64", st, [&] { launch_colloc_f64(m, deriv, d_ws, st); });
  double *rho[2] = {d_rho, d_rho_b}, *coef[2] = {d_coef, d_coef_b};
  for (int s = 0; s < 2; s++) {
    c.launch("rho_f64", st, [&] {
      launch_rho_f64(m, deriv, d_Dab + s * nbf2, d_ws, d_slabs, static_cast<int>(slabs.size()),
                     rho[s], st);
    });
    if (deriv == 2)
      c.launch("tau_f64", st, [&] {
        launch_tau_f64(m, d_Dab + s * nbf2, d_ws, d_slabs, static_cast<int>(slabs.size()),
                       rho[s], st);
      });
  }
  c.launch("func_pol", st, [&] {
    launch_func_pol(m, deriv, fs, bs.density_threshold, d_rho, d_rho_b, d_coef, d_coef_b,
                    d_epart_u, st);
  });
  for (int s = 0; s < 2; s++)
    c.launch("vxc_f64", st, [&] {
      launch_vxc_f64(m, deriv, d_ws, coef[s], d_tiles, static_cast<int>(tiles.size()),
                     d_Vab + s * nbf2, st);
    });
  c.launch("reduce", st, [&] { launch_reduce3(d_epart_u, m.nleaves, dout3, st); });
  for (int s = 0; s < 2; s++)
    cuda_check(cudaMemcpy2DAsync(dV + s * nbf, 2 * nbf * sizeof(double), d_Vab + s * nbf2,
                                 nbf * sizeof(double), nbf * sizeof(double), nbf,
                                 cudaMemcpyDeviceToDevice, st),
               "cudaMemcpy2DAsync");
  cuda_check(cudaGetLastError(), "kernel launch");
  fp64_ao_valid = true;
}

} // namespace occx

using namespace occx;

extern "C" {

int occ_xc_compute_vxc_unrestricted(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D,
                                    int precision, double *V, double *exc, double *nelec2) {
  if (!ctx || !mol || !D || !V || !exc)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
      throw ArgError("precision must be OCC_XC_FP64 or OCC_XC_MIXED");
    Molecule &M = *mol->impl;
    cudaStream_t st = ctx->impl->stream;
    M.prepare_uks();
    const size_t n2 = 2 * static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
    cuda_check(cudaMemcpyAsync(M.d_Duks, D, n2 * sizeof(double), cudaMemcpyHostToDevice, st),
               "cudaMemcpyAsync H2D");
    if (precision == OCC_XC_MIXED)
      M.build_mixed_uks(M.d_Duks, M.d_Vuks, M.d_out3, st);
    else
      M.build_fp64_uks(M.d_Duks, M.d_Vuks, M.d_out3, st);
    double out3[3];
    cuda_check(cudaMemcpyAsync(V, M.d_Vuks, n2 * sizeof(double), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaMemcpyAsync(out3, M.d_out3, sizeof(out3), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (precision == OCC_XC_MIXED && mixed_error_flag(M, st))
      throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
    *exc = out3[0];
    if (nelec2) {
      nelec2[0] = out3[1];
      nelec2[1] = out3[2];
    }
  });
}

int occ_xc_compute_vxc_unrestricted_device(occ_xc_context *ctx, occ_xc_molecule *mol,
                                           const double *d_D, int precision, double *d_V,
                                           double *d_out3, void *stream) {
  if (!ctx || !mol || !d_D || !d_V)
    return OCC_XC_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  return guarded(ctx, [&] {
    if (precision != OCC_XC_FP64 && precision != OCC_XC_MIXED)
      throw ArgError("precision must be OCC_XC_FP64 or OCC_XC_MIXED");
    Molecule &M = *mol->impl;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->impl->stream;
    M.prepare_uks();
    if (precision == OCC_XC_MIXED)
      M.build_mixed_uks(d_D, d_V, d_out3 ? d_out3 : M.d_out3, st);
    else
      M.build_fp64_uks(d_D, d_V, d_out3 ? d_out3 : M.d_out3, st);
  });
}

} // extern "C"
