// CPU oracle for the Kohn-Sham XC build -- TEST INFRASTRUCTURE ONLY.
//
// A plain FP64 restatement of OCC's restricted XC build
// (include/occ/dft/dft.h:192-388, compute_K_dft<deriv, Restricted>), used by
// the test suite, the smoke check and bench.py's CPU baseline as the checker.
// Nothing in the product links, loads or calls this library.
//
// Parity pins: the collocation is checked against the reference's own
// gau2grid (compiled under oracle/_ref on the development machine) and the
// PBE exchange known-answer test of tests/dft_tests.cpp:71-111.  The other
// functionals (Slater, VWN, B88, LYP, PBE correlation) are restated from the
// published papers because Libxc 6.2.2 (the reference's functional library,
// fetched at configure time) is not available; their derivatives are checked
// against finite differences of the energy density.
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

// Functional identifiers use Libxc's public numbers.
enum {
  ORC_LDA_X = 1,
  ORC_LDA_C_VWN = 7,
  ORC_LDA_C_VWN_RPA = 8,
  ORC_LDA_C_VWN_3 = 30,
  ORC_GGA_X_PBE = 101,
  ORC_GGA_X_B88 = 106,
  ORC_GGA_C_PBE = 130,
  ORC_GGA_C_LYP = 131,
  ORC_HYB_GGA_XC_B3LYP = 402,
  ORC_HYB_GGA_XC_B3LYP5 = 475,
  ORC_HYB_GGA_XC_PBEH = 406,
  ORC_HYB_GGA_XC_BHANDH = 435,
  ORC_HYB_GGA_XC_BHANDHLYP = 436,
  ORC_MGGA_X_TPSS = 202,
  ORC_MGGA_C_TPSS = 231,
};

// Evaluate one functional on n points (unpolarised).  exc is energy per
// particle, vrho = d(rho*exc)/drho, vsigma = d(rho*exc)/dsigma (GGA only;
// may be null for LDA).  Returns 0, or -1 for an unknown id.
int oracle_functional(int id, long n, const double *rho, const double *sigma,
                      double *exc, double *vrho, double *vsigma);
int oracle_functional_is_gga(int id);
// The polarised form (UKS): rho_a, rho_b, s_aa, s_ab, s_bb in; exc (per
// particle), vrho_a, vrho_b, vs_aa, vs_ab, vs_bb out (sigma arrays and
// their outputs may be null for an LDA).
int oracle_functional_polarized(int id, long n, const double *ra, const double *rb,
                                const double *saa, const double *sab, const double *sbb,
                                double *exc, double *vra, double *vrb, double *vsaa,
                                double *vsab, double *vsbb);

// Meta-GGA functionals (xc_oracle_mgga.cpp), unpolarised: rho, sigma, tau in;
// exc (per particle), vrho, vsigma, vtau out.  Returns -1 for an id that is
// not a meta-GGA.
int oracle_functional_is_mgga(int id);
int oracle_functional_mgga(int id, long n, const double *rho, const double *sigma,
                           const double *tau, double *exc, double *vrho, double *vsigma,
                           double *vtau);
// The polarised form: vr[2n] (a, b), vs[3n] (aa, ab, bb), vt[2n] (a, b).
int oracle_functional_mgga_polarized(int id, long n, const double *ra, const double *rb,
                                     const double *saa, const double *sab, const double *sbb,
                                     const double *ta, const double *tb, double *exc,
                                     double *vr, double *vs, double *vt);

// Collocation of one shell (values and, if deriv, gradients; deriv 2 adds the
// second derivatives xx, xy, xz, yy, yz, zz) at n points (xyz interleaved).
// Output layout: [ncomp][nfunc][n], ncomp = 1, 4 or 10.
int oracle_collocation(int l, int pure, int nprim, const double *exps,
                       const double *coefs, const double *origin, long n,
                       const double *xyz, int deriv, double *out);

// Shell decay radii (src/gto/gto.cpp:18-67).
void oracle_decay_cutoff(int nsh, const int *sh_l, const int *sh_nprim,
                         const int *sh_off, const double *exps,
                         const double *coefs, const double *sh_origin, int pure,
                         double threshold, double *extents);

// Morton sort + leaves (src/numint/spatial_grid_hierarchy.cpp:35-147).
// perm: sorted -> original index (n); leaves: (offset, count) pairs, returns
// the number of leaves; centres (3 per leaf) and radii may be null.
long oracle_morton_leaves(long n, const double *points, long target,
                          long min_leaf, long max_leaf, long *perm,
                          long *leaf_off, long *leaf_cnt, double *centres,
                          double *radii);

// The whole restricted XC build (LDA, GGA and meta-GGA: for a meta-GGA the
// density adds tau (src/gto/density.cpp:73-101) and V the tau term of
// src/dft/xc_potential_matrix.cpp:43-58).  D is OCC's mo.D (nbf x nbf, column-major);
// V (nbf x nbf) receives V_xc = -K of compute_JK.  func ids/coefs give the
// components summed as in src/dft/dft_kernels.cpp:55-58 (coefficients are
// Libxc-internal mixture weights, not OCC's never-applied scale factors).
// leaf_stride > 1 restricts the build to every leaf_stride-th leaf (used only
// to time a bounded CPU sample).  Returns 0 on success.
int oracle_xc_build(int nsh, const int *sh_l, const int *sh_nprim,
                    const int *sh_off, const double *exps, const double *coefs,
                    const double *sh_origin, int pure, long npts,
                    const double *points, const double *weights,
                    const double *D, int nfunc, const int *func_ids,
                    const double *func_coefs, double screen_threshold,
                    double density_threshold, long leaf_target, long leaf_min,
                    long leaf_max, int nthreads, long leaf_stride, double *V,
                    double *exc_out, double *nelec_out);

// The unrestricted (UKS) build: compute_K_dft<deriv, Unrestricted>
// (include/occ/dft/dft.h:192-388) with the polarised functionals.  D and V
// are 2 nbf x nbf column-major (alpha block above beta, OCC's mo.D);
// nelec2 (may be null) receives the integrated alpha and beta densities.
int oracle_xc_build_unrestricted(int nsh, const int *sh_l, const int *sh_nprim,
                                 const int *sh_off, const double *exps, const double *coefs,
                                 const double *sh_origin, int pure, long npts,
                                 const double *points, const double *weights, const double *D,
                                 int nfunc, const int *func_ids, const double *func_coefs,
                                 double screen_threshold, double density_threshold,
                                 long leaf_target, long leaf_min, long leaf_max, int nthreads,
                                 double *V, double *exc_out, double *nelec2);

// VV10 non-local correlation (src/dft/nonlocal_correlation.cpp:37-110):
// per point exc, vrho, vsigma (weighted) from rho, sigma in the given order.
void oracle_vv10_kernel(long n, const double *points, const double *weights, const double *rho,
                        const double *sigma, double b, double C, int nthreads, double *exc,
                        double *vrho, double *vsigma);
// NonLocalCorrelationFunctional::vv10 (nonlocal_correlation.cpp:331-388) on
// the given NLC grid: energy and (if V) V (nbf x nbf) for mo.D = D.
int oracle_nlc_vv10(int nsh, const int *sh_l, const int *sh_nprim, const int *sh_off,
                    const double *exps, const double *coefs, const double *sh_origin, int pure,
                    long npts, const double *points, const double *weights, const double *D,
                    double b, double C, int nthreads, double *V, double *energy);

// The restricted XC nuclear gradient (include/occ/dft/dft.h:599-749,
// src/dft/dft_gradient_kernels.cpp:472-595), screened path, grid weights held
// fixed.  sh_atom: atom of each shell; grad[3 * natoms] (x, y, z per atom)
// receives dE_xc/dR.  Collocation deriv 2 (out[10][nfunc][n]) serves it.
int oracle_xc_gradient(int nsh, const int *sh_l, const int *sh_nprim, const int *sh_off,
                       const double *exps, const double *coefs, const double *sh_origin,
                       const int *sh_atom, int natoms, int pure, long npts,
                       const double *points, const double *weights, const double *D,
                       int nfunc, const int *func_ids, const double *func_coefs,
                       double screen_threshold, double density_threshold, long leaf_target,
                       long leaf_min, long leaf_max, int nthreads, double *grad);

// The unrestricted XC nuclear gradient (dft.h:599-749, accumulate_gradient_
// contribution_U, src/dft/dft_gradient_kernels.cpp:175-470, 549-575): D is
// OCC's unrestricted mo.D (2 nbf x nbf); LDA, GGA and meta-GGA.
int oracle_xc_gradient_unrestricted(int nsh, const int *sh_l, const int *sh_nprim,
                                    const int *sh_off, const double *exps, const double *coefs,
                                    const double *sh_origin, const int *sh_atom, int natoms,
                                    int pure, long npts, const double *points,
                                    const double *weights, const double *D, int nfunc,
                                    const int *func_ids, const double *func_coefs,
                                    double screen_threshold, double density_threshold,
                                    long leaf_target, long leaf_min, long leaf_max, int nthreads,
                                    double *grad);

#ifdef __cplusplus
}
#endif
