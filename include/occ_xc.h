/*
 * occ_xc.h -- C ABI of the GB300 exchange-correlation (XC) build.
 *
 * A drop-in for the XC part of OCC's Kohn-Sham method: the molecule, its
 * AOBasis and a density matrix go in; E_xc and the V_xc matrix come out.
 * Plain C types only (no C++ or CUDA types), so any host language can bind
 * it; include/occ_xc.hpp is a C++ interface shaped like occ::dft::DFT over it.
 *
 * Conventions (those of OCC):
 *   - coordinates in Bohr;
 *   - shell coefficients as OCC's gto::Shell holds them after
 *     Shell::incorporate_shell_norm (occ_xc_normalize_shell does that step);
 *   - AO order: shells in the given order, Cartesian CCA order within a
 *     Cartesian shell, m = -l..l within a pure shell;
 *   - matrices nbf x nbf, column-major (Eigen's default), D = OCC's mo.D
 *     (C_occ C_occ^T for a restricted wavefunction; the build uses 2 D);
 *   - V receives V_xc = -K of DFT::compute_JK, and *exc E_xc.
 * Every entry point returns OCC_XC_OK (0) or a negative status; the message
 * is available from occ_xc_last_error().  No C++ exception crosses the ABI.
 * Calls on one context are serialised internally; different contexts may be
 * used from different threads.
 */
#ifndef OCC_XC_H
#define OCC_XC_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  OCC_XC_OK = 0,
  OCC_XC_ERR_ARG = -1,      /* invalid argument */
  OCC_XC_ERR_CUDA = -2,     /* CUDA runtime error */
  OCC_XC_ERR_METHOD = -3,   /* unknown or unsupported functional */
  OCC_XC_ERR_NOMEM = -4,    /* device memory / admission budget exhausted */
  OCC_XC_ERR_TIMEOUT = -5,  /* a bounded device wait gave up */
  OCC_XC_ERR_BUSY = -6,     /* request queue full */
  OCC_XC_ERR_INTERNAL = -7,
};

enum {
  OCC_XC_FP64 = 0,  /* plain path: every operation in FP64 */
  OCC_XC_MIXED = 1, /* contractions in 3xTF32 on tcgen05 tensor cores with FP32
                       accumulation; functionals, cross-block sums and the final
                       symmetrisation in FP64 */
};

typedef struct occ_xc_context occ_xc_context;
typedef struct occ_xc_molecule occ_xc_molecule;

/* Mirrors occ::numint::GridSettings (include/occ/numint/grid_settings.h:81-95). */
typedef struct {
  int max_angular_points;             /* 302 */
  int min_angular_points;             /* 110 */
  int radial_points;                  /* 50 (not used by the LMG radial grid) */
  double radial_precision;            /* 1e-12 */
  int reduced_first_row_element_grid; /* 1 */
  int treutler_alrichs_adjustment;    /* 1 */
  int pruning_scheme;                 /* 1 = NWChem, 0 = none */
} occ_xc_grid_settings;

/* Build knobs: DFT::set_xc_screening_threshold (include/occ/dft/dft.h:590),
 * the density threshold (dft.h:760) and the Morton leaf sizes
 * (include/occ/numint/spatial_grid_hierarchy.h:26-30). */
typedef struct {
  double xc_screening_threshold; /* 1e-10 */
  double density_threshold;      /* 1e-10 */
  int leaf_target;               /* 128 */
  int leaf_min;                  /* 32 */
  int leaf_max;                  /* 256 */
} occ_xc_build_settings;

typedef struct {
  int nbf, natoms, nshells, deriv;
  long npoints, nleaves;
  double flops_per_build;    /* 4 * sum_b n_b * m_b^2 (useful contraction FLOPs) */
  double device_bytes;          /* device memory held now (resident state and the
                                   private workspaces allocated so far) */
  double workspace_bytes;       /* per-build workspace of the FP64 path */
  double mixed_workspace_bytes; /* per-build workspace of the mixed path */
  double resident_bytes;        /* resident state alone (upper bound, no workspace) */
} occ_xc_molecule_info;

void occ_xc_default_grid_settings(occ_xc_grid_settings *out);
void occ_xc_default_build_settings(occ_xc_build_settings *out);

/* Replaces Shell::incorporate_shell_norm (src/gto/shell.cpp:180-186):
 * scales coefs[nprim] in place. */
int occ_xc_normalize_shell(int l, int nprim, const double *exps, double *coefs);

/* Replaces MolecularGrid(basis, settings).get_molecular_grid_points()
 * (src/numint/molecular_grid.cpp:11-140): host-only, needs no device.
 * Call with points == NULL to get *npoints; then with buffers of that size:
 * points[3*npoints] (x,y,z per point, Bohr), weights[npoints]. */
int occ_xc_molecular_grid(int natoms, const int *atomic_numbers, const double *xyz_bohr,
                          int nshells, const int *shell_l, const int *shell_atom,
                          const int *shell_nprim, const double *exponents,
                          const double *coefficients, int pure, const occ_xc_grid_settings *grid,
                          long *npoints, double *points, double *weights);

/* The same grid with the Becke partition weights computed on the context's
 * device (an FP32 pass finds the atoms whose cell functions matter at each
 * point, an FP64 pass evaluates those with OCC's formula); equal to the
 * host's to rounding.  Molecules created on a context build their grid this
 * way.  OCC_XC_ERR_ARG for more atoms than the kernel's shared memory holds
 * (about 2,500 on GB300). */
int occ_xc_molecular_grid_device(occ_xc_context *ctx, int natoms, const int *atomic_numbers,
                                 const double *xyz_bohr, int nshells, const int *shell_l,
                                 const int *shell_atom, const int *shell_nprim,
                                 const double *exponents, const double *coefficients, int pure,
                                 const occ_xc_grid_settings *grid, long *npoints, double *points,
                                 double *weights);

/* Replaces occ::numint::grid::lebedev(n) (include/occ/numint/lebedev.h,
 * src/numint/lebedev.cpp:5388-5503) for n in {6, 14, 26, 38, 50, 74, 86, 110,
 * 146, 170, 194, 230, 266, 302}: xyzw[4*n] receives x, y, z, weight per point
 * (weights sum to one).  Host-only.  Returns n, or 0 for an unsupported n. */
int occ_xc_lebedev(int n, double *xyzw);

/* Context: one CUDA device, one stream.  Replaces nothing in OCC (OCC has
 * no device state). */
int occ_xc_context_create(int device, occ_xc_context **out);
void occ_xc_context_destroy(occ_xc_context *ctx);
const char *occ_xc_last_error(const occ_xc_context *ctx);

/* Replaces DFT::DFT(method, basis, grid_settings) (include/occ/dft/dft.h:39,
 * src/dft/dft.cpp:19-35) for the XC part: builds the molecular grid
 * (MolecularGrid, src/numint/molecular_grid.cpp:11-256), the Morton leaves
 * and screening lists, and keeps them resident on the device.
 * method: OCC method name ("lda", "svwn5", "pbe", "blyp", "b3lyp", ...).
 * grid/build settings may be NULL for OCC's defaults. */
int occ_xc_molecule_create(occ_xc_context *ctx, int natoms, const int *atomic_numbers,
                           const double *xyz_bohr, int nshells, const int *shell_l,
                           const int *shell_atom, const int *shell_nprim,
                           const double *exponents, const double *coefficients, int pure,
                           const char *method, const occ_xc_grid_settings *grid,
                           const occ_xc_build_settings *build, occ_xc_molecule **out);
void occ_xc_molecule_destroy(occ_xc_molecule *mol);
int occ_xc_molecule_info_get(const occ_xc_molecule *mol, occ_xc_molecule_info *out);

/* Copies the molecular grid out in OCC's layout (atom blocks in atom order,
 * MolecularGridPoints, src/numint/molecular_grid_points.cpp:15-50):
 * points[3*npoints] (x,y,z per point), weights[npoints]. */
int occ_xc_molecule_grid(const occ_xc_molecule *mol, double *points, double *weights);

/* Replaces DFT::compute_vxc(mo) for a restricted wavefunction
 * (include/occ/dft/dft.h:395-429) together with
 * DFT::exchange_correlation_energy() (dft.h:83).  Host buffers; blocking.
 * nelec_out (may be NULL) receives the integrated density. */
int occ_xc_compute_vxc(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D,
                       int precision, double *V, double *exc, double *nelec_out);

/* Same build on device buffers, asynchronous on `stream` (a cudaStream_t, or
 * NULL for the context's stream).  d_exc2 receives {E_xc, integrated density}. */
int occ_xc_compute_vxc_device(occ_xc_context *ctx, occ_xc_molecule *mol, const double *d_D,
                              int precision, double *d_V, double *d_exc2, void *stream);

/* Replaces DFT::compute_vxc(mo) for an unrestricted wavefunction
 * (dft.h:395-429 -> compute_K_dft<deriv, Unrestricted>): D and V are
 * 2 nbf x nbf column-major, the alpha block above the beta block, D = OCC's
 * mo.D (each block 0.5 C_s C_s^T, src/qm/orb.h:68-83); the polarised forms of
 * the method's functionals.  precision: OCC_XC_FP64, or OCC_XC_MIXED (the
 * density and potential contractions on the tensor cores, once per spin).
 * nelec2 (may be NULL) receives the integrated alpha and beta densities. */
int occ_xc_compute_vxc_unrestricted(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D,
                                    int precision, double *V, double *exc, double *nelec2);
/* Same on device buffers, asynchronous on `stream` (NULL: the context's);
 * d_out3 (may be NULL) receives {E_xc, integrated rho_a, integrated rho_b}. */
int occ_xc_compute_vxc_unrestricted_device(occ_xc_context *ctx, occ_xc_molecule *mol,
                                           const double *d_D, int precision, double *d_V,
                                           double *d_out3, void *stream);

/* VV10 non-local correlation: replaces NonLocalCorrelationFunctional's
 * operator()(basis, mo) (src/dft/nonlocal_correlation.cpp:331-388), the
 * energy DFT::post_scf_nlc_correction (include/occ/dft/dft.h:476-483) adds
 * for the "-V" methods, restricted.  Parameters b and C (OCC's defaults 6.0
 * and 0.01); energy receives E_nlc, V (may be NULL) its nbf x nbf potential.
 * precision: OCC_XC_FP64, or OCC_XC_MIXED for the O(N^2) pair sums in FP32
 * (compensated; everything else FP64).  The first call builds the NLC grid
 * (OCC's GridSettings{110, 50, 50, 1e-7}) as a second resident grid. */
int occ_xc_nlc_vv10(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D, double b,
                    double C, int precision, double *energy, double *V);
/* The NLC grid in OCC's layout once built: its point count (-1 before the
 * first VV10 call), then points[3 * n] and weights[n]. */
int occ_xc_nlc_grid_points(const occ_xc_molecule *mol, long *npoints);
int occ_xc_nlc_grid(const occ_xc_molecule *mol, double *points, double *weights);

/* Seminumerical (COSX) exchange, the ESP form of OCC's
 * SemiNumericalExchange (include/occ/qm/seminumerical_exchange.h:104-118,
 * src/qm/seminumerical_exchange.cpp:233-250 set-up, :516-529 restricted K,
 * :714-855 the grid sweep), replacing its constructor and compute_K(mo) for
 * restricted and unrestricted wavefunctions (:616-648).  occ_xc_cosx_create
 * builds, on `mol`'s device
 * and over its basis, the grid of `grid` (NULL: GridSettings::for_sgx(50),
 * src/numint/grid_settings.cpp:59-68), its AO values, the numerical overlap
 * S_num and the overlap projector Q = S_num^-1 S; shells up to d
 * (OCC_XC_ERR_ARG above).  Every operation is FP64 unless
 * occ_xc_cosx_set_precision selects OCC_XC_MIXED. */
typedef struct occ_xc_cosx occ_xc_cosx;
int occ_xc_cosx_create(occ_xc_context *ctx, occ_xc_molecule *mol,
                       const occ_xc_grid_settings *grid, occ_xc_cosx **out);
void occ_xc_cosx_destroy(occ_xc_cosx *cx);
/* OCC_XC_FP64 (the default) or OCC_XC_MIXED: the ESP integrals of every
 * shell pair at every grid point (Boys function, Hermite integrals and their
 * contraction) in FP32, the rest (F, G, K', the projector) in FP64.  No
 * counterpart in OCC, whose ESP integrals are FP64. */
int occ_xc_cosx_set_precision(occ_xc_cosx *cx, int precision);
/* Points of the exchange grid. */
int occ_xc_cosx_grid_points(const occ_xc_cosx *cx, long *npoints);
/* K (nbf x nbf, symmetric) of mo.D = D (nbf x nbf); host buffers, blocking. */
int occ_xc_cosx_exchange(occ_xc_context *ctx, occ_xc_cosx *cx, const double *D, double *K);
/* The same on device buffers, asynchronous on `stream` (NULL: the context's). */
int occ_xc_cosx_exchange_device(occ_xc_context *ctx, occ_xc_cosx *cx, const double *d_D,
                                double *d_K, void *stream);
/* Unrestricted: D and K are 2 nbf x nbf, column-major, the alpha block above
 * the beta one (OCC's unrestricted mo.D, each block 0.5 C_s C_s^T); per spin
 * K_s = 1/2 (K'_s + K'_s^T) of Q (2 D_s), as compute_K_unrestricted
 * (src/qm/seminumerical_exchange.cpp:616-648).  Host buffers, blocking. */
int occ_xc_cosx_exchange_unrestricted(occ_xc_context *ctx, occ_xc_cosx *cx, const double *D,
                                      double *K);
/* The same on device buffers, asynchronous on `stream` (NULL: the context's). */
int occ_xc_cosx_exchange_unrestricted_device(occ_xc_context *ctx, occ_xc_cosx *cx,
                                             const double *d_D, double *d_K, void *stream);

/* Replaces DFT::compute_xc_gradient(mo) for a restricted wavefunction
 * (include/occ/dft/dft.h:599-749, src/dft/dft_gradient_kernels.cpp:472-595):
 * dE_xc/dR with the grid held fixed.  grad[3*natoms] receives x, y, z per
 * atom in Hartree/Bohr (the memory of OCC's 3 x natoms Mat3N); exc (may be
 * NULL) the E_xc of the same density.  precision: OCC_XC_FP64 (every
 * operation FP64; the first call allocates a workspace of AO values with
 * second derivatives, capped at 8 GiB per leaf group), or OCC_XC_MIXED (the
 * contractions on the tensor cores in 3xTF32, in a workspace beside the
 * build's).  Host buffers; blocking. */
int occ_xc_compute_xc_gradient(occ_xc_context *ctx, occ_xc_molecule *mol, const double *D,
                               int precision, double *grad, double *exc);

/* Same on device buffers, asynchronous on `stream` (NULL: the context's).
 * d_exc2 (may be NULL) receives {E_xc, integrated density}.  Allocates on a
 * molecule's first gradient of each precision only. */
int occ_xc_compute_xc_gradient_device(occ_xc_context *ctx, occ_xc_molecule *mol,
                                      const double *d_D, int precision, double *d_grad,
                                      double *d_exc2, void *stream);

/* Replaces DFT::compute_xc_gradient(mo) for an unrestricted wavefunction
 * (include/occ/dft/dft.h:599-749 with accumulate_gradient_contribution_U,
 * src/dft/dft_gradient_kernels.cpp:175-470, 549-575): D is OCC's unrestricted
 * mo.D (2 nbf x nbf, alpha block above beta, column-major); grad[3*natoms]
 * and exc as occ_xc_compute_xc_gradient.  precision OCC_XC_FP64 or
 * OCC_XC_MIXED (the contractions on the tensor cores in 3xTF32), for LDA, GGA
 * and meta-GGA methods.  Host buffers; blocking. */
int occ_xc_compute_xc_gradient_unrestricted(occ_xc_context *ctx, occ_xc_molecule *mol,
                                            const double *D, int precision, double *grad,
                                            double *exc);

/* Same on device buffers, asynchronous on `stream` (NULL: the context's).
 * d_exc3 (may be NULL) receives {E_xc, integrated rho_a, integrated rho_b}. */
int occ_xc_compute_xc_gradient_unrestricted_device(occ_xc_context *ctx, occ_xc_molecule *mol,
                                                   const double *d_D, int precision,
                                                   double *d_grad, double *d_exc3,
                                                   void *stream);

/* Cap (bytes) of the gradient workspace of one leaf group; leaves are
 * processed in groups under it (0: the default, 8 GiB).  Frees the
 * molecule's gradient state, which the next gradient rebuilds. */
int occ_xc_molecule_set_gradient_workspace_cap(occ_xc_context *ctx, occ_xc_molecule *mol,
                                              double bytes);

/* ---- batches: many molecules' XC builds in one launch sequence -------------
 * OCC builds one molecule at a time (a TBB loop over one grid); a batch runs
 * the blocks of all its molecules through the same kernel launches (the
 * tensor-core kernels persistent over one queue of blocks from every
 * molecule; LDA and GGA molecules go in one sequence each).  A molecule
 * appears at most once in a batch.  The batch owns one D, V and
 * {E_xc, integrated density} device buffer per molecule (same conventions as
 * occ_xc_compute_vxc_device); write D into them and read V / E_xc back. */
typedef struct occ_xc_batch occ_xc_batch;
int occ_xc_batch_create(occ_xc_context *ctx, int nmol, occ_xc_molecule *const *mols,
                        occ_xc_batch **out);
/* The batch keeps one shared per-build workspace.  Its molecules are split, in
 * order, into sub-batches whose mixed-path workspaces sum to at most
 * workspace_cap_bytes (a molecule above the cap forms its own); sub-batches
 * run one after the other through the same workspace, so a batch of any size
 * fits the device.  occ_xc_batch_create uses half of the free device memory
 * as the cap (workspace_cap_bytes <= 0 does the same). */
int occ_xc_batch_create_capped(occ_xc_context *ctx, int nmol, occ_xc_molecule *const *mols,
                               double workspace_cap_bytes, occ_xc_batch **out);
void occ_xc_batch_destroy(occ_xc_batch *batch);
int occ_xc_batch_buffers(occ_xc_batch *batch, int i, double **d_D, double **d_V,
                         double **d_exc2);
/* Asynchronous on stream (NULL: the context's stream).  OCC_XC_MIXED: one
 * launch sequence for the whole batch; OCC_XC_FP64: the molecules' FP64 builds
 * one after the other. */
int occ_xc_batch_compute(occ_xc_context *ctx, occ_xc_batch *batch, int precision, void *stream);
/* Synchronises stream; OCC_XC_ERR_TIMEOUT if a bounded device wait gave up. */
int occ_xc_batch_check(occ_xc_context *ctx, occ_xc_batch *batch, void *stream);
/* Host-buffer form: D[i], V[i] are nbf_i x nbf_i host matrices, exc[i] (and
 * nelec[i] if not NULL) receive E_xc and the integrated density; blocking. */
int occ_xc_batch_compute_host(occ_xc_context *ctx, occ_xc_batch *batch, int precision,
                              const double *const *D, double *const *V, double *exc,
                              double *nelec);
/* Blocking copies between host memory and molecule i's batch-owned buffers
 * (D: nbf_i x nbf_i in; V: nbf_i x nbf_i and exc2 = {E_xc, density} out). */
int occ_xc_batch_set_density(occ_xc_context *ctx, occ_xc_batch *batch, int i, const double *D);
int occ_xc_batch_get_result(occ_xc_context *ctx, occ_xc_batch *batch, int i, double *V,
                            double *exc2);

/* ---- CUDA graphs ----------------------------------------------------------
 * Capture niter consecutive builds of one molecule (build k reads d_D[k] and
 * writes d_V[k], d_exc2[k]; e.g. the XC builds of the iterations of an SCF
 * whose densities are known) or one build of a batch into one CUDA graph;
 * launching the graph replays them with no host work per kernel. */
typedef struct occ_xc_graph occ_xc_graph;
int occ_xc_graph_capture(occ_xc_context *ctx, occ_xc_molecule *mol, int precision, int niter,
                         const double *const *d_D, double *const *d_V, double *const *d_exc2,
                         occ_xc_graph **out);
int occ_xc_batch_graph_capture(occ_xc_context *ctx, occ_xc_batch *batch, int precision,
                               occ_xc_graph **out);
/* stream NULL: the stream of the context the graph was captured on. */
int occ_xc_graph_launch(occ_xc_graph *graph, void *stream);
void occ_xc_graph_destroy(occ_xc_graph *graph);

/* ---- serving loop ----------------------------------------------------------
 * Builds of many molecules through one GPU (OCC itself has no server; this
 * is the xc_submit / xc_poll layer in front of compute_vxc).  A client opens
 * a session per molecule -- the grid and screening are built on the calling
 * thread, no device memory yet -- then submits one density per SCF
 * iteration and collects V_xc / E_xc by ticket.  A worker thread owns the
 * GPU: each tick it takes the oldest pending build of up to max_batch
 * sessions (one per session, so a session's builds run in submission order)
 * and runs them through one launch sequence.  A session's device state --
 * grid, screening and a workspace in which its AO values stay resident
 * across iterations -- is materialised when it is admitted, which happens
 * only while the admitted sessions' device bytes (an upper bound computed at
 * open) fit the budget and its workspace fits the device pool;
 * a session that could never fit is refused at open with OCC_XC_ERR_NOMEM.
 * Closing a session frees its device state after its pending builds.  All
 * calls are thread-safe; errors are described by occ_xc_server_last_error()
 * of the calling thread. */
typedef struct occ_xc_server occ_xc_server;
typedef struct {
  double hbm_budget_bytes; /* 150e9 */
  int queue_capacity;      /* pending builds before submit returns BUSY (4096) */
  int max_batch;           /* builds per tick (64) */
  int precision;           /* OCC_XC_MIXED */
  double pool_bytes;       /* device pool of the sessions' workspaces, allocated at the
                              first admission (0: the budget, at most 40 % of the
                              memory free then) */
} occ_xc_server_settings;
typedef struct {
  long completed, failed, pending, ticks;
  long sessions_admitted, sessions_waiting;
  double mean_batch;            /* builds per tick */
  double p50_ms, p99_ms, max_ms; /* submit -> result ready, completed builds */
  double admitted_bytes, peak_admitted_bytes;
} occ_xc_server_stats;
void occ_xc_default_server_settings(occ_xc_server_settings *out);
const char *occ_xc_server_last_error(void);
int occ_xc_server_create(int device, const occ_xc_server_settings *settings,
                         occ_xc_server **out);
/* Stops the worker (a running tick finishes) and frees everything; builds
 * not yet run are dropped. */
void occ_xc_server_destroy(occ_xc_server *server);
/* Arguments as occ_xc_molecule_create. */
int occ_xc_server_open(occ_xc_server *server, int natoms, const int *atomic_numbers,
                       const double *xyz_bohr, int nshells, const int *shell_l,
                       const int *shell_atom, const int *shell_nprim, const double *exponents,
                       const double *coefficients, int pure, const char *method,
                       const occ_xc_grid_settings *grid, const occ_xc_build_settings *build,
                       uint64_t *session);
/* D: nbf x nbf host matrix (copied before the call returns).  OCC_XC_ERR_BUSY
 * when queue_capacity builds are pending. */
int occ_xc_server_submit(occ_xc_server *server, uint64_t session, const double *D,
                         uint64_t *ticket);
/* *done = 0: not finished.  *done = 1: V (nbf x nbf, may be NULL) and exc2 =
 * {E_xc, integrated density} (may be NULL) are written, the ticket is
 * released and the build's status is returned. */
int occ_xc_server_poll(occ_xc_server *server, uint64_t ticket, double *V, double *exc2,
                       int *done);
/* Blocks up to timeout_s; OCC_XC_ERR_TIMEOUT (ticket kept) if not finished. */
int occ_xc_server_wait(occ_xc_server *server, uint64_t ticket, double timeout_s, double *V,
                       double *exc2);
int occ_xc_server_close(occ_xc_server *server, uint64_t session);
/* paused != 0: no new ticks start (submissions still queue). */
int occ_xc_server_pause(occ_xc_server *server, int paused);
/* Molecule figures of the session; device_bytes = bytes held now (0 until
 * admitted), resident_bytes = its admission charge (resident state, upper
 * bound, plus its workspace in the pool, where its AO values stay resident). */
int occ_xc_server_session_info(occ_xc_server *server, uint64_t session,
                               occ_xc_molecule_info *out, int *admitted);
int occ_xc_server_stats_get(occ_xc_server *server, occ_xc_server_stats *out);

/* ---- build settings and autotuning ----------------------------------------
 * Replaces DFT::set_xc_screening_threshold (include/occ/dft/dft.h:590) and
 * the leaf sizes of SpatialGridHierarchy (spatial_grid_hierarchy.h:26-30):
 * new leaves and screening for the molecule, grid kept.  The molecule's
 * device buffers are reallocated: graphs captured on it become invalid. */
int occ_xc_molecule_set_build_settings(occ_xc_context *ctx, occ_xc_molecule *mol,
                                       const occ_xc_build_settings *build);

typedef struct {
  int leaf_target, leaf_min, leaf_max; /* chosen Morton leaf sizes */
  int vxc_tile_n;                      /* N of the mixed path's V_xc tile */
  int persistent_ctas;                 /* 0 = one per SM */
  double ms_per_build;                 /* measured at the choice */
  double default_ms_per_build;         /* measured at OCC's leaf sizes */
  double max_dexc;                     /* largest |E_xc - E_xc(default)| accepted */
  int candidates;                      /* builds configurations timed */
  int from_cache;                      /* 1: taken from OCC_XC_TUNE_CACHE, nothing timed */
} occ_xc_tune_result;
/* Times builds of the molecule with density D (host, nbf x nbf) at several
 * leaf sizes {64, 128, 256, 512}, V_xc tiles {128, 256} and CTA counts, keeps
 * candidates whose E_xc is within tol_exc of the default-settings build, and
 * (apply != 0) leaves the molecule set up with the fastest.  The choice is
 * appended to the file named by the environment variable OCC_XC_TUNE_CACHE
 * (when set) and read back from it on later calls.  Invalidates graphs
 * captured on the molecule. */
int occ_xc_molecule_autotune(occ_xc_context *ctx, occ_xc_molecule *mol, int precision,
                             const double *D, double tol_exc, int apply,
                             occ_xc_tune_result *out);
/* Sets a molecule up with a tuning result (leaf sizes, tile, CTAs) found for
 * a similar one, e.g. one molecule per size class of a batch. */
int occ_xc_molecule_apply_tuning(occ_xc_context *ctx, occ_xc_molecule *mol,
                                 const occ_xc_tune_result *tuning);

/* CTAs of the persistent tensor-core kernels (0 = one per SM, the default);
 * fewer leave SMs free for concurrent builds on other streams. */
int occ_xc_set_persistent_ctas(occ_xc_context *ctx, int ctas);

/* Bound, in polls, of every pipeline wait of the persistent tensor-core
 * kernels on this context's device (default 16777216 = 2^24).  A wait that
 * runs out sets the build's error flag; the kernel waits for its own bulk
 * copies and MMAs in flight (under the default bound), frees its tensor
 * memory and returns, and the call reports OCC_XC_ERR_TIMEOUT once; the next
 * build starts clean.  No counterpart in the reference (it has no GPU
 * pipeline); tests lower the bound, to 0 even, to make a wait run out. */
int occ_xc_set_wait_limit(occ_xc_context *ctx, unsigned int polls);

/* The FP64 build of occ_xc_compute_vxc_device for callers that cannot
 * allocate device memory -- code inside a host application that owns all of
 * the GPU's memory through its own pool, or code that must never block in the
 * allocator.  It has no counterpart in the reference (OCC allocates freely on
 * the host).  It calls no cudaMalloc, cudaFree or other allocating routine:
 * its scratch is one static device array of 64 MiB that every GPU loading
 * the library holds until the process exits.  A molecule whose scratch would
 * exceed 64 MiB (roughly a water molecule in a split-valence basis with a GGA)
 * is rejected with OCC_XC_ERR_ARG and a message, as is a molecule created on
 * another context.  The first call on a device looks up the array's device
 * address; under CUDA's lazy module loading that is also when the 64 MiB are
 * taken on that device, so make the first call at set-up, before the
 * caller's pool takes the GPU's memory and before any stream capture.  The
 * call makes the context's device current and restores the caller's current
 * device before it returns.  All calls share the array: calls that overlap
 * on the GPU race on it, so serialise them.  d_D, d_V and d_exc2 are as for
 * occ_xc_compute_vxc_device; the molecule is created beforehand with
 * occ_xc_molecule_create. */
int occ_xc_compute_vxc_noalloc(occ_xc_context *ctx, occ_xc_molecule *mol, const double *d_D,
                               double *d_V, double *d_exc2, void *stream);

/* Per-leaf view of the build plan (for tests and tooling): for each leaf
 * that has at least one significant shell, in Morton order, its point count
 * and its significant-AO count m_b.  Arrays sized nleaves (molecule info). */
int occ_xc_molecule_leaves(const occ_xc_molecule *mol, int *npoints, int *nbf_local);

/* Device-side kernel timing, the analogue of OCC's timing categories
 * (include/occ/core/timings.h:11-141, e.g. dft_xc): when enabled, every kernel
 * a build launches is bracketed by CUDA events on its stream.
 * occ_xc_profile_count synchronises and returns the number of kernel names;
 * occ_xc_profile_entry reads one (name valid until the next reset). */
int occ_xc_profile_enable(occ_xc_context *ctx, int on);
int occ_xc_profile_reset(occ_xc_context *ctx);
int occ_xc_profile_count(occ_xc_context *ctx);
int occ_xc_profile_entry(occ_xc_context *ctx, int i, const char **name, double *total_ms,
                         long *launches);
/* Number of kernels the library has launched on this context so far. */
long occ_xc_launch_count(const occ_xc_context *ctx);

#ifdef __cplusplus
}
#endif
#endif /* OCC_XC_H */
