/*
 * fosgpu.h -- C ABI of libfosgpu.so, the GB300 implementation of foeuler's
 * implicit inner loop (mianzhi/fosolvers).
 *
 * All entry points are extern "C" with plain pointers and sizes.  Host-pointer
 * entry points (fos_euler_rhs/pset/psol) are the drop-in replacements for the
 * three CVODE user callbacks of src/foeuler/foeuler.f90; *_dev entry points
 * take device pointers and run on the context's CUDA stream; fos_bdf_run is the
 * device-resident fixed-step BDF Newton--Krylov driver.
 *
 * Vector layout (every y / ydot / r / z argument): SoA by conserved variable,
 * [rho(1:nC), rhou(1:nC), rhov(1:nC), rhow(1:nC), rhoE(1:nC)], length 5*nC,
 * exactly the N_Vector layout of foeuler.f90:161-170.  Host-pointer entry
 * points take vectors in the caller's (reference) cell order; *_dev entry
 * points take vectors in the library's internal (renumbered) cell order, see
 * fos_ctx_permute_dev.
 *
 * Return codes follow the CVODE callback convention: 0 = success, > 0 =
 * recoverable failure (non-finite residual, zero pivot), < 0 = unrecoverable
 * (bad argument, CUDA error).  fos_last_error() describes the last failure.
 */
#ifndef FOSGPU_H
#define FOSGPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct fos_ctx fos_ctx;

/* Boundary condition codes (foeuler.f90:17-25).  FOS_BC_OUT_EXTRAP has no
 * reference counterpart: zero-gradient (supersonic) outflow, ghost = interior. */
enum {
  FOS_BC_WALL = 0,
  FOS_BC_IN_STATIC = 10,
  FOS_BC_IN_TOTAL = 11,
  FOS_BC_OUT = 20,
  FOS_BC_OUT_EXTRAP = 21,
  FOS_BC_FAR = 30
};

/* Precision of the Roe flux / preconditioner (flags of fos_ctx_create) */
enum {
  FOS_FLUX_FP64 = 0,   /* reference arithmetic, FP64 throughout */
  FOS_FLUX_FP32 = 1,   /* FP32 flux, FP64 accumulation and FD perturbation */
  FOS_ORDER_RCM = 0,   /* reverse Cuthill--McKee renumbering (default) */
  FOS_ORDER_NATURAL = 2,
  FOS_ILU_FP32 = 4,    /* ILU(0) factors and apply in FP32 */
  FOS_ILU_COLOR = 8,   /* ILU(0) on a multicolour ordering (few levels) */
  FOS_PREC_ILUT = 16,  /* pset/psol factor P with ILUT (FP64) instead of block ILU(0);
                          parameters from fos_ctx_set_ilut, default lfil 50, droptol 1e-6 */
  FOS_FLUX_HYBRID = 32 /* with FOS_FLUX_FP32: interior faces whose relative density or
                          pressure jump exceeds a threshold (fos_ctx_set_flux_threshold,
                          default 0.05) and all boundary faces are evaluated in FP64, the rest
                          in FP32 -- for shocked flows, where the FP32 rounding of the large
                          jumps puts the Newton residual's floor above its tolerance.  A
                          residual evaluation records the choice per face; a Jv reuses the
                          choice of the last residual on the context */
};

/* ------------------------------------------------------------------ setup */

/* Grid face arrays from element connectivity: the result of polyGrid%up and
 * polyFvGrid%up (polyGrid.f90:64-136, polyFvGrid.f90:48-227).  Elements are
 * TET (20) / HEX (21) cells and TRI (10) / QUAD (11) facets, iNE is m x nE
 * column-major with 1-based node ids.  Pairs come out in the reference order
 * (built per cell face, then ordered by max(iEP) with the same quicksort).
 * Returns an opaque handle; read it with fos_grid_sizes / fos_grid_copy. */
typedef struct fos_grid fos_grid;
int fos_grid_build(fos_grid** out, int nN, const double* pN, int nE, int m, const int* sE,
                   const int* nNE, const int* iNE, const int* gid);
/* out[0..6] = nC, nE, nP, nPi, nPb, maxFace, nF */
void fos_grid_sizes(const fos_grid* g, int* out);
/* iEP 2*nP (1-based), aP nP, normP 3*nP, pP 3*nP, v nC, neib maxFace*nC,
 * gid nE, p 3*nE (centroids), sE nE -- all in reference (sorted) element order.
 * Any output may be NULL. */
void fos_grid_copy(const fos_grid* g, int* iEP, double* aP, double* normP, double* pP,
                   double* v, int* neib, int* gid, double* p, int* sE);
void fos_grid_free(fos_grid* g);

/* Create a solver context from the face arrays of a polyFvGrid (the module
 * state that foeuler's init() builds, foeuler.f90:60-175).
 *   iEP      2*nP pair element ids (index_base 0 or 1), interior pairs first
 *   aP, normP, v  pair area, unit normal (3*nP), cell volume
 *   iBC      nE: row of the condition table per element (1-based, 0 = default wall)
 *   bcType   nBC condition codes, bcParam maxP*nBC (column-major, bc%p)
 *   flags    FOS_FLUX_*, FOS_ORDER_*, FOS_ILU_* bits
 * Uploads the grid to the current CUDA device.  Returns 0 or < 0. */
int fos_ctx_create(fos_ctx** out, int nC, int nE, int nPi, int nPb, const int* iEP,
                   const double* aP, const double* normP, const double* v, const int* iBC,
                   int nBC, const int* bcType, const double* bcParam, int maxP, double gamm,
                   double r, int index_base, int flags);
void fos_ctx_destroy(fos_ctx* ctx);
/* FOS_FLUX_HYBRID threshold: a face is evaluated in FP64 when |rho_R - rho_L| or
 * |p_R - p_L| exceeds theta times the smaller of the two sides' values.  Returns 0, or -1 for
 * theta <= 0 or a context without FOS_FLUX_HYBRID. */
int fos_ctx_set_flux_threshold(fos_ctx* ctx, double theta);
/* CUDA stream (cudaStream_t as void*) for all subsequent launches; NULL = legacy default */
int fos_ctx_set_stream(fos_ctx* ctx, void* stream);
/* out[0..8] = nC, nPi, nPb, nlev_fwd, nlev_bwd, nnzb, bandwidth, flags,
 * number of kernels launched so far on this context */
void fos_ctx_info(const fos_ctx* ctx, long* out);
/* reference<->internal order on the device: dir 0 = reference -> internal, 1 = back */
int fos_ctx_permute_dev(fos_ctx* ctx, const double* in, double* out, int dir);
/* internal cell id of every reference cell (old2new, 0-based), length nC */
int fos_ctx_renumbering(const fos_ctx* ctx, int* old2new);
/* position of every reference cell in the ILU(0) elimination order (0-based), after the
 * first pset; returns the number of colours (FOS_ILU_COLOR) or 0 (internal order) */
int fos_ctx_ilu_order(const fos_ctx* ctx, int* old2pos);
const char* fos_last_error(void);

/* ------------------------------------------------------------------ CVODE callbacks (host) */

/* rhs: dy/dt = -(sum of Roe face fluxes)/v with BC ghosts (foeuler.f90:349-375) */
int fos_euler_rhs(double t, const double* y, double* ydot, void* user_data);
/* pset: on jok == 0 assemble the Roe Jacobian (Euler.f90:159-333) and set *jcur = 1;
 * form P = I - gamma diag(1/v) J and factor it with block ILU(0)
 * (stub in the reference, foeuler.f90:378-405) */
int fos_euler_pset(double t, const double* y, const double* fy, int jok, int* jcur,
                   double gamma, void* user_data);
/* psol: z = P^{-1} r by the ILU(0) triangular solves (stub z = r in the reference,
 * foeuler.f90:408-437; SPARSKIT lusol, ilut.f:2272-2320) */
int fos_euler_psol(double t, const double* y, const double* fy, const double* r, double* z,
                   double gamma, double delta, int lr, void* user_data);

/* ------------------------------------------------------------------ device entry points */

int fos_euler_rhs_dev(fos_ctx* ctx, double t, const double* y, double* ydot);
/* The same residual as fos_euler_rhs_dev, for callers that cannot allocate device memory
 * when they evaluate it (a host code that owns a fixed device-memory budget and does all
 * allocation itself, or one that must not allocate inside its time loop).  It has no
 * counterpart in the reference.  Its scratch lives in one static device array of the
 * library (10.75 MiB on every device that loads it, held until exit) instead of the
 * context's buffers, so it serves grids of at most FOS_STATIC_MAX_CELLS cells and
 * FOS_STATIC_MAX_FACES faces and returns -1 beyond that.  The first call on a device looks
 * up the array's device address (make that first call before any stream capture).  All
 * calls share the array: calls whose kernels overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.  No part of the array needs to start
 * at zero.  Non-finite results are not flagged (use fos_euler_rhs for that).  The array's
 * address is looked up once per device and kept, so the library must not be used across a
 * cudaDeviceReset; the kernels of this call are not counted in fos_ctx_info's launches. */
#define FOS_STATIC_MAX_CELLS 65536
#define FOS_STATIC_MAX_FACES 147456
int fos_euler_rhs_dev_static(const fos_ctx* ctx, double t, const double* y, double* ydot);
/* Fused finite-difference Jacobian-vector product of G(y) = y - gamma f(y) - h:
 *   out = a*v + b*(f(y + s v) - fy)/s,  s = eps (1 + ||y||_2)/||v||_2
 * (the difference quotient CVODE's SPGMR forms through rhs); ynorm = ||y||_2.
 * a = 1, b = -gamma gives J_G v; a = 0, b = 1 gives J_f v. */
int fos_euler_jv_dev(fos_ctx* ctx, double t, const double* y, const double* fy, const double* v,
                     double* out, double a, double b, double ynorm, double eps);
/* The same product with ||v||_2 = vnorm supplied by the caller, as a Krylov method that
 * keeps its basis norms has it (CVODE's SPGMR passes unit basis vectors to the difference
 * quotient, and this library's driver takes ||v||^2 from the preconditioner's output pass):
 * no reduction pass over v.  vnorm = 0 gives out = a*v. */
int fos_euler_jv_dev_vnorm(fos_ctx* ctx, double t, const double* y, const double* fy,
                           const double* v, double* out, double a, double b, double ynorm,
                           double vnorm, double eps);
int fos_euler_pset_dev(fos_ctx* ctx, double t, const double* y, int jok, int* jcur,
                       double gamma);
int fos_euler_psol_dev(fos_ctx* ctx, const double* r, double* z);
/* Block Jacobian J (5x5 blocks, before scaling by -gamma/v): copies out the block CSR
 * whose rows and columns are ILU positions (fos_ctx_ilu_order maps reference cells to
 * positions).  rowptr nC+1, col nnzb, val 25*nnzb (row-major blocks).  Pass NULL to
 * query nnzb through the return value. */
long fos_euler_jac_copy(fos_ctx* ctx, int* rowptr, int* col, double* val);
/* The inverse of fos_euler_jac_copy: replace J by the caller's blocks (val 25*nnzb, the same
 * layout), e.g. a Jacobian assembled elsewhere or modified; the next fos_euler_pset[_dev]
 * with jok = 1 factors P = I - gamma diag(1/v) J from it (CVODE's jok contract: J kept, only
 * gamma new).  With FOS_ILU_FP32 the blocks are stored rounded to FP32.  No counterpart in
 * the reference (its pset is a stub).  Returns 0, or < 0 (FOS_PREC_ILUT contexts: -1). */
int fos_euler_jac_set(fos_ctx* ctx, const double* val);

/* ------------------------------------------------------------------ learned preconditioner */

/* A message-passing graph network over the cell-face graph used as a variable
 * (flexible-GMRES) preconditioner z = M(y; v); no counterpart in the reference.  Three
 * layers of width 64, BF16 weights, FP32 accumulation on the tensor cores.  Untrained
 * (fresh) networks are the identity.  Tetrahedral grids only. */
typedef struct fos_gnn fos_gnn;
int fos_gnn_create(fos_gnn** out, unsigned seed);
void fos_gnn_destroy(fos_gnn* g);
int fos_gnn_num_params(void);
int fos_gnn_get_params(const fos_gnn* g, float* host); /* FP32 master weights */
int fos_gnn_set_params(fos_gnn* g, const float* host);
/* z = M(y, gamma; v) on the context's graph (device vectors, internal order); gamma is the
 * BDF coefficient of J_G = I - gamma J (the network sees the local CFL number) */
int fos_gnn_apply_dev(fos_gnn* g, fos_ctx* ctx, const double* y, const double* v, double gamma,
                      double* z);
/* training: loss = mean((z/s_v - t/s_v)^2) over cells and components for the target
 * correction t; adds dloss/dweights to the gradient accumulator */
int fos_gnn_zero_grad(fos_gnn* g);
int fos_gnn_loss_grad_dev(fos_gnn* g, fos_ctx* ctx, const double* y, const double* v,
                          const double* t, double gamma, double* loss);
int fos_gnn_get_grad(const fos_gnn* g, float* host);
int fos_gnn_adam_step(fos_gnn* g, float lr, float beta1, float beta2, float eps,
                      float grad_scale);
/* network used by fos_bdf_run when opts.precond >= 2 (not owned by the context); g = NULL
   detaches.  Returns -2 on a grid with hexahedra (the network reads 4 neighbour slots). */
int fos_ctx_attach_gnn(fos_ctx* ctx, fos_gnn* g);

/* ------------------------------------------------------------------ ILUT */

/* Dual-threshold incomplete LU of a CSR matrix on the device: the reference's ILU class
 * (numerics/sparse.f90:52-63 type, :334-348 initILU, :370-383 factILU, :386-392 solveILU),
 * i.e. SPARSKIT ilut (ITSOL/ilut.f:38-382) and lusol (:2272-2320).  Given the same CSR
 * matrix the factors are bit-identical to ilut's.  CSR arrays are 0-based device arrays
 * (ia n+1, ja and a nnz); a row may list its columns in any order. */
typedef struct fos_ilut fos_ilut;
/* storage for n rows; lfil is clamped to n - 1 as initILU does (sparse.f90:341);
 * lfil < 0 returns -4 (ilut's ierr) */
int fos_ilut_create(fos_ilut** out, int n, int lfil);
/* factor (factILU): returns 0, -5 on a zero row (ilut's ierr), -6 if a dependency wait ran
 * out, -1 on bad arguments.  Synchronises the stream. */
int fos_ilut_factor_dev(fos_ilut* f, const int* ia, const int* ja, const double* a,
                        double droptol, void* stream);
/* x = (LU)^{-1} y (solveILU / lusol), device vectors, x may equal y; asynchronous */
int fos_ilut_solve_dev(fos_ilut* f, const double* y, double* x, void* stream);
/* after the stream has drained: 0, or -6 when a solve's dependency wait ran out */
int fos_ilut_status(fos_ilut* f);
/* Failure injection (tests of the bounded waits; no counterpart in the reference): every
 * dependency wait of the following factor and solve calls gives up after `polls` polls
 * (<= 0: the default 2^23), and row `withhold_row` (>= 0) is never published -- the factor
 * does not release it and the forward sweep does not store its unknown -- so every wait on
 * it runs out: fos_ilut_factor_dev returns -6 and a solve leaves fos_ilut_status at -6 with
 * NaN in the rows that waited.  withhold_row = -1 publishes every row again. */
int fos_ilut_set_wait_limit(fos_ilut* f, long polls, int withhold_row);
/* the factors in ilut's MSR layout on the host (1-based values): alu(1:n) the inverted
 * diagonal, jlu(1:n+1) row pointers, ju(1:n) the start of each U row; returns the used
 * length (all three pointers null: only the length), < 0 on error */
long fos_ilut_copy(const fos_ilut* f, double* alu, int* jlu, int* ju, long iwk);
/* out[0..5] = n, lfil, working-row capacity, kernels launched, levels of the L and U
 * dependency graphs (the sweeps claim rows level by level) */
int fos_ilut_info(const fos_ilut* f, long* out);
void fos_ilut_destroy(fos_ilut* f);
/* ILUT parameters of a context created with FOS_PREC_ILUT (fopbc's PBC_PREC_FILL = 50 and
 * PBC_PREC_DROPTOL = 1e-6 by default, modPbc.f90:21,658); takes effect at the next pset */
int fos_ctx_set_ilut(fos_ctx* ctx, int lfil, double droptol);

/* ------------------------------------------------------------------ driver */

typedef struct {
  int order;          /* 1 = BDF1; 2 = BDF2 (first step BDF1) */
  int nsteps;
  double dt;
  double newton_rtol; /* Newton: ||G(y)||_2 <= rtol ||y_n||_2 + atol sqrt(5 nC), FP64 */
  double newton_atol;
  int max_newton;
  int maxl;           /* (F)GMRES restart length */
  int max_restarts;
  double lin_rtol;    /* Krylov: ||r|| <= lin_rtol ||b|| */
  double jv_eps;      /* finite-difference increment scale; 0 = the default: sqrt(DBL_EPSILON)
                         for the FP64 flux, 1e-5 for the FP32 flux (whose rounding is relative
                         to the face jumps, not to the state) */
  int precond;        /* 0 = none, 1 = block ILU(0), 2 = learned network in flexible GMRES,
                         falling back to ILU(0) when it stagnates, falls behind the mean
                         residual reduction per iteration of the last ILU(0)-preconditioned
                         solve, or needs more iterations than that solve, after which the next
                         1, 4, 16, ... solves (four times more per consecutive fallback, reset
                         when the network converges a solve) use ILU(0) alone; 3 = learned network
                         without fallback (evaluation); 4 = ILU(0) followed by the learned
                         correction, z = u + N(y; u) with u = ILU(0) r, with the fallback
                         of 2; 5 = the same without fallback */
  int jac_reuse;      /* 0 = assemble J every BDF step (jok = 0), 1 = keep J from the first step */
  int resume;         /* 1 = continue the BDF history of the previous call (y must be its
                         result), and with msbp > 1 its preconditioner set-up count: CVODE
                         keeps its set-up across CVode calls */
  int msbp;           /* preconditioner set-up policy: 1 = pset at every BDF step (default);
                         m > 1 = CVODE's (cvLsSetup: MSBP = 20, DGMAX = 0.3): pset at the
                         first step of the call, when m steps have passed since the last one
                         or gamma changed by more than 30% since it, and when a step's Newton
                         iteration fails on a reused set-up (the step is retried with a fresh
                         one); otherwise psol uses the last factorisation */
  int predictor;      /* Newton's first iterate: 0 = y_n (default); 1 = CVODE's BDF predictor
                         at a constant step, the extrapolation through the last q + 1
                         accepted states (2 y_n - y_{n-1} at order 1, 3 y_n - 3 y_{n-1} +
                         y_{n-2} at order 2, lower while the history is shorter), with a
                         retry from y_n when Newton fails from it.  It pays on smooth flows
                         (fewer Newton iterations) and costs at shocks and transients, where
                         the fixed step cannot shrink as CVODE's would */
} fos_bdf_opts;

typedef struct {
  long n_rhs, n_jv, n_psol, n_pset, n_newton, n_lin_iters, n_steps, fails, n_fallback;
  double last_gnorm;
  double t;
  long n_learned;     /* applications of the learned preconditioner (of n_psol) */
  long n_gated;       /* learned mode: solves run with ILU(0) alone because the network's
                         last measured cost per decade of residual was no better */
  long n_reorth;      /* Arnoldi steps that needed the second Gram--Schmidt pass */
} fos_bdf_stats;

void fos_bdf_defaults(fos_bdf_opts* o);
/* One linear solve J_G x = b at state y (fy = f(y), device vectors, internal order) with
 * the driver's (F)GMRES(opts->maxl) to opts->lin_rtol and the preconditioner opts->precond
 * (the ILU(0) factorisation for (y, gamma) is made when needed).  stats->n_lin_iters
 * receives the Krylov iterations, stats->n_fallback the learned-to-ILU fallbacks.
 * Returns 0 converged, 1 not converged, 3 zero pivot, < 0 error. */
int fos_linear_solve_dev(fos_ctx* ctx, double t, const double* y, const double* fy,
                         double gamma, const double* b, double* x, const fos_bdf_opts* opts,
                         fos_bdf_stats* stats);
/* Advance y (device, internal order, 5*nC) by opts->nsteps fixed BDF steps from t0.
 * Returns 0, > 0 if a step failed to converge (1), hit a non-finite residual (2) or a
 * zero pivot (3); < 0 on errors.  A failed step is not taken: y is left at the last
 * accepted step (time stats->t, stats->n_steps steps taken). */
int fos_bdf_run(fos_ctx* ctx, double t0, double* y, const fos_bdf_opts* opts,
                fos_bdf_stats* stats);
/* Same with y a HOST array in the caller's (reference) cell order: copied to the device,
 * advanced, and copied back (the N_Vector-level entry point). */
int fos_bdf_run_host(fos_ctx* ctx, double t0, double* y, const fos_bdf_opts* opts,
                     fos_bdf_stats* stats);

/* ---------------------------------------------------------------- adaptive BDF
 * Variable-order (1..qmax <= 5), variable-step BDF with local error control, the time
 * stepping CVODE gives foeuler (CVodeCreate(CV_BDF), CVodeSStolerances, CVode to tout;
 * SUNDIALS.f90:745-845, foeuler.f90:14-15,171-174,450), restated from SUNDIALS' published
 * algorithm for the device driver: variable-coefficient BDF formulas at the actual past
 * times, an extrapolation predictor, the local error estimate
 * h / (t_{n+1} - t_{n-q}) ||y_{n+1} - y_pred|| in the weighted RMS norm with
 * weights 1 / (rtol |y_n| + atol), step factors 1 / ((b err)^(1/(k+1)) + 1e-6) with biases
 * b = 6 (orders q-1, q) and 10 (order q+1), order changes considered after q + 1 steps at
 * one order, steps changed only by factors >= 1.5, and on an error-test failure a factor
 * in [0.2, 0.9] (order 1 and 0.1 after three failures), on a Newton failure 0.25.  Each
 * step's nonlinear system is solved by the fixed-step driver's Newton--(F)GMRES with
 * `nk` (newton_rtol, maxl, precond, ...; nk->order, dt, nsteps and resume are unused).
 * The last step is shortened to land on tout.  No reference counterpart for the
 * interface; CVODE's adaptivity is the behaviour it restates. */
typedef struct {
  double rtol, atol;  /* local error tolerances (CVODE's RTOL 1e-6, ATOL 1e-12 in foeuler) */
  double h0;          /* first step size (> 0) */
  double hmin, hmax;  /* step bounds (hmax <= 0: unbounded) */
  int qmax;           /* maximum order, 1..5 */
  int max_steps;      /* attempted steps before giving up (<= 0: 100000) */
} fos_bdf_adapt_opts;
typedef struct {
  long n_accepted, n_err_fails, n_newton_fails;
  double h_last, t;
  int q_last;
  long steps_at_order[6];  /* accepted steps per order (index = order) */
} fos_bdf_adapt_stats;
void fos_bdf_adapt_defaults(fos_bdf_adapt_opts* o);
/* Advance y (device, internal order) from t0 to tout.  Returns 0 on reaching tout, 4 if
 * the step size fell below hmin or too many failures occurred at one step, 5 if
 * max_steps was exceeded, < 0 on errors.  nk_stats accumulates the Newton--Krylov work. */
int fos_bdf_adaptive(fos_ctx* ctx, double t0, double tout, double* y,
                     const fos_bdf_opts* nk, const fos_bdf_adapt_opts* ad,
                     fos_bdf_stats* nk_stats, fos_bdf_adapt_stats* ad_stats);

#ifdef __cplusplus
}
#endif
#endif
