/*
 * fos_oracle.h -- CPU oracle for the foeuler implicit inner loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * arithmetic (mianzhi/fosolvers, Fortran 2003 + SPARSKIT2 F77) used to check
 * the GPU library and to time the CPU baseline.  Nothing in the product
 * (fosolvers_gb300/, include/) links or calls it; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Parity pinning: the reference cannot be compiled here (Fortran, SUNDIALS
 * absent).  The restatement is pinned by the reference's own known-answer
 * tests that touch this path (src/test/ILU1.f90, matVecMul.f90,
 * BDFNewtonKrylov1.f90, NewtonKrylov1.f90, polyGrid1.f90, readVTK1.f90 face
 * order) plus property tests; the Roe residual, the Roe Jacobian and the BCs
 * have no known-answer test in the reference ("parity unpinned" for those
 * three, pinned only by line-by-line restatement and properties).
 *
 * Index conventions follow the reference: element, node and pair ids are
 * 1-based inside the grid arrays (iEP, neib, iNE); arrays are addressed
 * column-major like the Fortran (iEP[2*(i-1)+0] == iEP(1,i)).
 */
#ifndef FOS_ORACLE_H
#define FOS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* element shape codes (polyGrid.f90:10-21) */
enum { O_TRI = 10, O_QUAD = 11, O_TET = 20, O_HEX = 21 };
/* boundary condition codes (foeuler.f90:17-25) */
enum { O_BC_WALL = 0, O_BC_IN_STATIC = 10, O_BC_IN_TOTAL = 11, O_BC_OUT = 20, O_BC_FAR = 30,
       O_BC_OUT_EXTRAP = 21 /* zero-gradient supersonic outflow: NOT in the reference */ };

/* ---------------------------------------------------------------- grid */
typedef struct og_grid og_grid;
/* polyGrid%up + polyFvGrid getNeib/sort (polyGrid.f90:64-136, polyFvGrid.f90:48-227).
 * pN: 3*nN; sE,nNE,gid: nE; iNE: m*nE (1-based node ids, column-major). */
og_grid* og_grid_build(int nN, const double* pN, int nE, int m, const int* sE, const int* nNE,
                       const int* iNE, const int* gid);
void og_grid_free(og_grid* g);
/* sizes: out[0..6] = nC, nE, nP, nPi, nPb, maxFace, nF */
void og_grid_sizes(const og_grid* g, int* out);
/* copy out: iEP 2*nP (1-based), aP nP, normP 3*nP, pP 3*nP, v nC, neib maxFace*nC,
 * gid nE (sorted element order), p 3*nE (element centroids, sorted order), sE nE. Any may be NULL. */
void og_grid_copy(const og_grid* g, int* iEP, double* aP, double* normP, double* pP, double* v,
                  int* neib, int* gid, double* p, int* sE);
/* geometry primitives (geometry.f90) -- p is 3 x k column-major */
double og_a3p(const double* p);
void og_n3p(const double* p, double* n);
double og_v4p(const double* p);
double og_v8p(const double* p);
/* qsortI with permutation (sort.f90:15-65); perm is 1-based on return */
void og_qsort_perm(int n, int* a, int* perm);

/* ---------------------------------------------------------------- Euler */
typedef struct oe_ctx oe_ctx;
/* Module state of modFOEuler after init() (foeuler.f90:60-175), built from face arrays.
 * iEP 1-based 2*nP; neib maxFace*nC 1-based (0 = none); iBC nE (0 = default wall, else
 * 1-based row of the condition table); bcT nBC; bcP maxP*nBC (column-major).
 * rho0/rhou0/rhoE0 initialise ALL nE element slots (cells and ghost facets), like init(). */
oe_ctx* oe_new(int nC, int nE, int nPi, int nPb, const int* iEP, const double* aP,
               const double* normP, const double* v, int maxFace, const int* neib,
               const int* iBC, int nBC, const int* bcT, const double* bcP, int maxP,
               double gamm, double r, const double* rho0, const double* rhou0,
               const double* rhoE0);
void oe_free(oe_ctx* c);
/* number of OpenMP threads used by oe_rhs: 1 = reference pair order, serial (parity mode);
 * >1 = parallel pair loop with atomic scatter, the reference's own OpenMP structure */
void oe_set_threads(oe_ctx* c, int nthreads);
/* cell order of the ILU(0) factorisation in pset/psol: old2new[c] = position of reference
 * cell c (0-based); NULL = the reference's natural order.  ILU(0) depends on the order, so
 * parity with a renumbered GPU factorisation uses the GPU's order here. */
void oe_set_ilu_order(oe_ctx* c, const int* old2new);
/* pset/psol with ILUT (lfil, droptol; sized as the ILU class) instead of ilu0; lfil < 0
 * goes back to ilu0.  oe_ilut_factors: the last ILUT factors (MSR), returns iwk or -1 */
void oe_set_ilut(oe_ctx* c, int lfil, double droptol);
int oe_ilut_factors(const oe_ctx* c, const double** alu, const int** jlu, const int** ju);
/* the three CVODE callbacks (foeuler.f90:349-437) with N_Vector data as raw arrays;
 * ud is the oe_ctx*.  pset assembles findEulerJac, P = I - gamma*diag(1/v)*JacC in
 * interleaved (cell-major) scalar COO, coocsr, sorted rows, ilu0; psol = lusol. */
int oe_rhs(double t, const double* y, double* ydot, void* ud);
int oe_pset(double t, const double* y, const double* fy, int jok, int* jcur, double gamma,
            void* ud);
int oe_psol(double t, const double* y, const double* fy, const double* r, double* z,
            double gamma, double delta, int lr, void* ud);
/* findEulerJac on the state y (setBC + syncState first).  JacC is 5 x 5*(maxFace+1) x nC
 * column-major like the Fortran array; returns pointer to internal storage. */
const double* oe_jac(oe_ctx* c, const double* y);
/* last pset/psol internals: scalar CSR of P (1-based), n = 5*nC */
int oe_pmat(const oe_ctx* c, const double** a, const int** ja, const int** ia);
int oe_ilu_ierr(const oe_ctx* c);
/* ghost state after the last rhs (element slot n > nC): rho(nE), rhou(3*nE), rhoE(nE) */
void oe_elem_state(const oe_ctx* c, double* rho, double* rhou, double* rhoE);
/* 10x10 pair Jacobian eulerNFJ / eulerANFJ probes (Euler.f90:252-333), 5x5 column-major */
void oe_nfj(const double* norm, const double* u, double H, double gamm, double* out);
void oe_anfj(const double* norm, const double* u, double H, double cc, double gamm, double* out);

/* ---------------------------------------------------------------- SPARSKIT (1-based) */
void o_coocsr(int nrow, int nnz, const double* a, const int* ir, const int* jc, double* ao,
              int* jao, int* iao);
void o_csrsort(int n, double* a, int* ja, const int* ia); /* sort each row by column */
void o_amux(int n, const double* x, double* y, const double* a, const int* ja, const int* ia);
/* alu, jlu sized nnz+1 (MSR); ju n; iw n work.  returns ierr (0 ok, k = zero pivot at k) */
int o_ilu0(int n, const double* a, const int* ja, const int* ia, double* alu, int* jlu, int* ju,
           int* iw);
void o_lusol(int n, const double* y, double* x, const double* alu, const int* jlu, const int* ju);
void o_qsplit(double* a, int* ind, int n, int ncut);
/* ILUT: alu, jlu sized iwk (>= n*(2*lfil+1) suffices), ju n, w n+1, jw 2n (work).
 * returns ierr (0 ok, -1..-5 as SPARSKIT) */
int o_ilut(int n, const double* a, const int* ja, const int* ia, int lfil, double droptol,
           double* alu, int* jlu, int* ju, int iwk, double* w, int* jw);

/* ---------------------------------------------------------------- Newton-Krylov / BDF */
typedef int (*o_rhs_fn)(double t, const double* y, double* ydot, void* ud);
typedef int (*o_pset_fn)(double t, const double* y, const double* fy, int jok, int* jcur,
                         double gamma, void* ud);
typedef int (*o_psol_fn)(double t, const double* y, const double* fy, const double* r,
                         double* z, double gamma, double delta, int lr, void* ud);
typedef struct {
  int order;          /* 1 = BDF1, 2 = BDF2 (first step BDF1) */
  double dt;
  int nsteps;
  double newton_rtol; /* Newton: ||G(y)||_2 <= rtol*||y_n||_2 + atol*sqrt(n) */
  double newton_atol;
  int max_newton;
  int maxl;           /* GMRES restart length */
  int max_restarts;
  double lin_rtol;    /* GMRES: ||r|| <= lin_rtol*||b|| */
  double jv_eps;      /* sqrt(eps) for the finite-difference Jv increment */
  int use_prec;       /* 0 = identity psol */
  int msbp;           /* 1 = pset every step; m > 1 = CVODE's set-up policy (cvLsSetup:
                         at most m steps between set-ups, or a > 30% gamma change, or a
                         Newton failure on a reused set-up, after which the step is retried) */
  int predictor;      /* Newton's first iterate: 0 = y_n (default); 1 = extrapolation through
                         the last q + 1 accepted states (CVODE's BDF predictor at a constant
                         step: 2 y_n - y_{n-1} at order 1, 3 y_n - 3 y_{n-1} + y_{n-2} at
                         order 2; lower order while the history is shorter), retried from
                         y_n when Newton fails from it */
} o_bdf_opts;
typedef struct {
  long n_rhs, n_jv, n_psol, n_pset, n_newton, n_lin_iters, n_steps, fails;
  double last_gnorm;
} o_bdf_stats;
void o_bdf_defaults(o_bdf_opts* o);
/* the driver's finite-difference Jv: out = a v + b (f(y + s v) - fy)/s,
 * s = eps (1 + ynorm)/||v||_2; ytmp and ftmp are n-double work arrays */
int o_jv(int n, o_rhs_fn f, void* ud, double t, const double* y, const double* fy,
         const double* v, double* out, double a, double b, double ynorm, double eps,
         double* ytmp, double* ftmp);
/* fixed-step BDF1/BDF2 Newton--GMRES(maxl) with right preconditioning, CGS + DGKS Arnoldi.
 * y in/out (length n). returns 0 on success, >0 if a step failed to converge. */
int o_bdf_run(int n, o_rhs_fn rhs, o_pset_fn pset, o_psol_fn psol, void* ud, double t0,
              double* y, const o_bdf_opts* opts, o_bdf_stats* st);
/* Newton--GMRES on a steady G(x) = 0 written as the rhs callback (G = rhs(t=0,x)). */
typedef struct {
  double rtol, atol, h0, hmin, hmax;
  int qmax, max_steps;
} o_adapt_opts;
typedef struct {
  long n_accepted, n_err_fails, n_newton_fails;
  double h_last, t;
  int q_last;
  long steps_at_order[6];
} o_adapt_stats;
void o_adapt_defaults(o_adapt_opts* o);
/* variable-order, variable-step BDF from t0 to tout (0 ok, 2 rhs failure, 4 step failures,
 * 5 too many steps) */
int o_bdf_adaptive(int n, o_rhs_fn rhs, o_pset_fn pset, o_psol_fn psol, void* ud, double t0,
                   double tout, double* y, const o_bdf_opts* nk, const o_adapt_opts* ad,
                   o_bdf_stats* st, o_adapt_stats* as);
int o_newton_solve(int n, o_rhs_fn G, void* ud, double* x, double rtol, double atol,
                   int max_newton, int maxl, double lin_rtol, o_bdf_stats* st);

#ifdef __cplusplus
}
#endif
#endif
