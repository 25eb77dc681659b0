// fos_bdf.cu -- device-resident fixed-step BDF Newton--Krylov driver.
//
// The reference advances foeuler with CVODE (BDF + Newton + SPGMR, SUNDIALS.f90:745-845),
// which is not vendored.  This driver restates the published algorithm with fixed steps
// (the workloads prescribe fixed-step BDF1/BDF2) and keeps every vector in HBM:
//   BDF1: G(y) = y - dt f(y) - y_n                      gamma = dt
//   BDF2: G(y) = y - 2/3 dt f(y) - (4/3 y_n - 1/3 y_{n-1})  gamma = 2/3 dt (first step BDF1)
//   Newton: y_0 = y_n (or, with opts->predictor, the constant-step BDF extrapolation);
//           stop when ||G(y_k)||_2 <= rtol ||y_0||_2 + atol sqrt(N), in FP64
//   linear: right-preconditioned restarted GMRES(maxl) on J_G d = -G, Arnoldi by classical
//           Gram--Schmidt in FP64 with a second pass when ||w_1|| < min(1/sqrt(2), lin_rtol)
//           ||w_0|| (the DGKS test, threshold bounded by the Krylov tolerance),
//           Givens least squares on the host, stop at ||r|| <= lin_rtol ||G||
//   J_G v = v - gamma (f(y + s v) - f(y))/s, s = jv_eps (1 + ||y||)/||v|| (fused kernel)
//   preconditioner: pset once per BDF step (jok = 0 unless jac_reuse), psol = block ILU(0)
// All reductions are deterministic two-stage warp-shuffle reductions.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "fos_internal.h"


// Default scale of the finite-difference increment s = eps (1 + ||y||)/||v||.
// FP64 flux: sqrt(DBL_EPSILON), the classic balance of truncation against rounding.
// FP32 flux: 1e-5.  The flux-difference form rounds each face term relative to the face's
// jump, not to the state, so the rounding noise of f is about FLT_EPSILON times the relative
// jump between neighbours (1e-3 to 1e-2 on these meshes) and the balancing increment is
// near 1e-5.  sqrt(FLT_EPSILON) = 3.5e-4 is too large: s v is a global perturbation of l2
// norm eps (1 + ||y||), so on a Krylov vector concentrated on K of N unknowns (a shock) each
// of them moves by eps ||y|| / sqrt(K), sqrt(N/K) times more than on a spread-out vector,
// and the difference quotient leaves its linear range.  Measured: on the 2.36 M-tet bump at
// CFL 5 the Newton iteration diverged at 3.5e-4 (FP32 and FP64 flux alike) and converged at
// 1e-4 and below; on the 5.3 M-tet sine workload 1e-5 takes the FP64 path's Newton and
// Krylov counts (10 and 26 over five steps, against 11 and 29 at 3.5e-4).
static double jv_eps_default(const fos_ctx* c) {
  return (c->flags & FOS_FLUX_FP32) ? 1e-5 : std::sqrt(DBL_EPSILON);
}

namespace {

constexpr int kT = 256;
constexpr int kMaxVec = 32;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// block-reduce nv accumulators into part[l * gridDim.x + blockIdx.x]
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&acc)[NV], int nv, double* part) {
  __shared__ double sh[kT / 32][kMaxVec];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int l = 0; l < NV; l++) {
    if (l < nv) {
      double s = warp_sum(acc[l]);
      if (lane == 0) sh[wid][l] = s;
    }
  }
  __syncthreads();
  for (int l = threadIdx.x; l < nv; l += blockDim.x) {
    double s = 0.0;
    for (int w = 0; w < kT / 32; w++) s += sh[w][l];
    part[(size_t)l * gridDim.x + blockIdx.x] = s;
  }
}

// h[l] = V_l . w for l < NV (NV fixed at compile time: accumulators stay in registers),
// plus h[NV] = ||w||^2 when NRM
template <int NV, bool NRM>
__global__ void __launch_bounds__(kT) k_mdot(long n, const double* __restrict__ V, long ldv,
                                             const double* __restrict__ w,
                                             double* __restrict__ part) {
  constexpr int NA = NV + (NRM ? 1 : 0);
  double acc[NA];
#pragma unroll
  for (int l = 0; l < NA; l++) acc[l] = 0.0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double wi = w[i];
#pragma unroll
    for (int l = 0; l < NV; l++) acc[l] += V[(size_t)l * ldv + i] * wi;
    if (NRM) acc[NA - 1] += wi * wi;
  }
  block_reduce_store<NA>(acc, NA, part);
}

// w -= sum_l h[l] s2[l] V_l ; then part <- V_l . w (MODE 0, CGS2 second pass), ||w||^2
// (MODE 1), or both (MODE 2: the DGKS test and, when it fails, the second pass's
// coefficients come out of the same sweep over V).  s2 (null: all 1) are the squared
// scales of unnormalised basis vectors (v_l = s_l V_l), so h = V^T w gives the coefficients
// of the projection onto the v_l.
template <int NV, int MODE>
__global__ void __launch_bounds__(kT) k_update(long n, const double* __restrict__ V, long ldv,
                                               const double* __restrict__ h,
                                               const double* __restrict__ s2,
                                               double* __restrict__ w,
                                               double* __restrict__ part) {
  __shared__ double hs[NV];
  if (threadIdx.x < NV) hs[threadIdx.x] = s2 ? h[threadIdx.x] * s2[threadIdx.x] : h[threadIdx.x];
  __syncthreads();
  constexpr int NA = MODE == 0 ? NV : MODE == 1 ? 1 : NV + 1;
  double acc[NA];
#pragma unroll
  for (int l = 0; l < NA; l++) acc[l] = 0.0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double vv[NV];
    double wi = w[i];
#pragma unroll
    for (int l = 0; l < NV; l++) {
      vv[l] = V[(size_t)l * ldv + i];
      wi -= hs[l] * vv[l];
    }
    w[i] = wi;
    if (MODE != 1) {
#pragma unroll
      for (int l = 0; l < NV; l++) acc[l] += vv[l] * wi;
    }
    if (MODE != 0) acc[NA - 1] += wi * wi;
  }
  block_reduce_store<NA>(acc, NA, part);
}

// out[l] = sum of part[l * np ...]
__global__ void k_final(int nv, int np, const double* __restrict__ part, double* __restrict__ out) {
  const int l = blockIdx.x;
  if (l >= nv) return;
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[(size_t)l * np + i];
  __shared__ double sh[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) out[l] = t;
  }
}

__global__ void k_scale(long n, const double* __restrict__ x, double a, double* __restrict__ y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i];
}
__global__ void k_axpy(long n, double a, const double* __restrict__ x, double* __restrict__ y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}
// s = sum_l c[l] Z_l, summed from x (kAcc) or from zero; then x = s, or, with kAdd, yadd += s
// and x is not touched (the first restart cycle's correction added straight to the Newton
// iterate: the same sums as x = s followed by yadd += x).  The variants are compile-time and
// the vector loop is not unrolled, so no FP64 instruction is issued predicated off.
template <bool kAcc, bool kAdd>
__global__ void k_comb(long n, int nv, const double* __restrict__ Z, long ldz,
                       const double* __restrict__ cc, double* __restrict__ x,
                       double* __restrict__ yadd) {
  __shared__ double cs[kMaxVec];
  if (threadIdx.x < kMaxVec) cs[threadIdx.x] = threadIdx.x < nv ? cc[threadIdx.x] : 0.0;
  __syncthreads();
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  int l0 = 0;
  if constexpr (kAcc) {
    s = x[i];
  } else if (nv > 0) {
    s = cs[0] * Z[i];
    l0 = 1;
  }
#pragma unroll 1
  for (int l = l0; l < nv; l++) s = fma(cs[l], Z[(size_t)l * ldz + i], s);
  if constexpr (kAdd) yadd[i] += s;
  else x[i] = s;
}
// hist = y_n (q=1) or 4/3 y_n - 1/3 y_{n-1} (q=2)
__global__ void k_hist(long n, int q, const double* __restrict__ yn, const double* __restrict__ ym,
                       double* __restrict__ h) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  h[i] = q == 1 ? yn[i] : (4.0 / 3.0) * yn[i] - (1.0 / 3.0) * ym[i];
}
// Newton's first iterate, the extrapolation of order p through y_n, y_{n-1}, y_{n-2} at a
// constant step (CVODE's BDF predictor): p = 1: (y_n - y_{n-1}) + y_n; p = 2:
// 3 (y_n - y_{n-1}) + y_{n-2} (rounded operation by operation, as the oracle forms it)
template <int P>
__global__ void k_predict(long n, const double* __restrict__ yn, const double* __restrict__ ym,
                          const double* __restrict__ ym2, double* __restrict__ y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dlt = __dsub_rn(yn[i], ym[i]);
  y[i] = P == 1 ? __dadd_rn(dlt, yn[i]) : __dadd_rn(__dmul_rn(3.0, dlt), ym2[i]);
}
// G = y - gamma f - hist; b = -G (also into b2: the first Arnoldi vector, unnormalised);
// part0 <- sum G^2, part1 <- sum y^2
__global__ void __launch_bounds__(kT) k_newton_res(long n, const double* __restrict__ y,
                                                   const double* __restrict__ f,
                                                   const double* __restrict__ hist,
                                                   double gamma, double* __restrict__ b,
                                                   double* __restrict__ b2,
                                                   double* __restrict__ part) {
  double acc[2] = {0.0, 0.0};
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double yi = y[i];
    // -G = (gamma f - y) + hist, formed directly: round-to-nearest is symmetric, so this is
    // -(fma(-gamma, f, y) - hist) bit for bit, without a negation on the FP64 pipe
    const double B = fma(gamma, f[i], -yi) + hist[i];
    b[i] = B;
    b2[i] = B;
    acc[0] = fma(B, B, acc[0]);
    acc[1] = fma(yi, yi, acc[1]);
  }
  block_reduce_store<2>(acc, 2, part);
}

// out = sum_l c[l] p[l] (up to 8 vectors, summed in order l = 0, 1, ...)
struct Comb8 {
  const double* p[8];
  double c[8];
  int nv;
};
__global__ void k_lincomb(long n, Comb8 cb, double* __restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int l = 0; l < cb.nv; l++) s += cb.c[l] * cb.p[l][i];
  out[i] = s;
}
// part <- sum of (a_i / (rtol |w_i| + atol))^2 (weighted RMS norm, before the mean)
__global__ void __launch_bounds__(kT) k_wrms_part(long n, const double* __restrict__ a,
                                                  const double* __restrict__ w, double rtol,
                                                  double atol, double* __restrict__ part) {
  double acc[1] = {0.0};
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double e = a[i] / (rtol * fabs(w[i]) + atol);
    acc[0] += e * e;
  }
  block_reduce_store<1>(acc, 1, part);
}

inline int nb(long n) { return (int)((n + kT - 1) / kT); }

}  // namespace

struct fos_bdf_work {
  long N = 0;
  int maxl = 0;
  bool has_hist = false;  // yn holds the last accepted state, ym the one before
  int nhist = 0;          // accepted states held in yn, ym, ym2 (at most 3)
  int ilu_ref_its = -1;   // learned mode: iterations of the last ILU(0)-preconditioned solve
  double ilu_ref_rate = 1.0;  // learned mode: its mean residual reduction per iteration
  int learned_backoff = 0;  // learned mode: solves skipped after the last fallback
  int learned_skip = 0;     // learned mode: solves still to run with ILU(0) alone
  // learned mode, the cost model that gates the network: the fastest Krylov iteration seen
  // with ILU(0) and with the network (wall time, ms; 0 = none yet), and the network's mean
  // residual reduction per iteration in its last solve (-1 = not tried yet)
  double t_it_ilu = 0.0, t_it_net = 0.0;
  double net_rate = -1.0;
  int setup_age = -1;       // set-up policy: steps since the last set-up at the end of the
                            // last call (-1: none that a resumed call may keep)
  double gamma_setup = 0.0; // and the gamma it was made for
  long setup_serial = -1;   // the context's set-up count then (a set-up made outside the
                            // driver in between voids the kept one)
  double t_last = 0.0;
  double* ym2 = nullptr;  // the accepted state before ym (the order-2 predictor)
  double *V = nullptr, *Z = nullptr, *w = nullptr, *yn = nullptr, *ym = nullptr,
         *hist = nullptr, *f = nullptr, *b = nullptr, *d = nullptr, *part = nullptr,
         *sc = nullptr, *yh = nullptr, *u = nullptr;
  // adaptive driver only (allocated on first use): solution history, predictor, error
  // vectors of this and the previous step, scratch
  double* ay[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double *ypred = nullptr, *E = nullptr, *Eprev = nullptr, *atmp = nullptr;
  ~fos_bdf_work() {
    for (double* p : {V, Z, w, yn, ym, ym2, hist, f, b, d, part, sc, yh, u, ypred, E, Eprev,
                      atmp})
      if (p) cudaFree(p);
    for (double* p : ay)
      if (p) cudaFree(p);
  }
};
void fos_bdf_work_free(fos_bdf_work* w) { delete w; }

namespace {
using Work = fos_bdf_work;

int work_get(fos_ctx* c, int maxl, Work** out) {
  Work* wk = c->bdf;
  const long N = 5L * c->nC;
  if (wk && wk->maxl >= maxl) {
    *out = wk;
    return 0;
  }
  delete wk;
  c->bdf = nullptr;
  wk = new Work();
  wk->N = N;
  wk->maxl = maxl;
  c->bdf = wk;
  FOS_CUDA(cudaMalloc(&wk->V, sizeof(double) * N * (maxl + 1)));
  FOS_CUDA(cudaMalloc(&wk->Z, sizeof(double) * N * maxl));
  for (double** p : {&wk->w, &wk->yn, &wk->ym, &wk->ym2, &wk->hist, &wk->f, &wk->b, &wk->d,
                     &wk->yh, &wk->u})
    FOS_CUDA(cudaMalloc(p, sizeof(double) * N));
  FOS_CUDA(cudaMalloc(&wk->part, sizeof(double) * kRedBlocks * kMaxVec));
  FOS_CUDA(cudaMalloc(&wk->sc, sizeof(double) * 6 * kMaxVec));
  *out = wk;
  return 0;
}

}  // namespace

extern "C" void fos_bdf_defaults(fos_bdf_opts* o) {
  o->order = 1;
  o->nsteps = 1;
  o->dt = 1e-3;
  o->newton_rtol = 1e-8;
  o->newton_atol = 1e-12;
  o->max_newton = 10;
  o->maxl = 30;
  o->max_restarts = 4;
  o->lin_rtol = 1e-3;
  o->jv_eps = 0.0;  // 0 = sqrt(machine epsilon of the flux precision)
  o->precond = 1;
  o->jac_reuse = 0;
  o->msbp = 1;
  o->resume = 0;
  o->predictor = 0;
}

namespace {

struct Driver {
  fos_ctx* c;
  Work& wk;
  const fos_bdf_opts& o;
  fos_bdf_stats& st;
  double eps;
  // preconditioner of the current linear solve: 0 none, 1 ILU(0), 2/3 learned network,
  // 4/5 ILU(0) followed by the learned correction (2 and 4 fall back to ILU(0))
  int pc = 0;
  // learned mode: ILU(0) factorisation is made on demand (fallback) once per BDF step
  bool pset_done = false;
  bool keep_setup = false;  // the step reuses the last factorisation (msbp > 1)
  bool setup_made = false;  // a pset ran during the current step
  double t_step = 0.0, gamma_step = 0.0;
  const double* y_step = nullptr;
  int ilu_ref_its = -1;  // Krylov iterations of the last ILU(0)-preconditioned solve
  double ilu_ref_rate = 1.0;  // and its mean residual reduction per iteration
  // an ILU(0)-preconditioned solve reached residual res after its iterations
  void set_ilu_ref(int its, double res, double bnorm) {
    ilu_ref_its = its;
    ilu_ref_rate = (its > 0 && bnorm > 0.0 && res > 0.0) ? std::pow(res / bnorm, 1.0 / its) : 0.0;
  }

  int reduce(int nv, double* out) {  // k_final over wk.part into device out
    fos_launch(c, k_final, nv, 256, nv, kRedBlocks, wk.part, out);
    FOS_LAUNCH_CHECK();
    return 0;
  }
  template <bool NRM>
  int mdot(int nv, const double* V, long ldv, const double* w) {
    switch (nv) {
#define FOS_MDOT(K) \
  case K: fos_launch(c, k_mdot<K, NRM>, kRedBlocks, kT, wk.N, V, ldv, w, wk.part); break;
      FOS_MDOT(1) FOS_MDOT(2) FOS_MDOT(3) FOS_MDOT(4) FOS_MDOT(5) FOS_MDOT(6) FOS_MDOT(7)
      FOS_MDOT(8) FOS_MDOT(9) FOS_MDOT(10) FOS_MDOT(11) FOS_MDOT(12) FOS_MDOT(13) FOS_MDOT(14)
      FOS_MDOT(15) FOS_MDOT(16) FOS_MDOT(17) FOS_MDOT(18) FOS_MDOT(19) FOS_MDOT(20) FOS_MDOT(21)
      FOS_MDOT(22) FOS_MDOT(23) FOS_MDOT(24) FOS_MDOT(25) FOS_MDOT(26) FOS_MDOT(27) FOS_MDOT(28)
      FOS_MDOT(29) FOS_MDOT(30) FOS_MDOT(31)
#undef FOS_MDOT
      default: fos_set_error("mdot: too many vectors"); return -1;
    }
    FOS_LAUNCH_CHECK();
    return 0;
  }
  template <int MODE>
  int update(int nv, const double* V, long ldv, const double* h, double* w,
             const double* s2 = nullptr) {
    switch (nv) {
#define FOS_UPD(K) \
  case K: fos_launch(c, k_update<K, MODE>, kRedBlocks, kT, wk.N, V, ldv, h, s2, w, wk.part); break;
      FOS_UPD(1) FOS_UPD(2) FOS_UPD(3) FOS_UPD(4) FOS_UPD(5) FOS_UPD(6) FOS_UPD(7) FOS_UPD(8)
      FOS_UPD(9) FOS_UPD(10) FOS_UPD(11) FOS_UPD(12) FOS_UPD(13) FOS_UPD(14) FOS_UPD(15)
      FOS_UPD(16) FOS_UPD(17) FOS_UPD(18) FOS_UPD(19) FOS_UPD(20) FOS_UPD(21) FOS_UPD(22)
      FOS_UPD(23) FOS_UPD(24) FOS_UPD(25) FOS_UPD(26) FOS_UPD(27) FOS_UPD(28) FOS_UPD(29)
      FOS_UPD(30) FOS_UPD(31)
#undef FOS_UPD
      default: fos_set_error("update: too many vectors"); return -1;
    }
    FOS_LAUNCH_CHECK();
    return 0;
  }
  int fetch(const double* d, double* h, int n) {
    FOS_CUDA(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    FOS_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
  }
  double gamma_cur = 0.0;  // gamma of the current linear solve (input of the learned preconditioner)
  // z = M^-1 r; with d_zsq (plain ILU(0) only, else ignored) also ||z||^2 into d_zsq from
  // the apply's own pass over z -- the norm the next Jv of z needs.  Returns in *have_sq
  // whether it did.
  int psolve(const double* y, const double* r, double* z, double* d_zsq = nullptr,
             bool* have_sq = nullptr) {
    st.n_psol++;
    if (have_sq) *have_sq = false;
    if (pc == 0) {
      FOS_CUDA(cudaMemcpyAsync(z, r, sizeof(double) * wk.N, cudaMemcpyDeviceToDevice, c->stream));
      return 0;
    }
    if (pc >= 2) st.n_learned++;
    if (pc == 2 || pc == 3) return fos_gnn_precond(c, y, r, gamma_cur, z);
    if (pc >= 4) {  // z = u + N(y; u), u = ILU(0) r
      if (int rc = fos_ilu_apply(c, r, wk.u)) return rc;
      return fos_gnn_precond(c, y, wk.u, gamma_cur, z);
    }
    if (have_sq) *have_sq = d_zsq != nullptr;
    return fos_ilu_apply(c, r, z, d_zsq);
  }
  // Expected cost of a fixed residual reduction: iteration time / -log(rate per iteration).
  // The network is not applied while its last solve's rate at its iteration time buys that
  // reduction no cheaper than the last ILU(0) solve did -- the history already predicts a
  // loss.  A
  // slower ILU(0) solve (a harder state) reopens the gate; a network that was never tried,
  // or iterations not yet timed, leave it open.
  bool network_predicted_to_lose() const {
    if (wk.net_rate < 0.0 || ilu_ref_its < 0 || wk.t_it_ilu <= 0.0 || wk.t_it_net <= 0.0)
      return false;
    if (wk.net_rate >= 1.0) return true;
    if (!(ilu_ref_rate > 0.0)) return true;  // ILU(0) converged at once
    return wk.t_it_net * -std::log(ilu_ref_rate) >= wk.t_it_ilu * -std::log(wk.net_rate);
  }
  void note_iteration_time(double ms) {
    double& t = pc == 1 ? wk.t_it_ilu : wk.t_it_net;
    if (pc == 1 || pc == 2 || pc == 4) t = t > 0.0 ? std::min(t, ms) : ms;
  }
  // the network lost this solve: ILU(0) from here on, and the exponential back-off skips the
  // network for the next 1, 4, 16, ... solves, so a network that keeps losing to ILU(0)
  // costs a vanishing share of a long run
  void note_fallback() {
    st.n_fallback++;
    wk.learned_backoff = wk.learned_backoff ? std::min(4 * wk.learned_backoff, 1 << 20) : 1;
    wk.learned_skip = wk.learned_backoff;
    pc = 1;
  }
  int ensure_pset() {
    if (pset_done) return 0;
    int jcur = 0;
    const int jok = (o.jac_reuse && c->has_jac) ? 1 : 0;
    int rc = fos_euler_pset_dev(c, t_step, y_step, jok, &jcur, gamma_step);
    if (rc) return rc;
    st.n_pset++;
    pset_done = true;
    setup_made = true;
    return c->ilu_ierr ? 3 : 0;
  }
  // w = J_G v at state y with f(y) = fy
  // w = J_G v by the finite difference; have_sq: ||v||^2 is already in c->d_scal[0]
  int jv(const double* y, const double* fy, const double* v, double* w, double gamma,
         double ynorm, bool have_sq = false) {
    st.n_jv++;
    st.n_rhs++;
    int rc = have_sq ? 0 : fos_norm2_dev(c, v, wk.N, c->d_scal);
    if (rc) return rc;
    rc = fos_jv_sigma(c, c->d_scal, ynorm, eps, -gamma);
    if (rc) return rc;
    return fos_residual_launch(c, y, v, c->d_scal + 1, fy, w, 1.0, -gamma, 1);
  }

  long reorth = 0;
  bool last_reorth = false;  // the previous Arnoldi step needed the second Gram--Schmidt pass

  // Newton iteration for G(y) = y - gamma f(y) - hist = 0 at time tn from the initial
  // iterate y_0 in y, until ||G||_2 <= newton_rtol ||y_0||_2 + newton_atol sqrt(N); the
  // preconditioner is set up (lazily) once for the solve.  Returns 0 converged, 1 not
  // converged in max_newton, 2 non-finite residual, 3 zero pivot in ILU(0), < 0 error.
  int newton(double* y, double gamma, const double* hist, double tn) {
    const long N = wk.N;
    double hb[2], gtol = 0.0;
    for (int k = 0; k <= o.max_newton; k++) {
      FOS_CUDA(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
      int rc = fos_residual_launch(c, y, nullptr, nullptr, nullptr, wk.f, 0.0, 0.0, 0);
      if (rc) return rc;
      st.n_rhs++;
      fos_launch(c, k_newton_res, kRedBlocks, kT, N, (const double*)y, (const double*)wk.f,
                 hist, gamma, wk.b, wk.V, wk.part);
      if ((rc = reduce(2, wk.sc))) return rc;
      FOS_CUDA(cudaMemcpyAsync(hb, wk.sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      FOS_CUDA(cudaMemcpyAsync(c->h_scal, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      FOS_CUDA(cudaStreamSynchronize(c->stream));
      if (*(int*)c->h_scal) return 2;  // non-finite residual
      // the first pass also gives ||y_0||
      if (k == 0) gtol = o.newton_rtol * std::sqrt(hb[1]) + o.newton_atol * std::sqrt((double)N);
      const double gn = std::sqrt(hb[0]);
      st.last_gnorm = gn / gtol;
      if (gn <= gtol) return 0;
      if (k == o.max_newton) break;
      if (k == 0) {
        pset_done = keep_setup;
        t_step = tn;
        gamma_step = gamma;
        y_step = y;
      }
      // ||b|| = ||G|| (b = -G) for the linear tolerance and GMRES's first basis vector
      int its = 0;
      bool added = false;  // GMRES added d to y itself (it converged in its first cycle)
      rc = gmres(y, wk.f, gamma, std::sqrt(hb[1]), gn, &its, y, &added, true);
      st.n_lin_iters += its;
      st.n_newton++;
      if (rc < 0) return rc;
      if (rc == 3) return 3;  // zero pivot in the ILU(0) factorisation
      if (!added) {
        fos_launch(c, k_axpy, nb(N), kT, N, 1.0, wk.d, y);
        FOS_LAUNCH_CHECK();
      }
    }
    return 1;
  }
  // GMRES on J_G d = b; d starts at zero.  With a learned preconditioner (o.precond >= 2)
  // this is flexible GMRES (Z_j = M_j(V_j) kept); in modes 2 and 4 it falls back to ILU(0)
  // when the residual estimate stagnates (> 0.9 of the previous one), falls behind the last
  // ILU(0)-preconditioned solve's rate, or the iteration count reaches that solve's: the
  // cycle goes on with ILU(0) (a non-finite estimate restarts it from the current iterate).
  // With y_add (the Newton iterate, read by the Jv until the
  // end), a solve that converges in its first cycle adds d to y_add instead of storing d
  // (*added); otherwise d is left in wk.d.  v0_is_b: V_0 already holds b (the Newton
  // residual kernel wrote it there), used unnormalised in the first cycle.
  int gmres(const double* y, const double* fy, double gamma, double ynorm, double bnorm, int* its,
            double* y_add = nullptr, bool* added = nullptr, bool v0_is_b = false) {
    const long N = wk.N;
    const int m = o.maxl;
    pc = o.precond;
    gamma_cur = gamma;
    const bool with_fallback = pc == 2 || pc == 4;
    if (with_fallback && ilu_ref_its < 0) pc = 1;  // no ILU reference yet: this solve sets it
    if (with_fallback && pc != 1 && wk.learned_skip > 0) {  // back-off after a fallback
      wk.learned_skip--;
      pc = 1;
    }
    if (with_fallback && pc != 1 && network_predicted_to_lose()) {
      st.n_gated++;
      pc = 1;
    }
    const bool pure_ilu = pc == 1;
    if (pc == 1 || pc >= 4) {
      if (int rc = ensure_pset()) return rc;
    }
    int extra_cycles = 0;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), yv(m), hbuf(4 * kMaxVec);
    // The Arnoldi vectors are kept unnormalised: V_l holds W_l and v_l = sig[l] W_l with
    // sig[l] = 1 / ||W_l|| (W_0 = b in a Newton solve's first cycle, else the normalised
    // residual of the restart).  The new vector of step j
    // is J_G z'_j written straight into slot j+1, where z'_j = M(W_j) is the preconditioner
    // applied to the stored W_j; the Arnoldi relation uses z_j = sig[j] z'_j (the FD Jv and
    // ILU(0) are homogeneous, and flexible GMRES takes any z_j), so J_G z_j = sig[j] W_{j+1}
    // before orthogonalisation.  Orthogonalising W_{j+1} against the W_l with coefficients
    // sig[l]^2 (W_{j+1}, W_l) is the same projection; the Hessenberg column gets the factors
    // sig[j] sig[l], and the solution is sum_l y_l sig[l] z'_l.  No pass over the basis
    // normalises it.
    std::vector<double> sig(m + 1, 1.0), sig2(m + 1, 1.0);
    // Second Gram--Schmidt pass when ||w'|| < min(1/sqrt(2), lin_rtol) ||w||: the DGKS test
    // with its threshold bounded by the Krylov tolerance.  A single classical pass that
    // cancelled a factor k = ||w|| / ||w'|| leaves the new vector orthogonal to the basis to
    // ~eps k; with k below 1 / lin_rtol that is at most eps / lin_rtol per step (2e-13 at the
    // default 1e-3, 7e-12 over 30 steps), six orders inside the tolerance the solve is
    // checked against.  The second pass -- nearly a full sweep over the basis in FP64 -- runs
    // only on the steps that cancel more (the plain 1/sqrt(2) threshold reran it on almost
    // every step of a well-preconditioned solve, where J M^-1 v is close to v).
    const double reorth_frac = std::min(0.5, o.lin_rtol * o.lin_rtol);
    double* d_sig2 = wk.sc + 5 * kMaxVec;
    if (added) *added = false;
    bool d_written = false;  // wk.d holds the correction of the cycles so far
    *its = 0;
    if (bnorm == 0.0) {  // d = 0
      if (y_add) *added = true;
      else FOS_CUDA(cudaMemsetAsync(wk.d, 0, sizeof(double) * N, c->stream));
      return 0;
    }
    const double* rvec = wk.b;
    double beta = bnorm;
    for (int cyc = 0; cyc <= o.max_restarts + extra_cycles; cyc++) {
      if (cyc == 0 && v0_is_b) {  // W_0 = b, v_0 = b / beta
        sig[0] = 1.0 / beta;
        sig2[0] = sig[0] * sig[0];
      } else {
        fos_launch(c, k_scale, nb(N), kT, N, rvec, 1.0 / beta, wk.V);
        sig[0] = sig2[0] = 1.0;
      }
      FOS_CUDA(cudaMemcpyAsync(d_sig2, sig2.data(), sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
      bool fallback = false;
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int kend = 0;
      bool conv = false;
      for (int j = 0; j < m; j++) {
        double* vj = wk.V + (size_t)j * N;
        double* zj = wk.Z + (size_t)j * N;
        double* wj = wk.V + (size_t)(j + 1) * N;  // the new vector, orthogonalised in place
        bool have_sq = false;
        const auto t_it = std::chrono::steady_clock::now();
        int rc = psolve(y, vj, zj, c->d_scal, &have_sq);
        if (rc) return rc;
        rc = jv(y, fy, zj, wj, gamma, ynorm, have_sq);
        if (rc) return rc;
        (*its)++;
        const int nv = j + 1;
        // classical Gram--Schmidt, re-orthogonalised only when the first pass cancelled
        // more than the threshold above (Daniel--Gragg--Kaufman--Stewart test)
        // When the previous step needed the second pass, the first update also returns
        // V^T w' (MODE 2) so the second pass needs no separate sweep over V for its
        // coefficients; otherwise it returns ||w'||^2 only (MODE 1).
        const bool fused = last_reorth;
        if ((rc = mdot<true>(nv, wk.V, N, wj))) return rc;              // V^T w, ||w||^2
        if ((rc = reduce(nv + 1, wk.sc))) return rc;
        if (fused) {
          if ((rc = update<2>(nv, wk.V, N, wk.sc, wj, d_sig2))) return rc;  // w -= V s2 h; V^T w, ||w||^2
          if ((rc = reduce(nv + 1, wk.sc + kMaxVec))) return rc;
          if ((rc = fetch(wk.sc, hbuf.data(), 2 * kMaxVec))) return rc;
        } else {
          if ((rc = update<1>(nv, wk.V, N, wk.sc, wj, d_sig2))) return rc;  // w -= V s2 h, ||w||^2
          if ((rc = reduce(1, wk.sc + kMaxVec + nv))) return rc;
          if ((rc = fetch(wk.sc, hbuf.data(), kMaxVec + nv + 1))) return rc;
        }
        double* col = &H[(size_t)(m + 1) * j];
        for (int l = 0; l < nv; l++) col[l] = sig[j] * sig[l] * hbuf[l];
        double hn2 = hbuf[kMaxVec + nv];
        last_reorth = hn2 < reorth_frac * hbuf[nv];
        if (last_reorth) {
          const double* h2 = wk.sc + kMaxVec;  // V^T w' (device), from MODE 2 or a sweep
          if (!fused) {
            if ((rc = mdot<false>(nv, wk.V, N, wj))) return rc;
            if ((rc = reduce(nv, wk.sc + kMaxVec))) return rc;
          }
          if ((rc = update<1>(nv, wk.V, N, h2, wj, d_sig2))) return rc;
          if ((rc = reduce(1, wk.sc + 3 * kMaxVec))) return rc;
          if ((rc = fetch(wk.sc + kMaxVec, hbuf.data() + kMaxVec, 2 * kMaxVec + 1))) return rc;
          for (int l = 0; l < nv; l++) col[l] += sig[j] * sig[l] * hbuf[kMaxVec + l];
          hn2 = hbuf[3 * kMaxVec];
          reorth++;
          st.n_reorth++;
        }
        // the fetch synchronised the stream: the host clock has the iteration's whole cost
        note_iteration_time(std::chrono::duration<double, std::milli>(
                                std::chrono::steady_clock::now() - t_it).count());
        const double wn = std::sqrt(hn2);  // ||W_{j+1}||
        const double hn = sig[j] * wn;
        col[j + 1] = hn;
        if (wn > 0.0) {
          sig[j + 1] = 1.0 / wn;
          sig2[j + 1] = sig[j + 1] * sig[j + 1];
          FOS_CUDA(cudaMemcpyAsync(d_sig2 + j + 1, sig2.data() + j + 1, sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream));
        }
        for (int l = 0; l < j; l++) {
          const double t0 = cs[l] * col[l] + sn[l] * col[l + 1];
          col[l + 1] = -sn[l] * col[l] + cs[l] * col[l + 1];
          col[l] = t0;
        }
        const double den = std::sqrt(col[j] * col[j] + col[j + 1] * col[j + 1]);
        if (den == 0.0) { cs[j] = 1.0; sn[j] = 0.0; }
        else { cs[j] = col[j] / den; sn[j] = col[j + 1] / den; }
        col[j] = cs[j] * col[j] + sn[j] * col[j + 1];
        col[j + 1] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        kend = j + 1;
        if (std::fabs(g[j + 1]) <= o.lin_rtol * bnorm || hn == 0.0) { conv = true; break; }
        // learned modes fall back when they stagnate, reach the ILU(0) iteration count, or
        // fall behind the ILU(0) solve's mean reduction per iteration: the rest of the cycle
        // runs with ILU(0), and flexible GMRES keeps the directions the network gave.  A
        // non-finite estimate (a network output with NaN or Inf) leaves its column out and
        // restarts the cycle with ILU(0) from the current iterate.
        const bool bad = !std::isfinite(g[j + 1]) || !std::isfinite(hn);
        if ((pc == 2 || pc == 4) &&
            (bad || *its >= ilu_ref_its || std::fabs(g[j + 1]) > 0.9 * std::fabs(g[j]) ||
             std::fabs(g[j + 1]) > beta * std::pow(ilu_ref_rate, j + 1))) {
          if (bad) {
            kend = j;
            fallback = true;
            break;
          }
          wk.net_rate = std::pow(std::fabs(g[j + 1]) / beta, 1.0 / (j + 1));
          note_fallback();
          if (int rc = ensure_pset()) return rc;
          extra_cycles++;  // ILU(0) keeps its full restart budget
        }
      }
      for (int l = kend - 1; l >= 0; l--) {
        double s = g[l];
        for (int q = l + 1; q < kend; q++) s -= H[l + (size_t)(m + 1) * q] * yv[q];
        yv[l] = s / H[l + (size_t)(m + 1) * l];
      }
      for (int l = 0; l < kend; l++) yv[l] *= sig[l];  // z_l = sig[l] z'_l
      FOS_CUDA(cudaMemcpyAsync(wk.sc + 4 * kMaxVec, yv.data(), sizeof(double) * kend,
                               cudaMemcpyHostToDevice, c->stream));
      double* yadd = (conv && !d_written && y_add) ? y_add : nullptr;
      {
        const double* cz = wk.sc + 4 * kMaxVec;
        const double* Zc = wk.Z;
        if (yadd)  // (only while d holds nothing yet)
          fos_launch(c, k_comb<false, true>, nb(N), kT, N, kend, Zc, N, cz, wk.d, yadd);
        else if (d_written)
          fos_launch(c, k_comb<true, false>, nb(N), kT, N, kend, Zc, N, cz, wk.d, yadd);
        else
          fos_launch(c, k_comb<false, false>, nb(N), kT, N, kend, Zc, N, cz, wk.d, yadd);
      }
      FOS_LAUNCH_CHECK();
      if (yadd) *added = true;
      else d_written = true;
      if (conv) {
        if (pure_ilu) set_ilu_ref(*its, std::fabs(g[kend]), bnorm);
        if (with_fallback && pc != 1) {  // the network won this solve
          wk.learned_backoff = 0;
          wk.net_rate = *its > 0 ? std::pow(std::fabs(g[kend]) / bnorm, 1.0 / *its) : 0.0;
        }
        return 0;
      }
      if (fallback) {  // continue with ILU(0) from the current iterate
        note_fallback();
        if (int rc = ensure_pset()) return rc;
        extra_cycles++;
      } else if (cyc == o.max_restarts + extra_cycles) {
        return 1;
      }
      // restart from the true residual r = b - J_G d
      int rc = jv(y, fy, wk.d, wk.w, gamma, ynorm);
      if (rc) return rc;
      fos_launch(c, k_scale, nb(N), kT, N, wk.w, -1.0, wk.w);
      fos_launch(c, k_axpy, nb(N), kT, N, 1.0, wk.b, wk.w);
      if ((rc = fos_norm2_dev(c, wk.w, N, c->d_scal + 8))) return rc;
      if ((rc = fetch(c->d_scal + 8, hbuf.data(), 1))) return rc;
      beta = std::sqrt(hbuf[0]);
      if (beta <= o.lin_rtol * bnorm) {
        if (pure_ilu) set_ilu_ref(*its, beta, bnorm);
        return 0;
      }
      rvec = wk.w;
      // V_0 = w / beta (k_scale reads w before the Arnoldi loop overwrites it)
    }
    return 1;
  }
};

}  // namespace

extern "C" int fos_bdf_run(fos_ctx* c, double t0, double* y, const fos_bdf_opts* opts,
                           fos_bdf_stats* stats) {
  if (!c || !y || !opts || opts->maxl < 1 || opts->maxl > kMaxVec - 1 || opts->nsteps < 0 ||
      (opts->order != 1 && opts->order != 2) || !(opts->dt > 0.0) || opts->precond < 0 ||
      opts->precond > 5) {
    fos_set_error("fos_bdf_run: bad arguments (maxl must be in [1, 31], precond in [0, 5])");
    return -1;
  }
  fos_bdf_stats dummy;
  fos_bdf_stats& st = stats ? *stats : dummy;
  std::memset(&st, 0, sizeof(st));
  Work* wkp = nullptr;
  if (int rc = work_get(c, opts->maxl, &wkp)) return rc;
  Work& wk = *wkp;
  const long N = wk.N;
  // resume: continue the BDF history of the previous call when y is its result
  const bool resume = opts->resume && wk.has_hist;
  const double eps = opts->jv_eps > 0.0 ? opts->jv_eps : jv_eps_default(c);
  Driver dr{c, wk, *opts, st, eps};
  dr.ilu_ref_its = wk.ilu_ref_its;
  dr.ilu_ref_rate = wk.ilu_ref_rate;
  double t = t0;
  FOS_CUDA(cudaMemcpyAsync(wk.yn, y, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  if (!resume) {
    wk.has_hist = false;
    wk.nhist = 1;
  }
  // Newton's first iterate in y: y_n (which y holds at the start of every step: yn was
  // copied from y before the first step and from the accepted y after every step), or the
  // extrapolation of order p through the history
  auto pred_order = [&](int q) { return opts->predictor ? std::min(q, wk.nhist - 1) : 0; };
  auto predict = [&](int p) -> int {
    if (p == 1) fos_launch(c, k_predict<1>, nb(N), kT, N, wk.yn, wk.ym, wk.ym2, y);
    else if (p == 2) fos_launch(c, k_predict<2>, nb(N), kT, N, wk.yn, wk.ym, wk.ym2, y);
    else FOS_CUDA(cudaMemcpyAsync(y, wk.yn, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    FOS_LAUNCH_CHECK();
    return 0;
  };
  int status = 0;
  // preconditioner set-up policy (opts->msbp > 1: CVODE's cvLsSetup conditions); a resumed
  // call continues the previous call's count, as CVODE keeps its set-up across CVode calls
  bool have_setup = false;
  int last_setup = 0;
  double gamma_setup = 0.0;
  if (resume && wk.setup_age >= 0 && c->has_factor && wk.setup_serial == c->n_setup) {
    have_setup = true;
    last_setup = -wk.setup_age;
    gamma_setup = wk.gamma_setup;
  }
  int steps_done = 0;
  for (int s = 0; s < opts->nsteps && !status; s++) {
    const int q = (opts->order == 2 && (s >= 1 || resume)) ? 2 : 1;
    const double gamma = q == 1 ? opts->dt : 2.0 * opts->dt / 3.0;
    const double tn = t + opts->dt;
    fos_launch(c, k_hist, nb(N), kT, N, q, wk.yn, wk.ym, wk.hist);
    const int p = pred_order(q);
    if (p > 0)
      if (int rc = predict(p)) return rc;
    const bool reuse = opts->msbp > 1 && have_setup && c->has_factor &&
                       s - last_setup < opts->msbp &&
                       std::fabs(gamma / gamma_setup - 1.0) <= 0.3;
    dr.keep_setup = reuse;
    dr.setup_made = false;
    int nrc = dr.newton(y, gamma, wk.hist, tn);  // from the predicted y_0
    if (nrc == 1 && reuse) {  // failed on a reused set-up: retry the step with a fresh one
      if (int rc = predict(p)) return rc;
      dr.keep_setup = false;
      nrc = dr.newton(y, gamma, wk.hist, tn);
    }
    if ((nrc == 1 || nrc == 2) && p > 0) {  // the extrapolation failed (at a shock it can
                                            // leave the physical states): retry from y_n
      if (int rc = predict(0)) return rc;
      dr.keep_setup = false;
      nrc = dr.newton(y, gamma, wk.hist, tn);
    }
    if (dr.setup_made) {
      have_setup = true;
      last_setup = s;
      gamma_setup = gamma;
    }
    if (nrc < 0) return nrc;
    const bool conv = nrc == 0;
    if (nrc >= 2) status = nrc;
    if (!conv) {  // the failed step is not taken: y goes back to the last accepted state
      st.fails++;
      if (!status) status = 1;
      FOS_CUDA(cudaMemcpyAsync(y, wk.yn, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
      break;
    }
    std::swap(wk.ym2, wk.ym);  // y_{n-2} <- y_{n-1} <- y_n <- y
    std::swap(wk.ym, wk.yn);
    FOS_CUDA(cudaMemcpyAsync(wk.yn, y, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    t = tn;
    st.n_steps++;
    steps_done = s + 1;
    wk.has_hist = true;
    wk.nhist = std::min(wk.nhist + 1, 3);
  }
  if (status) {
    wk.has_hist = false;
    wk.nhist = 1;
  }
  wk.setup_age = (have_setup && !status) ? steps_done - last_setup : -1;
  wk.gamma_setup = gamma_setup;
  wk.setup_serial = c->n_setup;
  wk.ilu_ref_its = dr.ilu_ref_its;
  wk.ilu_ref_rate = dr.ilu_ref_rate;
  st.t = t;
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  return status;
}

extern "C" int fos_bdf_run_host(fos_ctx* c, double t0, double* y, const fos_bdf_opts* opts,
                                fos_bdf_stats* stats) {
  if (!c || !y || !opts) {
    fos_set_error("fos_bdf_run_host: bad arguments");
    return -1;
  }
  Work* wk = nullptr;
  if (int rc = work_get(c, opts->maxl, &wk)) return rc;
  if (int rc = fos_h2d_internal(c, y, wk->yh)) return rc;
  int rc = fos_bdf_run(c, t0, wk->yh, opts, stats);
  if (rc < 0) return rc;
  if (int rc2 = fos_d2h_reference(c, wk->yh, y)) return rc2;
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  return rc;
}

// ------------------------------------------------------------------ adaptive BDF
namespace {

// Lagrange basis at x on nodes t[0..m-1]: w[j] = prod_{k != j} (x - t_k) / (t_j - t_k)
void lagrange_at(const double* t, int m, double x, double* w) {
  for (int j = 0; j < m; j++) {
    double v = 1.0;
    for (int k = 0; k < m; k++)
      if (k != j) v *= (x - t[k]) / (t[j] - t[k]);
    w[j] = v;
  }
}
// derivatives of the Lagrange basis at the first node t[0]
void lagrange_deriv_at_first(const double* t, int m, double* d) {
  double d0 = 0.0;
  for (int k = 1; k < m; k++) d0 += 1.0 / (t[0] - t[k]);
  d[0] = d0;
  for (int j = 1; j < m; j++) {
    double v = 1.0 / (t[j] - t[0]);
    for (int k = 1; k < m; k++)
      if (k != j) v *= (t[0] - t[k]) / (t[j] - t[k]);
    d[j] = v;
  }
}
// CVODE's step factor from an error estimate at order k with bias b
double eta_of(double err, int k, double bias) {
  return 1.0 / (std::pow(bias * err, 1.0 / (k + 1)) + 1e-6);
}

int adapt_alloc(Work& wk, int qmax) {
  const long N = wk.N;
  for (int k = 0; k <= qmax; k++)
    if (!wk.ay[k]) FOS_CUDA(cudaMalloc(&wk.ay[k], sizeof(double) * N));
  for (double** p : {&wk.ypred, &wk.E, &wk.Eprev, &wk.atmp})
    if (!*p) FOS_CUDA(cudaMalloc(p, sizeof(double) * N));
  return 0;
}

struct Adapt {
  fos_ctx* c;
  Work& wk;
  Driver& dr;
  long N;
  int comb(double* out, int nv, const double* const* p, const double* coef) {
    Comb8 cb;
    cb.nv = nv;
    for (int l = 0; l < nv; l++) { cb.p[l] = p[l]; cb.c[l] = coef[l]; }
    fos_launch(c, k_lincomb, nb(N), kT, N, cb, out);
    FOS_LAUNCH_CHECK();
    return 0;
  }
  // ||a||_WRMS with weights from w
  int wrms(const double* a, const double* w, double rtol, double atol, double* out) {
    fos_launch(c, k_wrms_part, kRedBlocks, kT, N, a, w, rtol, atol, wk.part);
    if (int rc = dr.reduce(1, wk.sc + 5 * kMaxVec)) return rc;
    double h = 0.0;
    if (int rc = dr.fetch(wk.sc + 5 * kMaxVec, &h, 1)) return rc;
    *out = std::sqrt(h / (double)N);
    return 0;
  }
};

}  // namespace

extern "C" void fos_bdf_adapt_defaults(fos_bdf_adapt_opts* o) {
  o->rtol = 1e-6;
  o->atol = 1e-12;
  o->h0 = 1e-4;
  o->hmin = 0.0;
  o->hmax = 0.0;
  o->qmax = 5;
  o->max_steps = 0;
}

// Variable-order, variable-step BDF from t0 to tout (see fosgpu.h).  History: the last
// qmax + 1 accepted solutions Y[0] (newest) .. at times T[0] ..; a step of order q from
// t = T[0] with size h:
//   predictor   y_pred = sum_j L_j(t + h) Y[j], Lagrange on T[0..q] (the first step:
//               y_0 + h f(y_0)), error factor h / (t + h - T[q]) (first step 1/2);
//   corrector   Newton on y - gamma f(y) - hist = 0 with l_j the Lagrange derivatives at
//               t + h on the nodes (t + h, T[0..q-1]): gamma = 1 / l_0,
//               hist = -gamma sum_{j >= 1} l_j Y[j-1];
//   error test  err = factor ||y - y_pred||_WRMS <= 1.
extern "C" int fos_bdf_adaptive(fos_ctx* c, double t0, double tout, double* y,
                                const fos_bdf_opts* nk, const fos_bdf_adapt_opts* ad,
                                fos_bdf_stats* nk_stats, fos_bdf_adapt_stats* ad_stats) {
  if (!c || !y || !nk || !ad || nk->maxl < 1 || nk->maxl > kMaxVec - 1 || nk->precond < 0 ||
      nk->precond > 5 || ad->qmax < 1 || ad->qmax > 5 || !(ad->h0 > 0.0) || !(tout > t0) ||
      !(ad->rtol >= 0.0) || !(ad->atol > 0.0)) {
    fos_set_error("fos_bdf_adaptive: bad arguments (qmax in [1, 5], h0 > 0, tout > t0, atol > 0)");
    return -1;
  }
  fos_bdf_stats dummy;
  fos_bdf_stats& st = nk_stats ? *nk_stats : dummy;
  std::memset(&st, 0, sizeof(st));
  fos_bdf_adapt_stats adummy;
  fos_bdf_adapt_stats& as = ad_stats ? *ad_stats : adummy;
  std::memset(&as, 0, sizeof(as));
  Work* wkp = nullptr;
  if (int rc = work_get(c, nk->maxl, &wkp)) return rc;
  Work& wk = *wkp;
  if (int rc = adapt_alloc(wk, ad->qmax)) return rc;
  const long N = wk.N;
  const int qmax = ad->qmax;
  const long max_steps = ad->max_steps > 0 ? ad->max_steps : 100000;
  const double eps = nk->jv_eps > 0.0 ? nk->jv_eps : jv_eps_default(c);
  Driver dr{c, wk, *nk, st, eps};
  dr.ilu_ref_its = wk.ilu_ref_its;
  dr.ilu_ref_rate = wk.ilu_ref_rate;
  Adapt A{c, wk, dr, N};
  double* Y[6];
  double T[6];
  for (int k = 0; k <= qmax; k++) Y[k] = wk.ay[k];
  FOS_CUDA(cudaMemcpyAsync(Y[0], y, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  T[0] = t0;
  int nh = 1;  // solutions in the history
  // f(t0, y0) for the first predictor
  if (int rc = fos_residual_launch(c, Y[0], nullptr, nullptr, nullptr, wk.atmp, 0.0, 0.0, 0)) return rc;
  st.n_rhs++;
  double t = t0;
  double h = ad->h0;
  if (ad->hmax > 0.0) h = std::min(h, ad->hmax);
  int q = 1, nq = 0, nef = 0, ncf = 0;
  double h_prev = 0.0;
  bool have_eprev = false;
  long attempts = 0;
  int status = 0;
  // preconditioner set-up policy (nk->msbp > 1: CVODE's; steps counted as accepted steps)
  long last_setup = -1;
  double gamma_setup = 0.0;
  while (t < tout) {
    if (++attempts > max_steps) { status = 5; break; }
    if (t + h >= tout) h = tout - t;
    const double tn = t + h;
    // predictor
    double errfac;
    if (nh == 1) {
      const double* p[2] = {Y[0], wk.atmp};
      const double cf[2] = {1.0, h};
      if (int rc = A.comb(wk.ypred, 2, p, cf)) return rc;
      errfac = 0.5;
    } else {
      double w[6];
      lagrange_at(T, q + 1, tn, w);
      if (int rc = A.comb(wk.ypred, q + 1, Y, w)) return rc;
      errfac = h / (tn - T[q]);
    }
    FOS_CUDA(cudaMemcpyAsync(y, wk.ypred, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    // corrector coefficients
    double tau[6], dl[6];
    tau[0] = tn;
    for (int j = 0; j < q; j++) tau[j + 1] = T[j];
    lagrange_deriv_at_first(tau, q + 1, dl);
    const double gamma = 1.0 / dl[0];
    {
      double cf[5];
      for (int j = 1; j <= q; j++) cf[j - 1] = -gamma * dl[j];
      if (int rc = A.comb(wk.hist, q, Y, cf)) return rc;
    }
    const bool reuse = nk->msbp > 1 && last_setup >= 0 && c->has_factor &&
                       as.n_accepted - last_setup < nk->msbp &&
                       std::fabs(gamma / gamma_setup - 1.0) <= 0.3;
    dr.keep_setup = reuse;
    dr.setup_made = false;
    int nrc = dr.newton(y, gamma, wk.hist, tn);
    if (nrc > 0 && reuse) {  // failed on a reused set-up: the same step with a fresh one
      FOS_CUDA(cudaMemcpyAsync(y, wk.ypred, sizeof(double) * N, cudaMemcpyDeviceToDevice,
                               c->stream));
      dr.keep_setup = false;
      nrc = dr.newton(y, gamma, wk.hist, tn);
    }
    if (dr.setup_made) {
      last_setup = as.n_accepted;
      gamma_setup = gamma;
    }
    if (nrc < 0) return nrc;
    if (nrc != 0) {  // Newton failure (no convergence, non-finite residual, zero pivot)
      as.n_newton_fails++;
      if (++ncf > 10 || 0.25 * h < ad->hmin) { status = 4; break; }
      h *= 0.25;
      continue;
    }
    // local error estimate
    {
      const double* p[2] = {y, wk.ypred};
      const double cf[2] = {1.0, -1.0};
      if (int rc = A.comb(wk.E, 2, p, cf)) return rc;
    }
    double en = 0.0;
    if (int rc = A.wrms(wk.E, Y[0], ad->rtol, ad->atol, &en)) return rc;
    const double err = errfac * en;
    if (err > 1.0) {  // error-test failure: retry with a smaller step
      as.n_err_fails++;
      if (++nef > 7) { status = 4; break; }
      double eta;
      if (nef >= 3) {
        eta = 0.1;
        if (q > 1) { q = 1; nq = 0; have_eprev = false; }
      } else {
        eta = std::max(0.2, std::min(0.9, eta_of(err, q, 6.0)));
      }
      h *= eta;
      if (h < ad->hmin) { status = 4; break; }
      continue;
    }
    // accepted: step factor for this order, and for orders q -/+ 1 after q + 1 steps
    nef = ncf = 0;
    nq++;
    double eta = eta_of(err, q, 6.0);
    int qnew = q;
    if (nq >= q + 1) {
      if (q > 1) {  // order q - 1: its predictor on T[0..q-1]
        double w[6];
        lagrange_at(T, q, tn, w);
        if (int rc = A.comb(wk.atmp, q, Y, w)) return rc;
        const double* p[2] = {y, wk.atmp};
        const double cf[2] = {1.0, -1.0};
        if (int rc = A.comb(wk.atmp, 2, p, cf)) return rc;
        double e1 = 0.0;
        if (int rc = A.wrms(wk.atmp, Y[0], ad->rtol, ad->atol, &e1)) return rc;
        const double eta_dn = eta_of(h / (tn - T[q - 1]) * e1, q - 1, 6.0);
        if (eta_dn > eta) { eta = eta_dn; qnew = q - 1; }
      }
      if (q < qmax && have_eprev) {  // order q + 1: the change of the error vectors
        const double r = h / h_prev;
        const double* p[2] = {wk.E, wk.Eprev};
        const double cf[2] = {1.0, -std::pow(r, q + 1)};
        if (int rc = A.comb(wk.atmp, 2, p, cf)) return rc;
        double e2 = 0.0;
        if (int rc = A.wrms(wk.atmp, Y[0], ad->rtol, ad->atol, &e2)) return rc;
        const double eta_up = eta_of(e2 / (q + 2), q + 1, 10.0);
        if (eta_up > eta) { eta = eta_up; qnew = q + 1; }
      }
    }
    // history: the new solution becomes Y[0]
    double* last = Y[qmax];
    for (int k = qmax; k > 0; k--) { Y[k] = Y[k - 1]; T[k] = T[k - 1]; }
    Y[0] = last;
    T[0] = tn;
    FOS_CUDA(cudaMemcpyAsync(Y[0], y, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    nh = std::min(nh + 1, qmax + 1);
    std::swap(wk.E, wk.Eprev);
    have_eprev = true;
    h_prev = h;
    as.n_accepted++;
    as.steps_at_order[q]++;
    as.q_last = q;
    as.h_last = h;
    st.n_steps++;
    t = tn;
    if (qnew != q) { q = qnew; nq = 0; have_eprev = false; }
    if (q > nh - 1) q = nh - 1;
    if (eta < 1.5) eta = 1.0;
    h *= std::min(eta, 10.0);
    if (ad->hmax > 0.0) h = std::min(h, ad->hmax);
  }
  FOS_CUDA(cudaMemcpyAsync(y, Y[0], sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  wk.ilu_ref_its = dr.ilu_ref_its;
  wk.ilu_ref_rate = dr.ilu_ref_rate;
  wk.has_hist = false;  // the fixed-step history does not continue an adaptive run
  wk.nhist = 1;
  as.t = t;
  st.t = t;
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  return status;
}

// One linear solve J_G x = b at state y (f(y) = fy) with the driver's (F)GMRES and the
// preconditioner of opts->precond; the ILU(0) factorisation is made for (y, gamma) when
// needed.  Used to generate training pairs and to compare preconditioners.
extern "C" int fos_linear_solve_dev(fos_ctx* c, double t, const double* y, const double* fy,
                                    double gamma, const double* b, double* x,
                                    const fos_bdf_opts* opts, fos_bdf_stats* stats) {
  if (!c || !y || !fy || !b || !x || !opts || opts->maxl < 1 || opts->maxl > kMaxVec - 1 ||
      opts->precond < 0 || opts->precond > 5) {
    fos_set_error("fos_linear_solve_dev: bad arguments");
    return -1;
  }
  fos_bdf_stats dummy;
  fos_bdf_stats& st = stats ? *stats : dummy;
  std::memset(&st, 0, sizeof(st));
  Work* wkp = nullptr;
  if (int rc = work_get(c, opts->maxl, &wkp)) return rc;
  Work& wk = *wkp;
  const long N = wk.N;
  const double eps = opts->jv_eps > 0.0 ? opts->jv_eps : jv_eps_default(c);
  Driver dr{c, wk, *opts, st, eps};
  dr.ilu_ref_its = wk.ilu_ref_its;
  dr.ilu_ref_rate = wk.ilu_ref_rate;
  dr.t_step = t;
  dr.gamma_step = gamma;
  dr.y_step = y;
  FOS_CUDA(cudaMemcpyAsync(wk.b, b, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  if (int rc = fos_norm2_dev(c, y, N, c->d_scal + 24)) return rc;
  if (int rc = fos_norm2_dev(c, b, N, c->d_scal + 25)) return rc;
  double h2[2];
  FOS_CUDA(cudaMemcpyAsync(h2, c->d_scal + 24, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  int its = 0;
  int rc = dr.gmres(y, fy, gamma, std::sqrt(h2[0]), std::sqrt(h2[1]), &its);
  st.n_lin_iters = its;
  wk.ilu_ref_its = dr.ilu_ref_its;
  wk.ilu_ref_rate = dr.ilu_ref_rate;
  if (rc < 0) return rc;
  FOS_CUDA(cudaMemcpyAsync(x, wk.d, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  return rc;
}
