// fos_residual.cu -- the first-order Roe residual and the fused finite-difference
// Jacobian-vector product on sm_103a.
//
// Reference arithmetic: setBC (foeuler.f90:209-330), syncState (:186-206),
// findEulerPoly (Euler.f90:25-156), rhs divide-by-volume (foeuler.f90:366-372).
// Three kernels per evaluation, no floating-point atomics:
//   k_prim    per cell   primitives W = (rho,u,v,w,H,p,sqrt(rho)) from the SoA state
//                         (optionally y + s*v, the Jv perturbation, in FP64)
//   k_face    per face   Roe flux-difference-splitting flow, boundary ghosts computed
//                         in-register from the interior conserved state (setBC)
//   k_gather  per cell   deterministic CSR gather of -flow (cell is L) / +flow (cell
//                         is R) in ascending face order, times 1/v; Jv epilogue
//                         out = a v + b (f(y+sv) - fy)/s in FP64
// The FP32-flux variant (FOS_FLUX_FP32) computes the same flow in FP32 in the
// flux-difference form (the L/R central fluxes enter as F_R - F_L; the cell's own
// flux sums to zero over a closed cell) and accumulates it in FP64.
#include <cmath>

#include "fos_internal.h"
#include "fos_device.cuh"

namespace {

constexpr int kThreads = 256;

struct P64 {
  double rho, u, v, w, H, p, s;
};

__device__ __forceinline__ void load_prim(const double* __restrict__ W, int c, P64& P) {
  const double2* w2 = reinterpret_cast<const double2*>(W + 8 * (size_t)c);
  double2 a = __ldg(w2), b = __ldg(w2 + 1), d = __ldg(w2 + 2), e = __ldg(w2 + 3);
  P.rho = a.x; P.u = a.y; P.v = b.x; P.w = b.y; P.H = d.x; P.p = d.y; P.s = e.x;
}

__device__ __forceinline__ void prim_from_cons(double rho, double mx, double my, double mz,
                                               double E, double gm1, P64& P) {
  double inv = 1.0 / rho;
  P.rho = rho;
  P.u = mx * inv; P.v = my * inv; P.w = mz * inv;
  P.p = gm1 * (E - 0.5 * (mx * mx + my * my + mz * mz) * inv);
  P.H = (E + P.p) * inv;
  P.s = sqrt(rho);
}

// Roe flux-difference splitting flow through one face (Euler.f90:90-126), FP64,
// central part as the reference writes it: aP*(1/2 (F_L + F_R).n - 1/2 sum of waves)
__device__ __forceinline__ void roe_flow64(const P64& L, const P64& R, double nx, double ny,
                                           double nz, double aP, double gm1, double flow[5]) {
  const double inv = 1.0 / (L.s + R.s);
  const double ua = (L.s * L.u + R.s * R.u) * inv;
  const double va = (L.s * L.v + R.s * R.v) * inv;
  const double wa = (L.s * L.w + R.s * R.w) * inv;
  const double Ha = (L.s * L.H + R.s * R.H) * inv;
  const double rhoA = L.s * R.s;
  const double q2 = ua * ua + va * va + wa * wa;
  const double c2 = gm1 * (Ha - 0.5 * q2);
  const double ca = sqrt(c2);
  const double ic2 = 1.0 / c2;
  const double unA = ua * nx + va * ny + wa * nz;
  const double rJ = R.rho - L.rho, pJ = R.p - L.p;
  const double uJ = R.u - L.u, vJ = R.v - L.v, wJ = R.w - L.w;
  const double unJ = uJ * nx + vJ * ny + wJ * nz;
  // entropy + shear waves
  const double au = fabs(unA);
  const double wE = rJ - pJ * ic2;
  double d0 = au * wE;
  double d1 = au * (wE * ua + rhoA * (uJ - nx * unJ));
  double d2 = au * (wE * va + rhoA * (vJ - ny * unJ));
  double d3 = au * (wE * wa + rhoA * (wJ - nz * unJ));
  double d4 = au * (wE * (0.5 * q2) + rhoA * (ua * uJ + va * vJ + wa * wJ - unA * unJ));
  // acoustic waves
  const double s1 = fabs(unA - ca) * (0.5 * (pJ - rhoA * ca * unJ) * ic2);
  d0 += s1;
  d1 += s1 * (ua - nx * ca);
  d2 += s1 * (va - ny * ca);
  d3 += s1 * (wa - nz * ca);
  d4 += s1 * (Ha - unA * ca);
  const double s2 = fabs(unA + ca) * (0.5 * (pJ + rhoA * ca * unJ) * ic2);
  d0 += s2;
  d1 += s2 * (ua + nx * ca);
  d2 += s2 * (va + ny * ca);
  d3 += s2 * (wa + nz * ca);
  d4 += s2 * (Ha + unA * ca);
  const double unL = L.u * nx + L.v * ny + L.w * nz;
  const double unR = R.u * nx + R.v * ny + R.w * nz;
  const double mL = L.rho * unL, mR = R.rho * unR;
  flow[0] = aP * (0.5 * (mL + mR) - 0.5 * d0);
  flow[1] = aP * (0.5 * (mL * L.u + L.p * nx + mR * R.u + R.p * nx) - 0.5 * d1);
  flow[2] = aP * (0.5 * (mL * L.v + L.p * ny + mR * R.v + R.p * ny) - 0.5 * d2);
  flow[3] = aP * (0.5 * (mL * L.w + L.p * nz + mR * R.w + R.p * nz) - 0.5 * d3);
  flow[4] = aP * (0.5 * (mL * L.H + mR * R.H) - 0.5 * d4);
}

__global__ void __launch_bounds__(kThreads) k_prim64(int nC, const double* __restrict__ y,
                                                     const double* __restrict__ v,
                                                     const double* __restrict__ d_s, double gm1,
                                                     double* __restrict__ W) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  double U[5];
#pragma unroll
  for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + c];
  if (v) {
    const double s = *d_s;
#pragma unroll
    for (int q = 0; q < 5; q++) U[q] = U[q] + s * v[(size_t)q * nC + c];
  }
  P64 P;
  prim_from_cons(U[0], U[1], U[2], U[3], U[4], gm1, P);
  double2* w2 = reinterpret_cast<double2*>(W + 8 * (size_t)c);
  w2[0] = make_double2(P.rho, P.u);
  w2[1] = make_double2(P.v, P.w);
  w2[2] = make_double2(P.H, P.p);
  w2[3] = make_double2(P.s, 0.0);
}

__global__ void __launch_bounds__(kThreads) k_face64(
    int nFi, int nF, int nC, const int2* __restrict__ faceLR, const double2* __restrict__ faceNA,
    const double* __restrict__ W, const double* __restrict__ y, const double* __restrict__ v,
    const double* __restrict__ d_s, const int* __restrict__ bcT, const double* __restrict__ bcP,
    int maxP, double g, double r, double* __restrict__ F) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nF) return;
  const int2 lr = __ldg(faceLR + f);
  const double2 n01 = __ldg(faceNA + 2 * (size_t)f), n2a = __ldg(faceNA + 2 * (size_t)f + 1);
  const double nx = n01.x, ny = n01.y, nz = n2a.x, aP = n2a.y;
  P64 L, R;
  load_prim(W, lr.x, L);
  if (f < nFi) {
    load_prim(W, lr.y, R);
  } else {
    double U[5], G[5];
#pragma unroll
    for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + lr.x];
    if (v) {
      const double s = *d_s;
#pragma unroll
      for (int q = 0; q < 5; q++) U[q] = U[q] + s * v[(size_t)q * nC + lr.x];
    }
    const int row = lr.y;
    const int type = row > 0 ? bcT[row - 1] : FOS_BC_WALL;
    ghost_state(type, row > 0 ? bcP + (size_t)maxP * (row - 1) : nullptr, U, nx, ny, nz, g, r, G);
    prim_from_cons(G[0], G[1], G[2], G[3], G[4], g - 1.0, R);
  }
  double flow[5];
  roe_flow64(L, R, nx, ny, nz, aP, g - 1.0, flow);
#pragma unroll
  for (int q = 0; q < 5; q++) F[(size_t)q * nF + f] = flow[q];
}

// mode 0: out = sum/v ; mode 1: out = a*v + b*(sum/v - fy)/s
__global__ void __launch_bounds__(kThreads) k_gather(
    int nC, int nF, const int* __restrict__ crow, const int* __restrict__ cent,
    const double* __restrict__ F, const double* __restrict__ invV, int mode,
    const double* __restrict__ vv, const double* __restrict__ fy, const double* __restrict__ d_s,
    double a, double b, double* __restrict__ out, int* __restrict__ flag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const int e0 = __ldg(crow + c), e1 = __ldg(crow + c + 1);
  for (int e = e0; e < e1; e++) {
    const int ent = __ldg(cent + e);
    const int f = ent >> 1;
    const bool plus = ent & 1;
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const double x = __ldg(F + (size_t)q * nF + f);
      acc[q] = plus ? acc[q] + x : acc[q] - x;
    }
  }
  const double iv = __ldg(invV + c);
  bool bad = false;
  if (mode == 0) {
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const double o = acc[q] * iv;
      bad |= !isfinite(o);
      out[(size_t)q * nC + c] = o;
    }
  } else {
    const double s = *d_s;
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const size_t k = (size_t)q * nC + c;
      double o = a * vv[k];
      if (s > 0.0) o += b * ((acc[q] * iv - fy[k]) / s);
      bad |= !isfinite(o);
      out[k] = o;
    }
  }
  if (bad && flag) atomicOr(flag, 1);
}

// ------------------------------------------------------------------ FP32 flux
struct P32 {
  float rho, u, v, w, H, p, s;
};
__device__ __forceinline__ void load_prim32(const float* __restrict__ W, int c, P32& P) {
  const float4* w4 = reinterpret_cast<const float4*>(W + 8 * (size_t)c);
  float4 a = __ldg(w4), b = __ldg(w4 + 1);
  P.rho = a.x; P.u = a.y; P.v = a.z; P.w = a.w; P.H = b.x; P.p = b.y; P.s = b.z;
}

// Same Roe flow in FP32, flux-difference form: the cell's own flux F_L.n sums to zero
// over the closed cell, so L receives -aP(1/2 (F_R - F_L).n - 1/2 waves) and R receives
// -aP(1/2 (F_R - F_L).n + 1/2 waves); stored as (dF, waves) pairs per face.
__device__ __forceinline__ void roe_split32(const P32& L, const P32& R, float nx, float ny,
                                            float nz, float aP, float gm1, float dF[5],
                                            float dw[5]) {
  const float inv = 1.0f / (L.s + R.s);
  const float ua = (L.s * L.u + R.s * R.u) * inv;
  const float va = (L.s * L.v + R.s * R.v) * inv;
  const float wa = (L.s * L.w + R.s * R.w) * inv;
  const float Ha = (L.s * L.H + R.s * R.H) * inv;
  const float rhoA = L.s * R.s;
  const float q2 = ua * ua + va * va + wa * wa;
  const float c2 = gm1 * (Ha - 0.5f * q2);
  const float ca = sqrtf(c2);
  const float ic2 = 1.0f / c2;
  const float unA = ua * nx + va * ny + wa * nz;
  const float rJ = R.rho - L.rho, pJ = R.p - L.p;
  const float uJ = R.u - L.u, vJ = R.v - L.v, wJ = R.w - L.w;
  const float unJ = uJ * nx + vJ * ny + wJ * nz;
  const float au = fabsf(unA);
  const float wE = rJ - pJ * ic2;
  float d0 = au * wE;
  float d1 = au * (wE * ua + rhoA * (uJ - nx * unJ));
  float d2 = au * (wE * va + rhoA * (vJ - ny * unJ));
  float d3 = au * (wE * wa + rhoA * (wJ - nz * unJ));
  float d4 = au * (wE * (0.5f * q2) + rhoA * (ua * uJ + va * vJ + wa * wJ - unA * unJ));
  const float s1 = fabsf(unA - ca) * (0.5f * (pJ - rhoA * ca * unJ) * ic2);
  d0 += s1; d1 += s1 * (ua - nx * ca); d2 += s1 * (va - ny * ca); d3 += s1 * (wa - nz * ca);
  d4 += s1 * (Ha - unA * ca);
  const float s2 = fabsf(unA + ca) * (0.5f * (pJ + rhoA * ca * unJ) * ic2);
  d0 += s2; d1 += s2 * (ua + nx * ca); d2 += s2 * (va + ny * ca); d3 += s2 * (wa + nz * ca);
  d4 += s2 * (Ha + unA * ca);
  // F_R.n - F_L.n for the five components
  const float unL = L.u * nx + L.v * ny + L.w * nz;
  const float unR = R.u * nx + R.v * ny + R.w * nz;
  const float mL = L.rho * unL, mR = R.rho * unR;
  dF[0] = 0.5f * aP * (mR - mL);
  dF[1] = 0.5f * aP * (mR * R.u - mL * L.u + pJ * nx);
  dF[2] = 0.5f * aP * (mR * R.v - mL * L.v + pJ * ny);
  dF[3] = 0.5f * aP * (mR * R.w - mL * L.w + pJ * nz);
  dF[4] = 0.5f * aP * (mR * R.H - mL * L.H);
  dw[0] = 0.5f * aP * d0; dw[1] = 0.5f * aP * d1; dw[2] = 0.5f * aP * d2;
  dw[3] = 0.5f * aP * d3; dw[4] = 0.5f * aP * d4;
}

__global__ void __launch_bounds__(kThreads) k_prim32(int nC, const double* __restrict__ y,
                                                     const double* __restrict__ v,
                                                     const double* __restrict__ d_s, double gm1,
                                                     float* __restrict__ W) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  double U[5];
#pragma unroll
  for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + c];
  if (v) {
    const double s = *d_s;
#pragma unroll
    for (int q = 0; q < 5; q++) U[q] = U[q] + s * v[(size_t)q * nC + c];
  }
  // primitives in FP32 from the FP64 perturbed state
  const float rho = (float)U[0];
  const float inv = 1.0f / rho;
  const float mx = (float)U[1], my = (float)U[2], mz = (float)U[3], E = (float)U[4];
  const float p = (float)gm1 * (E - 0.5f * (mx * mx + my * my + mz * mz) * inv);
  float4* w4 = reinterpret_cast<float4*>(W + 8 * (size_t)c);
  w4[0] = make_float4(rho, mx * inv, my * inv, mz * inv);
  w4[1] = make_float4((E + p) * inv, p, sqrtf(rho), 0.0f);
}

__global__ void __launch_bounds__(kThreads) k_face32(
    int nFi, int nF, int nC, const int2* __restrict__ faceLR, const float4* __restrict__ faceNA,
    const float* __restrict__ W, const double* __restrict__ y, const double* __restrict__ v,
    const double* __restrict__ d_s, const int* __restrict__ bcT, const double* __restrict__ bcP,
    int maxP, double g, double r, float* __restrict__ F) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nF) return;
  const int2 lr = __ldg(faceLR + f);
  const float4 na = __ldg(faceNA + f);
  P32 L, R;
  load_prim32(W, lr.x, L);
  if (f < nFi) {
    load_prim32(W, lr.y, R);
  } else {
    double U[5], G[5];
#pragma unroll
    for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + lr.x];
    if (v) {
      const double s = *d_s;
#pragma unroll
      for (int q = 0; q < 5; q++) U[q] = U[q] + s * v[(size_t)q * nC + lr.x];
    }
    const int row = lr.y;
    const int type = row > 0 ? bcT[row - 1] : FOS_BC_WALL;
    ghost_state(type, row > 0 ? bcP + (size_t)maxP * (row - 1) : nullptr, U, na.x, na.y, na.z,
                g, r, G);
    const float rho = (float)G[0], inv = 1.0f / rho;
    const float mx = (float)G[1], my = (float)G[2], mz = (float)G[3], E = (float)G[4];
    R.rho = rho; R.u = mx * inv; R.v = my * inv; R.w = mz * inv;
    R.p = (float)(g - 1.0) * (E - 0.5f * (mx * mx + my * my + mz * mz) * inv);
    R.H = (E + R.p) * inv;
    R.s = sqrtf(rho);
  }
  float dF[5], dw[5];
  roe_split32(L, R, na.x, na.y, na.z, na.w, (float)(g - 1.0), dF, dw);
  // (dF, dw) pairs as float2 per component: F2[q*nF + f]
  float2* F2 = reinterpret_cast<float2*>(F);
#pragma unroll
  for (int q = 0; q < 5; q++) F2[(size_t)q * nF + f] = make_float2(dF[q], dw[q]);
}

// FP64 accumulation of the FP32 face terms: cell L gets -(dF - dw), cell R gets -(dF + dw)
__global__ void __launch_bounds__(kThreads) k_gather32(
    int nC, int nF, const int* __restrict__ crow, const int* __restrict__ cent,
    const float* __restrict__ F, const double* __restrict__ invV, int mode,
    const double* __restrict__ vv, const double* __restrict__ fy, const double* __restrict__ d_s,
    double a, double b, double* __restrict__ out, int* __restrict__ flag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const float2* F2 = reinterpret_cast<const float2*>(F);
  const int e0 = __ldg(crow + c), e1 = __ldg(crow + c + 1);
  for (int e = e0; e < e1; e++) {
    const int ent = __ldg(cent + e);
    const int f = ent >> 1;
    const bool isR = ent & 1;
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const float2 x = __ldg(F2 + (size_t)q * nF + f);
      acc[q] -= isR ? (double)x.x + (double)x.y : (double)x.x - (double)x.y;
    }
  }
  const double iv = __ldg(invV + c);
  bool bad = false;
  if (mode == 0) {
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const double o = acc[q] * iv;
      bad |= !isfinite(o);
      out[(size_t)q * nC + c] = o;
    }
  } else {
    const double s = *d_s;
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const size_t k = (size_t)q * nC + c;
      double o = a * vv[k];
      if (s > 0.0) o += b * ((acc[q] * iv - fy[k]) / s);
      bad |= !isfinite(o);
      out[k] = o;
    }
  }
  if (bad && flag) atomicOr(flag, 1);
}

__global__ void k_permute(int nC, const int* __restrict__ idx, const double* __restrict__ in,
                          double* __restrict__ out) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 5L * nC) return;
  const int q = (int)(k / nC), i = (int)(k - (long)q * nC);
  out[k] = in[(size_t)q * nC + idx[i]];
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__global__ void __launch_bounds__(kRedThreads) k_sumsq_part(const double* __restrict__ x, long n,
                                                            double* __restrict__ part) {
  double s = 0.0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double t = x[i];
    s += t * t;
  }
  __shared__ double sh[kRedThreads / 32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < kRedThreads / 32 ? sh[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

__global__ void k_sum_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  __shared__ double sh[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) *out = t;
  }
}

__global__ void k_sigma(double* scal, double ynorm, double eps) {
  const double vn2 = scal[0];
  scal[1] = vn2 > 0.0 ? eps * (1.0 + ynorm) / sqrt(vn2) : 0.0;
}

inline int nblk(long n, int t = kThreads) { return (int)((n + t - 1) / t); }

}  // namespace

int fos_residual_launch(fos_ctx* c, const double* y, const double* v, const double* d_s,
                        const double* fy, double* out, double a, double b, int mode) {
  const double gm1 = c->gamm - 1.0;
  if (c->flags & FOS_FLUX_FP32) {
    fos_launch(c, k_prim32, nblk(c->nC), kThreads, c->nC, y, v, d_s, gm1, c->d_W32);
    fos_launch(c, k_face32, nblk(c->nF), kThreads, 
        c->nFi, c->nF, c->nC, c->d_faceLR, c->d_faceNA32, c->d_W32, y, v, d_s, c->d_bcT,
        c->d_bcP, c->maxP, c->gamm, c->r, reinterpret_cast<float*>(c->d_F));
    fos_launch(c, k_gather32, nblk(c->nC), kThreads, 
        c->nC, c->nF, c->d_crow, c->d_cent, reinterpret_cast<const float*>(c->d_F), c->d_invV,
        mode, v, fy, d_s, a, b, out, c->d_flag);
  } else {
    fos_launch(c, k_prim64, nblk(c->nC), kThreads, c->nC, y, v, d_s, gm1, c->d_W);
    fos_launch(c, k_face64, nblk(c->nF), kThreads, c->nFi, c->nF, c->nC, c->d_faceLR,
                                                       c->d_faceNA, c->d_W, y, v, d_s, c->d_bcT,
                                                       c->d_bcP, c->maxP, c->gamm, c->r, c->d_F);
    fos_launch(c, k_gather, nblk(c->nC), kThreads, c->nC, c->nF, c->d_crow, c->d_cent,
                                                      c->d_F, c->d_invV, mode, v, fy, d_s, a, b,
                                                      out, c->d_flag);
  }
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_prim_launch(fos_ctx* c, const double* y) {
  fos_launch(c, k_prim64, nblk(c->nC), kThreads, c->nC, y, nullptr, nullptr, c->gamm - 1.0,
                                                    c->d_W);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_norm2_dev(fos_ctx* c, const double* x, long n, double* d_out_sq) {
  fos_launch(c, k_sumsq_part, kRedBlocks, kRedThreads, x, n, c->d_red);
  fos_launch(c, k_sum_final, 1, 1024, c->d_red, kRedBlocks, d_out_sq);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_jv_sigma(fos_ctx* c, double* d_scal, double ynorm, double eps) {
  fos_launch(c, k_sigma, 1, 1, d_scal, ynorm, eps);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_permute(fos_ctx* c, const double* in, double* out, int dir) {
  const int* idx = dir == 0 ? c->d_new2old : c->d_old2new;
  fos_launch(c, k_permute, nblk(5L * c->nC), kThreads, c->nC, idx, in, out);
  FOS_LAUNCH_CHECK();
  return 0;
}
