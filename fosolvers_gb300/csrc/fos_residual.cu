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
// The FP32-flux variant (FOS_FLUX_FP32) computes the same flow in FP32, in flux-difference
// form, from per-cell FP32 (hi, lo) primitive pairs (k_prim_hl), and fuses the interior
// faces into the cell gather (k_cell32: each interior face evaluated by both of its cells,
// bit-identically); boundary faces go through k_bface32 (ghost state and flow in FP64,
// stored as the difference from the cell's own flux).  Sums are in FP64 in both variants.
#include <cmath>
#include <mutex>
#include <string>

#include "fos_internal.h"
#include "fos_device.cuh"

namespace {

constexpr int kThreads = 64;  // residual and Jv at 96^3: 64 measured 1.5% faster than 128, 128 3% faster than 256

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

// kV: the state is y + s v (a Jv), else y (compile-time, as in k_prim_hl)
template <bool kV>
__global__ void __launch_bounds__(kThreads) k_prim64(int nC, const double* __restrict__ y,
                                                     const double* __restrict__ v,
                                                     const double* __restrict__ d_s, double gm1,
                                                     double* __restrict__ W) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  double U[5];
#pragma unroll
  for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + c];
  if constexpr (kV) {
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
  double2* F2 = reinterpret_cast<double2*>(F + 6 * (size_t)f);  // AoS, 48 B per face
  F2[0] = make_double2(flow[0], flow[1]);
  F2[1] = make_double2(flow[2], flow[3]);
  F2[2] = make_double2(flow[4], 0.0);
}

// Per-cell gather.  ELL layout: every cell has kW entry slots (face << 1 | cell-is-R,
// -1 = empty), loaded as one int4 for kW = 4 (tetrahedra), so all face loads of a cell
// are issued together; the fixed slot order gives a deterministic summation order.
// residual: out = sum/v ; Jv: out = a*v + b*(sum/v - fy)/s (gather_epilogue)
template <int kW>
__device__ __forceinline__ void load_ell(const int* __restrict__ ell, int c, int e[kW]) {
  if (kW == 4) {
    const int4 q = __ldg(reinterpret_cast<const int4*>(ell) + c);
    e[0] = q.x; e[1] = q.y; e[2] = q.z; e[3] = q.w;
  } else {
#pragma unroll
    for (int k = 0; k < kW; k++) e[k] = __ldg(ell + (size_t)kW * c + k);
  }
}

// The epilogue kind, a template parameter so that each kernel carries only its own FP64
// instructions (the FP64 pipe is GB300's scarcest): kEpiRhs out = acc / v; the Jv
// combination a v + (b / s)(acc / v - fy) with a = 1 (kEpiJv1), a = 0 (kEpiJv0) or any a
// (kEpiJvA).
enum { kEpiRhs = 0, kEpiJv1 = 1, kEpiJv0 = 2, kEpiJvA = 3 };
inline int epi_kind(int mode, double a) {
  return mode == 0 ? kEpiRhs : a == 1.0 ? kEpiJv1 : a == 0.0 ? kEpiJv0 : kEpiJvA;
}

// The epilogue in FP64; b / s comes precomputed in d_s[2] (k_sigma); non-finite results are
// flagged from the exponent bits (no FP64 compares)
template <int kE>
__device__ __forceinline__ void gather_epilogue(int nC, int c, const double acc[5], double iv,
                                                const double* __restrict__ vv,
                                                const double* __restrict__ fy,
                                                const double* __restrict__ d_s, double a,
                                                double* __restrict__ out, int* __restrict__ flag) {
  bool ok = true;
  if constexpr (kE == kEpiRhs) {
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const double o = acc[q] * iv;
      ok &= finite_bits(o);
      out[(size_t)q * nC + c] = o;
    }
  } else {
    const double bs = __ldg(d_s + 2);  // b / s
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const size_t k = (size_t)q * nC + c;
      const double t = fma(acc[q], iv, -fy[k]);
      double o;
      if constexpr (kE == kEpiJv1) o = fma(bs, t, vv[k]);
      else if constexpr (kE == kEpiJv0) o = bs * t;
      else o = fma(bs, t, a * vv[k]);
      ok &= finite_bits(o);
      out[k] = o;
    }
  }
  if (!ok && flag) atomicOr(flag, 1);
}

template <int kW, int kE>
__global__ void __launch_bounds__(kThreads) k_gather(
    int nC, const int* __restrict__ ell, const double* __restrict__ F,
    const double* __restrict__ invV, const double* __restrict__ vv,
    const double* __restrict__ fy, const double* __restrict__ d_s, double a,
    double* __restrict__ out, int* __restrict__ flag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  int e[kW];
  load_ell<kW>(ell, c, e);
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < kW; k++) {
    if (e[k] < 0) continue;
    const double sg = (e[k] & 1) ? 1.0 : -1.0;
    const double2* F2 = reinterpret_cast<const double2*>(F + 6 * (size_t)(e[k] >> 1));
    const double2 a0 = __ldg(F2), a1 = __ldg(F2 + 1), a2 = __ldg(F2 + 2);
    acc[0] += sg * a0.x; acc[1] += sg * a0.y; acc[2] += sg * a1.x; acc[3] += sg * a1.y;
    acc[4] += sg * a2.x;
  }
  gather_epilogue<kE>(nC, c, acc, __ldg(invV + c), vv, fy, d_s, a, out, flag);
}

using gather_fn = decltype(&k_gather<4, kEpiRhs>);
template <int kW>
gather_fn gather_kernel_w(int ek) {
  switch (ek) {
    case kEpiRhs: return k_gather<kW, kEpiRhs>;
    case kEpiJv1: return k_gather<kW, kEpiJv1>;
    case kEpiJv0: return k_gather<kW, kEpiJv0>;
    default: return k_gather<kW, kEpiJvA>;
  }
}
gather_fn gather_kernel(int ell_w, int ek) {
  return ell_w == 4 ? gather_kernel_w<4>(ek) : gather_kernel_w<6>(ek);
}

// ------------------------------------------------------------------ FP32 flux
// Per-cell primitives for the FP32 flux as FP32 (hi, lo) pairs x = hi + lo (~46 bits), so
// a face jump (hR - hL) + (lR - lL) keeps FP32 relative accuracy of the jump itself while
// the face arithmetic issues FP32 instructions only.  The primitives are formed in
// double-float arithmetic (df_*: FP32 pipe); only the Jv perturbation y + s v is FP64.
// Layout: 16 floats (64 B) per cell = (rho, u, v, w, H, p) hi, (rho, u, v, w, H, p) lo,
// sqrt(rho), 0, 0, 0.
// kV: the state is y + s v (a Jv), else y; a compile-time switch, so a residual issues no
// predicated-off FP64 FMAs
template <bool kV>
__global__ void __launch_bounds__(kThreads) k_prim_hl(int nC, const double* __restrict__ y,
                                                      const double* __restrict__ v,
                                                      const double* __restrict__ d_s, double gm1,
                                                      float* __restrict__ W) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  double U[5];
#pragma unroll
  for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + c];
  if constexpr (kV) {
    const double s = *d_s;
#pragma unroll
    for (int q = 0; q < 5; q++) U[q] = fma(s, v[(size_t)q * nC + c], U[q]);
  }
  const df2 r = df_from_double(U[0]), mx = df_from_double(U[1]), my = df_from_double(U[2]),
            mz = df_from_double(U[3]), E = df_from_double(U[4]), g = df_from_double(gm1);
  const df2 inv = df_rcp(r);
  const df2 u = df_mul(mx, inv), vv = df_mul(my, inv), w = df_mul(mz, inv);
  const df2 ke = df_add(df_add(df_mul(mx, u), df_mul(my, vv)), df_mul(mz, w));  // rho |u|^2
  const df2 p = df_mul(g, df_add(E, df_scale(ke, -0.5f)));
  const df2 H = df_mul(df_add(E, p), inv);
  float4* w4 = reinterpret_cast<float4*>(W + 16 * (size_t)c);
  w4[0] = make_float4(r.h, u.h, vv.h, w.h);
  w4[1] = make_float4(H.h, p.h, r.l, u.l);
  w4[2] = make_float4(vv.l, w.l, H.l, p.l);
  w4[3] = make_float4(sqrtf(r.h + r.l), 0.0f, 0.0f, 0.0f);
}

struct PHL {
  float h[6], l[6], s;
};
__device__ __forceinline__ void load_hl(const float* __restrict__ W, int c, PHL& P) {
  const float4* w4 = reinterpret_cast<const float4*>(W + 16 * (size_t)c);
  const float4 a = __ldg(w4), b = __ldg(w4 + 1), d = __ldg(w4 + 2), e = __ldg(w4 + 3);
  P.h[0] = a.x; P.h[1] = a.y; P.h[2] = a.z; P.h[3] = a.w; P.h[4] = b.x; P.h[5] = b.y;
  P.l[0] = b.z; P.l[1] = b.w; P.l[2] = d.x; P.l[3] = d.y; P.l[4] = d.z; P.l[5] = d.w;
  P.s = e.x;
}

// Roe flow from means / jumps in flux-difference form (the interior faces of the FP32 flux,
// in FP32; with FOS_FLUX_HYBRID the faces with large jumps, in FP64): dF = aP (F_R - F_L).n / 2
// expanded with d(ab) = mean(a) d(b) + d(a) mean(b) and mean(ab) = mean(a) mean(b) + d(a) d(b)/4,
// and dw = aP |A~| (U_R - U_L) / 2 from the Roe average (Euler.f90:90-126)
template <typename T>
__device__ __forceinline__ void roe_split_mj(T rm, T dr, T um, T du, T vm, T dv, T wm, T dww,
                                             T Hm, T dH, T dp, T ds, T ss, T ps, T nx, T ny, T nz,
                                             T aP, T gm1, T dF[5], T dw[5]) {
  const T half = T(0.5), quarter = T(0.25);
  const T unm = um * nx + vm * ny + wm * nz;
  const T dun = du * nx + dv * ny + dww * nz;
  const T mm = rm * unm + quarter * dr * dun;  // mean of m = rho un
  const T dm = rm * dun + dr * unm;            // jump of m
  const T h = half * aP;
  dF[0] = h * dm;
  dF[1] = h * (mm * du + dm * um + dp * nx);
  dF[2] = h * (mm * dv + dm * vm + dp * ny);
  dF[3] = h * (mm * dww + dm * wm + dp * nz);
  dF[4] = h * (mm * dH + dm * Hm);
  const T kap = half * ds / ss;
  const T ua = um + kap * du, va = vm + kap * dv, wa = wm + kap * dww, Ha = Hm + kap * dH;
  const T rhoA = ps;
  const T q2 = ua * ua + va * va + wa * wa;
  const T c2 = gm1 * (Ha - half * q2);
  const T ca = sqrt(c2);
  const T ic2 = T(1) / c2;
  const T unA = ua * nx + va * ny + wa * nz;
  const T au = fabs(unA);
  const T wE = dr - dp * ic2;
  T d0 = au * wE;
  T d1 = au * (wE * ua + rhoA * (du - nx * dun));
  T d2 = au * (wE * va + rhoA * (dv - ny * dun));
  T d3 = au * (wE * wa + rhoA * (dww - nz * dun));
  T d4 = au * (wE * (half * q2) + rhoA * (ua * du + va * dv + wa * dww - unA * dun));
  const T s1 = fabs(unA - ca) * (half * (dp - rhoA * ca * dun) * ic2);
  d0 += s1; d1 += s1 * (ua - nx * ca); d2 += s1 * (va - ny * ca); d3 += s1 * (wa - nz * ca);
  d4 += s1 * (Ha - unA * ca);
  const T s2 = fabs(unA + ca) * (half * (dp + rhoA * ca * dun) * ic2);
  d0 += s2; d1 += s2 * (ua + nx * ca); d2 += s2 * (va + ny * ca); d3 += s2 * (wa + nz * ca);
  d4 += s2 * (Ha + unA * ca);
  dw[0] = h * d0; dw[1] = h * d1; dw[2] = h * d2; dw[3] = h * d3; dw[4] = h * d4;
}

// Boundary faces [nFi, nF) of the FP32 flux (1% of the faces): the face's Roe flow minus the
// interior cell's own flux aP F(u_L).n, i.e. the flow in the difference form that k_cell32
// accumulates, stored as FP64 (5 of the face's 6 slots of F).
//   wall (mirrored ghost: equal rho, p, H, normal velocity reversed): the Roe average has
//     zero normal velocity and the flow reduces to aP (0, (p + rho un (un + c)) n, 0), c^2 =
//     (g-1)(H - |u_t|^2/2); the difference aP rho un (-1, (un + c) n - u, -H) is formed in
//     FP32 from the FP32 primitives (k_prim_hl, same state as y + s v);
//   other conditions (and walls too with FOS_FLUX_HYBRID, all64): k_face64's FP64 flow
//     (interior and ghost primitives from the conserved variables) minus the own flux, in FP64.
__global__ void __launch_bounds__(kThreads) k_bface32(
    int nFi, int nF, int nC, const int2* __restrict__ faceLR, const double2* __restrict__ faceNA,
    const float4* __restrict__ faceNA32, const float* __restrict__ Whl, float gm1f,
    const double* __restrict__ y, const double* __restrict__ v, const double* __restrict__ d_s,
    const int* __restrict__ bcT, const double* __restrict__ bcP, int maxP, double g, double r,
    double* __restrict__ F, int all64) {
  const int f = nFi + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nF) return;
  const int2 lr = __ldg(faceLR + f);
  const int row = lr.y;
  const int type = row > 0 ? bcT[row - 1] : FOS_BC_WALL;
  double2* F2 = reinterpret_cast<double2*>(F + 6 * (size_t)f);
  if (type == FOS_BC_WALL && !all64) {
    const float4 na = __ldg(faceNA32 + f);
    const float4* w4 = reinterpret_cast<const float4*>(Whl + 16 * (size_t)lr.x);
    const float4 a = __ldg(w4), b = __ldg(w4 + 1);  // (rho, u, v, w), (H, p, ...) hi parts
    const float un = a.y * na.x + a.z * na.y + a.w * na.z;
    const float q2 = a.y * a.y + a.z * a.z + a.w * a.w;
    const float c = sqrtf(gm1f * (b.x - 0.5f * (q2 - un * un)));
    const float m = na.w * a.x * un, k = un + c;
    F2[0] = make_double2(f2d_bits(-m), f2d_bits(m * (k * na.x - a.y)));
    F2[1] = make_double2(f2d_bits(m * (k * na.y - a.z)), f2d_bits(m * (k * na.z - a.w)));
    F2[2] = make_double2(f2d_bits(-m * b.x), 0.0);
    return;
  }
  const double2 n01 = __ldg(faceNA + 2 * (size_t)f), n2a = __ldg(faceNA + 2 * (size_t)f + 1);
  const double nx = n01.x, ny = n01.y, nz = n2a.x, aP = n2a.y;
  double U[5], G[5];
#pragma unroll
  for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + lr.x];
  if (v) {
    const double s = *d_s;
#pragma unroll
    for (int q = 0; q < 5; q++) U[q] = U[q] + s * v[(size_t)q * nC + lr.x];
  }
  ghost_state(type, row > 0 ? bcP + (size_t)maxP * (row - 1) : nullptr, U, nx, ny, nz, g, r, G);
  P64 L, R;
  prim_from_cons(U[0], U[1], U[2], U[3], U[4], g - 1.0, L);
  prim_from_cons(G[0], G[1], G[2], G[3], G[4], g - 1.0, R);
  double flow[5];
  roe_flow64(L, R, nx, ny, nz, aP, g - 1.0, flow);
  const double m = aP * L.rho * (L.u * nx + L.v * ny + L.w * nz), pa = aP * L.p;
  F2[0] = make_double2(flow[0] - m, flow[1] - (m * L.u + pa * nx));
  F2[1] = make_double2(flow[2] - (m * L.v + pa * ny), flow[3] - (m * L.w + pa * nz));
  F2[2] = make_double2(flow[4] - m * L.H, 0.0);
}

// Fused interior flux + cell gather for the FP32 flux (one pass, no face-flow array for
// interior faces).  Thread per cell: each interior face of the cell is evaluated in the
// face's own orientation (L = faceLR.x, R = faceLR.y) from the FP32 (hi, lo) means and
// jumps, FP32 instructions only, so
// the two cells of a face compute bit-identical (dF, dw) and the scheme stays exactly
// conservative; the cell then takes -(dF - dw) (cell is L) or -(dF + dw) (cell is R) in
// FP64, in ascending ELL order.  Boundary faces read the FP64 differences k_bface32 wrote.
// Each face is evaluated twice -- cheap FP32 arithmetic in exchange for the 2 x 48 B per face
// a face-flow array costs in HBM traffic.  Cells that are not closed (Sc non-null: warped
// faces) also take the own-flux sum the difference form leaves out, -F(u_c).S_c.
// kHyb (FOS_FLUX_HYBRID): a face whose relative density or pressure jump exceeds theta is
// evaluated in FP64 (the same expressions, from the FP64 values of the (hi, lo) pairs and
// the FP64 geometry); both cells decide from the same face-oriented values, so they agree.
// A residual (kEpiRhs) records the choice per face (fsel, written by the face's L cell); a
// Jv reuses it, so f(y + s v) and f(y) evaluate every face the same way.
template <int kW, bool kHyb, int kE, bool kSc>
__global__ void __launch_bounds__(kThreads) k_cell32(
    int nC, int nFi, const int* __restrict__ ell, const int* __restrict__ cnb,
    const float4* __restrict__ cna, const float* __restrict__ W, float gm1,
    const double* __restrict__ Fb, const float4* __restrict__ Sc,
    const double* __restrict__ invV,
    const double* __restrict__ vv, const double* __restrict__ fy, const double* __restrict__ d_s,
    double a, double* __restrict__ out, int* __restrict__ flag,
    const double2* __restrict__ faceNA64, unsigned char* __restrict__ fsel, float theta,
    double gm1d) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  int e[kW], nbr[kW];
  load_ell<kW>(ell, c, e);
  load_ell<kW>(cnb, c, nbr);  // the cells across the faces: no wait on the face arrays
  PHL P;
  load_hl(W, c, P);
  // FP64 accumulation in ELL order; the first face initialises the sums (every cell has
  // at least one face, and ELL rows are padded at the end).  The terms come negated from
  // the face arithmetic (FP32 or FP64, where negation is exact), so the sums are plain
  // additions: acc = n_0 + n_1 + ..., no FP64 negation for the first term
  double acc[5];
#pragma unroll
  for (int k = 0; k < kW; k++) {
    if (k > 0 && e[k] < 0) continue;
    const int f = e[k] >> 1;
    const bool isR = e[k] & 1;
    double t[5];  // the face's term: -(dF - dw) (cell is L) or -(dF + dw) (cell is R)
    if (f < nFi) {
      const float sw = isR ? 1.0f : -1.0f;
      const float4 na = __ldg(cna + (size_t)k * nC + c);
      PHL Q;
      load_hl(W, nbr[k], Q);
      // Orientation by signs, not by selecting L and R: the means are formed from P + Q
      // (symmetric) and the jumps as -sw ((Q.h - P.h) + (Q.l - P.l)), which is R - L bit for
      // bit either way (negation commutes with round-to-nearest)
      float m[6], d[6], dF[5], dw[5];
#pragma unroll
      for (int j = 0; j < 6; j++) {
        m[j] = 0.5f * (P.h[j] + Q.h[j]) + 0.5f * (P.l[j] + Q.l[j]);
        d[j] = -sw * ((Q.h[j] - P.h[j]) + (Q.l[j] - P.l[j]));
      }
      bool f64 = false;
      if (kHyb) {
        if (kE == kEpiRhs || !fsel) {
          f64 = fabsf(d[0]) > theta * fminf(P.h[0], Q.h[0]) ||
                fabsf(d[5]) > theta * fminf(P.h[5], Q.h[5]);
          if (kE == kEpiRhs && fsel && !isR) fsel[f] = f64 ? 1 : 0;
        } else {
          f64 = __ldg(fsel + f) != 0;
        }
      }
      if (kHyb && f64) {
        const PHL& L = isR ? Q : P;
        const PHL& R = isR ? P : Q;
        double md[6], dd[6], rl = 0.0, rr = 0.0;
#pragma unroll
        for (int j = 0; j < 6; j++) {
          const double xl = f2d_bits(L.h[j]) + f2d_bits(L.l[j]);
          const double xr = f2d_bits(R.h[j]) + f2d_bits(R.l[j]);
          md[j] = 0.5 * (xl + xr);
          dd[j] = xr - xl;
          if (j == 0) { rl = xl; rr = xr; }
        }
        const double2 n01 = __ldg(faceNA64 + 2 * (size_t)f), n2a = __ldg(faceNA64 + 2 * (size_t)f + 1);
        double dF64[5], dw64[5];
        const double sl = sqrt(rl), sr = sqrt(rr);
        roe_split_mj<double>(md[0], dd[0], md[1], dd[1], md[2], dd[2], md[3], dd[3], md[4],
                             dd[4], dd[5], sr - sl, sl + sr, sl * sr, n01.x, n01.y, n2a.x,
                             n2a.y, gm1d, dF64, dw64);
#pragma unroll
        for (int q = 0; q < 5; q++) t[q] = isR ? -dF64[q] - dw64[q] : dw64[q] - dF64[q];
      } else {
        roe_split_mj<float>(m[0], d[0], m[1], d[1], m[2], d[2], m[3], d[3], m[4], d[4], d[5],
                            -sw * (Q.s - P.s), P.s + Q.s, P.s * Q.s, na.x, na.y, na.z, na.w,
                            gm1, dF, dw);
#pragma unroll
        for (int q = 0; q < 5; q++) t[q] = f2d_bits(fmaf(-sw, dw[q], -dF[q]));
      }
    } else {  // boundary face (cell is L): the FP64 difference of k_bface32, negated
      const double2* F2 = reinterpret_cast<const double2*>(Fb + 6 * (size_t)f);
      const double2 a0 = __ldg(F2), a1 = __ldg(F2 + 1), a2 = __ldg(F2 + 2);
      t[0] = neg_bits(a0.x); t[1] = neg_bits(a0.y); t[2] = neg_bits(a1.x);
      t[3] = neg_bits(a1.y); t[4] = neg_bits(a2.x);
    }
#pragma unroll
    for (int q = 0; q < 5; q++) acc[q] = k == 0 ? t[q] : acc[q] + t[q];
  }
  // own flux through the closure vector (kSc: the grid has cells whose faces do not close):
  // rho u.S, rho u u.S + p S, rho H u.S.  A compile-time switch: as a run-time branch the
  // five FP64 subtractions were issued predicated off on every cell, occupying the FP64 pipe
  if constexpr (kSc) {
    const float4 S = __ldg(Sc + c);
    const float t = P.h[0] * (P.h[1] * S.x + P.h[2] * S.y + P.h[3] * S.z);
    acc[0] -= f2d_bits(t);
    acc[1] -= f2d_bits(fmaf(t, P.h[1], P.h[5] * S.x));
    acc[2] -= f2d_bits(fmaf(t, P.h[2], P.h[5] * S.y));
    acc[3] -= f2d_bits(fmaf(t, P.h[3], P.h[5] * S.z));
    acc[4] -= f2d_bits(t * P.h[4]);
  }
  gather_epilogue<kE>(nC, c, acc, __ldg(invV + c), vv, fy, d_s, a, out, flag);
}

using cell32_fn = decltype(&k_cell32<4, false, kEpiRhs, false>);
template <int kW, bool kHyb, bool kSc>
cell32_fn cell32_kernel_whs(int ek) {
  switch (ek) {
    case kEpiRhs: return k_cell32<kW, kHyb, kEpiRhs, kSc>;
    case kEpiJv1: return k_cell32<kW, kHyb, kEpiJv1, kSc>;
    case kEpiJv0: return k_cell32<kW, kHyb, kEpiJv0, kSc>;
    default: return k_cell32<kW, kHyb, kEpiJvA, kSc>;
  }
}
template <int kW, bool kHyb>
cell32_fn cell32_kernel_wh(int ek, bool sc) {
  return sc ? cell32_kernel_whs<kW, kHyb, true>(ek) : cell32_kernel_whs<kW, kHyb, false>(ek);
}
cell32_fn cell32_kernel(int ell_w, bool hyb, int ek, bool sc) {
  if (ell_w == 4)
    return hyb ? cell32_kernel_wh<4, true>(ek, sc) : cell32_kernel_wh<4, false>(ek, sc);
  return hyb ? cell32_kernel_wh<6, true>(ek, sc) : cell32_kernel_wh<6, false>(ek, sc);
}

__global__ void k_permute(int nC, int nplanes, const int* __restrict__ idx,
                          const double* __restrict__ in, double* __restrict__ out) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long)nplanes * nC) return;
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

// s, 1/s and b/s of the Jv (scal[1..3]; the epilogue reads them as d_s[0..2])
__global__ void k_sigma(double* scal, double ynorm, double eps, double b) {
  const double vn2 = scal[0];
  const double s = vn2 > 0.0 ? eps * (1.0 + ynorm) / sqrt(vn2) : 0.0;
  scal[1] = s;
  scal[2] = s > 0.0 ? 1.0 / s : 0.0;
  scal[3] = s > 0.0 ? b * scal[2] : 0.0;  // b (1/s), as the epilogue formed it
}

// the same with ||v||_2 supplied by the caller (no reduction pass over v)
__global__ void k_sigma_known(double* scal, double ynorm, double vnorm, double eps, double b) {
  const double s = vnorm > 0.0 ? eps * (1.0 + ynorm) / vnorm : 0.0;
  scal[0] = vnorm * vnorm;
  scal[1] = s;
  scal[2] = s > 0.0 ? 1.0 / s : 0.0;
  scal[3] = s > 0.0 ? b * scal[2] : 0.0;  // b (1/s), as the epilogue formed it
}

inline int nblk(long n, int t = kThreads) { return (int)((n + t - 1) / t); }

}  // namespace

int fos_residual_launch(fos_ctx* c, const double* y, const double* v, const double* d_s,
                        const double* fy, double* out, double a, double b, int mode) {
  (void)b;  // b / s comes from the preceding fos_jv_sigma* (d_s[2])
  const double gm1 = c->gamm - 1.0;
  const int ek = epi_kind(mode, a);
  if (c->flags & FOS_FLUX_FP32) {
    if (v) fos_launch(c, k_prim_hl<true>, nblk(c->nC), kThreads, c->nC, y, v, d_s, gm1, c->d_Whl);
    else fos_launch(c, k_prim_hl<false>, nblk(c->nC), kThreads, c->nC, y, v, d_s, gm1, c->d_Whl);
    const bool hyb = (c->flags & FOS_FLUX_HYBRID) != 0;
    if (c->nFb)
      fos_launch(c, k_bface32, nblk(c->nFb), kThreads, c->nFi, c->nF, c->nC,
                 (const int2*)c->d_faceLR, (const double2*)c->d_faceNA,
                 (const float4*)c->d_faceNA32, (const float*)c->d_Whl, (float)gm1, y, v, d_s,
                 (const int*)c->d_bcT, (const double*)c->d_bcP, c->maxP, c->gamm, c->r, c->d_F,
                 hyb ? 1 : 0);
    fos_launch(c, cell32_kernel(c->ell_w, hyb, ek, c->d_closure32 != nullptr), nblk(c->nC), kThreads, c->nC, c->nFi,
               (const int*)c->d_ell, (const int*)c->d_cnb, (const float4*)c->d_cna32,
               (const float*)c->d_Whl, (float)gm1, (const double*)c->d_F,
               (const float4*)c->d_closure32, (const double*)c->d_invV, v, fy, d_s, a,
               out, c->d_flag, (const double2*)c->d_faceNA, c->d_fsel, (float)c->hyb_theta, gm1);
  } else {
    if (v) fos_launch(c, k_prim64<true>, nblk(c->nC), kThreads, c->nC, y, v, d_s, gm1, c->d_W);
    else fos_launch(c, k_prim64<false>, nblk(c->nC), kThreads, c->nC, y, v, d_s, gm1, c->d_W);
    fos_launch(c, k_face64, nblk(c->nF), kThreads, c->nFi, c->nF, c->nC,
               (const int2*)c->d_faceLR, (const double2*)c->d_faceNA, (const double*)c->d_W, y, v,
               d_s, (const int*)c->d_bcT, (const double*)c->d_bcP, c->maxP, c->gamm, c->r,
               c->d_F);
    fos_launch(c, gather_kernel(c->ell_w, ek), nblk(c->nC), kThreads, c->nC,
               (const int*)c->d_ell, (const double*)c->d_F, (const double*)c->d_invV, v, fy, d_s,
               a, out, c->d_flag);
  }
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_prim_hl_launch(fos_ctx* c, const double* y) {
  fos_launch(c, k_prim_hl<false>, nblk(c->nC), kThreads, c->nC, y, nullptr, nullptr, c->gamm - 1.0,
             c->d_Whl);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_prim_launch(fos_ctx* c, const double* y) {
  fos_launch(c, k_prim64<false>, nblk(c->nC), kThreads, c->nC, y, nullptr, nullptr, c->gamm - 1.0,
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

int fos_sum_partials(fos_ctx* c, int np, double* d_out) {
  fos_launch(c, k_sum_final, 1, 1024, (const double*)c->d_red, np, d_out);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_jv_sigma(fos_ctx* c, double* d_scal, double ynorm, double eps, double b) {
  fos_launch(c, k_sigma, 1, 1, d_scal, ynorm, eps, b);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_jv_sigma_known(fos_ctx* c, double* d_scal, double ynorm, double vnorm, double eps,
                       double b) {
  fos_launch(c, k_sigma_known, 1, 1, d_scal, ynorm, vnorm, eps, b);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_permute(fos_ctx* c, const double* in, double* out, int dir) {
  const int* idx = dir == 0 ? c->d_new2old : c->d_old2new;
  fos_launch(c, k_permute, nblk(5L * c->nC), kThreads, c->nC, 5, idx, in, out);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_permute_plane(fos_ctx* c, const double* in, double* out, int dir, int q) {
  const int* idx = dir == 0 ? c->d_new2old : c->d_old2new;
  const size_t off = (size_t)q * c->nC;
  fos_launch(c, k_permute, nblk(c->nC), kThreads, c->nC, 1, idx, in + off, out + off);
  FOS_LAUNCH_CHECK();
  return 0;
}

// ------------------------------------------------------------------ allocation-free residual
// fos_euler_rhs_dev_static: the residual of fos_euler_rhs_dev for callers that cannot
// allocate device memory when they evaluate it -- a host code that hands the library a
// fixed memory budget and owns every allocation itself, or one that must not allocate
// inside its time loop.  Its scratch (per-cell primitives, 64 B per cell, and per-face
// flows, 48 B per face) lives in this file-scope device array instead of the context's
// buffers.  Every device that loads the library holds the array (10.75 MiB) until exit.
constexpr int kStaticMaxCells = FOS_STATIC_MAX_CELLS;
constexpr int kStaticMaxFaces = FOS_STATIC_MAX_FACES;
constexpr size_t kStaticCellBytes = 64ull * kStaticMaxCells;
static __device__ __align__(256) unsigned char g_rhs_scratch[kStaticCellBytes +
                                                             48ull * kStaticMaxFaces];

namespace {
constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_addr[kStaticMaxDevices] = {nullptr};  // device address of g_rhs_scratch

// Device address of the scratch array on the current device.  The host-side symbol is
// only a stand-in, so the address is asked for once per device (with that device current).
int static_scratch(void** out) {
  int dev = 0;
  FOS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kStaticMaxDevices) {
    fos_set_error("fos_euler_rhs_dev_static: device ordinal out of range");
    return -1;
  }
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    FOS_CUDA(cudaGetSymbolAddress(&p, g_rhs_scratch));
    g_static_addr[dev] = p;
  }
  *out = g_static_addr[dev];
  return 0;
}
}  // namespace

extern "C" int fos_euler_rhs_dev_static(const fos_ctx* c, double t, const double* y,
                                        double* ydot) {
  (void)t;
  if (!c || !y || !ydot) {
    fos_set_error("fos_euler_rhs_dev_static: bad arguments");
    return -1;
  }
  if (c->nC > kStaticMaxCells || c->nF > kStaticMaxFaces) {
    fos_set_error("fos_euler_rhs_dev_static: grid has " + std::to_string(c->nC) + " cells and " +
                  std::to_string(c->nF) + " faces; the static scratch holds at most " +
                  std::to_string(kStaticMaxCells) + " cells and " +
                  std::to_string(kStaticMaxFaces) + " faces");
    return -1;
  }
  int dev = 0;
  FOS_CUDA(cudaGetDevice(&dev));
  if (dev != c->device) {
    fos_set_error("fos_euler_rhs_dev_static: current device differs from the context's device");
    return -1;
  }
  void* base = nullptr;
  if (int rc = static_scratch(&base)) return rc;
  // every launch below writes all of its scratch before reading it, so nothing in the
  // shared array needs to start at zero
  unsigned char* bytes = static_cast<unsigned char*>(base);
  const double gm1 = c->gamm - 1.0;
  cudaStream_t s = c->stream;
  if (c->flags & FOS_FLUX_FP32) {
    float* Whl = reinterpret_cast<float*>(bytes);
    double* F = reinterpret_cast<double*>(bytes + kStaticCellBytes);
    k_prim_hl<false><<<nblk(c->nC), kThreads, 0, s>>>(c->nC, y, nullptr, nullptr, gm1, Whl);
    const bool hyb = (c->flags & FOS_FLUX_HYBRID) != 0;
    if (c->nFb)
      k_bface32<<<nblk(c->nFb), kThreads, 0, s>>>(c->nFi, c->nF, c->nC, c->d_faceLR,
                                                  c->d_faceNA, c->d_faceNA32, Whl, (float)gm1, y,
                                                  nullptr, nullptr, c->d_bcT, c->d_bcP, c->maxP,
                                                  c->gamm, c->r, F, hyb ? 1 : 0);
    // the face choice of the hybrid flux is made from this state (no record kept)
    cell32_kernel(c->ell_w, hyb, kEpiRhs, c->d_closure32 != nullptr)<<<nblk(c->nC), kThreads, 0, s>>>(
        c->nC, c->nFi, c->d_ell, c->d_cnb, c->d_cna32, Whl, (float)gm1, F, c->d_closure32,
        c->d_invV, nullptr, nullptr, nullptr, 0.0, ydot, nullptr, c->d_faceNA, nullptr,
        (float)c->hyb_theta, gm1);
  } else {
    double* W = reinterpret_cast<double*>(bytes);
    double* F = reinterpret_cast<double*>(bytes + kStaticCellBytes);
    k_prim64<false><<<nblk(c->nC), kThreads, 0, s>>>(c->nC, y, nullptr, nullptr, gm1, W);
    k_face64<<<nblk(c->nF), kThreads, 0, s>>>(c->nFi, c->nF, c->nC, c->d_faceLR, c->d_faceNA, W,
                                              y, nullptr, nullptr, c->d_bcT, c->d_bcP, c->maxP,
                                              c->gamm, c->r, F);
    gather_kernel(c->ell_w, kEpiRhs)<<<nblk(c->nC), kThreads, 0, s>>>(
        c->nC, c->d_ell, F, c->d_invV, nullptr, nullptr, nullptr, 0.0, ydot, nullptr);
  }
  FOS_LAUNCH_CHECK();
  return 0;
}
