// fos_device.cuh -- device helpers shared by the residual and Jacobian kernels.
#pragma once
#include "fos_internal.h"

// x^e for x > 0 as exp(e ln x).  The isentropic ratios below have x = 1 + (g-1)/2 M^2 >= 1;
// inline exp and log keep the ghost state free of function calls (pow is a called routine).
__device__ __forceinline__ double pow_pos(double x, double e) { return exp(e * log(x)); }

// Ghost conserved state of a boundary face (foeuler.f90:209-330); U = interior
// conserved (rho, mx, my, mz, E), n = unit normal out of the interior cell.  Inlined into
// each boundary kernel: as a called function (with the called pow) it raised "illegal
// instruction" faults from kernels allocated fewer registers (78-80) than the call chain
// used, on the condition types that reach pow.
__device__ __forceinline__ void ghost_state(int type, const double* __restrict__ bp, const double U[5],
                            double nx, double ny, double nz, double g, double r, double G[5]) {
  const double gm1 = g - 1.0;
  switch (type) {
    case FOS_BC_IN_STATIC: {
      double pG = bp[0], TG = bp[1], u0 = bp[2], u1 = bp[3], u2 = bp[4];
      double Mach = sqrt(u0 * u0 + u1 * u1 + u2 * u2) / sqrt(g * r * TG);
      double rG = pG / r / TG;
      if (Mach < 1.0) { u0 = U[1] / rG; u1 = U[2] / rG; u2 = U[3] / rG; }
      G[0] = rG; G[1] = rG * u0; G[2] = rG * u1; G[3] = rG * u2;
      G[4] = rG * (1.0 / gm1 * r * TG + 0.5 * (u0 * u0 + u1 * u1 + u2 * u2));
      return;
    }
    case FOS_BC_IN_TOTAL: {
      double ptG = bp[0], TtG = bp[1], u0 = bp[2], u1 = bp[3], u2 = bp[4];
      double q2 = u0 * u0 + u1 * u1 + u2 * u2;
      double TG = TtG - 0.5 * gm1 / g / r * q2;
      double Mach = sqrt(q2) / sqrt(g * r * TG);
      double pG = ptG * pow_pos(1.0 + 0.5 * gm1 * Mach * Mach, -g / gm1);
      double rG = pG / r / TG;
      if (Mach < 1.0) {
        double ui0 = U[1] / U[0], ui1 = U[2] / U[0], ui2 = U[3] / U[0];
        double sc = (ui0 * u0 + ui1 * u1 + ui2 * u2) / q2;
        u0 *= sc; u1 *= sc; u2 *= sc;
        q2 = u0 * u0 + u1 * u1 + u2 * u2;
        TG = TtG - 0.5 * gm1 / g / r * q2;
        Mach = sqrt(q2) / sqrt(g * r * TG);
        pG = ptG * pow_pos(1.0 + 0.5 * gm1 * Mach * Mach, -g / gm1);
        rG = pG / r / TG;
      }
      G[0] = rG; G[1] = rG * u0; G[2] = rG * u1; G[3] = rG * u2;
      G[4] = rG * (1.0 / gm1 * r * TG + 0.5 * q2);
      return;
    }
    case FOS_BC_OUT: {
      G[0] = U[0]; G[1] = U[1]; G[2] = U[2]; G[3] = U[3];
      G[4] = 1.0 / gm1 * bp[0] + 0.5 * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) / U[0];
      return;
    }
    case FOS_BC_OUT_EXTRAP: {
      for (int q = 0; q < 5; q++) G[q] = U[q];
      return;
    }
    case FOS_BC_FAR: {
      double pG = bp[0], TG = bp[1], g0 = bp[2], g1 = bp[3], g2 = bp[4];
      double rm = U[0], Em = U[4];
      double charO = (g0 * nx + g1 * ny + g2 * nz) - 2.0 * sqrt(g * r * TG) / gm1;
      double ui0 = U[1] / rm, ui1 = U[2] / rm, ui2 = U[3] / rm;
      double uu = ui0 * ui0 + ui1 * ui1 + ui2 * ui2;
      double charI = (ui0 * nx + ui1 * ny + ui2 * nz) + 2.0 * sqrt(g / rm / gm1 * (Em - 0.5 * uu * rm));
      double un0 = 0.5 * nx * (charI + charO), un1 = 0.5 * ny * (charI + charO),
             un2 = 0.5 * nz * (charI + charO);
      double a = 0.25 * gm1 * (charI - charO);
      double ut0, ut1, ut2, ptG, Mach;
      if (un0 * nx + un1 * ny + un2 * nz > 0.0) {
        double sN = nx * ui0 + ny * ui1 + nz * ui2;
        ut0 = ui0 - nx * sN; ut1 = ui1 - ny * sN; ut2 = ui2 - nz * sN;
        Mach = sqrt(uu) / sqrt(g / rm * gm1 * (Em - 0.5 * uu * rm));
        ptG = gm1 * (Em - 0.5 * uu * rm) * pow_pos(1.0 + 0.5 * gm1 * Mach * Mach, g / gm1);
      } else {
        ut0 = g0 - un0; ut1 = g1 - un1; ut2 = g2 - un2;
        Mach = sqrt(g0 * g0 + g1 * g1 + g2 * g2) / sqrt(g * r * TG);
        ptG = pG * pow_pos(1.0 + 0.5 * gm1 * Mach * Mach, g / gm1);
      }
      double u0 = un0 + ut0, u1 = un1 + ut1, u2 = un2 + ut2;
      double q2 = u0 * u0 + u1 * u1 + u2 * u2;
      TG = a * a / g / r;
      Mach = sqrt(q2) / a;
      pG = ptG * pow_pos(1.0 + 0.5 * gm1 * Mach * Mach, -g / gm1);
      double rG = pG / r / TG;
      G[0] = rG; G[1] = rG * u0; G[2] = rG * u1; G[3] = rG * u2;
      G[4] = rG * (1.0 / gm1 * r * TG + 0.5 * q2);
      return;
    }
    default: {  // FOS_BC_WALL: mirror the momentum (foeuler.f90:217-228)
      double dn = U[1] * nx + U[2] * ny + U[3] * nz;
      G[0] = U[0];
      G[1] = U[1] - 2.0 * dn * nx;
      G[2] = U[2] - 2.0 * dn * ny;
      G[3] = U[3] - 2.0 * dn * nz;
      G[4] = U[4];
      return;
    }
  }
}


// ------------------------------------------------------------------ FP64-pipe-free helpers
// GB300 executes FP64 arithmetic and FP64<->FP32 conversions at a small fraction of the FP32
// rate, so the FP32 kernels convert with integer instructions on the IEEE-754 fields.

// binary32 -> binary64 by re-biasing the exponent field (exact for normal numbers and zero;
// binary32 subnormals flush to zero; inf / nan stay inf / nan)
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned long long sgn = (unsigned long long)(b >> 31) << 63;
  const unsigned long long man = (unsigned long long)(b & 0x7fffffu) << 29;
  const unsigned long long e64 = (e == 0xffu) ? 0x7ffull : (unsigned long long)(e + 896u);
  const unsigned long long bits = (e == 0u) ? sgn : (sgn | (e64 << 52) | man);
  return __longlong_as_double((long long)bits);
}

// binary64 -> binary32 keeping the top 23 fraction bits (rounding toward zero); magnitudes
// below the binary32 normal range flush to zero, above it become infinity
__device__ __forceinline__ float d2f_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sgn = (unsigned)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7ffull);
  const unsigned man = (unsigned)((b >> 29) & 0x7fffffull);
  const int e32 = e - 896;
  unsigned bits;
  if (e == 0x7ff) bits = sgn | 0x7f800000u | (man ? 0x400000u : 0u);
  else if (e32 <= 0) bits = sgn;
  else if (e32 >= 255) bits = sgn | 0x7f800000u;
  else bits = sgn | ((unsigned)e32 << 23) | man;
  return __uint_as_float(bits);
}

// x = hi + lo with hi = x's top 24 significand bits (exact) and lo = the rest rounded toward
// zero to 24 bits: one FP64 subtraction, the rest integer instructions
__device__ __forceinline__ void split_hl_bits(double x, float& hi, float& lo) {
  const double xh = __longlong_as_double(__double_as_longlong(x) & ~0x1fffffffll);
  hi = d2f_trunc(xh);
  lo = d2f_trunc(x - xh);
}

// ------------------------------------------------------------------ double-float
// Unevaluated pairs x = h + l of binary32 numbers (|l| <= ulp(h)/2 after normalisation),
// about 2^-46 relative precision, from the error-free transformations of Knuth (TwoSum),
// Dekker (FastTwoSum) and the FMA form of Dekker's TwoProduct -- FP32 instructions only,
// for arithmetic that needs more than FP32 but runs on GB300's full-rate FP32 pipe instead
// of its 1/64-rate FP64 pipe.
struct df2 {
  float h, l;
};
__device__ __forceinline__ df2 df_fast_two_sum(float a, float b) {  // requires |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df2 df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df2 df_add(df2 x, df2 y) {
  const df2 s = df_two_sum(x.h, y.h);
  return df_fast_two_sum(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ df2 df_mul(df2 x, df2 y) {
  const float p = x.h * y.h;
  const float e = fmaf(x.h, y.l, fmaf(x.l, y.h, fmaf(x.h, y.h, -p)));
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ df2 df_scale(df2 x, float k) {  // k a power of two: exact
  return {x.h * k, x.l * k};
}
// 1/x: FP32 reciprocal of the head, one Newton correction r = 1 - x q0 carried in the tail
__device__ __forceinline__ df2 df_rcp(df2 x) {
  const float q0 = __frcp_rn(x.h);
  const float r = fmaf(-x.l, q0, fmaf(-x.h, q0, 1.0f));
  return df_fast_two_sum(q0, q0 * r);
}
// binary64 -> pair, exact to 48 bits: head = top 24 significand bits, tail = the next 24
// (truncated); integer instructions only.  Magnitudes outside [2^-74, 2^127) lose the tail.
__device__ __forceinline__ df2 df_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ffull);
  const unsigned rem = (unsigned)(b & 0x1fffffffull);  // the 29 bits below the head
  const int es = e - 948;  // binary32 exponent field of 2^(e - 1075)
  float l = 0.0f;
  if (rem != 0u && es >= 1 && es <= 254) {
    l = __uint2float_rz(rem) * __uint_as_float((unsigned)es << 23);
    if (b >> 63) l = -l;
  }
  return {d2f_trunc(x), l};
}
// -x by flipping the sign bit (an integer instruction, not the FP64 pipe)
__device__ __forceinline__ double neg_bits(double x) {
  return __hiloint2double(__double2hiint(x) ^ (int)0x80000000u, __double2loint(x));
}
// finiteness from the exponent field of the high word (one 32-bit integer test, no FP64
// compare)
__device__ __forceinline__ bool finite_bits(double x) {
  return ((unsigned)__double2hiint(x) & 0x7ff00000u) != 0x7ff00000u;
}

// 1/a in FP64 by Newton--Raphson iteration x <- x (2 - a x) from an FP32 seed (two steps
// take the ~2^-23 seed error to the FP64 rounding level); four FP64 FMAs
__device__ __forceinline__ double rcp64(double a) {
  double x = f2d_bits(__frcp_rn(d2f_trunc(a)));
  double e = fma(-a, x, 1.0);
  x = fma(x, e, x);
  e = fma(-a, x, 1.0);
  return fma(x, e, x);
}
