// fos_gnn.cu -- learned variable preconditioner: a message-passing graph network over the
// cell-face adjacency, used inside flexible GMRES (no counterpart in the reference).
//
// Model (hidden width H = 64, three message-passing layers; weights stored in BF16 for the
// forward pass, FP32 master copy for training; all sums accumulate in FP32):
//   node input  x_i (16): state / per-field RMS (5), v / per-channel RMS (5), log(v_i/mean v),
//               log of the local CFL number gamma (|u| + c) / v_i^(1/3), padding
//   edge input  e_ij (4): aP n_out / mean aP (3), aP / mean aP
//   h0_i      = bf16(relu(W0 x_i + b0))                                   W0: 64 x 16
//   layer l:   m_i = sum_{j in N(i)} (G_l e_ij + c_l) o h_j               G_l: 64 x 4
//              h_i <- bf16(relu(A_l [h_i ; bf16(m_i)] + b_l))             A_l: 64 x 128
//   output     z_i = s_v o (v_i / s_v + D h3_i + d)                        D: 5 x 64
// so an untrained network (D = 0) is the identity preconditioner.  The node products
// A_l [h; m] (forward) and A_l^T delta (backward) run on the tensor cores as
// mma.sync m16n8k16 BF16 x BF16 -> FP32; weight gradients are reduced per CTA and then
// across CTAs in a fixed order (deterministic, no floating-point atomics).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "fos_internal.h"
#include "fos_device.cuh"

namespace {

constexpr int H = 64;
constexpr int NIN = 16;
constexpr int NL = 3;
constexpr int NOUT = 8;  // 5 used
// parameter offsets (floats)
constexpr int OFF_W0 = 0;
constexpr int OFF_B0 = OFF_W0 + H * NIN;
constexpr int OFF_L0 = OFF_B0 + H;
constexpr int L_G = 0, L_C = H * 4, L_A = L_C + H, L_B = L_A + H * 2 * H, L_SIZE = L_B + H;
constexpr int OFF_D = OFF_L0 + NL * L_SIZE;
constexpr int OFF_DB = OFF_D + NOUT * H;
constexpr int NPARAM = OFF_DB + NOUT;

constexpr int kT = 128;    // 4 warps
constexpr int kTile = 64;  // cells per CTA tile

__device__ __forceinline__ unsigned short bf(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float fb(unsigned short b) {
  return __bfloat162float(__ushort_as_bfloat16(b));
}
__device__ __forceinline__ unsigned pack2(unsigned short lo, unsigned short hi) {
  return (unsigned)lo | ((unsigned)hi << 16);
}

__device__ __forceinline__ void mma16816(float c[4], const unsigned a[4], const unsigned b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Fragments of a row-major A tile (element (r, k) at A[r * lda + k]) and of a B tile given
// as element (k, n) at B[k * sk + n * sn]; both in shared memory as BF16 bits.
// (lda and k0 even, A 4-byte aligned: each register is one 32-bit shared load)
__device__ __forceinline__ void load_a(const unsigned short* A, int lda, int r0, int k0,
                                       unsigned a[4]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  const unsigned* p0 = reinterpret_cast<const unsigned*>(A + (r0 + g) * lda + k0 + 2 * t);
  const unsigned* p1 = reinterpret_cast<const unsigned*>(A + (r0 + g + 8) * lda + k0 + 2 * t);
  a[0] = p0[0];
  a[1] = p1[0];
  a[2] = p0[4];
  a[3] = p1[4];
}
// B fragment when k is contiguous: element (k, n) at B[n * ldn + k] (ldn, k0 even)
__device__ __forceinline__ void load_b_kc(const unsigned short* B, int ldn, int k0, int n0,
                                          unsigned b[2]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  const unsigned* p = reinterpret_cast<const unsigned*>(B + (n0 + g) * ldn + k0 + 2 * t);
  b[0] = p[0];
  b[1] = p[4];
}
__device__ __forceinline__ void load_b(const unsigned short* B, int sk, int sn, int k0, int n0,
                                       unsigned b[2]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  const unsigned short* p = B + (k0 + 2 * t) * sk + (n0 + g) * sn;
  b[0] = pack2(p[0], p[sk]);
  b[1] = pack2(p[8 * sk], p[9 * sk]);
}

struct GnnScales {
  float sy[3];   // rho, |rho u|, rho E  RMS
  float sv[5];   // per-channel RMS of v
  float amean;   // mean face area
  float lvmean;  // mean log volume
};

// gate of edge (i <- j) for features f0, f0+1: G e + c with e = (aP n_out(i), aP)/amean
__device__ __forceinline__ void gate2(const float* __restrict__ Gc, float ex, float ey, float ez,
                                      float ea, int f0, float& g0, float& g1) {
  const float* G = Gc;           // 64 x 4
  const float* cc = Gc + H * 4;  // 64
  g0 = cc[f0] + G[4 * f0] * ex + G[4 * f0 + 1] * ey + G[4 * f0 + 2] * ez + G[4 * f0 + 3] * ea;
  g1 = cc[f0 + 1] + G[4 * f0 + 4] * ex + G[4 * f0 + 5] * ey + G[4 * f0 + 6] * ez +
       G[4 * f0 + 7] * ea;
}

// ------------------------------------------------------------------ forward
// Input layer, 256 cells per CTA.  Phase 1: thread per cell computes the 16 features into
// shared memory.  Phase 2: a warp per cell, lane l owns hidden channels 2l, 2l+1 with its
// two rows of W0 (and b0) in registers as pairs: 16 packed FMAs per cell and lane, and the
// BF16 row of h0 leaves as one coalesced 128-byte store.
__global__ void __launch_bounds__(256) k_gnn_in(int nC, const double* __restrict__ y,
                                                const double* __restrict__ v,
                                                const double* __restrict__ invV, float gam_dt,
                                                float gas_g,
                                                const float* __restrict__ Wb,  // bf16-rounded FP32
                                                const GnnScales* __restrict__ sc,
                                                float* __restrict__ X0,
                                                unsigned short* __restrict__ h0) {
  __shared__ __align__(16) float xs[256][NIN];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int f0 = 2 * lane;
  float2 w[NIN];
#pragma unroll
  for (int k = 0; k < NIN; k++) w[k] = make_float2(Wb[OFF_W0 + NIN * f0 + k], Wb[OFF_W0 + NIN * (f0 + 1) + k]);
  const float2 bias = make_float2(Wb[OFF_B0 + f0], Wb[OFF_B0 + f0 + 1]);
  const int nchunk = (nC + 255) / 256;
  for (int chunk = blockIdx.x; chunk < nchunk; chunk += gridDim.x) {  // persistent
  const int c0 = chunk * 256;
  __syncthreads();  // the previous chunk's features are consumed
  {
    const int i = c0 + threadIdx.x;
    float x[NIN];
#pragma unroll
    for (int k = 0; k < NIN; k++) x[k] = 0.0f;
    if (i < nC) {
      const GnnScales s = *sc;
      x[0] = d2f_trunc(y[i]) / s.sy[0];
      x[1] = d2f_trunc(y[(size_t)nC + i]) / s.sy[1];
      x[2] = d2f_trunc(y[2 * (size_t)nC + i]) / s.sy[1];
      x[3] = d2f_trunc(y[3 * (size_t)nC + i]) / s.sy[1];
      x[4] = d2f_trunc(y[4 * (size_t)nC + i]) / s.sy[2];
#pragma unroll
      for (int q = 0; q < 5; q++) x[5 + q] = d2f_trunc(v[(size_t)q * nC + i]) / s.sv[q];
      const float iv = d2f_trunc(invV[i]);
      x[10] = -logf(iv) - s.lvmean;
      const float r = d2f_trunc(y[i]);
      const float mx = d2f_trunc(y[(size_t)nC + i]), my = d2f_trunc(y[2 * (size_t)nC + i]),
                  mz = d2f_trunc(y[3 * (size_t)nC + i]), E = d2f_trunc(y[4 * (size_t)nC + i]);
      const float q2 = (mx * mx + my * my + mz * mz) / (r * r);
      const float p = (gas_g - 1.0f) * (E - 0.5f * r * q2);
      const float cs = sqrtf(fmaxf(gas_g * p / r, 0.0f));
      const float cfl = gam_dt * (sqrtf(q2) + cs) * cbrtf(iv);
      x[11] = logf(fmaxf(cfl, 1e-12f));
      if (X0) {
        float4* xo = reinterpret_cast<float4*>(X0 + (size_t)NIN * i);
#pragma unroll
        for (int k = 0; k < NIN / 4; k++) xo[k] = make_float4(x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3]);
      }
    }
#pragma unroll
    for (int k = 0; k < NIN / 4; k++)
      *reinterpret_cast<float4*>(&xs[threadIdx.x][4 * k]) =
          make_float4(x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3]);
  }
  __syncthreads();
  // four cells per step (rows r0, r0 + 8, r0 + 16, r0 + 24): independent FMA chains
  constexpr int U = 4;
  for (int r0 = warp; r0 < 256; r0 += 8 * U) {
    float2 a[U];
#pragma unroll
    for (int u = 0; u < U; u++) a[u] = bias;
#pragma unroll
    for (int k4 = 0; k4 < NIN / 4; k4++) {
#pragma unroll
      for (int u = 0; u < U; u++) {
        const float4 xv = *reinterpret_cast<const float4*>(&xs[r0 + 8 * u][4 * k4]);
        a[u] = __ffma2_rn(w[4 * k4 + 0], make_float2(xv.x, xv.x), a[u]);
        a[u] = __ffma2_rn(w[4 * k4 + 1], make_float2(xv.y, xv.y), a[u]);
        a[u] = __ffma2_rn(w[4 * k4 + 2], make_float2(xv.z, xv.z), a[u]);
        a[u] = __ffma2_rn(w[4 * k4 + 3], make_float2(xv.w, xv.w), a[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int i = c0 + r0 + 8 * u;
      if (i < nC)
        reinterpret_cast<unsigned*>(h0 + (size_t)H * i)[lane] =
            pack2(bf(fmaxf(a[u].x, 0.0f)), bf(fmaxf(a[u].y, 0.0f)));
    }
  }
  }
}

// edge features of ELL entry ent seen from cell i; returns the neighbour cell or -1
__device__ __forceinline__ int edge_of(int ent, const int2* __restrict__ faceLR, int nFi,
                                       const float4* __restrict__ faceNA, float inv_amean,
                                       float& ex, float& ey, float& ez, float& ea) {
  if (ent < 0) return -1;
  const int f = ent >> 1;
  if (f >= nFi) return -1;  // boundary face: no neighbour
  const int2 lr = faceLR[f];
  const float4 na = faceNA[f];
  const float sgn = (ent & 1) ? -1.0f : 1.0f;  // cell is R: outward normal is -n
  const float a = na.w * inv_amean;
  ex = sgn * na.x * a;
  ey = sgn * na.y * a;
  ez = sgn * na.z * a;
  ea = a;
  return (ent & 1) ? lr.x : lr.y;
}

// One message-passing layer, persistent over tiles of 64 cells (128 threads):
//   A. edge phase: the 256 (cell, ELL slot) pairs of the tile -> neighbour index and edge
//      features in shared memory (all independent loads, one pass);
//   B. gather + gate (CUDA cores, FP32): warp w takes cells w, w+4, ..., four cells per
//      step, so 20 rows of h (128 B each) are in flight per warp;
//   C. [h; bf16(m)] A^T on the tensor cores (mma.sync m16n8k16, BF16 in, FP32 accumulate);
//   D. bias + relu -> BF16 into the warp's own rows of the tile, then coalesced 16-byte stores.
// The layer weights are loaded once per CTA.  HEAD (last layer) also applies the output
// head z = s_v (v / s_v + D h3 + d) from the tile in shared memory, so h3 is stored only
// when training keeps it.  Optionally keeps bf16(m) for the backward pass.
template <bool HEAD>
__global__ void __launch_bounds__(kT) k_gnn_layer(
    int nC, int nFi, const int* __restrict__ ell, const int2* __restrict__ faceLR,
    const float4* __restrict__ faceNA, const GnnScales* __restrict__ sc,
    const float* __restrict__ Wl,            // layer block of the bf16-rounded FP32 weights
    const unsigned short* __restrict__ Ab,   // layer A in BF16 bits, 64 x 128 row-major
    const unsigned short* __restrict__ hin, unsigned short* __restrict__ hout,
    unsigned short* __restrict__ mkeep, const float* __restrict__ Wb,
    const double* __restrict__ v, double* __restrict__ z, float* __restrict__ zhat) {
  constexpr int RS = 2 * H + 8;  // row stride (bf16) of the tiles: 272 B, 16-byte aligned
  __shared__ __align__(16) unsigned short Xs[kTile][RS];   // [h ; m], then the layer output
  __shared__ __align__(16) unsigned short As[H][RS];
  __shared__ float bs[H];
  __shared__ __align__(16) int nbr[kTile][4];
  __shared__ float4 ef[kTile][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  for (int k = threadIdx.x; k < H * (2 * H / 8); k += kT) {
    const int r = k / (2 * H / 8), c = k % (2 * H / 8);
    *reinterpret_cast<uint4*>(&As[r][8 * c]) = reinterpret_cast<const uint4*>(Ab)[k];
  }
  for (int k = threadIdx.x; k < H; k += kT) bs[k] = Wl[L_B + k];
  const GnnScales s = *sc;
  const float inv_amean = 1.0f / s.amean;
  const int f0 = 2 * lane;
  // the lane's gate rows G[f0], G[f0 + 1] and c[f0], c[f0 + 1] in registers, as pairs
  const float2 gx = make_float2(Wl[L_G + 4 * f0 + 0], Wl[L_G + 4 * f0 + 4]);
  const float2 gy = make_float2(Wl[L_G + 4 * f0 + 1], Wl[L_G + 4 * f0 + 5]);
  const float2 gz = make_float2(Wl[L_G + 4 * f0 + 2], Wl[L_G + 4 * f0 + 6]);
  const float2 ga = make_float2(Wl[L_G + 4 * f0 + 3], Wl[L_G + 4 * f0 + 7]);
  const float2 gc = make_float2(Wl[L_C + f0], Wl[L_C + f0 + 1]);
  // output head (last layer): B fragments of D^T (k = hidden channel, n = field) and d
  unsigned dfr[4][2] = {{0u, 0u}, {0u, 0u}, {0u, 0u}, {0u, 0u}};
  float dq[2] = {0.0f, 0.0f};
  if (HEAD) {
    const int n = g;  // field of this lane's B column
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      const int k0 = 16 * kk + 2 * t;
      auto w = [&](int k) { return n < 5 ? bf(Wb[OFF_D + H * n + k]) : (unsigned short)0; };
      dfr[kk][0] = pack2(w(k0), w(k0 + 1));
      dfr[kk][1] = pack2(w(k0 + 8), w(k0 + 9));
    }
    dq[0] = 2 * t < 5 ? Wb[OFF_DB + 2 * t] : 0.0f;
    dq[1] = 2 * t + 1 < 5 ? Wb[OFF_DB + 2 * t + 1] : 0.0f;
  }
  const int ntiles = (nC + kTile - 1) / kTile;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c0 = tile * kTile;
    // A. edges of the tile
    for (int p = threadIdx.x; p < kTile * 4; p += kT) {
      const int r = p >> 2, k = p & 3, i = c0 + r;
      int j = -1;
      float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (i < nC) {
        float ex, ey, ez, ea;
        j = edge_of(ell[4 * (size_t)i + k], faceLR, nFi, faceNA, inv_amean, ex, ey, ez, ea);
        if (j >= 0) e = make_float4(ex, ey, ez, ea);
      }
      nbr[r][k] = j;
      ef[r][k] = e;
    }
    __syncthreads();  // edges ready; the previous tile's output rows are stored
    // B. gather + gate, four cells per step; gate and message as packed FP32 FMAs
    //    (missing neighbours contribute (c + 0) * 0, which leaves the sum unchanged)
    constexpr int U = 4;
    for (int r0 = warp; r0 < kTile; r0 += 4 * U) {
      unsigned hv[U][4], hs[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int r = r0 + 4 * u, i = c0 + r;
        const int4 nb = *reinterpret_cast<const int4*>(&nbr[r][0]);
        const int js[4] = {nb.x, nb.y, nb.z, nb.w};
        hs[u] = i < nC ? reinterpret_cast<const unsigned*>(hin + (size_t)H * i)[lane] : 0u;
#pragma unroll
        for (int k = 0; k < 4; k++)
          hv[u][k] = js[k] >= 0 ? reinterpret_cast<const unsigned*>(hin + (size_t)H * js[k])[lane] : 0u;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int r = r0 + 4 * u, i = c0 + r;
        float2 m = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float4 e = ef[r][k];
          float2 gg = __ffma2_rn(gx, make_float2(e.x, e.x), gc);
          gg = __ffma2_rn(gy, make_float2(e.y, e.y), gg);
          gg = __ffma2_rn(gz, make_float2(e.z, e.z), gg);
          gg = __ffma2_rn(ga, make_float2(e.w, e.w), gg);
          const unsigned hb = hv[u][k];
          m = __ffma2_rn(gg, make_float2(__uint_as_float(hb << 16), __uint_as_float(hb & 0xffff0000u)), m);
        }
        const unsigned ms = pack2(bf(m.x), bf(m.y));
        if (mkeep && i < nC) reinterpret_cast<unsigned*>(mkeep + (size_t)H * i)[lane] = ms;
        reinterpret_cast<unsigned*>(&Xs[r][0])[lane] = hs[u];
        reinterpret_cast<unsigned*>(&Xs[r][H])[lane] = ms;
      }
    }
    __syncthreads();
    // C. tensor cores: rows 16*warp .. +15 of the tile, all 64 outputs, K = 128
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[nt][q] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 2 * H; kk += 16) {
      unsigned a[4];
      load_a(&Xs[0][0], RS, 16 * warp, kk, a);
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        unsigned b[2];
        // B(k, n) = A_l(n, k): k contiguous along the rows of As
        load_b_kc(&As[0][0], RS, kk, 8 * nt, b);
        mma16816(acc[nt], a, b);
      }
    }
    // D. bias + relu -> BF16.  The m16n8 accumulator layout of output columns 16 kk .. +15
    //    is the A-fragment layout of k-chunk kk, so the head runs from registers.
    unsigned ob[8][2];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = 8 * nt + 2 * t;
      ob[nt][0] = pack2(bf(fmaxf(acc[nt][0] + bs[col], 0.0f)), bf(fmaxf(acc[nt][1] + bs[col + 1], 0.0f)));
      ob[nt][1] = pack2(bf(fmaxf(acc[nt][2] + bs[col], 0.0f)), bf(fmaxf(acc[nt][3] + bs[col + 1], 0.0f)));
    }
    if (hout) {  // stage the warp's own rows (no other warp reads them in this tile)
      __syncwarp();
      const int ra = 16 * warp + g, rb = ra + 8;
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const int col = 8 * nt + 2 * t;
        *reinterpret_cast<unsigned*>(&Xs[ra][col]) = ob[nt][0];
        *reinterpret_cast<unsigned*>(&Xs[rb][col]) = ob[nt][1];
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int idx = lane + 32 * q, row = idx >> 3, chunk = idx & 7;
        const int i = c0 + 16 * warp + row;
        if (i < nC)
          reinterpret_cast<uint4*>(hout + (size_t)H * i)[chunk] =
              *reinterpret_cast<const uint4*>(&Xs[16 * warp + row][8 * chunk]);
      }
    }
    if (HEAD) {  // zhat = v / s_v + D h3 + d on the tensor cores (fields 0-4 of n = 8)
      float o[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int kk = 0; kk < 4; kk++) {
        const unsigned a[4] = {ob[2 * kk][0], ob[2 * kk][1], ob[2 * kk + 1][0], ob[2 * kk + 1][1]};
        mma16816(o, a, dfr[kk]);
      }
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int q = 2 * t + (e & 1);
        const int i = c0 + 16 * warp + g + ((e & 2) ? 8 : 0);
        if (q < 5 && i < nC) {
          const float svq = sc->sv[q];
          const float zh = d2f_trunc(v[(size_t)q * nC + i]) / svq + (o[e] + dq[e & 1]);
          if (zhat) zhat[(size_t)8 * i + q] = zh;
          if (z) z[(size_t)q * nC + i] = f2d_bits(zh * svq);
        }
      }
    }
  }
}

// ------------------------------------------------------------------ scales
__device__ __forceinline__ float warp_sumf(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
// partial sums of squares: y fields (rho, |m|^2, E), v channels (5), log volume, area
__global__ void __launch_bounds__(256) k_gnn_scale_part(int nC, int nF, const double* __restrict__ y,
                                                        const double* __restrict__ v,
                                                        const double* __restrict__ invV,
                                                        const float4* __restrict__ faceNA,
                                                        float* __restrict__ part) {
  float acc[10] = {0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nC; i += gridDim.x * blockDim.x) {
    const float r = d2f_trunc(y[i]);
    const float mx = d2f_trunc(y[(size_t)nC + i]), my = d2f_trunc(y[2 * (size_t)nC + i]),
                mz = d2f_trunc(y[3 * (size_t)nC + i]);
    const float E = d2f_trunc(y[4 * (size_t)nC + i]);
    acc[0] += r * r;
    acc[1] += mx * mx + my * my + mz * mz;
    acc[2] += E * E;
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const float vq = d2f_trunc(v[(size_t)q * nC + i]);
      acc[3 + q] += vq * vq;
    }
    acc[8] += -logf(d2f_trunc(invV[i]));
  }
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x)
    acc[9] += faceNA[f].w;
  __shared__ float sh[8][10];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 10; k++) {
    const float s = warp_sumf(acc[k]);
    if (lane == 0) sh[w][k] = s;
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    float s = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k][threadIdx.x];
    part[10 * blockIdx.x + threadIdx.x] = s;
  }
}
__global__ void k_gnn_scale_final(int nC, int nF, int np, const float* __restrict__ part,
                                  GnnScales* __restrict__ sc) {
  // one warp: lane l sums partials l, l+32, ... (fixed order), then a shuffle tree
  const int lane = threadIdx.x & 31;
  float s[10] = {0};
  for (int b = lane; b < np; b += 32)
#pragma unroll
    for (int k = 0; k < 10; k++) s[k] += part[10 * b + k];
#pragma unroll
  for (int k = 0; k < 10; k++) s[k] = warp_sumf(s[k]);
  if (lane != 0) return;
  const float tiny = 1e-30f;
  GnnScales o;
  o.sy[0] = sqrtf(s[0] / nC) + tiny;
  o.sy[1] = sqrtf(s[1] / (3.0f * nC)) + 1e-6f * o.sy[0];
  o.sy[2] = sqrtf(s[2] / nC) + tiny;
  float vmax = 0.0f;
  for (int q = 0; q < 5; q++) vmax = fmaxf(vmax, sqrtf(s[3 + q] / nC));
  for (int q = 0; q < 5; q++) o.sv[q] = sqrtf(s[3 + q] / nC) + 1e-6f * vmax + tiny;
  o.lvmean = s[8] / nC;
  o.amean = s[9] / nF;
  *sc = o;
}

// ------------------------------------------------------------------ backward
// loss and head backward: dz = 2 (zhat - t)/N; dh3 = D^T dz (FP32), dD/dd partials
__global__ void __launch_bounds__(256) k_gnn_out_bwd(int nC, const float* __restrict__ zhat,
                                                     const double* __restrict__ t,
                                                     const GnnScales* __restrict__ sc,
                                                     const unsigned short* __restrict__ h3,
                                                     const float* __restrict__ Wb, float invN,
                                                     float* __restrict__ dh3,
                                                     float* __restrict__ part) {
  // part layout per block: [0] loss, [1..5] dd, [6 .. 6+5*64) dD
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const GnnScales s = *sc;
  const int lane = threadIdx.x & 31;
  float dz[5] = {0, 0, 0, 0, 0}, loss = 0.0f;
  float h[H];
  if (i < nC) {
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const float th = d2f_trunc(t[(size_t)q * nC + i]) / s.sv[q];
      const float e = zhat[(size_t)8 * i + q] - th;
      loss += e * e;
      dz[q] = 2.0f * e * invN;
    }
    const uint4* src = reinterpret_cast<const uint4*>(h3 + (size_t)H * i);
#pragma unroll
    for (int k = 0; k < H / 8; k++) {
      const uint4 u = src[k];
      const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        h[8 * k + 2 * q] = fb((unsigned short)(w[q] & 0xffff));
        h[8 * k + 2 * q + 1] = fb((unsigned short)(w[q] >> 16));
      }
    }
    const float* D = Wb + OFF_D;
    float4* out = reinterpret_cast<float4*>(dh3 + (size_t)H * i);
#pragma unroll
    for (int k = 0; k < H / 4; k++) {
      float o[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int f = 4 * k + u;
        o[u] = D[f] * dz[0] + D[H + f] * dz[1] + D[2 * H + f] * dz[2] + D[3 * H + f] * dz[3] +
               D[4 * H + f] * dz[4];
      }
      out[k] = make_float4(o[0], o[1], o[2], o[3]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < H; k++) h[k] = 0.0f;
  }
  // per-warp sums, then a fixed-order sum over the warps of the CTA
  __shared__ float wsum[8][1 + 5 + 5 * H];
  const int w = threadIdx.x >> 5;
  for (int q = 0; q < 5; q++) {
    const float a = warp_sumf(dz[q]);
    if (lane == 0) wsum[w][1 + q] = a;
  }
  const float lw = warp_sumf(loss);
  if (lane == 0) wsum[w][0] = lw;
  for (int q = 0; q < 5; q++)
    for (int f = 0; f < H; f++) {
      const float a = warp_sumf(dz[q] * h[f]);
      if (lane == 0) wsum[w][6 + q * H + f] = a;
    }
  __syncthreads();
  for (int k = threadIdx.x; k < 1 + 5 + 5 * H; k += blockDim.x) {
    float a = 0.0f;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) a += wsum[ww][k];
    part[(size_t)(1 + 5 + 5 * H) * blockIdx.x + k] = a;
  }
}

// Layer backward, part 1 (tile of 64 cells, persistent over tiles):
//   delta = dh_out o (h_out > 0);  dX = delta A_l (tensor cores) -> dh_in (direct), dm
//   dA_l += delta^T X and db += sum delta, per CTA (tensor cores / FP32), one partial per CTA
__global__ void __launch_bounds__(kT) k_gnn_layer_bwd(
    int nC, const unsigned short* __restrict__ hin, const unsigned short* __restrict__ mkeep,
    const unsigned short* __restrict__ hout, const float* __restrict__ dhout,
    const unsigned short* __restrict__ Ab, float* __restrict__ dhin, float* __restrict__ dm,
    float* __restrict__ part) {
  __shared__ __align__(16) unsigned short Xs[kTile][2 * H + 8];   // [h_in ; m] rows
  __shared__ __align__(16) unsigned short Ds[kTile][H + 8];       // bf16(delta) rows
  __shared__ __align__(16) unsigned short As[H][2 * H + 8];
  __shared__ float dbs[kT / 32][H];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tq = lane & 3;
  for (int k = threadIdx.x; k < H * 2 * H; k += kT) As[k / (2 * H)][k % (2 * H)] = Ab[k];
  // dA accumulators: warp owns output rows 16*warp .. +15 (of 64), all 128 inputs
  float dA[16][4];
#pragma unroll
  for (int nt = 0; nt < 16; nt++)
#pragma unroll
    for (int q = 0; q < 4; q++) dA[nt][q] = 0.0f;
  float db0 = 0.0f, db1 = 0.0f;
  const int ntiles = (nC + kTile - 1) / kTile;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c0 = tile * kTile;
    __syncthreads();
    for (int r = warp; r < kTile; r += kT / 32) {
      const int i = c0 + r;
      unsigned hx = 0, mx = 0, dd = 0;
      if (i < nC) {
        hx = reinterpret_cast<const unsigned*>(hin + (size_t)H * i)[lane];
        mx = reinterpret_cast<const unsigned*>(mkeep + (size_t)H * i)[lane];
        const unsigned ho = reinterpret_cast<const unsigned*>(hout + (size_t)H * i)[lane];
        const float2 dh = reinterpret_cast<const float2*>(dhout + (size_t)H * i)[lane];
        const float d0 = fb((unsigned short)(ho & 0xffff)) > 0.0f ? dh.x : 0.0f;
        const float d1 = fb((unsigned short)(ho >> 16)) > 0.0f ? dh.y : 0.0f;
        db0 += d0;
        db1 += d1;
        dd = pack2(bf(d0), bf(d1));
      }
      reinterpret_cast<unsigned*>(&Xs[r][0])[lane] = hx;
      reinterpret_cast<unsigned*>(&Xs[r][H])[lane] = mx;
      reinterpret_cast<unsigned*>(&Ds[r][0])[lane] = dd;
    }
    __syncthreads();
    // dX (64 x 128) = delta (64 x 64) A_l (64 x 128); warp: rows 16*warp, all 128 cols
    {
      float acc[16][4];
#pragma unroll
      for (int nt = 0; nt < 16; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[nt][q] = 0.0f;
#pragma unroll
      for (int kk = 0; kk < H; kk += 16) {
        unsigned a[4];
        load_a(&Ds[0][0], H + 8, 16 * warp, kk, a);
#pragma unroll
        for (int nt = 0; nt < 16; nt++) {
          unsigned b[2];
          load_b(&As[0][0], 2 * H + 8, 1, kk, 8 * nt, b);  // B(k, n) = A_l(k, n)
          mma16816(acc[nt], a, b);
        }
      }
#pragma unroll
      for (int nt = 0; nt < 16; nt++) {
        const int col = 8 * nt + 2 * tq;
        const int ra = c0 + 16 * warp + g, rb = ra + 8;
        float* dst = col < H ? dhin : dm;
        const int cc = col < H ? col : col - H;
        if (ra < nC) reinterpret_cast<float2*>(dst + (size_t)H * ra)[cc / 2] = make_float2(acc[nt][0], acc[nt][1]);
        if (rb < nC) reinterpret_cast<float2*>(dst + (size_t)H * rb)[cc / 2] = make_float2(acc[nt][2], acc[nt][3]);
      }
    }
    // dA (64 x 128) += delta^T (64 x tile) X (tile x 128); warp: rows 16*warp
#pragma unroll
    for (int kk = 0; kk < kTile; kk += 16) {
      unsigned a[4];
      {
        // A(r, k) = delta^T(r, k) = Ds[k][r]
        const unsigned short* p0 = &Ds[kk + 2 * tq][16 * warp + g];
        a[0] = pack2(p0[0], p0[H + 8]);
        a[1] = pack2(p0[8], p0[H + 8 + 8]);
        a[2] = pack2(p0[8 * (H + 8)], p0[9 * (H + 8)]);
        a[3] = pack2(p0[8 * (H + 8) + 8], p0[9 * (H + 8) + 8]);
      }
#pragma unroll
      for (int nt = 0; nt < 16; nt++) {
        unsigned b[2];
        load_b(&Xs[0][0], 2 * H + 8, 1, kk, 8 * nt, b);  // B(k, n) = X(k, n)
        mma16816(dA[nt], a, b);
      }
    }
  }
  // write the per-CTA partials: [dA 64x128][db 64]
  float* P = part + (size_t)(H * 2 * H + H) * blockIdx.x;
#pragma unroll
  for (int nt = 0; nt < 16; nt++) {
    const int col = 8 * nt + 2 * tq;
    const int ra = 16 * warp + g, rb = ra + 8;
    P[2 * H * ra + col] = dA[nt][0];
    P[2 * H * ra + col + 1] = dA[nt][1];
    P[2 * H * rb + col] = dA[nt][2];
    P[2 * H * rb + col + 1] = dA[nt][3];
  }
  dbs[warp][2 * lane] = db0;
  dbs[warp][2 * lane + 1] = db1;
  __syncthreads();
  if (threadIdx.x < H) {
    float s = 0.0f;
    for (int w = 0; w < kT / 32; w++) s += dbs[w][threadIdx.x];
    P[H * 2 * H + threadIdx.x] = s;
  }
}

// Layer backward, part 2 (warp per cell j): through the message sums
//   dh_in_j += sum_{i in N(j)} g_ij o dm_i ;  dG += dm_i o h_j (x) e_ij ;  dc += dm_i o h_j
// where g_ij, e_ij are edge (i <- j) seen from i (outward normal of i = -that of j).
__global__ void __launch_bounds__(kT) k_gnn_edge_bwd(
    int nC, int nFi, const int* __restrict__ ell, const int2* __restrict__ faceLR,
    const float4* __restrict__ faceNA, const GnnScales* __restrict__ sc,
    const float* __restrict__ Wl, const unsigned short* __restrict__ hin,
    const float* __restrict__ dm, float* __restrict__ dhin, float* __restrict__ part) {
  __shared__ float Gs[H * 5];
  __shared__ float acc_s[kT / 32][H * 5];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < H * 5; k += kT) Gs[k] = Wl[L_G + k];
  __syncthreads();
  const float inv_amean = 1.0f / sc->amean;
  const int f0 = 2 * lane;
  float aG[2][5] = {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}};  // per feature: dG (4) and dc
  const int nw = gridDim.x * (kT / 32);
  for (int j = blockIdx.x * (kT / 32) + warp; j < nC; j += nw) {
    const unsigned hj = reinterpret_cast<const unsigned*>(hin + (size_t)H * j)[lane];
    const float h0 = fb((unsigned short)(hj & 0xffff)), h1 = fb((unsigned short)(hj >> 16));
    const int4 e4 = reinterpret_cast<const int4*>(ell)[j];
    const int ents[4] = {e4.x, e4.y, e4.z, e4.w};
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      float ex, ey, ez, ea;
      const int i = edge_of(ents[k], faceLR, nFi, faceNA, inv_amean, ex, ey, ez, ea);
      if (i < 0) continue;
      ex = -ex; ey = -ey; ez = -ez;  // edge (i <- j) seen from i
      float g0, g1;
      gate2(Gs, ex, ey, ez, ea, f0, g0, g1);
      const float2 d = reinterpret_cast<const float2*>(dm + (size_t)H * i)[lane];
      s0 += g0 * d.x;
      s1 += g1 * d.y;
      const float p0 = d.x * h0, p1 = d.y * h1;
      aG[0][0] += p0 * ex; aG[0][1] += p0 * ey; aG[0][2] += p0 * ez; aG[0][3] += p0 * ea; aG[0][4] += p0;
      aG[1][0] += p1 * ex; aG[1][1] += p1 * ey; aG[1][2] += p1 * ez; aG[1][3] += p1 * ea; aG[1][4] += p1;
    }
    float2* dst = reinterpret_cast<float2*>(dhin + (size_t)H * j) + lane;
    const float2 cur = *dst;
    *dst = make_float2(cur.x + s0, cur.y + s1);
  }
  // per-warp values into shared memory, then a fixed-order sum per CTA
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const int f = f0 + u;
#pragma unroll
    for (int k = 0; k < 4; k++) acc_s[warp][4 * f + k] = aG[u][k];
    acc_s[warp][H * 4 + f] = aG[u][4];
  }
  __syncthreads();
  float* P = part + (size_t)(H * 5) * blockIdx.x;
  for (int k = threadIdx.x; k < H * 5; k += kT) {
    float s = 0.0f;
    for (int w = 0; w < kT / 32; w++) s += acc_s[w][k];
    P[k] = s;
  }
}

// input layer backward: delta0 = dh0 o (h0 > 0); dW0 += delta0 x^T, db0 += delta0
__global__ void __launch_bounds__(256) k_gnn_in_bwd(int nC, const float* __restrict__ X0,
                                                    const unsigned short* __restrict__ h0,
                                                    const float* __restrict__ dh0,
                                                    float* __restrict__ part) {
  __shared__ float red[8][H * NIN + H];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // warp per cell: lane owns features 2 lane, 2 lane + 1
  float acc[2][NIN + 1];
#pragma unroll
  for (int u = 0; u < 2; u++)
#pragma unroll
    for (int k = 0; k <= NIN; k++) acc[u][k] = 0.0f;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int i = blockIdx.x * (blockDim.x >> 5) + w; i < nC; i += nw) {
    const unsigned hh = reinterpret_cast<const unsigned*>(h0 + (size_t)H * i)[lane];
    const float2 d = reinterpret_cast<const float2*>(dh0 + (size_t)H * i)[lane];
    const float d0 = fb((unsigned short)(hh & 0xffff)) > 0.0f ? d.x : 0.0f;
    const float d1 = fb((unsigned short)(hh >> 16)) > 0.0f ? d.y : 0.0f;
    const float* x = X0 + (size_t)NIN * i;
#pragma unroll
    for (int k = 0; k < NIN; k++) {
      const float xk = x[k];
      acc[0][k] += d0 * xk;
      acc[1][k] += d1 * xk;
    }
    acc[0][NIN] += d0;
    acc[1][NIN] += d1;
  }
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const int f = 2 * lane + u;
#pragma unroll
    for (int k = 0; k < NIN; k++) red[w][NIN * f + k] = acc[u][k];
    red[w][H * NIN + f] = acc[u][NIN];
  }
  __syncthreads();
  float* P = part + (size_t)(H * NIN + H) * blockIdx.x;
  for (int k = threadIdx.x; k < H * NIN + H; k += blockDim.x) {
    float s = 0.0f;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) s += red[ww][k];
    P[k] = s;
  }
}

// [loss, dd(5), dD(5 x 64)] -> gradient of d and of the first five rows of D
__global__ void k_gnn_head_grad(const float* __restrict__ hs, float* __restrict__ grad) {
  for (int k = threadIdx.x; k < 5 + 5 * H; k += blockDim.x) {
    if (k < 5) grad[OFF_DB + k] += hs[1 + k];
    else grad[OFF_D + (k - 5)] += hs[1 + k];
  }
}

// sum np partial vectors of length len (fixed order) into dst (+= when accumulate)
__global__ void k_sum_parts(int np, int len, const float* __restrict__ part,
                            float* __restrict__ dst, float scale) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= len) return;
  float s = 0.0f;
  for (int b = 0; b < np; b++) s += part[(size_t)len * b + k];
  dst[k] += scale * s;
}

// Adam on the FP32 master weights, then the bf16-rounded FP32 and BF16 copies
__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ gr,
                       float* __restrict__ m1, float* __restrict__ m2, float lr, float b1,
                       float b2, float eps, float c1, float c2, float* __restrict__ wb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float g = gr[k];
  const float a = b1 * m1[k] + (1.0f - b1) * g;
  const float b = b2 * m2[k] + (1.0f - b2) * g * g;
  m1[k] = a;
  m2[k] = b;
  const float nw = w[k] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  w[k] = nw;
  wb[k] = __bfloat162float(__float2bfloat16_rn(nw));
}
__global__ void k_round_bf16(int n, const float* __restrict__ w, float* __restrict__ wb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) wb[k] = __bfloat162float(__float2bfloat16_rn(w[k]));
}
__global__ void k_layer_bits(const float* __restrict__ wb, unsigned short* __restrict__ Ab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= NL * H * 2 * H) return;
  const int l = k / (H * 2 * H), r = k % (H * 2 * H);
  Ab[k] = bf(wb[OFF_L0 + l * L_SIZE + L_A + r]);
}

inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

struct fos_gnn {
  int device = 0;
  long cap = 0;  // cells the activation buffers hold
  float *w = nullptr, *wb = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr;
  unsigned short* Ab = nullptr;                 // BF16 bits of the three A_l
  unsigned short* h[NL + 1] = {nullptr};        // activations (bf16), h0..h3
  unsigned short* m[NL] = {nullptr};            // bf16(m) per layer (training)
  float *X0 = nullptr, *zhat = nullptr, *dh = nullptr, *dh2 = nullptr, *dmb = nullptr;
  float* part = nullptr;
  long part_len = 0;
  GnnScales* sc = nullptr;
  float* scp = nullptr;
  float* hs = nullptr;  // head partial sums
  int adam_t = 0;
  int layer_ctas = 0;  // persistent grid of the layer kernel (resident CTAs on the device)
  int in_ctas = 0;     // persistent grid of the input kernel
  ~fos_gnn() {
    void* ps[] = {w, wb, m1, m2, grad, Ab, X0, zhat, dh, dh2, dmb, part, sc, scp, hs};
    for (void* p : ps)
      if (p) cudaFree(p);
    for (auto p : h)
      if (p) cudaFree(p);
    for (auto p : m)
      if (p) cudaFree(p);
  }
};

namespace {
constexpr int kPartBlocks = 304;  // persistent CTAs of the reductions (2 x 152 SMs)
constexpr int kScaleBlocks = 1216;  // CTAs of the scale partial sums (8 x 152 SMs)

int gnn_reserve(fos_gnn* g, long nC) {
  if (g->cap >= nC) return 0;
  for (auto& p : g->h) { if (p) cudaFree(p); p = nullptr; }
  for (auto& p : g->m) { if (p) cudaFree(p); p = nullptr; }
  for (float** p : {&g->X0, &g->zhat, &g->dh, &g->dh2, &g->dmb})
    if (*p) { cudaFree(*p); *p = nullptr; }
  for (auto& p : g->h) FOS_CUDA(cudaMalloc(&p, sizeof(unsigned short) * H * (size_t)nC));
  for (auto& p : g->m) FOS_CUDA(cudaMalloc(&p, sizeof(unsigned short) * H * (size_t)nC));
  FOS_CUDA(cudaMalloc(&g->X0, sizeof(float) * NIN * (size_t)nC));
  FOS_CUDA(cudaMalloc(&g->zhat, sizeof(float) * 8 * (size_t)nC));
  FOS_CUDA(cudaMalloc(&g->dh, sizeof(float) * H * (size_t)nC));
  FOS_CUDA(cudaMalloc(&g->dh2, sizeof(float) * H * (size_t)nC));
  FOS_CUDA(cudaMalloc(&g->dmb, sizeof(float) * H * (size_t)nC));
  g->cap = nC;
  return 0;
}

// forward pass over the context's graph; training keeps m, X0 and zhat
int gnn_forward(fos_gnn* g, fos_ctx* c, const double* y, const double* v, double gamma, double* z,
                bool train) {
  if (int rc = gnn_reserve(g, c->nC)) return rc;
  if (c->ell_w != 4) {
    fos_set_error("learned preconditioner: tetrahedral grids only");
    return -2;
  }
  const int nC = c->nC;
  fos_launch(c, k_gnn_scale_part, kScaleBlocks, 256, nC, c->nF, y, v, (const double*)c->d_invV,
             (const float4*)c->d_faceNA32, g->scp);
  fos_launch(c, k_gnn_scale_final, 1, 32, nC, c->nF, kScaleBlocks, (const float*)g->scp, g->sc);
  fos_launch(c, k_gnn_in, std::max(1, std::min(nblk(nC, 256), g->in_ctas)), 256, nC, y, v, (const double*)c->d_invV,
             (float)gamma, (float)c->gamm, (const float*)g->wb, (const GnnScales*)g->sc, train ? g->X0 : (float*)nullptr,
             g->h[0]);
  const int ntiles = (nC + kTile - 1) / kTile;
  for (int l = 0; l < NL; l++) {
    const bool last = l == NL - 1;
    const int grid = std::max(1, std::min(ntiles, g->layer_ctas));
    auto kern = last ? k_gnn_layer<true> : k_gnn_layer<false>;
    fos_launch(c, kern, grid, kT, nC, c->nFi, (const int*)c->d_ell,
               (const int2*)c->d_faceLR, (const float4*)c->d_faceNA32, (const GnnScales*)g->sc,
               (const float*)(g->wb + OFF_L0 + l * L_SIZE),
               (const unsigned short*)(g->Ab + l * H * 2 * H), (const unsigned short*)g->h[l],
               (last && !train) ? (unsigned short*)nullptr : g->h[l + 1],
               train ? g->m[l] : (unsigned short*)nullptr, (const float*)g->wb, v, z,
               train ? g->zhat : (float*)nullptr);
  }
  FOS_LAUNCH_CHECK();
  return 0;
}
}  // namespace

extern "C" int fos_gnn_num_params(void) { return NPARAM; }

extern "C" int fos_gnn_create(fos_gnn** out, unsigned seed) {
  if (!out) return -1;
  fos_gnn* g = new fos_gnn();
  cudaGetDevice(&g->device);
  std::vector<float> w(NPARAM, 0.0f);
  std::mt19937 rng(seed);
  auto init = [&](int off, int rows, int cols) {  // He-uniform
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    const float a = std::sqrt(6.0f / cols);
    for (int k = 0; k < rows * cols; k++) w[off + k] = a * U(rng);
  };
  init(OFF_W0, H, 11);
  for (int l = 0; l < NL; l++) {
    const int o = OFF_L0 + l * L_SIZE;
    init(o + L_G, H, 4);
    for (int f = 0; f < H; f++) w[o + L_C + f] = 0.25f;  // mean-aggregation start
    init(o + L_A, H, 2 * H);
  }
  // output head D, d = 0: the untrained network is the identity preconditioner
  auto fail = [&](const char* what) {
    fos_set_error(std::string("fos_gnn_create: ") + what);
    delete g;
    return -100;
  };
  if (cudaMalloc(&g->w, sizeof(float) * NPARAM) || cudaMalloc(&g->wb, sizeof(float) * NPARAM) ||
      cudaMalloc(&g->m1, sizeof(float) * NPARAM) || cudaMalloc(&g->m2, sizeof(float) * NPARAM) ||
      cudaMalloc(&g->grad, sizeof(float) * NPARAM) ||
      cudaMalloc(&g->Ab, sizeof(unsigned short) * NL * H * 2 * H) ||
      cudaMalloc(&g->sc, sizeof(GnnScales)) || cudaMalloc(&g->scp, sizeof(float) * 10 * kScaleBlocks) ||
      cudaMalloc(&g->hs, sizeof(float) * 512))
    return fail("cudaMalloc");
  g->part_len = (long)kPartBlocks * (H * 2 * H + H);
  g->part_len = std::max<long>(g->part_len, (long)kPartBlocks * (H * NIN + H));
  if (cudaMalloc(&g->part, sizeof(float) * g->part_len)) return fail("cudaMalloc");
  {  // persistent grid of the layer kernel: every resident CTA of the device
    int nsm = 0, per_t = 0, per_f = 0, per_in = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, g->device) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_t, k_gnn_layer<true>, kT, 0) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_f, k_gnn_layer<false>, kT, 0) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_in, k_gnn_in, 256, 0))
      return fail("device attributes");
    g->layer_ctas = std::max(1, nsm * std::max(1, std::min(per_t, per_f)));
    g->in_ctas = std::max(1, nsm * std::max(1, per_in));
  }
  cudaMemcpy(g->w, w.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice);
  cudaMemset(g->m1, 0, sizeof(float) * NPARAM);
  cudaMemset(g->m2, 0, sizeof(float) * NPARAM);
  k_round_bf16<<<nblk(NPARAM, 256), 256>>>(NPARAM, g->w, g->wb);
  k_layer_bits<<<nblk(NL * H * 2 * H, 256), 256>>>(g->wb, g->Ab);
  if (cudaDeviceSynchronize() != cudaSuccess) return fail("init kernels");
  *out = g;
  return 0;
}

extern "C" void fos_gnn_destroy(fos_gnn* g) { delete g; }

extern "C" int fos_gnn_get_params(const fos_gnn* g, float* host) {
  if (!g || !host) return -1;
  FOS_CUDA(cudaMemcpy(host, g->w, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return NPARAM;
}

extern "C" int fos_gnn_set_params(fos_gnn* g, const float* host) {
  if (!g || !host) return -1;
  FOS_CUDA(cudaMemcpy(g->w, host, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  k_round_bf16<<<nblk(NPARAM, 256), 256>>>(NPARAM, g->w, g->wb);
  k_layer_bits<<<nblk(NL * H * 2 * H, 256), 256>>>(g->wb, g->Ab);
  FOS_CUDA(cudaDeviceSynchronize());
  return 0;
}

extern "C" int fos_gnn_apply_dev(fos_gnn* g, fos_ctx* c, const double* y, const double* v,
                                 double gamma, double* z) {
  if (!g || !c || !y || !v || !z) {
    fos_set_error("fos_gnn_apply_dev: bad arguments");
    return -1;
  }
  return gnn_forward(g, c, y, v, gamma, z, false);
}

int fos_gnn_precond(fos_ctx* c, const double* y, const double* r, double gamma, double* z) {
  if (!c->gnn) {
    fos_set_error("learned preconditioner requested but no network attached");
    return -1;
  }
  return gnn_forward(c->gnn, c, y, r, gamma, z, false);
}

extern "C" int fos_ctx_attach_gnn(fos_ctx* c, fos_gnn* g) {
  if (!c) return -1;
  if (g && c->ell_w != 4) {  // the network's message passing reads 4 neighbour slots
    fos_set_error("learned preconditioner: tetrahedral grids only");
    return -2;
  }
  c->gnn = g;
  return 0;
}

// Forward + backward of the normalised loss mean((zhat - t/s_v)^2) for one sample; the
// gradient is added to the device accumulator (fos_gnn_zero_grad clears it).  loss_out
// (host) receives the loss.
extern "C" int fos_gnn_loss_grad_dev(fos_gnn* g, fos_ctx* c, const double* y, const double* v,
                                     const double* t, double gamma, double* loss_out) {
  if (!g || !c || !y || !v || !t) {
    fos_set_error("fos_gnn_loss_grad_dev: bad arguments");
    return -1;
  }
  const int nC = c->nC;
  if (int rc = gnn_forward(g, c, y, v, gamma, nullptr, true)) return rc;
  const float invN = 1.0f / (5.0f * nC);
  // head
  const int nb_out = nblk(nC, 256);
  const int plen = 1 + 5 + 5 * H;
  if ((long)nb_out * plen > g->part_len) {
    cudaFree(g->part);
    g->part_len = (long)nb_out * plen;
    FOS_CUDA(cudaMalloc(&g->part, sizeof(float) * g->part_len));
  }
  fos_launch(c, k_gnn_out_bwd, nb_out, 256, nC, (const float*)g->zhat, t, (const GnnScales*)g->sc,
             (const unsigned short*)g->h[NL], (const float*)g->wb, invN, g->dh, g->part);
  // per-CTA [loss, dd, dD] partials -> hs, then into the gradient accumulator
  cudaMemsetAsync(g->hs, 0, sizeof(float) * plen, c->stream);
  fos_launch(c, k_sum_parts, nblk(plen, 256), 256, nb_out, plen, (const float*)g->part, g->hs, 1.0f);
  fos_launch(c, k_gnn_head_grad, 1, 512, (const float*)g->hs, g->grad);
  // layers, last to first
  float* dcur = g->dh;   // dL/dh_out
  float* dnext = g->dh2; // dL/dh_in
  for (int l = NL - 1; l >= 0; l--) {
    fos_launch(c, k_gnn_layer_bwd, kPartBlocks, kT, nC, (const unsigned short*)g->h[l],
               (const unsigned short*)g->m[l], (const unsigned short*)g->h[l + 1],
               (const float*)dcur, (const unsigned short*)(g->Ab + l * H * 2 * H), dnext,
               g->dmb, g->part);
    float* gl = g->grad + OFF_L0 + l * L_SIZE;
    fos_launch(c, k_sum_parts, nblk(H * 2 * H + H, 256), 256, kPartBlocks, H * 2 * H + H,
               (const float*)g->part, gl + L_A, 1.0f);  // dA then db (contiguous in params)
    fos_launch(c, k_gnn_edge_bwd, kPartBlocks, kT, nC, c->nFi, (const int*)c->d_ell,
               (const int2*)c->d_faceLR, (const float4*)c->d_faceNA32, (const GnnScales*)g->sc,
               (const float*)(g->wb + OFF_L0 + l * L_SIZE), (const unsigned short*)g->h[l],
               (const float*)g->dmb, dnext, g->part);
    fos_launch(c, k_sum_parts, nblk(H * 5, 256), 256, kPartBlocks, H * 5, (const float*)g->part,
               gl + L_G, 1.0f);  // dG then dc (contiguous)
    std::swap(dcur, dnext);
  }
  fos_launch(c, k_gnn_in_bwd, kPartBlocks, 256, nC, (const float*)g->X0,
             (const unsigned short*)g->h[0], (const float*)dcur, g->part);
  fos_launch(c, k_sum_parts, nblk(H * NIN + H, 256), 256, kPartBlocks, H * NIN + H,
             (const float*)g->part, g->grad + OFF_W0, 1.0f);  // dW0 then db0
  FOS_LAUNCH_CHECK();
  if (loss_out) {
    float lh = 0.0f;
    FOS_CUDA(cudaMemcpyAsync(&lh, g->hs, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    FOS_CUDA(cudaStreamSynchronize(c->stream));
    *loss_out = lh * invN;
  }
  return 0;
}

extern "C" int fos_gnn_zero_grad(fos_gnn* g) {
  if (!g) return -1;
  FOS_CUDA(cudaMemset(g->grad, 0, sizeof(float) * NPARAM));
  return 0;
}

extern "C" int fos_gnn_get_grad(const fos_gnn* g, float* host) {
  if (!g || !host) return -1;
  FOS_CUDA(cudaDeviceSynchronize());
  FOS_CUDA(cudaMemcpy(host, g->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return NPARAM;
}

// one Adam step on the accumulated gradient (scaled by grad_scale, e.g. 1/batch)
extern "C" int fos_gnn_adam_step(fos_gnn* g, float lr, float beta1, float beta2, float eps,
                                 float grad_scale) {
  if (!g) return -1;
  g->adam_t++;
  if (grad_scale != 1.0f) {
    std::vector<float> tmp(NPARAM);
    FOS_CUDA(cudaMemcpy(tmp.data(), g->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    for (float& x : tmp) x *= grad_scale;
    FOS_CUDA(cudaMemcpy(g->grad, tmp.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  }
  const float c1 = 1.0f - std::pow(beta1, (float)g->adam_t);
  const float c2 = 1.0f - std::pow(beta2, (float)g->adam_t);
  k_adam<<<nblk(NPARAM, 256), 256>>>(NPARAM, g->w, g->grad, g->m1, g->m2, lr, beta1, beta2, eps,
                                      c1, c2, g->wb);
  k_layer_bits<<<nblk(NL * H * 2 * H, 256), 256>>>(g->wb, g->Ab);
  FOS_CUDA(cudaGetLastError());
  FOS_CUDA(cudaDeviceSynchronize());
  return 0;
}
