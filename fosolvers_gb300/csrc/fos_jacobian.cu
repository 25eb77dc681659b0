// fos_jacobian.cu -- block-5x5 Roe Jacobian assembly and the block ILU(0)
// preconditioner (set-up and level-scheduled triangular solves) on sm_103a.
//
// Jacobian (Euler.f90:159-333): per pair i = (m, n), normal n from m to n,
//   JacP(1:5,1:5)  = -aP/2 (A(n; u_m, H_m) + |A~|(n; Roe avg)),   added to diag(m)
//   JacP(1:5,6:10) = -aP/2 (A(n; u_n, H_n) - |A~|),                block (m, n)
//   JacP(6:10,:)   = -JacP(1:5,:)                                  rows of n
// A = eulerNFJ (:252-276), |A~| = eulerANFJ (:279-333); boundary pairs add only
// their diagonal block (the ghost's dependence on the interior is ignored, :216-219).
// Each off-diagonal block belongs to exactly one face, so k_jac_face writes both
// off-diagonal blocks of an interior face directly; the diagonal block of a cell is
// then minus the sum of the off-diagonal blocks in its column (diag(m) += -block(n,m),
// diag(n) += -block(m,n)) plus its boundary faces' terms, gathered per cell in a
// fixed order by k_jac_diag.  No floating-point atomics.
//
// Preconditioner: P = I - gamma diag(1/v) J, factored by block ILU(0) (the block
// form of SPARSKIT ilu0, ITSOL/ilut.f:1793-1917: equal to scalar ILU(0) of the
// interleaved matrix), with the inverse of each diagonal block stored in place of the
// block like ilu0 stores the inverted diagonal.  The ILU works in "position" space: block row
// p is the p-th row of the elimination order (internal order, or colour-major for
// FOS_ILU_COLOR); each row's blocks are contiguous and sorted by position, so lower(p) =
// [prow[p], pdiag[p]) and upper(p) = (pdiag[p], prow[p+1]).  The factors are stored in two
// regions, every row's L blocks first and then every row's inverted diagonal and U blocks
// (plst / pdu), so that the forward and the backward sweep each stream one region without
// reading around the blocks they skip.  Rows are processed level by
// level: colours (contiguous ranges of p) for FOS_ILU_COLOR, otherwise the level sets of
// the lower / upper triangles (one more than the highest level among the row's lower /
// upper neighbours, cf. SPARSKIT levels, FORMATS/unary.f:1078).  Apply = lusol
// (ilut.f:2272-2320) in block form, on AoS copies of the vectors in position order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fos_internal.h"
#include "fos_device.cuh"

namespace {

constexpr int kT = 128;

struct Prim {
  double rho, u, v, w, H, p, s;
};
__device__ __forceinline__ void load_prim(const double* __restrict__ W, int c, Prim& P) {
  const double2* w2 = reinterpret_cast<const double2*>(W + 8 * (size_t)c);
  double2 a = w2[0], b = w2[1], d = w2[2], e = w2[3];
  P.rho = a.x; P.u = a.y; P.v = b.x; P.w = b.y; P.H = d.x; P.p = d.y; P.s = e.x;
}

// eulerNFJ entry (a, b) -- normal flux Jacobian dF.n/dU
template <typename T>
__device__ __forceinline__ T nfj(int a, int b, const T n[3], const T u[3], T H, T g, T v2, T vn) {
  const T g1 = g - T(1);
  if (a == 0) return (b >= 1 && b <= 3) ? n[b - 1] : T(0);
  if (a == 4) {
    if (b == 0) return (T(0.5) * g1 * v2 - H) * vn;
    if (b == 4) return g * vn;
    return H * n[b - 1] - g1 * u[b - 1] * vn;
  }
  const int i = a - 1;
  if (b == 0) return T(0.5) * g1 * v2 * n[i] - u[i] * vn;
  if (b == 4) return g1 * n[i];
  const int j = b - 1;
  return u[i] * n[j] + (T(1) - g) * n[i] * u[j] + (i == j ? vn : T(0));
}

// eulerANFJ (Euler.f90:279-333), row-major 25: |vn| T0 + |vn - c| r- l-^T + |vn + c| r+ l+^T,
// where the entropy/shear projector T0 equals I - r- l-^T - r+ l+^T plus the reference's
// entry at :300 (column 1, rows 2:4 hold -(1 + (g-1) M^2/2) u + vn n, i.e. an extra -u
// against the exact projector).  So
//   |A~| = |vn| (I + E) + (|vn - c| - |vn|) r- l-^T + (|vn + c| - |vn|) r+ l+^T,
//   E(1 + i, 0) = -u_i,
// the same matrix in two rank-1 updates of a diagonal instead of 25 T0 entries and two more
// rank-1 terms.
template <typename T>
__device__ __forceinline__ void anfj(const T n[3], const T u[3], T H, T c, T g, T out[25]) {
  const T g1 = g - T(1);
  const T v2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const T vn = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
  const T ic = T(1) / c;
  const T M2 = v2 * ic * ic, Mn = vn * ic;
  const T be = g1 * ic * ic;
  const T av = fabs(vn);
#pragma unroll
  for (int k = 0; k < 25; k++) out[k] = (k % 6 == 0) ? av : T(0);
#pragma unroll
  for (int i = 0; i < 3; i++) out[5 * (1 + i)] = -av * u[i];
#pragma unroll
  for (int sgn = -1; sgn <= 1; sgn += 2) {
    T rr[5], wl[5];
    rr[0] = T(1);
    for (int i = 0; i < 3; i++) rr[1 + i] = u[i] + T(sgn) * c * n[i];
    rr[4] = H + T(sgn) * vn * c;
    const T w = fabs(vn + T(sgn) * c) - av;
    wl[0] = w * (T(0.25) * g1 * M2 - T(sgn) * T(0.5) * Mn);
    for (int j = 0; j < 3; j++) wl[1 + j] = w * (-T(0.5) * be * u[j] + T(sgn) * T(0.5) * n[j] * ic);
    wl[4] = w * (T(0.5) * be);
    for (int a = 0; a < 5; a++)
      for (int b = 0; b < 5; b++) out[5 * a + b] = fma(rr[a], wl[b], out[5 * a + b]);
  }
}

// primitives of one side of a face in the arithmetic type of the assembly
template <typename T>
struct PrimT {
  T u[3], H, s;
};

// Blocks of face f from its two sides' primitives (Roe averages, Euler.f90:207-209): both
// off-diagonal blocks of an interior face, or the boundary pair's diagonal term
template <typename T, typename TJ>
__device__ __forceinline__ void jac_face_blocks(int f, int nFi, const T n[3], T aP,
                                                const PrimT<T>& L, const PrimT<T>& R, T gg,
                                                const int* __restrict__ fslot,
                                                TJ* __restrict__ J, TJ* __restrict__ Jb) {
  const T inv = T(1) / (L.s + R.s);
  const T ua[3] = {(L.s * L.u[0] + R.s * R.u[0]) * inv, (L.s * L.u[1] + R.s * R.u[1]) * inv,
                   (L.s * L.u[2] + R.s * R.u[2]) * inv};
  const T Ha = (L.s * L.H + R.s * R.H) * inv;
  const T ca = sqrt((gg - T(1)) * (Ha - T(0.5) * (ua[0] * ua[0] + ua[1] * ua[1] + ua[2] * ua[2])));
  T Ab[25];
  anfj<T>(n, ua, Ha, ca, gg, Ab);
  const T v2L = L.u[0] * L.u[0] + L.u[1] * L.u[1] + L.u[2] * L.u[2];
  const T vnL = L.u[0] * n[0] + L.u[1] * n[1] + L.u[2] * n[2];
  const T v2R = R.u[0] * R.u[0] + R.u[1] * R.u[1] + R.u[2] * R.u[2];
  const T vnR = R.u[0] * n[0] + R.u[1] * n[1] + R.u[2] * n[2];
  const T h = T(0.5) * aP;
  if (f < nFi) {
    TJ* oLR = J + 25 * (size_t)fslot[2 * f];      // block (L, R) = JacP(1:5,6:10)
    TJ* oRL = J + 25 * (size_t)fslot[2 * f + 1];  // block (R, L) = JacP(6:10,1:5)
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
      for (int b = 0; b < 5; b++) {
        oLR[5 * a + b] = (TJ)(-h * (nfj<T>(a, b, n, R.u, R.H, gg, v2R, vnR) - Ab[5 * a + b]));
        oRL[5 * a + b] = (TJ)(h * (nfj<T>(a, b, n, L.u, L.H, gg, v2L, vnL) + Ab[5 * a + b]));
      }
  } else {
    TJ* d = Jb + 25 * (size_t)(f - nFi);  // boundary pair's diagonal term
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
      for (int b = 0; b < 5; b++)
        d[5 * a + b] = (TJ)(-h * (nfj<T>(a, b, n, L.u, L.H, gg, v2L, vnL) + Ab[5 * a + b]));
  }
}

// ghost-side primitives of boundary face f (setBC, FP64; 1% of the faces)
__device__ __forceinline__ void ghost_prim(int f, int nC, int2 lr, const double* __restrict__ y,
                                           const int* __restrict__ bcT,
                                           const double* __restrict__ bcP, int maxP, double nx,
                                           double ny, double nz, double g, double r, Prim& R) {
  double U[5], G[5];
  for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + lr.x];
  const int row = lr.y;
  ghost_state(row > 0 ? bcT[row - 1] : FOS_BC_WALL,
              row > 0 ? bcP + (size_t)maxP * (row - 1) : nullptr, U, nx, ny, nz, g, r, G);
  const double inv = 1.0 / G[0];
  R.rho = G[0]; R.u = G[1] * inv; R.v = G[2] * inv; R.w = G[3] * inv;
  R.p = (g - 1.0) * (G[4] - 0.5 * (G[1] * G[1] + G[2] * G[2] + G[3] * G[3]) * inv);
  R.H = (G[4] + R.p) * inv;
  R.s = sqrt(G[0]);
}

// Ghost-side primitives (u, v, w, H, sqrt(rho)) of the boundary faces for k_jac_cell32, FP64,
// written into the face slots of the flow array (6 doubles per face; the residual rewrites
// them before it reads them), from the FP32 normals widened as the FP32 assembly uses them.
__global__ void __launch_bounds__(kT) k_jac_ghost64(int nFi, int nF, int nC,
                                                    const int2* __restrict__ faceLR,
                                                    const float4* __restrict__ faceNA32,
                                                    const double* __restrict__ y,
                                                    const int* __restrict__ bcT,
                                                    const double* __restrict__ bcP, int maxP,
                                                    double g, double r, double* __restrict__ Gb) {
  const int f = nFi + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nF) return;
  const int2 lr = __ldg(faceLR + f);
  const float4 na = __ldg(faceNA32 + f);
  Prim R;
  ghost_prim(f, nC, lr, y, bcT, bcP, maxP, f2d_bits(na.x), f2d_bits(na.y), f2d_bits(na.z), g, r,
             R);
  double2* G2 = reinterpret_cast<double2*>(Gb + 6 * (size_t)f);
  G2[0] = make_double2(R.u, R.v);
  G2[1] = make_double2(R.w, R.H);
  G2[2] = make_double2(R.s, 0.0);
}

// FP64 form: FP64 primitives and geometry
template <typename TJ>
__global__ void __launch_bounds__(kT) k_jac_face(int nFi, int nF, int nC,
                                                 const int2* __restrict__ faceLR,
                                                 const double2* __restrict__ faceNA,
                                                 const double* __restrict__ W,
                                                 const double* __restrict__ y,
                                                 const int* __restrict__ fslot,
                                                 const int* __restrict__ bcT,
                                                 const double* __restrict__ bcP, int maxP,
                                                 double g, double r, TJ* __restrict__ J,
                                                 TJ* __restrict__ Jb) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nF) return;
  const int2 lr = faceLR[f];
  const double2 n01 = faceNA[2 * (size_t)f], n2a = faceNA[2 * (size_t)f + 1];
  const double n[3] = {n01.x, n01.y, n2a.x};
  Prim L, R;
  load_prim(W, lr.x, L);
  if (f < nFi) load_prim(W, lr.y, R);
  else ghost_prim(f, nC, lr, y, bcT, bcP, maxP, n01.x, n01.y, n2a.x, g, r, R);
  const PrimT<double> PL = {{L.u, L.v, L.w}, L.H, L.s}, PR = {{R.u, R.v, R.w}, R.H, R.s};
  jac_face_blocks<double, TJ>(f, nFi, n, n2a.y, PL, PR, g, fslot, J, Jb);
}

// FP32 form: FP32 arithmetic from the per-cell FP32 (hi, lo) primitives of the residual
// (rounded to FP32) and the FP32 face geometry, so no FP64 instruction runs on interior
// faces (the FP32 preconditioner is assembled and stored in FP32)
__device__ __forceinline__ PrimT<float> load_prim_f32(const float* __restrict__ Whl, int c) {
  const float4* w4 = reinterpret_cast<const float4*>(Whl + 16 * (size_t)c);
  const float4 a = __ldg(w4), b = __ldg(w4 + 1), d = __ldg(w4 + 2), e = __ldg(w4 + 3);
  // hi: (rho, u, v, w) = a, (H, p) = b.xy; lo: (rho, u) = b.zw, (v, w, H, p) = d
  return {{a.y + b.w, a.z + d.x, a.w + d.y}, b.x + d.z, e.x};
}

// Cell-centric FP32 assembly: one thread per cell, cells in the internal (bandwidth-
// reduced) order, so neighbouring cells' primitives and face data are L2 hits.  A thread
// evaluates each face of its cell in the face's orientation (Roe average, |A~| -- the same
// expressions for both cells of the face -- and the neighbour's normal flux Jacobian) and
// keeps
//   off-diagonal block:  cell L: block (L, R) = -aP/2 (A(n; u_R) - |A~|)
//                        cell R: block (R, L) =  aP/2 (A(n; u_L) + |A~|)
//   diagonal:            -sum_f aP/2 (A(n_out; u_c) + |A~|) over all faces of the cell,
//                        in registers.
// A(n; u) is linear in n, so the cell's own-state terms sum to A(S_c/2; u_c), S_c = sum of
// aP n_out: zero for cells with planar faces (tetrahedra; the FP32 sum of the per-face terms
// would only add rounding) and formed once from the closure vector otherwise (warped
// hexahedra).  |A~| is even in n, so the diagonal takes -aP/2 |A~| from every face.  The row
// is staged (contiguous in position space) in shared memory; the warp then
// stores the 32 rows one after another, each as contiguous 128-byte pieces.  Each face is
// evaluated by both of its cells: FP32 arithmetic is cheap next to the scattered block
// stores and the re-read of every off-diagonal block that a face-then-diagonal assembly
// costs.
// One block row of the FP32 Jacobian for cell c (the body of k_jac_cell32, shared with the
// fused set-up k_pset32): the row's blocks go to st (row-major 25-float blocks at
// st + 25 (slot - s0)); sdiag = the diagonal block's slot - s0.  The multiply-adds are
// written out (fmaf), so both kernels produce the same bits.
template <int kW>
__device__ __forceinline__ void jac_row32(int c, int nC, int nFi, int s0, int sdiag,
                                          const int* __restrict__ ell,
                                          const int* __restrict__ cnb,
                                          const float4* __restrict__ cna,
                                          const int* __restrict__ fslot,
                                          const float* __restrict__ Whl,
                                          const double* __restrict__ Gb,
                                          const float4* __restrict__ Sc, float gg,
                                          float* __restrict__ st) {
  const PrimT<float> P = load_prim_f32(Whl, c);
  float D[25];
#pragma unroll
  for (int k = 0; k < 25; k++) D[k] = 0.0f;
#pragma unroll 1
  for (int k = 0; k < kW; k++) {
    const int ek = __ldg(ell + (size_t)kW * c + k);
    if (ek < 0) continue;
    const int f = ek >> 1;
    const bool isR = ek & 1;
    const float4 na = __ldg(cna + (size_t)k * nC + c);  // the face's FP32 geometry, per cell
    const float n[3] = {na.x, na.y, na.z};
    PrimT<float> Q;
    if (f < nFi) {
      Q = load_prim_f32(Whl, __ldg(cnb + (size_t)kW * c + k));  // the cell across the face
    } else {  // ghost primitives of k_jac_ghost64
      const double2* G2 = reinterpret_cast<const double2*>(Gb + 6 * (size_t)f);
      const double2 a0 = __ldg(G2), a1 = __ldg(G2 + 1), a2 = __ldg(G2 + 2);
      Q = {{d2f_trunc(a0.x), d2f_trunc(a0.y), d2f_trunc(a1.x)}, d2f_trunc(a1.y),
           d2f_trunc(a2.x)};
    }
    const PrimT<float>& L = (f < nFi && isR) ? Q : P;
    const PrimT<float>& R = (f < nFi && isR) ? P : Q;
    const float inv = 1.0f / (L.s + R.s);
    const float ua[3] = {(L.s * L.u[0] + R.s * R.u[0]) * inv, (L.s * L.u[1] + R.s * R.u[1]) * inv,
                         (L.s * L.u[2] + R.s * R.u[2]) * inv};
    const float Ha = (L.s * L.H + R.s * R.H) * inv;
    const float ca =
        sqrtf((gg - 1.0f) * (Ha - 0.5f * (ua[0] * ua[0] + ua[1] * ua[1] + ua[2] * ua[2])));
    float Ab[25];
    anfj<float>(n, ua, Ha, ca, gg, Ab);
    const float h = 0.5f * na.w;
    if (f >= nFi) {  // boundary pair: diagonal term only (its A(u_c) part is in S_c)
#pragma unroll
      for (int q = 0; q < 25; q++) D[q] = fmaf(-h, Ab[q], D[q]);
      continue;
    }
    // the neighbour's normal flux Jacobian with the face normal: +aP/2 for cell R, -aP/2 for L
    const float v2Q = Q.u[0] * Q.u[0] + Q.u[1] * Q.u[1] + Q.u[2] * Q.u[2];
    const float vnQ = Q.u[0] * n[0] + Q.u[1] * n[1] + Q.u[2] * n[2];
    const float sh = isR ? h : -h;
    float* off = st + 25 * (fslot[2 * f + (isR ? 1 : 0)] - s0);
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
      for (int b = 0; b < 5; b++) {
        off[5 * a + b] =
            fmaf(h, Ab[5 * a + b], __fmul_rn(sh, nfj<float>(a, b, n, Q.u, Q.H, gg, v2Q, vnQ)));
        D[5 * a + b] = fmaf(-h, Ab[5 * a + b], D[5 * a + b]);
      }
  }
  if (Sc) {  // -A(S_c/2; u_c): the own-state terms of a cell whose faces do not close
    const float4 S4 = __ldg(Sc + c);
    const float Sh[3] = {0.5f * S4.x, 0.5f * S4.y, 0.5f * S4.z};
    const float v2P = P.u[0] * P.u[0] + P.u[1] * P.u[1] + P.u[2] * P.u[2];
    const float vnP = P.u[0] * Sh[0] + P.u[1] * Sh[1] + P.u[2] * Sh[2];
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
      for (int b = 0; b < 5; b++)
        D[5 * a + b] = __fsub_rn(D[5 * a + b], nfj<float>(a, b, Sh, P.u, P.H, gg, v2P, vnP));
  }
  float* dg = st + 25 * sdiag;
#pragma unroll
  for (int k = 0; k < 25; k++) dg[k] = D[k];
}

template <int kW>
__global__ void __launch_bounds__(64) k_jac_cell32(
    int nC, int nFi, const int* __restrict__ ipos, const int* __restrict__ prow,
    const int* __restrict__ cdiag, const int* __restrict__ ell, const int* __restrict__ cnb,
    const float4* __restrict__ cna, const int* __restrict__ fslot,
    const float* __restrict__ Whl, const double* __restrict__ Gb, const float4* __restrict__ Sc,
    double g, float* __restrict__ J) {
  constexpr int kRow = (kW + 1) * 25;  // floats of a full block row
  __shared__ float stg[2][32][kRow];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = (blockIdx.x * 2 + warp) * 32 + lane;
  float* st = stg[warp][lane];
  int s0 = 0, nbk = 0;
  if (c < nC) {
    const int p = ipos[c];
    s0 = prow[p];
    nbk = prow[p + 1] - s0;
    jac_row32<kW>(c, nC, nFi, s0, cdiag[c] - s0, ell, cnb, cna, fslot, Whl, Gb, Sc,
                  d2f_trunc(g), st);
  }
  __syncwarp();
  // the warp's rows, one after another: row r = [25 s0_r, 25 (s0_r + nbk_r)) of J
  for (int rr = 0; rr < 32; rr++) {
    const int sr = __shfl_sync(0xffffffffu, s0, rr);
    const int nr = 25 * __shfl_sync(0xffffffffu, nbk, rr);
    float* dst = J + 25 * (size_t)sr;
    const float* src = stg[warp][rr];
    for (int k = lane; k < nr; k += 32) dst[k] = src[k];
  }
}

template <typename TJ>
__global__ void __launch_bounds__(kT) k_jac_diag(int nC, int nFi, const int* __restrict__ crow,
                                                 const int* __restrict__ cent,
                                                 const int* __restrict__ fslot,
                                                 const int* __restrict__ cdiag,
                                                 const TJ* __restrict__ Jb,
                                                 TJ* __restrict__ J) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  TJ D[25];
#pragma unroll
  for (int k = 0; k < 25; k++) D[k] = TJ(0);
  for (int e = crow[c]; e < crow[c + 1]; e++) {
    const int ent = cent[e], f = ent >> 1;
    if (f < nFi) {
      // cell is L: diag += JacP(1:5,1:5) = -block(R,L); cell is R: diag += -block(L,R)
      const TJ* o = J + 25 * (size_t)fslot[2 * f + ((ent & 1) ? 0 : 1)];
#pragma unroll
      for (int k = 0; k < 25; k++) D[k] -= o[k];
    } else {
      const TJ* o = Jb + 25 * (size_t)(f - nFi);
#pragma unroll
      for (int k = 0; k < 25; k++) D[k] += o[k];
    }
  }
  TJ* dst = J + 25 * (size_t)cdiag[c];
#pragma unroll
  for (int k = 0; k < 25; k++) dst[k] = D[k];
}

// invert a 5x5 block in place by Gauss--Jordan without pivoting (scalar ilu0 eliminates
// inside the diagonal block without pivoting too, ilut.f:1893-1898); false on a zero pivot
template <typename T>
__device__ __forceinline__ bool inv5(T a[25]) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 5; k++) {
    const T piv = a[5 * k + k];
    ok &= (piv != T(0));
    const T ip = T(1) / piv;
    // row k scaled; column k becomes the inverse's column
#pragma unroll
    for (int j = 0; j < 5; j++) a[5 * k + j] = (j == k) ? ip : a[5 * k + j] * ip;
#pragma unroll
    for (int i = 0; i < 5; i++) {
      if (i == k) continue;
      const T f = a[5 * i + k];
#pragma unroll
      for (int j = 0; j < 5; j++) a[5 * i + j] = (j == k) ? -f * ip : a[5 * i + j] - f * a[5 * k + j];
    }
  }
  return ok;
}

// One level of the block ILU(0) factorisation.  Five lanes per block row p (lane a owns
// row a of every block of row p), six rows per warp, 24 rows per CTA; the row's blocks
// live in shared memory while they are being eliminated:
//   P_p* = delta - gamma/v J_p*                         (copy of the row, fused)
//   for k in lower(p): L_pk = P_pk inv(D_k); P_pj -= L_pk U_kj for j in upper(k) in row p
//   D_p = P_pp -> inverted by Gauss--Jordan without pivoting across the five lanes
// A lane only touches its own row of row p's blocks and reads finished blocks of earlier
// rows from global memory, so the lanes of a row need no synchronisation until the
// diagonal inversion (warp shuffles).  The factor blocks are stored column-major (entry
// (i, j) at 5 j + i), so each store instruction here (lane a writes entry (a, k)) and each
// load instruction of the sweeps touches five consecutive floats per block row instead of
// five floats 20 bytes apart.
// The 5x5 block arithmetic of the factorisation, written out so that every kernel that
// factors (k_ilu_factor, k_pset32) rounds the same way:
//   (A B)(i, b) = sum_k A(i, k) B(k, b), k ascending, one fused multiply-add per term;
//   Gauss--Jordan step k on row a of D with rk = row k before the step.
__device__ __forceinline__ float ilu_dot5(const float A[5], const float* Bcol) {
  float acc = 0.0f;
#pragma unroll
  for (int k = 0; k < 5; k++) acc = fmaf(A[k], Bcol[k], acc);
  return acc;
}
__device__ __forceinline__ double ilu_dot5(const double A[5], const double* Bcol) {
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < 5; k++) acc = fma(A[k], Bcol[k], acc);
  return acc;
}
template <typename TF>
__device__ __forceinline__ TF ilu_mul(TF a, TF b) {
  if constexpr (sizeof(TF) == 4) return __fmul_rn(a, b); else return __dmul_rn(a, b);
}
template <typename TF>
__device__ __forceinline__ void ilu_gj_step(int a, int k, const TF rk[5], TF Da[5]) {
  const TF ip = TF(1) / rk[k];
  if (a == k) {
#pragma unroll
    for (int b = 0; b < 5; b++) Da[b] = (b == k) ? ip : ilu_mul(rk[b], ip);
  } else {
    const TF f = Da[k];
#pragma unroll
    for (int b = 0; b < 5; b++) Da[b] = (b == k) ? -ilu_mul(f, ip) : fma(-f, ilu_mul(rk[b], ip), Da[b]);
  }
}

template <typename TF>
__device__ __forceinline__ TF from64(double x) {
  if constexpr (sizeof(TF) == 4) return d2f_trunc(x); else return (TF)x;
}
template <typename TF>
__device__ __forceinline__ double to64(TF x) {
  if constexpr (sizeof(TF) == 4) return f2d_bits(x); else return (double)x;
}

constexpr int kRowsPerCta = 6 * (kT / 32);
constexpr int kMaxBlocksPerRow = 7;  // diagonal + up to 6 neighbours (hexahedra)

template <typename TF, typename TJ>
__global__ void __launch_bounds__(kT) k_ilu_factor(
    int n, const int* __restrict__ rows, int p0, const int* __restrict__ prow,
    const int* __restrict__ pdiag, const int* __restrict__ ord, const double* __restrict__ invV,
    double gamma, const TJ* __restrict__ J, const int* __restrict__ upd_ptr,
    const int3* __restrict__ upd, const int* __restrict__ plst, const int* __restrict__ pdu,
    TF* __restrict__ LU, int* __restrict__ ierr) {
  // update operands (inv(D_q), U_qj of earlier levels) of the first kPre operations of a row
  // are fetched into shared memory before the elimination, all loads in flight at once
  constexpr int kPre = sizeof(TF) == 4 ? 8 : 0;
  // row strides padded so that the 5 lanes x 6 rows of a warp (and the 6 rows' broadcast
  // operand reads) fall in distinct shared-memory banks: 185 = 7 x 25 + 10, 201 = 8 x 25 + 1
  constexpr int kSmRow = 185, kBsRow = kPre > 0 ? 201 : 25;
  __shared__ TF sm_[kRowsPerCta * kSmRow];
  __shared__ TF bsm_[kRowsPerCta * kBsRow];
  auto sm = [&](int r, int b) -> TF* { return sm_ + r * kSmRow + 25 * b; };
  auto bsm = [&](int r, int o) -> TF* { return bsm_ + r * kBsRow + 25 * o; };
  const int lane = threadIdx.x & 31;
  const int sub = lane / 5, a = lane - 5 * sub;
  const int lrow = (threadIdx.x >> 5) * 6 + (sub < 6 ? sub : 0);
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 6 + sub;
  const bool active = sub < 6 && t < n;
  const int p = active ? (rows ? rows[t] : p0 + t) : 0;
  TF D[5] = {TF(0), TF(0), TF(0), TF(0), TF(0)};
  int s0 = 0, sd = 0, o0 = 0, no = 0;
  if (active) {
    s0 = prow[p];
    sd = pdiag[p];
    o0 = upd_ptr[p];
    no = upd_ptr[p + 1] - o0;
    const int nb = prow[p + 1] - s0;
    if (kPre > 0) {
      TF pre[kPre > 0 ? kPre : 1][5];
#pragma unroll
      for (int o = 0; o < kPre; o++)
        if (o < no) {
          const TF* B = LU + 25 * (size_t)upd[o0 + o].y + 5 * a;  // column a
#pragma unroll
          for (int k = 0; k < 5; k++) pre[o][k] = B[k];
        }
#pragma unroll
      for (int o = 0; o < kPre; o++)
        if (o < no) {
#pragma unroll
          for (int k = 0; k < 5; k++) bsm(lrow, o)[5 * a + k] = pre[o][k];
        }
    }
    // P = I - (gamma / v) J in the factor's precision (FP32 arithmetic in the FP32 form)
    const TF sc = from64<TF>(gamma * invV[ord[p]]);
#pragma unroll
    for (int b = 0; b < kMaxBlocksPerRow; b++) {
      if (b >= nb) break;
      const TJ* src = J + 25 * (size_t)(s0 + b) + 5 * a;
      const bool dg = (s0 + b) == sd;
#pragma unroll
      for (int k = 0; k < 5; k++)
        sm(lrow, b)[5 * a + k] = fma(-sc, (TF)src[k], (dg && k == a) ? TF(1) : TF(0));
    }
  }
  __syncwarp();  // the five lanes of a row see each other's operand rows
  if (active) {
    for (int o = 0; o < no; o++) {
      const int3 op = upd[o0 + o];
      TF A[5];
      TF* Ar = sm(lrow, op.x - s0) + 5 * a;
#pragma unroll
      for (int k = 0; k < 5; k++) A[k] = Ar[k];
      const TF* B = (o < kPre) ? bsm(lrow, o) : LU + 25 * (size_t)op.y;  // column-major
      TF* dst = sm(lrow, (op.z < 0 ? op.x : op.z) - s0) + 5 * a;
#pragma unroll
      for (int b = 0; b < 5; b++) {
        TF Bc[5];
#pragma unroll
        for (int k = 0; k < 5; k++) Bc[k] = B[5 * b + k];
        const TF acc = ilu_dot5(A, Bc);
        dst[b] = op.z < 0 ? acc : dst[b] - acc;
      }
    }
#pragma unroll
    for (int b = 0; b < 5; b++) D[b] = sm(lrow, sd - s0)[5 * a + b];
  }
  const int base = lane - a;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 5; k++) {
    TF rk[5];
#pragma unroll
    for (int b = 0; b < 5; b++) rk[b] = __shfl_sync(0xffffffffu, D[b], base + k < 32 ? base + k : 0);
    ok &= !(active && rk[k] == TF(0));
    ilu_gj_step<TF>(a, k, rk, D);  // lane a's own row: D[b] == rk[b] when a == k
  }
  if (!active) return;
  if (!ok) atomicMin(ierr, p + 1);
#pragma unroll
  for (int b = 0; b < 5; b++) sm(lrow, sd - s0)[5 * a + b] = D[b];
  // block b of the row: L blocks into the L region, the diagonal and U blocks into the D/U one
  const int nb = prow[p + 1] - s0, nl = sd - s0, bl = plst[p], bdu = pdu[p];
  for (int b = 0; b < nb; b++) {
    TF* dst = LU + 25 * (size_t)(b < nl ? bl + b : bdu + (b - nl)) + a;  // row a, column-major
#pragma unroll
    for (int k = 0; k < 5; k++) dst[5 * k] = sm(lrow, b)[5 * a + k];
  }
}

// Fused FP32 set-up: one level (colour) of the block ILU(0) factorisation of
// P = I - gamma diag(1/v) J with the rows of J assembled in the same kernel, so J is never
// written to or read back from HBM.  Thread per row, a warp takes 32 rows of the level:
//   A. the row's Jacobian blocks (jac_row32, the arithmetic of k_jac_cell32) staged in shared
//      memory, then P = delta - (gamma/v) J in place;
//   B. the update operations with the finished rows of earlier levels (L_pq = P_pq inv(D_q),
//      P_pj -= L_pq U_qj, operands from LU), then the Gauss--Jordan inverse of the diagonal
//      block in registers -- every lane its own row, so the 32 rows' operand loads are in
//      flight together;
//   C. the warp stores its 32 rows one after another, each as its two contiguous ranges (L
//      blocks, then inverted diagonal and U blocks), transposed to the column-major factor
//      layout on the way, so the stores are coalesced.
// The arithmetic is k_ilu_factor's operation for operation (ilu_mul_sub, ilu_gj_step), so the
// factors equal the two-kernel path's bit for bit.
template <int kW>
__global__ void __launch_bounds__(64) k_pset32(
    int n, const int* __restrict__ rows, int p0, const int* __restrict__ prow,
    const int* __restrict__ pdiag, const int* __restrict__ ord, const double* __restrict__ invV,
    double gamma, int nC, int nFi, const int* __restrict__ ell, const int* __restrict__ cnb,
    const float4* __restrict__ cna, const int* __restrict__ fslot,
    const float* __restrict__ Whl, const double* __restrict__ Gb, const float4* __restrict__ Sc,
    double g, const int* __restrict__ upd_ptr, const int3* __restrict__ upd,
    const int* __restrict__ plst, const int* __restrict__ pdu, float* __restrict__ LU,
    int* __restrict__ ierr) {
  constexpr int kRow = (kW + 1) * 25;
  __shared__ float stg[2][32][kRow];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = (blockIdx.x * 2 + warp) * 32 + lane;
  float* st = stg[warp][lane];
  int p = 0, s0 = 0, nb = 0, sd = 0;
  if (t < n) {
    // A
    p = rows ? rows[t] : p0 + t;
    s0 = prow[p];
    nb = prow[p + 1] - s0;
    sd = pdiag[p] - s0;
    const int c = ord[p];
    jac_row32<kW>(c, nC, nFi, s0, sd, ell, cnb, cna, fslot, Whl, Gb, Sc, d2f_trunc(g), st);
    const float sc = d2f_trunc(gamma * invV[c]);
    for (int b = 0; b < nb; b++) {
      float* blk = st + 25 * b;
#pragma unroll
      for (int k = 0; k < 25; k++)
        blk[k] = fmaf(-sc, blk[k], (b == sd && k % 6 == 0) ? 1.0f : 0.0f);
    }
    // B
    const int o1 = upd_ptr[p + 1];
    for (int o = upd_ptr[p]; o < o1; o++) {
      const int3 op = upd[o];
      const float* Ab = st + 25 * (op.x - s0);
      const float* B = LU + 25 * (size_t)op.y;  // column-major, finished in earlier levels
      float* dst = st + 25 * ((op.z < 0 ? op.x : op.z) - s0);
      float Bv[25];
#pragma unroll
      for (int k = 0; k < 25; k++) Bv[k] = __ldg(B + k);
#pragma unroll
      for (int i = 0; i < 5; i++) {
        float A[5];
#pragma unroll
        for (int k = 0; k < 5; k++) A[k] = Ab[5 * i + k];
#pragma unroll
        for (int b = 0; b < 5; b++) {
          const float acc = ilu_dot5(A, Bv + 5 * b);
          dst[5 * i + b] = op.z < 0 ? acc : dst[5 * i + b] - acc;
        }
      }
    }
    float D[25];
#pragma unroll
    for (int k = 0; k < 25; k++) D[k] = st[25 * sd + k];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 5; k++) {
      float rk[5];
#pragma unroll
      for (int b = 0; b < 5; b++) rk[b] = D[5 * k + b];
      ok &= rk[k] != 0.0f;
#pragma unroll
      for (int a = 0; a < 5; a++) ilu_gj_step<float>(a, k, rk, D + 5 * a);
    }
    if (!ok) atomicMin(ierr, p + 1);
#pragma unroll
    for (int k = 0; k < 25; k++) st[25 * sd + k] = D[k];
  }
  __syncwarp();
  // C: row r's blocks [0, sd_r) go to the L region at plst, [sd_r, nb_r) to the D/U region at
  // pdu; factor entry (i, j) of a block sits at 5 j + i (column-major), staging at 5 i + j
  for (int rr = 0; rr < 32; rr++) {
    const int nbr = __shfl_sync(0xffffffffu, nb, rr);
    if (nbr == 0) continue;  // row past the end of the level
    const int sdr = __shfl_sync(0xffffffffu, sd, rr);
    const int pr = __shfl_sync(0xffffffffu, p, rr);
    const float* src = stg[warp][rr];
    float* dl = LU + 25 * (size_t)plst[pr];
    float* du = LU + 25 * (size_t)pdu[pr] - 25 * (size_t)sdr;
    for (int e = lane; e < 25 * nbr; e += 32) {
      const int b = e / 25, r = e - 25 * b, i = r % 5, j = r / 5;
      (b < sdr ? dl : du)[e] = src[25 * b + 5 * i + j];
    }
  }
}

// r (FP64 SoA, internal order) -> rv (AoS, 8 per row, position order).  The whole row is
// stored, padding included, in 16-byte stores: full 32-byte sectors, which the L2 writes
// back without first reading the rest of a partly written sector from DRAM.
template <typename TF>
__global__ void k_ilu_in(int nC, const int* __restrict__ ipos, const double* __restrict__ r,
                         TF* __restrict__ rv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nC) return;
  TF v[8];
#pragma unroll
  for (int a = 0; a < 5; a++) v[a] = from64<TF>(r[(size_t)a * nC + i]);
  v[5] = v[6] = v[7] = TF(0);
  TF* dst = rv + 8 * (size_t)ipos[i];
  if constexpr (sizeof(TF) == 4) {
    float4* d = reinterpret_cast<float4*>(dst);
    d[0] = make_float4(v[0], v[1], v[2], v[3]);
    d[1] = make_float4(v[4], v[5], v[6], v[7]);
  } else {
    double2* d = reinterpret_cast<double2*>(dst);
#pragma unroll
    for (int k = 0; k < 4; k++) d[k] = make_double2(v[2 * k], v[2 * k + 1]);
  }
}
// zv (AoS, position order) -> z (FP64 SoA, internal order)
template <typename TF>
__global__ void k_ilu_out(int nC, const int* __restrict__ ipos, const TF* __restrict__ zv,
                          double* __restrict__ z) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nC) return;
  const TF* src = zv + 8 * (size_t)ipos[i];
#pragma unroll
  for (int a = 0; a < 5; a++) z[(size_t)a * nC + i] = to64<TF>(src[a]);
}

// k_ilu_out plus the partial sums of z^2 (the norm the finite-difference Jv of z needs):
// fixed grid (kRedBlocks x kRedThreads), cells by grid stride, one partial per block in a
// fixed order, so the sum is deterministic.  With FP32 factors each thread sums its squares
// in FP32 (the norm only scales the increment s, and the Jv divides by the same s; a
// relative error of ~1e-6 in s is immaterial) and the block sums those partials in FP64:
// no FP64 instruction per element, the pipe GB300 has least of.
template <typename TF>
__global__ void __launch_bounds__(kRedThreads) k_ilu_out_sq(int nC, const int* __restrict__ ipos,
                                                            const TF* __restrict__ zv,
                                                            double* __restrict__ z,
                                                            double* __restrict__ part) {
  TF acc_t = TF(0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nC; i += gridDim.x * blockDim.x) {
    const TF* src = zv + 8 * (size_t)ipos[i];
#pragma unroll
    for (int a = 0; a < 5; a++) {
      const TF v = src[a];
      z[(size_t)a * nC + i] = to64<TF>(v);
      if constexpr (sizeof(TF) == 4) acc_t = fmaf(v, v, acc_t);
      else acc_t = fma(v, v, acc_t);
    }
  }
  double acc = to64<TF>(acc_t);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sh[kRedThreads / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kRedThreads / 32; w++) t += sh[w];
    part[blockIdx.x] = t;
  }
}

// Triangular sweeps in position space, five lanes per block row (lane a owns component
// a and reads row a of every 5x5 block, entries 5 apart in the column-major storage, so
// the five lanes of a row read consecutive floats).  The forward sweep overwrites rv with
// y in place (a row reads only its own rv and earlier rows' y).
//   forward:  y_p = r_p - sum_{q in lower(p)} L_pq y_q           (unit block diagonal)
//   backward: z_p = inv(D_p) (y_p - sum_{q in upper(p)} U_pq z_q)
// z_p = inv(D_p) comp, comp = the row's five components gathered from its lanes; stored with
// the row's padding so that the 32-byte sectors are written whole
template <typename TF>
__device__ __forceinline__ void ilu_diag_store(int lane, int a, bool active, int p, TF acc,
                                               const TF* __restrict__ Dr, TF* __restrict__ zv) {
  TF comp[5];
  const int base = lane - a;
#pragma unroll
  for (int b = 0; b < 5; b++) comp[b] = __shfl_sync(0xffffffffu, acc, base + b < 32 ? base + b : 0);
  if (!active) return;
  TF zz = 0;
#pragma unroll
  for (int b = 0; b < 5; b++) zz += __ldg(Dr + 5 * b) * comp[b];
  zv[8 * (size_t)p + a] = zz;
  if (a < 3) zv[8 * (size_t)p + 5 + a] = TF(0);
}

// a row's neighbour positions, kNW of them (-1 padded), in one or two 16-byte loads
template <int kNW>
__device__ __forceinline__ void load_nbrs(const int* __restrict__ nb, int p, int q[kNW]) {
  const int4* n4 = reinterpret_cast<const int4*>(nb + (size_t)kNW * p);
#pragma unroll
  for (int i = 0; i < kNW / 4; i++) {
    const int4 v = __ldg(n4 + i);
    q[4 * i] = v.x; q[4 * i + 1] = v.y; q[4 * i + 2] = v.z; q[4 * i + 3] = v.w;
  }
}

// kDiag: the level has no U blocks and is also the backward sweep's first level, so the
// launch finishes those rows (z_p = inv(D_p) y_p) instead of storing y_p.  The row's
// neighbours come from the fixed-width list nbL (kNW wide), so the gathers of the earlier
// rows' values wait on one index load, not on a load per column position.
template <typename TF, bool kDiag, int kNW>
__global__ void __launch_bounds__(kT) k_ilu_fwd(int n, const int* __restrict__ rows, int p0,
                                                const int* __restrict__ nbL,
                                                const int* __restrict__ plst,
                                                const int* __restrict__ pdu,
                                                const TF* __restrict__ LU, TF* __restrict__ yv,
                                                TF* __restrict__ zv) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / 5, a = lane - 5 * sub;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 6 + sub;
  const bool active = sub < 6 && t < n;
  if (!kDiag && !active) return;
  const int p = active ? (rows ? rows[t] : p0 + t) : 0;
  TF acc = TF(0);
  if (active) {
    int q[kNW];
    load_nbrs<kNW>(nbL, p, q);
    acc = yv[8 * (size_t)p + a];
    const TF* Lp = LU + 25 * (size_t)plst[p] + a;  // the row's L blocks, in order
#pragma unroll
    for (int k = 0; k < kNW; k++) {
      if (q[k] >= 0) {
        const TF* yq = yv + 8 * (size_t)q[k];
        const TF* B = Lp + 25 * k;
#pragma unroll
        for (int b = 0; b < 5; b++) acc -= __ldg(B + 5 * b) * yq[b];
      }
    }
  }
  if constexpr (kDiag)
    ilu_diag_store(lane, a, active, p, acc, LU + 25 * (size_t)(active ? pdu[p] : 0) + a, zv);
  else
    yv[8 * (size_t)p + a] = acc;
}

template <typename TF, int kNW>
__global__ void __launch_bounds__(kT) k_ilu_bwd(int n, const int* __restrict__ rows, int p0,
                                                const int* __restrict__ nbU,
                                                const int* __restrict__ pdu,
                                                const TF* __restrict__ LU,
                                                const TF* __restrict__ yv, TF* __restrict__ zv) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / 5, a = lane - 5 * sub;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 6 + sub;
  const bool active = sub < 6 && t < n;
  const int p = active ? (rows ? rows[t] : p0 + t) : 0;
  TF acc = TF(0);
  const TF* Dp = LU + a;  // inv(D_p), followed by the row's U blocks in order
  if (active) {
    int q[kNW];
    load_nbrs<kNW>(nbU, p, q);
    acc = yv[8 * (size_t)p + a];
    Dp += 25 * (size_t)pdu[p];
#pragma unroll
    for (int k = 0; k < kNW; k++) {
      if (q[k] >= 0) {
        const TF* zq = zv + 8 * (size_t)q[k];
        const TF* B = Dp + 25 * (k + 1);
#pragma unroll
        for (int b = 0; b < 5; b++) acc -= __ldg(B + 5 * b) * zq[b];
      }
    }
  }
  ilu_diag_store(lane, a, active, p, acc, Dp, zv);
}

}  // namespace

namespace {
inline int nb(long n, int t = kT) { return (int)((n + t - 1) / t); }
inline int nb_rows5(long rows) { return (int)((rows + 6 * (kT / 32) - 1) / (6 * (kT / 32))); }
template <typename T>
int up(T** dst, const std::vector<T>& v) {
  FOS_CUDA(cudaMalloc((void**)dst, std::max<size_t>(v.size(), 1) * sizeof(T)));
  if (!v.empty()) FOS_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}
}  // namespace

// Block sparsity in position space, ILU order, level sets and factor update lists (once).
int fos_jac_setup(fos_ctx* c) {
  if (c->d_prow) return 0;
  const int nC = c->nC, nFi = c->nFi;
  std::vector<int> deg(nC + 1, 0);
  for (int f = 0; f < nFi; f++) {
    deg[c->h_faceL[f] + 1]++;
    deg[c->h_faceR[f] + 1]++;
  }
  for (int i = 0; i < nC; i++) deg[i + 1] += deg[i];
  std::vector<int> adj(deg[nC]);
  {
    std::vector<int> pos(deg.begin(), deg.end() - 1);
    for (int f = 0; f < nFi; f++) {
      adj[pos[c->h_faceL[f]]++] = c->h_faceR[f];
      adj[pos[c->h_faceR[f]]++] = c->h_faceL[f];
    }
  }
  for (int i = 0; i < nC; i++)
    if (deg[i + 1] - deg[i] + 1 > kMaxBlocksPerRow) {
      fos_set_error("fos_jac_setup: a cell has more than 6 neighbours");
      return -2;
    }
  // ILU position of every internal row
  std::vector<int> ipos(nC), ord(nC);
  std::vector<int> cstart;
  c->ilu_colors = 0;
  if (c->flags & FOS_ILU_COLOR) {
    std::vector<int> color(nC, -1);
    int ncol = 0;
    for (int i = 0; i < nC; i++) {
      unsigned used = 0;
      for (int e = deg[i]; e < deg[i + 1]; e++)
        if (color[adj[e]] >= 0 && color[adj[e]] < 32) used |= 1u << color[adj[e]];
      int k = 0;
      while (used & (1u << k)) k++;
      color[i] = k;
      ncol = std::max(ncol, k + 1);
    }
    cstart.assign(ncol + 1, 0);
    for (int i = 0; i < nC; i++) cstart[color[i] + 1]++;
    for (int k = 0; k < ncol; k++) cstart[k + 1] += cstart[k];
    std::vector<int> fill(cstart.begin(), cstart.end() - 1);
    for (int i = 0; i < nC; i++) ipos[i] = fill[color[i]]++;
    c->ilu_colors = ncol;
  } else {
    for (int i = 0; i < nC; i++) ipos[i] = i;
  }
  for (int i = 0; i < nC; i++) ord[ipos[i]] = i;
  c->h_ilu_pos = ipos;
  // block rows in position order, blocks sorted by position
  std::vector<int> prow(nC + 1, 0), pcol, pdiag(nC), cdiag(nC);
  pcol.reserve((size_t)nC + 2 * (size_t)nFi);
  std::vector<int> tmp;
  for (int p = 0; p < nC; p++) {
    const int i = ord[p];
    tmp.clear();
    for (int e = deg[i]; e < deg[i + 1]; e++) tmp.push_back(ipos[adj[e]]);
    tmp.push_back(p);
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    for (int q : tmp) {
      if (q == p) pdiag[p] = (int)pcol.size();
      pcol.push_back(q);
    }
    prow[p + 1] = (int)pcol.size();
  }
  for (int i = 0; i < nC; i++) cdiag[i] = pdiag[ipos[i]];
  c->nnzb = (long)pcol.size();
  auto slot_of = [&](int p, int q) -> int {
    for (int s = prow[p]; s < prow[p + 1]; s++)
      if (pcol[s] == q) return s;
    return -1;
  };
  std::vector<int> fslot(2 * (size_t)nFi);
  for (int f = 0; f < nFi; f++) {
    const int pL = ipos[c->h_faceL[f]], pR = ipos[c->h_faceR[f]];
    fslot[2 * f] = slot_of(pL, pR);
    fslot[2 * f + 1] = slot_of(pR, pL);
  }
  // schedule: colours (contiguous position ranges) or level sets (lists of positions)
  std::vector<int> rows_f, rows_b;
  if (c->ilu_colors) {
    c->lev_f = cstart;
    c->lev_b = cstart;
    c->ilu_nlev_f = c->ilu_nlev_b = c->ilu_colors;
  } else {
    std::vector<int> lf(nC, 0), lb(nC, 0);
    int nlf = 0, nlb = 0;
    for (int p = 0; p < nC; p++) {
      int l = 0;
      for (int s = prow[p]; s < pdiag[p]; s++) l = std::max(l, lf[pcol[s]] + 1);
      lf[p] = l;
      nlf = std::max(nlf, l + 1);
    }
    for (int p = nC - 1; p >= 0; p--) {
      int l = 0;
      for (int s = pdiag[p] + 1; s < prow[p + 1]; s++) l = std::max(l, lb[pcol[s]] + 1);
      lb[p] = l;
      nlb = std::max(nlb, l + 1);
    }
    auto group = [&](const std::vector<int>& lev, int nl, std::vector<int>& ptr,
                     std::vector<int>& rows) {
      ptr.assign(nl + 1, 0);
      for (int p = 0; p < nC; p++) ptr[lev[p] + 1]++;
      for (int l = 0; l < nl; l++) ptr[l + 1] += ptr[l];
      rows.assign(nC, 0);
      std::vector<int> fill(ptr.begin(), ptr.end() - 1);
      for (int p = 0; p < nC; p++) rows[fill[lev[p]]++] = p;
    };
    group(lf, nlf, c->lev_f, rows_f);
    group(lb, nlb, c->lev_b, rows_b);
    c->ilu_nlev_f = nlf;
    c->ilu_nlev_b = nlb;
  }
  c->lev_f_hasL.assign(c->ilu_nlev_f, 0);
  for (int l = 0; l < c->ilu_nlev_f; l++)
    for (int k = c->lev_f[l]; k < c->lev_f[l + 1] && !c->lev_f_hasL[l]; k++) {
      const int p = rows_f.empty() ? k : rows_f[k];
      c->lev_f_hasL[l] = pdiag[p] > prow[p];
    }
  // colours: the forward sweep ends with the top colour and the backward one starts there;
  // a proper colouring leaves its rows without U blocks (checked)
  c->ilu_fuse_top = false;
  if (c->ilu_colors) {
    const int top = c->ilu_colors - 1;
    bool noU = true;
    for (int p = c->lev_f[top]; p < c->lev_f[top + 1] && noU; p++) noU = prow[p + 1] == pdiag[p] + 1;
    c->ilu_fuse_top = noU;
  }
  // factor storage: the L region (every row's L blocks by position), then the D/U region
  std::vector<int> plst(nC), pdu(nC);
  {
    int nl = 0;
    for (int p = 0; p < nC; p++) {
      plst[p] = nl;
      nl += pdiag[p] - prow[p];
    }
    for (int p = 0; p < nC; p++) pdu[p] = nl + (prow[p] - plst[p]);
  }
  // factor update lists (IKJ): for q in lower(p) by position: scale L_pq, then
  // P_pj -= L_pq U_qj for every j in upper(q) that is also in row p
  std::vector<int> upd_ptr(nC + 1, 0);
  std::vector<int3> upd;
  upd.reserve((size_t)nC * 8);
  for (int p = 0; p < nC; p++) {
    for (int s = prow[p]; s < pdiag[p]; s++) {
      const int q = pcol[s];
      upd.push_back(make_int3(s, pdu[q], -1));
      for (int t = pdiag[q] + 1; t < prow[q + 1]; t++) {
        const int sij = slot_of(p, pcol[t]);
        if (sij >= 0) upd.push_back(make_int3(s, pdu[q] + (t - pdiag[q]), sij));
      }
    }
    upd_ptr[p + 1] = (int)upd.size();
  }
  // the sweeps' fixed-width neighbour lists (one or two int4 loads per row instead of a
  // dependent load of every column position)
  {
    int mx = 0;
    for (int p = 0; p < nC; p++)
      mx = std::max(mx, std::max(pdiag[p] - prow[p], prow[p + 1] - pdiag[p] - 1));
    c->ilu_nbw = mx <= 4 ? 4 : 8;
    if (mx > 8) {
      fos_set_error("block ILU(0): a row has more than 8 neighbours");
      return -2;
    }
    const int w = c->ilu_nbw;
    std::vector<int> nbL((size_t)w * nC, -1), nbU((size_t)w * nC, -1);
    for (int p = 0; p < nC; p++) {
      for (int s = prow[p]; s < pdiag[p]; s++) nbL[(size_t)w * p + (s - prow[p])] = pcol[s];
      for (int s = pdiag[p] + 1; s < prow[p + 1]; s++)
        nbU[(size_t)w * p + (s - pdiag[p] - 1)] = pcol[s];
    }
    if (up(&c->d_pnbL, nbL) || up(&c->d_pnbU, nbU)) return -100;
  }
  c->h_prow = prow;
  c->h_pcol = pcol;
  if (up(&c->d_prow, prow) || up(&c->d_pcol, pcol) || up(&c->d_pdiag, pdiag) ||
      up(&c->d_cdiag, cdiag) || up(&c->d_ipos, ipos) || up(&c->d_ord, ord) ||
      up(&c->d_fslot, fslot) || up(&c->d_upd_ptr, upd_ptr) || up(&c->d_upd, upd) ||
      up(&c->d_plst, plst) || up(&c->d_pdu, pdu))
    return -100;
  if (!rows_f.empty() && (up(&c->d_lrows_f, rows_f) || up(&c->d_lrows_b, rows_b))) return -100;
  const bool f32 = (c->flags & FOS_ILU_FP32) != 0;
  const size_t jb = f32 ? sizeof(float) : sizeof(double);
  if (fos_pset_is_fused(c))  // J is assembled inside the factor; only its state is kept
    FOS_CUDA(cudaMalloc((void**)&c->d_yJ, 5 * sizeof(double) * (size_t)nC));
  else
    FOS_CUDA(cudaMalloc((void**)&c->d_Jraw, 25 * jb * (size_t)c->nnzb));
  FOS_CUDA(cudaMalloc((void**)&c->d_Jb, 25 * jb * (size_t)std::max(c->nFb, 1)));
  FOS_CUDA(cudaMalloc((void**)&c->d_ilu_tmp, 16 * sizeof(double) * (size_t)nC));  // 2 AoS vectors
  FOS_CUDA(cudaMalloc((void**)&c->d_ierr, sizeof(int)));
  if (f32)
    FOS_CUDA(cudaMalloc((void**)&c->d_LU32, 25 * sizeof(float) * (size_t)c->nnzb));
  else
    FOS_CUDA(cudaMalloc((void**)&c->d_LU, 25 * sizeof(double) * (size_t)c->nnzb));
  return 0;
}

bool fos_pset_is_fused(const fos_ctx* c) {
  return (c->flags & FOS_ILU_FP32) && !(c->flags & FOS_PREC_ILUT);
}

// storage for J on the fused path, made when J is first asked for (fos_euler_jac_copy /
// fos_euler_jac_set)
static int ensure_jraw(fos_ctx* c) {
  if (c->d_Jraw) return 0;
  const size_t jb = (c->flags & FOS_ILU_FP32) ? sizeof(float) : sizeof(double);
  FOS_CUDA(cudaMalloc((void**)&c->d_Jraw, 25 * jb * (size_t)c->nnzb));
  return 0;
}

template <typename TJ>
static int jac_assemble_t(fos_ctx* c, const double* y) {
  if (int rc = ensure_jraw(c)) return rc;
  TJ* J = reinterpret_cast<TJ*>(c->d_Jraw);
  TJ* Jb = reinterpret_cast<TJ*>(c->d_Jb);
  if constexpr (sizeof(TJ) == sizeof(float)) {
    if (int rc = fos_prim_hl_launch(c, y)) return rc;
    if (c->nFb)
      fos_launch(c, k_jac_ghost64, nb(c->nFb), kT, c->nFi, c->nF, c->nC,
                 (const int2*)c->d_faceLR, (const float4*)c->d_faceNA32, y,
                 (const int*)c->d_bcT, (const double*)c->d_bcP, c->maxP, c->gamm, c->r, c->d_F);
    const int grid = (c->nC + 63) / 64;
    if (c->ell_w == 4)
      fos_launch(c, k_jac_cell32<4>, grid, 64, c->nC, c->nFi, (const int*)c->d_ipos,
                 (const int*)c->d_prow, (const int*)c->d_cdiag, (const int*)c->d_ell,
                 (const int*)c->d_cnb, (const float4*)c->d_cna32, (const int*)c->d_fslot,
                 (const float*)c->d_Whl, (const double*)c->d_F, (const float4*)c->d_closure32,
                 c->gamm, J);
    else
      fos_launch(c, k_jac_cell32<6>, grid, 64, c->nC, c->nFi, (const int*)c->d_ipos,
                 (const int*)c->d_prow, (const int*)c->d_cdiag, (const int*)c->d_ell,
                 (const int*)c->d_cnb, (const float4*)c->d_cna32, (const int*)c->d_fslot,
                 (const float*)c->d_Whl, (const double*)c->d_F, (const float4*)c->d_closure32,
                 c->gamm, J);
    FOS_LAUNCH_CHECK();
    return 0;
  } else {
    if (int rc = fos_prim_launch(c, y)) return rc;
    fos_launch(c, k_jac_face<TJ>, nb(c->nF), kT, c->nFi, c->nF, c->nC,
               (const int2*)c->d_faceLR, (const double2*)c->d_faceNA, (const double*)c->d_W, y,
               (const int*)c->d_fslot, (const int*)c->d_bcT, (const double*)c->d_bcP, c->maxP,
               c->gamm, c->r, J, Jb);
  }
  fos_launch(c, k_jac_diag<TJ>, nb(c->nC), kT, c->nC, c->nFi, (const int*)c->d_crow,
             (const int*)c->d_cent, (const int*)c->d_fslot, (const int*)c->d_cdiag,
             (const TJ*)Jb, J);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_jac_assemble(fos_ctx* c, const double* y) {
  // the FP32 preconditioner is assembled and stored in FP32
  const int rc = (c->flags & FOS_ILU_FP32) ? jac_assemble_t<float>(c, y)
                                           : jac_assemble_t<double>(c, y);
  if (rc) return rc;
  c->has_jac = true;
  c->jraw_valid = true;
  return 0;
}

// The fused FP32 set-up: primitives and boundary ghosts of y, then one k_pset32 launch per
// level (colour) -- J assembled row by row inside the factor, never stored.
int fos_pset_fused(fos_ctx* c, const double* y, double gamma) {
  if (int rc = fos_prim_hl_launch(c, y)) return rc;
  if (c->nFb)
    fos_launch(c, k_jac_ghost64, nb(c->nFb), kT, c->nFi, c->nF, c->nC, (const int2*)c->d_faceLR,
               (const float4*)c->d_faceNA32, y, (const int*)c->d_bcT, (const double*)c->d_bcP,
               c->maxP, c->gamm, c->r, c->d_F);
  const int big = 0x7fffffff;
  FOS_CUDA(cudaMemcpyAsync(c->d_ierr, &big, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  for (int l = 0; l < c->ilu_nlev_f; l++) {
    const int n = c->lev_f[l + 1] - c->lev_f[l];
    const int* rows = c->d_lrows_f ? c->d_lrows_f + c->lev_f[l] : nullptr;
    auto k = c->ell_w == 4 ? k_pset32<4> : k_pset32<6>;
    fos_launch(c, k, (n + 63) / 64, 64, n, rows, c->lev_f[l], (const int*)c->d_prow,
               (const int*)c->d_pdiag, (const int*)c->d_ord, (const double*)c->d_invV, gamma,
               c->nC, c->nFi, (const int*)c->d_ell, (const int*)c->d_cnb,
               (const float4*)c->d_cna32, (const int*)c->d_fslot, (const float*)c->d_Whl,
               (const double*)c->d_F, (const float4*)c->d_closure32, c->gamm,
               (const int*)c->d_upd_ptr, (const int3*)c->d_upd, (const int*)c->d_plst,
               (const int*)c->d_pdu, c->d_LU32, c->d_ierr);
  }
  FOS_LAUNCH_CHECK();
  int* h = (int*)c->h_scal;
  FOS_CUDA(cudaMemcpyAsync(h, c->d_ierr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  c->ilu_ierr = (*h == big) ? 0 : *h;  // 1-based position of the first zero pivot
  c->has_factor = true;
  if (c->ilu_ierr) fos_set_error("block ILU(0): zero pivot");
  return 0;
}

template <typename TF, typename TJ>
static int ilu_factor_t(fos_ctx* c, double gamma, TF* LU) {
  for (int l = 0; l < c->ilu_nlev_f; l++) {
    const int n = c->lev_f[l + 1] - c->lev_f[l];
    const int* rows = c->d_lrows_f ? c->d_lrows_f + c->lev_f[l] : nullptr;
    fos_launch(c, k_ilu_factor<TF, TJ>, nb_rows5(n), kT, n, rows, c->lev_f[l],
               (const int*)c->d_prow, (const int*)c->d_pdiag, (const int*)c->d_ord,
               (const double*)c->d_invV, gamma, (const TJ*)c->d_Jraw, (const int*)c->d_upd_ptr,
               (const int3*)c->d_upd, (const int*)c->d_plst, (const int*)c->d_pdu, LU, c->d_ierr);
  }
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_ilu_factor(fos_ctx* c, double gamma) {
  if (c->flags & FOS_PREC_ILUT) return fos_ilut_ctx_factor(c, gamma);
  const int big = 0x7fffffff;
  FOS_CUDA(cudaMemcpyAsync(c->d_ierr, &big, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  int rc = (c->flags & FOS_ILU_FP32) ? ilu_factor_t<float, float>(c, gamma, c->d_LU32)
                                     : ilu_factor_t<double, double>(c, gamma, c->d_LU);
  if (rc) return rc;
  int* h = (int*)c->h_scal;
  FOS_CUDA(cudaMemcpyAsync(h, c->d_ierr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  c->ilu_ierr = (*h == big) ? 0 : *h;  // 1-based position of the first zero pivot
  c->has_factor = true;
  if (c->ilu_ierr) fos_set_error("block ILU(0): zero pivot");
  return 0;
}

template <typename TF>
static int ilu_apply_t(fos_ctx* c, const TF* LU, const double* r, double* z,
                       double* d_zsq = nullptr) {
  TF* yv = reinterpret_cast<TF*>(c->d_ilu_tmp);
  TF* zv = yv + 8 * (size_t)c->nC;
  fos_launch(c, k_ilu_in<TF>, nb(c->nC, 256), 256, c->nC, (const int*)c->d_ipos, r, yv);
  const int nf = c->ilu_nlev_f;
  for (int l = 0; l < nf; l++) {
    const int n = c->lev_f[l + 1] - c->lev_f[l];
    const int* rows = c->d_lrows_f ? c->d_lrows_f + c->lev_f[l] : nullptr;
    const bool top = c->ilu_fuse_top && l == nf - 1;
    if (!top && !c->lev_f_hasL[l]) continue;  // a level without L blocks keeps y = r
    auto k = top ? (c->ilu_nbw == 4 ? k_ilu_fwd<TF, true, 4> : k_ilu_fwd<TF, true, 8>)
                 : (c->ilu_nbw == 4 ? k_ilu_fwd<TF, false, 4> : k_ilu_fwd<TF, false, 8>);
    fos_launch(c, k, nb_rows5(n), kT, n, rows, c->lev_f[l], (const int*)c->d_pnbL,
               (const int*)c->d_plst, (const int*)c->d_pdu, LU, yv, zv);
  }
  for (int l = c->ilu_fuse_top ? 1 : 0; l < c->ilu_nlev_b; l++) {
    // colours run backwards for the upper sweep
    const int lc = c->ilu_colors ? c->ilu_nlev_b - 1 - l : l;
    const int n = c->lev_b[lc + 1] - c->lev_b[lc];
    const int* rows = c->d_lrows_b ? c->d_lrows_b + c->lev_b[lc] : nullptr;
    fos_launch(c, c->ilu_nbw == 4 ? k_ilu_bwd<TF, 4> : k_ilu_bwd<TF, 8>, nb_rows5(n), kT, n,
               rows, c->lev_b[lc], (const int*)c->d_pnbU, (const int*)c->d_pdu, LU,
               (const TF*)yv, zv);
  }
  if (d_zsq) {
    fos_launch(c, k_ilu_out_sq<TF>, kRedBlocks, kRedThreads, c->nC, (const int*)c->d_ipos,
               (const TF*)zv, z, c->d_red);
    FOS_LAUNCH_CHECK();
    return fos_sum_partials(c, kRedBlocks, d_zsq);
  }
  fos_launch(c, k_ilu_out<TF>, nb(c->nC, 256), 256, c->nC, (const int*)c->d_ipos,
             (const TF*)zv, z);
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_ilu_apply(fos_ctx* c, const double* r, double* z, double* d_zsq) {
  if (c->flags & FOS_PREC_ILUT) {
    if (int rc = fos_ilut_ctx_apply(c, r, z)) return rc;
    return d_zsq ? fos_norm2_dev(c, z, 5L * c->nC, d_zsq) : 0;
  }
  if (c->flags & FOS_ILU_FP32) return ilu_apply_t<float>(c, c->d_LU32, r, z, d_zsq);
  return ilu_apply_t<double>(c, c->d_LU, r, z, d_zsq);
}

// Block Jacobian in position space: rowptr (nC+1) / col (positions) / 25-value blocks.
extern "C" long fos_euler_jac_copy(fos_ctx* c, int* rowptr, int* col, double* val) {
  if (!c) return -1;
  if (fos_jac_setup(c)) return -100;
  if (rowptr) std::memcpy(rowptr, c->h_prow.data(), sizeof(int) * (c->nC + 1));
  if (col) std::memcpy(col, c->h_pcol.data(), sizeof(int) * c->nnzb);
  if (val) {
    if (!c->has_jac) {
      fos_set_error("fos_euler_jac_copy: no Jacobian assembled yet");
      return -2;
    }
    if (!c->jraw_valid) {  // fused set-up: assemble J of the last set-up's state now
      if (jac_assemble_t<float>(c, c->d_yJ)) return -100;
      c->jraw_valid = true;
    }
    const size_t n = 25 * (size_t)c->nnzb;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
      fos_set_error("fos_euler_jac_copy: stream error");
      return -100;
    }
    if (c->flags & FOS_ILU_FP32) {
      std::vector<float> tmp(n);
      if (cudaMemcpy(tmp.data(), c->d_Jraw, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        fos_set_error("fos_euler_jac_copy: copy failed");
        return -100;
      }
      for (size_t k = 0; k < n; k++) val[k] = tmp[k];
    } else if (cudaMemcpy(val, c->d_Jraw, n * sizeof(double), cudaMemcpyDeviceToHost) !=
               cudaSuccess) {
      fos_set_error("fos_euler_jac_copy: copy failed");
      return -100;
    }
  }
  return c->nnzb;
}

// The caller's Jacobian blocks in the layout fos_euler_jac_copy returns (rows and columns by
// ILU position, row-major 5x5 blocks, before scaling by -gamma/v); the next pset with jok = 1
// factors P = I - gamma diag(1/v) J from them.
extern "C" int fos_euler_jac_set(fos_ctx* c, const double* val) {
  if (!c || !val) {
    fos_set_error("fos_euler_jac_set: bad arguments");
    return -1;
  }
  if (c->flags & FOS_PREC_ILUT) {
    fos_set_error("fos_euler_jac_set: not available with FOS_PREC_ILUT");
    return -1;
  }
  if (int rc = fos_jac_setup(c)) return rc;
  if (int rc = ensure_jraw(c)) return rc;
  const size_t n = 25 * (size_t)c->nnzb;
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  if (c->flags & FOS_ILU_FP32) {
    std::vector<float> tmp(n);
    for (size_t k = 0; k < n; k++) tmp[k] = (float)val[k];
    FOS_CUDA(cudaMemcpy(c->d_Jraw, tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  } else {
    FOS_CUDA(cudaMemcpy(c->d_Jraw, val, n * sizeof(double), cudaMemcpyHostToDevice));
  }
  c->has_jac = true;
  c->jraw_valid = true;
  c->jac_user = true;
  return 0;
}

extern "C" int fos_ctx_ilu_order(const fos_ctx* c, int* old2pos) {
  if (!c || !old2pos || c->h_ilu_pos.empty()) {
    fos_set_error("fos_ctx_ilu_order: no factorisation set up yet");
    return -1;
  }
  for (int o = 0; o < c->nC; o++) old2pos[o] = c->h_ilu_pos[c->old2new[o]];
  return c->ilu_colors;
}
