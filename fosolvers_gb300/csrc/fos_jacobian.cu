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
// interleaved matrix), with the inverse of each diagonal block stored in its slot
// like ilu0 stores the inverted diagonal.  Rows are processed level by level:
// the level of a row is one more than the highest level among its lower-triangle
// neighbours (forward) / upper-triangle neighbours (backward), cf. SPARSKIT
// levels (FORMATS/unary.f:1078).  Apply = lusol (ilut.f:2272-2320) in block form.
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

// eulerANFJ as |vn| T0 + |vn - c| r- l-^T + |vn + c| r+ l+^T (row-major 25)
template <typename T>
__device__ __forceinline__ void anfj(const T n[3], const T u[3], T H, T c, T g, T out[25]) {
  const T g1 = g - 1.0;
  const T v2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const T vn = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
  const T ic = T(1) / c;
  const T M2 = v2 * ic * ic, Mn = vn * ic;
  const T be = g1 * ic * ic;
  const T k1 = T(1) + T(0.5) * g1 * M2;
  const T av = fabs(vn);
  // T0
  out[0] = av * (T(1) - T(0.5) * g1 * M2);
  for (int j = 0; j < 3; j++) out[1 + j] = av * (be * u[j]);
  out[4] = av * (-be);
  for (int i = 0; i < 3; i++) {
    out[5 * (1 + i)] = av * (-k1 * u[i] + vn * n[i]);
    for (int j = 0; j < 3; j++)
      out[5 * (1 + i) + 1 + j] = av * (be * u[i] * u[j] - n[i] * n[j] + (i == j ? T(1) : T(0)));
    out[5 * (1 + i) + 4] = av * (-be * u[i]);
  }
  out[20] = av * (vn * vn - T(0.5) * v2 * k1);
  for (int j = 0; j < 3; j++) out[21 + j] = av * (k1 * u[j] - vn * n[j]);
  out[24] = av * (-T(0.5) * g1 * M2);
#pragma unroll
  for (int sgn = -1; sgn <= 1; sgn += 2) {
    T rr[5], ll[5];
    rr[0] = T(1);
    for (int i = 0; i < 3; i++) rr[1 + i] = u[i] + T(sgn) * c * n[i];
    rr[4] = H + T(sgn) * vn * c;
    ll[0] = T(0.25) * g1 * M2 - T(sgn) * T(0.5) * Mn;
    for (int j = 0; j < 3; j++) ll[1 + j] = -T(0.5) * be * u[j] + T(sgn) * T(0.5) * n[j] * ic;
    ll[4] = T(0.5) * be;
    const T lam = fabs(vn + T(sgn) * c);
    for (int a = 0; a < 5; a++)
      for (int b = 0; b < 5; b++) out[5 * a + b] += lam * (rr[a] * ll[b]);
  }
}

template <typename T>
__global__ void __launch_bounds__(kT) k_jac_face(int nFi, int nF, int nC,
                                                 const int2* __restrict__ faceLR,
                                                 const double2* __restrict__ faceNA,
                                                 const double* __restrict__ W,
                                                 const double* __restrict__ y,
                                                 const int* __restrict__ fslot,
                                                 const int* __restrict__ bcT,
                                                 const double* __restrict__ bcP, int maxP,
                                                 double g, double r, double* __restrict__ J,
                                                 double* __restrict__ Jb) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nF) return;
  const int2 lr = faceLR[f];
  const double2 n01 = faceNA[2 * (size_t)f], n2a = faceNA[2 * (size_t)f + 1];
  const T n[3] = {(T)n01.x, (T)n01.y, (T)n2a.x};
  const T aP = (T)n2a.y;
  Prim L, R;
  load_prim(W, lr.x, L);
  if (f < nFi) {
    load_prim(W, lr.y, R);
  } else {
    double U[5], G[5];
    for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + lr.x];
    const int row = lr.y;
    ghost_state(row > 0 ? bcT[row - 1] : FOS_BC_WALL,
                row > 0 ? bcP + (size_t)maxP * (row - 1) : nullptr, U, n01.x, n01.y, n2a.x, g, r, G);
    const double inv = 1.0 / G[0];
    R.rho = G[0]; R.u = G[1] * inv; R.v = G[2] * inv; R.w = G[3] * inv;
    R.p = (g - 1.0) * (G[4] - 0.5 * (G[1] * G[1] + G[2] * G[2] + G[3] * G[3]) * inv);
    R.H = (G[4] + R.p) * inv;
    R.s = sqrt(G[0]);
  }
  // Roe averages (Euler.f90:207-209), arithmetic in T (FP64, or FP32 for the FP32 form)
  const T gg = (T)g;
  const T sL = (T)L.s, sR = (T)R.s;
  const T inv = T(1) / (sL + sR);
  const T ua[3] = {(sL * (T)L.u + sR * (T)R.u) * inv, (sL * (T)L.v + sR * (T)R.v) * inv,
                   (sL * (T)L.w + sR * (T)R.w) * inv};
  const T Ha = (sL * (T)L.H + sR * (T)R.H) * inv;
  const T ca = sqrt((gg - T(1)) * (Ha - T(0.5) * (ua[0] * ua[0] + ua[1] * ua[1] + ua[2] * ua[2])));
  T Ab[25];
  anfj<T>(n, ua, Ha, ca, gg, Ab);
  const T uL[3] = {(T)L.u, (T)L.v, (T)L.w}, uR[3] = {(T)R.u, (T)R.v, (T)R.w};
  const T HL = (T)L.H, HR = (T)R.H;
  const T v2L = uL[0] * uL[0] + uL[1] * uL[1] + uL[2] * uL[2];
  const T vnL = uL[0] * n[0] + uL[1] * n[1] + uL[2] * n[2];
  const T v2R = uR[0] * uR[0] + uR[1] * uR[1] + uR[2] * uR[2];
  const T vnR = uR[0] * n[0] + uR[1] * n[1] + uR[2] * n[2];
  const T h = T(0.5) * aP;
  if (f < nFi) {
    double* oLR = J + 25 * (size_t)fslot[2 * f];      // block (L, R) = JacP(1:5,6:10)
    double* oRL = J + 25 * (size_t)fslot[2 * f + 1];  // block (R, L) = JacP(6:10,1:5)
    for (int a = 0; a < 5; a++)
      for (int b = 0; b < 5; b++) {
        oLR[5 * a + b] = (double)(-h * (nfj<T>(a, b, n, uR, HR, gg, v2R, vnR) - Ab[5 * a + b]));
        oRL[5 * a + b] = (double)(h * (nfj<T>(a, b, n, uL, HL, gg, v2L, vnL) + Ab[5 * a + b]));
      }
  } else {
    double* d = Jb + 25 * (size_t)(f - nFi);  // boundary pair's diagonal term
    for (int a = 0; a < 5; a++)
      for (int b = 0; b < 5; b++)
        d[5 * a + b] = (double)(-h * (nfj<T>(a, b, n, uL, HL, gg, v2L, vnL) + Ab[5 * a + b]));
  }
}

__global__ void __launch_bounds__(kT) k_jac_diag(int nC, int nFi, const int* __restrict__ crow,
                                                 const int* __restrict__ cent,
                                                 const int* __restrict__ fslot,
                                                 const int* __restrict__ diag,
                                                 const double* __restrict__ Jb,
                                                 double* __restrict__ J) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  double D[25];
#pragma unroll
  for (int k = 0; k < 25; k++) D[k] = 0.0;
  for (int e = crow[c]; e < crow[c + 1]; e++) {
    const int ent = cent[e], f = ent >> 1;
    if (f < nFi) {
      // cell is L: diag += JacP(1:5,1:5) = -block(R,L); cell is R: diag += -block(L,R)
      const double* o = J + 25 * (size_t)fslot[2 * f + ((ent & 1) ? 0 : 1)];
#pragma unroll
      for (int k = 0; k < 25; k++) D[k] -= o[k];
    } else {
      const double* o = Jb + 25 * (size_t)(f - nFi);
#pragma unroll
      for (int k = 0; k < 25; k++) D[k] += o[k];
    }
  }
  double* dst = J + 25 * (size_t)diag[c];
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

// One level of the block ILU(0) factorisation, five lanes per block row i (lane a owns
// row a of every block of row i; six rows per warp):
//   LU_i* = P_i* = delta - gamma/v_i J_i*          (copy of the row, fused)
//   for k in lower(i) (ILU order): LU_ik = LU_ik inv(D_k); LU_ij -= LU_ik LU_kj (j in row i)
//   D_i = LU_ii -> inverted by Gauss--Jordan across the five lanes (shuffles)
// A lane only reads its own row of row i's blocks and whole blocks of finished rows, so
// the lanes of a row need no synchronisation until the diagonal inversion.
template <typename TF>
__global__ void __launch_bounds__(kT) k_ilu_factor5(
    int n, const int* __restrict__ rows, const int* __restrict__ rowptr,
    const int* __restrict__ diag, const double* __restrict__ invV, double gamma,
    const double* __restrict__ J, const int* __restrict__ upd_ptr, const int3* __restrict__ upd,
    TF* __restrict__ LU, int* __restrict__ ierr) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / 5, a = lane - 5 * sub;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 6 + sub;
  const bool active = sub < 6 && t < n;
  const int i = active ? rows[t] : 0;
  TF D[5] = {TF(0), TF(0), TF(0), TF(0), TF(0)};
  if (active) {
    const double s = gamma * invV[i];
    for (int sl = rowptr[i]; sl < rowptr[i + 1]; sl++) {
      const double* src = J + 25 * (size_t)sl + 5 * a;
      TF* dst = LU + 25 * (size_t)sl + 5 * a;
      const bool dg = sl == diag[i];
#pragma unroll
      for (int b = 0; b < 5; b++) dst[b] = (TF)(((dg && b == a) ? 1.0 : 0.0) - s * src[b]);
    }
    for (int o = upd_ptr[i]; o < upd_ptr[i + 1]; o++) {
      const int3 op = upd[o];
      TF A[5];
#pragma unroll
      for (int k = 0; k < 5; k++) A[k] = LU[25 * (size_t)op.x + 5 * a + k];
      const TF* B = LU + 25 * (size_t)op.y;
      TF* dst = LU + 25 * (size_t)(op.z < 0 ? op.x : op.z) + 5 * a;
#pragma unroll
      for (int b = 0; b < 5; b++) {
        TF p = 0;
#pragma unroll
        for (int k = 0; k < 5; k++) p += A[k] * B[5 * k + b];
        dst[b] = op.z < 0 ? p : dst[b] - p;
      }
    }
#pragma unroll
    for (int b = 0; b < 5; b++) D[b] = LU[25 * (size_t)diag[i] + 5 * a + b];
  }
  // Gauss--Jordan without pivoting: step k broadcasts row k (lane base + k)
  const int base = lane - a;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 5; k++) {
    TF rk[5];
#pragma unroll
    for (int b = 0; b < 5; b++) rk[b] = __shfl_sync(0xffffffffu, D[b], base + k < 32 ? base + k : 0);
    const TF piv = rk[k];
    ok &= !(active && piv == TF(0));
    const TF ip = TF(1) / piv;
    if (a == k) {
#pragma unroll
      for (int b = 0; b < 5; b++) D[b] = (b == k) ? ip : D[b] * ip;
    } else {
      const TF f = D[k];
#pragma unroll
      for (int b = 0; b < 5; b++) D[b] = (b == k) ? -f * ip : D[b] - f * (rk[b] * ip);
    }
  }
  if (!active) return;
  if (!ok) atomicMin(ierr, i + 1);
#pragma unroll
  for (int b = 0; b < 5; b++) LU[25 * (size_t)diag[i] + 5 * a + b] = D[b];
}

// Triangular sweeps, five lanes per block row (lane a owns component a and reads row a
// of every 5x5 block).  Intermediate vectors are AoS in TF (8 per row, 32 / 64 B), so the
// neighbour values of a row are one sector; r (in) and z (out) are the FP64 SoA vectors.
//   forward:  y_i = r_i - sum_{k in lower(i)} L_ik y_k           (unit block diagonal)
//   backward: z_i = inv(D_i) (y_i - sum_{j in upper(i)} U_ij z_j)
template <typename TF>
__device__ __forceinline__ TF from64(double x) {
  if constexpr (sizeof(TF) == 4) return d2f_trunc(x); else return (TF)x;
}
template <typename TF>
__device__ __forceinline__ double to64(TF x) {
  if constexpr (sizeof(TF) == 4) return f2d_bits(x); else return (double)x;
}

template <typename TF>
__global__ void __launch_bounds__(kT) k_ilu_fwd5(int n, int nC, const int* __restrict__ rows,
                                                 const int* __restrict__ rowptr,
                                                 const int* __restrict__ col,
                                                 const int* __restrict__ diag,
                                                 const TF* __restrict__ LU,
                                                 const double* __restrict__ r,
                                                 TF* __restrict__ yv) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / 5, a = lane - 5 * sub;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 6 + sub;
  if (sub >= 6 || t >= n) return;
  const int i = rows[t];
  TF acc = from64<TF>(r[(size_t)a * nC + i]);
  for (int s = rowptr[i]; s < diag[i]; s++) {
    const TF* yk = yv + 8 * (size_t)col[s];
    const TF* B = LU + 25 * (size_t)s + 5 * a;
#pragma unroll
    for (int b = 0; b < 5; b++) acc -= __ldg(B + b) * yk[b];
  }
  yv[8 * (size_t)i + a] = acc;
}

template <typename TF>
__global__ void __launch_bounds__(kT) k_ilu_bwd5(int n, int nC, const int* __restrict__ rows,
                                                 const int* __restrict__ rowptr,
                                                 const int* __restrict__ col,
                                                 const int* __restrict__ diag,
                                                 const TF* __restrict__ LU,
                                                 const TF* __restrict__ yv,
                                                 TF* __restrict__ zv, double* __restrict__ z) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / 5, a = lane - 5 * sub;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 6 + sub;
  const bool active = sub < 6 && t < n;
  const int i = active ? rows[t] : 0;
  TF acc = TF(0);
  if (active) {
    acc = yv[8 * (size_t)i + a];
    for (int s = diag[i] + 1; s < rowptr[i + 1]; s++) {
      const TF* zj = zv + 8 * (size_t)col[s];
      const TF* B = LU + 25 * (size_t)s + 5 * a;
#pragma unroll
      for (int b = 0; b < 5; b++) acc -= __ldg(B + b) * zj[b];
    }
  }
  TF comp[5];
  const int base = lane - a;
#pragma unroll
  for (int b = 0; b < 5; b++) comp[b] = __shfl_sync(0xffffffffu, acc, base + b < 32 ? base + b : 0);
  if (!active) return;
  const TF* Dr = LU + 25 * (size_t)diag[i] + 5 * a;
  TF zz = 0;
#pragma unroll
  for (int b = 0; b < 5; b++) zz += __ldg(Dr + b) * comp[b];
  zv[8 * (size_t)i + a] = zz;
  z[(size_t)a * nC + i] = to64<TF>(zz);
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

// Block sparsity, ILU order, level sets and factor update lists (once per context).
// Each block row holds its columns sorted by ILU position, so lower(i) = [rowptr, diag)
// and upper(i) = (diag, rowptr+1) in the ILU order (identity = the internal RCM order;
// FOS_ILU_COLOR = greedy colouring of the cell graph, colour-major).
int fos_jac_setup(fos_ctx* c) {
  if (c->d_rowptr) return 0;
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
  // ILU position of every internal row
  std::vector<int> ipos(nC);
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
    std::vector<int> cnt(ncol + 1, 0);
    for (int i = 0; i < nC; i++) cnt[color[i] + 1]++;
    for (int k = 0; k < ncol; k++) cnt[k + 1] += cnt[k];
    for (int i = 0; i < nC; i++) ipos[i] = cnt[color[i]]++;
    c->ilu_colors = ncol;
  } else {
    for (int i = 0; i < nC; i++) ipos[i] = i;
  }
  c->h_ilu_pos = ipos;
  std::vector<int> rowptr(nC + 1, 0), col, diag(nC);
  col.reserve((size_t)nC + 2 * (size_t)nFi);
  std::vector<int> tmp;
  for (int i = 0; i < nC; i++) {
    tmp.assign(adj.begin() + deg[i], adj.begin() + deg[i + 1]);
    tmp.push_back(i);
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    std::sort(tmp.begin(), tmp.end(), [&](int a, int b) { return ipos[a] < ipos[b]; });
    for (int j : tmp) {
      if (j == i) diag[i] = (int)col.size();
      col.push_back(j);
    }
    rowptr[i + 1] = (int)col.size();
  }
  c->nnzb = (long)col.size();
  auto slot_of = [&](int i, int j) -> int {
    for (int s = rowptr[i]; s < rowptr[i + 1]; s++)
      if (col[s] == j) return s;
    return -1;
  };
  std::vector<int> fslot(2 * (size_t)nFi);
  for (int f = 0; f < nFi; f++) {
    fslot[2 * f] = slot_of(c->h_faceL[f], c->h_faceR[f]);
    fslot[2 * f + 1] = slot_of(c->h_faceR[f], c->h_faceL[f]);
  }
  // level sets in the ILU order
  std::vector<int> order(nC);
  for (int i = 0; i < nC; i++) order[ipos[i]] = i;
  std::vector<int> lf(nC, 0), lb(nC, 0);
  int nlf = 0, nlb = 0;
  for (int q = 0; q < nC; q++) {
    const int i = order[q];
    int l = 0;
    for (int s = rowptr[i]; s < diag[i]; s++) l = std::max(l, lf[col[s]] + 1);
    lf[i] = l;
    nlf = std::max(nlf, l + 1);
  }
  for (int q = nC - 1; q >= 0; q--) {
    const int i = order[q];
    int l = 0;
    for (int s = diag[i] + 1; s < rowptr[i + 1]; s++) l = std::max(l, lb[col[s]] + 1);
    lb[i] = l;
    nlb = std::max(nlb, l + 1);
  }
  auto group = [&](const std::vector<int>& lev, int nl, std::vector<int>& ptr, std::vector<int>& rows) {
    ptr.assign(nl + 1, 0);
    for (int i = 0; i < nC; i++) ptr[lev[i] + 1]++;
    for (int l = 0; l < nl; l++) ptr[l + 1] += ptr[l];
    rows.assign(nC, 0);
    std::vector<int> pos(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < nC; i++) rows[pos[lev[i]]++] = i;
  };
  std::vector<int> rows_f, rows_b;
  group(lf, nlf, c->lev_f, rows_f);
  group(lb, nlb, c->lev_b, rows_b);
  c->ilu_nlev_f = nlf;
  c->ilu_nlev_b = nlb;
  // factor update lists (IKJ): for k in lower(i) in ILU order: scale L_ik, then
  // A_ij -= L_ik U_kj for every j in upper(k) that is also in row i
  std::vector<int> upd_ptr(nC + 1, 0);
  std::vector<int3> upd;
  upd.reserve((size_t)nC * 8);
  for (int i = 0; i < nC; i++) {
    for (int s = rowptr[i]; s < diag[i]; s++) {
      const int k = col[s];
      upd.push_back(make_int3(s, diag[k], -1));
      for (int t = diag[k] + 1; t < rowptr[k + 1]; t++) {
        const int sij = slot_of(i, col[t]);
        if (sij >= 0) upd.push_back(make_int3(s, t, sij));
      }
    }
    upd_ptr[i + 1] = (int)upd.size();
  }
  c->h_rowptr = rowptr;
  c->h_col = col;
  if (up(&c->d_rowptr, rowptr) || up(&c->d_col, col) || up(&c->d_diag, diag) ||
      up(&c->d_fslot, fslot) || up(&c->d_lrows_f, rows_f) || up(&c->d_lrows_b, rows_b) ||
      up(&c->d_upd_ptr, upd_ptr) || up(&c->d_upd, upd))
    return -100;
  FOS_CUDA(cudaMalloc((void**)&c->d_J, 25 * sizeof(double) * (size_t)c->nnzb));
  FOS_CUDA(cudaMalloc((void**)&c->d_Jb, 25 * sizeof(double) * (size_t)std::max(c->nFb, 1)));
  FOS_CUDA(cudaMalloc((void**)&c->d_ilu_tmp, 16 * sizeof(double) * (size_t)nC));  // 2 AoS vectors
  FOS_CUDA(cudaMalloc((void**)&c->d_ierr, sizeof(int)));
  if (c->flags & FOS_ILU_FP32)
    FOS_CUDA(cudaMalloc((void**)&c->d_LU32, 25 * sizeof(float) * (size_t)c->nnzb));
  else
    FOS_CUDA(cudaMalloc((void**)&c->d_LU, 25 * sizeof(double) * (size_t)c->nnzb));
  return 0;
}

int fos_jac_assemble(fos_ctx* c, const double* y) {
  int rc = fos_prim_launch(c, y);
  if (rc) return rc;
  if (c->flags & FOS_ILU_FP32)  // the FP32 preconditioner is assembled in FP32
    fos_launch(c, k_jac_face<float>, nb(c->nF), kT, c->nFi, c->nF, c->nC,
               (const int2*)c->d_faceLR, (const double2*)c->d_faceNA, (const double*)c->d_W, y,
               (const int*)c->d_fslot, (const int*)c->d_bcT, (const double*)c->d_bcP, c->maxP,
               c->gamm, c->r, c->d_J, c->d_Jb);
  else
    fos_launch(c, k_jac_face<double>, nb(c->nF), kT, c->nFi, c->nF, c->nC,
               (const int2*)c->d_faceLR, (const double2*)c->d_faceNA, (const double*)c->d_W, y,
               (const int*)c->d_fslot, (const int*)c->d_bcT, (const double*)c->d_bcP, c->maxP,
               c->gamm, c->r, c->d_J, c->d_Jb);
  fos_launch(c, k_jac_diag, nb(c->nC), kT, c->nC, c->nFi, (const int*)c->d_crow,
             (const int*)c->d_cent, (const int*)c->d_fslot, (const int*)c->d_diag,
             (const double*)c->d_Jb, c->d_J);
  FOS_LAUNCH_CHECK();
  c->has_jac = true;
  return 0;
}

int fos_ilu_factor(fos_ctx* c, double gamma) {
  const int big = 0x7fffffff;
  FOS_CUDA(cudaMemcpyAsync(c->d_ierr, &big, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  for (int l = 0; l < c->ilu_nlev_f; l++) {
    const int n = c->lev_f[l + 1] - c->lev_f[l];
    const int* rows = c->d_lrows_f + c->lev_f[l];
    if (c->flags & FOS_ILU_FP32)
      fos_launch(c, k_ilu_factor5<float>, nb_rows5(n), kT, n, rows, (const int*)c->d_rowptr,
                 (const int*)c->d_diag, (const double*)c->d_invV, gamma, (const double*)c->d_J,
                 (const int*)c->d_upd_ptr, (const int3*)c->d_upd, c->d_LU32, c->d_ierr);
    else
      fos_launch(c, k_ilu_factor5<double>, nb_rows5(n), kT, n, rows, (const int*)c->d_rowptr,
                 (const int*)c->d_diag, (const double*)c->d_invV, gamma, (const double*)c->d_J,
                 (const int*)c->d_upd_ptr, (const int3*)c->d_upd, c->d_LU, c->d_ierr);
  }
  FOS_LAUNCH_CHECK();
  int* h = (int*)c->h_scal;
  FOS_CUDA(cudaMemcpyAsync(h, c->d_ierr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  c->ilu_ierr = (*h == big) ? 0 : *h;  // 1-based internal row of the first zero pivot
  c->has_factor = true;
  if (c->ilu_ierr) fos_set_error("block ILU(0): zero pivot");
  return 0;
}

template <typename TF>
static int ilu_apply_t(fos_ctx* c, const TF* LU, const double* r, double* z) {
  TF* yv = reinterpret_cast<TF*>(c->d_ilu_tmp);
  TF* zv = yv + 8 * (size_t)c->nC;
  for (int l = 0; l < c->ilu_nlev_f; l++) {
    const int n = c->lev_f[l + 1] - c->lev_f[l];
    fos_launch(c, k_ilu_fwd5<TF>, nb_rows5(n), kT, n, c->nC,
               (const int*)(c->d_lrows_f + c->lev_f[l]), (const int*)c->d_rowptr,
               (const int*)c->d_col, (const int*)c->d_diag, LU, r, yv);
  }
  for (int l = 0; l < c->ilu_nlev_b; l++) {
    const int n = c->lev_b[l + 1] - c->lev_b[l];
    fos_launch(c, k_ilu_bwd5<TF>, nb_rows5(n), kT, n, c->nC,
               (const int*)(c->d_lrows_b + c->lev_b[l]), (const int*)c->d_rowptr,
               (const int*)c->d_col, (const int*)c->d_diag, LU, (const TF*)yv, zv, z);
  }
  FOS_LAUNCH_CHECK();
  return 0;
}

int fos_ilu_apply(fos_ctx* c, const double* r, double* z) {
  if (c->flags & FOS_ILU_FP32) return ilu_apply_t<float>(c, c->d_LU32, r, z);
  return ilu_apply_t<double>(c, c->d_LU, r, z);
}

extern "C" long fos_euler_jac_copy(fos_ctx* c, int* rowptr, int* col, double* val) {
  if (!c) return -1;
  if (fos_jac_setup(c)) return -100;
  if (rowptr) std::memcpy(rowptr, c->h_rowptr.data(), sizeof(int) * (c->nC + 1));
  if (col) std::memcpy(col, c->h_col.data(), sizeof(int) * c->nnzb);
  if (val) {
    if (!c->has_jac) {
      fos_set_error("fos_euler_jac_copy: no Jacobian assembled yet");
      return -2;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess ||
        cudaMemcpy(val, c->d_J, 25 * sizeof(double) * (size_t)c->nnzb, cudaMemcpyDeviceToHost) !=
            cudaSuccess) {
      fos_set_error("fos_euler_jac_copy: copy failed");
      return -100;
    }
  }
  return c->nnzb;
}

extern "C" int fos_ctx_ilu_order(const fos_ctx* c, int* old2pos) {
  if (!c || !old2pos || c->h_ilu_pos.empty()) {
    fos_set_error("fos_ctx_ilu_order: no factorisation set up yet");
    return -1;
  }
  for (int o = 0; o < c->nC; o++) old2pos[o] = c->h_ilu_pos[c->old2new[o]];
  return c->ilu_colors;
}
