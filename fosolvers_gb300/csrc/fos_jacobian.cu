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
__device__ __forceinline__ double nfj(int a, int b, const double n[3], const double u[3], double H,
                                      double g) {
  const double g1 = g - 1.0;
  const double v2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double vn = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
  if (a == 0) return (b >= 1 && b <= 3) ? n[b - 1] : 0.0;
  if (a == 4) {
    if (b == 0) return (0.5 * g1 * v2 - H) * vn;
    if (b == 4) return g * vn;
    return H * n[b - 1] - g1 * u[b - 1] * vn;
  }
  const int i = a - 1;
  if (b == 0) return 0.5 * g1 * v2 * n[i] - u[i] * vn;
  if (b == 4) return g1 * n[i];
  const int j = b - 1;
  return u[i] * n[j] + (1.0 - g) * n[i] * u[j] + (i == j ? vn : 0.0);
}

// eulerANFJ as |vn| T0 + |vn - c| r- l-^T + |vn + c| r+ l+^T (row-major 25)
__device__ __forceinline__ void anfj(const double n[3], const double u[3], double H, double c,
                                     double g, double out[25]) {
  const double g1 = g - 1.0;
  const double v2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double vn = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
  const double ic = 1.0 / c;
  const double M2 = v2 * ic * ic, Mn = vn * ic;
  const double be = g1 * ic * ic;
  const double k1 = 1.0 + 0.5 * g1 * M2;
  const double av = fabs(vn);
  // T0
  out[0] = av * (1.0 - 0.5 * g1 * M2);
  for (int j = 0; j < 3; j++) out[1 + j] = av * (be * u[j]);
  out[4] = av * (-be);
  for (int i = 0; i < 3; i++) {
    out[5 * (1 + i)] = av * (-k1 * u[i] + vn * n[i]);
    for (int j = 0; j < 3; j++)
      out[5 * (1 + i) + 1 + j] = av * (be * u[i] * u[j] - n[i] * n[j] + (i == j ? 1.0 : 0.0));
    out[5 * (1 + i) + 4] = av * (-be * u[i]);
  }
  out[20] = av * (vn * vn - 0.5 * v2 * k1);
  for (int j = 0; j < 3; j++) out[21 + j] = av * (k1 * u[j] - vn * n[j]);
  out[24] = av * (-0.5 * g1 * M2);
#pragma unroll
  for (int sgn = -1; sgn <= 1; sgn += 2) {
    double rr[5], ll[5];
    rr[0] = 1.0;
    for (int i = 0; i < 3; i++) rr[1 + i] = u[i] + sgn * c * n[i];
    rr[4] = H + sgn * vn * c;
    ll[0] = 0.25 * g1 * M2 - sgn * 0.5 * Mn;
    for (int j = 0; j < 3; j++) ll[1 + j] = -0.5 * be * u[j] + sgn * 0.5 * n[j] * ic;
    ll[4] = 0.5 * be;
    const double lam = fabs(vn + sgn * c);
    for (int a = 0; a < 5; a++)
      for (int b = 0; b < 5; b++) out[5 * a + b] += lam * (rr[a] * ll[b]);
  }
}

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
  const double n[3] = {n01.x, n01.y, n2a.x};
  const double aP = n2a.y;
  Prim L, R;
  load_prim(W, lr.x, L);
  if (f < nFi) {
    load_prim(W, lr.y, R);
  } else {
    double U[5], G[5];
    for (int q = 0; q < 5; q++) U[q] = y[(size_t)q * nC + lr.x];
    const int row = lr.y;
    ghost_state(row > 0 ? bcT[row - 1] : FOS_BC_WALL,
                row > 0 ? bcP + (size_t)maxP * (row - 1) : nullptr, U, n[0], n[1], n[2], g, r, G);
    const double inv = 1.0 / G[0];
    R.rho = G[0]; R.u = G[1] * inv; R.v = G[2] * inv; R.w = G[3] * inv;
    R.p = (g - 1.0) * (G[4] - 0.5 * (G[1] * G[1] + G[2] * G[2] + G[3] * G[3]) * inv);
    R.H = (G[4] + R.p) * inv;
    R.s = sqrt(G[0]);
  }
  // Roe averages (Euler.f90:207-209)
  const double inv = 1.0 / (L.s + R.s);
  const double ua[3] = {(L.s * L.u + R.s * R.u) * inv, (L.s * L.v + R.s * R.v) * inv,
                        (L.s * L.w + R.s * R.w) * inv};
  const double Ha = (L.s * L.H + R.s * R.H) * inv;
  const double ca = sqrt((g - 1.0) * (Ha - 0.5 * (ua[0] * ua[0] + ua[1] * ua[1] + ua[2] * ua[2])));
  double Ab[25];
  anfj(n, ua, Ha, ca, g, Ab);
  const double uL[3] = {L.u, L.v, L.w}, uR[3] = {R.u, R.v, R.w};
  const double h = 0.5 * aP;
  if (f < nFi) {
    double* oLR = J + 25 * (size_t)fslot[2 * f];      // block (L, R) = JacP(1:5,6:10)
    double* oRL = J + 25 * (size_t)fslot[2 * f + 1];  // block (R, L) = JacP(6:10,1:5)
    for (int a = 0; a < 5; a++)
      for (int b = 0; b < 5; b++) {
        oLR[5 * a + b] = -h * (nfj(a, b, n, uR, R.H, g) - Ab[5 * a + b]);
        oRL[5 * a + b] = h * (nfj(a, b, n, uL, L.H, g) + Ab[5 * a + b]);
      }
  } else {
    double* d = Jb + 25 * (size_t)(f - nFi);  // boundary pair's diagonal term
    for (int a = 0; a < 5; a++)
      for (int b = 0; b < 5; b++) d[5 * a + b] = -h * (nfj(a, b, n, uL, L.H, g) + Ab[5 * a + b]);
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

// LU = P = I - gamma/v J
__global__ void k_ilu_copy(int nC, const int* __restrict__ rowptr, const int* __restrict__ diag,
                           const double* __restrict__ invV, double gamma,
                           const double* __restrict__ J, double* __restrict__ LU) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nnz25 = 25L * rowptr[nC];
  if (t >= nnz25) return;
  const int slot = (int)(t / 25), k = (int)(t % 25);
  // row of the slot by binary search
  int lo = 0, hi = nC;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (rowptr[mid] <= slot) lo = mid; else hi = mid;
  }
  const double s = gamma * invV[lo];
  double val = -s * J[t];
  if (slot == diag[lo] && (k / 5) == (k % 5)) val += 1.0;
  LU[t] = val;
}

__device__ __forceinline__ void ld25(const double* __restrict__ p, double a[25]) {
#pragma unroll
  for (int k = 0; k < 25; k++) a[k] = p[k];
}

// invert a 5x5 block in place (Gauss--Jordan, partial pivoting); returns false on a zero pivot
__device__ bool inv5(double a[25]) {
  double b[25];
#pragma unroll
  for (int k = 0; k < 25; k++) b[k] = (k / 5 == k % 5) ? 1.0 : 0.0;
  for (int col = 0; col < 5; col++) {
    int piv = col;
    double best = fabs(a[5 * col + col]);
    for (int rr = col + 1; rr < 5; rr++)
      if (fabs(a[5 * rr + col]) > best) { best = fabs(a[5 * rr + col]); piv = rr; }
    if (!(best > 0.0)) return false;
    if (piv != col)
      for (int k = 0; k < 5; k++) {
        double t = a[5 * col + k]; a[5 * col + k] = a[5 * piv + k]; a[5 * piv + k] = t;
        t = b[5 * col + k]; b[5 * col + k] = b[5 * piv + k]; b[5 * piv + k] = t;
      }
    const double ip = 1.0 / a[5 * col + col];
    for (int k = 0; k < 5; k++) { a[5 * col + k] *= ip; b[5 * col + k] *= ip; }
    for (int rr = 0; rr < 5; rr++) {
      if (rr == col) continue;
      const double f = a[5 * rr + col];
      if (f == 0.0) continue;
      for (int k = 0; k < 5; k++) { a[5 * rr + k] -= f * a[5 * col + k]; b[5 * rr + k] -= f * b[5 * col + k]; }
    }
  }
#pragma unroll
  for (int k = 0; k < 25; k++) a[k] = b[k];
  return true;
}

// one level of the block ILU(0) factorisation: thread per row
__global__ void __launch_bounds__(kT) k_ilu_factor_level(int n, const int* __restrict__ rows,
                                                         const int* __restrict__ upd_ptr,
                                                         const int3* __restrict__ upd,
                                                         const int* __restrict__ diag,
                                                         double* __restrict__ LU,
                                                         int* __restrict__ ierr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = rows[t];
  for (int o = upd_ptr[i]; o < upd_ptr[i + 1]; o++) {
    const int3 op = upd[o];
    double A[25], B[25];
    ld25(LU + 25 * (size_t)op.x, A);
    ld25(LU + 25 * (size_t)op.y, B);
    if (op.z < 0) {  // L_ik = A_ik * inv(D_k)
      double* dst = LU + 25 * (size_t)op.x;
      for (int a = 0; a < 5; a++)
        for (int b = 0; b < 5; b++) {
          double s = 0.0;
          for (int k = 0; k < 5; k++) s += A[5 * a + k] * B[5 * k + b];
          dst[5 * a + b] = s;
        }
    } else {  // A_ij -= L_ik U_kj
      double* dst = LU + 25 * (size_t)op.z;
      for (int a = 0; a < 5; a++)
        for (int b = 0; b < 5; b++) {
          double s = dst[5 * a + b];
          for (int k = 0; k < 5; k++) s -= A[5 * a + k] * B[5 * k + b];
          dst[5 * a + b] = s;
        }
    }
  }
  double D[25];
  double* dd = LU + 25 * (size_t)diag[i];
  ld25(dd, D);
  if (!inv5(D)) {
    atomicMin(ierr, i + 1);
    return;
  }
#pragma unroll
  for (int k = 0; k < 25; k++) dd[k] = D[k];
}

__global__ void k_to_f32(long n, const double* __restrict__ a, float* __restrict__ b) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = (float)a[t];
}

// forward sweep of one level: y_i = r_i - sum_{k<i} L_ik y_k  (unit block diagonal)
template <typename TF>
__global__ void __launch_bounds__(kT) k_ilu_fwd(int n, int nC, const int* __restrict__ rows,
                                                const int* __restrict__ rowptr,
                                                const int* __restrict__ col,
                                                const int* __restrict__ diag,
                                                const TF* __restrict__ LU,
                                                const double* __restrict__ r,
                                                double* __restrict__ yv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = rows[t];
  TF acc[5];
#pragma unroll
  for (int q = 0; q < 5; q++) acc[q] = (TF)r[(size_t)q * nC + i];
  for (int s = rowptr[i]; s < diag[i]; s++) {
    const int k = col[s];
    TF yk[5];
#pragma unroll
    for (int q = 0; q < 5; q++) yk[q] = (TF)yv[(size_t)q * nC + k];
    const TF* B = LU + 25 * (size_t)s;
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
      for (int b = 0; b < 5; b++) acc[a] -= B[5 * a + b] * yk[b];
  }
#pragma unroll
  for (int q = 0; q < 5; q++) yv[(size_t)q * nC + i] = (double)acc[q];
}

// backward sweep of one level: z_i = inv(D_i) (y_i - sum_{j>i} U_ij z_j)
template <typename TF>
__global__ void __launch_bounds__(kT) k_ilu_bwd(int n, int nC, const int* __restrict__ rows,
                                                const int* __restrict__ rowptr,
                                                const int* __restrict__ col,
                                                const int* __restrict__ diag,
                                                const TF* __restrict__ LU,
                                                const double* __restrict__ yv,
                                                double* __restrict__ z) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = rows[t];
  TF acc[5];
#pragma unroll
  for (int q = 0; q < 5; q++) acc[q] = (TF)yv[(size_t)q * nC + i];
  for (int s = diag[i] + 1; s < rowptr[i + 1]; s++) {
    const int j = col[s];
    TF zj[5];
#pragma unroll
    for (int q = 0; q < 5; q++) zj[q] = (TF)z[(size_t)q * nC + j];
    const TF* B = LU + 25 * (size_t)s;
#pragma unroll
    for (int a = 0; a < 5; a++)
#pragma unroll
      for (int b = 0; b < 5; b++) acc[a] -= B[5 * a + b] * zj[b];
  }
  const TF* Di = LU + 25 * (size_t)diag[i];
#pragma unroll
  for (int a = 0; a < 5; a++) {
    TF s = 0;
#pragma unroll
    for (int b = 0; b < 5; b++) s += Di[5 * a + b] * acc[b];
    z[(size_t)a * nC + i] = (double)s;
  }
}

}  // namespace

namespace {
inline int nb(long n, int t = kT) { return (int)((n + t - 1) / t); }
template <typename T>
int up(T** dst, const std::vector<T>& v) {
  FOS_CUDA(cudaMalloc((void**)dst, std::max<size_t>(v.size(), 1) * sizeof(T)));
  if (!v.empty()) FOS_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}
}  // namespace

// Block sparsity, level sets and factor update lists (once per context).
int fos_jac_setup(fos_ctx* c) {
  if (c->d_rowptr) return 0;
  const int nC = c->nC, nFi = c->nFi;
  std::vector<std::vector<int>> nbr(nC);
  for (int f = 0; f < nFi; f++) {
    nbr[c->h_faceL[f]].push_back(c->h_faceR[f]);
    nbr[c->h_faceR[f]].push_back(c->h_faceL[f]);
  }
  std::vector<int> rowptr(nC + 1, 0), col, diag(nC);
  col.reserve((size_t)nC + 2 * (size_t)nFi);
  for (int i = 0; i < nC; i++) {
    auto& v = nbr[i];
    v.push_back(i);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    for (int j : v) {
      if (j == i) diag[i] = (int)col.size();
      col.push_back(j);
    }
    rowptr[i + 1] = (int)col.size();
  }
  c->nnzb = (long)col.size();
  auto slot_of = [&](int i, int j) -> int {
    auto b = col.begin() + rowptr[i], e = col.begin() + rowptr[i + 1];
    auto it = std::lower_bound(b, e, j);
    return (it != e && *it == j) ? (int)(it - col.begin()) : -1;
  };
  std::vector<int> fslot(2 * (size_t)nFi);
  for (int f = 0; f < nFi; f++) {
    fslot[2 * f] = slot_of(c->h_faceL[f], c->h_faceR[f]);
    fslot[2 * f + 1] = slot_of(c->h_faceR[f], c->h_faceL[f]);
  }
  // level sets
  std::vector<int> lf(nC, 0), lb(nC, 0);
  int nlf = 0, nlb = 0;
  for (int i = 0; i < nC; i++) {
    int l = 0;
    for (int s = rowptr[i]; s < diag[i]; s++) l = std::max(l, lf[col[s]] + 1);
    lf[i] = l;
    nlf = std::max(nlf, l + 1);
  }
  for (int i = nC - 1; i >= 0; i--) {
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
  // factor update lists (IKJ order): for k in lower(i) ascending: scale L_ik, then
  // A_ij -= L_ik U_kj for every j > k in row k that is also in row i's pattern
  std::vector<int> upd_ptr(nC + 1, 0);
  std::vector<int3> upd;
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
  FOS_CUDA(cudaMalloc((void**)&c->d_LU, 25 * sizeof(double) * (size_t)c->nnzb));
  FOS_CUDA(cudaMalloc((void**)&c->d_Jb, 25 * sizeof(double) * (size_t)std::max(c->nFb, 1)));
  FOS_CUDA(cudaMalloc((void**)&c->d_ilu_tmp, 5 * sizeof(double) * (size_t)nC));
  FOS_CUDA(cudaMalloc((void**)&c->d_ierr, sizeof(int)));
  if (c->flags & FOS_ILU_FP32)
    FOS_CUDA(cudaMalloc((void**)&c->d_LU32, 25 * sizeof(float) * (size_t)c->nnzb));
  return 0;
}

int fos_jac_assemble(fos_ctx* c, const double* y) {
  int rc = fos_prim_launch(c, y);
  if (rc) return rc;
  fos_launch(c, k_jac_face, nb(c->nF), kT, c->nFi, c->nF, c->nC, c->d_faceLR, c->d_faceNA,
                                               c->d_W, y, c->d_fslot, c->d_bcT, c->d_bcP,
                                               c->maxP, c->gamm, c->r, c->d_J, c->d_Jb);
  fos_launch(c, k_jac_diag, nb(c->nC), kT, c->nC, c->nFi, c->d_crow, c->d_cent, c->d_fslot,
                                               c->d_diag, c->d_Jb, c->d_J);
  FOS_LAUNCH_CHECK();
  c->has_jac = true;
  return 0;
}

int fos_ilu_factor(fos_ctx* c, double gamma) {
  const long n25 = 25L * c->nnzb;
  fos_launch(c, k_ilu_copy, nb(n25, 256), 256, c->nC, c->d_rowptr, c->d_diag, c->d_invV,
                                                   gamma, c->d_J, c->d_LU);
  const int big = 0x7fffffff;
  FOS_CUDA(cudaMemcpyAsync(c->d_ierr, &big, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  for (int l = 0; l < c->ilu_nlev_f; l++) {
    const int n = c->lev_f[l + 1] - c->lev_f[l];
    fos_launch(c, k_ilu_factor_level, nb(n), kT, n, c->d_lrows_f + c->lev_f[l], c->d_upd_ptr,
                                                     c->d_upd, c->d_diag, c->d_LU, c->d_ierr);
  }
  FOS_LAUNCH_CHECK();
  if (c->flags & FOS_ILU_FP32)
    fos_launch(c, k_to_f32, nb(n25, 256), 256, n25, c->d_LU, c->d_LU32);
  int* h = (int*)c->h_scal;
  FOS_CUDA(cudaMemcpyAsync(h, c->d_ierr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  c->ilu_ierr = (*h == big) ? 0 : *h;  // 1-based internal row of the first zero pivot
  if (c->ilu_ierr) fos_set_error("block ILU(0): zero pivot");
  return 0;
}

int fos_ilu_apply(fos_ctx* c, const double* r, double* z) {
  double* tmp = c->d_ilu_tmp;
  const bool f32 = (c->flags & FOS_ILU_FP32) != 0;
  for (int l = 0; l < c->ilu_nlev_f; l++) {
    const int n = c->lev_f[l + 1] - c->lev_f[l];
    if (f32)
      fos_launch(c, k_ilu_fwd<float>, nb(n), kT, n, c->nC, c->d_lrows_f + c->lev_f[l],
                                                    c->d_rowptr, c->d_col, c->d_diag, c->d_LU32,
                                                    r, tmp);
    else
      fos_launch(c, k_ilu_fwd<double>, nb(n), kT, n, c->nC, c->d_lrows_f + c->lev_f[l],
                                                     c->d_rowptr, c->d_col, c->d_diag, c->d_LU,
                                                     r, tmp);
  }
  for (int l = 0; l < c->ilu_nlev_b; l++) {
    const int n = c->lev_b[l + 1] - c->lev_b[l];
    if (f32)
      fos_launch(c, k_ilu_bwd<float>, nb(n), kT, n, c->nC, c->d_lrows_b + c->lev_b[l],
                                                    c->d_rowptr, c->d_col, c->d_diag, c->d_LU32,
                                                    tmp, z);
    else
      fos_launch(c, k_ilu_bwd<double>, nb(n), kT, n, c->nC, c->d_lrows_b + c->lev_b[l],
                                                     c->d_rowptr, c->d_col, c->d_diag, c->d_LU,
                                                     tmp, z);
  }
  FOS_LAUNCH_CHECK();
  return 0;
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
