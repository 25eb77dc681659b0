// fos_ctx.cu -- solver context: validation of the reference face arrays, the
// bandwidth-reducing renumbering (reverse Cuthill--McKee), the device layout of
// the grid, and the host-pointer CVODE callbacks (foeuler.f90:349-437).
//
// Device layout (internal cell order after renumbering):
//   state vectors      SoA by variable, 5*nC doubles (N_Vector layout)
//   faceLR  int2[nF]   interior faces (L, R) sorted by (min, max) cell id, then the
//                      boundary faces (L, condition row); L/R keep the reference
//                      orientation (normal points from L to R)
//   faceNA  double2[2*nF]  (nx, ny), (nz, area)
//   crow/cent          per-cell CSR of its faces, entry = face<<1 | (cell is R),
//                      ascending face id (fixed, deterministic summation order)
//   ell    int[4*nC]      the same entries at fixed width (one int4 load per tetrahedron)
//   W      double[8*nC]   per-cell primitives AoS (rho,u,v,w,H,p,sqrt(rho),0)
//   Whl    float[16*nC]   FP32 (hi, lo) primitives for the FP32 flux
//   F      double[6*nF]   per-face flows, AoS (5 + pad) so a gather reads 48 B per face
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "fos_internal.h"

static thread_local std::string g_err;
void fos_set_error(const std::string& msg) { g_err = msg; }
extern "C" const char* fos_last_error(void) { return g_err.c_str(); }

fos_ctx::~fos_ctx() {
  void* ptrs[] = {d_old2new, d_new2old, d_faceLR, d_faceNA, d_faceNA32, d_crow, d_cent, d_invV,
                  d_bcT, d_bcP, d_W, d_Whl, d_ell, d_F, d_stage, d_y, d_f, d_z, d_red, d_scal,
                  d_flag, d_prow, d_pcol, d_pdiag, d_cdiag, d_ipos, d_ord, d_fslot, d_Jraw,
                  d_LU, d_LU32, d_lrows_f, d_lrows_b, d_upd_ptr, d_upd, d_ilu_tmp, d_Jb, d_ierr,
                  d_closure32, d_pia, d_pja, d_pa, d_vol, d_ilut_x, d_plst, d_pdu, d_fsel,
                  d_yJ, d_cnb, d_cna32, d_pnbL, d_pnbU};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h_scal) cudaFreeHost(h_scal);
  for (cudaEvent_t e : ev_plane)
    if (e) cudaEventDestroy(e);
  if (ev_sync) cudaEventDestroy(ev_sync);
  if (copy_stream) cudaStreamDestroy(copy_stream);
  fos_bdf_work_free(bdf);
  fos_ilut_destroy(ilut);
}

namespace {

// reverse Cuthill--McKee over an undirected graph in CSR form
std::vector<int> rcm_order(int n, const std::vector<int>& xadj, const std::vector<int>& adj) {
  std::vector<int> deg(n), order;
  order.reserve(n);
  for (int i = 0; i < n; i++) deg[i] = xadj[i + 1] - xadj[i];
  std::vector<char> seen(n, 0);
  std::vector<int> level(n, -1);
  auto bfs_far = [&](int s, int& ecc) {  // farthest min-degree node from s
    std::vector<int> q{s};
    level.assign(n, -1);
    level[s] = 0;
    for (size_t h = 0; h < q.size(); h++) {
      int u = q[h];
      for (int k = xadj[u]; k < xadj[u + 1]; k++)
        if (level[adj[k]] < 0) {
          level[adj[k]] = level[u] + 1;
          q.push_back(adj[k]);
        }
    }
    ecc = level[q.back()];
    int best = q.back();
    for (int u : q)
      if (level[u] == ecc && (deg[u] < deg[best] || (deg[u] == deg[best] && u < best))) best = u;
    return best;
  };
  std::vector<int> nb;
  for (int root = 0; root < n; root++) {
    if (seen[root]) continue;
    // pseudo-peripheral start (George--Liu)
    int s = root, ecc = 0;
    int t = bfs_far(s, ecc);
    for (int it = 0; it < 8; it++) {
      int e2 = 0;
      int t2 = bfs_far(t, e2);
      if (e2 <= ecc) break;
      s = t; t = t2; ecc = e2;
    }
    s = t;
    size_t head = order.size();
    order.push_back(s);
    seen[s] = 1;
    while (head < order.size()) {
      int u = order[head++];
      nb.clear();
      for (int k = xadj[u]; k < xadj[u + 1]; k++)
        if (!seen[adj[k]]) nb.push_back(adj[k]);
      std::sort(nb.begin(), nb.end(), [&](int a, int b) {
        return deg[a] != deg[b] ? deg[a] < deg[b] : a < b;
      });
      for (int w : nb) {
        seen[w] = 1;
        order.push_back(w);
      }
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

template <typename T>
int upload(T** dst, const T* src, size_t n) {
  FOS_CUDA(cudaMalloc((void**)dst, std::max<size_t>(n, 1) * sizeof(T)));
  if (n) FOS_CUDA(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}
template <typename T>
int dalloc(T** dst, size_t n) {
  FOS_CUDA(cudaMalloc((void**)dst, std::max<size_t>(n, 1) * sizeof(T)));
  FOS_CUDA(cudaMemset(*dst, 0, std::max<size_t>(n, 1) * sizeof(T)));
  return 0;
}

bool supported_bc(int t) {
  return t == FOS_BC_WALL || t == FOS_BC_IN_STATIC || t == FOS_BC_IN_TOTAL || t == FOS_BC_OUT ||
         t == FOS_BC_OUT_EXTRAP || t == FOS_BC_FAR;
}

}  // namespace

#define FOS_TRY(call)          \
  do {                         \
    int rc_ = (call);          \
    if (rc_) {                 \
      delete c;                \
      return rc_;              \
    }                          \
  } while (0)

extern "C" int fos_ctx_create(fos_ctx** out, int nC, int nE, int nPi, int nPb, const int* iEP,
                              const double* aP, const double* normP, const double* v,
                              const int* iBC, int nBC, const int* bcType, const double* bcParam,
                              int maxP, double gamm, double r, int index_base, int flags) {
  if (!out || nC <= 0 || nE < nC || nPi < 0 || nPb < 0 || !iEP || !aP || !normP || !v ||
      (index_base != 0 && index_base != 1) || !(gamm > 1.0) || !(r > 0.0)) {
    fos_set_error("fos_ctx_create: bad arguments");
    return -1;
  }
  if (nBC > 0 && (!bcType || (maxP > 0 && !bcParam))) {
    fos_set_error("fos_ctx_create: condition table missing");
    return -1;
  }
  const int nP = nPi + nPb;
  // ---- validate the pair arrays: interior pairs first, then boundary pairs
  for (int i = 0; i < nP; i++) {
    long m = (long)iEP[2 * i] - index_base, n = (long)iEP[2 * i + 1] - index_base;
    bool ok = i < nPi ? (m >= 0 && m < nC && n >= 0 && n < nC && m != n)
                      : (m >= 0 && m < nC && n >= nC && n < nE);
    if (!ok) {
      fos_set_error("fos_ctx_create: pair " + std::to_string(i) + " has element ids out of range");
      return -2;
    }
    if (!(aP[i] >= 0.0) || !std::isfinite(normP[3 * i]) || !std::isfinite(normP[3 * i + 1]) ||
        !std::isfinite(normP[3 * i + 2])) {
      fos_set_error("fos_ctx_create: pair " + std::to_string(i) + " has bad geometry");
      return -2;
    }
  }
  for (int i = 0; i < nC; i++)
    if (!(v[i] > 0.0)) {
      fos_set_error("fos_ctx_create: cell " + std::to_string(i) + " has non-positive volume");
      return -2;
    }
  for (int k = 0; k < nBC; k++)
    if (!supported_bc(bcType[k])) {
      fos_set_error("fos_ctx_create: condition type " + std::to_string(bcType[k]) +
                    " not supported (UDF conditions need libmatheval)");
      return -3;
    }
  std::vector<int> brow(nPb, 0);
  for (int i = 0; i < nPb; i++) {
    int n = iEP[2 * (nPi + i) + 1] - index_base;
    int row = iBC ? iBC[n] : 0;
    if (row < 0 || row > nBC) {
      fos_set_error("fos_ctx_create: iBC row out of range");
      return -3;
    }
    if (row > 0) {
      int t = bcType[row - 1];
      int need = (t == FOS_BC_OUT) ? 1 : (t == FOS_BC_WALL || t == FOS_BC_OUT_EXTRAP) ? 0 : 5;
      if (maxP < need) {
        fos_set_error("fos_ctx_create: condition table has too few parameters");
        return -3;
      }
    }
    brow[i] = row;
  }

  fos_ctx* c = new fos_ctx();
  c->nC = nC; c->nE = nE; c->nPi = nPi; c->nPb = nPb; c->nP = nP; c->flags = flags;
  c->gamm = gamm; c->r = r; c->nBC = nBC; c->maxP = maxP;
  c->nFi = nPi; c->nFb = nPb; c->nF = nP;
  cudaGetDevice(&c->device);

  // ---- renumbering
  std::vector<int> xadj(nC + 1, 0), adj(2 * (size_t)nPi);
  for (int i = 0; i < nPi; i++) {
    xadj[iEP[2 * i] - index_base + 1]++;
    xadj[iEP[2 * i + 1] - index_base + 1]++;
  }
  for (int i = 0; i < nC; i++) xadj[i + 1] += xadj[i];
  {
    std::vector<int> pos(xadj.begin(), xadj.end() - 1);
    for (int i = 0; i < nPi; i++) {
      int m = iEP[2 * i] - index_base, n = iEP[2 * i + 1] - index_base;
      adj[pos[m]++] = n;
      adj[pos[n]++] = m;
    }
  }
  if (flags & FOS_ORDER_NATURAL) {
    c->new2old.resize(nC);
    std::iota(c->new2old.begin(), c->new2old.end(), 0);
  } else {
    c->new2old = rcm_order(nC, xadj, adj);
  }
  c->old2new.assign(nC, 0);
  for (int i = 0; i < nC; i++) c->old2new[c->new2old[i]] = i;
  long bw = 0;
  for (int i = 0; i < nPi; i++)
    bw = std::max<long>(bw, std::labs((long)c->old2new[iEP[2 * i] - index_base] -
                                      (long)c->old2new[iEP[2 * i + 1] - index_base]));
  c->bandwidth = bw;

  // ---- internal faces
  std::vector<int> forder(nP);
  std::iota(forder.begin(), forder.end(), 0);
  auto keyL = [&](int i) { return c->old2new[iEP[2 * i] - index_base]; };
  auto keyR = [&](int i) { return c->old2new[iEP[2 * i + 1] - index_base]; };
  std::sort(forder.begin(), forder.begin() + nPi, [&](int a, int b) {
    int a0 = std::min(keyL(a), keyR(a)), b0 = std::min(keyL(b), keyR(b));
    if (a0 != b0) return a0 < b0;
    int a1 = std::max(keyL(a), keyR(a)), b1 = std::max(keyL(b), keyR(b));
    if (a1 != b1) return a1 < b1;
    return a < b;
  });
  std::sort(forder.begin() + nPi, forder.end(), [&](int a, int b) {
    if (keyL(a) != keyL(b)) return keyL(a) < keyL(b);
    return a < b;
  });
  std::vector<int2> faceLR(nP);
  std::vector<double2> faceNA(2 * (size_t)nP);
  std::vector<float4> faceNA32(nP);
  for (int f = 0; f < nP; f++) {
    int i = forder[f];
    int L = keyL(i);
    int R = i < nPi ? keyR(i) : brow[i - nPi];
    faceLR[f] = make_int2(L, R);
    if (i < nPi) {
      c->h_faceL.push_back(L);
      c->h_faceR.push_back(R);
    }
    faceNA[2 * f] = make_double2(normP[3 * i], normP[3 * i + 1]);
    faceNA[2 * f + 1] = make_double2(normP[3 * i + 2], aP[i]);
    faceNA32[f] = make_float4((float)normP[3 * i], (float)normP[3 * i + 1],
                              (float)normP[3 * i + 2], (float)aP[i]);
  }
  std::vector<int> crow(nC + 1, 0), cent;
  for (int f = 0; f < nP; f++) {
    crow[faceLR[f].x + 1]++;
    if (f < nPi) crow[faceLR[f].y + 1]++;
  }
  for (int i = 0; i < nC; i++) crow[i + 1] += crow[i];
  cent.resize(crow[nC]);
  {
    std::vector<int> pos(crow.begin(), crow.end() - 1);
    for (int f = 0; f < nP; f++) {  // ascending f: entries end up sorted by face id
      cent[pos[faceLR[f].x]++] = f << 1;
      if (f < nPi) cent[pos[faceLR[f].y]++] = (f << 1) | 1;
    }
  }
  // ELL copy of the per-cell entries (fixed width: 4 for tetrahedra, 6 for hexahedra)
  int maxe = 0;
  for (int i = 0; i < nC; i++) maxe = std::max(maxe, crow[i + 1] - crow[i]);
  if (maxe > 6) {
    fos_set_error("fos_ctx_create: a cell has more than 6 faces");
    delete c;
    return -2;
  }
  c->ell_w = maxe <= 4 ? 4 : 6;
  std::vector<int> ell((size_t)c->ell_w * nC, -1);
  for (int i = 0; i < nC; i++)
    for (int e = crow[i]; e < crow[i + 1]; e++) ell[(size_t)c->ell_w * i + (e - crow[i])] = cent[e];
  std::vector<double> invV(nC);
  for (int i = 0; i < nC; i++) invV[c->old2new[i]] = 1.0 / v[i];
  c->h_vol.resize(nC);
  for (int i = 0; i < nC; i++) c->h_vol[c->old2new[i]] = v[i];
  // closure vector of every cell, sum over its faces of the outward aP n.  The FP32 flux
  // writes each face flow as the cell's own flux aP F(u_c).n plus a difference and drops the
  // own-flux part, whose sum is F(u_c).S_c: zero for cells with planar faces, not for
  // hexahedra with warped faces (the quad area vectors do not close), where it is restored
  std::vector<double> S(3 * (size_t)nC, 0.0);
  double amax = 0.0;
  for (int f = 0; f < nP; f++) {
    const double* an = &faceNA[2 * (size_t)f].x;  // nx, ny, nz, aP
    const double a = an[3];
    amax = std::max(amax, a);
    for (int d = 0; d < 3; d++) {
      S[3 * (size_t)faceLR[f].x + d] += a * an[d];
      if (f < nPi) S[3 * (size_t)faceLR[f].y + d] -= a * an[d];
    }
  }
  double smax = 0.0;
  for (double x : S) smax = std::max(smax, std::fabs(x));
  if (smax > 1e-12 * amax) {
    std::vector<float4> S32(nC);
    for (int i = 0; i < nC; i++)
      S32[i] = make_float4((float)S[3 * (size_t)i], (float)S[3 * (size_t)i + 1],
                           (float)S[3 * (size_t)i + 2], 0.0f);
    FOS_TRY(upload(&c->d_closure32, S32.data(), nC));
  }

  FOS_TRY(upload(&c->d_old2new, c->old2new.data(), nC));
  FOS_TRY(upload(&c->d_new2old, c->new2old.data(), nC));
  FOS_TRY(upload(&c->d_faceLR, faceLR.data(), nP));
  FOS_TRY(upload(&c->d_faceNA, faceNA.data(), 2 * (size_t)nP));
  FOS_TRY(upload(&c->d_faceNA32, faceNA32.data(), nP));
  FOS_TRY(upload(&c->d_crow, crow.data(), nC + 1));
  FOS_TRY(upload(&c->d_cent, cent.data(), cent.size()));
  FOS_TRY(upload(&c->d_ell, ell.data(), ell.size()));
  if (flags & (FOS_FLUX_FP32 | FOS_ILU_FP32)) {  // per-cell face slots of the FP32 flux and
                                                // Jacobian (copies of face data)
    const int w = c->ell_w;
    std::vector<int> cnb((size_t)w * nC);
    std::vector<float4> cna((size_t)w * nC, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int i = 0; i < nC; i++)
      for (int k = 0; k < w; k++) {
        const int e = ell[(size_t)w * i + k];
        int nb = i;
        if (e >= 0) {
          const int f = e >> 1;
          if (f < nPi) nb = (e & 1) ? faceLR[f].x : faceLR[f].y;
          cna[(size_t)k * nC + i] = faceNA32[f];
        }
        cnb[(size_t)w * i + k] = nb;
      }
    FOS_TRY(upload(&c->d_cnb, cnb.data(), cnb.size()));
    FOS_TRY(upload(&c->d_cna32, cna.data(), cna.size()));
  }
  FOS_TRY(dalloc(&c->d_Whl, 16 * (size_t)nC));
  if (flags & FOS_FLUX_HYBRID) {
    FOS_TRY(dalloc(&c->d_fsel, (size_t)nP));
    FOS_TRY(cudaMemset(c->d_fsel, 0, (size_t)nP) == cudaSuccess ? 0 : -100);
  }
  FOS_TRY(upload(&c->d_invV, invV.data(), nC));
  FOS_TRY(upload(&c->d_bcT, bcType, nBC));
  FOS_TRY(upload(&c->d_bcP, bcParam, (size_t)maxP * nBC));
  FOS_TRY(dalloc(&c->d_W, 8 * (size_t)nC));
  FOS_TRY(dalloc(&c->d_F, 6 * (size_t)nP));  // AoS flows, 48 B per face (FP64 or 2 x FP32)
  FOS_TRY(dalloc(&c->d_stage, 5 * (size_t)nC));
  FOS_TRY(dalloc(&c->d_y, 5 * (size_t)nC));
  FOS_TRY(dalloc(&c->d_f, 5 * (size_t)nC));
  FOS_TRY(dalloc(&c->d_z, 5 * (size_t)nC));
  FOS_TRY(dalloc(&c->d_red, (size_t)kRedBlocks * 64));
  FOS_TRY(dalloc(&c->d_scal, 256));
  FOS_TRY(dalloc(&c->d_flag, 4));
  if (cudaMallocHost((void**)&c->h_scal, 256 * sizeof(double)) != cudaSuccess) {
    fos_set_error("fos_ctx_create: cudaMallocHost failed");
    delete c;
    return -100;
  }
  *out = c;
  return 0;
}

extern "C" void fos_ctx_destroy(fos_ctx* ctx) { delete ctx; }

extern "C" int fos_ctx_set_flux_threshold(fos_ctx* ctx, double theta) {
  if (!ctx || !(theta > 0.0) || !(ctx->flags & FOS_FLUX_HYBRID)) {
    fos_set_error("fos_ctx_set_flux_threshold: bad arguments or no FOS_FLUX_HYBRID");
    return -1;
  }
  ctx->hyb_theta = theta;
  return 0;
}

extern "C" int fos_ctx_set_stream(fos_ctx* ctx, void* stream) {
  if (!ctx) return -1;
  ctx->stream = (cudaStream_t)stream;
  return 0;
}

extern "C" void fos_ctx_info(const fos_ctx* c, long* out) {
  out[0] = c->nC; out[1] = c->nPi; out[2] = c->nPb; out[3] = c->ilu_nlev_f;
  out[4] = c->ilu_nlev_b; out[5] = c->nnzb; out[6] = c->bandwidth; out[7] = c->flags;
  out[8] = c->n_launch;
}

extern "C" int fos_ctx_renumbering(const fos_ctx* c, int* old2new) {
  if (!c || !old2new) return -1;
  std::memcpy(old2new, c->old2new.data(), sizeof(int) * c->nC);
  return 0;
}

extern "C" int fos_ctx_permute_dev(fos_ctx* c, const double* in, double* out, int dir) {
  if (!c || !in || !out || in == out) {
    fos_set_error("fos_ctx_permute_dev: bad arguments (in-place not supported)");
    return -1;
  }
  return fos_permute(c, in, out, dir);
}

// ------------------------------------------------------------------ host callbacks
namespace {
int ensure_copy_stream(fos_ctx* c) {
  if (c->copy_stream) return 0;
  FOS_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  for (cudaEvent_t& e : c->ev_plane)
    FOS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  FOS_CUDA(cudaEventCreateWithFlags(&c->ev_sync, cudaEventDisableTiming));
  return 0;
}
}  // namespace

// Five planes (one per conserved variable): the copy of plane q + 1 runs while plane q is
// permuted, so only one plane's permutation is not hidden behind the copies.
int fos_h2d_internal(fos_ctx* c, const double* h, double* d_internal) {
  if (int rc = ensure_copy_stream(c)) return rc;
  const size_t n = (size_t)c->nC;
  // the staging buffer is free once the work queued so far on c->stream is done
  FOS_CUDA(cudaEventRecord(c->ev_sync, c->stream));
  FOS_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_sync, 0));
  for (int q = 0; q < 5; q++) {
    FOS_CUDA(cudaMemcpyAsync(c->d_stage + q * n, h + q * n, sizeof(double) * n,
                             cudaMemcpyHostToDevice, c->copy_stream));
    FOS_CUDA(cudaEventRecord(c->ev_plane[q], c->copy_stream));
    FOS_CUDA(cudaStreamWaitEvent(c->stream, c->ev_plane[q], 0));
    if (int rc = fos_permute_plane(c, c->d_stage, d_internal, 0, q)) return rc;
  }
  return 0;
}
int fos_d2h_reference(fos_ctx* c, const double* d_internal, double* h) {
  if (int rc = ensure_copy_stream(c)) return rc;
  const size_t n = (size_t)c->nC;
  for (int q = 0; q < 5; q++) {
    if (int rc = fos_permute_plane(c, d_internal, c->d_stage, 1, q)) return rc;
    FOS_CUDA(cudaEventRecord(c->ev_plane[q], c->stream));
    FOS_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_plane[q], 0));
    FOS_CUDA(cudaMemcpyAsync(h + q * n, c->d_stage + q * n, sizeof(double) * n,
                             cudaMemcpyDeviceToHost, c->copy_stream));
  }
  // later work on c->stream (and a synchronisation of it) comes after the copies
  FOS_CUDA(cudaEventRecord(c->ev_sync, c->copy_stream));
  FOS_CUDA(cudaStreamWaitEvent(c->stream, c->ev_sync, 0));
  return 0;
}

extern "C" int fos_euler_rhs(double t, const double* y, double* ydot, void* user_data) {
  (void)t;
  fos_ctx* c = (fos_ctx*)user_data;
  if (!c || !y || !ydot) {
    fos_set_error("fos_euler_rhs: bad arguments");
    return -1;
  }
  int rc = fos_h2d_internal(c, y, c->d_y);
  if (rc) return rc;
  FOS_CUDA(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
  rc = fos_residual_launch(c, c->d_y, nullptr, nullptr, nullptr, c->d_f, 0.0, 0.0, 0);
  if (rc) return rc;
  rc = fos_d2h_reference(c, c->d_f, ydot);
  if (rc) return rc;
  int* hflag = (int*)c->h_scal;
  FOS_CUDA(cudaMemcpyAsync(hflag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  return *hflag ? 1 : 0;  // non-finite residual: recoverable, CVODE retries with a smaller step
}

extern "C" int fos_euler_rhs_dev(fos_ctx* c, double t, const double* y, double* ydot) {
  (void)t;
  if (!c || !y || !ydot) {
    fos_set_error("fos_euler_rhs_dev: bad arguments");
    return -1;
  }
  return fos_residual_launch(c, y, nullptr, nullptr, nullptr, ydot, 0.0, 0.0, 0);
}

extern "C" int fos_euler_jv_dev(fos_ctx* c, double t, const double* y, const double* fy,
                                const double* v, double* out, double a, double b, double ynorm,
                                double eps) {
  (void)t;
  if (!c || !y || !fy || !v || !out) {
    fos_set_error("fos_euler_jv_dev: bad arguments");
    return -1;
  }
  // s = eps (1 + ||y||) / ||v|| evaluated on the device (scal[0] = ||v||^2, scal[1] = s)
  int rc = fos_norm2_dev(c, v, 5L * c->nC, c->d_scal);
  if (rc) return rc;
  rc = fos_jv_sigma(c, c->d_scal, ynorm, eps, b);
  if (rc) return rc;
  return fos_residual_launch(c, y, v, c->d_scal + 1, fy, out, a, b, 1);
}

extern "C" int fos_euler_jv_dev_vnorm(fos_ctx* c, double t, const double* y, const double* fy,
                                      const double* v, double* out, double a, double b,
                                      double ynorm, double vnorm, double eps) {
  (void)t;
  if (!c || !y || !fy || !v || !out || !(vnorm >= 0.0)) {
    fos_set_error("fos_euler_jv_dev_vnorm: bad arguments");
    return -1;
  }
  int rc = fos_jv_sigma_known(c, c->d_scal, ynorm, vnorm, eps, b);
  if (rc) return rc;
  return fos_residual_launch(c, y, v, c->d_scal + 1, fy, out, a, b, 1);
}

extern "C" int fos_euler_pset(double t, const double* y, const double* fy, int jok, int* jcur,
                              double gamma, void* user_data) {
  (void)fy;
  fos_ctx* c = (fos_ctx*)user_data;
  if (!c || !y) {
    fos_set_error("fos_euler_pset: bad arguments");
    return -1;
  }
  int rc = fos_h2d_internal(c, y, c->d_y);
  if (rc) return rc;
  rc = fos_euler_pset_dev(c, t, c->d_y, jok, jcur, gamma);
  if (rc) return rc;
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  return c->ilu_ierr ? 1 : 0;
}

extern "C" int fos_euler_psol(double t, const double* y, const double* fy, const double* r,
                              double* z, double gamma, double delta, int lr, void* user_data) {
  (void)t; (void)y; (void)fy; (void)gamma; (void)delta; (void)lr;
  fos_ctx* c = (fos_ctx*)user_data;
  if (!c || !r || !z) {
    fos_set_error("fos_euler_psol: bad arguments");
    return -1;
  }
  int rc = fos_h2d_internal(c, r, c->d_y);
  if (rc) return rc;
  rc = fos_euler_psol_dev(c, c->d_y, c->d_z);
  if (rc) return rc;
  rc = fos_d2h_reference(c, c->d_z, z);
  if (rc) return rc;
  FOS_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int fos_euler_pset_dev(fos_ctx* c, double t, const double* y, int jok, int* jcur,
                                  double gamma) {
  (void)t;
  if (!c || !y) {
    fos_set_error("fos_euler_pset_dev: bad arguments");
    return -1;
  }
  int rc = fos_jac_setup(c);
  if (rc) return rc;
  c->n_setup++;
  if (fos_pset_is_fused(c)) {
    // J is assembled inside the factor; jok = 1 reassembles it from the state of the last
    // jok = 0 call (the same J, bit for bit), or factors the caller's J (fos_euler_jac_set)
    if (jok == 0 || !c->has_jac) {
      FOS_CUDA(cudaMemcpyAsync(c->d_yJ, y, 5 * sizeof(double) * (size_t)c->nC,
                               cudaMemcpyDeviceToDevice, c->stream));
      c->has_jac = true;
      c->jraw_valid = false;
      c->jac_user = false;
      if (jcur) *jcur = 1;
      return fos_pset_fused(c, y, gamma);
    }
    if (jcur) *jcur = 0;
    return c->jac_user ? fos_ilu_factor(c, gamma) : fos_pset_fused(c, c->d_yJ, gamma);
  }
  if (jok == 0 || !c->has_jac) {
    rc = fos_jac_assemble(c, y);
    if (rc) return rc;
    if (jcur) *jcur = 1;
  } else if (jcur) {
    *jcur = 0;
  }
  return fos_ilu_factor(c, gamma);
}

extern "C" int fos_euler_psol_dev(fos_ctx* c, const double* r, double* z) {
  if (!c || !r || !z) {
    fos_set_error("fos_euler_psol_dev: bad arguments");
    return -1;
  }
  if (!c->has_factor) {
    fos_set_error("fos_euler_psol_dev: no factorisation (call pset first)");
    return -2;
  }
  return fos_ilu_apply(c, r, z);
}
