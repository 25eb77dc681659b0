// fos_internal.h -- private declarations shared by the libfosgpu translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fosgpu.h"

#include <cuda_runtime.h>

void fos_set_error(const std::string& msg);

#define FOS_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      fos_set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                 \
      return -100;                                                                       \
    }                                                                                    \
  } while (0)
#define FOS_LAUNCH_CHECK()                                                               \
  do {                                                                                   \
    cudaError_t e_ = cudaGetLastError();                                                 \
    if (e_ != cudaSuccess) {                                                             \
      fos_set_error(std::string("kernel launch: ") + cudaGetErrorString(e_));            \
      return -101;                                                                       \
    }                                                                                    \
  } while (0)

// fixed grid size of the deterministic two-stage reductions (independent of the device)
constexpr int kRedBlocks = 608;  // 4 x 152 SMs
constexpr int kRedThreads = 256;

struct fos_bdf_work;
struct fos_gnn;
void fos_bdf_work_free(fos_bdf_work* w);

struct fos_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // host <-> device state copies run plane by plane on their own stream, each overlapping
  // the permutation of the plane before (created at the first host-buffer call)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_plane[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t ev_sync = nullptr;
  int nC = 0, nE = 0, nPi = 0, nPb = 0, nP = 0, flags = 0;
  int nFi = 0, nFb = 0, nF = 0;  // internal faces: interior first, boundary after
  double gamm = 1.4, r = 1.0;
  int nBC = 0, maxP = 0;
  long bandwidth = 0;
  std::vector<int> old2new, new2old;
  std::vector<int> h_faceL, h_faceR;  // interior faces (internal ids)

  // ---- device grid
  int* d_old2new = nullptr;
  int* d_new2old = nullptr;
  int2* d_faceLR = nullptr;   // [nF] (L, R) internal ids; boundary faces: (L, bc row)
  double2* d_faceNA = nullptr;  // [2*nF] (nx, ny), (nz, aP)
  float4* d_faceNA32 = nullptr; // [nF]  (nx, ny, nz, aP) for the FP32 flux
  int* d_crow = nullptr;      // [nC+1] cell -> face entries
  int* d_cent = nullptr;      // (face << 1) | (cell is R)
  int* d_ell = nullptr;       // [ell_w*nC] the same entries, fixed width, -1 = empty
  // the FP32 flux's and Jacobian's per-cell face slots, so a cell's gathers wait on one
  // index load, not
  // two: [ell_w*nC] the cell across each face (the cell itself for boundary faces and empty
  // slots), and [ell_w][nC] slot-major copies of the faces' FP32 (nx, ny, nz, aP)
  int* d_cnb = nullptr;
  float4* d_cna32 = nullptr;
  int ell_w = 4;
  double* d_invV = nullptr;   // [nC]
  float4* d_closure32 = nullptr;  // [nC] sum of outward aP n over the cell's faces (FP32 flux);
                                  // null when every cell is closed
  unsigned char* d_fsel = nullptr;  // [nF] FOS_FLUX_HYBRID: 1 = face evaluated in FP64 by the
                                    // last residual (interior faces; written by the L cell)
  double hyb_theta = 0.05;          // relative density / pressure jump that selects FP64
  int* d_bcT = nullptr;       // [nBC]
  double* d_bcP = nullptr;    // [maxP*nBC]

  // ---- device work
  double* d_W = nullptr;      // [8*nC] primitive AoS (rho,u,v,w,H,p,sqrt(rho),0)
  float* d_Whl = nullptr;     // [16*nC] FP32 (hi, lo) primitives
  double* d_F = nullptr;      // [6*nF] face flows, AoS
  double* d_stage = nullptr;  // [5*nC] reference-order staging
  double* d_y = nullptr;      // [5*nC] internal-order callback buffers
  double* d_f = nullptr;
  double* d_z = nullptr;
  double* d_red = nullptr;    // [kRedBlocks * 64] reduction partials
  double* d_scal = nullptr;   // [256] device scalars
  int* d_flag = nullptr;      // non-finite flag
  double* h_scal = nullptr;   // pinned [256]

  // ---- Jacobian (block CSR in ILU position order) and ILU(0)
  long nnzb = 0;
  std::vector<int> h_prow, h_pcol;
  int* d_prow = nullptr;      // [nC+1] block rows by position
  int* d_pcol = nullptr;      // [nnzb] column positions, ascending per row
  int* d_pdiag = nullptr;     // [nC] slot of the diagonal block, by position
  int* d_cdiag = nullptr;     // [nC] slot of the diagonal block, by internal cell
  int* d_ipos = nullptr;      // [nC] internal cell -> position
  int* d_ord = nullptr;       // [nC] position -> internal cell
  int* d_fslot = nullptr;     // [2*nFi] slots of blocks (L,R) and (R,L) per interior face
  void* d_Jraw = nullptr;     // [25*nnzb] unscaled Jacobian blocks (FP64, FP32 for FOS_ILU_FP32)
  void* d_Jb = nullptr;       // [25*nFb] boundary-face diagonal terms (same type)
  int* d_ierr = nullptr;
  bool has_jac = false;       // a Jacobian exists for pset(jok = 1): in d_Jraw, or (the fused
                              // FP32 set-up) as the state d_yJ it is assembled from
  bool jraw_valid = false;    // d_Jraw holds that Jacobian
  bool jac_user = false;      // d_Jraw came from fos_euler_jac_set (factored from d_Jraw)
  double* d_yJ = nullptr;     // [5*nC] fused set-up: the state of the last assembly (jok = 0)
  // factors in two regions, so that each sweep streams one: the L blocks of every row (by
  // position), then the diagonal block and the U blocks of every row; diag blocks hold the
  // inverse; 25 entries per block, column-major.  Block storage of slot s in row p:
  // plst[p] + (s - prow[p]) below the diagonal, pdu[p] + (s - pdiag[p]) from it on.
  double* d_LU = nullptr;     // [25*nnzb] factors (FP64)
  float* d_LU32 = nullptr;    // [25*nnzb] factors (FP32)
  // the sweeps' neighbour lists at a fixed width (4, or 8 beyond four neighbours), by
  // position: L neighbours and U neighbours in block order, -1 padded
  int* d_pnbL = nullptr;
  int* d_pnbU = nullptr;
  int ilu_nbw = 4;
  int* d_plst = nullptr;      // [nC] storage block of the first L block of every position
  int* d_pdu = nullptr;       // [nC] storage block of the diagonal block of every position
  int ilu_nlev_f = 0, ilu_nlev_b = 0;
  std::vector<int> lev_f, lev_b;    // level pointers (colour starts when colouring)
  std::vector<char> lev_f_hasL;     // forward level l has L blocks (else y = r there: no launch)
  bool ilu_fuse_top = false;        // the last forward level is the first backward one and
                                    // has no U blocks: one launch forms z = inv(D) y there
  int* d_lrows_f = nullptr;         // level-ordered positions (null when levels are ranges)
  int* d_lrows_b = nullptr;
  int* d_upd_ptr = nullptr;   // [nC+1] per position
  int3* d_upd = nullptr;      // (slot_pq, storage block of inv(D_q) or U_qj, slot_pj or -1)
  int ilu_ierr = 0;
  int ilu_colors = 0;            // > 0: ILU order is colour-major (FOS_ILU_COLOR)
  bool has_factor = false;
  std::vector<int> h_ilu_pos;     // ILU position of every internal row
  double* d_ilu_tmp = nullptr;  // two AoS sweep vectors, 8 values per row each
  fos_bdf_work* bdf = nullptr;  // driver workspace, kept between calls

  // ---- ILUT preconditioner (FOS_PREC_ILUT): scalar CSR of P in ILU position order
  std::vector<double> h_vol;      // cell volumes, internal order
  fos_ilut* ilut = nullptr;
  int ilut_lfil = 50;
  double ilut_droptol = 1e-6;
  int* d_pia = nullptr;           // [5nC+1]
  int* d_pja = nullptr;           // [25 nnzb]
  double* d_pa = nullptr;         // [25 nnzb]
  double* d_vol = nullptr;        // [nC]
  double* d_ilut_x = nullptr;     // [5nC] position-order work vector
  long n_launch = 0;            // kernels launched through fos_launch
  long n_setup = 0;             // preconditioner set-ups (fos_euler_pset_dev calls) so far
  fos_gnn* gnn = nullptr;       // learned preconditioner (not owned)

  ~fos_ctx();
};

// every kernel of the library is launched through this (counts launches per context)
#ifdef __CUDACC__
template <typename... KArgs, typename... Args>
inline void fos_launch(fos_ctx* c, void (*k)(KArgs...), dim3 g, dim3 b, Args... args) {
  c->n_launch++;
  k<<<g, b, 0, c->stream>>>(args...);
}
#endif

// kernels / helpers implemented in fos_residual.cu
int fos_residual_launch(fos_ctx* c, const double* y, const double* v, const double* d_s,
                        const double* fy, double* out, double a, double b, int mode);
int fos_norm2_dev(fos_ctx* c, const double* x, long n, double* d_out_sq);
int fos_sum_partials(fos_ctx* c, int np, double* d_out);  // sum of c->d_red[0..np) in order
int fos_permute(fos_ctx* c, const double* in, double* out, int dir);
// plane q (0..4) only: out + q nC from in + q nC
int fos_permute_plane(fos_ctx* c, const double* in, double* out, int dir, int q);
// host state (reference order) -> device d_internal, and back; the copies run plane by plane
// on the copy stream, overlapped with the permutations on c->stream; d2h leaves c->stream
// waiting for the last copy (synchronise c->stream before reading h)
int fos_h2d_internal(fos_ctx* c, const double* h, double* d_internal);
int fos_d2h_reference(fos_ctx* c, const double* d_internal, double* h);
// s = eps (1 + ynorm)/||v||, 1/s and b/s into d_scal[1..3] (||v||^2 in d_scal[0])
int fos_jv_sigma(fos_ctx* c, double* d_scal, double ynorm, double eps, double b);
int fos_jv_sigma_known(fos_ctx* c, double* d_scal, double ynorm, double vnorm, double eps,
                       double b);
int fos_prim_hl_launch(fos_ctx* c, const double* y);  // FP32 (hi, lo) primitives
int fos_prim_launch(fos_ctx* c, const double* y);
int fos_gnn_precond(fos_ctx* c, const double* y, const double* r, double gamma, double* z);
// fos_jacobian.cu
int fos_jac_setup(fos_ctx* c);
int fos_jac_assemble(fos_ctx* c, const double* y);
// FP32 block ILU(0) without ILUT: pset assembles J inside the factor (k_pset32)
bool fos_pset_is_fused(const fos_ctx* c);
int fos_pset_fused(fos_ctx* c, const double* y, double gamma);
int fos_ilu_factor(fos_ctx* c, double gamma);
// z = P^-1 r; with d_zsq also ||z||^2 into d_zsq (device), from the same pass over z
int fos_ilu_apply(fos_ctx* c, const double* r, double* z, double* d_zsq = nullptr);
// fos_ilut.cu: the Euler preconditioner with ILUT (FOS_PREC_ILUT)
int fos_ilut_ctx_factor(fos_ctx* c, double gamma);
int fos_ilut_ctx_apply(fos_ctx* c, const double* r, double* z);
