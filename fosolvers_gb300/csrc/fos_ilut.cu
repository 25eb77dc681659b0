// fos_ilut.cu -- dual-threshold incomplete LU (ILUT) on the device.
//
// The reference's ILU class (numerics/sparse.f90:52-63,334-392) factors a CSR matrix with
// SPARSKIT's ilut (ITSOL/ilut.f:38-382) and applies it with lusol (:2272-2320).  Here the
// same algorithm runs one warp per row:
//
//   factor  rows are claimed in increasing order from an atomic ticket.  A row's working
//           copy (L part, U part, and a column -> position hash) lives in shared memory;
//           its L entries are eliminated in increasing column order, each waiting (bounded
//           spin) until the pivot row's own warp has published it.  A warp only waits on
//           rows whose tickets were taken before its own, by warps that are running, so the
//           wait always ends.  Every floating-point operation of a row is the one ilut
//           performs, in the same order, with the FMA contraction ilut does not have
//           written out (__dmul_rn / __dsub_rn): given the same CSR the factors are
//           bit-identical to SPARSKIT's.  Fill-in positions follow ilut's append order
//           (ballot prefix counts), and the quick-split runs on one lane.
//   solve   the forward and backward sweeps of lusol, rows claimed level by level of the L
//           and U dependency graphs, each unknown published by its own store and polled by
//           the rows that read it; the row sum is a fixed-order warp reduction.
//
// Storage: every row owns lfil slots for L and lfil for U (ilut keeps at most lfil L and
// lfil - 1 off-diagonal U entries per row), so the factor storage never runs out (the
// reference's -2 / -3); rows longer than the shared-memory working capacity are redone
// with a larger capacity.
#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "fos_internal.h"

struct fos_ilut {
  int n = 0, lfil = 0, device = 0;
  int* d_Lcol = nullptr;
  double* d_Lval = nullptr;
  int* d_Lcnt = nullptr;
  int* d_Ucol = nullptr;
  double* d_Uval = nullptr;
  int* d_Ucnt = nullptr;
  double* d_dinv = nullptr;
  int* d_done = nullptr;   // factor: epoch of the factorisation that published the row
  double* d_z = nullptr;   // forward-sweep result (kPending before each solve)
  int* d_levL = nullptr;   // level of every row in the L graph, published by the factor
  int* d_permF = nullptr;  // rows by forward / backward level: the solves' claim order
  int* d_permB = nullptr;
  int nlevF = 0, nlevB = 0;
  int* d_ctr = nullptr;    // [0] factor ticket [1] forward [2] backward [3] error [4] error row
  int* h_ctr = nullptr;    // pinned copy
  int fepoch = 0;
  int cap = 256;           // working-row capacity (entries of L and of U)
  long spin_limit = 0;     // polls of one dependency wait before giving up (0: kSpinLimit)
  int withhold = -1;       // failure injection: a row that is never published (-1: none)
  bool factored = false;
  long launches = 0;
  ~fos_ilut();
};

fos_ilut::~fos_ilut() {
  void* p[] = {d_Lcol, d_Lval, d_Lcnt, d_Ucol, d_Uval, d_Ucnt, d_dinv, d_done, d_z,
               d_levL, d_permF, d_permB, d_ctr};
  for (void* q : p)
    if (q) cudaFree(q);
  if (h_ctr) cudaFreeHost(h_ctr);
}

namespace {

constexpr int kWarps = 4;                 // warps (rows in flight) per CTA
constexpr long kSpinLimit = 1L << 23;     // polls of a dependency flag before giving up
constexpr int kErrCapacity = -1, kErrZeroRow = -5, kErrTimeout = -6;

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Spin until flag[j] >= epoch; false when the limit ran out or another warp already gave
// up (the error word is set), so no wait outlives a failure.
__device__ __forceinline__ bool wait_row(const int* flag, int j, int epoch, int* ctr, long spin) {
  for (long it = 0; it < spin; it++) {
    if (ld_acquire(flag + j) >= epoch) return true;
    if (*(volatile int*)(ctr + 3) == kErrTimeout) return false;
    if (it > 8) __nanosleep(32);
  }
  atomicCAS(ctr + 3, 0, kErrTimeout);
  return false;
}

__device__ __forceinline__ void set_error(int* ctr, int code, int row) {
  if (atomicCAS(ctr + 3, 0, code) == 0) ctr[4] = row;
}

// column -> position hash of a working row; L positions are stored as ~pos
__device__ __forceinline__ unsigned hslot(int key, unsigned mask) {
  return ((unsigned)key * 2654435761u) & mask;
}
__device__ __forceinline__ bool hfind(const int* hkey, const int* hpos, unsigned mask, int key,
                                      int& pos, unsigned& slot) {
  unsigned s = hslot(key, mask);
  for (;;) {
    const int k = hkey[s];
    if (k == key) { pos = hpos[s]; slot = s; return true; }
    if (k < 0) return false;
    s = (s + 1) & mask;
  }
}
__device__ __forceinline__ void hinsert(int* hkey, int* hpos, unsigned mask, int key, int pos) {
  unsigned s = hslot(key, mask);
  for (;;) {
    const int prev = atomicCAS(hkey + s, -1, key);
    if (prev < 0 || prev == key) { hpos[s] = pos; return; }
    s = (s + 1) & mask;
  }
}

// SPARSKIT qsplit (ilut.f:2376-2434) on one lane: the ncut largest |a| first.
__device__ __forceinline__ void qsplit(double* a, int* ind, int n, int ncut) {
  int first = 0, last = n - 1;
  const int cut = ncut - 1;
  if (cut < first || cut > last) return;
  for (;;) {
    int mid = first;
    const double key = fabs(a[mid]);
    for (int j = first + 1; j <= last; j++)
      if (fabs(a[j]) > key) {
        mid++;
        const double t = a[mid]; a[mid] = a[j]; a[j] = t;
        const int it = ind[mid]; ind[mid] = ind[j]; ind[j] = it;
      }
    const double t = a[mid]; a[mid] = a[first]; a[first] = t;
    const int it = ind[mid]; ind[mid] = ind[first]; ind[first] = it;
    if (mid == cut) return;
    if (mid > cut) last = mid - 1; else first = mid + 1;
  }
}

__device__ __forceinline__ unsigned lanes_below(int lane) { return (1u << lane) - 1u; }

// One row per warp; shared memory per warp: lval, uval [cap] doubles, lcol, ucol [cap] ints,
// hash keys and positions [4 cap] ints (56 cap bytes).  At most 2 cap keys go into the hash,
// so at least half of its slots stay empty and every probe sequence ends.
__global__ void __launch_bounds__(32 * kWarps) k_ilut_factor(
    int n, const int* __restrict__ ia, const int* __restrict__ ja, const double* __restrict__ a,
    int lfil, double droptol, int cap, int epoch, int* __restrict__ Lcol,
    double* __restrict__ Lval, int* __restrict__ Lcnt, int* __restrict__ Ucol,
    double* __restrict__ Uval, int* __restrict__ Ucnt, double* __restrict__ dinv,
    int* __restrict__ levL, int* __restrict__ done, int* __restrict__ ctr, long spin,
    int withhold) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned hmask = 4u * cap - 1u;
  unsigned char* base = smem + (size_t)wid * 56 * cap;
  double* lval = reinterpret_cast<double*>(base);
  double* uval = lval + cap;
  int* lcol = reinterpret_cast<int*>(uval + cap);
  int* ucol = lcol + cap;
  int* hkey = ucol + cap;
  int* hpos = hkey + 4 * cap;
  const size_t slot = (size_t)(lfil > 0 ? lfil : 1);
  for (;;) {
    int ii = 0;
    if (lane == 0) ii = atomicAdd(ctr, 1);
    ii = __shfl_sync(~0u, ii, 0);
    if (ii >= n) return;
    for (int k = lane; k < 4 * cap; k += 32) hkey[k] = -1;
    const int j1 = ia[ii], j2 = ia[ii + 1];
    double tnorm = 0.0;
    if (lane == 0)
      for (int k = j1; k < j2; k++) tnorm += fabs(a[k]);
    tnorm = __shfl_sync(~0u, tnorm, 0);
    bool ok = true;
    int lenl = 0, lenu = 1, len = 0;
    if (tnorm == 0.0) {
      if (lane == 0) set_error(ctr, kErrZeroRow, ii);
      ok = false;
    }
    tnorm = tnorm / (double)(j2 - j1);
    __syncwarp();
    if (ok) {
      // unpack: L in CSR order, U with the diagonal first, then CSR order
      if (lane == 0) {
        ucol[0] = ii;
        uval[0] = 0.0;
        hinsert(hkey, hpos, hmask, ii, 0);
      }
      __syncwarp();
      for (int c = j1; c < j2; c += 32) {
        const int k = c + lane;
        const bool valid = k < j2;
        const int col = valid ? ja[k] : 0;
        const double v = valid ? a[k] : 0.0;
        const bool isL = valid && col < ii, isU = valid && col > ii;
        const unsigned bl = __ballot_sync(~0u, isL), bu = __ballot_sync(~0u, isU);
        if (isL || isU) {
          const int p = isL ? lenl + __popc(bl & lanes_below(lane)) : lenu + __popc(bu & lanes_below(lane));
          if (p < cap) {
            if (isL) { lcol[p] = col; lval[p] = v; hinsert(hkey, hpos, hmask, col, ~p); }
            else { ucol[p] = col; uval[p] = v; hinsert(hkey, hpos, hmask, col, p); }
          }
        }
        if (valid && col == ii) uval[0] = v;
        lenl += __popc(bl);
        lenu += __popc(bu);
        __syncwarp();
      }
      if (lenl > cap || lenu > cap) ok = false;
    }
    // elimination of the L entries in increasing column order (ilut.f:150-226); lev = the
    // largest L-graph level among the rows of stored multipliers (a superset of the kept
    // ones, so 1 + lev is a valid level for the sweeps' claim order)
    int jj = 0, lev = 0;
    while (ok && jj < lenl) {
      int best = INT_MAX, bidx = -1;
      for (int k = jj + lane; k < lenl; k += 32)
        if (lcol[k] < best) { best = lcol[k]; bidx = k; }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int ob = __shfl_xor_sync(~0u, best, o), oi = __shfl_xor_sync(~0u, bidx, o);
        if (ob < best) { best = ob; bidx = oi; }
      }
      const int jrow = best, k = bidx;
      if (lane == 0 && k != jj) {
        const int cj = lcol[jj];
        lcol[jj] = jrow; lcol[k] = cj;
        const double t = lval[jj]; lval[jj] = lval[k]; lval[k] = t;
        int pos;
        unsigned s1, s2;
        hfind(hkey, hpos, hmask, jrow, pos, s1);
        hfind(hkey, hpos, hmask, cj, pos, s2);
        hpos[s1] = ~jj;
        hpos[s2] = ~k;
      }
      __syncwarp();
      // lane 0 waits for the pivot row; every lane then acquires the flag itself, which
      // orders its reads of the row after the pivot warp's release
      bool ready = false;
      if (lane == 0) ready = wait_row(done, jrow, epoch, ctr, spin);
      if (!__shfl_sync(~0u, ready, 0)) { ok = false; break; }
      (void)ld_acquire(done + jrow);
      const double fact = __dmul_rn(lval[jj], dinv[jrow]);
      if (fabs(fact) <= droptol) { jj++; __syncwarp(); continue; }
      lev = max(lev, levL[jrow]);
      const int ulen = Ucnt[jrow];
      const int* uc = Ucol + (size_t)jrow * slot;
      const double* uv = Uval + (size_t)jrow * slot;
      for (int c = 0; c < ulen; c += 32) {
        const int idx = c + lane;
        const bool valid = idx < ulen;
        int j = 0, pos = 0;
        unsigned sl = 0;
        double s = 0.0;
        bool found = false;
        if (valid) {
          j = uc[idx];
          s = __dmul_rn(fact, uv[idx]);
          found = hfind(hkey, hpos, hmask, j, pos, sl);
        }
        const bool fill = valid && !found;
        const unsigned bu = __ballot_sync(~0u, fill && j >= ii);
        const unsigned bl = __ballot_sync(~0u, fill && j < ii);
        if (valid && found) {
          if (pos >= 0) uval[pos] = __dsub_rn(uval[pos], s);
          else lval[~pos] = __dsub_rn(lval[~pos], s);
        } else if (fill) {
          if (j >= ii) {
            const int p = lenu + __popc(bu & lanes_below(lane));
            if (p < cap) { ucol[p] = j; uval[p] = -s; hinsert(hkey, hpos, hmask, j, p); }
          } else {
            const int p = lenl + __popc(bl & lanes_below(lane));
            if (p < cap) { lcol[p] = j; lval[p] = -s; hinsert(hkey, hpos, hmask, j, ~p); }
          }
        }
        lenu += __popc(bu);
        lenl += __popc(bl);
        __syncwarp();
      }
      if (lenl > cap || lenu > cap) { ok = false; break; }
      if (lane == 0) { lval[len] = fact; lcol[len] = jrow; }
      len++;
      jj++;
      __syncwarp();
    }
    if (!ok) {
      if (lane == 0) {
        if (lenl > cap || lenu > cap) set_error(ctr, kErrCapacity, ii);
        Lcnt[ii] = 0;
        Ucnt[ii] = 0;
        dinv[ii] = 0.0;
        levL[ii] = 1;
        __threadfence();
        if (ii != withhold) st_release(done + ii, epoch);
      }
      __syncwarp();
      continue;
    }
    // U part first (the rows below wait for it): drop |w| <= droptol * tnorm keeping the
    // order, keep the largest (ilut.f:258-287), publish U and the inverted pivot
    const double thr = __dmul_rn(droptol, tnorm);
    int cnt = 0;
    for (int c = 1; c < lenu; c += 32) {
      const int idx = c + lane;
      const bool valid = idx < lenu;
      const double v = valid ? uval[idx] : 0.0;
      const int col = valid ? ucol[idx] : 0;
      const bool keep = valid && fabs(v) > thr;
      const unsigned b = __ballot_sync(~0u, keep);
      __syncwarp();
      if (keep) {
        const int d = 1 + cnt + __popc(b & lanes_below(lane));
        uval[d] = v;
        ucol[d] = col;
      }
      cnt += __popc(b);
      __syncwarp();
    }
    const int lenu2 = cnt + 1;
    const int keepu = min(lenu2, lfil);
    if (lane == 0) qsplit(uval + 1, ucol + 1, lenu2 - 1, keepu);
    __syncwarp();
    const int nu = max(keepu - 1, 0);
    for (int k = lane; k < nu; k += 32) {
      Ucol[(size_t)ii * slot + k] = ucol[1 + k];
      Uval[(size_t)ii * slot + k] = uval[1 + k];
    }
    if (lane == 0) {
      double w0 = uval[0];
      if (w0 == 0.0) w0 = __dmul_rn(__dadd_rn(0.0001, droptol), tnorm);
      dinv[ii] = 1.0 / w0;
      Ucnt[ii] = nu;
      levL[ii] = lev + 1;
    }
    __threadfence();
    __syncwarp();
    if (lane == 0 && ii != withhold) st_release(done + ii, epoch);
    // L part afterwards, off the rows-below path: the lfil largest multipliers (:236-254);
    // only the sweeps read it, after this kernel
    const int keepl = min(len, lfil);
    if (lane == 0) qsplit(lval, lcol, len, keepl);
    __syncwarp();
    for (int k = lane; k < keepl; k += 32) {
      Lcol[(size_t)ii * slot + k] = lcol[k];
      Lval[(size_t)ii * slot + k] = lval[k];
    }
    if (lane == 0) Lcnt[ii] = keepl;
    __syncwarp();
  }
}

// The sweeps publish each solved unknown by its own 64-bit store: the output vectors start
// filled with kPending, a signalling-NaN pattern that no arithmetic produces (results that
// would carry it are stored as the canonical NaN), and a row polls the unknowns it reads
// until they stop being kPending.  One L2 round trip per dependency, no flags, no fences.
constexpr unsigned long long kPending = 0x7ff4deadbeefcafeull;
// warps of a sweep: about kLookahead levels' worth of rows in flight.  More only add warps
// that spin on unknowns many levels ahead and load L2 with their polls.
#ifndef FOS_ILUT_LOOKAHEAD
#define FOS_ILUT_LOOKAHEAD 2
#endif
constexpr int kLookahead = FOS_ILUT_LOOKAHEAD;
#ifndef FOS_ILUT_MIN_WARPS
#define FOS_ILUT_MIN_WARPS 304
#endif

__device__ __forceinline__ double ld_poll(const double* p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_publish(double* p, double v) {
  if (__double_as_longlong(v) == (long long)kPending) v = __longlong_as_double(0x7ff8000000000000ll);
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ bool pending(double v) {
  return __double_as_longlong(v) == (long long)kPending;
}
// wait for an unknown: bounded spin, false (and the error word set) when the limit ran out
__device__ __forceinline__ double wait_value(const double* x, int j, double v, int* ctr, bool& ok,
                                             long spin) {
  for (long it = 0; pending(v); it++) {
    if (it >= spin) { atomicCAS(ctr + 3, 0, kErrTimeout); ok = false; return 0.0; }
    if (*(volatile int*)(ctr + 3) == kErrTimeout) { ok = false; return 0.0; }
    if (it > 8) __nanosleep(32);
    v = ld_poll(x + j);
  }
  return v;
}

__global__ void k_fill_pending(long n, double* __restrict__ x) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = __longlong_as_double((long long)kPending);
}

// sum_k A_ik x_k over a row's cnt stored entries, lanes over entries two at a time (both
// loads in flight before either is waited for); fixed-order warp reduction.  A wait that
// ran out makes the sum NaN, so the failure reaches callers that only look at the result
// (the Krylov driver's non-finite checks) as well as fos_ilut_status.
__device__ __forceinline__ double row_dot(const int* __restrict__ col, const double* __restrict__ val,
                                         int cnt, const double* x, int* ctr, int lane, long spin) {
  double s = 0.0;
  bool ok = true;
  for (int k = lane; k < cnt; k += 64) {
    const int j0 = col[k];
    const bool two = k + 32 < cnt;
    const int j1 = two ? col[k + 32] : j0;
    double v0 = ld_poll(x + j0), v1 = ld_poll(x + j1);
    v0 = wait_value(x, j0, v0, ctr, ok, spin);
    s += val[k] * v0;
    if (two) {
      v1 = wait_value(x, j1, v1, ctr, ok, spin);
      s += val[k + 32] * v1;
    }
  }
  if (!ok) s = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(~0u, s, o);
  return s;
}

// lusol forward sweep (ilut.f:2300-2305): z_i = y_i - sum_k L_ik z_k into z (kPending on
// entry), and x_i set to kPending for the backward sweep (x may be y: row i reads y_i only).
// Rows are claimed in order of their level in the L dependency graph (perm): the rows in
// flight are mostly independent, and a row's dependencies have lower levels, hence earlier
// claims.
__global__ void __launch_bounds__(256) k_ilut_fwd(int n, int lfil, const int* __restrict__ Lcol,
                                                  const double* __restrict__ Lval,
                                                  const int* __restrict__ Lcnt,
                                                  const int* __restrict__ perm,
                                                  const double* y, double* z, double* x,
                                                  int* __restrict__ ctr, long spin,
                                                  int withhold) {
  const int lane = threadIdx.x & 31;
  const size_t slot = (size_t)(lfil > 0 ? lfil : 1);
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(ctr + 1, 1);
    t = __shfl_sync(~0u, t, 0);
    if (t >= n) return;
    const int i = perm[t];
    const double yi = y[i];  // own operand first, so its load overlaps the dependency polls
    const double s = row_dot(Lcol + (size_t)i * slot, Lval + (size_t)i * slot, Lcnt[i], z, ctr, lane,
                             spin);
    if (lane == 0) {
      x[i] = __longlong_as_double((long long)kPending);
      if (i != withhold) st_publish(z + i, yi - s);
    }
  }
}

// lusol backward sweep (:2309-2315): x_i = dinv_i (z_i - sum_k U_ik x_k) into x (kPending on
// entry), rows claimed by level in the U dependency graph
__global__ void __launch_bounds__(256) k_ilut_bwd(int n, int lfil, const int* __restrict__ Ucol,
                                                  const double* __restrict__ Uval,
                                                  const int* __restrict__ Ucnt,
                                                  const double* __restrict__ dinv,
                                                  const int* __restrict__ perm,
                                                  const double* __restrict__ z, double* x,
                                                  int* __restrict__ ctr, long spin) {
  const int lane = threadIdx.x & 31;
  const size_t slot = (size_t)(lfil > 0 ? lfil : 1);
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(ctr + 2, 1);
    t = __shfl_sync(~0u, t, 0);
    if (t >= n) return;
    const int i = perm[t];
    const double zi = z[i], di = dinv[i];
    const double s = row_dot(Ucol + (size_t)i * slot, Uval + (size_t)i * slot, Ucnt[i], x, ctr, lane,
                             spin);
    if (lane == 0) st_publish(x + i, di * (zi - s));
  }
}

// CSR sanity before the factor kernel indexes with it: ia[0] = 0, ia non-decreasing, every
// column in [0, n); bad[0] = 1 + first failing row
__global__ void k_ilut_check(int n, const int* __restrict__ ia, const int* __restrict__ ja,
                             int* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = ia[i], e = ia[i + 1];
  bool ok = b >= 0 && e >= b && (i > 0 || b == 0);
  if (ok)
    for (int k = b; k < e; k++) {
      const int j = ja[k];
      if (j < 0 || j >= n) { ok = false; break; }
    }
  if (!ok) atomicMin(bad, i + 1);
}

int grid_for(const void* kernel, int threads, size_t smem, long rows_per_cta, long n) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
  const long need = (n + rows_per_cta - 1) / rows_per_cta;
  return (int)std::max(1L, std::min(need, (long)std::max(per, 1) * sms));
}

template <typename T>
int alloc(T** p, size_t count) {
  if (cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) {
    fos_set_error("fos_ilut: cudaMalloc failed");
    return -100;
  }
  return 0;
}

}  // namespace

extern "C" int fos_ilut_create(fos_ilut** out, int n, int lfil) {
  if (!out || n <= 0) {
    fos_set_error("fos_ilut_create: bad arguments");
    return -1;
  }
  if (lfil < 0) {  // ilut.f:998, ierr = -4
    fos_set_error("fos_ilut_create: lfil < 0");
    return -4;
  }
  fos_ilut* f = new fos_ilut();
  f->n = n;
  f->lfil = std::min(lfil, n - 1);  // initILU, sparse.f90:341
  cudaGetDevice(&f->device);
  const size_t slots = (size_t)n * (size_t)std::max(f->lfil, 1);
  int rc = 0;
  rc = rc ? rc : alloc(&f->d_Lcol, slots);
  rc = rc ? rc : alloc(&f->d_Lval, slots);
  rc = rc ? rc : alloc(&f->d_Ucol, slots);
  rc = rc ? rc : alloc(&f->d_Uval, slots);
  rc = rc ? rc : alloc(&f->d_Lcnt, n);
  rc = rc ? rc : alloc(&f->d_Ucnt, n);
  rc = rc ? rc : alloc(&f->d_dinv, n);
  rc = rc ? rc : alloc(&f->d_done, n);
  rc = rc ? rc : alloc(&f->d_z, n);
  rc = rc ? rc : alloc(&f->d_levL, n);
  rc = rc ? rc : alloc(&f->d_permF, n);
  rc = rc ? rc : alloc(&f->d_permB, n);
  rc = rc ? rc : alloc(&f->d_ctr, 8);
  if (!rc && cudaMallocHost((void**)&f->h_ctr, 8 * sizeof(int)) != cudaSuccess) {
    fos_set_error("fos_ilut_create: cudaMallocHost failed");
    rc = -100;
  }
  if (!rc) {
    if (cudaMemset(f->d_done, 0, sizeof(int) * n) != cudaSuccess) {
      fos_set_error("fos_ilut_create: cudaMemset failed");
      rc = -100;
    }
  }
  if (rc) {
    delete f;
    return rc;
  }
  *out = f;
  return 0;
}

extern "C" void fos_ilut_destroy(fos_ilut* f) { delete f; }

// Claim orders of the two sweeps: rows sorted (stably) by their level in the L graph
// (published by the factor kernel) and in the U graph (1 + the largest U level among the
// rows its U entries read), computed here on the host from the stored U columns, fetched
// in chunks of rows from the bottom up so host memory stays small at any size.
static int solve_orders(fos_ilut* f, cudaStream_t s) {
  const int n = f->n;
  const size_t slot = (size_t)std::max(f->lfil, 1);
  auto by_level = [n](const std::vector<int>& lv, int nlev, std::vector<int>& perm) {
    std::vector<int> start(nlev + 2, 0);
    for (int i = 0; i < n; i++) start[lv[i] + 1]++;
    for (int l = 0; l <= nlev; l++) start[l + 1] += start[l];
    perm.resize(n);
    for (int i = 0; i < n; i++) perm[start[lv[i]]++] = i;
  };
  std::vector<int> lev(n), perm;
  FOS_CUDA(cudaMemcpyAsync(lev.data(), f->d_levL, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  FOS_CUDA(cudaStreamSynchronize(s));
  int nl = 0;
  for (int i = 0; i < n; i++) nl = std::max(nl, lev[i]);
  by_level(lev, nl, perm);
  f->nlevF = nl;
  FOS_CUDA(cudaMemcpyAsync(f->d_permF, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  FOS_CUDA(cudaStreamSynchronize(s));
  const int chunk = (int)std::max<size_t>(1, (size_t)(16u << 20) / (slot * sizeof(int)));
  std::vector<int> cnt(chunk), col(slot * chunk);
  int nu = 0;
  for (int hi = n; hi > 0; hi -= chunk) {
    const int lo = std::max(0, hi - chunk), m = hi - lo;
    FOS_CUDA(cudaMemcpyAsync(cnt.data(), f->d_Ucnt + lo, sizeof(int) * m, cudaMemcpyDeviceToHost, s));
    FOS_CUDA(cudaMemcpyAsync(col.data(), f->d_Ucol + slot * lo, sizeof(int) * slot * m,
                             cudaMemcpyDeviceToHost, s));
    FOS_CUDA(cudaStreamSynchronize(s));
    for (int i = hi - 1; i >= lo; i--) {  // rows above i are final: U columns are > i
      int mx = 0;
      const int* c = col.data() + slot * (i - lo);
      for (int k = 0; k < cnt[i - lo]; k++) mx = std::max(mx, lev[c[k]]);
      lev[i] = mx + 1;
      nu = std::max(nu, mx + 1);
    }
  }
  by_level(lev, nu, perm);
  f->nlevB = nu;
  FOS_CUDA(cudaMemcpyAsync(f->d_permB, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  FOS_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int fos_ilut_factor_on(fos_ilut* f, const int* ia, const int* ja, const double* a,
                       double droptol, cudaStream_t s) {
  if (!f || !ia || !ja || !a) {
    fos_set_error("fos_ilut_factor_dev: bad arguments");
    return -1;
  }
  int dev = 0, smem_max = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  {
    const int big = INT_MAX;
    FOS_CUDA(cudaMemcpyAsync(f->d_ctr + 5, &big, sizeof(int), cudaMemcpyHostToDevice, s));
    k_ilut_check<<<(f->n + 255) / 256, 256, 0, s>>>(f->n, ia, ja, f->d_ctr + 5);
    f->launches++;
    FOS_CUDA(cudaGetLastError());
    FOS_CUDA(cudaMemcpyAsync(f->h_ctr + 5, f->d_ctr + 5, sizeof(int), cudaMemcpyDeviceToHost, s));
    FOS_CUDA(cudaStreamSynchronize(s));
    if (f->h_ctr[5] != INT_MAX) {
      fos_set_error("fos_ilut_factor_dev: malformed CSR at row " + std::to_string(f->h_ctr[5]));
      return -1;
    }
  }
  for (;;) {
    const size_t smem = (size_t)kWarps * 56 * f->cap;
    if (smem > (size_t)smem_max) {
      fos_set_error("fos_ilut_factor_dev: a row outgrew the largest working capacity (" +
                    std::to_string(f->cap / 2) + " entries of L and of U)");
      return -1;
    }
    FOS_CUDA(cudaFuncSetAttribute(k_ilut_factor, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    FOS_CUDA(cudaMemsetAsync(f->d_ctr, 0, 5 * sizeof(int), s));
    f->fepoch++;
    const int grid = grid_for((const void*)k_ilut_factor, 32 * kWarps, smem, kWarps, f->n);
    k_ilut_factor<<<grid, 32 * kWarps, smem, s>>>(f->n, ia, ja, a, f->lfil, droptol, f->cap,
                                                  f->fepoch, f->d_Lcol, f->d_Lval, f->d_Lcnt,
                                                  f->d_Ucol, f->d_Uval, f->d_Ucnt, f->d_dinv,
                                                  f->d_levL, f->d_done, f->d_ctr,
                                                  f->spin_limit > 0 ? f->spin_limit : kSpinLimit,
                                                  f->withhold);
    f->launches++;
    FOS_CUDA(cudaGetLastError());
    FOS_CUDA(cudaMemcpyAsync(f->h_ctr, f->d_ctr, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
    FOS_CUDA(cudaStreamSynchronize(s));
    const int err = f->h_ctr[3], row = f->h_ctr[4];
    if (err == kErrCapacity) {  // a row outgrew the working copy: redo with twice the room
      f->cap *= 2;
      continue;
    }
    f->factored = err == 0;
    if (f->factored)
      if (int rc = solve_orders(f, s)) return rc;
    if (err == kErrZeroRow) {
      fos_set_error("fos_ilut_factor_dev: zero row " + std::to_string(row + 1));
      return -5;
    }
    if (err == kErrTimeout) {
      fos_set_error("fos_ilut_factor_dev: a dependency wait ran out");
      return -6;
    }
    return 0;
  }
}

int fos_ilut_solve_on(fos_ilut* f, const double* y, double* x, cudaStream_t s) {
  if (!f || !y || !x || !f->factored) {
    fos_set_error("fos_ilut_solve_dev: bad arguments or no factorisation");
    return -1;
  }
  FOS_CUDA(cudaMemsetAsync(f->d_ctr, 0, 4 * sizeof(int), s));
  const long spin = f->spin_limit > 0 ? f->spin_limit : kSpinLimit;
  k_fill_pending<<<(f->n + 255) / 256, 256, 0, s>>>(f->n, f->d_z);
  // rows in flight: kLookahead levels of the average width, at least one CTA per SM
  auto sweep_grid = [&](int nlev) {
    const long width = (f->n + std::max(nlev, 1) - 1) / std::max(nlev, 1);
    const long warps = std::max((long)FOS_ILUT_MIN_WARPS, kLookahead * width);
    return std::min(grid_for((const void*)k_ilut_fwd, 256, 0, 8, f->n), (int)((warps + 7) / 8));
  };
  k_ilut_fwd<<<sweep_grid(f->nlevF), 256, 0, s>>>(f->n, f->lfil, f->d_Lcol, f->d_Lval, f->d_Lcnt,
                                                  f->d_permF, y, f->d_z, x, f->d_ctr, spin,
                                                  f->withhold);
  k_ilut_bwd<<<sweep_grid(f->nlevB), 256, 0, s>>>(f->n, f->lfil, f->d_Ucol, f->d_Uval, f->d_Ucnt,
                                                  f->d_dinv, f->d_permB, f->d_z, x, f->d_ctr, spin);
  f->launches += 3;
  FOS_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int fos_ilut_factor_dev(fos_ilut* f, const int* ia, const int* ja, const double* a,
                                   double droptol, void* stream) {
  return fos_ilut_factor_on(f, ia, ja, a, droptol, (cudaStream_t)stream);
}

extern "C" int fos_ilut_solve_dev(fos_ilut* f, const double* y, double* x, void* stream) {
  return fos_ilut_solve_on(f, y, x, (cudaStream_t)stream);
}

// Failure injection for tests: the wait limit and a row that is never published.
extern "C" int fos_ilut_set_wait_limit(fos_ilut* f, long polls, int withhold_row) {
  if (!f || withhold_row < -1 || withhold_row >= f->n) {
    fos_set_error("fos_ilut_set_wait_limit: bad arguments");
    return -1;
  }
  f->spin_limit = polls > 0 ? polls : 0;
  f->withhold = withhold_row;
  return 0;
}

// Solve status after the stream has drained: 0, or -6 when a dependency wait ran out.
extern "C" int fos_ilut_status(fos_ilut* f) {
  if (!f) return -1;
  int h = 0;
  FOS_CUDA(cudaMemcpy(&h, f->d_ctr + 3, sizeof(int), cudaMemcpyDeviceToHost));
  if (h == kErrTimeout) {
    fos_set_error("fos_ilut: a dependency wait ran out");
    return -6;
  }
  return 0;
}

// The factors in SPARSKIT's MSR layout on the host (1-based values, as ilut returns them):
// alu(1:n) the inverted diagonal, jlu(1) = n + 2, row i = its L then its U entries from
// ju(i).  Returns the used length of alu/jlu (jlu(n+1) - 1), or < 0.
extern "C" long fos_ilut_copy(const fos_ilut* f, double* alu, int* jlu, int* ju, long iwk) {
  if (!f || !f->factored) {
    fos_set_error("fos_ilut_copy: no factorisation");
    return -1;
  }
  const int n = f->n;
  const size_t slot = (size_t)std::max(f->lfil, 1);
  std::vector<int> lc(n), uc(n);
  if (cudaMemcpy(lc.data(), f->d_Lcnt, sizeof(int) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(uc.data(), f->d_Ucnt, sizeof(int) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
    fos_set_error("fos_ilut_copy: cudaMemcpy failed");
    return -100;
  }
  long total = n + 1;
  for (int i = 0; i < n; i++) total += lc[i] + uc[i];
  if (!alu || !jlu || !ju) return total;
  if (iwk < total) {
    fos_set_error("fos_ilut_copy: iwk too small");
    return -2;
  }
  std::vector<int> col(slot * n);
  std::vector<double> val(slot * n), dv(n);
  if (cudaMemcpy(dv.data(), f->d_dinv, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
    fos_set_error("fos_ilut_copy: cudaMemcpy failed");
    return -100;
  }
  for (int i = 0; i < n; i++) alu[i] = dv[i];
  alu[n] = 0.0;
  long q = n + 1;  // 0-based position of the next entry (1-based n + 2)
  jlu[0] = n + 2;
  if (cudaMemcpy(col.data(), f->d_Lcol, sizeof(int) * slot * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(val.data(), f->d_Lval, sizeof(double) * slot * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
    fos_set_error("fos_ilut_copy: cudaMemcpy failed");
    return -100;
  }
  std::vector<int> ucol(slot * n);
  std::vector<double> uval(slot * n);
  if (cudaMemcpy(ucol.data(), f->d_Ucol, sizeof(int) * slot * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(uval.data(), f->d_Uval, sizeof(double) * slot * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
    fos_set_error("fos_ilut_copy: cudaMemcpy failed");
    return -100;
  }
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < lc[i]; k++, q++) {
      alu[q] = val[(size_t)i * slot + k];
      jlu[q] = col[(size_t)i * slot + k] + 1;
    }
    ju[i] = (int)(q + 1);
    for (int k = 0; k < uc[i]; k++, q++) {
      alu[q] = uval[(size_t)i * slot + k];
      jlu[q] = ucol[(size_t)i * slot + k] + 1;
    }
    jlu[i + 1] = (int)(q + 1);
  }
  return q;
}

extern "C" int fos_ilut_info(const fos_ilut* f, long* out) {
  if (!f || !out) return -1;
  out[0] = f->n;
  out[1] = f->lfil;
  out[2] = f->cap;
  out[3] = f->launches;
  out[4] = f->nlevF;
  out[5] = f->nlevB;
  return 0;
}

// ---------------------------------------------------------------- the Euler preconditioner
// With FOS_PREC_ILUT, pset factors the scalar P = I - gamma diag(1/v) J with ILUT instead of
// block ILU(0), the way fopbc wires its ILU class (modPbc.f90:676-711: COO -> setCOO ->
// fact(droptol) -> lusol).  P is laid out in the ILU position order, unknown 5p + a for
// component a of the cell at position p, each row's columns ascending (blocks by position,
// components within a block).  psol permutes r into that order, solves, and permutes back.
namespace {

__global__ void k_pcsr_rows(int nC, const int* __restrict__ prow, int* __restrict__ ia) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > 5 * nC) return;
  if (r == 5 * nC) { ia[r] = 25 * prow[nC]; return; }
  const int p = r / 5, a = r - 5 * p;
  ia[r] = 25 * prow[p] + 5 * a * (prow[p + 1] - prow[p]);
}

__global__ void k_pcsr_cols(int nC, const int* __restrict__ prow, const int* __restrict__ pcol,
                            int* __restrict__ ja) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= 5 * nC) return;
  const int p = r / 5, a = r - 5 * p, s0 = prow[p], nb = prow[p + 1] - s0;
  int* dst = ja + 25 * (size_t)s0 + 5 * a * nb;
  for (int s = 0; s < nb; s++)
    for (int b = 0; b < 5; b++) dst[5 * s + b] = 5 * pcol[s0 + s] + b;
}

// P entries as the oracle forms them: (1 on the diagonal) - (gamma / v) J, no contraction
template <typename TJ>
__global__ void k_pcsr_vals(int nC, const int* __restrict__ prow, const int* __restrict__ pdiag,
                            const int* __restrict__ ord, const double* __restrict__ vol,
                            double gamma, const TJ* __restrict__ J, double* __restrict__ A) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= 5 * nC) return;
  const int p = r / 5, a = r - 5 * p, s0 = prow[p], nb = prow[p + 1] - s0;
  const double sc = gamma / vol[ord[p]];
  double* dst = A + 25 * (size_t)s0 + 5 * a * nb;
  for (int s = 0; s < nb; s++)
    for (int b = 0; b < 5; b++) {
      const double d = (s0 + s == pdiag[p] && a == b) ? 1.0 : 0.0;
      dst[5 * s + b] = __dsub_rn(d, __dmul_rn(sc, (double)J[25 * (size_t)(s0 + s) + 5 * a + b]));
    }
}

__global__ void k_ilut_in(int nC, const int* __restrict__ ipos, const double* __restrict__ r,
                          double* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nC) return;
  const size_t q = 5 * (size_t)ipos[i];
#pragma unroll
  for (int a = 0; a < 5; a++) x[q + a] = r[(size_t)a * nC + i];
}

__global__ void k_ilut_out(int nC, const int* __restrict__ ipos, const double* __restrict__ x,
                           double* __restrict__ z) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nC) return;
  const size_t q = 5 * (size_t)ipos[i];
#pragma unroll
  for (int a = 0; a < 5; a++) z[(size_t)a * nC + i] = x[q + a];
}

inline int blocks(long n, int t = 256) { return (int)((n + t - 1) / t); }

}  // namespace

int fos_ilut_ctx_factor(fos_ctx* c, double gamma) {
  const int nC = c->nC, n = 5 * nC;
  if (!c->has_jac) {
    fos_set_error("ILUT: no Jacobian assembled");
    return -1;
  }
  if (c->ilut && c->ilut->lfil != std::min(c->ilut_lfil, n - 1)) {
    fos_ilut_destroy(c->ilut);
    c->ilut = nullptr;
  }
  if (!c->d_pia) {
    const size_t nnz = 25 * (size_t)c->nnzb;
    if (nnz > (size_t)INT_MAX) {
      fos_set_error("ILUT: P has more than 2^31 - 1 entries");
      return -2;
    }
    FOS_CUDA(cudaMalloc((void**)&c->d_pia, sizeof(int) * (n + 1)));
    FOS_CUDA(cudaMalloc((void**)&c->d_pja, sizeof(int) * nnz));
    FOS_CUDA(cudaMalloc((void**)&c->d_pa, sizeof(double) * nnz));
    FOS_CUDA(cudaMalloc((void**)&c->d_vol, sizeof(double) * nC));
    FOS_CUDA(cudaMalloc((void**)&c->d_ilut_x, sizeof(double) * n));
    FOS_CUDA(cudaMemcpy(c->d_vol, c->h_vol.data(), sizeof(double) * nC, cudaMemcpyHostToDevice));
    fos_launch(c, k_pcsr_rows, blocks(n + 1), 256, nC, (const int*)c->d_prow, c->d_pia);
    fos_launch(c, k_pcsr_cols, blocks(n), 256, nC, (const int*)c->d_prow, (const int*)c->d_pcol,
               c->d_pja);
  }
  if (!c->ilut)
    if (int rc = fos_ilut_create(&c->ilut, n, c->ilut_lfil)) return rc;
  if (c->flags & FOS_ILU_FP32)
    fos_launch(c, k_pcsr_vals<float>, blocks(n), 256, nC, (const int*)c->d_prow,
               (const int*)c->d_pdiag, (const int*)c->d_ord, (const double*)c->d_vol, gamma,
               (const float*)c->d_Jraw, c->d_pa);
  else
    fos_launch(c, k_pcsr_vals<double>, blocks(n), 256, nC, (const int*)c->d_prow,
               (const int*)c->d_pdiag, (const int*)c->d_ord, (const double*)c->d_vol, gamma,
               (const double*)c->d_Jraw, c->d_pa);
  FOS_LAUNCH_CHECK();
  const long before = c->ilut->launches;
  const int rc = fos_ilut_factor_on(c->ilut, c->d_pia, c->d_pja, c->d_pa, c->ilut_droptol,
                                    c->stream);
  c->n_launch += c->ilut->launches - before;
  c->has_factor = rc == 0;
  c->ilu_ierr = rc == -5 ? 1 : 0;
  return rc == -5 ? 0 : rc;  // a zero row is reported like a zero pivot (recoverable)
}

int fos_ilut_ctx_apply(fos_ctx* c, const double* r, double* z) {
  if (!c->ilut || !c->has_factor) {
    fos_set_error("ILUT: no factorisation");
    return -1;
  }
  fos_launch(c, k_ilut_in, blocks(c->nC), 256, c->nC, (const int*)c->d_ipos, r, c->d_ilut_x);
  const long before = c->ilut->launches;
  if (int rc = fos_ilut_solve_on(c->ilut, c->d_ilut_x, c->d_ilut_x, c->stream)) return rc;
  c->n_launch += c->ilut->launches - before;
  fos_launch(c, k_ilut_out, blocks(c->nC), 256, c->nC, (const int*)c->d_ipos,
             (const double*)c->d_ilut_x, z);
  FOS_LAUNCH_CHECK();
  return 0;
}

extern "C" int fos_ctx_set_ilut(fos_ctx* c, int lfil, double droptol) {
  if (!c || lfil < 0 || !(droptol >= 0.0)) {
    fos_set_error("fos_ctx_set_ilut: bad arguments (lfil >= 0, droptol >= 0)");
    return -1;
  }
  c->ilut_lfil = lfil;
  c->ilut_droptol = droptol;
  c->has_factor = false;
  return 0;
}
