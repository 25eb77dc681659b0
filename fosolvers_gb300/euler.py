"""Host-side mirror of foeuler's module interface (src/foeuler/foeuler.f90, modFOEuler).

`PolyFvGrid` holds the face arrays of a polyFvGrid after `grid%up()`
(polyFvGrid.f90:48-57); `FOEuler` holds what `init()` sets up (grid, condition
table, gas constants; foeuler.f90:60-175) and exposes the three CVODE callbacks
with the reference's names and argument meaning:

    rhs(t, y, ydot) -> int                       foeuler.f90:349-375
    pset(t, y, fy, jok, gamma) -> (int, jcur)    foeuler.f90:378-405
    psol(t, y, fy, r, z, gamma, delta, lr) -> int  foeuler.f90:408-437

Return codes are CVODE's: 0 ok, >0 recoverable, <0 fatal (raised as
RuntimeError here, like the reference's `stop` on set-up errors).  All compute
runs in libfosgpu.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import BdfOpts, BdfStats, check, dptr, iptr

FLUX_FP64, FLUX_FP32 = 0, 1
ORDER_RCM, ORDER_NATURAL = 0, 2
ILU_FP32, ILU_COLOR = 4, 8
PREC_ILUT = 16  # pset/psol with ILUT (FP64) instead of block ILU(0)
FLUX_HYBRID = 32  # with FLUX_FP32: faces with large density / pressure jumps in FP64
JV_EPS_FP32 = 1e-5  # default finite-difference increment scale of the FP32 flux (the driver's)


@dataclass
class PolyFvGrid:
    nC: int
    nE: int
    nP: int
    nPi: int
    nPb: int
    maxFace: int
    iEP: np.ndarray     # (nP, 2) int32, 1-based element ids
    aP: np.ndarray      # (nP,)
    normP: np.ndarray   # (nP, 3)
    pP: np.ndarray      # (nP, 3)
    v: np.ndarray       # (nC,)
    neib: np.ndarray    # (nC, maxFace) int32, 1-based (0 = none)
    gid: np.ndarray     # (nE,) int32
    p: np.ndarray       # (nE, 3) element centroids
    sE: np.ndarray      # (nE,) int32

    @classmethod
    def from_mesh(cls, mesh) -> "PolyFvGrid":
        """Element connectivity -> face arrays (readGMSH + grid%up) through fos_grid_build."""
        L = _lib.lib()
        pN = np.ascontiguousarray(mesh.pN, np.float64)
        iNE = np.ascontiguousarray(mesh.iNE, np.int32)
        m = iNE.shape[1]
        h = C.c_void_p()
        check(L.fos_grid_build(C.byref(h), mesh.nN, dptr(pN), mesh.nE, m,
                               iptr(np.ascontiguousarray(mesh.sE, np.int32)),
                               iptr(np.ascontiguousarray(mesh.nNE, np.int32)), iptr(iNE),
                               iptr(np.ascontiguousarray(mesh.gid, np.int32))), "fos_grid_build")
        try:
            sz = np.zeros(7, np.int32)
            L.fos_grid_sizes(h, iptr(sz))
            nC, nE, nP, nPi, nPb, mf, _ = (int(x) for x in sz)
            iEP = np.zeros((nP, 2), np.int32)
            aP = np.zeros(nP)
            normP = np.zeros((nP, 3))
            pP = np.zeros((nP, 3))
            v = np.zeros(nC)
            neib = np.zeros((nC, mf), np.int32)
            gid = np.zeros(nE, np.int32)
            p = np.zeros((nE, 3))
            sE = np.zeros(nE, np.int32)
            L.fos_grid_copy(h, iptr(iEP), dptr(aP), dptr(normP), dptr(pP), dptr(v), iptr(neib),
                            iptr(gid), dptr(p), iptr(sE))
        finally:
            L.fos_grid_free(h)
        return cls(nC, nE, nP, nPi, nPb, mf, iEP, aP, normP, pP, v, neib, gid, p, sE)


class FOEuler:
    """GPU context for one grid: the state modFOEuler keeps between CVODE callbacks."""

    def __init__(self, grid: PolyFvGrid, iBC=None, bc_type=None, bc_param=None,
                 gamm: float = 1.4, r: float = 1.0, flags: int = 0, stream=None):
        L = _lib.lib()
        self.grid = grid
        self.nC = grid.nC
        self.N = 5 * grid.nC
        self.gamm, self.r, self.flags = gamm, r, flags
        iBC = np.zeros(grid.nE, np.int32) if iBC is None else np.ascontiguousarray(iBC, np.int32)
        bc_type = np.zeros(0, np.int32) if bc_type is None else np.ascontiguousarray(bc_type, np.int32)
        nBC = int(bc_type.shape[0])
        if bc_param is None or nBC == 0:
            bcp = np.zeros((max(nBC, 1), 5))
        else:
            bcp = np.asarray(bc_param, np.float64).reshape(nBC, -1)
        maxP = int(bcp.shape[1])
        bcp = np.ascontiguousarray(bcp)  # row = condition: column-major bc%p(maxP, nBC)
        self._keep = (iBC, bc_type, bcp)
        h = C.c_void_p()
        check(L.fos_ctx_create(C.byref(h), grid.nC, grid.nE, grid.nPi, grid.nPb,
                               iptr(np.ascontiguousarray(grid.iEP)), dptr(np.ascontiguousarray(grid.aP)),
                               dptr(np.ascontiguousarray(grid.normP)), dptr(np.ascontiguousarray(grid.v)),
                               iptr(iBC), nBC, iptr(bc_type) if nBC else None,
                               dptr(bcp) if nBC else None, maxP, gamm, r, 1, flags),
              "fos_ctx_create")
        self._h = h
        if stream is not None:
            self.set_stream(stream)

    # ---------------------------------------------------------------- lifetime
    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().fos_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream):
        """stream: a torch.cuda.Stream, a raw cudaStream_t int, or None."""
        raw = getattr(stream, "cuda_stream", stream)
        check(_lib.lib().fos_ctx_set_stream(self._h, C.c_void_p(raw or 0)), "fos_ctx_set_stream")

    def info(self) -> dict:
        out = np.zeros(9, np.int64)
        _lib.lib().fos_ctx_info(self._h, out.ctypes.data_as(C.POINTER(C.c_long)))
        keys = ["nC", "nPi", "nPb", "nlev_fwd", "nlev_bwd", "nnzb", "bandwidth", "flags", "launches"]
        return dict(zip(keys, (int(x) for x in out)))

    def renumbering(self) -> np.ndarray:
        o2n = np.zeros(self.nC, np.int32)
        check(_lib.lib().fos_ctx_renumbering(self._h, iptr(o2n)), "fos_ctx_renumbering")
        return o2n

    def ilu_order(self) -> np.ndarray:
        """Position of every reference cell in the ILU(0) elimination order (after pset)."""
        pos = np.zeros(self.nC, np.int32)
        check(_lib.lib().fos_ctx_ilu_order(self._h, iptr(pos)), "fos_ctx_ilu_order")
        return pos

    # ---------------------------------------------------------------- CVODE callbacks (host)
    def rhs(self, t: float, y: np.ndarray, ydot: np.ndarray) -> int:
        return check(_lib.lib().fos_euler_rhs(t, dptr(y), dptr(ydot), self._h), "rhs")

    def pset(self, t: float, y: np.ndarray, fy: np.ndarray | None, jok: int, gamma: float):
        jcur = C.c_int(0)
        rc = _lib.lib().fos_euler_pset(t, dptr(y), dptr(fy) if fy is not None else None, jok,
                                       C.byref(jcur), gamma, self._h)
        return check(rc, "pset"), jcur.value

    def psol(self, t, y, fy, r, z, gamma, delta=0.0, lr=1) -> int:
        return check(_lib.lib().fos_euler_psol(t, dptr(y) if y is not None else None,
                                               dptr(fy) if fy is not None else None, dptr(r),
                                               dptr(z), gamma, delta, lr, self._h), "psol")

    # ---------------------------------------------------------------- device entry points
    # device vectors are torch CUDA tensors (float64, 5*nC) in the internal cell order
    def to_internal(self, y_ref_dev, out_dev):
        check(_lib.lib().fos_ctx_permute_dev(self._h, y_ref_dev.data_ptr(), out_dev.data_ptr(), 0),
              "permute")

    def to_reference(self, y_dev, out_ref_dev):
        check(_lib.lib().fos_ctx_permute_dev(self._h, y_dev.data_ptr(), out_ref_dev.data_ptr(), 1),
              "permute")

    def rhs_dev(self, t, y_dev, ydot_dev) -> int:
        return check(_lib.lib().fos_euler_rhs_dev(self._h, t, y_dev.data_ptr(), ydot_dev.data_ptr()),
                     "rhs_dev")

    def rhs_dev_static(self, t, y_dev, ydot_dev) -> int:
        """rhs_dev without device allocation (scratch in the library's static array)."""
        return check(_lib.lib().fos_euler_rhs_dev_static(self._h, t, y_dev.data_ptr(),
                                                         ydot_dev.data_ptr()), "rhs_dev_static")

    def jv_dev(self, t, y_dev, fy_dev, v_dev, out_dev, a, b, ynorm, eps=0.0) -> int:
        if eps <= 0.0:
            eps = JV_EPS_FP32 if self.flags & FLUX_FP32 \
                else float(np.sqrt(np.finfo(np.float64).eps))
        return check(_lib.lib().fos_euler_jv_dev(self._h, t, y_dev.data_ptr(), fy_dev.data_ptr(),
                                                 v_dev.data_ptr(), out_dev.data_ptr(), a, b,
                                                 ynorm, eps), "jv_dev")

    def jv_dev_vnorm(self, t, y_dev, fy_dev, v_dev, out_dev, a, b, ynorm, vnorm,
                     eps=0.0) -> int:
        """jv_dev with ||v||_2 known to the caller (no reduction pass over v)."""
        if eps <= 0.0:
            eps = JV_EPS_FP32 if self.flags & FLUX_FP32 \
                else float(np.sqrt(np.finfo(np.float64).eps))
        return check(_lib.lib().fos_euler_jv_dev_vnorm(self._h, t, y_dev.data_ptr(),
                                                       fy_dev.data_ptr(), v_dev.data_ptr(),
                                                       out_dev.data_ptr(), a, b, ynorm, vnorm,
                                                       eps), "jv_dev_vnorm")

    def pset_dev(self, t, y_dev, jok, gamma):
        jcur = C.c_int(0)
        rc = _lib.lib().fos_euler_pset_dev(self._h, t, y_dev.data_ptr(), jok, C.byref(jcur), gamma)
        return check(rc, "pset_dev"), jcur.value

    def psol_dev(self, r_dev, z_dev) -> int:
        return check(_lib.lib().fos_euler_psol_dev(self._h, r_dev.data_ptr(), z_dev.data_ptr()),
                     "psol_dev")

    def jacobian(self):
        """(rowptr, col, val[nnzb,5,5]) of the last assembled J in internal order."""
        L = _lib.lib()
        nnzb = check(L.fos_euler_jac_copy(self._h, None, None, None), "jac_copy")
        rowptr = np.zeros(self.nC + 1, np.int32)
        col = np.zeros(nnzb, np.int32)
        val = np.zeros(25 * nnzb)
        check(L.fos_euler_jac_copy(self._h, iptr(rowptr), iptr(col), dptr(val)), "jac_copy")
        return rowptr, col, val.reshape(nnzb, 5, 5)

    def set_jacobian(self, val: np.ndarray):
        """Replace the stored Jacobian blocks (val[nnzb, 5, 5], the layout of jacobian());
        the next pset with jok = 1 factors P from them."""
        v = np.ascontiguousarray(val, np.float64).reshape(-1)
        check(_lib.lib().fos_euler_jac_set(self._h, dptr(v)), "jac_set")

    # ---------------------------------------------------------------- driver
    @staticmethod
    def bdf_defaults(**kw) -> BdfOpts:
        o = BdfOpts()
        _lib.lib().fos_bdf_defaults(C.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def bdf_run(self, y_dev, opts: BdfOpts, t0: float = 0.0):
        """Advance the device state (internal order) by opts.nsteps fixed BDF steps."""
        st = BdfStats()
        rc = check(_lib.lib().fos_bdf_run(self._h, t0, y_dev.data_ptr(), C.byref(opts), C.byref(st)),
                   "fos_bdf_run")
        return rc, st.as_dict()

    @staticmethod
    def adapt_defaults(**kw):
        o = _lib.AdaptOpts()
        _lib.lib().fos_bdf_adapt_defaults(C.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def bdf_adaptive(self, y_dev, t0: float, tout: float, nk: BdfOpts, ad):
        """Advance the device state (internal order) from t0 to tout with the variable-order,
        variable-step BDF driver; returns (rc, Newton-Krylov stats, step-control stats)."""
        st, ast = BdfStats(), _lib.AdaptStats()
        rc = check(_lib.lib().fos_bdf_adaptive(self._h, t0, tout, y_dev.data_ptr(), C.byref(nk),
                                               C.byref(ad), C.byref(st), C.byref(ast)),
                   "fos_bdf_adaptive")
        return rc, st.as_dict(), ast.as_dict()

    def set_flux_threshold(self, theta: float):
        """Relative density / pressure jump above which a face of the FLUX_HYBRID flux is
        evaluated in FP64 (default 0.05)."""
        check(_lib.lib().fos_ctx_set_flux_threshold(self._h, float(theta)), "set_flux_threshold")

    def set_ilut(self, lfil: int = 50, droptol: float = 1e-6):
        """ILUT parameters of a context created with PREC_ILUT (fopbc's fill 50 and drop
        tolerance 1e-6 by default, modPbc.f90:21,658); used from the next pset on."""
        check(_lib.lib().fos_ctx_set_ilut(self._h, int(lfil), float(droptol)), "set_ilut")

    def attach_gnn(self, gnn):
        """Learned preconditioner used by bdf_run / linear_solve when opts.precond >= 2
        (tetrahedral grids only: raises on a grid with hexahedra)."""
        check(_lib.lib().fos_ctx_attach_gnn(self._h, gnn.handle if gnn is not None else None),
              "attach_gnn")
        self._gnn = gnn

    def linear_solve(self, y_dev, fy_dev, gamma, b_dev, x_dev, opts: BdfOpts, t: float = 0.0):
        """One (F)GMRES solve of J_G x = b at state y; returns (rc, stats)."""
        st = BdfStats()
        rc = check(_lib.lib().fos_linear_solve_dev(self._h, t, y_dev.data_ptr(), fy_dev.data_ptr(),
                                                   gamma, b_dev.data_ptr(), x_dev.data_ptr(),
                                                   C.byref(opts), C.byref(st)), "linear_solve")
        return rc, st.as_dict()

    def bdf_run_host(self, y: np.ndarray, opts: BdfOpts, t0: float = 0.0):
        """Same on a host array in reference order (copied in and out)."""
        st = BdfStats()
        rc = check(_lib.lib().fos_bdf_run_host(self._h, t0, dptr(y), C.byref(opts), C.byref(st)),
                   "fos_bdf_run_host")
        return rc, st.as_dict()
