"""ctypes binding of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker / baseline; never by the fosolvers_gb300 package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

RHS_FN = C.CFUNCTYPE(C.c_int, C.c_double, _dp, _dp, _vp)
PSET_FN = C.CFUNCTYPE(C.c_int, C.c_double, _dp, _dp, C.c_int, _ip, C.c_double, _vp)
PSOL_FN = C.CFUNCTYPE(C.c_int, C.c_double, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, _vp)


class BdfOpts(C.Structure):
    _fields_ = [("order", C.c_int), ("dt", C.c_double), ("nsteps", C.c_int),
                ("newton_rtol", C.c_double), ("newton_atol", C.c_double),
                ("max_newton", C.c_int), ("maxl", C.c_int), ("max_restarts", C.c_int),
                ("lin_rtol", C.c_double), ("jv_eps", C.c_double), ("use_prec", C.c_int),
                ("msbp", C.c_int), ("predictor", C.c_int)]


class AdaptOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("h0", C.c_double),
                ("hmin", C.c_double), ("hmax", C.c_double), ("qmax", C.c_int),
                ("max_steps", C.c_int)]


class AdaptStats(C.Structure):
    _fields_ = [("n_accepted", C.c_long), ("n_err_fails", C.c_long),
                ("n_newton_fails", C.c_long), ("h_last", C.c_double), ("t", C.c_double),
                ("q_last", C.c_int), ("steps_at_order", C.c_long * 6)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "steps_at_order"}
        d["steps_at_order"] = list(self.steps_at_order)
        return d


class BdfStats(C.Structure):
    _fields_ = [("n_rhs", C.c_long), ("n_jv", C.c_long), ("n_psol", C.c_long),
                ("n_pset", C.c_long), ("n_newton", C.c_long), ("n_lin_iters", C.c_long),
                ("n_steps", C.c_long), ("fails", C.c_long), ("last_gnorm", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_SIGS = {
    "og_grid_build": (_vp, [C.c_int, _dp, C.c_int, C.c_int, _ip, _ip, _ip, _ip]),
    "og_grid_free": (None, [_vp]),
    "og_grid_sizes": (None, [_vp, _ip]),
    "og_grid_copy": (None, [_vp, _ip, _dp, _dp, _dp, _dp, _ip, _ip, _dp, _ip]),
    "og_a3p": (C.c_double, [_dp]),
    "og_v4p": (C.c_double, [_dp]),
    "og_v8p": (C.c_double, [_dp]),
    "og_n3p": (None, [_dp, _dp]),
    "og_qsort_perm": (None, [C.c_int, _ip, _ip]),
    "oe_new": (_vp, [C.c_int, C.c_int, C.c_int, C.c_int, _ip, _dp, _dp, _dp, C.c_int, _ip, _ip,
                     C.c_int, _ip, _dp, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp]),
    "oe_free": (None, [_vp]),
    "oe_set_threads": (None, [_vp, C.c_int]),
    "oe_set_ilu_order": (None, [_vp, _ip]),
    "oe_set_ilut": (None, [_vp, C.c_int, C.c_double]),
    "oe_ilut_factors": (C.c_int, [_vp, C.POINTER(_dp), C.POINTER(_ip), C.POINTER(_ip)]),
    "oe_rhs": (C.c_int, [C.c_double, _dp, _dp, _vp]),
    "oe_pset": (C.c_int, [C.c_double, _dp, _dp, C.c_int, _ip, C.c_double, _vp]),
    "oe_psol": (C.c_int, [C.c_double, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, _vp]),
    "oe_jac": (_dp, [_vp, _dp]),
    "oe_pmat": (C.c_int, [_vp, C.POINTER(_dp), C.POINTER(_ip), C.POINTER(_ip)]),
    "oe_ilu_ierr": (C.c_int, [_vp]),
    "oe_elem_state": (None, [_vp, _dp, _dp, _dp]),
    "oe_nfj": (None, [_dp, _dp, C.c_double, C.c_double, _dp]),
    "oe_anfj": (None, [_dp, _dp, C.c_double, C.c_double, C.c_double, _dp]),
    "o_coocsr": (None, [C.c_int, C.c_int, _dp, _ip, _ip, _dp, _ip, _ip]),
    "o_csrsort": (None, [C.c_int, _dp, _ip, _ip]),
    "o_amux": (None, [C.c_int, _dp, _dp, _dp, _ip, _ip]),
    "o_ilu0": (C.c_int, [C.c_int, _dp, _ip, _ip, _dp, _ip, _ip, _ip]),
    "o_lusol": (None, [C.c_int, _dp, _dp, _dp, _ip, _ip]),
    "o_qsplit": (None, [_dp, _ip, C.c_int, C.c_int]),
    "o_ilut": (C.c_int, [C.c_int, _dp, _ip, _ip, C.c_int, C.c_double, _dp, _ip, _ip, C.c_int,
                         _dp, _ip]),
    "o_bdf_defaults": (None, [C.POINTER(BdfOpts)]),
    "o_jv": (C.c_int, [C.c_int, _vp, _vp, C.c_double, _dp, _dp, _dp, _dp, C.c_double,
                       C.c_double, C.c_double, C.c_double, _dp, _dp]),
    "o_bdf_run": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, C.c_double, _dp, C.POINTER(BdfOpts),
                            C.POINTER(BdfStats)]),
    "o_newton_solve": (C.c_int, [C.c_int, _vp, _vp, _dp, C.c_double, C.c_double, C.c_int, C.c_int,
                                 C.c_double, C.POINTER(BdfStats)]),
    "o_adapt_defaults": (None, [C.POINTER(AdaptOpts)]),
    "o_bdf_adaptive": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, C.c_double, C.c_double, _dp,
                                 C.POINTER(BdfOpts), C.POINTER(AdaptOpts), C.POINTER(BdfStats),
                                 C.POINTER(AdaptStats)]),
}

_libs: dict = {}
_default = "checker"


def lib(variant: str | None = None):
    """The oracle library: "checker" (portable build, the default) or "tuned" (the same
    source built for the host's instruction set, for CPU timing; bit-identical results)."""
    v = variant or _default
    if v not in _libs:
        path = _build.build() if v == "checker" else _build.build_tuned()
        l = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _libs[v] = l
    return _libs[v]


def set_default(variant: str) -> None:
    """Library used by every later call that names none ("checker" or "tuned")."""
    global _default
    if variant not in ("checker", "tuned"):
        raise ValueError(variant)
    _default = variant


def lib_path(variant: str | None = None) -> str:
    return lib(variant)._name


def dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def ip(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def ilut(n, a, ja, ia, lfil, droptol):
    """The reference's ILU class on a CSR matrix with 1-based ja/ia (numerics/sparse.f90:
    initILU :334-348 clamps lfil to n - 1 and sizes alu/jlu to n*min(2*lfil+1, n); factILU
    :370-383 calls ilut).  Returns (ierr, alu, jlu, ju) in MSR form."""
    lfil = min(lfil, n - 1)
    iwk = n * min(2 * lfil + 1, n)
    alu, jlu = np.zeros(iwk), np.zeros(iwk, np.int32)
    ju, w, jw = np.zeros(n, np.int32), np.zeros(n + 1), np.zeros(2 * n, np.int32)
    ierr = lib().o_ilut(n, dp(np.ascontiguousarray(a, np.float64)),
                        ip(np.ascontiguousarray(ja, np.int32)), ip(np.ascontiguousarray(ia, np.int32)),
                        lfil, droptol, dp(alu), ip(jlu), ip(ju), iwk, dp(w), ip(jw))
    return ierr, alu, jlu, ju


def lusol(n, y, alu, jlu, ju):
    x = np.zeros(n)
    lib().o_lusol(n, dp(np.ascontiguousarray(y, np.float64)), dp(x), dp(alu), ip(jlu), ip(ju))
    return x


def grid_build(mesh, variant=None) -> dict:
    """Reference face construction (polyGrid%up + getNeib + sort) on a Mesh."""
    L = lib(variant)
    pN = np.ascontiguousarray(mesh.pN, np.float64)
    iNE = np.ascontiguousarray(mesh.iNE, np.int32)
    g = L.og_grid_build(mesh.nN, dp(pN), mesh.nE, iNE.shape[1],
                        ip(np.ascontiguousarray(mesh.sE, np.int32)),
                        ip(np.ascontiguousarray(mesh.nNE, np.int32)), ip(iNE),
                        ip(np.ascontiguousarray(mesh.gid, np.int32)))
    try:
        sz = np.zeros(7, np.int32)
        L.og_grid_sizes(g, ip(sz))
        nC, nE, nP, nPi, nPb, mf, nF = (int(x) for x in sz)
        out = dict(nC=nC, nE=nE, nP=nP, nPi=nPi, nPb=nPb, maxFace=mf, nF=nF,
                   iEP=np.zeros((nP, 2), np.int32), aP=np.zeros(nP), normP=np.zeros((nP, 3)),
                   pP=np.zeros((nP, 3)), v=np.zeros(nC), neib=np.zeros((nC, mf), np.int32),
                   gid=np.zeros(nE, np.int32), p=np.zeros((nE, 3)), sE=np.zeros(nE, np.int32))
        L.og_grid_copy(g, ip(out["iEP"]), dp(out["aP"]), dp(out["normP"]), dp(out["pP"]),
                       dp(out["v"]), ip(out["neib"]), ip(out["gid"]), dp(out["p"]), ip(out["sE"]))
    finally:
        L.og_grid_free(g)
    return out


class Euler:
    """oe_ctx: the reference foeuler module state restated on the CPU."""

    def __init__(self, grid, iBC, bc_type, bc_param, gamm, r, elem_state, threads=1,
                 variant=None):
        self.L = L = lib(variant)
        self.nC, self.nE = grid["nC"] if isinstance(grid, dict) else grid.nC, \
            grid["nE"] if isinstance(grid, dict) else grid.nE
        gg = grid if isinstance(grid, dict) else grid.__dict__
        rho, ru, rv, rw, rE = (np.ascontiguousarray(x, np.float64) for x in elem_state)
        rhou = np.ascontiguousarray(np.stack([ru, rv, rw], axis=1))
        nBC = int(len(bc_type))
        bcp = np.ascontiguousarray(np.asarray(bc_param, np.float64).reshape(max(nBC, 1), -1)) \
            if nBC else np.zeros((1, 5))
        self._keep = [np.ascontiguousarray(gg["iEP"], np.int32), np.ascontiguousarray(gg["aP"]),
                      np.ascontiguousarray(gg["normP"]), np.ascontiguousarray(gg["v"]),
                      np.ascontiguousarray(gg["neib"], np.int32),
                      np.ascontiguousarray(iBC, np.int32),
                      np.ascontiguousarray(bc_type, np.int32) if nBC else np.zeros(1, np.int32),
                      bcp, rho, rhou, rE]
        k = self._keep
        self.h = L.oe_new(self.nC, self.nE, gg["nPi"], gg["nPb"], ip(k[0]), dp(k[1]), dp(k[2]),
                          dp(k[3]), gg["maxFace"], ip(k[4]), ip(k[5]), nBC, ip(k[6]), dp(k[7]),
                          int(bcp.shape[1]), gamm, r, dp(rho), dp(rhou), dp(rE))
        self.set_threads(threads)

    def set_threads(self, n):
        self.L.oe_set_threads(self.h, int(n))

    def set_ilu_order(self, old2new):
        """ILU(0) cell order (old -> new, 0-based); None = natural reference order."""
        if old2new is None:
            self.L.oe_set_ilu_order(self.h, None)
        else:
            self._perm = np.ascontiguousarray(old2new, np.int32)
            self.L.oe_set_ilu_order(self.h, ip(self._perm))

    def set_ilut(self, lfil=50, droptol=1e-6):
        """pset/psol with ILUT (the ILU class of numerics/sparse.f90) instead of ilu0;
        lfil=None goes back to ilu0."""
        self.L.oe_set_ilut(self.h, -1 if lfil is None else int(lfil), float(droptol))

    def ilut_factors(self):
        """(alu, jlu, ju) of the last ILUT factorisation, MSR arrays trimmed to their use."""
        alu, jlu, ju = _dp(), _ip(), _ip()
        iwk = self.L.oe_ilut_factors(self.h, C.byref(alu), C.byref(jlu), C.byref(ju))
        if iwk < 0:
            raise RuntimeError("no ILUT set")
        n = 5 * self.nC
        jl = np.ctypeslib.as_array(jlu, shape=(iwk,))
        used = int(jl[n]) - 1
        return (np.ctypeslib.as_array(alu, shape=(iwk,))[:used].copy(), jl[:used].copy(),
                np.ctypeslib.as_array(ju, shape=(n,)).copy())

    def close(self):
        if self.h:
            self.L.oe_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rhs(self, t, y, ydot):
        return self.L.oe_rhs(t, dp(y), dp(ydot), self.h)

    def pset(self, t, y, fy, jok, gamma):
        jc = C.c_int(0)
        rc = self.L.oe_pset(t, dp(y), dp(fy) if fy is not None else None, jok, C.byref(jc), gamma,
                           self.h)
        return rc, jc.value

    def psol(self, t, y, fy, r, z, gamma, delta=0.0, lr=1):
        return self.L.oe_psol(t, None, None, dp(r), dp(z), gamma, delta, lr, self.h)

    def jac(self, y, maxFace):
        ptr = self.L.oe_jac(self.h, dp(y))
        n = 5 * (5 * maxFace + 5) * self.nC
        a = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
        # Fortran JacC(5, 5*(maxFace+1), nC) column-major -> [cell, block col, row]
        return a.reshape(self.nC, 5 * maxFace + 5, 5)

    def pmat(self):
        a, ja, ia = _dp(), _ip(), _ip()
        nnz = self.L.oe_pmat(self.h, C.byref(a), C.byref(ja), C.byref(ia))
        n = 5 * self.nC
        return (np.ctypeslib.as_array(a, shape=(nnz,)).copy(),
                np.ctypeslib.as_array(ja, shape=(nnz,)).copy(),
                np.ctypeslib.as_array(ia, shape=(n + 1,)).copy())

    def elem_state(self):
        rho = np.zeros(self.nE)
        rhou = np.zeros(3 * self.nE)
        rE = np.zeros(self.nE)
        self.L.oe_elem_state(self.h, dp(rho), dp(rhou), dp(rE))
        return rho, rhou.reshape(-1, 3), rE

    def jv(self, y, fy, v, out, a, b, ynorm, eps, work=None):
        """The oracle driver's finite-difference Jv (o_jv) through this context's rhs."""
        if work is None:
            work = (np.empty_like(y), np.empty_like(y))
        return self.L.o_jv(y.size, C.cast(self.L.oe_rhs, _vp), self.h, 0.0, dp(y), dp(fy), dp(v),
                           dp(out), a, b, ynorm, eps, dp(work[0]), dp(work[1]))

    def callbacks(self):
        L = self.L
        return (C.cast(L.oe_rhs, _vp), C.cast(L.oe_pset, _vp), C.cast(L.oe_psol, _vp))


def bdf_defaults(**kw) -> BdfOpts:
    o = BdfOpts()
    lib().o_bdf_defaults(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def bdf_run(n, rhs, pset, psol, ud, y, opts, t0=0.0, variant=None):
    """rhs/pset/psol: raw C function pointers (c_void_p) or ctypes CFUNCTYPE objects."""
    st = BdfStats()
    as_vp = lambda f: f if isinstance(f, (C.c_void_p, int)) or f is None else C.cast(f, _vp)
    rc = lib(variant).o_bdf_run(n, as_vp(rhs), as_vp(pset), as_vp(psol), ud, t0, dp(y), C.byref(opts),
                         C.byref(st))
    return rc, st.as_dict()


def adapt_defaults(**kw) -> AdaptOpts:
    o = AdaptOpts()
    lib().o_adapt_defaults(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def bdf_adaptive(n, rhs, pset, psol, ud, y, t0, tout, nk, ad):
    """Variable-order, variable-step BDF from t0 to tout; returns (rc, stats, step stats)."""
    st, ast = BdfStats(), AdaptStats()
    as_vp = lambda f: f if isinstance(f, (C.c_void_p, int)) or f is None else C.cast(f, _vp)
    rc = lib().o_bdf_adaptive(n, as_vp(rhs), as_vp(pset), as_vp(psol), ud, t0, tout, dp(y),
                              C.byref(nk), C.byref(ad), C.byref(st), C.byref(ast))
    return rc, st.as_dict(), ast.as_dict()
