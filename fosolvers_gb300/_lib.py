"""ctypes binding of libfosgpu.so (the C ABI in include/fosgpu.h).

The library is the only compute path: if it is missing or fails to load, every
entry point raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libfosgpu.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)
_vp = C.c_void_p


class BdfOpts(C.Structure):
    _fields_ = [("order", C.c_int), ("nsteps", C.c_int), ("dt", C.c_double),
                ("newton_rtol", C.c_double), ("newton_atol", C.c_double),
                ("max_newton", C.c_int), ("maxl", C.c_int), ("max_restarts", C.c_int),
                ("lin_rtol", C.c_double), ("jv_eps", C.c_double), ("precond", C.c_int),
                ("jac_reuse", C.c_int), ("resume", C.c_int), ("msbp", C.c_int),
                ("predictor", C.c_int)]


class BdfStats(C.Structure):
    _fields_ = [("n_rhs", C.c_long), ("n_jv", C.c_long), ("n_psol", C.c_long),
                ("n_pset", C.c_long), ("n_newton", C.c_long), ("n_lin_iters", C.c_long),
                ("n_steps", C.c_long), ("fails", C.c_long), ("n_fallback", C.c_long),
                ("last_gnorm", C.c_double), ("t", C.c_double), ("n_learned", C.c_long),
                ("n_gated", C.c_long), ("n_reorth", C.c_long)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdaptOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("h0", C.c_double),
                ("hmin", C.c_double), ("hmax", C.c_double), ("qmax", C.c_int),
                ("max_steps", C.c_int)]


class AdaptStats(C.Structure):
    _fields_ = [("n_accepted", C.c_long), ("n_err_fails", C.c_long),
                ("n_newton_fails", C.c_long), ("h_last", C.c_double), ("t", C.c_double),
                ("q_last", C.c_int), ("steps_at_order", C.c_long * 6)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "steps_at_order"}
        d["steps_at_order"] = list(self.steps_at_order)
        return d


# name -> (restype, argtypes)
_SIGS = {
    "fos_grid_build": (C.c_int, [C.POINTER(_vp), C.c_int, _dp, C.c_int, C.c_int, _ip, _ip, _ip, _ip]),
    "fos_grid_sizes": (None, [_vp, _ip]),
    "fos_grid_copy": (None, [_vp, _ip, _dp, _dp, _dp, _dp, _ip, _ip, _dp, _ip]),
    "fos_grid_free": (None, [_vp]),
    "fos_ctx_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.c_int, C.c_int, C.c_int, _ip, _dp, _dp,
                                 _dp, _ip, C.c_int, _ip, _dp, C.c_int, C.c_double, C.c_double,
                                 C.c_int, C.c_int]),
    "fos_ctx_destroy": (None, [_vp]),
    "fos_ctx_set_stream": (C.c_int, [_vp, _vp]),
    "fos_ctx_info": (None, [_vp, _lp]),
    "fos_ctx_permute_dev": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "fos_ctx_renumbering": (C.c_int, [_vp, _ip]),
    "fos_ctx_ilu_order": (C.c_int, [_vp, _ip]),
    "fos_last_error": (C.c_char_p, []),
    "fos_euler_rhs": (C.c_int, [C.c_double, _dp, _dp, _vp]),
    "fos_euler_pset": (C.c_int, [C.c_double, _dp, _dp, C.c_int, _ip, C.c_double, _vp]),
    "fos_euler_psol": (C.c_int, [C.c_double, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, _vp]),
    "fos_euler_rhs_dev": (C.c_int, [_vp, C.c_double, _vp, _vp]),
    "fos_euler_rhs_dev_static": (C.c_int, [_vp, C.c_double, _vp, _vp]),
    "fos_euler_jv_dev": (C.c_int, [_vp, C.c_double, _vp, _vp, _vp, _vp, C.c_double, C.c_double,
                                   C.c_double, C.c_double]),
    "fos_euler_jv_dev_vnorm": (C.c_int, [_vp, C.c_double, _vp, _vp, _vp, _vp, C.c_double,
                                         C.c_double, C.c_double, C.c_double, C.c_double]),
    "fos_euler_pset_dev": (C.c_int, [_vp, C.c_double, _vp, C.c_int, _ip, C.c_double]),
    "fos_euler_psol_dev": (C.c_int, [_vp, _vp, _vp]),
    "fos_euler_jac_copy": (C.c_long, [_vp, _ip, _ip, _dp]),
    "fos_euler_jac_set": (C.c_int, [_vp, _dp]),
    "fos_gnn_create": (C.c_int, [C.POINTER(_vp), C.c_uint]),
    "fos_gnn_destroy": (None, [_vp]),
    "fos_gnn_num_params": (C.c_int, []),
    "fos_gnn_get_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "fos_gnn_set_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "fos_gnn_apply_dev": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, _vp]),
    "fos_gnn_zero_grad": (C.c_int, [_vp]),
    "fos_gnn_loss_grad_dev": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_double, _dp]),
    "fos_gnn_get_grad": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "fos_gnn_adam_step": (C.c_int, [_vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
    "fos_ctx_attach_gnn": (C.c_int, [_vp, _vp]),
    "fos_ilut_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.c_int]),
    "fos_ilut_factor_dev": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, _vp]),
    "fos_ilut_solve_dev": (C.c_int, [_vp, _vp, _vp, _vp]),
    "fos_ilut_status": (C.c_int, [_vp]),
    "fos_ctx_set_flux_threshold": (C.c_int, [_vp, C.c_double]),
    "fos_ilut_set_wait_limit": (C.c_int, [_vp, C.c_long, C.c_int]),
    "fos_ilut_copy": (C.c_long, [_vp, _dp, _ip, _ip, C.c_long]),
    "fos_ilut_info": (C.c_int, [_vp, _lp]),
    "fos_ilut_destroy": (None, [_vp]),
    "fos_ctx_set_ilut": (C.c_int, [_vp, C.c_int, C.c_double]),
    "fos_bdf_defaults": (None, [C.POINTER(BdfOpts)]),
    "fos_bdf_run": (C.c_int, [_vp, C.c_double, _vp, C.POINTER(BdfOpts), C.POINTER(BdfStats)]),
    "fos_bdf_run_host": (C.c_int, [_vp, C.c_double, _dp, C.POINTER(BdfOpts), C.POINTER(BdfStats)]),
    "fos_bdf_adapt_defaults": (None, [C.POINTER(AdaptOpts)]),
    "fos_bdf_adaptive": (C.c_int, [_vp, C.c_double, C.c_double, _vp, C.POINTER(BdfOpts),
                                   C.POINTER(AdaptOpts), C.POINTER(BdfStats),
                                   C.POINTER(AdaptStats)]),
    "fos_linear_solve_dev": (C.c_int, [_vp, C.c_double, _vp, _vp, C.c_double, _vp, _vp,
                                       C.POINTER(BdfOpts), C.POINTER(BdfStats)]),
}

_lib = None


def lib():
    """Load libfosgpu.so once; raises if it is not built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built: run __graft_entry__.build() or "
                               "python fosolvers_gb300/build.py")
        l = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def last_error() -> str:
    return (lib().fos_last_error() or b"").decode()


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def check(rc: int, what: str) -> int:
    if rc < 0:
        raise RuntimeError(f"{what} failed ({rc}): {last_error()}")
    return rc
