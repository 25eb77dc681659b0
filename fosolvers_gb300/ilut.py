"""The reference's ILU class (src/libfosolvers/numerics/sparse.f90:52-63,334-392) on the GPU.

    p = ILU(n_eq, lfill)           initILU: lfill clamped to n_eq - 1
    p.set_coo(iA, jA, A)           setCOO without clean-up: coocsr, rows keep the COO order
    p.fact(eps)                    factILU: SPARSKIT ilut with drop tolerance eps (default 0)
    x = p.solve(rhs)               solveILU: lusol

Indices in set_coo are 1-based like the Fortran arrays.  `factor_csr` / `solve_dev` take
0-based CSR arrays and vectors already on the device (torch CUDA tensors).  The work runs
in libfosgpu.so (fos_ilut_*); there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


def coo_to_csr(n: int, iA, jA, A):
    """coocsr (SPARSKIT formats.f:164) semantics with 0-based output: entries of a row keep
    their COO order."""
    iA = np.asarray(iA, np.int64) - 1
    jA = np.asarray(jA, np.int64) - 1
    A = np.asarray(A, np.float64)
    order = np.argsort(iA, kind="stable")
    ia = np.zeros(n + 1, np.int32)
    np.add.at(ia, iA + 1, 1)
    ia = np.cumsum(ia).astype(np.int32)
    return ia, jA[order].astype(np.int32), A[order]


class ILU:
    def __init__(self, n_eq: int, lfill: int):
        self.n = int(n_eq)
        h = C.c_void_p()
        check(_lib.lib().fos_ilut_create(C.byref(h), self.n, int(lfill)), "fos_ilut_create")
        self.handle = h
        self._csr = None

    def __del__(self):
        try:
            if self.handle:
                _lib.lib().fos_ilut_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    @property
    def lfil(self) -> int:
        out = (C.c_long * 6)()
        _lib.lib().fos_ilut_info(self.handle, out)
        return int(out[1])

    def set_coo(self, iA, jA, A):
        import torch
        ia, ja, a = coo_to_csr(self.n, iA, jA, A)
        self._csr = tuple(torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (ia, ja, a))

    def factor_csr(self, ia_dev, ja_dev, a_dev, droptol: float = 0.0, stream=None) -> int:
        raw = getattr(stream, "cuda_stream", stream) or 0
        return check(_lib.lib().fos_ilut_factor_dev(self.handle, ia_dev.data_ptr(), ja_dev.data_ptr(),
                                                    a_dev.data_ptr(), float(droptol), C.c_void_p(raw)),
                     "fos_ilut_factor_dev")

    def fact(self, eps: float = 0.0) -> int:
        if self._csr is None:
            raise RuntimeError("ILU.fact: set_coo first")
        return self.factor_csr(*self._csr, droptol=eps)

    def solve_dev(self, y_dev, x_dev, stream=None):
        raw = getattr(stream, "cuda_stream", stream) or 0
        check(_lib.lib().fos_ilut_solve_dev(self.handle, y_dev.data_ptr(), x_dev.data_ptr(),
                                            C.c_void_p(raw)), "fos_ilut_solve_dev")

    def solve(self, rhs) -> np.ndarray:
        import torch
        y = torch.from_numpy(np.ascontiguousarray(rhs, np.float64)).cuda()
        x = torch.empty_like(y)
        self.solve_dev(y, x)
        torch.cuda.synchronize()
        check(_lib.lib().fos_ilut_status(self.handle), "fos_ilut_status")
        return x.cpu().numpy()

    def set_wait_limit(self, polls: int = 0, withhold_row: int = -1):
        """Failure injection: the polls of every dependency wait (0: the default) and a row
        that is never published (-1: none), for the following factor and solve calls."""
        check(_lib.lib().fos_ilut_set_wait_limit(self.handle, int(polls), int(withhold_row)),
              "fos_ilut_set_wait_limit")

    def msr(self):
        """(alu, jlu, ju): the factors in ilut's MSR layout, 1-based values."""
        L = _lib.lib()
        used = L.fos_ilut_copy(self.handle, None, None, None, 0)
        check(int(used) if used < 0 else 0, "fos_ilut_copy")
        alu = np.zeros(used)
        jlu = np.zeros(used, np.int32)
        ju = np.zeros(self.n, np.int32)
        got = L.fos_ilut_copy(self.handle, _lib.dptr(alu), _lib.iptr(jlu), _lib.iptr(ju), used)
        check(int(got) if got < 0 else 0, "fos_ilut_copy")
        return alu[:got], jlu[:got], ju
