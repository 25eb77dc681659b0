"""The variable-order, variable-step BDF restatement (CVODE's step and order control) on the
oracle, on the CPU: scalar ODEs with known solutions (non-stiff decay and a stiff
relaxation onto cos t), tolerance proportionality, order selection, landing on tout, and
the Euler equations on a small Sod box against a tighter-tolerance run."""
import ctypes as C
import math

import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import PolyFvGrid
from oracle import pyoracle as O

RHS = C.CFUNCTYPE(C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)


def scalar_run(f, y0, t1, rtol, h0=1e-3, qmax=5):
    cb = RHS(lambda t, y, yd, ud: (yd.__setitem__(0, f(t, y[0])), 0)[1])
    y = np.array([y0], np.float64)
    nk = O.bdf_defaults(newton_rtol=1e-12, newton_atol=1e-14, use_prec=0, maxl=5)
    ad = O.adapt_defaults(rtol=rtol, atol=1e-12, h0=h0, qmax=qmax)
    rc, st, ast = O.bdf_adaptive(1, cb, None, None, None, y, 0.0, t1, nk, ad)
    assert rc == 0, (st, ast)
    return y[0], st, ast


@pytest.mark.parametrize("rtol", [1e-4, 1e-6, 1e-8])
def test_decay_error_tracks_tolerance(rtol):
    y, st, ast = scalar_run(lambda t, y: -y, 1.0, 2.0, rtol)
    err = abs(y - math.exp(-2.0)) / math.exp(-2.0)
    print(rtol, err, ast)
    assert ast["t"] == 2.0
    assert err <= 50 * rtol
    assert ast["n_accepted"] < 600


def test_higher_orders_are_used_and_save_steps():
    _, _, a5 = scalar_run(lambda t, y: -y, 1.0, 5.0, 1e-8, qmax=5)
    _, _, a1 = scalar_run(lambda t, y: -y, 1.0, 5.0, 1e-8, qmax=1)
    print(a5, a1)
    assert sum(a5["steps_at_order"][3:]) > 0
    assert a5["n_accepted"] < a1["n_accepted"] / 5


def test_stiff_relaxation_takes_large_steps():
    """y' = -1000 (y - cos t): after the transient the step is limited by the smooth
    solution, not by the stiffness (an explicit method would need h < 2e-3)."""
    lam = 1000.0

    def exact(t):
        # y(0) = 0: y = lam/(lam^2+1) (lam cos t + sin t) - lam^2/(lam^2+1) e^{-lam t}
        return (lam / (lam * lam + 1) * (lam * math.cos(t) + math.sin(t))
                - lam * lam / (lam * lam + 1) * math.exp(-lam * t))

    y, st, ast = scalar_run(lambda t, y: -lam * (y - math.cos(t)), 0.0, 3.0, 1e-6, h0=1e-5)
    print(ast, y, exact(3.0))
    assert abs(y - exact(3.0)) <= 1e-4
    assert ast["h_last"] > 5e-3
    assert ast["n_accepted"] < 500


def test_euler_sod_box_against_tighter_tolerance():
    wl = M.make_workload("sod16", scale=6)
    grid = PolyFvGrid.from_mesh(wl.mesh)
    e = O.Euler(grid.__dict__, M.ibc_for(wl.mesh, wl.bc_gid), wl.bc_type, wl.bc_param, wl.gamm,
                wl.r, wl.elem_state)
    rhs, pset, psol = e.callbacks()
    y0 = M.soa(wl.elem_state, grid.nC)
    n = 5 * grid.nC
    out = {}
    for rtol in (1e-4, 1e-7):
        y = y0.copy()
        nk = O.bdf_defaults(newton_rtol=1e-10)
        ad = O.adapt_defaults(rtol=rtol, atol=1e-10, h0=1e-4)
        rc, st, ast = O.bdf_adaptive(n, rhs, pset, psol, e.h, y, 0.0, 0.05, nk, ad)
        assert rc == 0, (st, ast)
        assert ast["t"] == 0.05
        out[rtol] = (y, ast)
    e.close()
    a, b = out[1e-4][0].reshape(5, -1), out[1e-7][0].reshape(5, -1)
    err = max(np.abs(a[q] - b[q]).max() / np.abs(b[q]).max() for q in (0, 4))
    print("sod adaptive", err, out[1e-4][1], out[1e-7][1])
    assert err <= 1e-2
    assert out[1e-7][1]["n_accepted"] > out[1e-4][1]["n_accepted"]
