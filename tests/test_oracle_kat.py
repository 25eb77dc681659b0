"""The oracle against the reference's own known-answer tests (src/test/*.f90) and
against properties the reference arithmetic must have.  CPU only."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as O


# ---------------------------------------------------------------- reference KATs
COO = dict(iA=np.array([1, 2, 2, 3, 3, 4, 4], np.int32), jA=np.array([1, 2, 1, 3, 4, 4, 2], np.int32),
           A=np.array([1.0, 2.0, -1.0, 5.0, -4.0, 2.0, -1.0]))


def _csr():
    L = O.lib()
    ao, jao, iao = np.zeros(7), np.zeros(7, np.int32), np.zeros(5, np.int32)
    L.o_coocsr(4, 7, O.dp(COO["A"]), O.ip(COO["iA"]), O.ip(COO["jA"]), O.dp(ao), O.ip(jao), O.ip(iao))
    return ao, jao, iao


def test_matvecmul_kat(oracle_lib):
    """src/test/matVecMul.f90:11-21: amux(x) = [1,2,3,4] within 1e-9."""
    ao, jao, iao = _csr()
    x = np.array([1.0, 1.5, 14.0 / 5.0, 11.0 / 4.0])
    y = np.zeros(4)
    oracle_lib.o_amux(4, O.dp(x), O.dp(y), O.dp(ao), O.ip(jao), O.ip(iao))
    assert np.linalg.norm(y - [1, 2, 3, 4]) <= 1e-9


def test_ilu1_kat(oracle_lib):
    """src/test/ILU1.f90:11-22 (ILUT with no fill); ILU(0) is exact on this pattern:
    ilu0 + lusol must give x = [1, 3/2, 14/5, 11/4] within 1e-9."""
    ao, jao, iao = _csr()
    oracle_lib.o_csrsort(4, O.dp(ao), O.ip(jao), O.ip(iao))  # ilu0 needs L before U per row
    alu, jlu = np.zeros(10), np.zeros(10, np.int32)
    ju, iw = np.zeros(4, np.int32), np.zeros(4, np.int32)
    ierr = oracle_lib.o_ilu0(4, O.dp(ao), O.ip(jao), O.ip(iao), O.dp(alu), O.ip(jlu), O.ip(ju), O.ip(iw))
    assert ierr == 0
    x = np.zeros(4)
    oracle_lib.o_lusol(4, O.dp(np.array([1.0, 2.0, 3.0, 4.0])), O.dp(x), O.dp(alu), O.ip(jlu), O.ip(ju))
    assert np.linalg.norm(x - [1.0, 1.5, 2.8, 2.75]) <= 1e-9


def test_ilu0_zero_pivot_reports_row(oracle_lib):
    """ilu0 returns ierr = k on a zero pivot at step k (ilut.f:1896,1911)."""
    A = np.array([1.0, 0.0, 1.0])
    ia = np.array([1, 2, 3, 4], np.int32)
    ja = np.array([1, 2, 3], np.int32)
    alu, jlu = np.zeros(6), np.zeros(6, np.int32)
    ju, iw = np.zeros(3, np.int32), np.zeros(3, np.int32)
    assert oracle_lib.o_ilu0(3, O.dp(A), O.ip(ja), O.ip(ia), O.dp(alu), O.ip(jlu), O.ip(ju), O.ip(iw)) == 2


def test_newton_krylov_kat(oracle_lib):
    """src/test/NewtonKrylov1.f90:9-16: y = [2,4,-8]x + [1,2,3] = 0 -> [-1/2, -1/2, 3/8]."""
    @O.RHS_FN
    def g(t, x, y, ud):
        for i, (a, b) in enumerate(zip([2.0, 4.0, -8.0], [1.0, 2.0, 3.0])):
            y[i] = a * x[i] + b
        return 0
    x = np.zeros(3)
    st = O.BdfStats()
    rc = oracle_lib.o_newton_solve(3, C.cast(g, C.c_void_p), None, O.dp(x), 1e-8, 1e-12, 10, 30,
                                   1e-12, C.byref(st))
    assert rc == 0
    assert np.linalg.norm(x - [-0.5, -0.5, 0.375]) <= 1e-9


def test_bdf_newton_krylov_kat():
    """src/test/BDFNewtonKrylov1.f90:10-23 with the fixed-step driver: x' = y, y' = -x from
    (1, 0) to t = 2, rtol 1e-8, atol 1e-12, ||s - (cos t, -sin t)|| <= 1e-6.  Re-derived
    step: BDF2's global error ~ (2/9) dt^2 t, so dt = 5e-4 (4000 steps) gives ~2e-7."""
    @O.RHS_FN
    def f(t, x, dx, ud):
        dx[0] = x[1]
        dx[1] = -x[0]
        return 0
    opts = O.bdf_defaults(order=2, dt=5e-4, nsteps=4000, use_prec=0, newton_rtol=1e-8,
                          newton_atol=1e-12)
    s = np.array([1.0, 0.0])
    rc, st = O.bdf_run(2, f, None, None, None, s, opts)
    assert rc == 0 and st["n_steps"] == 4000
    assert np.linalg.norm(s - [np.cos(2.0), -np.sin(2.0)]) <= 1e-6


def test_unit_hex_volume(oracle_lib):
    """src/test/polyGrid1.f90:10-16: the unit hexahedron of data/grid_simple.vtk has v = 1
    within 1e-14 (v8p)."""
    p = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1],
                  [0, 1, 1]], np.float64)
    assert abs(oracle_lib.og_v8p(O.dp(np.ascontiguousarray(p))) - 1.0) < 1e-14


def test_tet_face_tables_point_outward():
    """getINF TET faces [1,3,2],[1,2,4],[1,4,3],[2,3,4] with n3p give outward normals on a
    positively oriented tetrahedron (polyGrid.f90:236-247, geometry.f90:38-49)."""
    from fosolvers_gb300 import mesh as M
    m = M.box_mesh(1, 1, 1, jitter=0.0)
    g = O.grid_build(m)
    cen = g["p"][: g["nC"]]
    for i, (a, b) in enumerate(g["iEP"]):
        d = g["pP"][i] - cen[a - 1]
        assert np.dot(d, g["normP"][i]) > 0.0


# ---------------------------------------------------------------- Jacobian properties
def _nfj(n, u, H, g=1.4):
    out = np.zeros(25)
    O.lib().oe_nfj(O.dp(np.ascontiguousarray(n, np.float64)), O.dp(np.ascontiguousarray(u, np.float64)),
                   H, g, O.dp(out))
    return out.reshape(5, 5, order="F")


def _anfj(n, u, H, c, g=1.4):
    out = np.zeros(25)
    O.lib().oe_anfj(O.dp(np.ascontiguousarray(n, np.float64)), O.dp(np.ascontiguousarray(u, np.float64)),
                    H, c, g, O.dp(out))
    return out.reshape(5, 5, order="F")


def _flux_n(U, n, g=1.4):
    rho, m, E = U[0], U[1:4], U[4]
    u = m / rho
    p = (g - 1) * (E - 0.5 * rho * u @ u)
    un = u @ n
    return np.concatenate([[rho * un], rho * u * un + p * n, [(E + p) * un]])


@pytest.mark.parametrize("seed", range(4))
def test_nfj_is_flux_derivative(seed):
    """eulerNFJ (Euler.f90:252-276) equals the finite-difference derivative of F(U).n."""
    rng = np.random.default_rng(seed)
    g = 1.4
    n = rng.normal(size=3)
    n /= np.linalg.norm(n)
    rho, u, p = 1.0 + rng.random(), rng.normal(size=3), 1.0 + rng.random()
    U = np.concatenate([[rho], rho * u, [p / (g - 1) + 0.5 * rho * u @ u]])
    H = (U[4] + p) / rho
    A = _nfj(n, u, H, g)
    h = 1e-6
    Afd = np.stack([(_flux_n(U + h * e, n) - _flux_n(U - h * e, n)) / (2 * h) for e in np.eye(5)], 1)
    assert np.abs(A - Afd).max() <= 1e-7 * np.abs(A).max()


@pytest.mark.parametrize("seed", range(4))
def test_anfj_is_abs_of_nfj(seed):
    """eulerANFJ (Euler.f90:279-333) equals R |Lambda| R^-1 of eulerNFJ built independently,
    except column 1, rows 2:4 of the |vn| (entropy + shear) term: the reference writes
    -(1 + (g-1)/2 M^2) u + vn n (Euler.f90:300) where the exact projector has
    -(g-1)/2 M^2 u + vn n, i.e. an extra -|vn| u.  The restatement keeps the reference."""
    rng = np.random.default_rng(100 + seed)
    g = 1.4
    n = rng.normal(size=3)
    n /= np.linalg.norm(n)
    u = 0.7 * rng.normal(size=3)
    c = 1.0 + rng.random()
    H = c * c / (g - 1) + 0.5 * u @ u
    A = _nfj(n, u, H, g)
    lam, R = np.linalg.eig(A)
    absA = (R * np.abs(lam.real)) @ np.linalg.inv(R)
    assert np.abs(absA.imag).max() < 1e-10
    expect = absA.real.copy()
    expect[1:4, 0] -= abs(u @ n) * u
    assert np.abs(_anfj(n, u, H, c, g) - expect).max() <= 1e-10 * np.abs(absA).max()
