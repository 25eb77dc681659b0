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


def test_ilu1_kat_ilut():
    """src/test/ILU1.f90:11-22 as the reference runs it: ILU%init(4, 7, 4) (lfil clamped to
    3), setCOO without clean-up (rows keep the COO order: row 2 is [2, 1], row 4 is [4, 2]),
    fact(0) = ilut with droptol 0, solve = lusol: x = [1, 3/2, 14/5, 11/4] within 1e-9."""
    ao, jao, iao = _csr()
    assert list(jao[iao[1] - 1:iao[2] - 1]) == [2, 1]
    ierr, alu, jlu, ju = O.ilut(4, ao, jao, iao, 4, 0.0)
    assert ierr == 0
    x = O.lusol(4, [1.0, 2.0, 3.0, 4.0], alu, jlu, ju)
    assert np.linalg.norm(x - [1.0, 1.5, 2.8, 2.75]) <= 1e-9


def _dense_lu_of_msr(n, alu, jlu, ju):
    """L (unit lower) and U (upper, diagonal un-inverted) as dense matrices."""
    L, U = np.eye(n), np.zeros((n, n))
    for i in range(n):
        U[i, i] = 1.0 / alu[i]
        for k in range(jlu[i] - 1, ju[i] - 1):
            L[i, jlu[k] - 1] = alu[k]
        for k in range(ju[i] - 1, jlu[i + 1] - 1):
            U[i, jlu[k] - 1] = alu[k]
    return L, U


def _random_csr(n, density, seed, dominance=4.0):
    rng = np.random.default_rng(seed)
    A = (rng.random((n, n)) < density) * rng.normal(size=(n, n))
    A += np.diag(dominance + np.abs(A).sum(1) * 0.1 + rng.random(n))
    ia = np.zeros(n + 1, np.int32)
    ja, a = [], []
    for i in range(n):
        cols = np.flatnonzero(A[i])
        rng.shuffle(cols)  # ilut takes rows in any column order
        ja += list(cols + 1)
        a += list(A[i, cols])
        ia[i + 1] = ia[i] + len(cols)
    return A, np.array(a), np.array(ja, np.int32), ia + 1


def test_ilut_without_dropping_is_exact_lu():
    """lfil = n - 1 and droptol = 0 keep every entry: L U = A (no pivoting)."""
    n = 40
    A, a, ja, ia = _random_csr(n, 0.15, 1)
    ierr, alu, jlu, ju = O.ilut(n, a, ja, ia, n, 0.0)
    assert ierr == 0
    L, U = _dense_lu_of_msr(n, alu, jlu, ju)
    np.testing.assert_allclose(L @ U, A, atol=1e-12 * np.abs(A).max())


def test_ilut_dual_threshold_limits():
    """Every L row keeps at most lfil entries and every U row at most lfil - 1 off-diagonal
    entries (the quick-split keeps min(lenu, lfil) including the diagonal slot); stored U
    entries exceed droptol * mean |a| of their row; quick-split keeps the largest."""
    n, lfil, tol = 60, 5, 1e-3
    A, a, ja, ia = _random_csr(n, 0.3, 2)
    ierr, alu, jlu, ju = O.ilut(n, a, ja, ia, lfil, tol)
    assert ierr == 0
    for i in range(n):
        nl = ju[i] - jlu[i]
        nu = jlu[i + 1] - ju[i]
        assert nl <= lfil and nu <= lfil - 1
        tnorm = np.abs(A[i]).sum() / np.count_nonzero(A[i])
        u = alu[ju[i] - 1:jlu[i + 1] - 1]
        assert np.all(np.abs(u) > tol * tnorm)
        assert np.all(jlu[ju[i] - 1:jlu[i + 1] - 1] > i + 1)
        assert np.all(jlu[jlu[i] - 1:ju[i] - 1] < i + 1)


def test_qsplit_partitions_by_magnitude():
    rng = np.random.default_rng(4)
    for n, cut in ((1, 1), (7, 3), (50, 10), (50, 50), (30, 1)):
        a = rng.normal(size=n)
        ind = np.arange(n, dtype=np.int32)
        a0 = a.copy()
        O.lib().o_qsplit(O.dp(a), O.ip(ind), n, cut)
        np.testing.assert_array_equal(a, a0[ind])
        assert np.abs(a[:cut]).min() >= np.abs(a[cut - 1:]).max() - 0.0


def test_ilut_error_codes():
    """-5 zero row, -4 negative lfil, -3 U storage exhausted: the ILU class sizes alu to
    n*min(2*lfil+1, n), which for n = 2 is 4 < n + 2, so even a diagonal matrix fails."""
    L = O.lib()

    def run(a, ja, ia, lfil, iwk):
        n = len(ia) - 1
        w, jw = np.zeros(n + 1), np.zeros(2 * n, np.int32)
        alu, jlu, ju = np.zeros(iwk), np.zeros(iwk, np.int32), np.zeros(n, np.int32)
        return L.o_ilut(n, O.dp(np.array(a)), O.ip(np.array(ja, np.int32)),
                        O.ip(np.array(ia, np.int32)), lfil, 0.0, O.dp(alu), O.ip(jlu), O.ip(ju),
                        iwk, O.dp(w), O.ip(jw))

    assert run([1.0, 0.0], [1, 2], [1, 2, 3], 1, 16) == -5
    assert run([1.0, 1.0], [1, 2], [1, 2, 3], -1, 16) == -4
    assert run([1.0, 1.0], [1, 2], [1, 2, 3], 1, 16) == 0
    assert O.ilut(2, np.array([1.0, 1.0]), np.array([1, 2], np.int32),
                  np.array([1, 2, 3], np.int32), 1, 0.0)[0] == -3


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


def test_tuned_build_is_bit_identical():
    """The CPU baseline times the oracle built for the host's instruction set; with
    multiply-add contraction off in both builds it must compute exactly what the checker
    computes: residual, grid, and two BDF2 steps with ILU(0) (single thread, so the
    summation order is fixed)."""
    from fosolvers_gb300 import mesh as M
    wl = M.make_workload("sine96", scale=6, seed=1)
    grids = [O.grid_build(wl.mesh, variant=v) for v in ("checker", "tuned")]
    for k in ("iEP", "aP", "normP", "v", "neib"):
        assert np.array_equal(grids[0][k], grids[1][k]), k
    ibc = M.ibc_for(wl.mesh, wl.bc_gid)
    out = []
    for v in ("checker", "tuned"):
        e = O.Euler(grids[0], ibc, wl.bc_type, wl.bc_param, wl.gamm, wl.r, wl.elem_state,
                    variant=v)
        y = M.soa(wl.elem_state, grids[0]["nC"])
        f = np.zeros_like(y)
        assert e.rhs(0.0, y, f) == 0
        rhs, pset, psol = e.callbacks()
        rc, st = O.bdf_run(y.size, rhs, pset, psol, e.h, y,
                           O.bdf_defaults(order=2, dt=wl.dt, nsteps=2), variant=v)
        assert rc == 0
        out.append((f, y, st))
        e.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_failed_step_keeps_last_accepted_state():
    """A BDF step whose Newton iteration fails (GMRES(1) without restarts or preconditioner,
    an unreachable linear tolerance, two Newton iterations, the supersonic bump at CFL ~5) is
    not taken: the driver returns 1 and y is the last accepted state."""
    from fosolvers_gb300 import mesh as M
    wl = M.make_workload("bump192", scale=8)
    g = O.grid_build(wl.mesh)
    e = O.Euler(g, M.ibc_for(wl.mesh, wl.bc_gid), wl.bc_type, wl.bc_param, wl.gamm, wl.r,
                wl.elem_state)
    y0 = M.soa(wl.elem_state, g["nC"])
    rhs, pset, psol = e.callbacks()
    y = y0.copy()
    rc, st = O.bdf_run(y.size, rhs, pset, psol, e.h, y,
                       O.bdf_defaults(order=1, dt=wl.dt, nsteps=2, maxl=1, max_restarts=0,
                                      lin_rtol=1e-30, max_newton=2, use_prec=0))
    assert rc == 1 and st["n_steps"] == 0 and st["fails"] == 1 and st["n_newton"] == 2
    assert np.array_equal(y, y0)
    # the same context advances normally afterwards
    rc, st = O.bdf_run(y.size, rhs, pset, psol, e.h, y,
                       O.bdf_defaults(order=1, dt=wl.dt, nsteps=1))
    assert rc == 0 and st["n_steps"] == 1
    e.close()


def test_bdf_predictor_extrapolates():
    """The constant-step BDF predictor (predictor = 1): on the smooth sine state Newton
    starts from 2 y_n - y_{n-1} (order 1) and 3 y_n - 3 y_{n-1} + y_{n-2} (order 2) and needs
    fewer iterations than from y_n, landing on the same BDF solution within the Newton
    tolerance; the first step, with no history, is the same as from y_n."""
    from fosolvers_gb300 import mesh as M
    wl = M.make_workload("sine96", scale=8)
    g = O.grid_build(wl.mesh)
    e = O.Euler(g, M.ibc_for(wl.mesh, wl.bc_gid), wl.bc_type, wl.bc_param, wl.gamm, wl.r,
                wl.elem_state)
    y0 = M.soa(wl.elem_state, g["nC"])
    rhs, pset, psol = e.callbacks()
    res = {}
    for pred in (0, 1):
        for n in (1, 8):
            y = y0.copy()
            rc, st = O.bdf_run(y.size, rhs, pset, psol, e.h, y,
                               O.bdf_defaults(order=2, dt=wl.dt, nsteps=n, predictor=pred))
            assert rc == 0
            res[pred, n] = (y, st)
    e.close()
    assert np.array_equal(res[0, 1][0], res[1, 1][0])  # no history: the same first step
    assert res[1, 8][1]["n_newton"] < res[0, 8][1]["n_newton"]
    a, b = res[0, 8][0].reshape(5, -1), res[1, 8][0].reshape(5, -1)
    assert max(np.abs(a[q] - b[q]).max() / np.abs(a[q]).max() for q in range(5)) < 1e-5


def test_oracle_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the oracle's option and statistics structs have the header's
    size and field offsets, checked against gcc's layout of oracle/fos_oracle.h."""
    import shutil
    import subprocess
    from pathlib import Path
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    root = Path(__file__).resolve().parents[1]
    structs = {"o_bdf_opts": O.BdfOpts, "o_bdf_stats": O.BdfStats, "o_adapt_opts": O.AdaptOpts,
               "o_adapt_stats": O.AdaptStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fos_oracle.h"',
             'int main(void) {']
    for cname, st in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in st._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(root / "oracle"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True,
                               text=True).stdout.split("\n"):
        if line:
            a, b, v = line.split()
            got[a, b] = int(v)
    for cname, st in structs.items():
        assert got[cname, "size"] == C.sizeof(st), cname
        for fname, _ in st._fields_:
            assert got[cname, fname] == getattr(st, fname).offset, (cname, fname)
