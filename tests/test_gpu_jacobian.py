"""GPU block Jacobian and block ILU(0) against the oracle.

J: every 5x5 block of the GPU block-CSR (internal order) equals the oracle's JacC
(findEulerJac, reference order) within 1e-12 of the largest entry.  ILU: z = P^-1 r
from the GPU's level-scheduled block ILU(0) equals SPARSKIT ilu0 + lusol on the scalar
interleaved matrix within 1e-10 (block ILU(0) with dense diagonal blocks is scalar ILU(0)
of the interleaved matrix), with the oracle factoring in the GPU's cell order (ILU(0)
depends on the order)."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import ILU_COLOR, ILU_FP32
from helpers import Case, hex_workload, perturbed, rel_err, with_all_conditions

pytestmark = pytest.mark.gpu


def _workload(name):
    if name == "hex8":  # six-face cells: block rows of up to 7 blocks
        return hex_workload(8, seed=1)
    if name == "conds6":  # every condition type on the box sides
        return with_all_conditions(M.make_workload("sod16", scale=6))
    if name == "conds-hex8":
        return with_all_conditions(hex_workload(8, seed=1))
    return M.make_workload("sine96", scale=8, seed=1)


@pytest.fixture(scope="module",
                params=["sine8", "bump16", "sine8-colour", "hex8", "hex8-colour", "conds6"])
def case(request, cuda):
    if request.param.startswith("hex") or request.param == "conds6":
        return Case(_workload(request.param.split("-")[0]),
                    flags=ILU_COLOR if "colour" in request.param else 0)
    if request.param == "sine8":
        return Case(M.make_workload("sine96", scale=8, seed=1))
    if request.param == "sine8-colour":
        return Case(M.make_workload("sine96", scale=8, seed=1), flags=ILU_COLOR)
    return Case(M.make_workload("bump192", scale=16))


def test_jacobian_blocks_match_oracle(case):
    _check_blocks(case, 1e-12)


@pytest.mark.parametrize("name", ["sine8", "hex8", "conds6", "conds-hex8"])
def test_fp32_jacobian_blocks(cuda, name):
    """The cell-centric FP32 assembly (FP32 (hi, lo) primitives, FP32 face arithmetic, FP64
    ghost states) against the FP64 oracle: every block within 1e-5 of the largest entry."""
    _check_blocks(Case(_workload(name), flags=ILU_FP32), 1e-5)


def _check_blocks(c: Case, tol: float):
    y = perturbed(c.y0, c.nC, 3)
    mf = c.grid.maxFace
    ref = c.oracle.jac(y, mf)  # [cell, col, row]
    rc, jcur = c.gpu.pset(0.0, y, None, 0, 1e-3)
    assert rc == 0 and jcur == 1
    rowptr, col, val = c.gpu.jacobian()
    pos = c.gpu.ilu_order()  # block rows / columns are ILU positions
    scale = np.abs(ref).max()
    nblk = 0
    for cell in range(c.nC):
        p = pos[cell]
        cols = list(col[rowptr[p]:rowptr[p + 1]])
        blocks = [(cell, 0)] + [(k - 1, j + 1) for j, k in enumerate(c.grid.neib[cell]) if 1 <= k <= c.nC]
        assert len(blocks) == len(cols)
        for other, j in blocks:
            s = rowptr[p] + cols.index(pos[other])
            want = ref[cell, 5 * j:5 * j + 5, :].T
            assert np.abs(val[s] - want).max() <= tol * scale
            nblk += 1
    assert nblk == len(col)


def test_ilu_apply_matches_sparskit(case):
    c = case
    y = perturbed(c.y0, c.nC, 4)
    gamma = 5e-3
    c.match_ilu_order()
    assert c.oracle.pset(0.0, y, None, 0, gamma) == (0, 1)
    rc, _ = c.gpu.pset(0.0, y, None, 0, gamma)
    assert rc == 0
    rng = np.random.default_rng(8)
    for _ in range(2):
        r = rng.normal(size=c.N)
        z_ref = np.zeros_like(r)
        z = np.zeros_like(r)
        c.oracle.psol(0.0, None, None, r, z_ref, gamma)
        assert c.gpu.psol(0.0, y, None, r, z, gamma) == 0
        assert rel_err(z, z_ref) <= 1e-10
    info = c.gpu.info()
    assert info["nlev_fwd"] >= 2 and info["nlev_bwd"] >= 2
    if c.flags & ILU_COLOR:
        assert info["nlev_fwd"] <= c.grid.maxFace + 2 and info["nlev_bwd"] <= c.grid.maxFace + 2


def test_pset_jok_reuses_jacobian(case):
    """jok = 1 keeps J and only re-scales by the new gamma (CVODE pset contract)."""
    c = case
    y = perturbed(c.y0, c.nC, 6)
    c.match_ilu_order()
    c.gpu.pset(0.0, y, None, 0, 1e-3)
    rc, jcur = c.gpu.pset(0.0, 2.0 * y, None, 1, 2e-3)
    assert rc == 0 and jcur == 0
    c.oracle.pset(0.0, y, None, 0, 1e-3)
    assert c.oracle.pset(0.0, 2.0 * y, None, 1, 2e-3) == (0, 0)
    r = np.random.default_rng(1).normal(size=c.N)
    z, z_ref = np.zeros_like(r), np.zeros_like(r)
    c.oracle.psol(0.0, None, None, r, z_ref, 2e-3)
    c.gpu.psol(0.0, y, None, r, z, 2e-3)
    assert rel_err(z, z_ref) <= 1e-10


@pytest.mark.parametrize("name,extra", [("sine8", 0), ("hex8", 0), ("sine8", ILU_COLOR),
                                        ("hex8", ILU_COLOR)])
def test_fp32_ilu_apply(cuda, name, extra):
    """FP32 factors and sweeps in the level-scheduled and the colour order (where the last
    forward colour also applies inv(D) and the colour without L blocks takes no launch)."""
    c = Case(_workload(name), flags=ILU_FP32 | extra)
    y = perturbed(c.y0, c.nC, 4)
    c.match_ilu_order()
    c.oracle.pset(0.0, y, None, 0, 5e-3)
    c.gpu.pset(0.0, y, None, 0, 5e-3)
    r = np.random.default_rng(2).normal(size=c.N)
    z, z_ref = np.zeros_like(r), np.zeros_like(r)
    c.oracle.psol(0.0, None, None, r, z_ref, 5e-3)
    c.gpu.psol(0.0, y, None, r, z, 5e-3)
    assert rel_err(z, z_ref) <= 1e-5


@pytest.mark.parametrize("name,extra", [("sine8", ILU_COLOR), ("sine8", 0), ("hex8", ILU_COLOR),
                                        ("conds6", ILU_COLOR)])
def test_fused_fp32_setup_equals_two_kernel_path(cuda, name, extra):
    """The FP32 set-up assembles J inside the factor (k_pset32) and never stores it.  Its
    factors must equal the two-kernel path's (k_jac_cell32 writes J, k_ilu_factor factors it)
    bit for bit: J is materialised with fos_euler_jac_copy, loaded back with fos_euler_jac_set
    and factored by pset(jok = 1) through the two-kernel path; both applies must agree
    exactly.  jok = 1 without a loaded J reassembles J from the state of the last jok = 0
    call, so a second state passed with jok = 1 must not change the factors either."""
    c = Case(_workload(name), flags=ILU_FP32 | extra)
    y = perturbed(c.y0, c.nC, 7)
    g = 4e-3
    assert c.gpu.pset(0.0, y, None, 0, g) == (0, 1)
    r = np.random.default_rng(3).normal(size=c.N)
    z_fused, z_reuse, z_two = (np.zeros_like(r) for _ in range(3))
    assert c.gpu.psol(0.0, y, None, r, z_fused, g) == 0
    assert c.gpu.pset(0.0, 1.5 * y, None, 1, g) == (0, 0)  # J of y, not of 1.5 y
    assert c.gpu.psol(0.0, y, None, r, z_reuse, g) == 0
    assert np.array_equal(z_fused, z_reuse)
    rowptr, col, val = c.gpu.jacobian()
    c.gpu.set_jacobian(val)
    assert c.gpu.pset(0.0, y, None, 1, g) == (0, 0)
    assert c.gpu.psol(0.0, y, None, r, z_two, g) == 0
    assert np.array_equal(z_fused, z_two)
