"""The oracle's ILU(0) (SPARSKIT ilu0/lusol restated, scalar, interleaved cell-major
order) equals block ILU(0) in the same cell order, for the natural order and for a
renumbering: the identity the GPU's block factorisation relies on.  CPU only."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from helpers import Case, perturbed, rel_err


def block_ilu0_solve(P: np.ndarray, nC: int, order: np.ndarray, r: np.ndarray) -> np.ndarray:
    """Block ILU(0) (IKJ) of the interleaved matrix P in the cell order `order`
    (order[c] = position of cell c), then the two triangular solves; SoA in/out."""
    inv = np.argsort(order)
    B = lambda i, j: P[5 * inv[i]:5 * inv[i] + 5, 5 * inv[j]:5 * inv[j] + 5]
    pat = [[j for j in range(nC) if i == j or np.any(B(i, j) != 0)] for i in range(nC)]
    LU = {(i, j): B(i, j).copy() for i in range(nC) for j in pat[i]}
    Dinv = {}
    for i in range(nC):
        for k in [k for k in pat[i] if k < i]:
            LU[(i, k)] = LU[(i, k)] @ Dinv[k]
            for j in [j for j in pat[k] if j > k]:
                if (i, j) in LU:
                    LU[(i, j)] -= LU[(i, k)] @ LU[(k, j)]
        Dinv[i] = np.linalg.inv(LU[(i, i)])
    rr = r.reshape(5, nC).T[inv]
    yv = np.zeros_like(rr)
    for i in range(nC):
        yv[i] = rr[i] - sum((LU[(i, k)] @ yv[k] for k in pat[i] if k < i), np.zeros(5))
    z = np.zeros_like(rr)
    for i in reversed(range(nC)):
        z[i] = Dinv[i] @ (yv[i] - sum((LU[(i, j)] @ z[j] for j in pat[i] if j > i), np.zeros(5)))
    out = np.zeros_like(z)
    out[inv] = z
    return out.T.reshape(-1)


@pytest.mark.parametrize("permute", [False, True])
def test_scalar_ilu0_is_block_ilu0(permute):
    c = Case(M.make_workload("sine96", scale=2, seed=1))
    nC = c.nC
    order = np.random.default_rng(3).permutation(nC).astype(np.int32) if permute else np.arange(nC, dtype=np.int32)
    c.oracle.set_ilu_order(order if permute else None)
    y = perturbed(c.y0, nC, 4)
    assert c.oracle.pset(0.0, y, None, 0, 5e-3)[0] == 0
    a, ja, ia = c.oracle.pmat()
    n = 5 * nC
    P = np.zeros((n, n))
    for i in range(n):
        for k in range(ia[i] - 1, ia[i + 1] - 1):
            P[i, ja[k] - 1] = a[k]
    # P is stored in the ILU order; bring it back to the natural interleaved order
    perm = np.concatenate([5 * order[c_] + np.arange(5) for c_ in range(nC)])
    Pn = P[np.ix_(perm, perm)]
    r = np.random.default_rng(8).normal(size=n)
    z = np.zeros(n)
    c.oracle.psol(0.0, None, None, r, z, 5e-3)
    assert rel_err(block_ilu0_solve(Pn, nC, order, r), z) <= 1e-12
    # and it really is an approximate inverse of P: ||P z - r|| small relative to ||r||
    zc = z.reshape(5, nC).T.reshape(-1)
    rc = r.reshape(5, nC).T.reshape(-1)
    assert np.linalg.norm(Pn @ zc - rc) < 0.5 * np.linalg.norm(rc)
