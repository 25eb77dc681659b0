"""The adaptive BDF driver on the GPU against the oracle's restatement of the same step and
order control: identical accepted / rejected step history and orders, final state within
1e-9 relative (FP64 form); and the FP32 form reaching tout with the same kind of history and
a state within 1e-5 of the FP64 run."""
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import FLUX_FP32, ILU_COLOR, ILU_FP32
from helpers import Case, rel_err
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

T1 = 0.05


def gpu_adaptive(c: Case, rtol):
    import torch
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    c.gpu.to_internal(yr, y)
    nk = c.gpu.bdf_defaults(newton_rtol=1e-10)
    ad = c.gpu.adapt_defaults(rtol=rtol, atol=1e-10, h0=1e-4)
    rc, st, ast = c.gpu.bdf_adaptive(y, 0.0, T1, nk, ad)
    assert rc == 0, (st, ast)
    c.gpu.to_reference(y, yr)
    torch.cuda.synchronize()
    return yr.cpu().numpy(), st, ast


def test_adaptive_matches_oracle(cuda):
    c = Case(M.make_workload("sod16", scale=8))
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    y_ref = c.y0.copy()
    rc, st_ref, ast_ref = O.bdf_adaptive(c.N, rhs, pset, psol, c.oracle.h, y_ref, 0.0, T1,
                                         O.bdf_defaults(newton_rtol=1e-10),
                                         O.adapt_defaults(rtol=1e-6, atol=1e-10, h0=1e-4))
    assert rc == 0
    y, st, ast = gpu_adaptive(c, 1e-6)
    print("gpu", ast, "\noracle", ast_ref)
    for k in ("n_accepted", "n_err_fails", "n_newton_fails", "q_last", "steps_at_order"):
        assert ast[k] == ast_ref[k], k
    assert ast["t"] == T1
    err = rel_err(y, y_ref)
    print("adaptive parity", err)
    assert err <= 1e-9


def test_adaptive_fp32_form(cuda):
    c64 = Case(M.make_workload("sod16", scale=8))
    c32 = Case(M.make_workload("sod16", scale=8), flags=FLUX_FP32 | ILU_FP32 | ILU_COLOR)
    y64, _, a64 = gpu_adaptive(c64, 1e-6)
    y32, _, a32 = gpu_adaptive(c32, 1e-6)
    print("fp64", a64, "\nfp32", a32)
    assert a32["t"] == T1
    assert abs(a32["n_accepted"] - a64["n_accepted"]) <= 0.2 * a64["n_accepted"]
    assert rel_err(y32, y64) <= 1e-5


def test_adaptive_cvode_setup_policy_matches_oracle(cuda):
    """The adaptive drivers with CVODE's preconditioner set-up policy (MSBP 20, DGMAX 0.3):
    the same accepted / rejected history and pset count as the oracle's, fewer psets than
    accepted steps, state within 1e-9."""
    import torch
    c = Case(M.make_workload("sod16", scale=8))
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    y_ref = c.y0.copy()
    rc, st_ref, ast_ref = O.bdf_adaptive(c.N, rhs, pset, psol, c.oracle.h, y_ref, 0.0, T1,
                                         O.bdf_defaults(newton_rtol=1e-10, msbp=20),
                                         O.adapt_defaults(rtol=1e-6, atol=1e-10, h0=1e-4))
    assert rc == 0
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    c.gpu.to_internal(yr, y)
    rc, st, ast = c.gpu.bdf_adaptive(y, 0.0, T1, c.gpu.bdf_defaults(newton_rtol=1e-10, msbp=20),
                                     c.gpu.adapt_defaults(rtol=1e-6, atol=1e-10, h0=1e-4))
    assert rc == 0, (st, ast)
    c.gpu.to_reference(y, yr)
    torch.cuda.synchronize()
    print("gpu", st, ast, "\noracle", st_ref, ast_ref)
    for k in ("n_accepted", "n_err_fails", "n_newton_fails", "q_last", "steps_at_order"):
        assert ast[k] == ast_ref[k], k
    assert st["n_pset"] == st_ref["n_pset"] < ast["n_accepted"]
    assert rel_err(yr.cpu().numpy(), y_ref) <= 1e-9
