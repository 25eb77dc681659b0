"""Parity against the committed golden vectors (tests/golden/make_oracle_golden.py): the
oracle must reproduce them (CPU, a regression pin of the oracle itself), and the GPU FP64
path in the reference's natural cell order (FOS_ORDER_NATURAL, so ILU(0) eliminates in the
same order as the oracle's ilu0) must match them without the oracle running: residual
within 1e-11, finite-difference Jv within 1e-6, ILU(0) apply within 1e-10, the state after
config 1's 20 BDF1 steps within 1e-10 with the same Newton and Krylov counts."""
from pathlib import Path

import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import ORDER_NATURAL
from helpers import Case, perturbed, rel_err
from oracle import pyoracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
EPS = float(np.sqrt(np.finfo(float).eps))
GAMMA = 5e-3


def load(name):
    return dict(np.load(GOLDEN / name))


def inputs(c: Case, g=None):
    """The perturbed state (the fixture's own copy where it stores one), v and r."""
    y = g["y"] if g is not None and "y" in g else perturbed(c.y0, c.nC, 11)
    v = np.random.default_rng(0).normal(size=y.size)
    r = np.random.default_rng(8).normal(size=y.size)
    return y, v, r


# ---------------------------------------------------------------- the oracle (CPU)
@pytest.mark.parametrize("name,wl", [("oracle_sod16.npz", lambda: M.make_workload("sod16")),
                                     ("oracle_sine12.npz",
                                      lambda: M.make_workload("sine96", scale=12, seed=3))])
def test_oracle_reproduces_residual_and_jv(name, wl):
    g = load(name)
    c = Case(wl())
    y, v, _ = inputs(c, g)
    f = c.oracle_rhs(y)
    assert rel_err(f, g["f"]) <= 1e-14
    s = EPS * (1 + np.linalg.norm(y)) / np.linalg.norm(v)
    assert rel_err((c.oracle_rhs(y + s * v) - f) / s, g["jv"]) <= 1e-12


def test_oracle_reproduces_ilu_apply_and_bdf():
    g = load("oracle_sod16.npz")
    wl = M.make_workload("sod16")
    c = Case(wl)
    y, _, r = inputs(c)
    assert c.oracle.pset(0.0, y, None, 0, GAMMA) == (0, 1)
    z = np.zeros_like(r)
    c.oracle.psol(0.0, None, None, r, z, GAMMA)
    assert rel_err(z, g["z"]) <= 1e-14
    rhs, pset, psol = c.oracle.callbacks()
    yb = c.y0.copy()
    rc, st = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, yb,
                       O.bdf_defaults(order=1, dt=wl.dt, nsteps=wl.nsteps, use_prec=1))
    assert rc == 0
    assert st["n_newton"] == int(g["n_newton"]) and st["n_lin_iters"] == int(g["n_lin_iters"])
    assert rel_err(yb, g["y20"]) <= 1e-13


# ---------------------------------------------------------------- the GPU against the fixtures
@pytest.mark.gpu
@pytest.mark.parametrize("name,wl", [("oracle_sod16.npz", lambda: M.make_workload("sod16")),
                                     ("oracle_sine12.npz",
                                      lambda: M.make_workload("sine96", scale=12, seed=3))])
def test_gpu_residual_and_jv_match_golden(cuda, name, wl):
    import torch
    g = load(name)
    c = Case(wl(), flags=ORDER_NATURAL)
    y, v, _ = inputs(c, g)
    f = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, f) == 0
    assert rel_err(f, g["f"]) <= 1e-11
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    yi, fi, vi, out, tmp = (torch.empty(y.size, dtype=torch.float64, device="cuda") for _ in range(5))
    c.gpu.to_internal(dev(y), yi)
    c.gpu.rhs_dev(0.0, yi, fi)
    c.gpu.to_internal(dev(v), vi)
    c.gpu.jv_dev(0.0, yi, fi, vi, out, 0.0, 1.0, float(np.linalg.norm(y)), EPS)
    c.gpu.to_reference(out, tmp)
    torch.cuda.synchronize()
    assert rel_err(tmp.cpu().numpy(), g["jv"]) <= 1e-6


@pytest.mark.gpu
def test_gpu_ilu_apply_and_bdf_match_golden(cuda):
    import torch
    g = load("oracle_sod16.npz")
    wl = M.make_workload("sod16")
    c = Case(wl, flags=ORDER_NATURAL)
    y, _, r = inputs(c)
    rc, jcur = c.gpu.pset(0.0, y, None, 0, GAMMA)
    assert rc == 0 and jcur == 1
    z = np.zeros_like(r)
    assert c.gpu.psol(0.0, y, None, r, z, GAMMA) == 0
    assert rel_err(z, g["z"]) <= 1e-10
    yr = torch.from_numpy(c.y0).cuda()
    yi = torch.empty_like(yr)
    c.gpu.to_internal(yr, yi)
    rc, st = c.gpu.bdf_run(yi, c.gpu.bdf_defaults(order=1, dt=wl.dt, nsteps=wl.nsteps, precond=1))
    assert rc == 0, st
    c.gpu.to_reference(yi, yr)
    torch.cuda.synchronize()
    assert st["n_newton"] == int(g["n_newton"]) and st["n_lin_iters"] == int(g["n_lin_iters"])
    assert rel_err(yr.cpu().numpy(), g["y20"]) <= 1e-10
