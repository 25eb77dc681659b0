"""Regenerate the oracle's golden vectors under tests/golden/ (CPU only; the oracle is the
C restatement of the reference arithmetic in oracle/).  All in the reference's natural
cell order (ilu0 in the natural order), so a GPU context created with FOS_ORDER_NATURAL
reproduces them without any order matching.

oracle_sod16.npz   config 1 (16^3 x 6 = 24,576 tets, Sod, walls): the residual f at a
                   perturbed state (perturbed(y0, seed 11)), the finite-difference Jv of
                   that state along a seeded normal v (seed 0, s = sqrt(eps)(1+|y|)/|v|),
                   z = P^-1 r from pset (gamma 5e-3) + psol on that state (r: seed 8), and
                   the state after the configuration's 20 BDF1 steps (dt 1e-3, Newton 1e-8,
                   GMRES(30) + ILU(0)).
oracle_sine12.npz  config 2's state on a 12^3 x 6 mesh (seed 3): residual and Jv as above,
                   with the perturbed state y itself (the sinusoidal state comes from numpy's
                   sin, whose last bit differs between x86-64 and AArch64 builds, and the
                   difference quotient magnifies that by 1/s ~ 1e8).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE.parent))

from fosolvers_gb300 import mesh as M  # noqa: E402
from helpers import Case, perturbed  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

EPS = float(np.sqrt(np.finfo(float).eps))
GAMMA = 5e-3


def residual_and_jv(c: Case):
    y = perturbed(c.y0, c.nC, 11)
    f = c.oracle_rhs(y)
    v = np.random.default_rng(0).normal(size=y.size)
    s = EPS * (1 + np.linalg.norm(y)) / np.linalg.norm(v)
    jv = (c.oracle_rhs(y + s * v) - f) / s
    return y, f, v, jv


def sod16():
    wl = M.make_workload("sod16")
    c = Case(wl)
    y, f, v, jv = residual_and_jv(c)
    assert c.oracle.pset(0.0, y, None, 0, GAMMA) == (0, 1)
    r = np.random.default_rng(8).normal(size=c.N)
    z = np.zeros_like(r)
    c.oracle.psol(0.0, None, None, r, z, GAMMA)
    rhs, pset, psol = c.oracle.callbacks()
    yb = c.y0.copy()
    rc, st = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, yb,
                       O.bdf_defaults(order=1, dt=wl.dt, nsteps=wl.nsteps, use_prec=1))
    assert rc == 0, st
    return dict(f=f, jv=jv, z=z, y20=yb, n_newton=st["n_newton"], n_lin_iters=st["n_lin_iters"])


def sine12():
    c = Case(M.make_workload("sine96", scale=12, seed=3))
    y, f, _, jv = residual_and_jv(c)
    return dict(f=f, jv=jv, y=y)


def main():
    np.savez_compressed(HERE / "oracle_sod16.npz", **sod16())
    np.savez_compressed(HERE / "oracle_sine12.npz", **sine12())
    for n in ("oracle_sod16.npz", "oracle_sine12.npz"):
        print(n, (HERE / n).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
