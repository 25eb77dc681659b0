"""Learned variable preconditioner: the graph network of libfosgpu (fos_gnn_*) and its
training on (residual, ILU-GMRES Newton correction) pairs generated by the plain solver.

All compute runs in libfosgpu.so; this module only orchestrates (data generation through
the C ABI, the optimiser loop, checkpoints)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import NamedTuple

import numpy as np

from . import _lib
from ._lib import check


class GNN:
    """Handle of a fos_gnn (BF16 weights, FP32 master copy on the device)."""

    def __init__(self, seed: int = 0):
        h = C.c_void_p()
        check(_lib.lib().fos_gnn_create(C.byref(h), seed), "fos_gnn_create")
        self._h = h
        self.nparam = _lib.lib().fos_gnn_num_params()

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().fos_gnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        w = np.zeros(self.nparam, np.float32)
        check(_lib.lib().fos_gnn_get_params(self._h, w.ctypes.data_as(C.POINTER(C.c_float))), "get_params")
        return w

    def set_params(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        check(_lib.lib().fos_gnn_set_params(self._h, w.ctypes.data_as(C.POINTER(C.c_float))), "set_params")

    def grad(self) -> np.ndarray:
        g = np.zeros(self.nparam, np.float32)
        check(_lib.lib().fos_gnn_get_grad(self._h, g.ctypes.data_as(C.POINTER(C.c_float))), "get_grad")
        return g

    def zero_grad(self):
        check(_lib.lib().fos_gnn_zero_grad(self._h), "zero_grad")

    def apply_dev(self, ctx, y_dev, v_dev, z_dev, gamma: float):
        check(_lib.lib().fos_gnn_apply_dev(self._h, ctx.handle, y_dev.data_ptr(), v_dev.data_ptr(),
                                           gamma, z_dev.data_ptr()), "gnn_apply")

    def loss_grad_dev(self, ctx, y_dev, v_dev, t_dev, gamma: float) -> float:
        loss = C.c_double(0.0)
        check(_lib.lib().fos_gnn_loss_grad_dev(self._h, ctx.handle, y_dev.data_ptr(), v_dev.data_ptr(),
                                               t_dev.data_ptr(), gamma, C.byref(loss)), "gnn_loss_grad")
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, grad_scale=1.0):
        check(_lib.lib().fos_gnn_adam_step(self._h, lr, beta1, beta2, eps, grad_scale), "adam")

    def save(self, path):
        np.save(Path(path), self.params())

    def load(self, path):
        self.set_params(np.load(Path(path)))


# ---------------------------------------------------------------------- training data
class Sample(NamedTuple):
    """One training sample in the context's internal cell order: state y, right-hand side
    b of J_G x = b, target t = the solution, gamma, and u = ILU(0) b at (y, gamma) -- the
    network's input in the ILU-then-correction form (precond 4/5)."""
    ctx: object
    y: object
    b: object
    t: object
    gamma: float
    u: object


def random_state(x: np.ndarray, rng, gamm: float = 1.4):
    """Piecewise-constant states in the spirit of the Sod tube: 1-3 random planes split the
    domain into regions with random density, pressure and velocity, plus a weak smooth
    perturbation; returns conserved variables for points x (n, 3)."""
    from .mesh import conserved
    n = x.shape[0]
    label = np.zeros(n, np.int64)
    for k in range(rng.integers(1, 4)):
        nrm = rng.normal(size=3)
        nrm /= np.linalg.norm(nrm)
        off = nrm @ rng.uniform(0.2, 0.8, 3)
        label = 2 * label + (x @ nrm > off)
    nreg = int(label.max()) + 1
    rho_r = rng.uniform(0.2, 1.5, nreg)
    p_r = rng.uniform(0.2, 1.5, nreg)
    u_r = rng.uniform(-0.2, 0.2, (nreg, 3))
    ph = rng.uniform(0, 2 * np.pi, 3)
    wave = 0.02 * np.sin(2 * np.pi * (x[:, 0] + ph[0])) * np.sin(2 * np.pi * (x[:, 1] + ph[1]))
    rho = rho_r[label] * (1.0 + wave)
    p = p_r[label]
    u, v, w = (u_r[label, k] for k in range(3))
    return conserved(rho, u, v, w, p, gamm)


def smooth_field(x: np.ndarray, rng, nwaves: int = 3) -> np.ndarray:
    """Five unit-RMS fields (SoA), each a sum of nwaves random plane sine waves of wave
    numbers 1-4 -- the low-frequency half of the operator samples' directions."""
    out = np.zeros((5, x.shape[0]))
    for q in range(5):
        for _ in range(nwaves):
            kv = rng.integers(1, 5, size=3) * rng.choice([-1, 1], size=3)
            out[q] += np.sin(2.0 * np.pi * (x @ kv) + rng.uniform(0, 2 * np.pi))
        out[q] /= np.sqrt((out[q] ** 2).mean()) + 1e-30
    return out.reshape(-1)


def generate_pairs(n_meshes: int, seed: int = 0, sizes=(12, 20), newton_iters: int = 2,
                   bdf_steps: int = 2, cfl=(0.03, 0.3), lin_rtol: float = 1e-6, flags: int = 0,
                   states=("random", "sine"), n_random: int = 3, lean: bool = False,
                   keep_u: bool = True):
    """(y, v, t, gamma) training samples on the device, from the plain solver.

    At each sampled state of a BDF1 run (seeded meshes, random piecewise or sinusoidal
    states, CFL drawn from `cfl`):
      * Newton samples: v = -G(y_k) for the first Newton iterates and t = the ILU(0)-GMRES
        solution of J_G t = v (the correction the plain solver computes);
      * operator samples: t = w for random w (white noise mixed with a smooth field) and
        v = J_G w from the fused finite-difference Jv kernel -- exact pairs that cover the
        directions FGMRES feeds the preconditioner besides the first residual.
    lean: once a mesh's samples are made, they move to a fresh context on the same grid
    (same internal order) that has never factored anything, and the generating context
    with its Jacobian and ILU(0) storage (~2 KB per cell) is freed -- what lets hundreds
    of meshes' samples stay on the device.  keep_u=False drops u (only the
    ILU-then-correction form trains on it).
    Returns a list of Sample."""
    import torch
    from . import mesh as M
    from .euler import FOEuler, PolyFvGrid
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    out = []
    for k in range(n_meshes):
        first = len(out)
        n = int(rng.integers(sizes[0], sizes[1] + 1))
        m = M.box_mesh(n, n, n, jitter=0.1, seed=seed * 1000 + k)
        xc = m.centroids()
        kind = states[k % len(states)]
        st = random_state(xc, rng) if kind == "random" else M.sine_state(xc, seed * 1000 + k)
        grid = PolyFvGrid.from_mesh(m)
        ctx = FOEuler(grid, flags=flags)
        y_ref = torch.from_numpy(M.soa(st, grid.nC)).cuda()
        y = torch.empty_like(y_ref)
        ctx.to_internal(y_ref, y)
        h = 1.0 / n
        smooth_ref = torch.from_numpy(smooth_field(xc[:grid.nC], rng)).cuda()
        smooth = torch.empty_like(smooth_ref)
        ctx.to_internal(smooth_ref, smooth)
        for s in range(bdf_steps):
            dt = float(rng.uniform(*cfl)) * h / 1.5
            yn = y.clone()
            yk = y.clone()
            f = torch.empty_like(yk)
            for it in range(newton_iters):
                ctx.rhs_dev(0.0, yk, f)
                b = dt * f - (yk - yn)  # -G(y_k) for BDF1
                x = torch.empty_like(b)
                opts = ctx.bdf_defaults(precond=1, lin_rtol=lin_rtol, max_restarts=8)
                ctx.linear_solve(yk, f, dt, b, x, opts)  # leaves ILU(0) factored at (yk, dt)
                u = None
                if keep_u:
                    u = torch.empty_like(b)
                    ctx.psol_dev(b, u)
                out.append(Sample(ctx, yk.clone(), b, x, dt, u))
                if it + 1 < newton_iters:
                    yk = yk + x
            ctx.rhs_dev(0.0, yn, f)
            ctx.pset_dev(0.0, yn, 0, dt)
            ynorm = float(torch.linalg.norm(yn))
            scale = yn.view(5, -1).abs().mean(dim=1, keepdim=True)
            for r in range(n_random):
                a = float(rng.uniform(0.0, 1.0))
                noise = torch.randn(yn.shape, generator=gen, device="cuda", dtype=yn.dtype)
                w = (a * noise.view(5, -1) + (1 - a) * smooth.view(5, -1)) * scale
                w = w.reshape(-1).contiguous()
                v = torch.empty_like(w)
                ctx.jv_dev(0.0, yn, f, w, v, 1.0, -dt, ynorm)
                u = None
                if keep_u:
                    u = torch.empty_like(v)
                    ctx.psol_dev(v, u)
                out.append(Sample(ctx, yn.clone(), v, w, dt, u))
            rc, _ = ctx.bdf_run(y, ctx.bdf_defaults(order=1, dt=dt, nsteps=1))
            if rc != 0:
                break
        if lean:
            light = FOEuler(grid, flags=flags)
            out[first:] = [sm._replace(ctx=light) for sm in out[first:]]
            ctx.close()
            del ctx
            torch.cuda.empty_cache()
    # keep finite samples only (a state the solver could not advance is dropped)
    return [sm for sm in out
            if all(bool(torch.isfinite(x).all()) for x in (sm.y, sm.b, sm.t, sm.u) if x is not None)]


def train(gnn: GNN, pairs, epochs: int = 20, lr: float = 2e-3, seed: int = 0, log=None,
          after_ilu: bool = False):
    """Adam over the samples (one sample = one mesh-sized batch); returns the loss history.
    after_ilu trains the correction form (input u = ILU(0) b, precond 4/5) instead of the
    stand-alone form (input b, precond 2/3)."""
    rng = np.random.default_rng(seed)
    hist = []
    n = len(pairs)
    for ep in range(epochs):
        order = rng.permutation(n)
        tot = 0.0
        lr_ep = lr * (0.5 * (1 + np.cos(np.pi * ep / max(epochs, 1))))  # cosine decay
        used = 0
        for i in order:
            sm = pairs[i]
            gnn.zero_grad()
            loss = gnn.loss_grad_dev(sm.ctx, sm.y, sm.u if after_ilu else sm.b, sm.t, sm.gamma)
            if not np.isfinite(loss):  # no step from a non-finite loss or gradient
                continue
            tot += loss
            used += 1
            gnn.adam_step(lr=max(lr_ep, 1e-5))
        hist.append(tot / max(used, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4e}")
    return hist


def krylov_iterations(pairs_ctx, precond: int, lin_rtol: float = 1e-6, maxl: int = 30,
                      timing: bool = False):
    """Krylov iterations (and fallbacks) of the linear solves of the given pairs; with
    timing, also the summed CUDA-event time of the solves in ms (the ILU(0) factorisation,
    where the solve makes one, included)."""
    import torch
    its, fb, ms = [], 0, 0.0
    for (c, y, b, t, gam, _u) in pairs_ctx:
        f = torch.empty_like(y)
        c.rhs_dev(0.0, y, f)
        x = torch.empty_like(b)
        opts = c.bdf_defaults(precond=precond, lin_rtol=lin_rtol, maxl=maxl, max_restarts=8)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        rc, st = c.linear_solve(y, f, gam, b, x, opts)
        e1.record()
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
        its.append(st["n_lin_iters"])
        fb += st["n_fallback"]
    return (its, fb, ms) if timing else (its, fb)


DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "weights" / "gnn_sine.npy"


def _main(argv=None):
    """python -m fosolvers_gb300.learned train --out W.npy [--meshes M --sizes A B ...]

    Generates samples with the plain solver on seeded meshes, trains the network on the GPU
    and prints held-out Krylov iterations (none / learned / ILU(0)) at two tolerances."""
    import argparse
    import time
    ap = argparse.ArgumentParser(prog="python -m fosolvers_gb300.learned")
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--out", default=str(DEFAULT_WEIGHTS))
    ap.add_argument("--meshes", type=int, default=24)
    ap.add_argument("--sizes", type=int, nargs=2, default=(24, 40))
    ap.add_argument("--test-meshes", type=int, default=2)
    ap.add_argument("--test-size", type=int, default=48)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--cfl", type=float, nargs=2, default=(0.03, 0.3))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--flags", type=int, default=0)
    ap.add_argument("--newton-iters", type=int, default=2)
    ap.add_argument("--bdf-steps", type=int, default=2)
    ap.add_argument("--n-random", type=int, default=3)
    ap.add_argument("--lean", action="store_true",
                    help="free each generating context's preconditioner storage (many meshes)")
    ap.add_argument("--tols", type=float, nargs="+", default=(1e-3, 1e-6))
    ap.add_argument("--compare", default=None,
                    help="also evaluate these weights on the same held-out solves")
    a = ap.parse_args(argv)
    t0 = time.time()
    tr = generate_pairs(a.meshes, seed=a.seed, sizes=tuple(a.sizes), cfl=tuple(a.cfl), flags=a.flags,
                        newton_iters=a.newton_iters, bdf_steps=a.bdf_steps, n_random=a.n_random,
                        lean=a.lean, keep_u=not a.lean)
    te = generate_pairs(a.test_meshes, seed=a.seed + 1000, sizes=(a.test_size, a.test_size),
                        cfl=tuple(a.cfl), flags=a.flags)
    print(f"samples: {len(tr)} training, {len(te)} held out ({time.time() - t0:.1f} s)", flush=True)
    g = GNN(seed=a.seed)
    t0 = time.time()
    hist = train(g, tr, epochs=a.epochs, lr=a.lr, log=lambda s: print(s, flush=True))
    print(f"trained in {time.time() - t0:.1f} s: loss {hist[0]:.4e} -> {hist[-1]:.4e}", flush=True)
    Path(a.out).parent.mkdir(parents=True, exist_ok=True)
    g.save(a.out)
    print("saved", a.out, flush=True)
    del tr
    nets = [("learned", g)]
    if a.compare:
        g0 = GNN(seed=0)
        g0.load(a.compare)
        nets.append(("compared", g0))
    for tol in a.tols:
        r = {}
        for name, pc in (("none", 0), ("ILU(0)", 1)):
            its, fb, ms = krylov_iterations(te, pc, lin_rtol=tol, timing=True)
            r[name] = {"iterations": sum(its), "ms": round(ms, 1), "fallbacks": fb}
        for label, net in nets:
            for s in te:
                s.ctx.attach_gnn(net)
            for name, pc in ((label, 3), (label + "+fallback", 2)):
                its, fb, ms = krylov_iterations(te, pc, lin_rtol=tol, timing=True)
                r[name] = {"iterations": sum(its), "ms": round(ms, 1), "fallbacks": fb}
        print(f"held-out ({len(te)} solves at {a.test_size}^3 x 6) at {tol:g}: {r}", flush=True)


if __name__ == "__main__":
    _main()
