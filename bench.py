#!/usr/bin/env python3
"""bench.py -- BDF steps/s of foeuler's implicit inner loop on one GB300.

Workload (default, 5,308,416 tets): unit cube of 96^3 hexahedra x 6 Kuhn tetrahedra
with seeded +-0.1h interior-node jitter, sinusoidal density/velocity state, p = 1,
slip walls, BDF2 at dt = 5e-4, Newton tolerance 1e-8, forcing 1e-3.  Default arm (the
metric's configuration): FP32 Roe flux with FP64 accumulation, FP32 block ILU(0), and the
trained network as the variable preconditioner of flexible GMRES(30) with the automatic
ILU(0) fallback.  The same line carries the same steps with ILU(0) alone in FP32 and the
plain FP64 ILU(0)-GMRES(30) path on the same mesh and state (the target's denominator).
A "step" is one BDF step of the whole mesh (residuals, Jacobian assembly, ILU(0)
factor and apply, Krylov iterations) with the state resident in HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  `value` is device-resident throughput (CUDA events on the
library's stream); `e2e` is the same metric through the host-buffer C-ABI entry
point fos_bdf_run_host with the state copied host->device and back every step;
`roofline` covers the operation with the largest share of the step, timed with CUDA
events over repeated launches; `cpu_baseline` times the CPU oracle (a C restatement
of the reference arithmetic) on this machine's host cores on a bounded sample.
N > 1 runs independent replicas (the path is not partitioned across GPUs here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "BDF steps/s at 5.3M tets, 1 GB300: FP32+learned FGMRES vs FP64 ILU, tol 1e-8"
UNIT = "BDF steps/s"
FULL_CELLS = 96 ** 3 * 6
# network apply, bytes per cell moved by the layer-by-layer kernels: scales (y, v, 1/V,
# face geometry: 120), input layer (y, v, 1/V in, h0 out: 216), 3 message-passing layers
# (h in and out in BF16, ELL row, face pair and geometry: 368 each), output (h3, v, z: 208)
GNN_BYTES_PER_CELL = 120 + 216 + 3 * 368 + 208
# DRAM traffic per cell of each operation in the FP32 form, from one ncu capture of the
# same workload at 64^3 x 6 tets (dram__bytes_read.sum + dram__bytes_write.sum summed over
# the operation's kernels, L2 flushed before every kernel, so an upper bound); traffic
# grows with the cell count, so the full-size figure is this times nC.  Summary and
# command: profiles/traffic_sine64_fp32.md
TRAFFIC_FP32_BYTES_PER_CELL = {"residual": 235.0, "jv": 403.1,
                               "ilu_apply": 800.0, "gnn_apply": 1162.1}
# FP64-pipe lane-instructions per cell of the FP32 form's residual (k_prim_hl<0> +
# k_cell32 residual epilogue) and Jv (k_prim_hl<1> + k_cell32 Jv epilogue), counted by ncu
# (sm__inst_executed_pipe_fp64 x 32 / cells; profiles/fp64_pipe_sine64.md).  GB300 retires
# 2 FP64 lanes per clock per SM, so these put a second roof under the operations, beside HBM.
FP64_INSTR_PER_CELL_FP32 = {"residual": 20.0, "jv": 30.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="sine96")
    ap.add_argument("--scale", type=int, default=None, help="hexes along x (small cases)")
    ap.add_argument("--mode", choices=["fp64", "fp32", "fp32h", "fp32ilu"], default="fp32",
                    help="fp64: FP64 flux + FP64 ILU(0); fp32: FP32 flux + FP32 ILU(0); "
                         "fp32h: FP32 flux with FP64 faces where the density or pressure jump "
                         "exceeds 5%% and on boundaries (shocked flows) + FP32 ILU(0); "
                         "fp32ilu: FP64 flux + FP32 ILU(0)")
    ap.add_argument("--precond", choices=["ilu", "none", "learned"], default="learned",
                    help="learned: the trained network in FGMRES with ILU(0) fallback")
    ap.add_argument("--weights", default=None, help="network weights (.npy) for --precond learned")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the FP64 ILU(0) reference arm on the same mesh")
    ap.add_argument("--ilu-order", choices=["rcm", "color"], default="color",
                    help="ILU(0) elimination order: internal RCM order or greedy colouring")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-oracle baseline")
    ap.add_argument("--no-ops", action="store_true", help="skip the per-operation timing")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--op-reps", type=int, default=5)
    ap.add_argument("--msbp", type=int, default=20,
                    help="preconditioner set-up policy of every arm: m > 1 = CVODE's, which drives "
                         "the reference's callbacks (cvLsSetup: at most m steps between set-ups, "
                         "or on a 30%% gamma change or a Newton failure; CVODE's MSBP is 20); "
                         "1 = pset at every BDF step")
    ap.add_argument("--tight-rtol", type=float, default=1e-9,
                    help="Newton tolerance of the untimed tightened-tolerance comparison of the "
                         "arm with the FP64 path (0: skip)")
    ap.add_argument("--no-cvode", action="store_true",
                    help="skip the arms under the other set-up policy (alt_setup_policy: every "
                         "step when --msbp > 1, CVODE's MSBP 20 when --msbp 1)")
    ap.add_argument("--ilut", action="store_true",
                    help="the ILUT preconditioner arm (FP64 flux, ILUT(lfil, droptol) on P in the "
                         "RCM order) against block ILU(0) on the same mesh, with the oracle's "
                         "SPARSKIT ilut on the same P as the CPU baseline; its own JSON line")
    ap.add_argument("--lfil", type=int, default=50, help="ILUT fill (fopbc: 50)")
    ap.add_argument("--droptol", type=float, default=1e-6, help="ILUT drop tolerance (fopbc: 1e-6)")
    ap.add_argument("--profile-ops", action="store_true",
                    help="profiling target: one warm-up round, then one residual, Jv, pset, "
                         "ILU(0) apply and network apply on the workload; no JSON line")
    return ap.parse_args()


def profile_ops(args):
    """Kernel sequence for ncu: a warm-up round of every operation, a synchronize, then
    exactly one rhs_dev, jv_dev, pset_dev, psol_dev and network apply, in that order."""
    import torch
    from __graft_entry__ import build
    build()
    from fosolvers_gb300 import mesh as M
    from fosolvers_gb300.euler import PolyFvGrid
    from fosolvers_gb300.learned import GNN, DEFAULT_WEIGHTS
    wl = M.make_workload(args.workload, scale=args.scale)
    grid = PolyFvGrid.from_mesh(wl.mesh)
    ctx = make_ctx(grid, M.ibc_for(wl.mesh, wl.bc_gid), wl, args.mode, args.ilu_order,
                   torch.cuda.current_stream())
    gnn = GNN(seed=0)
    gnn.load(args.weights or DEFAULT_WEIGHTS)
    y0 = torch.from_numpy(M.soa(wl.elem_state, grid.nC)).cuda()
    y = torch.empty_like(y0)
    ctx.to_internal(y0, y)
    f, out = torch.empty_like(y), torch.empty_like(y)
    v = torch.randn(y.shape, dtype=y.dtype, device=y.device,
                    generator=torch.Generator(device=y.device).manual_seed(0))
    ynorm = float(torch.linalg.norm(y))
    gamma = wl.dt * (2.0 / 3.0 if wl.order == 2 else 1.0)
    for _ in range(2):
        ctx.rhs_dev(0.0, y, f)
        ctx.jv_dev(0.0, y, f, v, out, 1.0, -gamma, ynorm)
        ctx.pset_dev(0.0, y, 0, gamma)
        ctx.psol_dev(v, out)
        gnn.apply_dev(ctx, y, v, out, gamma)
        torch.cuda.synchronize()
    print(json.dumps({"profile_ops": args.workload, "cells": grid.nC, "faces": grid.nP,
                      "mode": args.mode, "finite": bool(torch.isfinite(out).all())}))
    ctx.close()


def run_ilut(args):
    """ILUT arm: BDF steps/s of the FP64 flux with GMRES(30) + ILUT(lfil, droptol) and with
    block ILU(0), both in the RCM order; the ILUT factorisation (P formed and factored,
    Jacobian reused) and one psol timed with CUDA events; the oracle's ilut + lusol on the
    same state as the CPU baseline (one core, SPARSKIT is serial)."""
    import torch
    from __graft_entry__ import build
    build()
    from fosolvers_gb300 import mesh as M
    from fosolvers_gb300.euler import FOEuler, PolyFvGrid, PREC_ILUT
    from oracle import pyoracle as O
    scale = args.scale or 24
    wl = M.make_workload(args.workload, scale=scale)
    grid = PolyFvGrid.from_mesh(wl.mesh)
    ibc = M.ibc_for(wl.mesh, wl.bc_gid)
    nC = grid.nC
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    y0_ref = torch.from_numpy(M.soa(wl.elem_state, nC)).to(dev)
    gamma = wl.dt * (2.0 / 3.0 if wl.order == 2 else 1.0)
    out = {}
    for name, flags in (("ilut", PREC_ILUT), ("ilu0", 0)):
        ctx = FOEuler(grid, ibc, wl.bc_type, wl.bc_param, wl.gamm, wl.r, flags=flags,
                      stream=stream)
        if flags:
            ctx.set_ilut(args.lfil, args.droptol)
        y0 = torch.empty_like(y0_ref)
        ctx.to_internal(y0_ref, y0)
        mk = lambda n: ctx.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=n, precond=1,
                                        msbp=args.msbp)
        ms, st, launches, _, _ = timed_bdf(ctx, y0, mk, args, dev, stream, None)
        rec = {"steps_per_s": args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
               "n_newton": st["n_newton"], "n_lin_iters": st["n_lin_iters"],
               "gpu_launches": launches}
        ctx.pset_dev(0.0, y0, 0, gamma)
        r = torch.randn(y0.shape, dtype=y0.dtype, device=dev,
                        generator=torch.Generator(device=dev).manual_seed(0))
        z = torch.empty_like(r)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        torch.cuda.synchronize(dev)
        ev[0].record(stream)
        for _ in range(3):
            ctx.pset_dev(0.0, y0, 1, gamma)
        ev[1].record(stream)
        for _ in range(10):
            ctx.psol_dev(r, z)
        ev[2].record(stream)
        torch.cuda.synchronize(dev)
        rec["factor_ms"] = ev[0].elapsed_time(ev[1]) / 3
        rec["psol_ms"] = ev[1].elapsed_time(ev[2]) / 10
        if flags:
            order = ctx.ilu_order()
        out[name] = rec
        ctx.close()
    # CPU baseline: the oracle's ilut + lusol on P of the same state, the GPU's cell order
    e = O.Euler(grid.__dict__, ibc, wl.bc_type, wl.bc_param, wl.gamm, wl.r, wl.elem_state)
    e.set_ilu_order(order)
    e.set_ilut(args.lfil, args.droptol)
    y = M.soa(wl.elem_state, nC)
    e.pset(0.0, y, None, 0, gamma)
    t0 = time.perf_counter()
    rc, _ = e.pset(0.0, y, None, 1, gamma)
    t_fact = time.perf_counter() - t0
    r = np.random.default_rng(0).normal(size=5 * nC)
    z = np.zeros_like(r)
    t0 = time.perf_counter()
    e.psol(0.0, None, None, r, z, gamma)
    t_sol = time.perf_counter() - t0
    alu, jlu, ju = e.ilut_factors()
    stored = int(jlu[5 * nC]) - 1 - (5 * nC + 1)
    e.close()
    g = out["ilut"]
    line = {
        "metric": f"ILUT({args.lfil}, {args.droptol:g}) factorisation of P = I - gamma J/v, "
                  "1 GB300 vs SPARSKIT ilut restated (1 core)",
        "value": g["factor_ms"], "unit": "ms", "higher_is_better": False, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"{args.workload} at {scale}^3 x 6 = {nC} tets, "
                               f"{5 * nC} unknowns", "lfil": args.lfil, "droptol": args.droptol,
                   "order": "RCM (internal)", "stored_lu_entries": stored,
                   "stored_per_row": round(stored / (5 * nC), 2)},
        "ilut": g, "ilu0": out["ilu0"],
        "cpu_baseline": {"factor_ms": 1e3 * t_fact, "psol_ms": 1e3 * t_sol, "cores": 1,
                         "kind": "port", "rc": rc,
                         "sample": "the oracle's o_ilut (ITSOL/ilut.f:38-382 restated) on the "
                                   "same P, and o_lusol, one call each"},
        "speedup_factor": 1e3 * t_fact / g["factor_ms"], "speedup_psol": 1e3 * t_sol / g["psol_ms"],
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ clocks
class Clocks:
    """nvidia-smi sampler during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index: int):
        self.dev = dev_index
        self.proc = None
        self.path = Path(f"/tmp/fos_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.dev)], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ distributed
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def allmax(pg, x: float, device=None) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU oracle baseline
# The oracle is the reference arithmetic restated in C (the Fortran reference cannot be built
# here: no Fortran compiler), timed as the "tuned" build: the host's instruction set, like the
# reference's own -march=native build, and OpenMP with the reference's structure -- the
# residual's face loop in parallel with atomic scatter (Euler.f90:71-155), the Jacobian
# assembly, SPARSKIT ilu0/lusol and the Krylov driver serial.
def _oracle_context(wl, grid: dict, threads: int):
    from fosolvers_gb300 import mesh as M
    from oracle import pyoracle as O
    O.set_default("tuned")
    ibc = M.ibc_for(wl.mesh, wl.bc_gid)
    return O.Euler(grid, ibc, wl.bc_type, wl.bc_param, wl.gamm, wl.r, wl.elem_state,
                   threads=threads)


def cpu_oracle_fullsize(wl, grid: dict, nsteps: int = 1, msbp: int = 1) -> dict:
    """cpu_baseline of the GPU arm: the oracle on the same workload at its full size -- the
    residual, Jv and ILU(0) apply rates (the ILU(0) factored once in the reference's natural
    order) and `nsteps` whole BDF steps from the initial state (about 15-25 s of CPU work at
    96^3 x 6 on a 16-core host)."""
    from fosolvers_gb300 import mesh as M
    from oracle import pyoracle as O
    threads = os.cpu_count() or 1
    t_setup = time.perf_counter()
    e = _oracle_context(wl, grid, threads)
    nC = grid["nC"]
    y = M.soa(wl.elem_state, nC)
    f = np.zeros_like(y)
    gamma = wl.dt * (2.0 / 3.0 if wl.order == 2 else 1.0)
    e.rhs(0.0, y, f)  # first touch of the work arrays
    setup_s = time.perf_counter() - t_setup

    def timed(fn, reps):
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps

    t_rhs = timed(lambda: e.rhs(0.0, y, f), 3)
    v = np.random.default_rng(0).normal(size=y.size)
    out = np.empty_like(y)
    work = (np.empty_like(y), np.empty_like(y))
    ynorm = float(np.linalg.norm(y))
    eps = float(np.sqrt(np.finfo(np.float64).eps))
    t_jv = timed(lambda: e.jv(y, f, v, out, 1.0, -gamma, ynorm, eps, work), 3)
    t0 = time.perf_counter()
    rc_p, _ = e.pset(0.0, y, f, 0, gamma)
    t_pset = time.perf_counter() - t0
    z = np.empty_like(y)
    t_psol = timed(lambda: e.psol(0.0, None, None, v, z, gamma), 2)
    rhs, pset, psol = e.callbacks()
    yb = y.copy()
    t0 = time.perf_counter()
    rc, st = O.bdf_run(y.size, rhs, pset, psol, e.h, yb,
                       O.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=nsteps, msbp=msbp))
    t_bdf = time.perf_counter() - t0
    e.close()
    return {
        "value": st["n_steps"] / t_bdf if rc == 0 else None, "unit": UNIT, "cores": threads,
        "kind": "port",
        "sample": (f"{st['n_steps']} whole BDF step(s) of the workload at its full size ({nC} "
                   f"cells: {st['n_newton']} Newton, {st['n_lin_iters']} Krylov iterations, "
                   f"{t_bdf:.2f} s) plus one residual, Jv, pset and ILU(0) apply timed "
                   f"separately; the oracle built for this host's ISA, OpenMP in the residual "
                   f"loops (atomic scatter as Euler.f90:71-155), the rest serial as in the "
                   f"reference (no extrapolation)"),
        "rc": rc, "setup_s": round(setup_s, 2),
        "per_op": {"residual_evals_per_s": 1.0 / t_rhs, "jv_per_s": 1.0 / t_jv,
                   "ilu_apply_per_s": 1.0 / t_psol, "pset_s": t_pset, "pset_rc": rc_p},
        "oracle_lib": os.path.relpath(O.lib_path(), ROOT),
    }


def run_reference(args, world, rank, pg):
    """The reference arm: the oracle (the reference arithmetic restated in C, tuned build,
    OpenMP residual loops on every host core) on the bench workload at its full size, from
    the oracle's own grid construction (polyGrid%up + getNeibPolyFvGrid + sortPolyFvGrid
    restated), through its CVODE-shaped callbacks and fixed-step BDF Newton--GMRES(30)
    driver with SPARSKIT ilu0 in the reference's natural cell order: W untimed BDF steps,
    then K timed BDF steps from the same initial state.  Nothing of the GPU library runs."""
    if rank != 0:
        return
    from fosolvers_gb300 import mesh as M
    from oracle import pyoracle as O
    threads = os.cpu_count() or 1
    t_setup = time.perf_counter()
    wl = M.make_workload(args.workload, scale=args.scale)
    O.set_default("tuned")
    grid = O.grid_build(wl.mesh)
    e = _oracle_context(wl, grid, threads)
    nC = grid["nC"]
    y0 = M.soa(wl.elem_state, nC)
    rhs, pset, psol = e.callbacks()
    opts = lambda n: O.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=n, msbp=args.msbp)
    setup_s = time.perf_counter() - t_setup
    if args.warmup:
        yw = y0.copy()
        rc_w, _ = O.bdf_run(y0.size, rhs, pset, psol, e.h, yw, opts(args.warmup))
        assert rc_w == 0, f"oracle warm-up failed: {rc_w}"
    y = y0.copy()
    t0 = time.perf_counter()
    rc, st = O.bdf_run(y0.size, rhs, pset, psol, e.h, y, opts(args.steps))
    dt = time.perf_counter() - t0
    e.close()
    assert rc == 0, f"oracle run failed: {rc} {st}"
    value = args.steps / dt
    size = "at its full size" if args.scale is None else f"at scale {args.scale}"
    sample = (f"{args.steps} BDF steps of the workload {size} ({nC} cells) after "
              f"{args.warmup} untimed ones, from the same initial state ({st['n_newton']} "
              f"Newton, {st['n_lin_iters']} Krylov iterations, {dt:.1f} s); the oracle built "
              f"for this host's ISA, OpenMP on {threads} threads in the residual loops "
              f"(atomic scatter as Euler.f90:71-155), Jacobian, ilu0/lusol and Krylov serial "
              f"as in the reference")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded mesh and state)",
        "config": {"workload": workload_desc(args.workload) if args.scale is None else
                   f"{args.workload} at scale {args.scale}", "cells": nC,
                   "pset": "every BDF step" if args.msbp == 1 else f"CVODE policy, MSBP {args.msbp}",
                   "runner": "CPU oracle (the reference arithmetic restated in C; the Fortran "
                             "reference cannot be compiled here)",
                   "oracle_lib": os.path.relpath(O.lib_path(), ROOT),
                   "setup_s": round(setup_s, 2)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "stats": st,
    }
    print(json.dumps(line), flush=True)


def workload_desc(name: str) -> str:
    return {
        "sine96": "unit cube 96^3 hexes x 6 = 5,308,416 tets, +-0.1h node jitter (seed 0), "
                  "sinusoidal rho/u state, p = 1, slip walls, BDF2 dt = 5e-4, Newton rtol 1e-8, "
                  "GMRES(30) forcing 1e-3",
        "sod16": "unit cube 16^3 x 6 = 24,576 tets, Sod, walls, BDF1 dt = 1e-3",
        "bump192": "bump channel 192x64x32 x 6 = 2,359,296 tets, Mach 2 inflow, BDF1 CFL~5",
        "bump320": "bump channel 320x107x53 x 6 = 10,888,320 tets, Mach 2 inflow, BDF2 CFL~5",
    }.get(name, name)


# ------------------------------------------------------------------ GPU arm
PRECOND = {"none": 0, "ilu": 1, "learned": 2}


def make_ctx(grid, ibc, wl, mode, ilu_order, stream):
    from fosolvers_gb300.euler import FLUX_FP32, FLUX_HYBRID, ILU_COLOR, ILU_FP32, FOEuler
    flags = {"fp32": FLUX_FP32 | ILU_FP32, "fp32h": FLUX_FP32 | FLUX_HYBRID | ILU_FP32,
             "fp32ilu": ILU_FP32, "fp64": 0}[mode]
    if ilu_order == "color":
        flags |= ILU_COLOR
    return FOEuler(grid, ibc, wl.bc_type, wl.bc_param, wl.gamm, wl.r, flags=flags, stream=stream)


def timed_bdf(ctx, y0, mk, args, dev, stream, pg, clocks=None):
    """W untimed BDF steps, then K BDF steps from the same initial state timed with CUDA
    events on the library stream (barrier + synchronize on both sides)."""
    import torch
    y = y0.clone()
    rc, _ = ctx.bdf_run(y, mk(args.warmup))
    assert rc == 0, f"warm-up failed: {rc}"
    torch.cuda.synchronize(dev)
    y = y0.clone()
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize(dev)
    launches0 = ctx.info()["launches"]
    if clocks:
        clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    rc, st = ctx.bdf_run(y, mk(args.steps))
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    clk = clocks.stop() if clocks else None
    if pg is not None:
        pg.barrier()
    assert rc == 0, f"timed run failed: {rc} {st}"
    return ev0.elapsed_time(ev1), st, ctx.info()["launches"] - launches0, clk, y


def field_rel_err(a, b, nC):
    """max over density, momentum (as a vector) and energy of max|a-b| / max|b|."""
    a, b = a.reshape(5, nC), b.reshape(5, nC)
    e = [float((a[0] - b[0]).abs().max() / b[0].abs().max()),
         float((a[1:4] - b[1:4]).norm(dim=0).max() / b[1:4].norm(dim=0).max()),
         float((a[4] - b[4]).abs().max() / b[4].abs().max())]
    return max(e)


def per_variable_err(a, b, nC):
    """max |a - b| / max |b| of each conserved variable (rho, rho u, rho v, rho w, rho E)."""
    a, b = a.reshape(5, nC), b.reshape(5, nC)
    names = ("rho", "rhou", "rhov", "rhow", "rhoE")
    return {n: float((a[q] - b[q]).abs().max() / b[q].abs().max()) for q, n in enumerate(names)}


def cell_rel_err(a, b, nC):
    """largest per-cell relative error ||a_c - b_c|| / ||b_c|| over the 5 conserved values."""
    a, b = a.reshape(5, nC), b.reshape(5, nC)
    return float(((a - b).norm(dim=0) / b.norm(dim=0)).max())


def main():
    args = parse()
    if args.profile_ops:
        profile_ops(args)
        return
    if args.ilut:
        run_ilut(args)
        return
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
        if pg is not None:
            pg.barrier()
        return
    import torch
    from __graft_entry__ import build
    build()
    from fosolvers_gb300 import mesh as M
    from fosolvers_gb300.euler import PolyFvGrid

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t_setup = time.perf_counter()
    wl = M.make_workload(args.workload, scale=args.scale)
    grid = PolyFvGrid.from_mesh(wl.mesh)
    ibc = M.ibc_for(wl.mesh, wl.bc_gid)
    stream = torch.cuda.current_stream(dev)
    ctx = make_ctx(grid, ibc, wl, args.mode, args.ilu_order, stream)
    nC, nF = grid.nC, grid.nP
    N = 5 * nC
    y0_host = M.soa(wl.elem_state, nC)
    y0_ref = torch.from_numpy(y0_host).to(dev)
    y0 = torch.empty_like(y0_ref)
    ctx.to_internal(y0_ref, y0)
    precond = PRECOND[args.precond]
    gnn = None
    if args.precond == "learned":
        from fosolvers_gb300.learned import GNN
        gnn = GNN(seed=0)
        from fosolvers_gb300.learned import DEFAULT_WEIGHTS
        gnn.load(args.weights or DEFAULT_WEIGHTS)
        ctx.attach_gnn(gnn)

    def mk_for(pc):
        return lambda n, **kw: ctx.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=n, precond=pc,
                                                msbp=args.msbp, **kw)

    mk = mk_for(precond)
    setup_s = time.perf_counter() - t_setup

    # headline: K BDF steps with the state in HBM (inputs > L2: state 0.2 GB, factors ~3-5 GB)
    ms, st, launches, clk, y = timed_bdf(ctx, y0, mk, args, dev, stream, pg, Clocks(local))
    ms_max = allmax(pg, ms, dev)
    value = world * args.steps / (ms_max / 1000.0)

    # the same steps with ILU(0) alone in the same precision (learned runs only)
    alt = {}
    if args.precond == "learned" and not args.no_compare:
        ms_i, st_i, _, _, _ = timed_bdf(ctx, y0, mk_for(1), args, dev, stream, pg)
        alt[f"{args.mode}_ilu"] = {"value": world * args.steps / (allmax(pg, ms_i, dev) / 1e3),
                                   "ms_per_step": ms_i / args.steps,
                                   "n_lin_iters": st_i["n_lin_iters"]}
    # the headline arm under the other preconditioner set-up policy: a pset at every BDF step
    # when the headline follows CVODE (psets at the first step, on the BDF1 -> BDF2 gamma
    # change and every MSBP steps), CVODE's MSBP 20 when the headline sets up every step
    cvode = None
    alt_msbp = 1 if args.msbp > 1 else 20
    if not args.no_compare and not args.no_cvode:
        mk_c = lambda n, **kw: ctx.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=n,
                                                precond=precond, msbp=alt_msbp, **kw)
        ms_c, st_c, _, _, _ = timed_bdf(ctx, y0, mk_c, args, dev, stream, pg)
        cvode = {"msbp": alt_msbp, "value": world * args.steps / (allmax(pg, ms_c, dev) / 1e3),
                 "ms_per_step": ms_c / args.steps, "n_pset": st_c["n_pset"],
                 "n_lin_iters": st_c["n_lin_iters"]}
    # the headline arm with CVODE's constant-step BDF predictor as Newton's first iterate
    # (fos_bdf_opts.predictor = 1; the default starts from y_n)
    alt_pred = None
    if not args.no_compare and not args.no_cvode:
        mk_p = lambda n, **kw: mk(n, predictor=1, **kw)
        ms_p, st_p, _, _, _ = timed_bdf(ctx, y0, mk_p, args, dev, stream, pg)
        alt_pred = {"predictor": 1, "value": world * args.steps / (allmax(pg, ms_p, dev) / 1e3),
                    "ms_per_step": ms_p / args.steps, "n_newton": st_p["n_newton"],
                    "n_lin_iters": st_p["n_lin_iters"]}

    # end to end: host buffer in the caller's cell order, copied in and out every step
    e2e = None
    if not args.no_e2e:
        yh = torch.from_numpy(y0_host.copy()).pin_memory()
        yhn = yh.numpy()
        ctx.bdf_run_host(yhn, mk(1))  # warm
        yhn[:] = y0_host
        t0 = time.perf_counter()
        for k in range(args.steps):
            rc_e, _ = ctx.bdf_run_host(yhn, mk(1, resume=1 if k else 0))
            assert rc_e == 0
        e2e_s = allmax(pg, time.perf_counter() - t0, dev)
        e2e = {"value": world * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N}

    # per-operation timing (CUDA events on the library stream)
    ops = {}
    if not args.no_ops:
        f = torch.empty_like(y)
        v = torch.randn(N, dtype=torch.float64, device=dev)
        out = torch.empty_like(y)
        ynorm = float(torch.linalg.norm(y))
        gamma = wl.dt * (2.0 / 3.0 if wl.order == 2 else 1.0)
        info = ctx.info()
        nnzb = info["nnzb"]
        fb = 8 if args.mode == "fp64" else 4

        def timeit(fn, reps):
            fn()
            torch.cuda.synchronize(dev)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            return a.elapsed_time(b) / reps

        R = args.op_reps
        t_rhs = timeit(lambda: ctx.rhs_dev(0.0, y, f), 3 * R)
        # Jv as the Krylov driver calls it: ||v|| known from the preconditioner's output pass
        vnorm = float(torch.linalg.norm(v))
        t_jv = timeit(lambda: ctx.jv_dev_vnorm(0.0, y, f, v, out, 1.0, -gamma, ynorm, vnorm),
                      3 * R)
        t_pset = timeit(lambda: ctx.pset_dev(0.0, y, 0, gamma), max(2, R // 2))
        t_psol = timeit(lambda: ctx.psol_dev(v, out), R)
        lev = info["nlev_fwd"] + info["nlev_bwd"]
        a_, f_ = nC, nF
        n_gnn = st["n_learned"] if gnn is not None else 0
        # algorithmic bytes (what the operation must move at least, in this layout):
        #   residual  state in (40) + f out (40) + 1/V (8) per cell; face pair (8) and
        #             geometry (16 FP32 / 32 FP64) per face
        #   Jv        + v, f(y) in per cell (80)
        #   ILU apply the factors (25 values per block) + r in / z out (80 per cell)
        #   pset      state in, geometry, J written, J read and LU written by the factor
        gb = 8 + (16 if args.mode in ("fp32", "fp32h") else 32)
        #   pset      FP32 factors (fused set-up: J assembled inside the factor, never stored):
        #             state in (40 per cell), face pair and geometry, the factors written
        #             (25 values per block), and every inv(D_q) and U_qp block read once by the
        #             rows below it (one per cell and one per interior face);
        #             FP64: state, geometry, J written, J read and the factors written
        if fb == 4:
            pset_bytes = 40 * a_ + gb * f_ + 25 * fb * nnzb + 25 * fb * (a_ + grid.nPi)
        else:
            pset_bytes = 48 * a_ + gb * f_ + 3 * 25 * fb * nnzb
        ops = {
            "residual": {"ms": t_rhs, "bytes": 88 * a_ + gb * f_, "count": st["n_rhs"] - st["n_jv"]},
            "jv": {"ms": t_jv, "bytes": 168 * a_ + gb * f_, "count": st["n_jv"]},
            "ilu_apply": {"ms": t_psol, "bytes": 25 * fb * nnzb + 80 * a_,
                          "count": st["n_psol"] - n_gnn, "levels": lev},
            "pset": {"ms": t_pset, "bytes": pset_bytes, "count": st["n_pset"]},
        }
        if gnn is not None:
            t_gnn = timeit(lambda: gnn.apply_dev(ctx, y, v, out, gamma), R)
            ops["gnn_apply"] = {"ms": t_gnn, "bytes": GNN_BYTES_PER_CELL * a_, "count": n_gnn}
        for k, o in ops.items():
            o["GBps"] = o["bytes"] / (o["ms"] * 1e-3) / 1e9
            o["ms_per_step"] = o["ms"] * o["count"] / args.steps
    info = ctx.info()
    y_out = torch.empty_like(y)
    ctx.to_reference(y, y_out)
    # the same K steps of this arm at a tightened Newton tolerance (untimed): the state
    # difference from the FP64 path at the same tolerance shows how much of the difference at
    # the workload's 1e-8 is the Newton tolerance rather than the arithmetic
    y_tight = None
    if args.tight_rtol > 0 and args.mode != "fp64" and not args.no_compare:
        yt = y0.clone()
        rc_t, st_t = ctx.bdf_run(yt, mk(args.steps, newton_rtol=args.tight_rtol, max_newton=20))
        if rc_t == 0:
            y_tight = torch.empty_like(yt)
            ctx.to_reference(yt, y_tight)
    ctx.close()

    # the plain FP64 ILU(0)-GMRES path on the same mesh and state: the target's denominator
    vs64 = None
    if args.mode != "fp64" and not args.no_compare:
        ctx64 = make_ctx(grid, ibc, wl, "fp64", args.ilu_order, stream)
        y064 = torch.empty_like(y0_ref)
        ctx64.to_internal(y0_ref, y064)
        mk64 = lambda n, **kw: ctx64.bdf_defaults(**{**dict(order=wl.order, dt=wl.dt, nsteps=n,
                                                            precond=1, msbp=args.msbp), **kw})
        ms64, st64, _, _, y64 = timed_bdf(ctx64, y064, mk64, args, dev, stream, pg)
        v64 = world * args.steps / (allmax(pg, ms64, dev) / 1000.0)
        yb = torch.empty_like(y)
        ctx64.to_reference(y64, yb)  # both states in the reference cell order
        vs64 = {"value": v64, "ms_per_step": ms64 / args.steps, "ratio": value / v64,
                "n_lin_iters": st64["n_lin_iters"],
                # both runs converge Newton to ||G||_2 <= 1e-8 ||y||_2; the max-norm field
                # error reflects that tolerance at 26.5M unknowns, the l2 error the precision
                "state_rel_err_vs_fp64": field_rel_err(y_out, yb, nC),
                "state_rel_l2_vs_fp64": float((y_out - yb).norm() / yb.norm()),
                "state_err_per_variable": per_variable_err(y_out, yb, nC)}
        vs64["state_cell_rel_err_vs_fp64"] = cell_rel_err(y_out, yb, nC)
        # yardstick: the FP64 flux with the learned preconditioner, i.e. the FP64 path's own
        # arithmetic on another Krylov path, against the FP64 ILU(0) path -- the difference
        # the Newton tolerance alone allows between two FP64 runs
        if gnn is not None:
            ctx64.attach_gnn(gnn)
            yl = y064.clone()
            rc_l, _ = ctx64.bdf_run(yl, mk64(args.steps, precond=2))
            ctx64.attach_gnn(None)
            if rc_l == 0:
                ylb = torch.empty_like(yl)
                ctx64.to_reference(yl, ylb)
                vs64["fp64_learned_vs_fp64"] = {
                    "state_rel_err": field_rel_err(ylb, yb, nC),
                    "state_cell_rel_err": cell_rel_err(ylb, yb, nC),
                    "state_rel_l2": float((ylb - yb).norm() / yb.norm())}
        if y_tight is not None:
            yt64 = y064.clone()
            rc_t, _ = ctx64.bdf_run(yt64, mk64(args.steps, newton_rtol=args.tight_rtol,
                                               max_newton=20))
            if rc_t == 0:
                ytb = torch.empty_like(yt64)
                ctx64.to_reference(yt64, ytb)
                vs64["tight_newton_rtol"] = {
                    "newton_rtol": args.tight_rtol,
                    "state_rel_err_vs_fp64": field_rel_err(y_tight, ytb, nC),
                    "state_cell_rel_err_vs_fp64": cell_rel_err(y_tight, ytb, nC),
                    "state_rel_l2_vs_fp64": float((y_tight - ytb).norm() / ytb.norm())}
        if cvode is not None:
            mk64c = lambda n, **kw: ctx64.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=n,
                                                       precond=1, msbp=alt_msbp, **kw)
            ms64c, st64c, _, _, _ = timed_bdf(ctx64, y064, mk64c, args, dev, stream, pg)
            cvode["fp64_value"] = world * args.steps / (allmax(pg, ms64c, dev) / 1e3)
            cvode["fp64_n_pset"] = st64c["n_pset"]
            cvode["ratio"] = cvode["value"] / cvode["fp64_value"]
        ctx64.close()

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = peaks.get("hbm_gbs", 6800.0)
    roof = None
    if ops:
        dom = max(ops, key=lambda k: ops[k]["ms_per_step"])
        o = ops[dom]
        tr = TRAFFIC_FP32_BYTES_PER_CELL.get(dom) if args.mode == "fp32" else None
        roof = {"bound": "hbm", "achieved": round(o["GBps"], 1), "peak": hbm, "unit": "GB/s",
                "frac": round(o["GBps"] / hbm, 4),
                "traffic": round(tr * nC) if tr else None, "algorithmic_bytes": o["bytes"],
                "op": dom, "peak_source": "measured (hbm_gbs)" if peaks else "fallback",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per cell at "
                                  "64^3 x 6 (L2 flushed per kernel) x cells" if tr else None,
                "per_op": {k: {"ms": round(v["ms"], 4), "GBps": round(v["GBps"], 1),
                               "frac": round(v["GBps"] / hbm, 4), "per_step": v["count"] / args.steps,
                               "ms_per_step": round(v["ms_per_step"], 3)}
                           for k, v in ops.items()}}
        if args.mode == "fp32":
            # the FP64 pipe's share of the operation's time: its FP64 lane-instructions at
            # 2 per clock per SM, at the median SM clock sampled during the timed region
            sms = torch.cuda.get_device_properties(dev).multi_processor_count
            mhz = (clk or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
            for k, n in FP64_INSTR_PER_CELL_FP32.items():
                if k in roof["per_op"]:
                    t_fp64 = n * nC / (2.0 * sms * mhz * 1e6)
                    roof["per_op"][k]["fp64_pipe"] = {
                        "instr_per_cell": n, "ms_at_pipe_peak": round(t_fp64 * 1e3, 4),
                        "frac": round(t_fp64 / (ops[k]["ms"] * 1e-3), 4)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cb = cpu_oracle_fullsize(wl, grid.__dict__, nsteps=1, msbp=args.msbp)
            cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "per_op",
                                      "oracle_lib")}
        except Exception as exc:  # the baseline never blocks the GPU line
            cpu = {"value": None, "error": repr(exc)}
    # absolute rates at the workload's cell count (device-resident, CUDA events):
    # residual evaluations/s and Jv/s from the per-operation timing
    thr = {"bdf_steps_per_s": value, "cells": nC}
    if roof and roof.get("per_op"):
        po = roof["per_op"]
        if "residual" in po:
            thr["residual_evals_per_s"] = round(1e3 / po["residual"]["ms"], 1)
        if "jv" in po:
            thr["jv_per_s"] = round(1e3 / po["jv"]["ms"], 1)
        if "ilu_apply" in po:
            thr["ilu_apply_per_s"] = round(1e3 / po["ilu_apply"]["ms"], 1)
    if cpu and cpu.get("per_op"):
        thr["cpu"] = {k: (round(v, 3) if isinstance(v, float) else v)
                      for k, v in cpu["per_op"].items()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "fp32": "f32 flux/ILU, f64 Newton+Krylov",
                      "fp32h": "f32 flux (f64 on faces with >5% jumps and boundaries), f32 "
                               "ILU, f64 Newton+Krylov",
                      "fp32ilu": "f64 flux, f32 ILU, f64 Newton+Krylov"}[args.mode],
            "data": "synthetic (seeded mesh and state)",
            "config": {"workload": workload_desc(args.workload) if args.scale is None else
                       f"{args.workload} at scale {args.scale}",
                       "cells": nC, "faces": nF, "mode": args.mode, "precond": args.precond,
                       "pset": "every BDF step" if args.msbp == 1 else f"CVODE policy, MSBP {args.msbp}",
                       "ilu_order": args.ilu_order, "ilu_levels": [info["nlev_fwd"], info["nlev_bwd"]],
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                       "l2": "inputs larger than L2 (state 0.2 GB, ILU factors ~3-5 GB); no flush",
                       "setup_s": round(setup_s, 2)},
            "clocks": clk, "e2e": e2e, "gpu_launches": launches,
            "roofline": roof, "throughput": thr, "cpu_baseline": cpu,
            "vs_fp64_ilu": vs64, "same_precision_ilu": alt or None,
            "alt_setup_policy": cvode, "alt_predictor": alt_pred,
            "stats": {k: st[k] for k in ("n_rhs", "n_jv", "n_psol", "n_pset", "n_newton",
                                          "n_lin_iters", "n_steps", "n_fallback", "n_learned",
                                          "n_gated", "n_reorth")},
        }
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
