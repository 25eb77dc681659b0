"""The learned preconditioner's kernels against the numpy reference (oracle/gnn_ref.py):
forward output and every weight gradient, with BF16 weights and activations on both sides.
Tolerances: 2e-2 relative (norm-wise per parameter block) -- BF16 rounding of activations
can flip at different summation orders."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from helpers import Case, perturbed
from oracle import gnn_ref as R

pytestmark = pytest.mark.gpu


def _setup(seed=0, scale=5):
    import torch
    from fosolvers_gb300.learned import GNN
    c = Case(M.make_workload("sine96", scale=scale, seed=seed))
    g = GNN(seed=seed)
    w = g.params()
    rng = np.random.default_rng(seed)
    w[R.OFF_D:R.OFF_DB] = 0.05 * rng.standard_normal(R.OFF_DB - R.OFF_D).astype(np.float32)
    w[R.OFF_DB:] = 0.01 * rng.standard_normal(R.NPARAM - R.OFF_DB).astype(np.float32)
    for l in range(R.NL):
        o = R.OFF_L0 + l * R.L_SIZE
        w[o + R.L_B:o + R.L_SIZE] = 0.05
    g.set_params(w)
    y = perturbed(c.y0, c.nC, seed + 1)
    v = rng.standard_normal(c.N)
    t = v + 0.1 * rng.standard_normal(c.N)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    ints = []
    for a in (y, v, t):
        out = torch.empty(c.N, dtype=torch.float64, device="cuda")
        c.gpu.to_internal(dev(a), out)
        ints.append(out)
    return c, g, w, (y, v, t), ints


def test_gnn_forward_matches_reference(cuda):
    import torch
    c, g, w, (y, v, t), (yi, vi, ti) = _setup()
    zi = torch.empty_like(vi)
    g.apply_dev(c.gpu, yi, vi, zi, 2e-3)
    zr = torch.empty_like(zi)
    c.gpu.to_reference(zi, zr)
    z = zr.cpu().numpy()
    graph = R.Graph(c.grid)
    z_ref = R.forward(R.split(w), graph, y, v, 2e-3)
    corr, corr_ref = z - v, z_ref - v
    err = np.linalg.norm(corr - corr_ref) / np.linalg.norm(corr_ref)
    print("gnn forward rel err", err)
    assert np.linalg.norm(corr_ref) > 0
    assert err <= 2e-2


def test_gnn_gradients_match_reference(cuda):
    c, g, w, (y, v, t), (yi, vi, ti) = _setup(seed=3)
    g.zero_grad()
    loss = g.loss_grad_dev(c.gpu, yi, vi, ti, 2e-3)
    grad = g.grad()
    graph = R.Graph(c.grid)
    loss_ref, grad_ref = R.loss_grad(w, graph, y, v, t, 2e-3)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    blocks = {"W0": (R.OFF_W0, R.OFF_B0), "b0": (R.OFF_B0, R.OFF_L0), "D": (R.OFF_D, R.OFF_DB),
              "d": (R.OFF_DB, R.NPARAM)}
    for l in range(R.NL):
        o = R.OFF_L0 + l * R.L_SIZE
        blocks.update({f"G{l}": (o + R.L_G, o + R.L_C), f"c{l}": (o + R.L_C, o + R.L_A),
                       f"A{l}": (o + R.L_A, o + R.L_B), f"b{l}": (o + R.L_B, o + R.L_SIZE)})
    for name, (a, b) in blocks.items():
        ref = grad_ref[a:b]
        err = np.linalg.norm(grad[a:b] - ref) / max(np.linalg.norm(ref), 1e-30)
        print(f"grad {name}: rel err {err:.2e}  |ref| {np.linalg.norm(ref):.3e}")
        assert err <= 2e-2, name


def test_gnn_untrained_is_identity(cuda):
    import torch
    from fosolvers_gb300.learned import GNN
    c = Case(M.make_workload("sine96", scale=4, seed=1))
    g = GNN(seed=7)
    v = torch.randn(c.N, dtype=torch.float64, device="cuda")
    y = torch.empty_like(v)
    c.gpu.to_internal(torch.from_numpy(c.y0).cuda(), y)
    z = torch.empty_like(v)
    g.apply_dev(c.gpu, y, v, z, 1e-3)
    torch.cuda.synchronize()
    rel = (z - v).abs().max().item() / v.abs().max().item()
    assert rel <= 1e-6  # float32 round trip of v / s_v * s_v
