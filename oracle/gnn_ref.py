"""numpy reference of the learned preconditioner (forward, loss, backward) -- TEST
INFRASTRUCTURE ONLY, the oracle the GPU network kernels are tested against.

Same model and parameter layout as the library's network, with BF16 rounding at the
same points: weights; h0, m and h after each layer.  Sums are in float32.  It runs in
the reference cell order on the face arrays of a PolyFvGrid; the GPU works in its
internal order, so tests permute before comparing.  The loss is
mean((v/s_v + D h3 + d - t/s_v)^2) over cells and the five components.
"""
from __future__ import annotations

import numpy as np

H, NIN, NL, NOUT = 64, 16, 3, 8
OFF_W0 = 0
OFF_B0 = OFF_W0 + H * NIN
OFF_L0 = OFF_B0 + H
L_G, L_C = 0, H * 4
L_A = L_C + H
L_B = L_A + H * 2 * H
L_SIZE = L_B + H
OFF_D = OFF_L0 + NL * L_SIZE
OFF_DB = OFF_D + NOUT * H
NPARAM = OFF_DB + NOUT


def bf16(x):
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rnd = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rnd) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32)


def trunc32(x):
    """float64 -> float32 rounding toward zero (the GPU's integer conversion)."""
    x = np.asarray(x, np.float64)
    f = x.astype(np.float32)
    over = np.abs(f.astype(np.float64)) > np.abs(x)
    f[over] = np.nextafter(f[over], np.float32(0))
    return f


class Graph:
    """Directed edges (i <- j) with features seen from i, from the reference face arrays."""

    def __init__(self, grid):
        self.invv = trunc32(1.0 / grid.v)
        nC = grid.nC
        inner = np.arange(grid.nPi)
        L = grid.iEP[inner, 0] - 1
        R = grid.iEP[inner, 1] - 1
        n = grid.normP[inner].astype(np.float32)
        a = grid.aP[inner].astype(np.float32)
        amean = np.float32(grid.aP.astype(np.float32).sum(dtype=np.float32) / np.float32(grid.nP))
        an = (a / amean)[:, None]
        self.dst = np.concatenate([L, R])  # i
        self.src = np.concatenate([R, L])  # j
        e_out = np.concatenate([n * an, -n * an])  # outward normal of i, scaled
        self.e = np.concatenate([e_out, np.concatenate([an, an])], axis=1).astype(np.float32)
        self.nC = nC
        self.logv = -np.log(self.invv)


def split(w):
    w = bf16(np.asarray(w, np.float32))
    p = {"W0": w[OFF_W0:OFF_B0].reshape(H, NIN), "b0": w[OFF_B0:OFF_L0], "layers": [],
         "D": w[OFF_D:OFF_DB].reshape(NOUT, H)[:5], "d": w[OFF_DB:OFF_DB + 5]}
    for l in range(NL):
        o = OFF_L0 + l * L_SIZE
        p["layers"].append({"G": w[o + L_G:o + L_C].reshape(H, 4), "c": w[o + L_C:o + L_A],
                            "A": w[o + L_A:o + L_B].reshape(H, 2 * H), "b": w[o + L_B:o + L_SIZE]})
    return p


def scales(graph, y, v):
    nC = graph.nC
    y = y.reshape(5, nC).astype(np.float64)
    v = v.reshape(5, nC).astype(np.float64)
    sy0 = np.sqrt((y[0] ** 2).mean())
    sy1 = np.sqrt((y[1:4] ** 2).sum(0).mean() / 3.0) + 1e-6 * sy0
    sy2 = np.sqrt((y[4] ** 2).mean())
    rv = np.sqrt((v ** 2).mean(1))
    sv = rv + 1e-6 * rv.max() + 1e-30
    return np.float32([sy0, sy1, sy1, sy1, sy2]), sv.astype(np.float32), np.float32(graph.logv.mean())


def forward(params, graph, y, v, gamma, keep=False, gas_g=1.4):
    nC = graph.nC
    sy, sv, lvm = scales(graph, y, v)
    x = np.zeros((nC, NIN), np.float32)
    x[:, 0:5] = trunc32(y.reshape(5, nC)).T / sy
    x[:, 5:10] = trunc32(v.reshape(5, nC)).T / sv
    x[:, 10] = graph.logv - lvm
    yt = trunc32(y.reshape(5, nC))
    q2 = (yt[1] ** 2 + yt[2] ** 2 + yt[3] ** 2) / (yt[0] * yt[0])
    p = np.float32(gas_g - 1.0) * (yt[4] - np.float32(0.5) * yt[0] * q2)
    cs = np.sqrt(np.maximum(np.float32(gas_g) * p / yt[0], 0))
    cfl = np.float32(gamma) * (np.sqrt(q2) + cs) * np.cbrt(graph.invv)
    x[:, 11] = np.log(np.maximum(cfl, np.float32(1e-12)))
    h = bf16(np.maximum(x @ params["W0"].T + params["b0"], 0))
    hs, ms = [h], []
    for L in params["layers"]:
        g = graph.e @ L["G"].T + L["c"]  # (edges, H)
        msg = g * hs[-1][graph.src]
        m = np.zeros((nC, H), np.float32)
        np.add.at(m, graph.dst, msg)
        m = bf16(m)
        X = np.concatenate([hs[-1], m], axis=1)
        h = bf16(np.maximum(X @ L["A"].T + L["b"], 0))
        ms.append(m)
        hs.append(h)
    vh = trunc32(v.reshape(5, nC)).T / sv
    zhat = vh + hs[-1] @ params["D"].T + params["d"]
    z = (zhat * sv).T.reshape(-1).astype(np.float64)
    if keep:
        return z, dict(x=x, hs=hs, ms=ms, zhat=zhat, sv=sv)
    return z


def loss_grad(w, graph, y, v, t, gamma):
    """Loss and gradient (FP32 master layout) of mean((zhat - t/s_v)^2)."""
    p = split(w)
    nC = graph.nC
    _, st = forward(p, graph, y, v, gamma, keep=True)
    th = trunc32(t.reshape(5, nC)).T / st["sv"]
    e = st["zhat"] - th
    N = 5 * nC
    loss = float((e.astype(np.float64) ** 2).sum() / N)
    g = np.zeros(NPARAM, np.float32)
    dz = (2.0 * e / N).astype(np.float32)
    h3 = st["hs"][-1]
    D = np.zeros((NOUT, H), np.float32)
    D[:5] = dz.T @ h3
    g[OFF_D:OFF_DB] = D.reshape(-1)
    g[OFF_DB:OFF_DB + 5] = dz.sum(0)
    dh = dz @ p["D"]
    for l in reversed(range(NL)):
        L = p["layers"][l]
        o = OFF_L0 + l * L_SIZE
        hin, m, hout = st["hs"][l], st["ms"][l], st["hs"][l + 1]
        delta = dh * (hout > 0)
        db = bf16(delta)
        X = np.concatenate([hin, m], axis=1)
        g[o + L_A:o + L_B] = (db.T @ X).reshape(-1)
        g[o + L_B:o + L_SIZE] = delta.sum(0)
        dX = db @ L["A"]
        dhin = dX[:, :H].copy()
        dm = dX[:, H:]
        # m_i = sum_j g_ij h_j  over edges (i <- j)
        gate = graph.e @ L["G"].T + L["c"]
        np.add.at(dhin, graph.src, gate * dm[graph.dst])
        dg = dm[graph.dst] * hin[graph.src]  # (edges, H)
        g[o + L_G:o + L_C] = (dg.T @ graph.e).reshape(-1)
        g[o + L_C:o + L_A] = dg.sum(0)
        dh = dhin
    d0 = dh * (st["hs"][0] > 0)
    g[OFF_W0:OFF_B0] = (d0.T @ st["x"]).reshape(-1)
    g[OFF_B0:OFF_L0] = d0.sum(0)
    return loss, g
