"""FP64 numpy restatement of the learned preconditioner's network.

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward / backward
kernels (nalu-wind_gb300/csrc/learned.cu). Same architecture and loss:
  u = D^-1 rc, s = rms(u), x = u / s, (W h)_I = sum_J w_IJ h_J (no diagonal)
  H0 = relu([x, W x] W0); Hl = relu([H(l-1), W H(l-1)] Wl), l = 1..3
  ec = s * H3 wout
  alpha = ec' rc / ec' Ac ec,  Ac = D (I - W), D = diag(1 / dinv)
  L = (cA - (ec' rc)^2 / ec' Ac ec) / eA
(the energy norm of the error left by smoothing and the alpha-scaled
coarse correction, normalised by the energy norm of the error; alpha and
the removed energy are 0 unless ec' Ac ec > 0; the gradient takes Ac as
symmetric, as the GPU kernels do).
Parameters are the library's flat layout: W0 (2 x 64) | W1 | W2 | W3
(128 x 64 each, row-major) | wout (64). This network has no counterpart
in the reference (its preconditioners are Ifpack2 / MueLu).

With bf16=True the restatement rounds to bfloat16 (round to nearest even)
at the points where the GPU kernels store BF16: the weights W1..W3, every
hidden activation H, every aggregated activation W H, and every masked
activation gradient dZ. Everything else stays FP64, so the remaining
difference to the GPU is its FP32 accumulation.
"""
from __future__ import annotations

import numpy as np

H = 64


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    w0 = p[o:o + 2 * H].reshape(2, H); o += 2 * H
    ws = []
    for _ in range(3):
        ws.append(p[o:o + 2 * H * H].reshape(2 * H, H)); o += 2 * H * H
    wout = p[o:o + H]
    return w0, ws, wout


def bf16(a):
    """Round to bfloat16 (nearest even) through float32, returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def agg_matrix(cg):
    """Dense (nc x nc) matrix of w_IJ without the diagonal (small graphs)."""
    nc = cg["nc"]
    W = np.zeros((nc, nc))
    for I in range(nc):
        for q in range(cg["cptr"][I], cg["cptr"][I + 1]):
            J = cg["ccol"][q]
            if J != I:
                W[I, J] += float(cg["wgt"][q])
    return W


def coarse_operator(cg):
    """Dense Ac = D (I - W) from the weights and inverse diagonal."""
    W = agg_matrix(cg)
    dinv = np.asarray(cg["dinv"], np.float64)
    d = np.where(dinv != 0, 1.0 / np.where(dinv != 0, dinv, 1.0), 0.0)
    return d[:, None] * (np.eye(len(d)) - W)


def loss_and_grad(p, cg, rc, ea, ca, bf16_points=False):
    """Loss, flat parameter gradient and coarse correction ec for one pair.

    rc = R (r - A z1), ea = ||e||_A^2, ca = ||e - z1||_A^2.
    """
    rnd = bf16 if bf16_points else (lambda a: a)
    w0, ws, wout = unpack(p)
    ws = [rnd(w) for w in ws]
    W = agg_matrix(cg)
    u = np.asarray(rc, np.float64) * np.asarray(cg["dinv"], np.float64)
    s = np.sqrt(np.mean(u * u))
    x = u / s if s > 0 else np.zeros_like(u)
    ax = W @ x
    X0 = np.stack([x, ax], 1)
    Z = [X0 @ w0]
    Hs = [rnd(np.maximum(Z[0], 0))]
    Xs = []
    for l in range(3):
        Xl = np.concatenate([Hs[-1], rnd(W @ Hs[-1])], 1)
        Xs.append(Xl)
        Z.append(Xl @ ws[l])
        Hs.append(rnd(np.maximum(Z[-1], 0)))
    y = Hs[-1] @ wout
    ec = s * y
    rc = np.asarray(rc, np.float64)
    aec = coarse_operator(cg) @ ec
    num, den = ec @ rc, ec @ aec
    alpha = num / den if den > 0 else 0.0
    L = (ca - (num * num / den if den > 0 else 0.0)) / ea
    dy = s * 2 * alpha * (alpha * aec - rc) / ea
    g_wout = Hs[-1].T @ dy
    dH = np.outer(dy, wout)
    g_ws = [None] * 3
    for l in range(2, -1, -1):
        dZ = rnd(dH * (Hs[l + 1] > 0))
        g_ws[l] = Xs[l].T @ dZ
        dX = dZ @ ws[l].T
        dH = dX[:, :H] + W.T @ dX[:, H:]
    dZ0 = dH * (Hs[0] > 0)
    g_w0 = X0.T @ dZ0
    g = np.concatenate([g_w0.ravel()] + [gw.ravel() for gw in g_ws] + [g_wout])
    return L, g, ec
