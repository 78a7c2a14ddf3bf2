"""CPU FP64 restatement of the learned preconditioner's message-passing network.

TEST INFRASTRUCTURE ONLY: the CUDA kernels (nonlocal_gb300/csrc/mpnn.cu) are
checked against this module; nothing in the product imports it.

The network has no counterpart in the reference (it is one of the added
patterns around the reference's CG + ILLT path): a 4-layer message-passing
net over the graph of the local stiffness pattern, acting as a correction
on top of the ILLT preconditioner inside flexible CG:

    A_hat   = D^-1/2 |offdiag(K_local)| D^-1/2   (symmetric, zero diagonal)
    X0      = [r / rms(r), z / rms(z)]            z = ILLT^-1 r        (n x 2)
    U_0     = [X0, A_hat X0]                                           (n x 4)
    H_1     = tanh(U_0 W_1)                       W_1: 4 x 64
    U_l     = [H_l, A_hat H_l]                                         (n x 128)
    H_l+1   = tanh(U_l W_l+1)                     W_2, W_3: 128 x 64
    y       = U_3 w_4                             w_4: 128 x 1
    P(r)    = z + rms(z) y

No biases and an odd activation make the correction odd and, through the
input normalisation, homogeneous of degree 1 in r.  Training minimises the
relative energy-norm error of P(r) against the exact error e = A^-1 r:

    L = (P(r) - e)^T A (P(r) - e) / (e^T A e)
"""
from __future__ import annotations

import numpy as np

HIDDEN = 64
SHAPES = {"w1": (4, HIDDEN), "w2": (2 * HIDDEN, HIDDEN), "w3": (2 * HIDDEN, HIDDEN), "w4": (2 * HIDDEN, 1)}


def normalized_adjacency(rowptr, col, val, n):
    """Dense-free CSR of A_hat from an upper-stored symmetric matrix (scipy-free)."""
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    diag = np.zeros(n)
    on = col == rows
    diag[rows[on]] = np.abs(val[on])
    off = ~on
    r, c, v = rows[off], col[off], np.abs(val[off])
    d = np.where(diag > 0, diag, 1.0)
    w = v / np.sqrt(d[r] * d[c])
    rr = np.concatenate([r, c])
    cc = np.concatenate([c, r])
    ww = np.concatenate([w, w])
    order = np.lexsort((cc, rr))
    rr, cc, ww = rr[order], cc[order], ww[order]
    rp = np.concatenate([[0], np.cumsum(np.bincount(rr, minlength=n))])
    return rp, cc, ww


def spmm(adj, x):
    rp, c, w = adj
    out = np.zeros_like(x)
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    np.add.at(out, rows, w[:, None] * x[c] if x.ndim == 2 else w * x[c])
    return out


def init_weights(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    out = {}
    for k, (fi, fo) in SHAPES.items():
        out[k] = rng.standard_normal((fi, fo)) * scale * np.sqrt(1.0 / fi)
    out["w4"] *= 0.1
    return out


def rms(v):
    return float(np.sqrt(np.mean(v * v)))


def forward(adj, r, z, W):
    """Returns P(r) and the cache for backward."""
    sr, sz = rms(r), rms(z)
    x0 = np.stack([r / sr, z / sz], axis=1)
    u0 = np.concatenate([x0, spmm(adj, x0)], axis=1)
    h1 = np.tanh(u0 @ W["w1"])
    u1 = np.concatenate([h1, spmm(adj, h1)], axis=1)
    h2 = np.tanh(u1 @ W["w2"])
    u2 = np.concatenate([h2, spmm(adj, h2)], axis=1)
    h3 = np.tanh(u2 @ W["w3"])
    u3 = np.concatenate([h3, spmm(adj, h3)], axis=1)
    y = (u3 @ W["w4"])[:, 0]
    cache = dict(u0=u0, h1=h1, u1=u1, h2=h2, u2=u2, h3=h3, u3=u3, sz=sz)
    return z + sz * y, cache


def loss_and_grad(adj, a_mul, r, z, e, W):
    """Relative energy-norm loss and its gradient with respect to every weight.
    a_mul(v) = A v (the nonlocal system matrix)."""
    p, c = forward(adj, r, z, W)
    d = p - e
    ad = a_mul(d)
    ee = float(e @ a_mul(e))
    loss = float(d @ ad) / ee
    gy = (2.0 / ee) * ad * c["sz"]                  # dL/dy
    g = {}
    g["w4"] = c["u3"].T @ gy[:, None]
    du = gy[:, None] @ W["w4"].T                    # n x 128
    dh = du[:, :HIDDEN] + spmm(adj, du[:, HIDDEN:])
    for l, (u, h) in ((3, (c["u2"], c["h3"])), (2, (c["u1"], c["h2"])), (1, (c["u0"], c["h1"]))):
        dp = dh * (1.0 - h * h)
        g[f"w{l}"] = u.T @ dp
        if l > 1:
            du = dp @ W[f"w{l}"].T
            dh = du[:, :HIDDEN] + spmm(adj, du[:, HIDDEN:])
    return loss, g
