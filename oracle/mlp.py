"""CPU restatement of the SHAKE-seeding network (TEST INFRASTRUCTURE ONLY).

The network is this build's own addition (the reference has no learned component): a 9 -> 64 ->
64 -> 3 SiLU perceptron whose parameters are one float32 blob

    W1[64][9] b1[64] W2[64][64] b2[64] W3[3][64] b3[3] | xmean[9] xinvstd[9] ymean[3] ystd[3]

The GPU kernels compute with the trained weights rounded to BF16 (round to nearest even) and
accumulate in FP32; this module computes the same function and its parameter gradient in float64
from the same BF16-rounded weights, so GPU results agree to FP32 rounding.  It also restates the
feature map and target of one 3-constraint molecule, and the SHAKE sweep of move_shake
(src/move.f90:470-515) for a single isolated molecule with the multiplier bookkeeping.
"""
from __future__ import annotations

import numpy as np

NI, NH, NO = 9, 64, 3
OW1 = 0
OB1 = OW1 + NH * NI
OW2 = OB1 + NH
OB2 = OW2 + NH * NH
OW3 = OB2 + NH
OB3 = OW3 + NO * NH
NPARAM = OB3 + NO
OXM = NPARAM
OXS = OXM + NI
OYM = OXS + NI
OYS = OYM + NO
NW = OYS + NO


def bf16_round(w: np.ndarray) -> np.ndarray:
    """float32 -> nearest-even BF16, returned as float32."""
    u = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(blob: np.ndarray):
    b = np.asarray(blob, dtype=np.float32)
    wr = b.copy()
    wr[:NPARAM] = bf16_round(b[:NPARAM])
    w = wr.astype(np.float64)
    return dict(
        W1=w[OW1:OB1].reshape(NH, NI), b1=w[OB1:OW2], W2=w[OW2:OB2].reshape(NH, NH), b2=w[OB2:OW3],
        W3=w[OW3:OB3].reshape(NO, NH), b3=w[OB3:NPARAM], xm=w[OXM:OXS], xs=w[OXS:OYM], ym=w[OYM:OYS],
        ys=w[OYS:NW])


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_d(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(blob: np.ndarray, X: np.ndarray) -> np.ndarray:
    p = unpack(blob)
    x = (np.asarray(X, np.float64) - p["xm"]) * p["xs"]
    h1 = silu(x @ p["W1"].T + p["b1"])
    h2 = silu(h1 @ p["W2"].T + p["b2"])
    y = h2 @ p["W3"].T + p["b3"]
    return y * p["ys"] + p["ym"]


def loss_grad(blob: np.ndarray, X: np.ndarray, T: np.ndarray):
    """Mean over samples of sum_c ((y_c - t_c) / ystd_c)^2 in normalised units, and its gradient
    with respect to the NPARAM trained parameters (evaluated at the BF16-rounded weights)."""
    p = unpack(blob)
    n = X.shape[0]
    x = (np.asarray(X, np.float64) - p["xm"]) * p["xs"]
    z1 = x @ p["W1"].T + p["b1"]
    h1 = silu(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = silu(z2)
    y = h2 @ p["W3"].T + p["b3"]
    tn = (np.asarray(T, np.float64) - p["ym"]) / p["ys"]
    e = y - tn
    loss = float((e * e).sum() / n)
    d3 = 2.0 * e / n
    d2 = (d3 @ p["W3"]) * silu_d(z2)
    d1 = (d2 @ p["W2"]) * silu_d(z1)
    g = np.zeros(NPARAM)
    g[OW1:OB1] = (d1.T @ x).ravel()
    g[OB1:OW2] = d1.sum(0)
    g[OW2:OB2] = (d2.T @ h1).ravel()
    g[OB2:OW3] = d2.sum(0)
    g[OW3:OB3] = (d3.T @ h2).ravel()
    g[OB3:NPARAM] = d3.sum(0)
    return loss, g


def features(p: np.ndarray, r: np.ndarray, l2: np.ndarray) -> np.ndarray:
    """Invariants of one molecule: p[c], r[c] = unconstrained / previous bond vectors of
    constraint c (3x3), l2[c] = constraint length squared."""
    f = np.zeros(9)
    for c in range(3):
        d = (c + 1) % 3
        f[c] = (l2[c] - p[c] @ p[c]) / l2[c]
        f[3 + c] = (p[c] @ r[c]) / l2[c]
        f[6 + c] = (p[c] @ r[d]) / np.sqrt(l2[c] * l2[d])
    return f


def shake_molecule(pos: np.ndarray, old: np.ndarray, pairs, l2, mii, tol2: float, maxit: int,
                   seed_y: np.ndarray | None = None):
    """SHAKE of one isolated molecule (src/move.f90:470-515 with the per-molecule stop rule;
    tol2 is the reference's 2*tol, compared against |l^2 - p^2| / l^2): returns (positions,
    sweeps, accumulated multipliers scaled by mii_a + mii_b)."""
    x = np.array(pos, np.float64)
    G = np.zeros(len(pairs))
    if seed_y is not None:
        for c, (a, b) in enumerate(pairs):
            r = old[a] - old[b]
            g = seed_y[c] / (mii[a] + mii[b])
            G[c] += g
            x[a] += r * mii[a] * g
            x[b] -= r * mii[b] * g
    moving = np.ones(len(x), bool)
    sweeps = 0
    for it in range(maxit + 1):
        moved = np.zeros(len(x), bool)
        upd = False
        for c, (a, b) in enumerate(pairs):
            if not (moving[a] or moving[b]):
                continue
            pv = x[a] - x[b]
            diff = l2[c] - pv @ pv
            if abs(diff) > l2[c] * tol2:
                r = old[a] - old[b]
                aux = diff / (2.0 * (mii[a] + mii[b]) * (r @ pv))
                G[c] += aux
                x[a] += r * mii[a] * aux
                x[b] -= r * mii[b] * aux
                moved[a] = moved[b] = True
                upd = True
        moving = moved
        sweeps = it + 1
        if not upd:
            break
    return x, sweeps, np.array([G[c] * (mii[a] + mii[b]) for c, (a, b) in enumerate(pairs)])
