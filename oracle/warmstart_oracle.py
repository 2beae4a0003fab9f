"""CPU oracle of the learned warm start (features, MLP loss and gradient).

TEST INFRASTRUCTURE ONLY: imported by tests/ to check the library's CUDA
kernels (gputucker_gb300/csrc/warmstart.cu); never on the product path.  The
warm start has no reference counterpart (GPUTucker always starts from uniform
[0,1) draws, tucker.cuh:84-97), so this restates the library's own definitions
in float64 numpy:

  features of row i of mode n: log(1+c_i), mean and std of its values; for each
  other mode m (increasing), over the row's nonzeros: mean and std of mu_m[i_m]
  (the mean value of the co-indexed row of mode m), mean of lc_m = log(1+c_m[i_m]),
  and the cross moments E[x mu_m], E[x mu_m^2], E[x lc_m]; E[x prod_m mu_m];
  one-hot of n.
  network: y = W3 relu(W2 relu(W1 x + b1) + b2) + b3; loss = mean (y - t)^2.
"""

from __future__ import annotations

import numpy as np


def row_features(idx, vals, rows, mode):
    """Raw features of every row [0, rows[mode]) of `mode` (float64), F = 4 + 6(N-1) + N."""
    N = len(idx)
    vals = np.asarray(vals, np.float64)
    mu, lc = [], []
    for m in range(N):
        c = np.bincount(idx[m], minlength=rows[m]).astype(np.float64)
        s = np.bincount(idx[m], weights=vals, minlength=rows[m])
        mu.append(np.divide(s, c, out=np.zeros_like(s), where=c > 0))
        lc.append(np.log1p(c))
    n = mode
    R = rows[n]
    c = np.bincount(idx[n], minlength=R).astype(np.float64)
    inv = np.divide(1.0, c, out=np.zeros_like(c), where=c > 0)

    def row_mean(w):
        return np.bincount(idx[n], weights=w, minlength=R) * inv

    mean = row_mean(vals)
    D = N - 1
    F = 4 + 6 * D + N
    out = np.zeros((R, F))
    out[:, 0] = np.log1p(c)
    out[:, 1] = mean
    out[:, 2] = np.sqrt(np.maximum(0.0, row_mean(vals * vals) - mean * mean))
    prod = vals.copy()
    d = 0
    for m in range(N):
        if m == n:
            continue
        a = mu[m][idx[m]]
        b = lc[m][idx[m]]
        am = row_mean(a)
        out[:, 3 + 6 * d] = am
        out[:, 4 + 6 * d] = np.sqrt(np.maximum(0.0, row_mean(a * a) - am * am))
        out[:, 5 + 6 * d] = row_mean(b)
        out[:, 6 + 6 * d] = row_mean(vals * a)
        out[:, 7 + 6 * d] = row_mean(vals * a * a)
        out[:, 8 + 6 * d] = row_mean(vals * b)
        prod = prod * a
        d += 1
    out[:, 3 + 6 * D] = row_mean(prod)
    out[:, 4 + 6 * D + n] = 1.0
    return out


def unpack(params, F, H, J):
    p = np.asarray(params, np.float64)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + J * H].reshape(J, H); o += J * H
    b3 = p[o:o + J]; o += J
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def forward(params, x, F, H, J):
    W1, b1, W2, b2, W3, b3 = unpack(params, F, H, J)
    x = np.asarray(x, np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    return h2 @ W3.T + b3, (x, z1, h1, z2, h2)


def loss_grad(params, x, t, F, H, J):
    """Loss = mean over batch and outputs of (y - t)^2 and its flat gradient."""
    W1, b1, W2, b2, W3, b3 = unpack(params, F, H, J)
    y, (x, z1, h1, z2, h2) = forward(params, x, F, H, J)
    t = np.asarray(t, np.float64)
    n = y.size
    loss = float(np.sum((y - t) ** 2) / n)
    dy = 2.0 * (y - t) / n
    gW3 = dy.T @ h2
    gb3 = dy.sum(0)
    d2 = (dy @ W3) * (z2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (z1 > 0)
    gW1 = d1.T @ x
    gb1 = d1.sum(0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
