"""TEST INFRASTRUCTURE ONLY: CPU FP64 oracle of the learned CG warm start.

The reference has no learned component; this restates the network the GPU
kernels implement so their forward pass, gradients and Adam steps can be
checked:

    x  = (f - f_mean) / f_std                      8 features
    z1 = W1 x + b1,  h1 = silu(z1)                 64
    z2 = W2 h1 + b2, h2 = silu(z2)                 64
    y  = w3 . h2 + b3
    t  = t_mean + t_std * y                         prediction of the target

silu(z) = z / (1 + exp(-z)) (Elfwing et al. 2018); Adam as in Kingma & Ba
(2015) with bias correction.  `bf16=True` rounds x, W1, h1 and W2 to bfloat16
(round to nearest even) where the tensor-core path does, so the GPU forward can
be compared with a tight tolerance.

Parameter vector layout (float32, length 4801):
    W1[64][8], b1[64], W2[64][64], b2[64], w3[64], b3
Normalisation vector (length 18): f_mean[8], f_std[8], t_mean, t_std.
"""
from __future__ import annotations

import numpy as np

N_IN, N_H = 8, 64
N_PARAMS = N_H * N_IN + N_H + N_H * N_H + N_H + N_H + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_H * N_IN].reshape(N_H, N_IN); o += N_H * N_IN
    b1 = p[o:o + N_H]; o += N_H
    W2 = p[o:o + N_H * N_H].reshape(N_H, N_H); o += N_H * N_H
    b2 = p[o:o + N_H]; o += N_H
    w3 = p[o:o + N_H]; o += N_H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def pack(W1, b1, W2, b2, w3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]]).astype(np.float64)


def bf16_round(a):
    """Round float64/float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / N_IN), size=(N_H, N_IN))
    W2 = rng.normal(0, np.sqrt(2.0 / N_H), size=(N_H, N_H))
    w3 = rng.normal(0, np.sqrt(1.0 / N_H), size=N_H) * 0.1
    return pack(W1, np.zeros(N_H), W2, np.zeros(N_H), w3, 0.0)


def forward(params, norm, feats, bf16=False, cache=False):
    W1, b1, W2, b2, w3, b3 = unpack(params)
    norm = np.asarray(norm, dtype=np.float64)
    x = (np.asarray(feats, dtype=np.float64) - norm[:N_IN]) / norm[N_IN:2 * N_IN]
    if bf16:
        x, W1, W2 = bf16_round(x), bf16_round(W1), bf16_round(W2)
    z1 = x @ W1.T + b1
    h1 = silu(z1)
    if bf16:
        h1 = bf16_round(h1)
    z2 = h1 @ W2.T + b2
    h2 = silu(z2)
    y = h2 @ w3 + b3
    t = norm[2 * N_IN] + norm[2 * N_IN + 1] * y
    if cache:
        return t, (x, z1, h1, z2, h2, y)
    return t


def loss_and_grad(params, norm, feats, target, bf16=False):
    """Mean squared error on the normalised output y (target -> (t - t_mean) / t_std)
    and its gradient.  `bf16=True` rounds where the tensor-core gradient pass
    does: x, W1, W2, h1 (operands of the forward products and of dW2 / dW1),
    dz2 (operand of dz1 = dz2 W2 and of dW2) and dz1 (operand of dW1); the
    rest (biases, silu, the final layer, dy, sums) stays exact."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    norm = np.asarray(norm, dtype=np.float64)
    x = (np.asarray(feats, dtype=np.float64) - norm[:N_IN]) / norm[N_IN:2 * N_IN]
    r = bf16_round if bf16 else (lambda a: a)
    x, W1r, W2r = r(x), r(W1), r(W2)
    z1 = x @ W1r.T + b1
    h1 = r(silu(z1))
    z2 = h1 @ W2r.T + b2
    h2 = silu(z2)
    y = h2 @ w3 + b3
    ty = (np.asarray(target, dtype=np.float64) - norm[2 * N_IN]) / norm[2 * N_IN + 1]
    n = y.shape[0]
    e = y - ty
    loss = float(np.mean(e * e))
    dy = 2.0 * e / n
    gw3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = r(np.outer(dy, w3) * dsilu(z2))
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = r((dz2 @ W2r) * dsilu(z1))
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    return loss, pack(gW1, gb1, gW2, gb2, gw3, gb3)


def param_groups():
    """Slices of the parameter vector: W1, b1, W2, b2, w3, b3."""
    o, out = 0, {}
    for name, size in (("W1", N_H * N_IN), ("b1", N_H), ("W2", N_H * N_H), ("b2", N_H), ("w3", N_H), ("b3", 1)):
        out[name] = slice(o, o + size)
        o += size
    return out


class Adam:
    def __init__(self, params, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.p = np.asarray(params, dtype=np.float64).copy()
        self.m = np.zeros_like(self.p)
        self.v = np.zeros_like(self.p)
        self.t = 0
        self.lr, self.b1, self.b2, self.eps = lr, b1, b2, eps

    def step(self, g):
        self.t += 1
        self.m = self.b1 * self.m + (1 - self.b1) * g
        self.v = self.b2 * self.v + (1 - self.b2) * g * g
        mh = self.m / (1 - self.b1**self.t)
        vh = self.v / (1 - self.b2**self.t)
        self.p = self.p - self.lr * mh / (np.sqrt(vh) + self.eps)
        return self.p
