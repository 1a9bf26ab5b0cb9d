"""CPU reference of the learned initial guess's network (test infrastructure only).

numpy restatement of the forward pass, loss and gradients that the tcgen05 kernels of
cpfft_gb300/csrc/mlp.cu compute, with the same BF16 rounding points: the normalised
inputs, the activations and the backward products' left operands are rounded to BF16
(round to nearest even), weights are the BF16 copies of the FP32 master parameters, and
every product is accumulated in FP64 here (FP32 on the GPU).  Parameter layout: the
packed FP32 vector of mlp.cuh (W1 [128][32], b1, W2 [128][128], b2, W3 [16][128], b3).

Only tests/ import this module.
"""
import numpy as np

NIN, NOUT, KIN, NH, NO = 20, 7, 32, 128, 16
P_W1 = 0
P_B1 = P_W1 + NH * KIN
P_W2 = P_B1 + NH
P_B2 = P_W2 + NH * NH
P_W3 = P_B2 + NH
P_B3 = P_W3 + NO * NH
P_TOTAL = P_B3 + NO
N_NORM = 2 * NIN + 2 * NOUT


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[P_W1:P_B1].reshape(NH, KIN), p[P_B1:P_W2], p[P_W2:P_B2].reshape(NH, NH),
            p[P_B2:P_W3], p[P_W3:P_B3].reshape(NO, NH), p[P_B3:P_TOTAL])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def exact(x):
    """No rounding (the FP64 network, for finite-difference checks of the gradient)."""
    return np.asarray(x, dtype=np.float64)


def normalise(X, norm, rnd=bf16):
    x = np.zeros((X.shape[0], KIN))
    x[:, :NIN] = (X - norm[:NIN]) * norm[NIN:2 * NIN]
    return rnd(x)


def forward(p, norm, X, rnd=bf16):
    """Raw features X (n, 20) -> raw outputs (n, 7) and the intermediates."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    W1, W2, W3 = rnd(W1), rnd(W2), rnd(W3)
    x = normalise(np.asarray(X, dtype=np.float64), norm, rnd)
    z1 = x @ W1.T + b1
    a1 = rnd(silu(z1))
    z2 = a1 @ W2.T + b2
    a2 = rnd(silu(z2))
    y = a2 @ W3.T + b3
    out = y[:, :NOUT] * norm[2 * NIN + NOUT:] + norm[2 * NIN:2 * NIN + NOUT]
    return out, (x, z1, a1, z2, a2, y)


def loss_grad(p, norm, X, T, rnd=bf16):
    """Mean squared error in normalised output units and its gradient (P_TOTAL)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    W2b, W3b = rnd(W2), rnd(W3)
    _, (x, z1, a1, z2, a2, y) = forward(p, norm, X, rnd)
    n = x.shape[0]
    t = (np.asarray(T, dtype=np.float64) - norm[2 * NIN:2 * NIN + NOUT]) / norm[2 * NIN + NOUT:]
    d = np.zeros((n, NO))
    d[:, :NOUT] = y[:, :NOUT] - t
    loss = (d ** 2).sum() / (n * NOUT)
    dy = rnd(2.0 * d / (n * NOUT))
    g = np.zeros(P_TOTAL)
    g[P_B3:P_TOTAL] = (2.0 * d / (n * NOUT)).sum(axis=0)
    g[P_W3:P_B3] = (dy.T @ a2).ravel()
    dz2 = (dy @ W3b) * dsilu(z2)
    g[P_B2:P_W3] = dz2.sum(axis=0)
    dz2b = rnd(dz2)
    g[P_W2:P_B2] = (dz2b.T @ a1).ravel()
    dz1 = (dz2b @ W2b) * dsilu(z1)
    g[P_B1:P_W2] = dz1.sum(axis=0)
    g[P_W1:P_B1] = (rnd(dz1).T @ x).ravel()
    return loss, g
