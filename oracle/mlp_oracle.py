"""CPU oracle of the warm-start MLP (TEST INFRASTRUCTURE ONLY).

FP64 numpy restatement of the network the library trains (din -> 128 -> 128 -> 128 -> dout,
SiLU) and of its weighted-MSE gradient, evaluated with the BF16-rounded weights the GPU
forward pass uses.  The reference has no learned component; this checks the hand-written
CUDA forward / backward kernels.  Parameter layout: W0 (128 x din), b0, W1 (128 x 128), b1,
W2 (128 x 128), b2, W3 (dout x 128), b3, row-major, concatenated.
"""
import numpy as np

WIDTH = 128


def unpack(p, din, dout):
    o = 0
    out = []
    for shape in ((WIDTH, din), (WIDTH,), (WIDTH, WIDTH), (WIDTH,), (WIDTH, WIDTH), (WIDTH,), (dout, WIDTH), (dout,)):
        n = int(np.prod(shape))
        out.append(np.asarray(p[o:o + n], dtype=np.float64).reshape(shape))
        o += n
    return out


def silu(x):
    return x / (1 + np.exp(-x))


def dsilu(x):
    s = 1 / (1 + np.exp(-x))
    return s * (1 + x * (1 - s))


def forward(p, X, din, dout):
    W0, b0, W1, b1, W2, b2, W3, b3 = unpack(p, din, dout)
    z0 = X @ W0.T + b0
    z1 = silu(z0) @ W1.T + b1
    z2 = silu(z1) @ W2.T + b2
    y = silu(z2) @ W3.T + b3
    return y, (z0, z1, z2)


def loss_and_grad(p, X, T, wt, din, dout):
    X = np.asarray(X, np.float64)
    W0, b0, W1, b1, W2, b2, W3, b3 = unpack(p, din, dout)
    y, (z0, z1, z2) = forward(p, X, din, dout)
    n = X.shape[0]
    r = y - T
    loss = float(np.sum(wt * r * r) / n)
    dy = 2 * wt * r / n
    a2 = silu(z2)
    gW3 = dy.T @ a2
    gb3 = dy.sum(0)
    g2 = (dy @ W3) * dsilu(z2)
    a1 = silu(z1)
    gW2 = g2.T @ a1
    gb2 = g2.sum(0)
    g1 = (g2 @ W2) * dsilu(z1)
    a0 = silu(z0)
    gW1 = g1.T @ a0
    gb1 = g1.sum(0)
    g0 = (g1 @ W1) * dsilu(z0)
    gW0 = g0.T @ X
    gb0 = g0.sum(0)
    grad = np.concatenate([a.ravel() for a in (gW0, gb0, gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, grad
