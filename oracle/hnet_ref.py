"""CPU reference of the learned smoothing-length network (test use only).

Same layout as the CUDA kernels (gasoline_gb300/csrc/mlp.cu): parameters
W1[32x3] b1[32] W2[32x32] b2[32] W3[32] b3, tanh hidden layers, scalar
output, loss 0.5*mean((out - y)^2).  FP64 forward/backward in numpy, and a
central finite-difference gradient to pin the analytic one.  The network
has no counterpart in the reference.
"""
import numpy as np

H = 32
NP = H * 3 + H + H * H + H + H + 1


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    o = 0
    W1 = w[o:o + 3 * H].reshape(H, 3); o += 3 * H
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    W3 = w[o:o + H]; o += H
    b3 = w[o]
    return W1, b1, W2, b2, W3, b3


def forward(w, x):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3 + b3


def loss_grad(w, x, y):
    """Loss 0.5*mean((f(x)-y)^2) and its gradient (flat, same layout)."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    z1 = x @ W1.T + b1
    h1 = np.tanh(z1)
    z2 = h1 @ W2.T + b2
    h2 = np.tanh(z2)
    o = h2 @ W3 + b3
    d = (o - y) / n
    loss = 0.5 * np.mean((o - y) ** 2)
    gW3 = h2.T @ d
    gb3 = d.sum()
    dz2 = np.outer(d, W3) * (1 - h2 ** 2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (1 - h1 ** 2)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g


def fd_grad(w, x, y, eps=1e-6):
    w = np.asarray(w, dtype=np.float64).copy()
    g = np.zeros_like(w)
    for k in range(len(w)):
        old = w[k]
        w[k] = old + eps
        lp, _ = loss_grad(w, x, y)
        w[k] = old - eps
        lm, _ = loss_grad(w, x, y)
        w[k] = old
        g[k] = (lp - lm) / (2 * eps)
    return g
