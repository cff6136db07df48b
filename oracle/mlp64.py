"""FP64 numpy restatement of the tuner MLP (TEST INFRASTRUCTURE ONLY).

The network of gromacs-fmm_gb300/csrc/tuner.cu: x -> tanh(W1 x + b1) ->
tanh(W2 . + b2) -> W3 . + b3, parameters laid out W1 b1 W2 b2 W3 b3 (row-major
W[out][in]), loss = mean over rows of sum_j (y - t)^2.  The tests compare the
GPU kernels' forward pass and gradients with this one.
"""
import numpy as np


def unpack(p, I, H, O):
    p = np.asarray(p, np.float64)
    k = 0
    W1 = p[k:k + H * I].reshape(H, I); k += H * I
    b1 = p[k:k + H]; k += H
    W2 = p[k:k + H * H].reshape(H, H); k += H * H
    b2 = p[k:k + H]; k += H
    W3 = p[k:k + O * H].reshape(O, H); k += O * H
    b3 = p[k:k + O]
    return W1, b1, W2, b2, W3, b3


def forward(p, x, I, H, O):
    W1, b1, W2, b2, W3, b3 = unpack(p, I, H, O)
    x = np.asarray(x, np.float64)
    a1 = np.tanh(x @ W1.T + b1)
    a2 = np.tanh(a1 @ W2.T + b2)
    return a2 @ W3.T + b3


def loss_grad(p, x, t, I, H, O):
    W1, b1, W2, b2, W3, b3 = unpack(p, I, H, O)
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    B = len(x)
    z1 = x @ W1.T + b1
    a1 = np.tanh(z1)
    z2 = a1 @ W2.T + b2
    a2 = np.tanh(z2)
    y = a2 @ W3.T + b3
    loss = np.sum((y - t) ** 2) / B
    dy = 2 * (y - t) / B
    gW3 = dy.T @ a2
    gb3 = dy.sum(0)
    d2 = (dy @ W3) * (1 - a2 ** 2)
    gW2 = d2.T @ a1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (1 - a1 ** 2)
    gW1 = d1.T @ x
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
