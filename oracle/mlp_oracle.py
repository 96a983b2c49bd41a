"""ORACLE -- test infrastructure only.  FP64 numpy restatement of the sweep
surrogate (spp_gb300/csrc/mlp.cu): in -> 128 -> 128 -> 1 with GELU (tanh
form), weights rounded to BF16 (round to nearest even) as the kernels read
them, mean-squared-error loss and its exact gradient, and Adam (Kingma & Ba,
2015)."""
import math

import numpy as np

H = 128
C_GELU = math.sqrt(2.0 / math.pi)


def bf16(a):
    """FP32 values rounded to BF16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    rnd = ((u >> 16) & 1) + 0x7FFF
    v = ((u + rnd) & 0xFFFF0000).astype(np.uint32)
    return v.view(np.float32).astype(np.float64)


def unpack(theta, in_dim):
    o = 0
    W1 = theta[o:o + H * in_dim].reshape(H, in_dim); o += H * in_dim
    b1 = theta[o:o + H]; o += H
    W2 = theta[o:o + H * H].reshape(H, H); o += H * H
    b2 = theta[o:o + H]; o += H
    W3 = theta[o:o + H]; o += H
    b3 = theta[o]
    return W1, b1, W2, b2, W3, b3


def gelu(z):
    t = np.tanh(C_GELU * (z + 0.044715 * z ** 3))
    return 0.5 * z * (1 + t)


def dgelu(z):
    t = np.tanh(C_GELU * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * C_GELU * (1 + 3 * 0.044715 * z * z)


def forward(theta32, x):
    """theta32: FP32 masters of one member; x: [B][in]."""
    x = np.asarray(x, np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(bf16(theta32), x.shape[1])
    z1 = x @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    y = h2 @ W3 + b3
    return y, (x, z1, h1, z2, h2, W2, W3)


def loss_grad(theta32, x, t, w=None):
    """Weighted squared error sum_s w_s (y_s - t_s)^2 / sum_s w_s (w None:
    the mean) and its gradient."""
    y, (x, z1, h1, z2, h2, W2, W3) = forward(theta32, x)
    B = len(t)
    t = np.asarray(t, np.float64)
    w = np.full(B, 1.0 / B) if w is None else np.asarray(w, np.float64) / np.sum(w)
    loss = np.sum(w * (y - t) ** 2)
    dy = 2 * w * (y - t)
    gW3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = np.outer(dy, W3) * dgelu(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * dgelu(z1)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g


def adam(theta, g, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
