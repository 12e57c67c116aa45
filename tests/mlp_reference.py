"""FP64 reference of the proposal network (42 -> 64 -> 64 -> 1, ReLU) used
to check the GPU inference and gradient kernels. The GPU computes with bf16
parameters, so the reference rounds the fp32 parameters to bf16 first."""

import numpy as np

N_IN, H = 42, 64


def bf16_round(p):
    b = np.ascontiguousarray(p, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    o = 0
    W1 = p[o:o + N_IN * H].reshape(N_IN, H); o += N_IN * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, X):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    a1 = b1 + X @ W1
    h1 = np.maximum(a1, 0)
    a2 = b2 + h1 @ W2
    h2 = np.maximum(a2, 0)
    return b3 + h2 @ w3, (a1, h1, a2, h2)


def gradient(p, X, t):
    """Gradient of 1/(2n) sum (z - t)^2 and the loss."""
    X = X.astype(np.float64)
    n = len(X)
    W1, b1, W2, b2, w3, b3 = unpack(p)
    z, (a1, h1, a2, h2) = forward(p, X)
    r = z - t
    dz = r / n
    dw3 = h2.T @ dz
    db3 = dz.sum()
    d2 = dz[:, None] * w3[None, :] * (a2 > 0)
    dW2 = h1.T @ d2
    db2 = d2.sum(0)
    d1 = (d2 @ W2.T) * (a1 > 0)
    dW1 = X.T @ d1
    db1 = d1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
    return g, 0.5 * float(np.mean(r * r))


def forward_bf16_hidden(p, X):
    """The tensor-core inference path: layer-1 activations rounded to bf16
    before layer 2 (parameters already bf16-rounded by the caller)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    h1 = bf16_round(np.maximum(b1 + X @ W1, 0).astype(np.float32))
    h2 = np.maximum(b2 + h1 @ W2, 0)
    return b3 + h2 @ w3
