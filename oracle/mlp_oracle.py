"""FP64 NumPy restatement of the creep surrogate network and its gradient.

TEST INFRASTRUCTURE ONLY: the GPU training kernels' gradients are checked against this,
and this against central finite differences.  Same architecture and parameter layout as the
library (4 -> 64 -> 64 -> 1, SiLU, loss = mean (y - t)^2 with t = (log10 s - mu) / sigma).
With w2_bf16 the hidden layer's weights W2 enter as the library holds them, rounded to BF16
(round to nearest even), and the gradient is the library's quantization-aware one: forward and
backward with the rounded W2, the W2 gradient taken for the FP32 master (straight-through)."""
import numpy as np

H = 64
OFF_W1, OFF_B1 = 0, 256
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
OFF_NORM = OFF_B3 + 1
N_PARAMS = OFF_NORM + 2
N_TRAIN = OFF_NORM


def bf16_round(x):
    """FP32 values rounded to BF16 (round to nearest even on the top 16 bits), as float64"""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def unpack(p, w2_bf16=False):
    p = np.asarray(p, dtype=np.float64)
    W2 = p[OFF_W2:OFF_B2]
    if w2_bf16:
        W2 = bf16_round(W2.astype(np.float32))
    return (p[OFF_W1:OFF_B1].reshape(H, 4), p[OFF_B1:OFF_W2], W2.reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3], p[OFF_NORM], p[OFF_NORM + 1])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X, w2_bf16=False):
    W1, b1, W2, b2, w3, b3, _, _ = unpack(p, w2_bf16)
    z1 = X @ W1.T + b1
    h1 = silu(z1)
    z2 = h1 @ W2.T + b2
    h2 = silu(z2)
    return h2 @ w3 + b3, (z1, h1, z2, h2)


def loss_and_grad(p, X, target, w2_bf16=False):
    X = np.asarray(X, dtype=np.float64)
    W1, b1, W2, b2, w3, b3, mu, sig = unpack(p, w2_bf16)
    t = (np.asarray(target, dtype=np.float64) - mu) / sig
    y, (z1, h1, z2, h2) = forward(p, X, w2_bf16)
    n = len(t)
    err = y - t
    loss = np.mean(err ** 2)
    dy = 2.0 * err / n
    g = np.zeros(N_TRAIN)
    g[OFF_W3:OFF_B3] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    dz2 = (dy[:, None] * w3[None, :]) * dsilu(z2)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2) * dsilu(z1)
    g[OFF_W1:OFF_B1] = (dz1.T @ X).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g


def loss_only(p, X, target):
    W1, b1, W2, b2, w3, b3, mu, sig = unpack(p)
    t = (np.asarray(target, dtype=np.float64) - mu) / sig
    y, _ = forward(p, X)
    return np.mean((y - t) ** 2)
