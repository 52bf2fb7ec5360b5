"""CPU oracle of libdegpu's step-size MLP (numpy, float64 accumulation) -- TEST
INFRASTRUCTURE ONLY: forward and backward with the same bf16 rounding points as the
kernels (inputs, weights and hidden activations rounded to bfloat16; straight-through
gradients), used to check the GPU gradients and the tensor-core inference."""
import numpy as np

H = 64


def bf16(x):
    """Round float32 to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def unpack(P, n_in):
    o = 0
    W1 = P[o:o + H * n_in].reshape(H, n_in); o += H * n_in
    b1 = P[o:o + H]; o += H
    W2 = P[o:o + H * H].reshape(H, H); o += H * H
    b2 = P[o:o + H]; o += H
    W3 = P[o:o + 2 * H].reshape(2, H); o += 2 * H
    b3 = P[o:o + 2]
    return W1, b1, W2, b2, W3, b3


def sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(P, mean, std, x):
    n_in = x.shape[1]
    W1, b1, W2, b2, W3, b3 = [a.astype(np.float64) for a in unpack(P, n_in)]
    W1q, W2q, W3q = (bf16(W).astype(np.float64) for W in (W1, W2, W3))
    xn = bf16(((x - mean) * (1.0 / std)).astype(np.float32)).astype(np.float64)
    z1 = xn @ W1q.T + b1
    h1 = bf16((z1 * sig(z1)).astype(np.float32)).astype(np.float64)
    z2 = h1 @ W2q.T + b2
    h2 = bf16((z2 * sig(z2)).astype(np.float32)).astype(np.float64)
    y = h2 @ W3q.T + b3
    return y, (xn, z1, h1, z2, h2, W1q, W2q, W3q)


def grad(P, mean, std, x, t, w=None):
    """Mean over the batch of sum_o w (y - t)^2 and its gradient w.r.t. the packed params."""
    n_in = x.shape[1]
    B = x.shape[0]
    y, (xn, z1, h1, z2, h2, W1q, W2q, W3q) = forward(P, mean, std, x)
    w = np.ones_like(y) if w is None else w
    r = y - t
    loss = (w * r * r).sum() / B
    dy = 2 * w * r / B
    ds = lambda z: sig(z) + z * sig(z) * (1 - sig(z))
    dW3 = dy.T @ h2
    db3 = dy.sum(0)
    dz2 = (dy @ W3q) * ds(z2)
    dW2 = dz2.T @ h1
    db2 = dz2.sum(0)
    dz1 = (dz2 @ W2q) * ds(z1)
    dW1 = dz1.T @ xn
    db1 = dz1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return loss, g
