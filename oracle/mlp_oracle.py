"""TEST INFRASTRUCTURE ONLY — numpy restatement of the pruning model (costal_gb300/csrc/mlp.cu).

F → 128 (ReLU) → 128 (ReLU) → 1, parameters packed as W1[128][F] b1 W2[128][128] b2 W3[128] b3,
loss = mean pinball loss at `quantile` of (y − out). Used to check the GPU forward pass and the GPU
gradient (tests/test_mlp.py). The reference has no learned part, so this oracle restates the
model's own definition (float64 arithmetic; `infer` with the inference kernel's bf16 roundings).
"""

import numpy as np

H = 128


def unpack(params, F):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]; o += 1
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def param_count(F):
    return H * F + H + H * H + H + H + 1


def forward(params, feat):
    F = feat.shape[1]
    W1, b1, W2, b2, W3, b3 = unpack(params, F)
    x = np.asarray(feat, dtype=np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    return h2 @ W3 + b3, (x, h1, h2)


def bf16(a):
    """Round to bfloat16 (nearest, ties to even), as float64: what the inference kernel's operands hold."""
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def infer(params, feat):
    """The inference kernel's arithmetic (mlp.cu k_infer): the weights of both hidden layers, the
    features and the first layer's activations rounded to bf16, products accumulated exactly (the
    kernel accumulates in FP32), biases, the output weights and the second layer's activations as given."""
    F = feat.shape[1]
    W1, b1, W2, b2, W3, b3 = unpack(params, F)
    x = bf16(feat)
    h1 = bf16(np.maximum(x @ bf16(W1).T + b1, 0.0))
    h2 = np.maximum(h1 @ bf16(W2).T + b2, 0.0)
    return h2 @ W3 + b3


def gradient(params, feat, y, quantile):
    F = feat.shape[1]
    W1, b1, W2, b2, W3, b3 = unpack(params, F)
    out, (x, h1, h2) = forward(params, feat)
    m = len(y)
    g = np.where(out > np.asarray(y, dtype=np.float64), 1.0 - quantile, -quantile) / m
    gW3 = h2.T @ g
    gb3 = g.sum()
    dz2 = (g[:, None] * W3[None, :]) * (h2 > 0)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(axis=0)
    dz1 = (dz2 @ W2) * (h1 > 0)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(axis=0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
