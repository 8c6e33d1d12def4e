"""CPU restatement of the learned branching scorer (test infrastructure only).

numpy in float64: the 16 -> 128 -> 128 -> 1 ReLU network, the weighted
binary cross-entropy on its logit and the gradient of that loss by the chain
rule, written out layer by layer.  It checks the engine's GPU training
kernels (scs_mlp_grad) and, with the BF16 rounding emulated, its tensor-core
inference (scs_mlp_infer).  The scorer has no counterpart in the reference,
so this restatement is pinned against finite differences, not against
reference outputs.

Parameter vector layout (as the model file): W1[16][128], b1[128],
W2[128][128], b2[128], W3[128], b3 -- W[in][out].
"""
import numpy as np

N_IN, N_H = 16, 128
NPARAM = N_IN * N_H + N_H + N_H * N_H + N_H + N_H + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    i = 0
    W1 = p[i:i + N_IN * N_H].reshape(N_IN, N_H); i += N_IN * N_H
    b1 = p[i:i + N_H]; i += N_H
    W2 = p[i:i + N_H * N_H].reshape(N_H, N_H); i += N_H * N_H
    b2 = p[i:i + N_H]; i += N_H
    W3 = p[i:i + N_H]; i += N_H
    b3 = p[i]
    return W1, b1, W2, b2, W3, b3


def init_params(seed=0):
    """He-uniform weights, zero biases (float32)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((N_IN, N_H), (N_H, N_H), (N_H, 1)):
        lim = np.sqrt(6.0 / fan_in)
        parts.append(rng.uniform(-lim, lim, size=fan_in * fan_out))
        parts.append(np.zeros(fan_out))
    return np.concatenate(parts).astype(np.float32)


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return h2 @ W3 + b3


def loss_grad(p, X, y, w=None):
    """Weighted mean BCE-with-logits and its gradient (float64)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    w = np.ones(len(y)) if w is None else np.asarray(w, dtype=np.float64)
    a1 = X @ W1 + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ W3 + b3
    ws = w.sum()
    sp = np.where(z > 0, z + np.log1p(np.exp(-z)), np.log1p(np.exp(z)))
    loss = float((w * (sp - y * z)).sum() / ws)
    dz = w * (1.0 / (1.0 + np.exp(-z)) - y) / ws
    gW3 = h2.T @ dz
    gb3 = dz.sum()
    d2 = np.outer(dz, W3) * (a2 > 0)
    gW2 = h1.T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ W2.T) * (a1 > 0)
    gW1 = X.T @ d1
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def forward_bf16(p, X):
    """The tensor-core inference as arithmetic: inputs, weights and hidden
    activations rounded to bf16, products summed in float64 (the device sums
    in FP32), biases in float32."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, dtype=np.float32))
    X = bf16(np.asarray(X, dtype=np.float32)).astype(np.float64)
    h1 = bf16(np.maximum(X @ bf16(W1).astype(np.float64) + b1, 0.0).astype(np.float32))
    h2 = bf16(np.maximum(h1.astype(np.float64) @ bf16(W2).astype(np.float64) + b2,
                         0.0).astype(np.float32))
    return h2.astype(np.float64) @ bf16(W3).astype(np.float64) + b3
