"""CPU reference of the propagator scorer's network — TEST INFRASTRUCTURE ONLY.

Only tests/ import this module, to check the device training kernels
(lala-pc_gb300/csrc/pir_sched.cu): forward, weighted binary cross-entropy with
logits and its parameter gradient, in float64, with the weights rounded to
BF16 exactly as the device rounds its FP32 master copy before use.
Parameter layout: W1[32][8], b1[32], W2[32][32], b2[32], W3[32], b3.
"""
import numpy as np

NF, NH = 8, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NF
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NPARAM = OFF_B3 + 1


def bf16_round(p):
    """FP32 -> BF16 -> FP32, round to nearest even (finite values)."""
    u = np.ascontiguousarray(p, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(NH, NF), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(NH, NH),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def forward_inference(params, X):
    """Scores as the device's inference path computes them: features,
    weights and the first hidden layer rounded to BF16, sums in float64 (the
    device accumulates in FP32, in its own order)."""
    W1, b1, W2, b2, W3, b3 = unpack(bf16_round(params))
    X = np.asarray(bf16_round(np.asarray(X, np.float32)), np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0)
    h1 = np.asarray(bf16_round(h1.astype(np.float32)), np.float64)
    h2 = np.maximum(h1 @ W2.T + b2, 0)
    return h2 @ W3 + b3


def loss_and_grad(params, X, Y, pos_weight=1.0, round_bf16=True):
    """Mean weighted BCE-with-logits over the batch and its gradient (float64)."""
    p = bf16_round(params) if round_bf16 else np.asarray(params, np.float32)
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    n = len(Y)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ W3 + b3
    w = np.where(Y > 0.5, pos_weight, 1.0)
    sp = np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z)))  # softplus(z), stable
    loss = np.sum(w * (sp - Y * z)) / n
    dz = w * (1 / (1 + np.exp(-z)) - Y) / n
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = h2.T @ dz
    g[OFF_B3] = dz.sum()
    d2 = (dz[:, None] * W3[None, :]) * (a2 > 0)
    g[OFF_W2:OFF_B2] = (d2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    g[OFF_W1:OFF_B1] = (d1.T @ X).ravel()
    g[OFF_B1:OFF_W2] = d1.sum(0)
    return loss, g


def forward(params, X):
    W1, b1, W2, b2, W3, b3 = unpack(bf16_round(params))
    h1 = np.maximum(np.asarray(X, np.float64) @ W1.T + b1, 0)
    h2 = np.maximum(h1 @ W2.T + b2, 0)
    return h2 @ W3 + b3
