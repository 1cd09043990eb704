"""CPU reference of the learned pair filter (test infrastructure only).

The 16 -> 64 -> 64 -> 1 ReLU network of pastis_gb300/csrc/pg_filter.cu and
its loss (mean weighted binary cross-entropy with logits), in float64 numpy.
With ``bf16=True`` the operands of every tensor-core product are rounded to
bfloat16 where the kernels round them (weights, x, h1 before layer 2, dh2
before the backward products, dh1 before the layer-1 weight gradient), so
the GPU and this reference differ only by FP32 accumulation order.

Parameter layout (shared with the kernels): W1 [64][16] output-major, b1 [64],
W2 [64][64] output-major, b2 [64], w3 [64], b3.
"""
import numpy as np

NF, NH = 16, 64
P_W1 = 0
P_B1 = P_W1 + NH * NF
P_W2 = P_B1 + NH
P_B2 = P_W2 + NH * NH
P_W3 = P_B2 + NH
P_B3 = P_W3 + NH
NPARAM = P_B3 + 1


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    return (P[P_W1:P_B1].reshape(NH, NF), P[P_B1:P_W2], P[P_W2:P_B2].reshape(NH, NH),
            P[P_B2:P_W3], P[P_W3:P_B3], P[P_B3])


def forward(P, X, bf16_ops=True):
    r = bf16 if bf16_ops else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(P)
    X = r(X)
    a1 = X @ r(W1).T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = r(h1) @ r(W2).T + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ w3 + b3
    return z, (X, h1, h2)


def loss_and_grad(P, X, y, w, bf16_ops=True):
    r = bf16 if bf16_ops else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(P)
    n = len(y)
    z, (Xr, h1, h2) = forward(P, X, bf16_ops)
    y = np.asarray(y, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    loss = np.sum(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))) / n
    p = 1.0 / (1.0 + np.exp(-z))
    dz = w * (p - y) / n
    g = np.zeros(NPARAM)
    g[P_B3] = dz.sum()
    g[P_W3:P_B3] = h2.T @ dz
    dh2 = dz[:, None] * w3[None, :] * (h2 > 0)
    g[P_B2:P_W3] = dh2.sum(0)
    g[P_W2:P_B2] = (r(dh2).T @ r(h1)).ravel()
    dh1 = (r(dh2) @ r(W2)) * (h1 > 0)
    g[P_B1:P_W2] = dh1.sum(0)
    g[P_W1:P_B1] = (r(dh1).T @ Xr).ravel()
    return loss, g
