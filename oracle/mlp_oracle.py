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


# residue group of each code in ARNDCQEGHILKMFPSTWYVBZX*J (4 = none):
# hydrophobic AVLIMFWC, polar NQSTYGP, positive RKH, negative DE
GROUP = np.array([0, 2, 1, 3, 0, 1, 3, 1, 2, 0, 0, 2, 0, 0, 1, 1, 1, 0, 1, 0, 4, 4, 4, 4, 4],
                 dtype=np.int64)
WIN_BEFORE, WIN_LEN = 32, 64


def composition(codes, offs):
    """Fraction of each sequence's residues in the four groups (float32)."""
    codes = np.asarray(codes, dtype=np.int64)
    offs = np.asarray(offs, dtype=np.int64)
    ns = len(offs) - 1
    seq_of = np.repeat(np.arange(ns), np.diff(offs))
    counts = np.zeros((ns, 5), dtype=np.float32)
    np.add.at(counts, (seq_of, GROUP[np.minimum(codes, 24)]), 1.0)
    lens = np.diff(offs).astype(np.float32)
    inv = np.where(lens > 0, np.float32(1.0) / np.maximum(lens, 1), np.float32(0.0)).astype(np.float32)
    return counts[:, :4] * inv[:, None]


def _window(codes, ro, m, co, n, r0, c0, sm):
    s = cnt = 0
    for t in range(-WIN_BEFORE, WIN_LEN - WIN_BEFORE):
        i, j = r0 + t, c0 + t
        if i < 0 or j < 0 or i >= m or j >= n:
            continue
        s += int(sm[codes[ro + i] * 25 + codes[co + j]])
        cnt += 1
    return np.float32(s) / (np.float32(4.0) * np.float32(cnt)) if cnt else np.float32(0.0)


def features(pairs, codes, offs, sm):
    """The 16 pair features of k_features (pastis_gb300/csrc/pg_filter.cu) in
    float32, for pairs whose row and column sequences both index (codes, offs);
    returned unrounded (n x 16 float32).  Pure-Python per pair: small inputs."""
    codes = np.asarray(codes, dtype=np.int64)
    offs = np.asarray(offs, dtype=np.int64)
    comp = composition(codes, offs)
    f32 = np.float32
    out = np.zeros((len(pairs), NF), dtype=np.float32)
    for k, pr in enumerate(pairs):
        r, c = int(pr["row"]), int(pr["col"])
        m, n = int(offs[r + 1] - offs[r]), int(offs[c + 1] - offs[c])
        mm, n1 = f32(max(m, 1)), f32(max(n, 1))
        L = max(mm, n1)
        cnt = int(pr["count"])
        two = cnt >= 2
        rs0, cs0, rs1, cs1 = int(pr["rs0"]), int(pr["cs0"]), int(pr["rs1"]), int(pr["cs1"])
        d0 = (f32(cs0) - f32(rs0)) / L
        d1 = (f32(cs1) - f32(rs1)) / L
        f = out[k]
        f[0] = np.log2(f32(1.0) + f32(cnt)) * f32(0.25)
        f[1] = f32(int(pr["score"])) * f32(1.0 / 32.0)
        f[2] = 1.0 if two else 0.0
        f[3] = d0
        f[4] = d1 if two else 0.0
        f[5] = abs(d0 - d1) if two else 0.0
        f[6] = f32(rs0) / mm
        f[7] = f32(cs0) / n1
        w = _window(codes, offs[r], m, offs[c], n, rs0, cs0, sm)
        if two and (rs1 != rs0 or cs1 != cs0):
            w = max(w, _window(codes, offs[r], m, offs[c], n, rs1, cs1, sm))
        f[8] = w
        f[9] = np.log2(mm) * f32(1.0 / 12.0)
        f[10] = np.log2(n1) * f32(1.0 / 12.0)
        f[11] = abs(np.log2(mm / n1))
        f[12:16] = np.abs(comp[r] - comp[c])
    return out
