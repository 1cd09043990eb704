"""The CPU reference of the pair-filter network (oracle/mlp_oracle.py): its
analytic gradients against central finite differences, in exact float64."""
import numpy as np


def test_gradients_match_finite_differences():
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(0)
    P = rng.normal(0, 0.3, M.NPARAM)
    X = rng.random((37, M.NF))
    y = (rng.random(37) < 0.4).astype(float)
    w = rng.uniform(0.5, 2.0, 37)
    loss, g = M.loss_and_grad(P, X, y, w, bf16_ops=False)
    eps = 1e-6
    idx = np.concatenate([rng.choice(np.arange(M.P_W1, M.P_B1), 12, replace=False),
                          rng.choice(np.arange(M.P_B1, M.P_W2), 6, replace=False),
                          rng.choice(np.arange(M.P_W2, M.P_B2), 20, replace=False),
                          rng.choice(np.arange(M.P_B2, M.P_W3), 6, replace=False),
                          rng.choice(np.arange(M.P_W3, M.P_B3), 6, replace=False), [M.P_B3]])
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += eps
        Pm[i] -= eps
        num = (M.loss_and_grad(Pp, X, y, w, False)[0] - M.loss_and_grad(Pm, X, y, w, False)[0]) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(num), (i, num, g[i])


def test_bf16_rounding():
    from oracle import mlp_oracle as M
    v = np.array([1.0, 1.00390625, 1.0078125, -3.14159, 65504.0, 1e-8], dtype=np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125   # ties to even
    assert abs(r[3] + 3.140625) < 1e-9
    bits = r.astype(np.float32).view(np.uint32)
    assert (bits & 0xFFFF == 0).all()


def test_feature_restatement_by_hand():
    """Two identical 40-residue sequences, seed at (5, 5): the diagonal window
    [5 - 32, 5 + 32) covers positions 0..36, so feature 8 is their mean
    self-score / 4."""
    from oracle import mlp_oracle as M
    from oracle import oracle as O
    from pastis_gb300 import capi
    sm = O.blosum62().reshape(-1)
    rng = np.random.default_rng(3)
    s = rng.integers(0, 20, 40)
    codes = np.concatenate([s, s]).astype(np.uint8)
    offs = np.array([0, 40, 80], dtype=np.uint64)
    pr = np.zeros(1, dtype=capi.PAIR_DTYPE)
    pr["row"], pr["col"], pr["rs0"], pr["cs0"], pr["count"], pr["score"] = 0, 1, 5, 5, 1, 20
    f = M.features(pr, codes, offs, sm)[0]
    self_score = sum(int(sm[a * 25 + a]) for a in s[:37])
    assert np.isclose(f[8], self_score / (4.0 * 37))
    assert f[3] == 0 and f[11] == 0 and np.all(f[12:] == 0)
    assert np.isclose(f[0], np.log2(2.0) / 4) and np.isclose(f[1], 20 / 32)
    comp = M.composition(codes, offs)
    assert np.allclose(comp.sum(axis=1), 1.0)
