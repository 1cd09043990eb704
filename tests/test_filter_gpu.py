"""The learned pair filter on the GPU: tensor-core forward and backward kernels
against the CPU reference (oracle/mlp_oracle.py, same bf16 rounding points),
training, the filtered alignment path, and what the trained network gains
over PASTIS's own k-mer prune."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev_features(X):
    import torch
    from oracle import mlp_oracle as M
    Xb = torch.from_numpy(np.asarray(X, dtype=np.float32)).to("cuda:0").to(torch.bfloat16).contiguous()
    return Xb, M.bf16(Xb.float().cpu().numpy())


def test_forward_and_gradients_match_reference(native):
    import torch
    from oracle import mlp_oracle as M
    from pastis_gb300.filter import Filter
    rng = np.random.default_rng(1)
    n = 1000
    f = Filter(0, seed=3)
    P = rng.normal(0, 0.25, M.NPARAM).astype(np.float32)
    f.set_params(P)
    Xb, Xr = _dev_features(rng.random((n, M.NF)) * 2 - 0.5)
    y = (rng.random(n) < 0.3).astype(np.float32)
    w = rng.uniform(0.5, 3.0, n).astype(np.float32)
    z = torch.empty(n, dtype=torch.float32, device="cuda:0")
    f.predict(Xb.data_ptr(), n, z.data_ptr())
    torch.cuda.synchronize()
    z_ref, _ = M.forward(P, Xr, bf16_ops=True)
    assert np.allclose(z.cpu().numpy(), z_ref, rtol=2e-3, atol=2e-3)
    yd = torch.from_numpy(y).cuda()
    wd = torch.from_numpy(w).cuda()
    g, loss = f.gradients(Xb.data_ptr(), yd.data_ptr(), wd.data_ptr(), n)
    loss_ref, g_ref = M.loss_and_grad(P, Xr, y, w, bf16_ops=True)
    assert abs(loss - loss_ref) <= 1e-3 * max(1.0, abs(loss_ref))
    for name, a, b in (("W1", M.P_W1, M.P_B1), ("b1", M.P_B1, M.P_W2), ("W2", M.P_W2, M.P_B2),
                       ("b2", M.P_B2, M.P_W3), ("w3", M.P_W3, M.P_B3), ("b3", M.P_B3, M.NPARAM)):
        gg, rr = g[a:b], g_ref[a:b]
        # the kernels and the reference share every bf16 rounding point; what
        # remains is the order of float32 sums (measured: about 1e-7 of the
        # largest gradient), so an indexing slip on any weight shows here
        err = np.abs(gg - rr).max() / (np.abs(rr).max() + 1e-12)
        assert err < 1e-5, (name, err)
    f.close()


def test_training_reduces_loss(native):
    import torch
    from pastis_gb300.filter import Filter
    rng = np.random.default_rng(2)
    n = 20000
    X = rng.random((n, 16)).astype(np.float32)
    y = ((X[:, 3] - 0.5) ** 2 + (X[:, 8] - 0.5) ** 2 < 0.12).astype(np.float32)  # nonlinear target
    Xb, _ = _dev_features(X)
    yd = torch.from_numpy(y).cuda()
    wd = torch.ones(n, device="cuda:0")
    f = Filter(0, seed=5)
    first = f.train_step(Xb.data_ptr(), yd.data_ptr(), wd.data_ptr(), n, 3e-3)
    for _ in range(300):
        last = f.train_step(Xb.data_ptr(), yd.data_ptr(), wd.data_ptr(), n, 3e-3)
    assert last < 0.6 * first
    z = torch.empty(n, device="cuda:0")
    f.predict(Xb.data_ptr(), n, z.data_ptr())
    acc = ((z.cpu().numpy() > 0) == (y > 0.5)).mean()
    assert acc > 0.9
    f.close()


def test_filtered_alignment_contract(native):
    import torch
    from pastis_gb300 import capi, synth
    from pastis_gb300.filter import Filter
    w = synth.generate("xdrop1m", seed=12, scale=0.002)
    ctx = capi.Context(capi.config(capi.MODE_XDROP))
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    plain = ctx.align(w.pairs)
    n = len(w.pairs)
    d_pairs = torch.from_numpy(w.pairs.view(np.uint8).copy()).cuda()
    d_out = torch.empty(n * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda:0")
    f = Filter(0, seed=1)
    kept = f.align_filtered(ctx, -float("inf"), d_pairs.data_ptr(), n, d_out.data_ptr())
    torch.cuda.synchronize()
    assert kept == n
    got = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    assert got.tobytes() == plain.tobytes()       # nothing pruned: identical to the plain aligner
    kept = f.align_filtered(ctx, float("inf"), d_pairs.data_ptr(), n, d_out.data_ptr())
    torch.cuda.synchronize()
    got = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    assert kept == 0 and (got["flags"] & capi.RF_FILTERED).all() and (got["score_aln"] == 0).all()
    f.close()
    ctx.close()


def test_trained_filter_beats_kmer_prune(native):
    """Train on labels from this library's SW kernel; at >= 99.5 % recall of
    the held-out positives the network keeps fewer candidates than the best
    count or k-mer-score threshold (PASTIS's own prune) at the same recall."""
    import torch
    from pastis_gb300 import capi, synth
    from pastis_gb300 import filter as F
    w = synth.generate("xdrop1m", seed=31, scale=0.06, homolog_frac=0.3)
    scores, labels = F.sw_labels(w)
    assert 0.05 < labels.mean() < 0.6
    ctx = capi.Context(capi.config(capi.MODE_XDROP))
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    n = len(w.pairs)
    d_pairs = torch.from_numpy(w.pairs.view(np.uint8).copy()).cuda()
    feats = torch.empty(n * 16 * 2, dtype=torch.uint8, device="cuda:0")
    probe = F.Filter(0, seed=1)
    probe.features(ctx, d_pairs.data_ptr(), n, feats.data_ptr())
    probe.close()
    # the threshold keeps 99.7 % of the validation positives so that the
    # held-out test split stays at or above the 99.5 % target
    f, thr, m = F.train(w, feats, labels, epochs=4, recall=0.997)
    assert m["val"]["recall"] >= 0.997
    assert m["test"]["recall"] >= 0.995
    assert m["test"]["kept_fraction"] < m["kmer_rule_kept_at_same_recall"]
    f.close()
    ctx.close()


def test_features_match_oracle(native):
    """k_features against the float32 restatement in oracle/mlp_oracle.py,
    after bf16 rounding: at most one bf16 step apart (log2 may differ in the
    last float32 bit), and identical for almost every value."""
    import torch
    from oracle import mlp_oracle as M
    from oracle import oracle as O
    from pastis_gb300 import capi, synth
    from pastis_gb300.filter import Filter
    w = synth.generate("xdrop1m", seed=44, scale=0.003)
    ctx = capi.Context(capi.config(capi.MODE_XDROP))
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    n = len(w.pairs)
    d_pairs = torch.from_numpy(w.pairs.view(np.uint8).copy()).cuda()
    feats = torch.empty(n * 32, dtype=torch.uint8, device="cuda:0")
    f = Filter(0, seed=1)
    f.features(ctx, d_pairs.data_ptr(), n, feats.data_ptr())
    torch.cuda.synchronize()
    got = feats.cpu().numpy().view(np.uint16).reshape(n, 16).astype(np.int64)
    ref = M.features(w.pairs, w.seq, w.offs, O.blosum62().reshape(-1))
    ref_bits = (M.bf16(ref).astype(np.float32).view(np.uint32) >> 16).astype(np.int64)
    diff = np.abs(got - ref_bits)
    assert diff.max() <= 1
    assert (diff == 0).mean() > 0.99
    # the seed window separates homologs from random pairs on this generator
    win = ref[:, 8]
    assert win[w.homolog == 1].mean() > win[w.homolog == 0].mean() + 0.2
    f.close()
    ctx.close()
