"""Learned candidate-pair filter: training, threshold choice and evaluation.

PASTIS prunes candidates before alignment by k-mer overlap alone
(count <= ckthr or score <= mosthr, src/DistPWRunner.cpp:48-54).  This module
trains the library's 16-64-64-1 BF16 network (pastis_gb300/csrc/pg_filter.cu)
to do the same job better: labels come from this library's own Smith-Waterman
kernel (a pair is worth aligning when its local score reaches the per-length
threshold below), the decision threshold is set on held-out pairs for a recall
target, and the plain aligner remains the judge of what the filter drops.

Label: S >= T(m, n) = ceil((ln(K m n) + ln(1/E)) / lambda), the smallest score
whose Karlin-Altschul E-value m n K exp(-lambda S) is at most E = 1e-3, with
the published gapped BLOSUM62 parameters lambda = 0.267, K = 0.041; S is the
local score under gap open -11 / extend -2 taken by name.
"""
import ctypes
import math

import numpy as np

from . import capi

LAMBDA, KARLIN_K, EVALUE = 0.267, 0.041, 1e-3


def score_threshold(m, n):
    m = np.maximum(np.asarray(m, dtype=np.float64), 1.0)
    n = np.maximum(np.asarray(n, dtype=np.float64), 1.0)
    return np.ceil((np.log(KARLIN_K * m * n) + math.log(1.0 / EVALUE)) / LAMBDA)


class Filter:
    """One pg_filter (network parameters and Adam state on a device)."""

    def __init__(self, device=0, seed=1):
        self.lib = capi.load()
        h = ctypes.c_void_p()
        capi._check(self.lib.pg_filter_create(device, seed, ctypes.byref(h)))
        self.h = h
        self.nparams = int(self.lib.pg_filter_nparams())

    def close(self):
        if getattr(self, "h", None):
            self.lib.pg_filter_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        out = np.zeros(self.nparams, dtype=np.float32)
        capi._check(self.lib.pg_filter_params(self.h, out.ctypes.data, 1))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        capi._check(self.lib.pg_filter_params(self.h, p.ctypes.data, 0))

    def features(self, ctx, d_pairs, n, d_feat, stream=None, roff=0, coff=0):
        capi._check(self.lib.pg_filter_features(self.h, ctx.h, d_pairs, n, roff, coff, d_feat,
                                                 stream))

    def predict(self, d_feat, n, d_logits, stream=None):
        capi._check(self.lib.pg_filter_predict(self.h, d_feat, n, d_logits, stream))

    def gradients(self, d_feat, d_y, d_w, n, stream=None):
        out = np.zeros(self.nparams + 1, dtype=np.float32)
        capi._check(self.lib.pg_filter_gradients(self.h, d_feat, d_y, d_w, n, out.ctypes.data,
                                                  stream))
        return out[:-1], float(out[-1])

    def train_step(self, d_feat, d_y, d_w, n, lr, stream=None):
        loss = ctypes.c_float()
        capi._check(self.lib.pg_filter_train_step(self.h, d_feat, d_y, d_w, n, lr,
                                                   ctypes.byref(loss), stream))
        return loss.value

    def align_filtered(self, ctx, threshold, d_pairs, n, d_out, stream=None, roff=0, coff=0):
        kept = ctypes.c_uint64()
        capi._check(self.lib.pg_align_filtered(ctx.h, self.h, threshold, d_pairs, n, roff, coff,
                                                d_out, stream, ctypes.byref(kept)))
        return int(kept.value)


def sw_labels(w, device=0):
    """Local SW score of every pair (this library's kernel, gap open -11 /
    extend -2 by name, the model the Karlin-Altschul parameters above are
    published for) and the label."""
    ctx = capi.Context(capi.config(capi.MODE_SW, device=device, gap_semantics=capi.GAPS_NOMINAL))
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    res = ctx.align(w.pairs)
    ctx.close()
    L = w.lengths()
    thr = score_threshold(L[w.pairs["row"]], L[w.pairs["col"]])
    return res["score"].astype(np.int64), (res["score"] >= thr).astype(np.float32)


def recall_threshold(logits, labels, recall):
    """Largest threshold keeping at least `recall` of the positives."""
    pos = np.sort(logits[labels > 0.5])
    if len(pos) == 0:
        return float("inf")
    k = int(math.floor((1.0 - recall) * len(pos)))
    return float(np.nextafter(pos[k], -np.inf)) if k > 0 else float(np.nextafter(pos[0], -np.inf))


def kmer_rule_at_recall(pairs, labels, recall):
    """The best single-feature rule of PASTIS's own prune (count or k-mer score
    above a threshold) that keeps `recall` of the positives: fraction kept."""
    best = 1.0
    for key in ("count", "score"):
        v = pairs[key].astype(np.int64)
        for t in np.unique(v):
            keep = v > t
            pos = labels > 0.5
            if pos.sum() == 0 or keep[pos].mean() < recall:
                continue
            best = min(best, keep.mean())
    return best


def train(w, feats_dev, labels, device=0, epochs=4, batch=8192, lr=3e-3, pos_weight=4.0, seed=1,
          val_frac=0.1, test_frac=0.1, recall=0.995, log=None):
    """Train on (features on the device, labels on the host).  Returns the
    filter, the chosen threshold and a metrics dict over the held-out split."""
    import torch
    n = len(labels)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n)
    n_test = int(n * test_frac)
    n_val = int(n * val_frac)
    test, val, tr = perm[:n_test], perm[n_test:n_test + n_val], perm[n_test + n_val:]
    dev = torch.device("cuda", device)
    X = feats_dev  # torch uint8 / bf16 tensor, n x 16 bf16 as raw bytes
    Xb = X.view(torch.bfloat16).view(n, capi_features())
    y = torch.from_numpy(labels).to(dev)
    wts = torch.where(y > 0.5, torch.tensor(pos_weight, device=dev), torch.tensor(1.0, device=dev))
    f = Filter(device, seed)
    tr_t = torch.from_numpy(tr).to(dev)
    losses = []
    for ep in range(epochs):
        order = tr_t[torch.randperm(len(tr_t), device=dev)]
        lr_ep = lr * (0.5 ** ep)
        for s in range(0, len(order), batch):
            idx = order[s:s + batch]
            xb = Xb[idx].contiguous()
            yb = y[idx].contiguous()
            wb = wts[idx].contiguous()
            loss = f.train_step(xb.data_ptr(), yb.data_ptr(), wb.data_ptr(), len(idx), lr_ep)
            losses.append(loss)
        if log:
            log("epoch %d mean loss %.4f" % (ep, float(np.mean(losses[-max(1, len(order) // batch):]))))
    logits = torch.empty(n, dtype=torch.float32, device=dev)
    f.predict(Xb.data_ptr(), n, logits.data_ptr())
    torch.cuda.synchronize(dev)
    z = logits.cpu().numpy()
    thr = recall_threshold(z[val], labels[val], recall)
    keep = z >= thr
    pos = labels > 0.5

    def metrics(ix):
        k, p = keep[ix], pos[ix]
        return {"pairs": int(len(ix)), "positives": int(p.sum()),
                "recall": float(k[p].mean()) if p.any() else float("nan"),
                "precision": float(p[k].mean()) if k.any() else float("nan"),
                "kept_fraction": float(k.mean())}
    out = {"threshold": thr, "val": metrics(val), "test": metrics(test),
           "train_loss_last": float(np.mean(losses[-20:])),
           "kmer_rule_kept_at_same_recall": kmer_rule_at_recall(w.pairs[test], labels[test],
                                                                 recall)}
    return f, thr, out


def capi_features():
    return 16


def workload_features(w, device=0, mode=None):
    """Features of every pair of a workload, on the device (torch uint8 tensor
    holding n x 16 BF16 values)."""
    import torch
    mode = capi.MODE_XDROP if mode is None else mode
    ctx = capi.Context(capi.config(mode, device=device))
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    n = len(w.pairs)
    dev = torch.device("cuda", device)
    d_pairs = torch.from_numpy(w.pairs.view(np.uint8).copy()).to(dev)
    feats = torch.empty(n * capi_features() * 2, dtype=torch.uint8, device=dev)
    probe = Filter(device, seed=1)
    probe.features(ctx, d_pairs.data_ptr(), n, feats.data_ptr())
    torch.cuda.synchronize(dev)
    probe.close()
    ctx.close()
    return feats


def fit(w, device=0, recall=0.995, epochs=4, log=None, labels=None):
    """Label a training workload with the SW kernel (or take the labels
    given, e.g. whether the plain aligner's result passes the coverage/ANI
    filter), compute its features and train a filter on them.  Returns
    (filter, threshold, metrics)."""
    import time
    t0 = time.perf_counter()
    if labels is None:
        _, labels = sw_labels(w, device)
    labels = np.asarray(labels, dtype=np.float32)
    t1 = time.perf_counter()
    feats = workload_features(w, device)
    f, thr, m = train(w, feats, labels, device=device, epochs=epochs, recall=recall, log=log)
    t2 = time.perf_counter()
    m["label_seconds"] = t1 - t0
    m["train_seconds"] = t2 - t1
    m["pairs"] = int(len(labels))
    m["positive_fraction"] = float(labels.mean())
    return f, thr, m
