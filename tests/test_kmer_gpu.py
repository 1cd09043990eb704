"""GPU candidate generation (pg_candidates) against the pair-by-pair CPU
restatement (oracle/kmer_oracle.py): every pair and every field."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["row", "col", "rs0", "cs0", "rs1", "cs1", "count", "score"]


@pytest.fixture(scope="module")
def fam(native):
    from pastis_gb300 import synth
    # families of 2-50 at 30-90 % identity, short sequences so the oracle is quick
    return synth.generate("sw100k", seed=77, scale=0.01, fam_min=2, fam_max=50, id_lo=0.3,
                          id_hi=0.9, len_median=120.0)


def as_rows(out):
    return [tuple(int(p[f]) for f in FIELDS) for p in out]


@pytest.mark.parametrize("k,stride,alph,prune,ckthr,rows,cols", [
    (6, 1, 0, 0, 0, (0, 200), (0, 200)),
    (6, 1, 0, 1, 0, (0, 200), (0, 200)),
    (4, 2, 0, 2, 0, (20, 180), (40, 200)),
    (5, 1, 1, 1, 1, (0, 200), (0, 200)),
    (3, 3, 1, 0, 2, (50, 120), (10, 90)),
])
def test_candidates_match_oracle(fam, k, stride, alph, prune, ckthr, rows, cols):
    from oracle import kmer_oracle as K
    from oracle import oracle as O
    from pastis_gb300 import capi
    ctx = capi.Context(capi.config(capi.MODE_XDROP))
    ctx.set_seqs(0, fam.ascii, fam.offs)
    ctx.share_row_seqs()
    kc = capi.kmer_config(k=k, stride=stride, alphabet=alph, prune=prune, ckthr=ckthr)
    got = ctx.candidates(kc, rows, cols)
    exp = K.candidates(fam.seq, fam.offs, rows, cols, O.blosum62(), k=k, stride=stride,
                       alph=alph, prune=prune, ckthr=ckthr)
    assert len(exp) > 0
    assert as_rows(got) == [tuple(e[f] for f in FIELDS) for e in exp]
    ctx.close()


def test_candidates_errors(fam):
    from pastis_gb300 import capi
    ctx = capi.Context(capi.config(capi.MODE_XDROP))
    ctx.set_seqs(0, fam.ascii, fam.offs)
    ctx.share_row_seqs()
    n = len(fam.offs) - 1
    with pytest.raises(capi.PgError):
        ctx.candidates(capi.kmer_config(k=7), (0, n), (0, n))        # 25^7 > 2^31
    with pytest.raises(capi.PgError):
        ctx.candidates(capi.kmer_config(), (0, n + 1), (0, n))
    with pytest.raises(capi.PgError):
        ctx.candidates(capi.kmer_config(k=2, max_products=10), (0, n), (0, n))
    assert len(ctx.candidates(capi.kmer_config(), (5, 5), (0, n))) == 0
    ctx.close()


def test_product_and_prune_counts(fam):
    """The counts the many-to-many bench reports (the reference's c_nnz and
    prune_sym log lines): on a diagonal block the product is symmetric, so it
    holds twice the even/odd-pruned pairs plus one diagonal entry per sequence
    with a k-mer; the ckthr prune only removes pairs; a count-only call
    (no output buffer) agrees with the materialised candidates."""
    import ctypes

    from pastis_gb300 import capi
    ctx = capi.Context(capi.config(capi.MODE_XDROP))
    ctx.set_seqs(0, fam.ascii, fam.offs)
    ctx.share_row_seqs()
    blk = (0, 200)

    def count(prune, ckthr):
        kc = capi.kmer_config(k=6, stride=1, prune=prune, ckthr=ckthr)
        n = ctypes.c_uint64()
        rc = ctx.lib.pg_candidates(ctx.h, ctypes.byref(kc), blk[0], blk[1], blk[0], blk[1], None,
                                   0, ctypes.byref(n), None)
        assert rc in (capi.PG_OK, capi.PG_ERR_RANGE)
        return int(n.value)

    full = ctx.candidates(capi.kmer_config(k=6, stride=1, prune=capi.PRUNE_NONE), blk, blk)
    eo = ctx.candidates(capi.kmer_config(k=6, stride=1, prune=capi.PRUNE_EVEN_ODD), blk, blk)
    diag = int((full["row"] == full["col"]).sum())
    L = fam.lengths()[blk[0]:blk[1]]
    assert diag == int((L >= 6).sum())
    assert len(full) == 2 * len(eo) + diag
    assert count(capi.PRUNE_NONE, 0) == len(full)
    assert count(capi.PRUNE_EVEN_ODD, 0) == len(eo)
    thr = count(capi.PRUNE_EVEN_ODD, 1)
    assert thr == int((eo["count"] > 1).sum()) and thr < len(eo)
    ctx.close()


def test_triples_are_the_nonzero_score_aln_entries(fam):
    """Candidates -> alignment -> triples, all on the device; the triples equal
    the host-side selection of score_aln != 0 with block offsets added."""
    import torch
    from pastis_gb300 import capi
    ctx = capi.Context(capi.config(capi.MODE_XDROP))
    ctx.set_seqs(0, fam.ascii, fam.offs)
    ctx.share_row_seqs()
    n_seq = len(fam.offs) - 1
    rows, cols = (10, n_seq), (0, n_seq - 5)
    pairs = ctx.candidates(capi.kmer_config(prune=capi.PRUNE_EVEN_ODD), rows, cols)
    res = ctx.align(pairs, rows[0], cols[0])
    n = len(pairs)
    d_pairs = torch.from_numpy(pairs.view(np.uint8).copy()).cuda()
    d_res = torch.from_numpy(res.view(np.uint8).copy()).cuda()
    r = torch.empty(n, dtype=torch.int64, device="cuda:0")
    c = torch.empty(n, dtype=torch.int64, device="cuda:0")
    v = torch.empty(n, dtype=torch.float32, device="cuda:0")
    k = capi.triples_device(d_pairs.data_ptr(), d_res.data_ptr(), n, rows[0], cols[0],
                            r.data_ptr(), c.data_ptr(), v.data_ptr())
    sel = res["score_aln"] != 0
    assert 0 < k == int(sel.sum()) < n
    assert np.array_equal(r[:k].cpu().numpy(), pairs["row"][sel].astype(np.int64) + rows[0])
    assert np.array_equal(c[:k].cpu().numpy(), pairs["col"][sel].astype(np.int64) + cols[0])
    assert np.array_equal(v[:k].cpu().numpy(), res["score_aln"][sel])
    ctx.close()
