"""The affine gap model of the X-drop extension (PG_F_XDROP_AFFINE): the
oracle's form against the linear form where the two must agree and on a case
where only the affine form crosses a gap; the GPU kernel (k_xda) against the
oracle bit for bit, through the C ABI."""
import numpy as np
import pytest


def _homologs(rng, n, lo, hi):
    """n (v, h) residue-code pairs: h a mutated copy of v (substitutions and
    short indels) or an unrelated sequence."""
    out = []
    for i in range(n):
        m = int(rng.integers(lo, hi))
        v = rng.integers(0, 20, m).astype(np.uint8)
        if i % 3 == 2:
            h = rng.integers(0, 20, int(rng.integers(lo, hi))).astype(np.uint8)
        else:
            h = []
            for r in v:
                u = rng.random()
                if u < 0.05:
                    continue                       # deletion
                if u < 0.10:
                    h.extend(rng.integers(0, 20, int(rng.integers(1, 4))))   # insertion
                h.append(r if rng.random() < 0.7 else rng.integers(0, 20))
            h = np.array(h, dtype=np.uint8)
        out.append((v, h))
    return out


@pytest.mark.parametrize("g", [-11, -5, -1])
def test_affine_equals_linear_when_gap_scores_agree(oracle_mod, g):
    """With first == further == the linear gap score the three-state
    recurrence is the linear one: every extension ends at the same cell after
    the same band cells."""
    O = oracle_mod
    rng = np.random.default_rng(7 - g)
    lin = O.make_params(gap_first=g, gap_ext=g, xdrop_gap=g, xdrop=49)
    aff = O.make_params(gap_first=g, gap_ext=g, xdrop_gap=g, xdrop=49, flags=O.F_XDROP_AFFINE)
    for v, h in _homologs(rng, 60, 20, 300):
        s = int(rng.integers(0, min(len(v), len(h))))
        seed = (s, s + 1, s, s + 1)
        assert O.xdrop_extend(v, h, lin, *seed) == O.xdrop_extend(v, h, aff, *seed)


def test_affine_crosses_a_gap_the_linear_form_stops_at(oracle_mod):
    """V = W^10 P^4 W^10, H = W^20, seed at the first W.  X = 10: the linear
    gap -5 makes the 4-residue insertion cost 20, so the band dies inside it;
    affine -3 / -1 costs 6 and the extension reaches both sequence ends."""
    O = oracle_mod
    v = O.encode("W" * 10 + "PPPP" + "W" * 10)
    h = O.encode("W" * 20)
    seed = (0, 1, 0, 1)          # bh, eh, bv, ev
    lin = O.make_params(gap_first=-3, gap_ext=-1, xdrop_gap=-5, xdrop=10)
    aff = O.make_params(gap_first=-3, gap_ext=-1, xdrop_gap=-5, xdrop=10,
                        flags=O.F_XDROP_AFFINE)
    (bh, eh, bv, ev), _ = O.xdrop_extend(v, h, aff, *seed)
    assert (bh, eh, bv, ev) == (0, 20, 0, 24)
    (bh, eh, bv, ev), _ = O.xdrop_extend(v, h, lin, *seed)
    assert ev <= 12 and eh <= 12
    # the global alignment of the affine infix opens one gap of four
    r = O.global_(v, h, aff)
    assert r["score"] == 20 * 11 - 3 - 3 * 1 and r["gap_opens"] == 1


def test_affine_batch_is_deterministic_and_differs_from_linear(oracle_mod):
    """Over a batch the affine flag changes the extension (some infixes differ
    from the linear form's) and nothing else about the pipeline: the cells
    count only band cells and global DP cells, identity stays in [0, 100]."""
    from pastis_gb300 import synth
    O = oracle_mod
    w = synth.generate("xdrop1m", seed=31, scale=0.0005)
    codes = O.encode(bytes(w.ascii))
    lin = O.pastis_params()
    aff = O.pastis_params(flags=O.F_XDROP_AFFINE)
    a = O.batch(1, codes, w.offs, codes, w.offs, w.pairs, aff)
    b = O.batch(1, codes, w.offs, codes, w.offs, w.pairs, aff, nthreads=1)
    c = O.batch(1, codes, w.offs, codes, w.offs, w.pairs, lin)
    assert a.tobytes() == b.tobytes()
    assert (a["score"] != c["score"]).any()
    assert ((a["identity"] >= 0) & (a["identity"] <= 100)).all()


# ----------------------------------------------------------------- GPU

FIELDS = ["score", "aln_len", "matches", "gap_opens", "beg_h", "end_h", "beg_v", "end_v",
          "identity", "score_aln", "seed_used", "flags", "cells"]


def _gpu_vs_oracle(O, w, cfg):
    from pastis_gb300 import capi
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    got = ctx.align(w.pairs)
    # k_xda, k_hist, k_bucket, k_dirsize, k_ga_dir, k_ga_pair, k_tb_ga (+ the
    # checked 16-bit pass where long regions need it)
    assert ctx.last_launches() in (7, 8)
    ctx.close()
    first, ext, xg = capi.resolved_gaps(cfg)
    p = O.make_params(gap_first=first, gap_ext=ext, xdrop_gap=xg, xdrop=cfg.xdrop,
                      seed_len=cfg.seed_len, seed_count=cfg.seed_count, tie=cfg.tie,
                      flags=cfg.flags, cov_thr=cfg.cov_thr, ani_thr=cfg.ani_thr)
    codes = O.encode(bytes(w.ascii))
    exp = O.batch(1, codes, w.offs, codes, w.offs, w.pairs, p)
    for f in FIELDS:
        a, b = got[f], exp[f]
        if f in ("identity", "score_aln"):
            a, b = a.view(np.uint32), b.view(np.uint32)
        bad = np.flatnonzero(a != b)
        assert len(bad) == 0, (f, len(bad), int(bad[0]), w.pairs[bad[0]])
    return got


@pytest.mark.gpu
@pytest.mark.parametrize("gaps", [0, 1])
@pytest.mark.parametrize("xdrop", [49, 10])
def test_affine_xdrop_parity(native, oracle_mod, gaps, xdrop):
    from pastis_gb300 import capi, synth
    w = synth.generate("xdrop1m", seed=202, scale=0.005)
    cfg = capi.config(capi.MODE_XDROP, gap_semantics=gaps, xdrop=xdrop,
                      flags=capi.F_XDROP_AFFINE)
    got = _gpu_vs_oracle(oracle_mod, w, cfg)
    assert (got["flags"] & capi.RF_PASSED).any()


@pytest.mark.gpu
def test_affine_xdrop_long_sequences(native, oracle_mod):
    """Sequences up to 5000 residues: the warp's ring spans the longest one."""
    from pastis_gb300 import capi, synth
    w = synth.generate("uneven10m", seed=17, scale=0.00003)
    cfg = capi.config(capi.MODE_XDROP, flags=capi.F_XDROP_AFFINE | capi.F_SKIP_SPURIOUS_SEED)
    _gpu_vs_oracle(oracle_mod, w, cfg)
