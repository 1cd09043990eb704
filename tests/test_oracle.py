"""The CPU oracle against the committed known-answer fixtures (tests/golden/kat.json).

Parity with SeqAn itself is unpinned (SeqAn is not in the reference checkout);
these fixtures pin the DP definitions: hand-derived cases and exhaustive
enumeration of all alignments of short sequences."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "kat.json")


def _cases(kind):
    with open(GOLDEN) as f:
        return [c for c in json.load(f)["cases"] if c["kind"] == kind]


@pytest.mark.parametrize("case", _cases("local") + _cases("global"),
                         ids=lambda c: "%s-%s-%s-%d" % (c["kind"], c["v"] or "0", c["h"] or "0",
                                                        c["gap_first"]))
def test_dp_known_answers(case, oracle_mod):
    O = oracle_mod
    p = O.make_params(gap_first=case["gap_first"], gap_ext=case["gap_ext"])
    f = O.local if case["kind"] == "local" else O.global_
    r = f(O.encode(case["v"]), O.encode(case["h"]), p)
    for k, v in case["expected"].items():
        got = int(r["flags"]) & O.RF_EMPTY if k == "empty" else int(r[k])
        assert got == v, (k, v, got, case.get("derivation", ""))


@pytest.mark.parametrize("case", _cases("xdrop_extend"), ids=lambda c: c["v"])
def test_xdrop_known_answers(case, oracle_mod):
    O = oracle_mod
    p = O.make_params(xdrop_gap=case["xdrop_gap"], xdrop=case["xdrop"])
    (bh, eh, bv, ev), _ = O.xdrop_extend(O.encode(case["v"]), O.encode(case["h"]), p,
                                         *case["seed"])
    assert dict(bh=bh, eh=eh, bv=bv, ev=ev) == case["expected"], case["derivation"]


def test_blosum62_properties(oracle_mod):
    m = oracle_mod.blosum62().astype(int)
    assert (m == m.T).all()
    assert m[10, 10] == 4 and (m[24] == m[10]).all()  # J scores as L
    assert m[17, 17] == 11 and m[23, 23] == 1 and m[0, 23] == -4


def test_identity_rounding(oracle_mod):
    """identity = (float)(100.0 * M / L) computed in double, as computeAlignmentStats."""
    O = oracle_mod
    p = O.make_params()
    r = O.global_(O.encode("WWWWWWWW"), O.encode("WWWWGWWWW"), p)
    assert r["identity"] == np.float32(100.0 * 8 / 9)
    # through the --sfa pair path the filter sets score_aln = identity / 100 (f32)
    v = O.encode("MKWWWWWWWWQR")
    h = O.encode("MKWWWWGWWWWQR")
    seq = np.concatenate([v, h])
    offs = np.array([0, len(v), len(v) + len(h)], dtype=np.uint64)
    pr = np.zeros(1, dtype=O.PAIR_DTYPE)
    pr["row"], pr["col"] = 0, 1
    out = O.batch(0, seq, offs, seq, offs, pr, p)[0]
    ident = np.float32(100.0 * out["matches"] / out["aln_len"])
    assert out["identity"] == ident
    assert out["score_aln"] == np.float32(ident / np.float32(100.0))
    assert out["flags"] & O.RF_PASSED


def test_local_swap_invariance(oracle_mod):
    """BLOSUM62 is symmetric: swapping V and H keeps the local score."""
    O = oracle_mod
    rng = np.random.default_rng(3)
    p = O.make_params()
    for _ in range(50):
        a = rng.integers(0, 20, rng.integers(1, 60)).astype(np.uint8)
        b = rng.integers(0, 20, rng.integers(1, 60)).astype(np.uint8)
        assert O.local(a, b, p)["score"] == O.local(b, a, p)["score"]
        assert O.global_(a, b, p)["score"] == O.global_(b, a, p)["score"]


def test_local_dominates_xdrop_region(oracle_mod):
    """A global alignment of any sub-region scores at most the local optimum."""
    O = oracle_mod
    rng = np.random.default_rng(5)
    p = O.make_params()
    for _ in range(40):
        a = rng.integers(0, 20, rng.integers(20, 80)).astype(np.uint8)
        b = a.copy()
        b[rng.random(len(b)) < 0.3] = rng.integers(0, 20)
        loc = O.local(a, b, p)["score"]
        bh, eh, bv, ev = 5, 11, 5, 11
        (bh, eh, bv, ev), _ = O.xdrop_extend(a, b, p, bh, eh, bv, ev)
        g = O.global_(a[bv:ev], b[bh:eh], p)["score"]
        assert g <= loc


@pytest.mark.parametrize("tie", [0, 1, 2, 3])
@pytest.mark.parametrize("gaps", [(-11, -2), (-2, -11), (-5, -5)])
def test_packed_dp_equals_plain(oracle_mod, tie, gaps):
    """The batch path's packed DP makes exactly the plain DP's choices."""
    O = oracle_mod
    rng = np.random.default_rng(100 + tie)
    p = O.make_params(gap_first=gaps[0], gap_ext=gaps[1], tie=tie)
    letters = O.encode("ARNDCQEGHILKMFPSTWYVW")
    for k in range(150):
        a = letters[rng.integers(0, len(letters), rng.integers(0, 70))]
        b = a.copy() if k % 3 == 0 else letters[rng.integers(0, len(letters), rng.integers(0, 70))]
        if k % 3 == 0 and len(b):
            b[rng.random(len(b)) < 0.3] = letters[rng.integers(0, 20)]
            b = np.delete(b, rng.integers(0, len(b), min(3, len(b))))
        for local_ in (True, False):
            slow = (O.local if local_ else O.global_)(a, b, p)
            fast = O.align_fast(a, b, p, local_)
            assert slow.tobytes() == fast.tobytes(), (k, local_, slow, fast)


def test_batch_matches_single(oracle_mod):
    """orc_batch (OpenMP) equals the single-pair functions, in both modes."""
    O = oracle_mod
    rng = np.random.default_rng(11)
    seqs = [rng.integers(0, 20, rng.integers(10, 120)).astype(np.uint8) for _ in range(30)]
    offs = np.concatenate([[0], np.cumsum([len(s) for s in seqs])]).astype(np.uint64)
    res = np.concatenate(seqs)
    pairs = np.zeros(200, dtype=O.PAIR_DTYPE)
    pairs["row"] = rng.integers(0, 30, 200)
    pairs["col"] = rng.integers(0, 30, 200)
    L = np.diff(offs).astype(int)
    pairs["rs0"] = [rng.integers(0, L[r] - 5) for r in pairs["row"]]
    pairs["cs0"] = [rng.integers(0, L[c] - 5) for c in pairs["col"]]
    pairs["count"] = 1
    p = O.make_params()
    for mode in (0, 1):
        out = O.batch(mode, res, offs, res, offs, pairs, p, nthreads=4)
        for i in range(0, 200, 17):
            v = seqs[pairs["row"][i]]
            h = seqs[pairs["col"][i]]
            if mode == 0:
                one = O.local(v, h, p)
                assert out[i]["score"] == one["score"] and out[i]["aln_len"] == one["aln_len"]
            else:
                assert out[i]["beg_h"] <= pairs["cs0"][i] or out[i]["flags"] & O.RF_BAD_SEED
    with pytest.raises(IndexError):
        bad = pairs.copy()
        bad["row"][0] = 30
        O.batch(0, res, offs, res, offs, bad, p)
