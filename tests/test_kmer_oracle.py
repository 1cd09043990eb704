"""The CPU restatement of candidate generation (oracle/kmer_oracle.py) on
hand-derived cases: k-mer codes, count, seeds, score, alphabets, prunes."""
import numpy as np

LETTERS = "ARNDCQEGHILKMFPSTWYVBZX*J"


def enc(s):
    return np.array([LETTERS.index(ch) for ch in s], dtype=np.uint8)


def seqset(*seqs):
    codes = np.concatenate([enc(s) for s in seqs])
    offs = np.cumsum([0] + [len(s) for s in seqs]).astype(np.uint64)
    return codes, offs


def test_shared_kmers_by_hand():
    """ACDEFGHIK vs XXACDEFGYY, k = 3: shared ACD CDE DEF EFG; codes (base 25)
    103, 2581, 2038, 4082, so first = ACD at (0, 2), second = EFG at (3, 5);
    self scores 19, 20, 17, 17."""
    from oracle import kmer_oracle as K
    from oracle import oracle as O
    codes, offs = seqset("ACDEFGHIK", "XXACDEFGYY")
    out = K.candidates(codes, offs, (0, 1), (1, 2), O.blosum62(), k=3)
    assert out == [{"row": 0, "col": 0, "rs0": 0, "cs0": 2, "rs1": 3, "cs1": 5, "count": 4,
                    "score": 20}]


def test_repeated_kmer_counts_every_occurrence_pair():
    from oracle import kmer_oracle as K
    from oracle import oracle as O
    codes, offs = seqset("WWWWW", "WWWW")      # WWW: 3 x 2 occurrences
    out = K.candidates(codes, offs, (0, 1), (1, 2), O.blosum62(), k=3)
    assert out[0]["count"] == 6 and out[0]["score"] == 33
    assert (out[0]["rs0"], out[0]["cs0"], out[0]["rs1"], out[0]["cs1"]) == (0, 0, 2, 1)


def test_single_shared_kmer_has_zero_second_seed():
    from oracle import kmer_oracle as K
    from oracle import oracle as O
    codes, offs = seqset("MKVLA", "GGMKVGG")
    out = K.candidates(codes, offs, (0, 1), (1, 2), O.blosum62(), k=3)
    assert out == [{"row": 0, "col": 0, "rs0": 0, "cs0": 2, "rs1": 0, "cs1": 0, "count": 1,
                    "score": 5 + 5 + 4}]


def test_murphy10_merges_groups():
    """ILV and LIM fall in one murphy10 group (I); the representative's self
    score (I: 4) counts for each letter."""
    from oracle import kmer_oracle as K
    from oracle import oracle as O
    codes, offs = seqset("ILV", "LIM")
    assert K.candidates(codes, offs, (0, 1), (1, 2), O.blosum62(), k=3) == []
    out = K.candidates(codes, offs, (0, 1), (1, 2), O.blosum62(), k=3, alph=1)
    assert out[0]["count"] == 1 and out[0]["score"] == 12


def test_prunes_and_thresholds():
    from oracle import kmer_oracle as K
    from oracle import oracle as O
    codes, offs = seqset("MKVLAW", "MKVLAW", "MKVLAW", "MKVLAW")
    sm = O.blosum62()
    full = K.candidates(codes, offs, (0, 4), (0, 4), sm, k=3)
    assert len(full) == 16
    eo = {(p["row"], p["col"]) for p in K.candidates(codes, offs, (0, 4), (0, 4), sm, k=3, prune=1)}
    # exactly one of (r, c) / (c, r), never the diagonal
    assert len(eo) == 6 and all((c, r) not in eo and r != c for r, c in eo)
    up = {(p["row"], p["col"]) for p in K.candidates(codes, offs, (0, 4), (0, 4), sm, k=3, prune=2)}
    assert up == {(r, c) for r in range(4) for c in range(4) if r < c}
    assert K.candidates(codes, offs, (0, 4), (0, 4), sm, k=3, ckthr=4) == []
    assert len(K.candidates(codes, offs, (0, 4), (0, 4), sm, k=3, ckthr=3)) == 16
    # column-major order, block-relative indices
    blk = K.candidates(codes, offs, (1, 3), (2, 4), sm, k=3)
    assert [(p["row"], p["col"]) for p in blk] == [(0, 0), (1, 0), (0, 1), (1, 1)]
