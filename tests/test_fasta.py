"""FASTA ingest: the CPU restatement of PASTIS's parser (oracle/fasta_oracle.py)
on hand cases, and the GPU parser (pg_set_seqs_fasta) against it."""
import numpy as np
import pytest

LETTERS = "ARNDCQEGHILKMFPSTWYVBZX*J"

EDGE = (b"junk before the first record\n"
        b">s0 first\nACDEFG\nHIKLM\n"
        b">s1 short\nAC\n"
        b">s2 star and u\nAC*DEuU\nGG\n"
        b">s3 name > with gt\nMKVLAW\n"
        b">s4 name only, next record follows\n"
        b">s5\nAAAAAAAA>s6 starts mid-line\nCC\n"
        b">s7 tail\nWWWWWWW\n\n")


def test_oracle_by_hand():
    from oracle import fasta_oracle as F
    kept, orig, removed = F.parse(EDGE, 6)
    # s1 (2 residues) is checked and removed; s4 (empty, its name line is followed
    # directly by the next record) and s6... s5 ends mid-line so it is not
    # checked; s6 "CC" is followed by a newline and '>' so it is checked
    assert removed == [1, 6]
    assert orig == [0, 2, 3, 4, 5, 7]
    assert kept[0] == b"ACDEFGHIKLM"
    assert kept[1] == b"ACDETTGG"
    assert kept[2] == b"MKVLAW"
    assert kept[3] == b""
    assert kept[4] == b"AAAAAAAA"
    assert kept[5] == b"WWWWWWW"
    # a short last record is removed; k = 0 keeps everything
    assert F.parse(b">a\nACDEFG\n>b\nAC", 6)[2] == [1]
    assert F.parse(EDGE, 0)[2] == []


def random_fasta(rng, n):
    out = []
    for i in range(n):
        L = int(rng.integers(0, 400))
        seq = "".join(rng.choice(list("ACDEFGHIKLMNPQRSTVWYU*xbz"), L))
        width = int(rng.choice([60, 80, 1000]))
        lines = [seq[j:j + width] for j in range(0, len(seq), width)] or [""]
        out.append(">seq%d some > description\n" % i + "\n".join(lines))
    return ("\n".join(out) + "\n").encode()


@pytest.mark.gpu
@pytest.mark.parametrize("k", [0, 6, 50])
def test_gpu_parse_matches_oracle(native, k):
    from oracle import fasta_oracle as F
    from pastis_gb300 import capi
    rng = np.random.default_rng(k + 3)
    for text in (EDGE, random_fasta(rng, 3000)):
        kept, orig, removed = F.parse(text, k)
        ctx = capi.Context(capi.config(capi.MODE_SW))
        gi, nrm = ctx.set_seqs_fasta(0, text, k)
        codes, offs = ctx.get_seqs(0)
        assert nrm == len(removed) and list(gi) == orig
        # same residues as pg_set_seqs of the oracle's sequences
        ref = capi.Context(capi.config(capi.MODE_SW))
        asc = b"".join(kept)
        roffs = np.cumsum([0] + [len(s) for s in kept]).astype(np.uint64)
        ref.set_seqs(0, np.frombuffer(asc, dtype=np.uint8) if asc else np.zeros(0, np.uint8), roffs)
        rc, ro = ref.get_seqs(0)
        assert np.array_equal(offs, ro) and np.array_equal(codes, rc)
        ctx.close()
        ref.close()
