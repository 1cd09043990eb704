"""Generate tests/golden/kat.json: known-answer cases for the alignment stage.

Two sources, both independent of the oracle's DP code:

1. Hand-derived cases (the derivation is stored with each case).
2. Exhaustive enumeration: every alignment of two short sequences is listed
   and scored directly (a gap run of length L scores max(L*first,
   first + (L-1)*ext): the DP may reopen a gap, and the best split of a run
   is either one open or all opens).  The best score is the expected score;
   statistics are expected only where every optimal alignment has the same
   (columns, matches, gap runs) and, for local alignment, the same
   coordinates.

The reference ships no test vectors (its only input, tests/scope_77k.fa, is
missing) and SeqAn is absent, so these cases pin the DP definitions, not
SeqAn's bits.  Run: python tests/golden/make_golden.py
"""
import itertools
import json
import os
import random

LETTERS = "ARNDCQEGHILKMFPSTWYVBZX*J"
B62_ROWS = """
 4 -1 -2 -2  0 -1 -1  0 -2 -1 -1 -1 -1 -2 -1  1  0 -3 -2  0 -2 -1  0 -4
-1  5  0 -2 -3  1  0 -2  0 -3 -2  2 -1 -3 -2 -1 -1 -3 -2 -3 -1  0 -1 -4
-2  0  6  1 -3  0  0  0  1 -3 -3  0 -2 -3 -2  1  0 -4 -2 -3  3  0 -1 -4
-2 -2  1  6 -3  0  2 -1 -1 -3 -4 -1 -3 -3 -1  0 -1 -4 -3 -3  4  1 -1 -4
 0 -3 -3 -3  9 -3 -4 -3 -3 -1 -1 -3 -1 -2 -3 -1 -1 -2 -2 -1 -3 -3 -2 -4
-1  1  0  0 -3  5  2 -2  0 -3 -2  1  0 -3 -1  0 -1 -2 -1 -2  0  3 -1 -4
-1  0  0  2 -4  2  5 -2  0 -3 -3  1 -2 -3 -1  0 -1 -3 -2 -2  1  4 -1 -4
 0 -2  0 -1 -3 -2 -2  6 -2 -4 -4 -2 -3 -3 -2  0 -2 -2 -3 -3 -1 -2 -1 -4
-2  0  1 -1 -3  0  0 -2  8 -3 -3 -1 -2 -1 -2 -1 -2 -2  2 -3  0  0 -1 -4
-1 -3 -3 -3 -1 -3 -3 -4 -3  4  2 -3  1  0 -3 -2 -1 -3 -1  3 -3 -3 -1 -4
-1 -2 -3 -4 -1 -2 -3 -4 -3  2  4 -2  2  0 -3 -2 -1 -2 -1  1 -4 -3 -1 -4
-1  2  0 -1 -3  1  1 -2 -1 -3 -2  5 -1 -3 -1  0 -1 -3 -2 -2  0  1 -1 -4
-1 -1 -2 -3 -1  0 -2 -3 -2  1  2 -1  5  0 -2 -1 -1 -1 -1  1 -3 -1 -1 -4
-2 -3 -3 -3 -2 -3 -3 -3 -1  0  0 -3  0  6 -4 -2 -2  1  3 -1 -3 -3 -1 -4
-1 -2 -2 -1 -3 -1 -1 -2 -2 -3 -3 -1 -2 -4  7 -1 -1 -4 -3 -2 -2 -1 -2 -4
 1 -1  1  0 -1  0  0  0 -1 -2 -2  0 -1 -2 -1  4  1 -3 -2 -2  0  0  0 -4
 0 -1  0 -1 -1 -1 -1 -2 -2 -1 -1 -1 -1 -2 -1  1  5 -2 -2  0 -1 -1  0 -4
-3 -3 -4 -4 -2 -2 -3 -2 -2 -3 -2 -3 -1  1 -4 -3 -2 11  2 -3 -4 -3 -2 -4
-2 -2 -2 -3 -2 -1 -2 -3  2 -1 -1 -2 -1  3 -3 -2 -2  2  7 -1 -3 -2 -1 -4
 0 -3 -3 -3 -1 -2 -2 -3 -3  3  1 -2  1 -1 -2 -2  0 -3 -1  4 -3 -2 -1 -4
-2 -1  3  4 -3  0  1 -1  0 -3 -4  0 -3 -3 -2  0 -1 -4 -3 -3  4  1 -1 -4
-1  0  0  1 -3  3  4 -2  0 -3 -3  1 -1 -3 -1  0 -1 -3 -2 -2  1  4 -1 -4
 0 -1 -1 -1 -2 -1 -1 -1 -1 -1 -1 -1 -1 -1 -2  0  0 -2 -1 -1 -1 -1 -1 -4
-4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4  1
"""


def b62():
    rows = [[int(x) for x in ln.split()] for ln in B62_ROWS.strip().splitlines()]
    idx = {c: i for i, c in enumerate(LETTERS[:24])}

    def s(a, b):
        a = "L" if a == "J" else a
        b = "L" if b == "J" else b
        return rows[idx[a]][idx[b]]
    return s


S = b62()


def alignments(a, b):
    """All global alignments as lists of (x, y) with None for a gap."""
    if not a and not b:
        yield []
        return
    if a and b:
        for rest in alignments(a[1:], b[1:]):
            yield [(a[0], b[0])] + rest
    if a:
        for rest in alignments(a[1:], b):
            yield [(a[0], None)] + rest
    if b:
        for rest in alignments(a, b[1:]):
            yield [(None, b[0])] + rest


def score_and_stats(cols, first, ext):
    sc, M, G = 0, 0, 0
    k = 0
    while k < len(cols):
        x, y = cols[k]
        if x is not None and y is not None:
            sc += S(x, y)
            M += x == y
            k += 1
            continue
        kind = x is None  # True: gap in V (horizontal)
        L = 0
        while k < len(cols) and (cols[k][0] is None) == kind and \
                (cols[k][0] is None or cols[k][1] is None):
            L += 1
            k += 1
        sc += max(L * first, first + (L - 1) * ext)
        G += 1
    return sc, len(cols), M, G


def brute_global(v, h, first, ext):
    best, stats = None, set()
    for al in alignments(v, h):
        sc, L, M, G = score_and_stats(al, first, ext)
        if best is None or sc > best:
            best, stats = sc, {(L, M, G)}
        elif sc == best:
            stats.add((L, M, G))
    return best, stats


def brute_local(v, h, first, ext):
    best, keys = 0, {(0, 0, 0, None)}
    for i0 in range(len(v)):
        for i1 in range(i0 + 1, len(v) + 1):
            for j0 in range(len(h)):
                for j1 in range(j0 + 1, len(h) + 1):
                    for al in alignments(v[i0:i1], h[j0:j1]):
                        # local alignments begin and end with an aligned pair
                        if al[0][0] is None or al[0][1] is None or al[-1][0] is None or al[-1][1] is None:
                            continue
                        sc, L, M, G = score_and_stats(al, first, ext)
                        key = (L, M, G, (i0, i1, j0, j1))
                        if sc > best:
                            best, keys = sc, {key}
                        elif sc == best and sc > 0:
                            keys.add(key)
    return best, keys


def main():
    cases = []
    gaps = {"nominal": (-11, -2), "as_called": (-2, -11)}
    # ---- hand-derived
    hand = [
        ("local", "ACDEFGHIK", "ACDEFGHIK", "nominal",
         dict(score=53, aln_len=9, matches=9, gap_opens=0, beg_v=0, end_v=9, beg_h=0, end_h=9),
         "identical: sum of self scores A4 C9 D6 E5 F6 G6 H8 I4 K5 = 53"),
        ("global", "ACDEFGHIK", "ACDGHIK", "nominal",
         dict(score=29, aln_len=9, matches=7, gap_opens=1),
         "7 matches (42) and one run of 2 gaps opposite EF: 42 - 11 - 2 = 29"),
        ("global", "ACDEFGHIK", "ACDGHIK", "as_called",
         dict(score=38, aln_len=9, matches=7, gap_opens=1),
         "first -2 / further -11: two reopened positions score -4 > -13: 42 - 4 = 38; one run"),
        ("local", "WWWWW", "WWAWW", "nominal",
         dict(score=41, aln_len=5, matches=4, gap_opens=0, beg_v=0, end_v=5, beg_h=0, end_h=5),
         "one substitution: 4 x W/W 11 + W/A -3 = 41 beats 22"),
        ("global", "WWWWWWWW", "WWWWGWWWW", "nominal",
         dict(score=77, aln_len=9, matches=8, gap_opens=1), "gap of 1: 88 - 11"),
        ("global", "WWWWWWWW", "WWWWGGWWWW", "nominal",
         dict(score=75, aln_len=10, matches=8, gap_opens=1), "gap of 2: 88 - 11 - 2"),
        ("global", "WWWWWWWW", "WWWWGGGWWWW", "nominal",
         dict(score=73, aln_len=11, matches=8, gap_opens=1), "gap of 3: 88 - 11 - 2 - 2"),
        ("global", "WWWWWWWW", "WWWWGWWWW", "as_called",
         dict(score=86, aln_len=9, matches=8, gap_opens=1), "gap of 1: 88 - 2"),
        ("global", "WWWWWWWW", "WWWWGGWWWW", "as_called",
         dict(score=84, aln_len=10, matches=8, gap_opens=1), "gap of 2: 88 - 2 - 2 (reopen)"),
        ("global", "WWWWWWWW", "WWWWGGGWWWW", "as_called",
         dict(score=82, aln_len=11, matches=8, gap_opens=1), "gap of 3: 88 - 6, still one run"),
        ("local", "WWW", "PPP", "nominal",
         dict(score=0, aln_len=0, matches=0, gap_opens=0, empty=1), "all mismatches: empty"),
        ("local", "W", "W", "nominal",
         dict(score=11, aln_len=1, matches=1, gap_opens=0, beg_v=0, end_v=1, beg_h=0, end_h=1),
         "length 1"),
        ("global", "W", "A", "nominal", dict(score=-3, aln_len=1, matches=0, gap_opens=0),
         "W/A -3 beats two gaps -22"),
        ("global", "W", "A", "as_called", dict(score=-3, aln_len=1, matches=0, gap_opens=0),
         "W/A -3 beats two gaps -4"),
        ("global", "", "AAA", "nominal", dict(score=-15, aln_len=3, matches=0, gap_opens=1),
         "empty V: -11 - 2 - 2"),
        ("global", "", "AAA", "as_called", dict(score=-6, aln_len=3, matches=0, gap_opens=1),
         "empty V: three reopened positions, one run"),
        ("local", "AW", "TW", "nominal",
         dict(score=11, aln_len=1, matches=1, gap_opens=0, beg_v=1, end_v=2, beg_h=1, end_h=2),
         "A/T scores 0: a prefix of score 0 is not part of the local alignment"),
    ]
    for kind, v, h, g, exp, why in hand:
        first, ext = gaps[g]
        cases.append(dict(source="hand", kind=kind, v=v, h=h, gap_first=first, gap_ext=ext,
                          expected=exp, derivation=why))
    # X-drop: only the diagonal survives (gap -1000); the extension runs to the
    # last live anti-diagonal, past the best cell (SeqAn's longest extension)
    cases.append(dict(
        source="hand", kind="xdrop_extend", v="ACDEFGWWPPPP", h="ACDEFGWWCCCC",
        xdrop_gap=-1000, xdrop=10, seed=[0, 6, 0, 6],
        expected=dict(bh=0, eh=11, bv=0, ev=11),
        derivation="diagonal 11, 22, 19, 16, 13, 10; threshold 22 - 10 = 12 kills 10 at "
                   "anti-diagonal 12, odd anti-diagonals are all gaps (dead), so the last "
                   "live cell two anti-diagonals back is (5, 5): extension by 5, not 2"))
    cases.append(dict(
        source="hand", kind="xdrop_extend", v="ACDEFGHIKL", h="ACDEFGHIKL", xdrop_gap=-2,
        xdrop=49, seed=[3, 9, 3, 9], expected=dict(bh=0, eh=10, bv=0, ev=10),
        derivation="identical sequences: both extensions reach the sequence ends"))
    cases.append(dict(
        source="hand", kind="xdrop_extend", v="WWWACDEFG", h="PPPPPACDEFG", xdrop_gap=-1000,
        xdrop=10, seed=[5, 11, 3, 9], expected=dict(bh=3, eh=11, bv=1, ev=9),
        derivation="seed at the ends on the right (no suffix); left W/P -4 three times: "
                   "-4 >= -10 live, -8 live, -12 dead; the end is the best cell of the last "
                   "live anti-diagonal, (2, 2) with -8, even though it scores below the "
                   "seed: bh 5 - 2 = 3, bv 3 - 2 = 1"))
    # ---- exhaustive
    rng = random.Random(7)
    alpha = "ARNDCQEGHILKMFPSTWYV"
    for t in range(160):
        v = "".join(rng.choice(alpha) for _ in range(rng.randint(0, 4)))
        h = "".join(rng.choice(alpha) for _ in range(rng.randint(0, 4)))
        g = "nominal" if t % 2 == 0 else "as_called"
        first, ext = gaps[g]
        if t % 4 < 2:
            sc, stats = brute_global(v, h, first, ext)
            exp = dict(score=sc)
            if len(stats) == 1:
                L, M, G = next(iter(stats))
                exp.update(aln_len=L, matches=M, gap_opens=G)
            cases.append(dict(source="exhaustive", kind="global", v=v, h=h, gap_first=first,
                              gap_ext=ext, expected=exp))
        else:
            sc, keys = brute_local(v, h, first, ext)
            exp = dict(score=sc)
            if sc == 0:
                exp.update(aln_len=0, matches=0, gap_opens=0, empty=1)
            elif len(keys) == 1:
                L, M, G, (i0, i1, j0, j1) = next(iter(keys))
                exp.update(aln_len=L, matches=M, gap_opens=G, beg_v=i0, end_v=i1, beg_h=j0,
                           end_h=j1)
            cases.append(dict(source="exhaustive", kind="local", v=v, h=h, gap_first=first,
                              gap_ext=ext, expected=exp))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat.json")
    with open(out, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "matrix": "BLOSUM62",
                   "cases": cases}, f, indent=1)
    print("wrote", out, len(cases), "cases")


if __name__ == "__main__":
    main()
