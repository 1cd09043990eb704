"""CPU restatement of PASTIS's candidate generation (test infrastructure only).

Follows src/kmer/KmerOps.cpp:31-87 (k-mers of each sequence: every stride-th
position, code by Horner over the alphabet's codes, value = offset and the
k-mer's self score over the alphabet's representative letters), the product
C = A·Aᵀ of src/sim_search.cpp:154-157, the KmerIntersectLoc semiring of
inc/sr.hpp:30-117 and the symmetric prunes of src/sim_search.cpp:172-186 and
:403-412.  It works pair by pair (set intersection of the two sequences' k-mer
tables), independently of the GPU's sort-and-join, so it suits small inputs.

Decisions the reference leaves to CombBLAS's accumulation order, stated here
and in the kernels alike: count is the number of occurrence pairs sharing a
k-mer (a k-mer seen twice in one sequence counts twice), wrapped to 16 bits as
the semiring's ushort sum does; first = offsets of the smallest
(code, row offset, col offset), second = those of the largest, (0, 0) when the
count is 1 (the default-constructed pair of inc/Types.hpp:170-171).
"""
import numpy as np

# murphy10 code of each residue code ARNDCQEGHILKMFPSTWYVBZX*J, and the
# residue code of each murphy10 group's representative letter
MURPHY = [0, 1, 2, 2, 3, 2, 2, 4, 5, 6, 6, 1, 6, 7, 8, 9, 9, 7, 7, 6, 10, 11, 12, 13, 14]
MURPHY_REP = [0, 11, 3, 4, 7, 8, 9, 13, 14, 15, 20, 21, 22, 23, 24]


def alphabet(alph, sm):
    """(code map, base, per-code self score) of PG_ALPH_PROTEIN (0) or
    PG_ALPH_MURPHY10 (1) with the 25 x 25 score table sm."""
    sm = np.asarray(sm).reshape(25, 25)
    if alph == 0:
        return list(range(25)), 25, [int(sm[a, a]) for a in range(25)]
    return MURPHY, 15, [int(sm[r, r]) for r in MURPHY_REP]


def kmer_table(codes, k, stride, cmap, base, cost):
    """{kmer code: (self score, [offsets])} of one sequence."""
    out = {}
    L = len(codes)
    if L < k:
        return out
    for pos in range(0, L - k + 1, stride):
        code = 0
        sc = 0
        for j in range(k):
            a = cmap[int(codes[pos + j])]
            code = code * base + a
            sc += cost[a]
        out.setdefault(code, (sc, []))[1].append(pos)
    return out


def keep_pair(prune, r, c):
    if prune == 1:
        if r == c:
            return False
        odd = ((r ^ c) & 1) != 0
        return (not odd) if r > c else odd
    if prune == 2:
        return r < c
    return True


def candidates(codes, offs, rows, cols, sm, k=6, stride=1, alph=0, prune=0, ckthr=0,
               mosthr=-1):
    """Candidate pairs of rows [r0, r1) x cols [c0, c1) of one sequence set,
    block-relative, in column-major order; a list of dicts with the fields of
    pg_pair."""
    cmap, base, cost = alphabet(alph, sm)
    offs = np.asarray(offs, dtype=np.int64)
    tab = {}

    def table(s):
        if s not in tab:
            tab[s] = kmer_table(codes[offs[s]:offs[s + 1]], k, stride, cmap, base, cost)
        return tab[s]

    out = []
    for c in range(cols[0], cols[1]):
        tc = table(c)
        for r in range(rows[0], rows[1]):
            if not keep_pair(prune, r, c):
                continue
            tr = table(r)
            common = sorted(set(tr) & set(tc))
            if not common:
                continue
            count = sum(len(tr[x][1]) * len(tc[x][1]) for x in common)
            score = max(tr[x][0] for x in common)
            lo, hi = common[0], common[-1]
            first = (min(tr[lo][1]), min(tc[lo][1]))
            last = (max(tr[hi][1]), max(tc[hi][1]))
            cnt16 = count & 0xffff
            if not (cnt16 > ckthr and score > mosthr):
                continue
            out.append({"row": r - rows[0], "col": c - cols[0], "rs0": first[0], "cs0": first[1],
                        "rs1": last[0] if count >= 2 else 0, "cs1": last[1] if count >= 2 else 0,
                        "count": cnt16, "score": score})
    return out
