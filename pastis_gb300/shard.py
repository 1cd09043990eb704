"""Sharding of a candidate-pair batch over ranks (one GPU per rank).

The alignment stage is rank-local in PASTIS: each rank aligns the nonzeros of
its own block of the candidate matrix (src/DistPWRunner.cpp:81 works on
C.seqptr() only) and no data crosses ranks inside the stage.  Here a batch is
cut into contiguous pair ranges of nearly equal DP work (sum of m*n), so
ranks finish together; results stay on their rank, as PASTIS's per-rank
triples do, and are concatenated in rank order when one process needs them.
"""
import numpy as np


def pair_cost(pairs, lengths, bl_roff=0, bl_coff=0):
    """DP cells m*n of every pair (the SW work; an upper bound for X-drop)."""
    L = np.asarray(lengths, dtype=np.int64)
    return L[pairs["row"].astype(np.int64) + bl_roff] * L[pairs["col"].astype(np.int64) + bl_coff]


def balanced_ranges(cost, nparts):
    """Cut [0, len(cost)) into nparts contiguous ranges of nearly equal total
    cost.  Returns a list of (begin, end)."""
    cost = np.asarray(cost, dtype=np.float64)
    n = len(cost)
    if nparts <= 1 or n == 0:
        return [(0, n)] + [(n, n)] * max(0, nparts - 1)
    c = np.concatenate([[0.0], np.cumsum(cost)])
    total = c[-1]
    cuts = [0]
    for k in range(1, nparts):
        cuts.append(int(np.searchsorted(c, total * k / nparts, side="left")))
    cuts.append(n)
    cuts = np.maximum.accumulate(np.clip(cuts, 0, n))
    return [(int(cuts[k]), int(cuts[k + 1])) for k in range(nparts)]


def my_range(cost, rank, world):
    return balanced_ranges(cost, world)[rank]
