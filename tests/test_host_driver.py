"""The C++ batch driver pw_aln_batch (mirror of src/DistPWRunner.cpp:25-165) on
CPU, with the oracle plugged in as the aligner through the callback hook:
k-mer threshold prune, --bsz batching (including the empty trailing batch),
block offsets, and the post-prune of entries whose score_aln is 0."""
import numpy as np
import pytest


def _block(seed=1, nseq=40, nnz=300):
    rng = np.random.default_rng(seed)
    from oracle import oracle as O
    letters = np.frombuffer(O.LETTERS[:20].encode(), dtype=np.uint8)
    seqs = []
    for i in range(nseq):
        if i % 2 and seqs:
            s = seqs[-1].copy()
            mut = rng.random(len(s)) < 0.25
            s[mut] = letters[rng.integers(0, 20, mut.sum())]
        else:
            s = letters[rng.integers(0, 20, rng.integers(20, 90))]
        seqs.append(s)
    offs = np.concatenate([[0], np.cumsum([len(s) for s in seqs])]).astype(np.uint64)
    res = np.concatenate(seqs)
    rows = rng.integers(0, nseq - 4, nnz).astype(np.uint64)
    cols = rows + rng.integers(0, 4, nnz).astype(np.uint64)
    order = np.lexsort((rows, cols))
    rows, cols = rows[order], cols[order]
    return res, offs, rows, cols, rng


def _oracle_cb(O, mode, res, offs, p):
    codes = O.encode(bytes(res))

    def cb(pairs, ro, co):
        out = O.batch(mode, codes, offs, codes, offs, pairs, p, bl_roff=ro, bl_coff=co,
                      nthreads=2)
        return out["score_aln"]
    return cb


@pytest.mark.parametrize("batch_sz", [1, 7, 50, 299, 300, 10 ** 10])
def test_batches_and_prunes_xdrop(native, oracle_mod, batch_sz):
    from pastis_gb300 import capi
    O = oracle_mod
    res, offs, rows, cols, rng = _block()
    vals = np.zeros(len(rows), dtype=capi.KMERLOC_DTYPE)
    vals["count"] = rng.integers(1, 4, len(rows))
    vals["score"] = rng.integers(-1, 30, len(rows))
    L = np.diff(offs).astype(int)
    vals["first_r"] = [rng.integers(0, L[r] - 6) for r in rows]
    vals["first_c"] = [rng.integers(0, L[c] - 6) for c in cols]
    vals["score_aln"] = 0.5  # stale values must be overwritten
    p = O.make_params(gap_first=-2, gap_ext=-11, xdrop_gap=-11)
    ckthr, mosthr = 1, 3.0
    r2, c2, v2, st = capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, res, offs,
                                      batch_sz=batch_sz, ckthr=ckthr, mosthr=mosthr,
                                      callback=_oracle_cb(O, 1, res, offs, p))
    keep = ~((vals["count"] <= ckthr) | (vals["score"] <= mosthr))
    assert st["nnz_in"] == len(rows) and st["nnz_kmer_thr"] == keep.sum()
    n = int(keep.sum())
    assert st["batches"] == n // min(batch_sz, 10 ** 10) + 1
    assert st["empty_batches"] == (1 if n % batch_sz == 0 else 0)
    # expected: oracle on the kept entries, then drop score_aln == 0
    pr = np.zeros(n, dtype=O.PAIR_DTYPE)
    pr["row"], pr["col"] = rows[keep], cols[keep]
    pr["rs0"], pr["cs0"] = vals["first_r"][keep], vals["first_c"][keep]
    pr["count"] = vals["count"][keep]
    exp = O.batch(1, O.encode(bytes(res)), offs, O.encode(bytes(res)), offs, pr, p)
    ok = exp["score_aln"] != 0
    assert st["nnz_aln"] == ok.sum()
    assert (r2 == rows[keep][ok]).all() and (c2 == cols[keep][ok]).all()
    assert (v2["score_aln"] == exp["score_aln"][ok]).all()


def test_sw_block_offsets(native, oracle_mod):
    """bl_roffset / bl_coffset shift the sequence indices (PWAlign.hpp:47-52)."""
    from pastis_gb300 import capi
    O = oracle_mod
    res, offs, rows, cols, rng = _block(seed=2)
    rows = rows % 10
    cols = cols % 10
    vals = np.zeros(len(rows), dtype=capi.KMERLIGHT_DTYPE)
    vals["count"] = 2
    p = O.make_params()
    r2, c2, v2, st = capi.pw_aln_batch(capi.MODE_SW, rows, cols, vals, res, offs, bl_roff=20,
                                      bl_coff=25, batch_sz=64,
                                      callback=_oracle_cb(O, 0, res, offs, p))
    pr = np.zeros(len(rows), dtype=O.PAIR_DTYPE)
    pr["row"], pr["col"] = rows, cols
    exp = O.batch(0, O.encode(bytes(res)), offs, O.encode(bytes(res)), offs, pr, p, bl_roff=20,
                  bl_coff=25)
    ok = exp["score_aln"] != 0
    assert st["nnz_aln"] == ok.sum()
    assert (v2["score_aln"] == exp["score_aln"][ok]).all()


def test_empty_block(native):
    from pastis_gb300 import capi
    res = np.frombuffer(b"ACDEFG", dtype=np.uint8)
    offs = np.array([0, 6], dtype=np.uint64)
    called = []
    r2, c2, v2, st = capi.pw_aln_batch(capi.MODE_SW, [], [], np.zeros(0, capi.KMERLIGHT_DTYPE),
                                      res, offs, callback=lambda *a: called.append(1))
    assert st["nnz_in"] == 0 and st["batches"] == 0 and not called


def test_matrix_market_writer(native, tmp_path):
    """1-based coordinates, the header PASTIS's --align-file carries, values
    that read back to the same float; out-of-range triples rejected."""
    import numpy as np
    import pytest
    from pastis_gb300 import capi
    path = tmp_path / "sim.mtx"
    vals = np.array([0.5, 0.123456789, 1.0 / 3.0], dtype=np.float32)
    capi.write_mm(path, 10, 12, [0, 9, 3], [11, 0, 3], vals)
    lines = path.read_text().splitlines()
    assert lines[0] == "%%MatrixMarket matrix coordinate real general"
    assert lines[1] == "10 12 3"
    got = [ln.split() for ln in lines[2:]]
    assert [(int(a), int(b)) for a, b, _ in got] == [(1, 12), (10, 1), (4, 4)]
    assert np.array_equal(np.array([float(v) for _, _, v in got], dtype=np.float32), vals)
    with pytest.raises(capi.PgError):
        capi.write_mm(path, 10, 12, [10], [0], [1.0])


def _xdrop_block(O, seed=3):
    from pastis_gb300 import capi
    res, offs, rows, cols, rng = _block(seed=seed, nnz=400)
    vals = np.zeros(len(rows), dtype=capi.KMERLOC_DTYPE)
    vals["count"] = rng.integers(1, 4, len(rows))
    vals["score"] = rng.integers(-1, 30, len(rows))
    L = np.diff(offs).astype(int)
    vals["first_r"] = [rng.integers(0, L[r] - 6) for r in rows]
    vals["first_c"] = [rng.integers(0, L[c] - 6) for c in cols]
    return res, offs, rows, cols, vals


@pytest.mark.parametrize("stop_after", [1, 3, 5])
def test_resume_after_a_stop_between_batches(native, oracle_mod, stop_after):
    """The run is stopped on the host after batch k (as a job stopped between
    batches); a second call from next_batch on the written-back triples ends
    with the LocalMat an uninterrupted run gives."""
    from pastis_gb300 import capi
    O = oracle_mod
    res, offs, rows, cols, vals = _xdrop_block(O)
    p = O.make_params(gap_first=-2, gap_ext=-11, xdrop_gap=-11)
    cb = _oracle_cb(O, 1, res, offs, p)
    kw = dict(batch_sz=40, ckthr=1, mosthr=3.0, callback=cb)
    full = capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, res, offs, **kw)
    assert full[3]["complete"] and full[3]["next_batch"] == full[3]["batches"]
    seen = []

    def stop(b, beg, end):
        seen.append((b, beg, end))
        return b + 1 < stop_after

    r1, c1, v1, s1 = capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, res, offs,
                                      on_batch=stop, **kw)
    assert not s1["complete"] and s1["next_batch"] == stop_after
    assert seen[-1][0] == stop_after - 1 and s1["last_end"] == seen[-1][2] == 40 * stop_after
    # nothing after the k-mer prune ran: every surviving nonzero is still there
    assert s1["nnz_aln"] == s1["nnz_kmer_thr"] == len(r1)
    aligned = v1["score_aln"][:s1["last_end"]]
    assert (v1["score_aln"][s1["last_end"]:] == 0).all() and (aligned != 0).any()
    r2, c2, v2, s2 = capi.pw_aln_batch(capi.MODE_XDROP, r1, c1, v1, res, offs,
                                      start_batch=s1["next_batch"], **kw)
    assert s2["complete"] and s2["batches"] == full[3]["batches"] - stop_after
    assert (r2 == full[0]).all() and (c2 == full[1]).all()
    assert v2.tobytes() == full[2].tobytes()


def test_failed_batch_surfaces_its_code_and_keeps_earlier_batches(native, oracle_mod):
    """An aligner error in batch 2 (the host-side stand-in for a failed upload
    or a failed pg_align) returns its code; batches 0 and 1 keep their
    score_aln, and a resume from batch 2 completes the stage."""
    from pastis_gb300 import capi
    O = oracle_mod
    res, offs, rows, cols, vals = _xdrop_block(O, seed=4)
    p = O.make_params(gap_first=-2, gap_ext=-11, xdrop_gap=-11)
    good = _oracle_cb(O, 1, res, offs, p)
    calls = []

    def flaky(pairs, ro, co):
        calls.append(len(pairs))
        if len(calls) == 3:
            return capi.PG_ERR_CUDA
        return good(pairs, ro, co)

    kw = dict(batch_sz=50, ckthr=1, mosthr=3.0)
    full = capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, res, offs, callback=good, **kw)
    with pytest.raises(capi.BatchError) as ei:
        capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, res, offs, callback=flaky, **kw)
    e = ei.value
    assert e.code == capi.PG_ERR_CUDA
    r1, c1, v1, s1 = e.partial
    assert s1["next_batch"] == 2 and s1["last_end"] == 100 and not s1["complete"]
    # the earlier batches' results equal the uninterrupted run's for the same entries
    ref = capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, res, offs, callback=good,
                            on_batch=lambda b, beg, end: b < 1, **kw)
    assert v1[:100].tobytes() == ref[2][:100].tobytes()
    r2, c2, v2, s2 = capi.pw_aln_batch(capi.MODE_XDROP, r1, c1, v1, res, offs, callback=good,
                                      start_batch=2, **kw)
    assert s2["complete"] and v2.tobytes() == full[2].tobytes()
    assert (r2 == full[0]).all() and (c2 == full[1]).all()


def test_callback_exception_is_a_state_error(native, oracle_mod):
    from pastis_gb300 import capi
    res, offs, rows, cols, vals = _xdrop_block(oracle_mod, seed=5)

    def boom(pairs, ro, co):
        raise ValueError("host-side failure")

    with pytest.raises(capi.BatchError) as ei:
        capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, res, offs, callback=boom,
                          batch_sz=64)
    assert ei.value.code == capi.PG_ERR_STATE and ei.value.partial[3]["next_batch"] == 0
