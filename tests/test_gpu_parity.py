"""GPU kernels (through the C ABI) against the CPU oracle, every output field
bit for bit: score, coordinates, columns, matches, gap runs, identity,
score_aln, flags, seed choice and the per-pair cell count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["score", "aln_len", "matches", "gap_opens", "beg_h", "end_h", "beg_v", "end_v",
          "identity", "score_aln", "seed_used", "flags", "cells"]


def oracle_params(O, cfg):
    from pastis_gb300 import capi
    first, ext, xg = capi.resolved_gaps(cfg)
    return O.make_params(gap_first=first, gap_ext=ext, xdrop_gap=xg, xdrop=cfg.xdrop,
                         seed_len=cfg.seed_len, seed_count=cfg.seed_count, tie=cfg.tie,
                         flags=cfg.flags, cov_thr=cfg.cov_thr, ani_thr=cfg.ani_thr)


def assert_same(got, exp, pairs=None):
    bad = np.zeros(len(got), dtype=bool)
    for f in FIELDS:
        a, b = got[f], exp[f]
        if f in ("identity", "score_aln"):
            a, b = a.view(np.uint32), b.view(np.uint32)
        bad |= a != b
    if bad.any():
        i = int(np.flatnonzero(bad)[0])
        diff = {f: (got[f][i], exp[f][i]) for f in FIELDS if got[f][i] != exp[f][i]}
        raise AssertionError("%d of %d pairs differ; first #%d %s pair=%s" % (
            bad.sum(), len(got), i, diff, None if pairs is None else pairs[i]))


def run_both(mode, w, cfg, O, pairs=None, roff=0, coff=0, share=True):
    from pastis_gb300 import capi
    pairs = w.pairs if pairs is None else pairs
    ctx = capi.Context(cfg)
    ascii_ = w.ascii
    ctx.set_seqs(0, ascii_, w.offs)
    if share:
        ctx.share_row_seqs()
    else:
        ctx.set_seqs(1, ascii_, w.offs)
    got = ctx.align(pairs, roff, coff)
    # traceback form by default: X-drop: k_xtask_hist, k_xtask_bucket, k_xdr,
    # k_xd_wide, k_hist, k_bucket, k_dirsize, k_ga_dir, k_ga_pair, k_tb_ga; SW:
    # k_hist, k_bucket, k_dirsize, k_sw_dir, k_tb_sw; one more (the checked
    # 16-bit pass) where long regions need it
    base = 10 if mode == capi.MODE_XDROP else 5
    assert ctx.last_launches() in (base, base + 1)
    codes = O.encode(bytes(ascii_))
    exp = O.batch(mode, codes, w.offs, codes, w.offs, pairs, oracle_params(O, cfg),
                  bl_roff=roff, bl_coff=coff)
    ctx.close()
    return got, exp


@pytest.fixture(scope="module")
def sw_small(native):
    from pastis_gb300 import synth
    return synth.generate("sw100k", seed=101, scale=0.02)


@pytest.fixture(scope="module")
def xd_small(native):
    from pastis_gb300 import synth
    return synth.generate("xdrop1m", seed=202, scale=0.005)


@pytest.mark.parametrize("tie", [0, 1, 2, 3])
@pytest.mark.parametrize("gaps", [0, 1])
def test_sw_parity(sw_small, oracle_mod, tie, gaps):
    from pastis_gb300 import capi
    cfg = capi.config(capi.MODE_SW, tie=tie, gap_semantics=gaps)
    got, exp = run_both(0, sw_small, cfg, oracle_mod)
    assert_same(got, exp, sw_small.pairs)
    assert (got["flags"] & capi.RF_PASSED).any()


@pytest.mark.parametrize("tie", [0, 1, 2, 3])
@pytest.mark.parametrize("gaps", [0, 1])
def test_xdrop_parity(xd_small, oracle_mod, tie, gaps):
    from pastis_gb300 import capi
    cfg = capi.config(capi.MODE_XDROP, tie=tie, gap_semantics=gaps)
    got, exp = run_both(1, xd_small, cfg, oracle_mod)
    assert_same(got, exp, xd_small.pairs)
    assert (got["seed_used"] == 1).any() and (got["flags"] & capi.RF_PASSED).any()


@pytest.mark.parametrize("gaps,xdrop", [(0, 49), (1, 49), (0, 200), (0, 10), (0, 0)])
def test_register_window_extension(xd_small, oracle_mod, gaps, xdrop):
    """The register-window extension gives the oracle's results, also where
    most windows overflow it (the nominal gaps, X = 200) and the warp kernel
    takes the rest."""
    from pastis_gb300 import capi
    w = xd_small
    cfg = capi.config(capi.MODE_XDROP, gap_semantics=gaps, xdrop=xdrop)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    ctx.set_tuning(xd_stepped=2)
    got = ctx.align(w.pairs)
    # order (2), k_xdr, k_xd_wide, then the traceback form's k_hist, k_bucket,
    # k_dirsize, k_ga_dir, k_ga_pair, k_tb_ga
    assert ctx.last_launches() in (10, 11)
    ctx.close()
    O = oracle_mod
    codes = O.encode(bytes(w.ascii))
    exp = O.batch(1, codes, w.offs, codes, w.offs, w.pairs, oracle_params(O, cfg))
    assert_same(got, exp, w.pairs)


@pytest.mark.parametrize("flags,xdrop,seed_count", [(1, 49, 2), (0, 10, 2), (0, 200, 2),
                                                      (0, 49, 1), (0, 0, 2)])
def test_xdrop_switches(xd_small, oracle_mod, flags, xdrop, seed_count):
    from pastis_gb300 import capi
    cfg = capi.config(capi.MODE_XDROP, flags=flags, xdrop=xdrop, seed_count=seed_count)
    got, exp = run_both(1, xd_small, cfg, oracle_mod)
    assert_same(got, exp, xd_small.pairs)


def test_long_sequences_row_blocks(native, oracle_mod):
    """Lengths up to 5000: many row blocks through the per-warp scratch row."""
    from pastis_gb300 import capi, synth
    w = synth.generate("uneven10m", seed=303, scale=0.00003)
    for mode in (capi.MODE_SW, capi.MODE_XDROP):
        cfg = capi.config(mode)
        got, exp = run_both(mode, w, cfg, oracle_mod)
        assert_same(got, exp, w.pairs)
    assert w.lengths().max() > 1000


def test_wide_band_uses_global_ring(native, oracle_mod):
    """Cheap gaps and a huge X make the X-drop band wider than the shared ring."""
    from pastis_gb300 import capi, synth
    w = synth.generate("xdrop1m", seed=404, scale=0.0003, len_median=900.0, len_max=3000)
    cfg = capi.config(capi.MODE_XDROP, gap_semantics=capi.GAPS_NOMINAL, xdrop=5000)
    got, exp = run_both(1, w, cfg, oracle_mod)
    assert_same(got, exp, w.pairs)


def _toy(seqs):
    from pastis_gb300 import synth
    from oracle import oracle as O
    codes = [O.encode(s) for s in seqs]
    offs = np.concatenate([[0], np.cumsum([len(c) for c in codes])]).astype(np.uint64)
    seq = np.concatenate(codes) if codes else np.zeros(0, np.uint8)
    return synth.Workload("toy", seq, offs, np.zeros(0, dtype=O.PAIR_DTYPE), np.zeros(0, np.uint8),
                          np.zeros(0, np.uint8), np.zeros(len(seqs), np.uint32))


EDGE_SEQS = ["", "W", "A", "ACDEFGHIKLMNPQRSTVWY", "acdefghiklmnpqrstvwy", "BZX*JBZX*J",
             "UUOO??ACDE", "W" * 300, "MKVLAAGIVGLLLAC" * 20, "PPPPPPPPPP"]


@pytest.mark.parametrize("mode", [0, 1])
def test_edge_cases(native, oracle_mod, mode):
    """Empty and length-1 sequences, non-standard and lower-case letters, seeds
    at (0,0), seeds past the sequence end, identical pairs."""
    from pastis_gb300 import capi
    O = oracle_mod
    w = _toy(EDGE_SEQS)
    n = len(EDGE_SEQS)
    L = np.diff(w.offs).astype(int)
    rows, cols = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    pairs = np.zeros(n * n * 3, dtype=O.PAIR_DTYPE)
    pairs["row"] = np.tile(rows.ravel(), 3)
    pairs["col"] = np.tile(cols.ravel(), 3)
    k = n * n
    pairs["count"] = 1
    # block 1: seeds at (0, 0); block 2: second seed mid-way; block 3: seeds past the end
    pairs["rs1"][k:2 * k] = L[pairs["row"][k:2 * k]] // 2
    pairs["cs1"][k:2 * k] = L[pairs["col"][k:2 * k]] // 2
    pairs["count"][k:2 * k] = 2
    pairs["rs0"][2 * k:] = L[pairs["row"][2 * k:]] + 3
    pairs["cs0"][2 * k:] = np.maximum(L[pairs["col"][2 * k:]] - 2, 0)
    cfg = capi.config(mode)
    got, exp = run_both(mode, w, cfg, O, pairs=pairs)
    assert_same(got, exp, pairs)
    if mode == 1:
        assert (got["flags"] & capi.RF_BAD_SEED).any()


def test_block_offsets_and_separate_columns(sw_small, oracle_mod):
    from pastis_gb300 import capi
    nseq = len(sw_small.offs) - 1
    pairs = sw_small.pairs[:500].copy()
    pairs["row"] = pairs["row"] % (nseq - 37)
    pairs["col"] = pairs["col"] % (nseq - 123)
    cfg = capi.config(capi.MODE_SW)
    got, exp = run_both(0, sw_small, cfg, oracle_mod, pairs=pairs, roff=37, coff=123,
                        share=False)
    assert_same(got, exp, pairs)


def test_errors_and_empty_batch(sw_small, native):
    from pastis_gb300 import capi
    ctx = capi.Context(capi.config(capi.MODE_SW))
    with pytest.raises(capi.PgError) as e:
        ctx.align(sw_small.pairs[:4])
    assert e.value.code == capi.PG_ERR_STATE
    ctx.set_seqs(0, sw_small.ascii, sw_small.offs)
    ctx.share_row_seqs()
    out = ctx.align(sw_small.pairs[:0])
    assert len(out) == 0 and ctx.last_launches() == 0
    bad = sw_small.pairs[:8].copy()
    bad["row"][3] = len(sw_small.offs) + 5
    with pytest.raises(capi.PgError) as e:
        ctx.align(bad)
    assert e.value.code == capi.PG_ERR_ARG
    # the context stays usable after an error
    ok = ctx.align(sw_small.pairs[:8])
    assert (ok["cells"] > 0).all()
    too_long = np.full(65536, ord("A"), dtype=np.uint8)
    with pytest.raises(capi.PgError) as e:
        ctx.set_seqs(0, too_long, np.array([0, 65536], dtype=np.uint64))
    assert e.value.code == capi.PG_ERR_RANGE


def test_max_length_sequence(native, oracle_mod):
    """A 65535-residue sequence (the u16 limit of PASTIS, FastaData.hpp:109)."""
    from pastis_gb300 import capi
    O = oracle_mod
    rng = np.random.default_rng(9)
    letters = "ARNDCQEGHILKMFPSTWYV"
    big = "".join(rng.choice(list(letters), 65535))
    small = big[30000:30040]
    w = _toy([big, small])
    pairs = np.zeros(2, dtype=O.PAIR_DTYPE)
    pairs["row"] = [0, 1]
    pairs["col"] = [1, 0]
    pairs["rs0"], pairs["cs0"] = [30010, 10], [10, 30010]
    pairs["count"] = 1
    for mode in (0, 1):
        got, exp = run_both(mode, w, capi.config(mode), O, pairs=pairs)
        assert_same(got, exp, pairs)


def test_cpp_driver_on_gpu(sw_small, oracle_mod):
    """The C++ pw_aln_batch with the GPU aligner equals the oracle-driven run."""
    from pastis_gb300 import capi
    O = oracle_mod
    w = sw_small
    pairs = w.pairs[:1500]
    rows = pairs["row"].astype(np.uint64)
    cols = pairs["col"].astype(np.uint64)
    vals = np.zeros(len(pairs), dtype=capi.KMERLOC_DTYPE)
    vals["count"] = pairs["count"]
    vals["score"] = pairs["score"]
    vals["first_r"], vals["first_c"] = pairs["rs0"], pairs["cs0"]
    vals["second_r"], vals["second_c"] = pairs["rs1"], pairs["cs1"]
    cfg = capi.config(capi.MODE_XDROP)
    r_gpu, c_gpu, v_gpu, st = capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, w.ascii, w.offs,
                                               batch_sz=400, ckthr=0, cfg=cfg)
    codes = O.encode(bytes(w.ascii))
    p = oracle_params(O, cfg)
    r_cpu, c_cpu, v_cpu, st2 = capi.pw_aln_batch(
        capi.MODE_XDROP, rows, cols, vals, w.ascii, w.offs, batch_sz=400, ckthr=0,
        callback=lambda pr, ro, co: O.batch(1, codes, w.offs, codes, w.offs, pr, p, ro, co)["score_aln"])
    assert st["nnz_aln"] == st2["nnz_aln"] and st["batches"] == 4
    assert (r_gpu == r_cpu).all() and (c_gpu == c_cpu).all()
    assert (v_gpu["score_aln"].view(np.uint32) == v_cpu["score_aln"].view(np.uint32)).all()
    # stopped on the host after batch 1 and resumed from batch 2 with the GPU
    # aligner: the same final triples
    r1, c1, v1, s1 = capi.pw_aln_batch(capi.MODE_XDROP, rows, cols, vals, w.ascii, w.offs,
                                      batch_sz=400, ckthr=0, cfg=cfg,
                                      on_batch=lambda b, beg, end: b < 1)
    assert s1["next_batch"] == 2 and not s1["complete"]
    r2, c2, v2, s2 = capi.pw_aln_batch(capi.MODE_XDROP, r1, c1, v1, w.ascii, w.offs,
                                      batch_sz=400, ckthr=0, cfg=cfg, start_batch=2)
    assert s2["complete"] and (r2 == r_gpu).all() and (c2 == c_gpu).all()
    assert v2.tobytes() == v_gpu.tobytes()


@pytest.mark.parametrize("mode", [0, 1])
def test_tuning_and_graph_replay_keep_results(native, oracle_mod, mode):
    """Every launch tuning (grid sizes, bucket order, rows per lane, graph
    capture and replay) gives the oracle's results byte for byte."""
    import torch
    from pastis_gb300 import capi, synth
    w = synth.generate("sw100k" if mode == capi.MODE_SW else "xdrop1m", seed=211,
                       scale=0.01 if mode == capi.MODE_SW else 0.004)
    cfg = capi.config(mode)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    O = oracle_mod
    codes = O.encode(bytes(w.ascii))
    exp = O.batch(mode, codes, w.offs, codes, w.offs, w.pairs, oracle_params(O, cfg))
    kernels = 5 if mode == capi.MODE_XDROP else 3
    for t in ({}, {"bucket_order": 0}, {"rows_max": 3}, {"rows_max": 1, "dp_blocks_per_sm": 1},
              {"xd_blocks_per_sm": 2}, {"graph": 1}, {"graph": 1, "bucket_order": 0},
              {"xd_int16": 1}, {"xd_int16": 1, "graph": 1}, {"dp_traceback": 1},
              {"dp_traceback": 1, "dir_arena_mb": 1}, {"dp_traceback": 1, "rows_max": 3},
              {"dp_traceback": 1, "bucket_order": 0, "graph": 1}, {"dp_traceback": 2},
              {"dp_traceback": 2, "dir_arena_mb": 1}, {"dp_traceback": 2, "rows_max": 3},
              {"dp_traceback": 2, "bucket_order": 0}, {"dp_traceback": 3},
              {"dp_traceback": 3, "dir_arena_mb": 1}, {"dp_traceback": 3, "rows_max": 3},
              {"dp_traceback": 3, "bucket_order": 0}, {"xd_stepped": 0}, {"xd_stepped": 1}, {"xd_stepped": 2},
              {"xd_stepped": 0, "xd_blocks_per_sm": 2}):
        ctx.set_tuning(capi.default_tuning(), **t)
        for rep in range(2):                 # the second call replays the graph
            got = ctx.align(w.pairs)
            assert_same(got, exp, w.pairs)
            ext_ms, aln_ms = ctx.kernel_ms()     # the timing events survive a replay
            assert ext_ms >= 0 and aln_ms > 0, t
        want = kernels if t.get("bucket_order", 1) else kernels - 2
        # the extension tasks' longest-first order (two launches) goes with
        # the bucket order and the register-window extension kernel
        if (mode == capi.MODE_XDROP and t.get("bucket_order", 1) and not t.get("xd_int16")
                and t.get("xd_stepped", -1) in (-1, 2)):
            want += 2
        if not t.get("dp_traceback"):
            assert ctx.last_launches() == want, t
    # device entry point with graph replay on a caller stream
    n = len(w.pairs)
    d_pairs = torch.from_numpy(w.pairs.view(np.uint8).copy()).cuda()
    d_out = torch.empty(n * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda:0")
    s = torch.cuda.Stream()
    for _ in range(3):
        d_out.zero_()
        torch.cuda.synchronize()
        ctx.align_device(d_pairs.data_ptr(), n, d_out.data_ptr(), s.cuda_stream)
        s.synchronize()
        got = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
        assert_same(got, exp, w.pairs)
    with pytest.raises(capi.PgError):
        ctx.set_tuning(rows_max=9)
    with pytest.raises(capi.PgError):
        ctx.set_tuning(graph=2)
    with pytest.raises(capi.PgError):
        ctx.set_tuning(dp_traceback=4)
    ctx.close()


def test_int16_extension_saturation_reruns_in_32_bits(native, oracle_mod):
    """Pairs of identical 3500-residue sequences rich in W and C push the
    X-drop score past the 16-bit lanes' limit (30000): those extensions are
    rerun in 32 bits and every result still equals the oracle's."""
    from pastis_gb300 import capi
    rng = np.random.default_rng(17)
    letters = np.frombuffer(b"WCWCWYHW", dtype=np.uint8)
    seqs = [letters[rng.integers(0, len(letters), 3500)] for _ in range(3)]
    seqs.append(np.frombuffer(b"ACDEFGHIKLMNPQRSTVWY" * 20, dtype=np.uint8))
    ascii_ = np.concatenate(seqs)
    offs = np.cumsum([0] + [len(x) for x in seqs]).astype(np.uint64)
    pairs = np.zeros(4, dtype=capi.PAIR_DTYPE)
    pairs["row"] = [0, 1, 2, 3]
    pairs["col"] = [0, 1, 2, 3]
    pairs["rs0"] = pairs["cs0"] = [1700, 10, 3000, 50]
    pairs["rs1"] = pairs["cs1"] = [100, 3400, 3000, 300]
    pairs["count"] = 2
    cfg = capi.config(capi.MODE_XDROP)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, ascii_, offs)
    ctx.share_row_seqs()
    ctx.set_tuning(xd_int16=1)
    got = ctx.align(pairs)
    O = oracle_mod
    codes = O.encode(bytes(ascii_))
    exp = O.batch(capi.MODE_XDROP, codes, offs, codes, offs, pairs, oracle_params(O, cfg))
    assert_same(got, exp, pairs)
    assert got["score"][0] > 30000
    ctx.close()


@pytest.mark.parametrize("tie", [0, 1, 2, 3])
@pytest.mark.parametrize("gaps", [0, 1])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("form", [1, 2, 3])
def test_traceback_form_parity(sw_small, xd_small, oracle_mod, tie, gaps, mode, form):
    """The traceback form of the DP (direction nibbles in HBM, then a walk
    back), on 32-bit lanes (form 1), 16-bit lanes (form 2) and 16-bit lanes
    with two regions per warp (form 3), gives the oracle's results under every
    tie policy and gap model."""
    from pastis_gb300 import capi
    w = sw_small if mode == capi.MODE_SW else xd_small
    cfg = capi.config(mode, tie=tie, gap_semantics=gaps)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    ctx.set_tuning(dp_traceback=form)
    got = ctx.align(w.pairs)
    O = oracle_mod
    codes = O.encode(bytes(w.ascii))
    exp = O.batch(mode, codes, w.offs, codes, w.offs, w.pairs, oracle_params(O, cfg))
    assert_same(got, exp, w.pairs)
    ctx.close()


def test_traceback_form_long_regions(native, oracle_mod):
    """Regions over 1023 rows and columns (several stripes of 256 rows, the
    wide-statistics case of the other form), both modes, small arena chunks;
    in form 2 the regions over the 16-bit limit (m + n > 2723 with BLOSUM62)
    share the batch with 16-bit ones of several stripes of 64 R rows."""
    from pastis_gb300 import capi, synth
    w = synth.generate("uneven10m", seed=5, scale=0.00003)
    O = oracle_mod
    codes = O.encode(bytes(w.ascii))
    for mode in (capi.MODE_SW, capi.MODE_XDROP):
        cfg = capi.config(mode)
        exp = O.batch(mode, codes, w.offs, codes, w.offs, w.pairs, oracle_params(O, cfg))
        for form in (1, 2, 3):
            ctx = capi.Context(cfg)
            ctx.set_seqs(0, w.ascii, w.offs)
            ctx.share_row_seqs()
            ctx.set_tuning(dp_traceback=form, dir_arena_mb=2)
            got = ctx.align(w.pairs)
            assert_same(got, exp, w.pairs)
            ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_pair_form_row_boundaries(native, oracle_mod, mode):
    """Form 3 runs the 16-bit regions of up to 32 R rows two per warp, each on
    half of it.  Row counts at and around every multiple of 32 up to 256 (and
    past it, on the whole warp), partners of very different column counts,
    enough regions per warp that most find a partner, and a batch of one region
    of each row count (each runs alone); two tie policies."""
    from pastis_gb300 import capi
    O = oracle_mod
    rng = np.random.default_rng(29)
    alpha = np.frombuffer(b"ACDEFGHIKLMNPQRSTVWY", dtype=np.uint8)
    ms = [1, 2, 31, 32, 33, 63, 64, 65, 95, 96, 97, 128, 129, 160, 192, 224, 255, 256, 257, 300]
    ns = [1, 3, 40, 250, 700]
    root = rng.integers(0, 20, 800)
    seqs = []
    for L in ms + ns:
        s = root[:L].copy()
        mut = rng.random(L) < 0.25
        s[mut] = rng.integers(0, 20, int(mut.sum()))
        seqs.append(alpha[s].tobytes().decode())
    w = _toy(seqs)
    npairs = 12000
    pairs = np.zeros(npairs, dtype=O.PAIR_DTYPE)
    pairs["row"] = rng.integers(0, len(ms), npairs)
    pairs["col"] = len(ms) + rng.integers(0, len(ns), npairs)
    pairs["count"] = 1
    single = np.zeros(len(ms), dtype=O.PAIR_DTYPE)
    single["row"] = np.arange(len(ms))
    single["col"] = len(ms) + 3
    single["count"] = 1
    codes = O.encode(bytes(w.ascii))
    for tie in (0, 3):
        cfg = capi.config(mode, tie=tie)
        ctx = capi.Context(cfg)
        ctx.set_seqs(0, w.ascii, w.offs)
        ctx.share_row_seqs()
        ctx.set_tuning(dp_traceback=3)
        for pp in (pairs, single):
            got = ctx.align(pp)
            exp = O.batch(mode, codes, w.offs, codes, w.offs, pp, oracle_params(O, cfg))
            assert_same(got, exp, pp)
        ctx.close()


@pytest.mark.parametrize("form", [2, 3])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("scale", [8, 10])
def test_traceback16_limit_splits_the_batch(sw_small, xd_small, oracle_mod, mode, scale, form):
    """A substitution table scaled by 8 (largest magnitude 88) leaves 16-bit
    lanes only to regions with m + n <= 336, so one batch runs on both lane
    widths; scaled by 10 (magnitude 110) no region qualifies.  Forms 2 and 3
    (form 3 puts the short 16-bit regions two per warp).  Results equal the
    oracle's run with the same table."""
    from pastis_gb300 import capi
    O = oracle_mod
    w = sw_small if mode == capi.MODE_SW else xd_small
    sm = np.ascontiguousarray(O.blosum62().astype(np.int32) * scale).clip(-127, 127).astype(np.int8)
    cfg = capi.config(mode)
    cfg.score_matrix = sm.ctypes.data
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    ctx.set_tuning(dp_traceback=form)
    got = ctx.align(w.pairs)
    codes = O.encode(bytes(w.ascii))
    first, ext, xg = capi.resolved_gaps(cfg)
    p = O.make_params(gap_first=first, gap_ext=ext, xdrop_gap=xg, xdrop=cfg.xdrop,
                      seed_len=cfg.seed_len, seed_count=cfg.seed_count, tie=cfg.tie,
                      flags=cfg.flags, cov_thr=cfg.cov_thr, ani_thr=cfg.ani_thr, sm=sm)
    exp = O.batch(mode, codes, w.offs, codes, w.offs, w.pairs, p)
    assert_same(got, exp, w.pairs)
    lens = np.diff(w.offs.astype(np.int64))
    tot = lens[w.pairs["row"]] + lens[w.pairs["col"]]
    if scale == 8 and mode == capi.MODE_SW:
        assert (tot <= 336).any() and (tot > 336).any()
    ctx.close()



@pytest.mark.parametrize("mode", [0, 1])
def test_checked_16bit_regions(native, oracle_mod, mode):
    """Regions past the provable 16-bit size (m + n > 2723 with BLOSUM62) run
    the checked 16-bit form.  Identical 3500-residue W/C-rich pairs push H
    past 30000, so their DP is redone on 32-bit lanes; long unrelated pairs
    stay in range and finish on 16-bit lanes.  Every result equals the
    oracle's."""
    from pastis_gb300 import capi
    rng = np.random.default_rng(23)
    rich = np.frombuffer(b"WCWCWYHW", dtype=np.uint8)
    std = np.frombuffer(b"ACDEFGHIKLMNPQRSTVWY", dtype=np.uint8)
    seqs = [rich[rng.integers(0, len(rich), 3500)] for _ in range(2)]
    seqs += [std[rng.integers(0, len(std), int(L))] for L in (3000, 2900, 1800, 2600)]
    ascii_ = np.concatenate(seqs)
    offs = np.cumsum([0] + [len(x) for x in seqs]).astype(np.uint64)
    pairs = np.zeros(5, dtype=capi.PAIR_DTYPE)
    pairs["row"] = [0, 1, 2, 3, 4]
    pairs["col"] = [0, 1, 3, 5, 2]
    pairs["rs0"] = pairs["cs0"] = [1700, 10, 5, 100, 50]
    pairs["rs1"] = pairs["cs1"] = [100, 3400, 40, 900, 1200]
    pairs["count"] = 2
    cfg = capi.config(mode)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, ascii_, offs)
    ctx.share_row_seqs()
    assert ctx.get_tuning().dp_traceback == 3
    got = ctx.align(pairs)
    O = oracle_mod
    codes = O.encode(bytes(ascii_))
    exp = O.batch(mode, codes, offs, codes, offs, pairs, oracle_params(O, cfg))
    assert_same(got, exp, pairs)
    assert got["score"][0] > 30000 and got["score"][1] > 30000
    ctx.close()
