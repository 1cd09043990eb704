"""GPU against the oracle at the benchmark's sizes: paths that only appear on
large batches (a million regions in bucket order, the direction arena split
into several chunks, residue sets larger than L2, long Smith-Waterman pairs)
are compared field by field like the small cases in test_gpu_parity.py."""
import numpy as np
import pytest

from test_gpu_parity import assert_same, oracle_params

pytestmark = pytest.mark.gpu


def _ctx(cfg, w, **tuning):
    from pastis_gb300 import capi
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    if tuning:
        ctx.set_tuning(**tuning)
    return ctx


def _oracle(O, mode, w, pairs, cfg):
    codes = O.encode(bytes(w.ascii))
    return O.batch(mode, codes, w.offs, codes, w.offs, pairs, oracle_params(O, cfg),
                   nthreads=O.max_threads())


def test_xdrop1m_full_batch(native, oracle_mod):
    """The whole 1M-pair X-drop batch aligned in one call (the benchmark's
    batch, seed 20260101); a random 100k of its pairs checked against the
    oracle."""
    from pastis_gb300 import capi, synth
    w = synth.generate("xdrop1m", seed=20260101)
    assert len(w.pairs) == 1_000_000
    cfg = capi.config(capi.MODE_XDROP)
    ctx = _ctx(cfg, w)
    got = ctx.align(w.pairs)
    ctx.close()
    idx = np.sort(np.random.default_rng(11).choice(len(w.pairs), 100_000, replace=False))
    exp = _oracle(oracle_mod, 1, w, w.pairs[idx], cfg)
    assert_same(got[idx], exp, w.pairs[idx])


@pytest.mark.parametrize("mode", [0, 1])
def test_arena_chunks_on_50k_pairs(native, oracle_mod, mode):
    """A direction-arena cap far below the batch's need runs the 50k-pair batch
    in many chunks; every pair matches the oracle and the uncapped run."""
    from pastis_gb300 import capi, synth
    w = synth.generate("sw100k" if mode == 0 else "xdrop1m", seed=6060,
                       scale=0.5 if mode == 0 else 0.05)
    assert len(w.pairs) == 50_000
    cfg = capi.config(mode)
    ctx = _ctx(cfg, w, dir_arena_mb=256)
    got = ctx.align(w.pairs)
    ctx.set_tuning(dir_arena_mb=0)
    whole = ctx.align(w.pairs)
    ctx.close()
    assert got.tobytes() == whole.tobytes()
    exp = _oracle(oracle_mod, mode, w, w.pairs, cfg)
    assert_same(got, exp, w.pairs)


def test_long_smith_waterman_pairs(native, oracle_mod):
    """Smith-Waterman on the uneven-length batch's long pairs (both sides over
    1000 residues, up to 5000): checked 16-bit regions and their 32-bit redo,
    row blocks, many arena chunks."""
    from pastis_gb300 import capi, synth
    w = synth.generate("uneven10m_sw", seed=7070, scale=0.0005)
    L = w.lengths()
    m, n = L[w.pairs["row"]], L[w.pairs["col"]]
    long_ = (m > 1000) & (n > 1000)
    pairs = np.concatenate([w.pairs[long_][:200], w.pairs[~long_][:800]])
    assert long_.sum() >= 100
    cfg = capi.config(capi.MODE_SW)
    ctx = _ctx(cfg, w)
    got = ctx.align(pairs)
    ctx.close()
    exp = _oracle(oracle_mod, 0, w, pairs, cfg)
    assert_same(got, exp, pairs)
    assert (got["flags"] & capi.RF_PASSED).any()


@pytest.mark.parametrize("stepped", [-1, 0, 1, 2])
def test_xdrop_residues_beyond_l2(native, oracle_mod, stepped):
    """A residue set of about 90 MB (more than half of L2, where the default
    picks the run-to-end extension kernel) under each extension form."""
    from pastis_gb300 import capi, synth
    w = synth.generate("uneven10m", seed=8080, scale=0.05, npairs=200_000)
    assert len(w.seq) > 64 << 20 and len(w.pairs) == 10_000
    cfg = capi.config(capi.MODE_XDROP)
    ctx = _ctx(cfg, w, xd_stepped=stepped)
    got = ctx.align(w.pairs)
    ctx.close()
    exp = _oracle(oracle_mod, 1, w, w.pairs, cfg)
    assert_same(got, exp, w.pairs)
