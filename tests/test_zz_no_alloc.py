"""pg_align_sw_noalloc: local alignment without any device allocation.

Some callers cannot allocate device memory: plugins running inside a host
framework that owns the device memory pool (they must not bypass its
allocator), and step loops that must not call the allocator between steps.
For them the library keeps the kernel's scratch in one fixed device array, and
the caller passes every input and output as device buffers.  These tests call that
entry point through the C ABI twice in a row and require the same bytes that
the ordinary entry point (pg_align, which allocates its own scratch) returns.
This file is collected last, and each test also passes when run alone in a
fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(seed, scale):
    import torch
    from pastis_gb300 import capi, synth
    w = synth.generate("sw100k", seed=seed, scale=scale)
    dev = torch.device("cuda:0")
    bufs = {
        "codes": torch.from_numpy(w.seq.copy()).to(dev),
        "offs": torch.from_numpy(w.offs.view(np.int64).copy()).to(dev),
        "pairs": torch.from_numpy(w.pairs.view(np.uint8).copy()).to(dev),
        "out": torch.empty(len(w.pairs) * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev),
    }
    return w, bufs


def _call(cfg, w, b, max_col_len, npairs=None):
    from pastis_gb300 import capi
    nseq = len(w.offs) - 1
    n = len(w.pairs) if npairs is None else npairs
    return capi.load().pg_align_sw_noalloc(
        ctypes.byref(cfg), b["codes"].data_ptr(), b["offs"].data_ptr(), nseq,
        b["codes"].data_ptr(), b["offs"].data_ptr(), nseq, max_col_len, b["pairs"].data_ptr(), n,
        0, 0, b["out"].data_ptr(), None)


@pytest.mark.parametrize("tie", [0, 3])
def test_noalloc_matches_pg_align_twice(native, tie):
    from pastis_gb300 import capi
    w, b = _setup(seed=909, scale=0.01)
    cfg = capi.config(capi.MODE_SW, tie=tie)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    expected = ctx.align(w.pairs)
    ctx.close()
    maxlen = int(w.lengths().max())
    for _ in range(2):
        b["out"].fill_(0xAB)          # stale bytes must not survive a call
        rc = _call(cfg, w, b, maxlen)
        assert rc == capi.PG_OK, capi.load().pg_last_error()
        got = np.frombuffer(b["out"].cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
        assert got.tobytes() == expected.tobytes()
    assert (expected["flags"] & capi.RF_PASSED).any()


def test_noalloc_rejects_sizes_beyond_its_scratch(native):
    from pastis_gb300 import capi
    w, b = _setup(seed=910, scale=0.002)
    cfg = capi.config(capi.MODE_SW)
    maxlen = int(w.lengths().max())
    assert _call(cfg, w, b, 65536) == capi.PG_ERR_RANGE
    assert _call(cfg, w, b, maxlen - 1) == capi.PG_ERR_RANGE
    assert _call(capi.config(capi.MODE_XDROP), w, b, maxlen) == capi.PG_ERR_ARG
    assert _call(cfg, w, b, maxlen, npairs=0) == capi.PG_OK
    # still correct after the rejected calls
    assert _call(cfg, w, b, maxlen) == capi.PG_OK


def test_noalloc_rejects_bad_pairs_and_codes(native):
    """A pair naming a sequence past the end gives PG_ERR_ARG and the empty
    result for that pair; a row over 65535 residues gives PG_ERR_RANGE; a
    residue code outside 0..24 gives PG_ERR_ARG with nothing aligned; the
    other pairs' results are still pg_align's."""
    import torch
    from pastis_gb300 import capi
    w, b = _setup(seed=911, scale=0.002)
    cfg = capi.config(capi.MODE_SW)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    expected = ctx.align(w.pairs)
    ctx.close()
    maxlen = int(w.lengths().max())
    nseq = len(w.offs) - 1
    empty = np.zeros(1, dtype=capi.RESULT_DTYPE)
    empty["flags"] = capi.RF_EMPTY

    bad = w.pairs.copy()
    bad["row"][3] = nseq
    b["pairs"].copy_(torch.from_numpy(bad.view(np.uint8).copy()))
    assert _call(cfg, w, b, maxlen) == capi.PG_ERR_ARG
    got = np.frombuffer(b["out"].cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    assert got[3].tobytes() == empty.tobytes()
    keep = np.arange(len(got)) != 3
    assert got[keep].tobytes() == expected[keep].tobytes()

    # a row of 70000 residues appended as sequence nseq (the columns stay short)
    long_codes = np.concatenate([w.seq, np.zeros(70000, np.uint8)])
    long_offs = np.concatenate([w.offs, [w.offs[-1] + 70000]]).astype(np.uint64)
    lb = dict(b)
    lb["codes"] = torch.from_numpy(long_codes).cuda()
    lb["offs"] = torch.from_numpy(long_offs.view(np.int64).copy()).cuda()
    lp = w.pairs.copy()
    lp["row"][5] = nseq
    lb["pairs"] = torch.from_numpy(lp.view(np.uint8).copy()).cuda()
    rc = capi.load().pg_align_sw_noalloc(
        ctypes.byref(cfg), lb["codes"].data_ptr(), lb["offs"].data_ptr(), nseq + 1,
        b["codes"].data_ptr(), b["offs"].data_ptr(), nseq, maxlen, lb["pairs"].data_ptr(),
        len(lp), 0, 0, b["out"].data_ptr(), None)
    assert rc == capi.PG_ERR_RANGE
    got = np.frombuffer(b["out"].cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    assert got[5].tobytes() == empty.tobytes()

    # a residue code of 25: rejected before any pair is aligned
    codes = w.seq.copy()
    codes[7] = 25
    cb = dict(b)
    cb["codes"] = torch.from_numpy(codes).cuda()
    cb["pairs"] = torch.from_numpy(w.pairs.view(np.uint8).copy()).cuda()
    b["out"].fill_(0xAB)
    assert _call(cfg, w, cb, maxlen) == capi.PG_ERR_ARG
    assert (b["out"].cpu().numpy() == 0xAB).all()

    # and the array serves a correct call afterwards
    b["pairs"].copy_(torch.from_numpy(w.pairs.view(np.uint8).copy()))
    assert _call(cfg, w, b, maxlen) == capi.PG_OK
    got = np.frombuffer(b["out"].cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    assert got.tobytes() == expected.tobytes()
