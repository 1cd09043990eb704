"""pg_align_sw_noalloc: local alignment without any device allocation.

Some callers cannot allocate device memory: code recorded into a stream
capture, plugins running inside a host framework that owns the device
allocator, and loops that must not call the allocator between steps.  For them
the library keeps the kernel's scratch in one fixed device array, and the
caller passes every input and output as device buffers.  These tests call that
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
