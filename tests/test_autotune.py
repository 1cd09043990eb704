"""Autotuner host logic on the CPU: search, choice and cache, against a fake
context whose batch time depends on the tuning."""
import numpy as np


class FakeCtx:
    def __init__(self):
        self.t = None
        self.calls = 0

    def set_tuning(self, t=None, **fields):
        d = t.as_dict() if t is not None else {}
        d.update(fields)
        self.t = d
        return d

    def kernel_ms(self):
        t = self.t
        ms = 10.0 + (2.0 if t["bucket_order"] == 0 else 0.0) + (0.5 if t["dp_traceback"] else 0.0)
        ms += 1.0 if t["dp_blocks_per_sm"] == 1 else 0.0
        return 0.0, ms


def test_search_picks_fastest_and_caches(native, tmp_path, monkeypatch):
    from pastis_gb300 import autotune
    monkeypatch.setenv("PG_TUNING_CACHE", str(tmp_path / "t.json"))
    ctx = FakeCtx()
    best, rep = autotune.tune(ctx, lambda: None, key="k1", reps=2)
    assert best["dp_blocks_per_sm"] == 0 and best["bucket_order"] == 1
    assert best["graph"] == 1
    assert ctx.t["graph"] == 1 and not rep["cached"]
    assert rep["candidates"] == 48
    ctx2 = FakeCtx()
    best2, rep2 = autotune.tune(ctx2, lambda: None, key="k1")
    assert rep2["cached"] and best2 == best and ctx2.t["dp_traceback"] == 0


def test_signature_rounds_to_powers_of_two(native):
    from pastis_gb300 import autotune, capi
    pairs = np.zeros(1000, dtype=capi.PAIR_DTYPE)
    pairs["row"] = np.arange(1000) % 10
    pairs["col"] = (np.arange(1000) + 1) % 10
    L = np.array([100, 200, 300, 400, 500, 600, 700, 800, 900, 1000])
    s = autotune.signature(1, pairs, L)
    assert s.startswith("mode1-n1024-")
    assert s == autotune.signature(1, pairs, L + 1)
