"""bench.py's reference arm runs on CPU: one JSON line with the keys the
benchmark contract names (metric, value, unit, steps, e2e with zero copy
bytes, cpu_baseline describing the run, impl = reference), the same config
record as the GPU arm, and no CUDA library of this package mapped."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# runs bench.main() and then lists the shared objects of this repository the
# process mapped
_PROBE = r"""
import runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
try:
    runpy.run_path("bench.py", run_name="__main__")
finally:
    maps = open("/proc/self/maps").read().split("\n")
    libs = sorted({ln.split()[-1] for ln in maps if ln.endswith(".so") and "_build" in ln})
    print("MAPPED " + " ".join(libs))
"""


def test_reference_arm_json_line(native):
    out = subprocess.run([sys.executable, "-c", _PROBE, "--impl", "reference",
                          "--workload", "sw100k", "--scale", "0.005", "--steps", "2",
                          "--warmup", "1"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "GCUPS" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    mapped = [ln for ln in out.stdout.splitlines() if ln.startswith("MAPPED")][0].split()[1:]
    assert not any(m.endswith("libpastis_gb300.so") or m.endswith("libpastis_host.so")
                   for m in mapped), mapped
    assert any(m.endswith("liboracle.so") for m in mapped), mapped


def test_both_arms_print_the_same_config(native):
    """The GPU arm and the reference arm build their config record with the
    same function from the same batch."""
    sys.path.insert(0, ROOT)
    import bench

    class A:
        workload, scale = "xdrop1m", 0.001

    w = bench.rank_batch(A.workload, A.scale, 0, 1)
    c1 = bench.line_config(A, len(w.pairs), len(w.offs) - 1, 1)
    c2 = bench.line_config(A, len(w.pairs), len(w.offs) - 1, 1)
    assert c1 == c2 and c1["pairs"] == len(w.pairs) and c1["mode"] == "xdrop"


def test_rank_batches_partition_the_batch(native):
    """With N ranks each rank takes a balanced contiguous range of an N-times
    larger batch; the ranges cover it exactly."""
    sys.path.insert(0, ROOT)
    import numpy as np

    import bench
    from pastis_gb300 import synth
    full = synth.generate("xdrop1m", seed=bench.SEED, scale=0.001,
                          npairs=synth.PRESETS["xdrop1m"]["npairs"] * 3)
    parts = [bench.rank_batch("xdrop1m", 0.001, r, 3) for r in range(3)]
    got = np.concatenate([p.pairs for p in parts])
    assert got.tobytes() == full.pairs.tobytes()
    L = full.lengths()
    cost = [int((L[p.pairs["row"]] * L[p.pairs["col"]]).sum()) for p in parts]
    assert max(cost) < 1.2 * min(cost)


def test_parity_record_counts_byte_differences(oracle_mod):
    sys.path.insert(0, ROOT)
    import numpy as np

    import bench
    a = np.zeros(5, dtype=oracle_mod.RESULT_DTYPE)
    b = a.copy()
    b["identity"][1] = -0.0            # same value, different bits: a mismatch
    b["score"][3] = 7
    r = bench.parity_record(a, b, "test")
    assert r["pairs_checked"] == 5 and r["mismatches"] == 2
    assert r["field_mismatches"] == {"identity": 1, "score": 1}
