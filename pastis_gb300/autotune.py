"""Autotuner for the batch launch shape (pg_tuning).

The choices it makes never change a result, only how fast a batch runs:
resident blocks per SM of the DP kernels and of the X-drop extension, the
form of the X-drop extension (a direction per step, or each task run to its
end), the bucketed pair order, the form of the alignment DP, and CUDA-graph
replay of the batch's launches.
Candidates are timed with the library's own CUDA events (pg_kernel_ms) on a
batch the caller supplies,
normally a sample of the real one, and the winner is cached in a JSON file
keyed by device and a workload signature (mode, batch size and length
quantiles, rounded to powers of two) so later runs on the same kind of batch
skip the search.
"""
import itertools
import json
import os
import statistics
import time

import numpy as np

from . import capi

GRID = {
    "dp_blocks_per_sm": (1, 0),      # 0 = occupancy limit (2 on GB300)
    "xd_blocks_per_sm": (4, 0),      # 0 = occupancy limit (7 on GB300)
    "bucket_order": (1, 0),
    "xd_stepped": (2, 1, 0),         # X-drop extension: register window, ring a direction per
                                     # step, ring run to end
    "dp_traceback": (3, 0),          # 3 = traceback form on 16-bit lanes, 0 = statistics
}


def cache_path():
    return os.environ.get("PG_TUNING_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "pastis_gb300",
                                       "tuning.json"))


def _p2(x):
    x = max(1, int(x))
    return 1 << (x - 1).bit_length()


def signature(mode, pairs, lengths):
    """Workload key: mode, batch size and the 50/90/99th percentile of the
    taller sequence of each pair, each rounded up to a power of two."""
    L = np.asarray(lengths, dtype=np.int64)
    tall = np.maximum(L[pairs["row"]], L[pairs["col"]]) if len(pairs) else np.zeros(1)
    q = [int(_p2(v)) for v in np.percentile(tall, [50, 90, 99])]
    return "mode%d-n%d-p50_%d-p90_%d-p99_%d" % (mode, _p2(len(pairs)), *q)


def _device_name(device):
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return "cuda%d" % device


def _time(ctx, run, reps):
    run()
    ctx.kernel_ms()
    ms = []
    for _ in range(reps):
        run()
        a, b = ctx.kernel_ms()
        ms.append(a + b)
    return statistics.median(ms)


def tune(ctx, run, key=None, device=0, reps=3, grid=None, use_cache=True, log=None,
         validate=None):
    """Time every candidate tuning with `run()` (one batch on ctx) and set the
    fastest on ctx, with graph replay on.  With `validate` (a run of the full
    batch) the winner is timed against the context's tuning before the search
    and kept only if faster: a sample can mislead when a few long pairs dominate it.
    Returns (tuning dict, report)."""
    path = cache_path()
    dev = _device_name(device)
    entry = "%s|%s" % (dev, key) if key else None
    if use_cache and entry and os.path.exists(path):
        try:
            cached = json.load(open(path)).get(entry)
        except (OSError, ValueError):
            cached = None
        if cached:
            ctx.set_tuning(capi.default_tuning(), **cached["tuning"])
            return cached["tuning"], {"cached": True, "key": entry, "ms": cached.get("ms")}
    initial = ctx.get_tuning().as_dict() if validate is not None else None
    grid = GRID if grid is None else grid
    names = list(grid)
    rows = []
    t0 = time.perf_counter()
    for vals in itertools.product(*(grid[k] for k in names)):
        cand = dict(zip(names, vals), graph=0)
        ctx.set_tuning(capi.default_tuning(), **cand)
        ms = _time(ctx, run, reps)
        rows.append((ms, cand))
        if log:
            log("%-70s %.3f ms" % (cand, ms))
    rows.sort(key=lambda r: r[0])
    best = dict(rows[0][1], graph=1)
    validated = None
    if validate is not None:
        base = dict(initial)
        ctx.set_tuning(capi.default_tuning(), **best)
        t_best = _time(ctx, validate, 2)
        ctx.set_tuning(capi.default_tuning(), **base)
        t_base = _time(ctx, validate, 2)
        validated = {"best_ms": t_best, "default_ms": t_base}
        if t_base < t_best:
            best = base
    ctx.set_tuning(capi.default_tuning(), **best)
    report = {"cached": False, "key": entry, "ms": rows[0][0], "search_s": time.perf_counter() - t0,
              "candidates": len(rows), "validated_on_full_batch": validated, "default_ms": next(
                  (m for m, c in rows if c == {"dp_blocks_per_sm": 0, "xd_blocks_per_sm": 0,
                                               "bucket_order": 1, "graph": 0,
                                               "xd_stepped": 2, "dp_traceback": 3}),
                  None)}
    if entry:
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            data = {}
            if os.path.exists(path):
                try:
                    data = json.load(open(path))
                except ValueError:
                    data = {}
            data[entry] = {"tuning": best, "ms": rows[0][0]}
            tmp = path + ".tmp%d" % os.getpid()
            json.dump(data, open(tmp, "w"), indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:
            pass
    return best, report
