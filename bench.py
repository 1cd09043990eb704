#!/usr/bin/env python
"""Throughput of the batched pairwise-alignment stage on GB300.

Default workload (xdrop1m): seeded X-drop extension (x = 49, k = 6, up to two
seeds) + global alignment with statistics + coverage/ANI filter over 1M
synthetic candidate pairs from 200k proteins (lognormal lengths, median 250,
clamp 30-1000; half homologs at 30-80 % identity), BLOSUM62 with PASTIS's gap
parameters -11 / -2.  A step is one pass of the aligner over the whole batch.

  value  GCUPS with inputs resident in HBM (device buffers, pg_align_device)
  e2e    GCUPS through pg_align with pinned host buffers: pair upload and
         result download inside the timed region

--impl reference times the CPU restatement of the reference's SeqAn path
(the oracle; SeqAn itself is absent from the reference checkout) on all host
cores, on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GCUPS & alignments/s, batched SW/X-drop: GPU plain vs tuned+filtered vs CPU"
DPX_OPS_PER_CELL = 4  # E, F, H add-max and the max with the third term, int32
SW_WORKLOADS = ("sw100k", "filter5m")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="xdrop1m",
                    choices=["xdrop1m", "sw100k", "uneven10m", "filter5m", "manytomany"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU work per baseline sample (seconds)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--set-tuning", default="",
                    help="launch tuning of the plain arm, e.g. dp_traceback=0,bucket_order=1")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuned arm (tuned)")
    ap.add_argument("--no-filter", action="store_true",
                    help="skip the learned-filter arm (tuned_filtered)")
    ap.add_argument("--filter-train-frac", type=float, default=0.5,
                    help="training batch size as a fraction of the timed batch")
    ap.add_argument("--blocks", type=int, default=4,
                    help="manytomany: row and column blocks of the k-mer SpGEMM")
    ap.add_argument("--bsz", type=int, default=10_000_000,
                    help="manytomany: pairs per alignment batch (--bsz)")
    ap.add_argument("--filter-train-pairs", type=int, default=500_000,
                    help="manytomany: candidate pairs labelled to train the filter")
    return ap.parse_args()


def workload_desc(name, n, scale):
    base = {
        "xdrop1m": "seeded X-drop (x=49, k=6, <=2 seeds) + global alignment + stats + "
                   "coverage/ANI filter, %d candidate pairs over %d synthetic proteins "
                   "(lognormal lengths median 250 clamp 30-1000, 50%% homologs at 30-80%% "
                   "identity, 2%% indels)",
        "sw100k": "affine Smith-Waterman + stats + coverage/ANI filter, %d pairs over %d "
                  "synthetic proteins (lognormal lengths median 250 clamp 30-1000)",
        "uneven10m": "seeded X-drop, %d pairs over %d proteins, lengths 80%% lognormal "
                     "median 300 + 20%% uniform 1000-5000",
        "filter5m": "affine Smith-Waterman + stats + coverage/ANI filter, %d pairs over %d "
                    "synthetic proteins (lognormal lengths median 250 clamp 30-1000, 30%% "
                    "homologs)",
    }[name]
    from pastis_gb300 import synth
    p = synth.PRESETS[name]
    return base % (n, int(round(p["nseqs"] * scale)))


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_sample(w, mode, p, budget_s, threads):
    """Oracle over a prefix of the pairs sized to about budget_s of CPU time."""
    from oracle import oracle as O
    codes = O.encode(bytes(w.ascii))
    n = min(len(w.pairs), 500)
    while True:
        t = time.perf_counter()
        out = O.batch(mode, codes, w.offs, codes, w.offs, w.pairs[:n], p, nthreads=threads)
        dt = time.perf_counter() - t
        if dt >= budget_s * 0.5 or n >= len(w.pairs):
            cells = int(out["cells"].astype(np.uint64).sum())
            return cells, n, dt
        n = min(len(w.pairs), int(n * max(2.0, budget_s / max(dt, 1e-3) * 0.9)))


def oracle_params(cfg):
    from oracle import oracle as O
    from pastis_gb300 import capi
    first, ext, xg = capi.resolved_gaps(cfg)
    return O.make_params(gap_first=first, gap_ext=ext, xdrop_gap=xg, xdrop=cfg.xdrop,
                         seed_len=cfg.seed_len, seed_count=cfg.seed_count, tie=cfg.tie,
                         flags=cfg.flags, cov_thr=cfg.cov_thr, ani_thr=cfg.ani_thr)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, rank):
    """CPU restatement of the reference path, all host cores, bounded sample per step."""
    from oracle import oracle as O
    from pastis_gb300 import capi, synth
    if rank != 0:
        return
    O.build()
    w = synth.generate(args.workload, seed=20260101, scale=args.scale)
    mode = capi.MODE_SW if args.workload in SW_WORKLOADS else capi.MODE_XDROP
    cfg = capi.config(mode)
    p = oracle_params(cfg)
    cores = host_cores()
    # size one step to about 10 s of CPU time
    cells, n, dt = cpu_sample(w, mode, p, 10.0, cores)
    codes = O.encode(bytes(w.ascii))
    sub = w.pairs[:n]
    for _ in range(args.warmup):
        O.batch(mode, codes, w.offs, codes, w.offs, sub[:max(1, n // 10)], p, nthreads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = O.batch(mode, codes, w.offs, codes, w.offs, sub, p, nthreads=cores)
    dt = time.perf_counter() - t0
    cells = int(out["cells"].astype(np.uint64).sum())
    gcups = cells * args.steps / dt / 1e9
    sample = "first %d of %d pairs of the workload per step" % (n, len(w.pairs))
    line = {
        "metric": METRIC, "value": gcups, "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": args.workload + ": " + workload_desc(args.workload, len(w.pairs),
                                                                    args.scale),
                   "mode": "xdrop" if mode else "sw", "pairs_per_step": n},
        "impl": "reference",
        "alignments_per_s": n * args.steps / dt,
        "cpu_baseline": {"value": gcups, "unit": "GCUPS", "cores": cores, "kind": "port",
                         "sample": sample + "; the reference's SeqAn path cannot be built "
                                            "(empty submodules), the oracle restates it"},
        "e2e": {"value": gcups, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, local_rank):
    import torch
    from pastis_gb300 import capi, synth
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    dev = local_rank
    torch.cuda.set_device(dev)
    mode = capi.MODE_SW if args.workload in SW_WORKLOADS else capi.MODE_XDROP
    # weak scaling: every rank aligns its own batch of the same shape
    w = synth.generate(args.workload, seed=20260101 + rank, scale=args.scale)
    n = len(w.pairs)
    cfg = capi.config(mode, device=dev)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    if args.set_tuning:
        ctx.set_tuning(**{k: int(v) for k, v in
                          (kv.split("=") for kv in args.set_tuning.split(","))})

    # a dedicated stream: the kernels and the timing events must share it
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    d_pairs = torch.from_numpy(w.pairs.view(np.uint8).copy()).to(f"cuda:{dev}")
    d_out = torch.empty(n * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{dev}")

    def step():
        ctx.align_device(d_pairs.data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    res = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    alg_cells = int(res["cells"].astype(np.uint64).sum())

    clocks = Clocks(dev)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    exec0 = ctx.exec_cells_split()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    kern_ms = [0.0, 0.0]
    t_wall = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(k & 0xff)          # evict the previous step's working set from L2
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
        # per-kernel event times of this step (the library's events on the
        # same stream); reading them waits for the step, between timed windows
        km = ctx.kernel_ms()
        kern_ms[0] += km[0]
        kern_ms[1] += km[1]
    torch.cuda.synchronize(dev)
    t_wall = time.perf_counter() - t_wall
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    launches = ctx.last_launches() * args.steps
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    exec1 = ctx.exec_cells_split()
    exec_xd = (exec1[0] - exec0[0]) / args.steps
    exec_dp = (exec1[1] - exec0[1]) / args.steps
    exec_cells = exec_xd + exec_dp
    dp_ms = kern_ms[1] / args.steps
    xd_ms = kern_ms[0] / args.steps
    if dist is not None:
        t = torch.tensor([total_ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    gcups = alg_cells * world / (ms_step * 1e-3) / 1e9
    aln_s = n * world / (ms_step * 1e-3)

    # end to end: pinned host pairs in, results out, through pg_align
    h_pairs = torch.empty(n * capi.PAIR_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    h_pairs.numpy()[:] = w.pairs.view(np.uint8)
    h_out = torch.empty(n * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    pv = h_pairs.numpy().view(capi.PAIR_DTYPE)
    ov = h_out.numpy().view(capi.RESULT_DTYPE)
    ctx.align(pv, out=ov)
    e2e_t = []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        ctx.align(pv, out=ov)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(e2e_t)
    if dist is not None:
        t = torch.tensor([e2e_s], device=f"cuda:{dev}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_gcups = alg_cells * world / e2e_s / 1e9
    same = bool((ov.view(np.uint8) == res.view(np.uint8)).all())

    line = None
    if rank == 0:
        peak_ops = capi.dpx_peak(dev)
        form = ctx.get_tuning().dp_traceback
        # 16-bit lanes: each packed op advances two cells, so the same op rate
        # bounds twice the cells (the conservative peak for a mixed batch)
        cells_per_op = 2 if form >= 2 else 1
        peak_gcups = peak_ops * cells_per_op / DPX_OPS_PER_CELL / 1e9
        # dominant kernel: the alignment DP (k_ga / k_sw), its own cells and time
        achieved = exec_dp / (dp_ms * 1e-3) / 1e9
        traffic = None
        dp_kernel = {0: "k_ga" if mode else "k_sw",
                     1: "k_ga_dir + k_tb_ga" if mode else "k_sw_dir + k_tb_sw",
                     2: ("k_ga_dir + k_tb_ga" if mode else "k_sw_dir + k_tb_sw")
                     + " (16-bit lanes)",
                     3: ("k_ga_dir + k_ga_pair + k_tb_ga" if mode else "k_sw_dir + k_tb_sw")
                     + " (16-bit lanes, two regions per warp)"}[form]
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            # ncu DRAM bytes per pair of the same kernel on this workload
            tr = json.load(open(tpath)).get(args.workload)
            if tr and tr.get("bytes_per_pair") and tr.get("kernel") == dp_kernel:
                traffic = tr["bytes_per_pair"] * n
        peaks = {}
        ppath = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(ppath):
            peaks = json.load(open(ppath))
        lens = w.lengths()
        alg_bytes = int((lens[w.pairs["row"]] + lens[w.pairs["col"]]).sum()) + n * (
            capi.PAIR_DTYPE.itemsize + capi.RESULT_DTYPE.itemsize)
        hbm_gbs = alg_bytes / (ms_step * 1e-3) / 1e9
        line = {
            "metric": METRIC, "value": gcups, "unit": "GCUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic",
            "config": {"workload": args.workload + ": " + workload_desc(args.workload, n,
                                                                        args.scale),
                       "mode": "xdrop" if mode else "sw", "pairs": n,
                       "scoring": "BLOSUM62; gap_open -11, gap_ext -2 given to the score "
                                  "model in SeqAn's constructor order, as PASTIS calls it",
                       "l2": "flushed between timed steps (512 MiB write, outside the "
                             "timed region)",
                       "parallelism": "dp%d (independent pair batches per GPU)" % world},
            "alignments_per_s": aln_s,
            "algorithmic_cells_per_step": alg_cells,
            "executed_cells_per_step": exec_cells,
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": {"value": e2e_gcups, "unit": "GCUPS",
                    "alignments_per_s": n * world / e2e_s,
                    "h2d_bytes_per_step": n * capi.PAIR_DTYPE.itemsize,
                    "d2h_bytes_per_step": n * capi.RESULT_DTYPE.itemsize,
                    "matches_device_run": same},
            "kernel_ms_per_step": {"extension": xd_ms, "alignment": dp_ms},
            "executed_cells_split": {"extension": exec_xd, "alignment": exec_dp},
            "roofline": {"bound": "dpx", "achieved": achieved, "peak": peak_gcups,
                         "unit": "GCUPS", "frac": achieved / peak_gcups, "traffic": traffic,
                         "kernel": dp_kernel,
                         "kernel_ms": dp_ms, "kernel_cells": exec_dp,
                         "peak_source": "measured %.4g DPX add-max/s (pg_dpx_peak) / %d "
                                        "DPX ops per cell%s" % (
                                            peak_ops, DPX_OPS_PER_CELL,
                                            ", x 2 cells per packed 16-bit op" if form == 2
                                            else " (int32)"),
                         "hbm": {"achieved_GBps": hbm_gbs,
                                 "peak_GBps": peaks.get("hbm_gbs"),
                                 "frac": hbm_gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs")
                                 else None,
                                 "note": "algorithmic bytes: residues of both sequences, "
                                         "the pair record and the result per pair"}},
            "wall_s_timed": t_wall,
        }
    if rank == 0 and not args.no_tune:
        line["tuned"] = tuned_arm(args, w, ctx, mode, dev, stream, flush, d_pairs, res, ms_step)
    if rank == 0 and not args.no_filter:
        line["tuned_filtered"] = filtered_arm(args, w, ctx, dev, stream, flush, d_pairs, res,
                                              ms_step)
        line["tuned_filtered"]["tuning"] = ctx.get_tuning().as_dict()
    if not args.no_cpu_baseline and rank == 0:
        cores = host_cores()
        p = oracle_params(cfg)
        cells, ns, dt = cpu_sample(w, mode, p, args.cpu_seconds, cores)
        line["cpu_baseline"] = {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": cores,
                                "kind": "port",
                                "sample": "first %d of %d pairs (%.3g cells) in %.1f s" % (
                                    ns, n, cells, dt),
                                "alignments_per_s": ns / dt}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def tuned_arm(args, w, ctx, mode, dev, stream, flush, d_pairs, plain_res, plain_ms):
    """The autotuned launch shape (pastis_gb300/autotune.py) with CUDA-graph
    replay, on the same batch; the search runs on a sample of the batch."""
    import torch
    from pastis_gb300 import autotune, capi
    n = len(w.pairs)
    ns = min(n, 250_000)
    d_out = torch.empty(n * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}")

    def run_sample():
        ctx.align_device(d_pairs.data_ptr(), ns, d_out.data_ptr(), stream.cuda_stream)

    def run_full():
        ctx.align_device(d_pairs.data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)

    key = autotune.signature(mode, w.pairs, w.lengths())
    best, rep = autotune.tune(ctx, run_sample, key=key, device=dev, use_cache=False,
                              validate=run_full if ns < n else None)
    for _ in range(max(args.warmup, 3)):
        ctx.align_device(d_pairs.data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize(dev)
    got = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    same = got.tobytes() == plain_res.tobytes()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        ev[k][0].record(stream)
        ctx.align_device(d_pairs.data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    return {"alignments_per_s": n / (ms * 1e-3), "ms_per_step": ms,
            "vs_plain_alignments_per_s": plain_ms / ms, "tuning": best,
            "results_identical_to_plain": bool(same),
            "search": {"sample_pairs": ns, "candidates": rep.get("candidates"),
                       "seconds": rep.get("search_s"), "best_sample_ms": rep.get("ms"),
                       "default_sample_ms": rep.get("default_ms"), "key": key,
                       "full_batch_check": rep.get("validated_on_full_batch")}}


def filtered_arm(args, w, ctx, dev, stream, flush, d_pairs, plain_res, plain_ms):
    """The learned pair filter in front of the same aligner on the same batch.

    A filter is trained (this library's BF16 kernels) on a separate batch of
    the same generator, labelled by the SW kernel; its threshold keeps 99.5 %
    of the positive validation pairs.  Timed per step: features, network,
    compaction, alignment of the kept pairs, scatter of the results.  Recall
    is measured on the timed batch itself against SW labels of every pair."""
    import torch
    from pastis_gb300 import capi, synth
    from pastis_gb300 import filter as F
    n = len(w.pairs)
    wt = synth.generate(args.workload, seed=20260101 + 7919,
                        scale=args.scale * args.filter_train_frac)
    # the threshold keeps 99.7 % of the validation positives so that the
    # recall measured on the (different) timed batch stays above 99.5 %
    f, thr, fm = F.fit(wt, dev, recall=0.997)
    _, labels = F.sw_labels(w, dev)
    torch.cuda.set_stream(stream)
    d_out = torch.empty(n * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}")
    kept = 0
    for _ in range(max(args.warmup, 3)):
        kept = f.align_filtered(ctx, thr, d_pairs.data_ptr(), n, d_out.data_ptr(),
                                stream.cuda_stream)
    torch.cuda.synchronize(dev)
    got = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    keep = (got["flags"] & capi.RF_FILTERED) == 0
    same = got[keep].tobytes() == plain_res[keep].tobytes()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        ev[k][0].record(stream)
        f.align_filtered(ctx, thr, d_pairs.data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    # the filter's own share: features + network over the whole batch
    feats = torch.empty(n * 32, dtype=torch.uint8, device=f"cuda:{dev}")
    logits = torch.empty(n, dtype=torch.float32, device=f"cuda:{dev}")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(1)
    e0.record(stream)
    f.features(ctx, d_pairs.data_ptr(), n, feats.data_ptr(), stream.cuda_stream)
    f.predict(feats.data_ptr(), n, logits.data_ptr(), stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    pos = labels > 0.5
    out = {
        "alignments_per_s": n / (ms * 1e-3),
        "ms_per_step": ms,
        "vs_plain_alignments_per_s": plain_ms / ms,
        "kept_pairs": int(kept), "kept_fraction": kept / n,
        "recall": float(keep[pos].mean()) if pos.any() else None,
        "precision": float(pos[keep].mean()) if keep.any() else None,
        "positives": int(pos.sum()),
        "kept_results_identical_to_plain": bool(same),
        "filter_ms": e0.elapsed_time(e1),
        "threshold_logit": thr,
        "label": "SW score (BLOSUM62, open -11 / extend -2) >= ceil((ln(K m n) + ln 1000) / "
                 "lambda), lambda 0.267, K 0.041",
        "training": {"pairs": fm["pairs"], "positive_fraction": fm["positive_fraction"],
                     "label_s": fm["label_seconds"], "train_s": fm["train_seconds"],
                     "val_recall": fm["val"]["recall"], "test_recall": fm["test"]["recall"],
                     "test_kept_fraction": fm["test"]["kept_fraction"],
                     "kmer_rule_kept_at_same_recall": fm["kmer_rule_kept_at_same_recall"]},
        "alignments_per_s_counts": "candidate pairs resolved per second (pruned pairs get "
                                   "score_aln 0 and the filtered flag)",
    }
    f.close()
    return out


def gen_candidates(ctx, kc, rows, cols, dev, stream):
    """One block's candidate pairs on the device (torch uint8 tensor)."""
    import ctypes
    import torch
    from pastis_gb300 import capi
    cap = 1 << 22
    while True:
        buf = torch.empty(cap * capi.PAIR_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}")
        n = ctypes.c_uint64()
        rc = ctx.lib.pg_candidates(ctx.h, ctypes.byref(kc), int(rows[0]), int(rows[1]),
                                   int(cols[0]), int(cols[1]), buf.data_ptr(), cap,
                                   ctypes.byref(n), stream.cuda_stream)
        if rc == capi.PG_ERR_RANGE and n.value > cap:
            cap = int(n.value)
            continue
        capi._check(rc)
        return buf[:int(n.value) * capi.PAIR_DTYPE.itemsize], int(n.value)


def run_manytomany(args, rank, world, local_rank):
    """Blocked many-to-many search: GPU k-mer SpGEMM candidates (k = 6,
    stride 1, even/odd symmetric prune, ckthr = 1) streamed in --bsz batches
    through the plain X-drop aligner and through the filtered one, each batch
    ending in similarity triples; the host-core oracle on a sample of the same
    pairs."""
    import types
    import torch
    from pastis_gb300 import capi, synth
    from pastis_gb300 import filter as F
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    dev = local_rank
    torch.cuda.set_device(dev)
    w = synth.generate("manytomany", seed=20260101, scale=args.scale)
    ns = len(w.offs) - 1
    cfg = capi.config(capi.MODE_XDROP, device=dev)
    ctx = capi.Context(cfg)
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    if args.set_tuning:
        ctx.set_tuning(**{k: int(v) for k, v in
                          (kv.split("=") for kv in args.set_tuning.split(","))})
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    nb = args.blocks
    bounds = np.linspace(0, ns, nb + 1).astype(np.int64)
    blocks = [(i, j) for i in range(nb) for j in range(nb)][rank::world]
    kc = capi.kmer_config(k=6, stride=1, prune=capi.PRUNE_EVEN_ODD, ckthr=1)

    def sync():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    # 1. candidates
    sync()
    t0 = time.perf_counter()
    cand = []
    for i, j in blocks:
        rows, cols = (bounds[i], bounds[i + 1]), (bounds[j], bounds[j + 1])
        buf, n = gen_candidates(ctx, kc, rows, cols, dev, stream)
        cand.append((int(rows[0]), int(cols[0]), buf, n))
    sync()
    gen_s = time.perf_counter() - t0
    ncand = sum(c[3] for c in cand)
    bsz = args.bsz
    R = capi.RESULT_DTYPE.itemsize
    P = capi.PAIR_DTYPE.itemsize
    out = torch.empty(bsz * R, dtype=torch.uint8, device=f"cuda:{dev}")
    tr = torch.empty(bsz, dtype=torch.int64, device=f"cuda:{dev}")
    tc = torch.empty(bsz, dtype=torch.int64, device=f"cuda:{dev}")
    tv = torch.empty(bsz, dtype=torch.float32, device=f"cuda:{dev}")

    def batches():
        for roff, coff, buf, n in cand:
            for s in range(0, n, bsz):
                m = min(bsz, n - s)
                yield roff, coff, buf[s * P:(s + m) * P], m

    # warm-up: the first batch of each path once, untimed
    for roff, coff, pb, m in batches():
        ctx.align_device(pb.data_ptr(), m, out.data_ptr(), stream.cuda_stream, roff, coff)
        capi.triples_device(pb.data_ptr(), out.data_ptr(), m, roff, coff, tr.data_ptr(),
                            tc.data_ptr(), tv.data_ptr(), stream.cuda_stream)
        break

    # 2. plain path: alignment + triples per batch; per-pair pass mask kept for recall
    plain_pass = []
    cells = 0
    ntrip = 0
    sync()
    t0 = time.perf_counter()
    for roff, coff, pb, m in batches():
        ctx.align_device(pb.data_ptr(), m, out.data_ptr(), stream.cuda_stream, roff, coff)
        ntrip += capi.triples_device(pb.data_ptr(), out.data_ptr(), m, roff, coff, tr.data_ptr(),
                                     tc.data_ptr(), tv.data_ptr(), stream.cuda_stream)
        res = out[:m * R].view(torch.int32).view(m, R // 4)
        cells += int(res[:, 9].to(torch.int64).sum().item())
        plain_pass.append(res[:, 7].view(torch.float32) != 0)
    sync()
    plain_s = time.perf_counter() - t0

    # 3. filter trained on SW labels of a sample of these candidates
    rng = np.random.default_rng(5)
    host_pairs = []
    for roff, coff, buf, n in cand:
        pv = np.frombuffer(buf.cpu().numpy().tobytes(), dtype=capi.PAIR_DTYPE).copy()
        pv["row"] += roff
        pv["col"] += coff
        host_pairs.append(pv)
    allp = np.concatenate(host_pairs) if host_pairs else np.zeros(0, dtype=capi.PAIR_DTYPE)
    sample = allp[rng.permutation(len(allp))[:min(len(allp), args.filter_train_pairs)]]
    ws = types.SimpleNamespace(pairs=sample, ascii=w.ascii, offs=w.offs,
                               lengths=w.lengths)
    # label: the plain aligner's own verdict (coverage/ANI filter passed)
    lab = (ctx.align(sample)["score_aln"] != 0).astype(np.float32)
    f, thr, fm = F.fit(ws, dev, recall=0.997, labels=lab)
    torch.cuda.set_stream(stream)
    for roff, coff, pb, m in batches():
        f.align_filtered(ctx, thr, pb.data_ptr(), m, out.data_ptr(), stream.cuda_stream, roff, coff)
        break

    # 4. filtered path
    fpass = []
    ftrip = 0
    sync()
    t0 = time.perf_counter()
    for roff, coff, pb, m in batches():
        f.align_filtered(ctx, thr, pb.data_ptr(), m, out.data_ptr(), stream.cuda_stream, roff, coff)
        ftrip += capi.triples_device(pb.data_ptr(), out.data_ptr(), m, roff, coff, tr.data_ptr(),
                                     tc.data_ptr(), tv.data_ptr(), stream.cuda_stream)
        res = out[:m * R].view(torch.int32).view(m, R // 4)
        fpass.append(res[:, 7].view(torch.float32) != 0)
    sync()
    filt_s = time.perf_counter() - t0
    pp = torch.cat(plain_pass) if plain_pass else torch.zeros(0, dtype=torch.bool)
    fp = torch.cat(fpass) if fpass else torch.zeros(0, dtype=torch.bool)
    kept_trip = int((pp & fp).sum().item())
    plain_trip = int(pp.sum().item())
    f.close()

    stats = torch.tensor([gen_s, plain_s, filt_s], dtype=torch.float64, device=f"cuda:{dev}")
    counts = torch.tensor([ncand, cells, ntrip, ftrip, plain_trip, kept_trip], dtype=torch.int64,
                          device=f"cuda:{dev}")
    if dist is not None:
        dist.all_reduce(stats, op=dist.ReduceOp.MAX)
        dist.all_reduce(counts)
    gen_s, plain_s, filt_s = (float(x) for x in stats.tolist())
    ncand, cells, ntrip, ftrip, plain_trip, kept_trip = (int(x) for x in counts.tolist())
    if rank == 0:
        line = {
            "metric": METRIC, "value": cells / plain_s / 1e9, "unit": "GCUPS",
            "n_gpus": world, "steps": 1, "warmup": 0, "ms_per_step": plain_s * 1e3,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic",
            "config": {"workload": "manytomany: %d synthetic proteins (families of 2-50 at "
                                   "30-90%% identity), all-vs-all k-mer candidates (k=6, stride "
                                   "1, even/odd symmetric prune, ckthr=1) in %dx%d blocks, "
                                   "X-drop x=49 in batches of %d" % (ns, nb, nb, bsz),
                       "mode": "xdrop"},
            "candidates": {"pairs": ncand, "seconds": gen_s, "pairs_per_s": ncand / gen_s},
            "plain": {"seconds": plain_s, "alignments_per_s": ncand / plain_s,
                      "gcups": cells / plain_s / 1e9, "triples": ntrip},
            "tuned_filtered": {"seconds": filt_s, "alignments_per_s": ncand / filt_s,
                               "vs_plain_alignments_per_s": plain_s / filt_s, "triples": ftrip,
                               "recall_of_plain_triples": kept_trip / max(plain_trip, 1),
                               "training": {"pairs": fm["pairs"],
                                            "positive_fraction": fm["positive_fraction"],
                                            "val_recall": fm["val"]["recall"]}},
            "end_to_end_s": {"plain": gen_s + plain_s, "tuned_filtered": gen_s + filt_s},
        }
        if not args.no_cpu_baseline:
            p = oracle_params(cfg)
            sub = types.SimpleNamespace(pairs=allp[rng.permutation(len(allp))], ascii=w.ascii,
                                        offs=w.offs)
            c, n, dt = cpu_sample(sub, capi.MODE_XDROP, p, args.cpu_seconds, host_cores())
            line["cpu_baseline"] = {"value": c / dt / 1e9, "unit": "GCUPS", "cores": host_cores(),
                                    "kind": "port", "sample": "%d random candidate pairs in "
                                                              "%.1f s" % (n, dt),
                                    "alignments_per_s": n / dt}
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    from pastis_gb300 import build
    build.build()
    if args.impl == "reference":
        run_reference(args, rank)
    elif args.workload == "manytomany":
        run_manytomany(args, rank, world, local_rank)
    else:
        run_gpu(args, rank, world, local_rank)


import numpy as np  # noqa: E402

if __name__ == "__main__":
    main()
