#!/usr/bin/env python
"""Throughput of the batched pairwise-alignment stage on GB300.

Default workload (xdrop1m): seeded X-drop extension (x = 49, k = 6, up to two
seeds) + global alignment with statistics + coverage/ANI filter over 1M
synthetic candidate pairs from 200k proteins (lognormal lengths, median 250,
clamp 30-1000; half homologs at 30-80 % identity), BLOSUM62 with PASTIS's gap
parameters -11 / -2.  A step is one pass of the aligner over the whole batch.

  value           GCUPS with inputs resident in HBM (device buffers,
                  pg_align_device), algorithmic cells (both seeds in full)
  executed_gcups  the cells the kernels computed (a repeated seed or region
                  is not recomputed) over the same time
  e2e             GCUPS through pg_align with pinned host buffers: pair upload
                  and result download inside the timed region
  parity          the oracle's results for the cpu_baseline sample (and up to
                  --parity-pairs pairs) against the GPU's, every byte of every
                  pg_result
  workloads       the sw100k Smith-Waterman batch (plain and filtered) measured
                  in the same run

With --gpus N (torchrun) every rank aligns its Sum(m*n)-balanced range of an
N-times larger batch over the same proteins (pastis_gb300/shard.py): weak
scaling, no collective on the data path.

--impl reference times the CPU restatement of the reference's SeqAn path
(the oracle; SeqAn itself is absent from the reference checkout) on all host
cores.  It maps no library of this package but the synthetic generator: each
timed step aligns the next window of the same batch, wrapping around.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GCUPS & alignments/s, batched SW/X-drop: GPU plain vs tuned+filtered vs CPU"
# roofline model: E, F and H as add-max DPX-class ops plus the max with the
# third term, per cell on 32-bit lanes
DPX_OPS_PER_CELL = 4
SW_WORKLOADS = ("sw100k", "filter5m", "uneven10m_sw")
SEED = 20260101


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="xdrop1m",
                    choices=["xdrop1m", "sw100k", "uneven10m", "uneven10m_sw", "filter5m",
                             "manytomany"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU work per baseline sample (seconds)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--parity-pairs", type=int, default=300_000,
                    help="pairs of the timed batch checked against the oracle (at least the "
                         "cpu_baseline sample)")
    ap.add_argument("--set-tuning", default="",
                    help="launch tuning of the plain arm, e.g. dp_traceback=0,bucket_order=1")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuned arm (tuned)")
    ap.add_argument("--no-filter", action="store_true",
                    help="skip the learned-filter arm (tuned_filtered)")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the sw100k record of the default run")
    ap.add_argument("--filter-train-frac", type=float, default=0.5,
                    help="training batch size as a fraction of the timed batch")
    ap.add_argument("--blocks", type=int, default=4,
                    help="manytomany: row and column blocks of the k-mer SpGEMM")
    ap.add_argument("--bsz", type=int, default=10_000_000,
                    help="manytomany: pairs per alignment batch (--bsz)")
    ap.add_argument("--filter-train-pairs", type=int, default=500_000,
                    help="manytomany: candidate pairs labelled to train the filter")
    return ap.parse_args()


def workload_desc(name, n, nseqs):
    base = {
        "xdrop1m": "seeded X-drop (x=49, k=6, <=2 seeds) + global alignment + stats + "
                   "coverage/ANI filter, %d candidate pairs over %d synthetic proteins "
                   "(lognormal lengths median 250 clamp 30-1000, 50%% homologs at 30-80%% "
                   "identity, 2%% indels)",
        "sw100k": "affine Smith-Waterman + stats + coverage/ANI filter, %d pairs over %d "
                  "synthetic proteins (lognormal lengths median 250 clamp 30-1000)",
        "uneven10m": "seeded X-drop, %d pairs over %d proteins, lengths 80%% lognormal "
                     "median 300 + 20%% uniform 1000-5000, min 20",
        "uneven10m_sw": "affine Smith-Waterman + stats + coverage/ANI filter, %d pairs over %d "
                        "proteins, lengths 80%% lognormal median 300 + 20%% uniform 1000-5000, "
                        "min 20",
        "filter5m": "affine Smith-Waterman + stats + coverage/ANI filter, %d pairs over %d "
                    "synthetic proteins (lognormal lengths median 250 clamp 30-1000, 30%% "
                    "homologs)",
    }[name]
    return base % (n, nseqs)


def mode_of(workload):
    return 0 if workload in SW_WORKLOADS else 1


def line_config(args, n, nseqs, world):
    """The config record both arms print (the same dict for the same run)."""
    mode = mode_of(args.workload)
    return {"workload": args.workload + ": " + workload_desc(args.workload, n, nseqs),
            "mode": "xdrop" if mode else "sw", "pairs": n,
            "scoring": "BLOSUM62; gap_open -11, gap_ext -2 given to the score model in SeqAn's "
                       "constructor order, as PASTIS calls it",
            "l2": "GPU arm: flushed between timed steps (512 MiB write, outside the timed "
                  "region)",
            "parallelism": "dp%d: each rank aligns its Sum(m*n)-balanced range of a %d-rank "
                           "batch (independent pairs, no collective)" % (world, world)}


def rank_batch(workload, scale, rank, world):
    """This rank's pairs: a batch of world x the preset's pairs over the same
    proteins, cut into Sum(m*n)-balanced contiguous ranges (shard.py).  At one
    rank it is the preset's batch."""
    from pastis_gb300 import synth
    from pastis_gb300.shard import my_range, pair_cost
    npairs = synth.PRESETS[workload]["npairs"] * world
    w = synth.generate(workload, seed=SEED, scale=scale, npairs=npairs)
    if world == 1:
        return w
    b, e = my_range(pair_cost(w.pairs, w.lengths()), rank, world)
    return w.subset(slice(b, e))


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
                 "--format=csv,noheader,nounits", "-lms", "100"],
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


def oracle_codes(w):
    from oracle import oracle as O
    return O.encode(bytes(w.ascii))


def cpu_sample(w, mode, p, budget_s, threads, codes=None):
    """Oracle over a prefix of the pairs sized to about budget_s of CPU time.
    Returns (cells, pairs, seconds, results)."""
    from oracle import oracle as O
    codes = oracle_codes(w) if codes is None else codes
    n = min(len(w.pairs), 500)
    while True:
        t = time.perf_counter()
        out = O.batch(mode, codes, w.offs, codes, w.offs, w.pairs[:n], p, nthreads=threads)
        dt = time.perf_counter() - t
        if dt >= budget_s * 0.5 or n >= len(w.pairs):
            cells = int(out["cells"].astype(np.uint64).sum())
            return cells, n, dt, out
        n = min(len(w.pairs), int(n * max(2.0, budget_s / max(dt, 1e-3) * 0.9)))


def parity_record(got, exp, what):
    """Byte comparison of every pg_result field of the GPU's results with the
    oracle's for the same pairs."""
    g = np.ascontiguousarray(got).view(np.uint8).reshape(len(got), -1)
    e = np.ascontiguousarray(exp).view(np.uint8).reshape(len(exp), -1)
    bad = (g != e).any(axis=1)
    per = {}
    for f in exp.dtype.names:
        a = np.ascontiguousarray(got[f]).view(np.uint8).reshape(len(got), -1)
        b = np.ascontiguousarray(exp[f]).view(np.uint8).reshape(len(exp), -1)
        k = int((a != b).any(axis=1).sum())
        if k:
            per[f] = k
    return {"pairs_checked": int(len(got)), "mismatches": int(bad.sum()),
            "fields": list(exp.dtype.names), "field_mismatches": per,
            "compare": "raw bytes of every pg_result field (f32 identity and score_aln as bit "
                       "patterns)", "pairs": what}


def oracle_params_for(mode):
    """The oracle's parameters for this bench's configuration: PASTIS's
    defaults in SeqAn's constructor order (pg_config_default's)."""
    from oracle import oracle as O
    return O.pastis_params(as_called=True)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, rank, world):
    """CPU restatement of the reference path on all host cores.  Each timed
    step aligns the next window of the batch (wrapping), sized so that the
    whole run takes a few minutes; GCUPS = cells of all timed windows / their
    time."""
    from oracle import oracle as O
    from pastis_gb300 import build
    if rank != 0:
        return
    build.build(only={"libpastis_synth.so"})
    O.build()
    w = rank_batch(args.workload, args.scale, 0, world)
    N = len(w.pairs)
    mode = mode_of(args.workload)
    p = oracle_params_for(mode)
    cores = host_cores()
    codes = oracle_codes(w)
    # window size: about 150 s for the whole run, 2 to 10 s per step
    per_step = min(10.0, max(2.0, 150.0 / max(1.0, args.steps + 0.2 * args.warmup)))
    _, ns, _, _ = cpu_sample(w, mode, p, per_step, cores, codes)
    ns = max(1, min(ns, N))

    def window(k):
        b = (k * ns) % N
        idx = np.arange(b, b + ns) % N
        return w.pairs[idx]

    for k in range(args.warmup):
        sub = window(k)
        O.batch(mode, codes, w.offs, codes, w.offs, sub[:max(1, ns // 10)], p, nthreads=cores)
    cells = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        out = O.batch(mode, codes, w.offs, codes, w.offs, window(k), p, nthreads=cores)
        cells += int(out["cells"].astype(np.uint64).sum())
    dt = time.perf_counter() - t0
    gcups = cells / dt / 1e9
    covered = min(N, ns * args.steps)
    sample = ("each step aligns the next %d of the batch's %d pairs (wrapping), %d distinct "
              "pairs over the %d timed steps; the reference's SeqAn path cannot be built "
              "(empty submodules), the oracle restates it" % (ns, N, covered, args.steps))
    line = {
        "metric": METRIC, "value": gcups, "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": line_config(args, N, int(len(w.offs) - 1), world),
        "impl": "reference",
        "alignments_per_s": ns * args.steps / dt,
        "pairs_per_step": ns,
        "cpu_baseline": {"value": gcups, "unit": "GCUPS", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": gcups, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_steps(step, stream, flush, steps):
    """CUDA-event time (ms) of each of `steps` calls of step() on `stream`,
    L2 flushed before each, outside the timed window."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for k in range(steps):
        flush.fill_(k & 0xff)
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def run_gpu(args, rank, world, local_rank):
    import torch
    from pastis_gb300 import capi
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    dev = local_rank
    torch.cuda.set_device(dev)
    mode = mode_of(args.workload)
    w = rank_batch(args.workload, args.scale, rank, world)
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
    tot = torch.tensor([total_ms, float(alg_cells), float(exec_cells), float(n)],
                       dtype=torch.float64, device=f"cuda:{dev}")
    if dist is not None:
        mx = tot[:1].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tot)
        tot[0] = mx[0]
    total_ms, all_cells, all_exec, all_pairs = (float(x) for x in tot.tolist())
    ms_step = total_ms / args.steps
    gcups = all_cells / (ms_step * 1e-3) / 1e9
    aln_s = all_pairs / (ms_step * 1e-3)

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
    e2e_gcups = all_cells / e2e_s / 1e9
    same = bool((ov.view(np.uint8) == res.view(np.uint8)).all())

    line = None
    if rank == 0:
        peak_ops = capi.dpx_peak(dev)
        form = ctx.get_tuning().dp_traceback
        # 16-bit lanes: each packed op advances two cells, so the same op rate
        # bounds twice the cells (the conservative peak for a mixed batch)
        cells_per_op = 2 if form >= 2 else 1
        peak_gcups = peak_ops * cells_per_op / DPX_OPS_PER_CELL / 1e9
        # dominant kernel: the alignment DP and its traceback, executed cells
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
        if form >= 2:
            peak_src = ("measured %.4g DPX add-max/s (pg_dpx_peak, int32) / %d DPX-class ops "
                        "per cell x 2 cells per packed 16-bit op (model; the 16-bit kernels "
                        "issue max/add.s16x2, not add-max)" % (peak_ops, DPX_OPS_PER_CELL))
        else:
            peak_src = ("measured %.4g DPX add-max/s (pg_dpx_peak, int32) / %d DPX-class ops "
                        "per cell (model)" % (peak_ops, DPX_OPS_PER_CELL))
        line = {
            "metric": METRIC, "value": gcups, "unit": "GCUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic",
            "config": line_config(args, n, int(len(w.offs) - 1), world),
            "alignments_per_s": aln_s,
            "executed_gcups": all_exec / (ms_step * 1e-3) / 1e9,
            "cells_note": "value counts algorithmic cells (both seeds in full, the CPU "
                          "baseline's definition); executed_gcups the cells the kernels "
                          "computed",
            "algorithmic_cells_per_step": alg_cells,
            "executed_cells_per_step": exec_cells,
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": {"value": e2e_gcups, "unit": "GCUPS",
                    "alignments_per_s": all_pairs / e2e_s,
                    "h2d_bytes_per_step": n * capi.PAIR_DTYPE.itemsize,
                    "d2h_bytes_per_step": n * capi.RESULT_DTYPE.itemsize,
                    "matches_device_run": same},
            "kernel_ms_per_step": {"extension": xd_ms, "alignment": dp_ms},
            "executed_cells_split": {"extension": exec_xd, "alignment": exec_dp},
            "roofline": {"bound": "dpx", "achieved": achieved, "peak": peak_gcups,
                         "unit": "GCUPS", "frac": achieved / peak_gcups, "traffic": traffic,
                         "kernel": dp_kernel,
                         "kernel_ms": dp_ms, "kernel_cells": exec_dp,
                         "peak_source": peak_src,
                         "hbm": {"achieved_GBps": hbm_gbs,
                                 "peak_GBps": peaks.get("hbm_gbs"),
                                 "frac": hbm_gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs")
                                 else None,
                                 "note": "algorithmic bytes: residues of both sequences, "
                                         "the pair record and the result per pair"}},
            "wall_s_timed": t_wall,
        }
        if mode == 1 and xd_ms > 0:
            line["extension"] = {"kernel_ms": xd_ms, "executed_cells": exec_xd,
                                 "executed_gcups": exec_xd / (xd_ms * 1e-3) / 1e9}
    if rank == 0 and not args.no_tune:
        line["tuned"] = tuned_arm(args, w, ctx, mode, dev, stream, flush, d_pairs, res, ms_step)
    if rank == 0 and not args.no_filter:
        line["tuned_filtered"] = filtered_arm(args.workload, args, w, ctx, dev, stream, flush,
                                              d_pairs, res, ms_step)
        line["tuned_filtered"]["tuning"] = ctx.get_tuning().as_dict()
    if rank == 0:
        cores = host_cores()
        p = oracle_params_for(mode)
        codes = oracle_codes(w)
        exp = None
        if not args.no_cpu_baseline:
            cells, ns, dt, exp = cpu_sample(w, mode, p, args.cpu_seconds, cores, codes)
            line["cpu_baseline"] = {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": cores,
                                    "kind": "port",
                                    "sample": "first %d of %d pairs (%.3g cells) in %.1f s" % (
                                        ns, n, cells, dt),
                                    "alignments_per_s": ns / dt}
        want = min(n, args.parity_pairs)
        if exp is None:
            exp = np.zeros(0, dtype=res.dtype)
        if len(exp) < want:
            from oracle import oracle as O
            more = O.batch(mode, codes, w.offs, codes, w.offs, w.pairs[len(exp):want], p,
                           nthreads=cores)
            exp = np.concatenate([exp, more])
        if len(exp):
            line["parity"] = parity_record(res[:len(exp)], exp,
                                           "the first %d pairs of the timed batch" % len(exp))
    if rank == 0 and args.workload == "xdrop1m" and not args.no_workloads:
        line["workloads"] = {"sw100k": sw100k_record(args, dev, stream, flush)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def sw100k_record(args, dev, stream, flush):
    """The sw100k Smith-Waterman batch (100k pairs over 20k proteins) in the
    same run: plain GCUPS, parity of every pair against the oracle, and the
    learned filter in front of the same aligner."""
    import torch
    from pastis_gb300 import capi, synth
    w = synth.generate("sw100k", seed=SEED, scale=args.scale)
    n = len(w.pairs)
    ctx = capi.Context(capi.config(capi.MODE_SW, device=dev))
    ctx.set_seqs(0, w.ascii, w.offs)
    ctx.share_row_seqs()
    torch.cuda.set_stream(stream)
    d_pairs = torch.from_numpy(w.pairs.view(np.uint8).copy()).to(f"cuda:{dev}")
    d_out = torch.empty(n * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}")

    def step():
        ctx.align_device(d_pairs.data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    res = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    cells = int(res["cells"].astype(np.uint64).sum())
    e0 = ctx.exec_cells_split()
    ms = statistics.mean(time_steps(step, stream, flush, max(args.steps, 5)))
    e1 = ctx.exec_cells_split()
    km = ctx.kernel_ms()
    out = {"config": "sw100k: " + workload_desc("sw100k", n, int(len(w.offs) - 1)),
           "value": cells / (ms * 1e-3) / 1e9, "unit": "GCUPS", "ms_per_step": ms,
           "alignments_per_s": n / (ms * 1e-3),
           "executed_cells_per_step": (e1[1] - e0[1]) / max(args.steps, 5),
           "alignment_kernel_ms_last_step": km[1]}
    if not args.no_filter:
        out["tuned_filtered"] = filtered_arm("sw100k", args, w, ctx, dev, stream, flush, d_pairs,
                                             res, ms)
    from oracle import oracle as O
    p = oracle_params_for(capi.MODE_SW)
    codes = oracle_codes(w)
    t0 = time.perf_counter()
    exp = O.batch(capi.MODE_SW, codes, w.offs, codes, w.offs, w.pairs, p, nthreads=host_cores())
    dt = time.perf_counter() - t0
    out["parity"] = parity_record(res, exp, "every pair of the batch")
    out["cpu_baseline"] = {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": host_cores(),
                           "kind": "port", "sample": "all %d pairs in %.1f s" % (n, dt)}
    ctx.close()
    return out


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


def filtered_arm(workload, args, w, ctx, dev, stream, flush, d_pairs, plain_res, plain_ms):
    """The learned pair filter in front of the same aligner on the same batch.

    A filter is trained (this library's BF16 kernels) on a separate batch of
    the same generator, labelled by the SW kernel; its threshold keeps 99.7 %
    of the positive validation pairs.  Timed per step: features, network,
    compaction, alignment of the kept pairs, scatter of the results.  Recall
    is measured on the timed batch itself against SW labels of every pair.

    ceiling: the same aligner on the positive pairs alone (a perfect filter,
    with no filter cost), which bounds what any pair filter can gain here."""
    import torch
    from pastis_gb300 import capi, synth
    from pastis_gb300 import filter as F
    n = len(w.pairs)
    wt = synth.generate(workload, seed=SEED + 7919, scale=args.scale * args.filter_train_frac)
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
    # the perfect filter: only the positives, already compacted on the device
    npos = int(pos.sum())
    ceiling = None
    if npos:
        d_pos = torch.from_numpy(w.pairs[pos].view(np.uint8).copy()).to(f"cuda:{dev}")
        d_pout = torch.empty(npos * capi.RESULT_DTYPE.itemsize, dtype=torch.uint8,
                             device=f"cuda:{dev}")

        def pos_step():
            ctx.align_device(d_pos.data_ptr(), npos, d_pout.data_ptr(), stream.cuda_stream)

        for _ in range(2):
            pos_step()
        pms = statistics.mean(time_steps(pos_step, stream, flush, args.steps))
        ceiling = {"ms_per_step": pms, "aligned_pairs": npos,
                   "alignments_per_s": n / (pms * 1e-3),
                   "vs_plain_alignments_per_s": plain_ms / pms,
                   "note": "aligning only the pairs the label marks positive, no filter cost: "
                           "the most any pair filter can gain on this batch"}
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
        "ceiling": ceiling,
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


def count_candidates(ctx, kc, blocks, bounds, stream):
    """Candidate pairs of the blocks under kc, counted without output."""
    import ctypes
    from pastis_gb300 import capi
    tot = 0
    for i, j in blocks:
        n = ctypes.c_uint64()
        rc = ctx.lib.pg_candidates(ctx.h, ctypes.byref(kc), int(bounds[i]), int(bounds[i + 1]),
                                   int(bounds[j]), int(bounds[j + 1]), None, 0, ctypes.byref(n),
                                   stream.cuda_stream)
        if rc != capi.PG_OK and not (rc == capi.PG_ERR_RANGE and n.value > 0):
            capi._check(rc)
        tot += int(n.value)
    return tot


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
    # the counts the reference logs per block, untimed: the product's nonzeros
    # before any prune (c_nnz, src/sim_search.cpp:164-165) and after the
    # symmetric prune (prune_sym, :189-190); ncand is after the ckthr prune too
    prod_nnz, sym_nnz = (count_candidates(ctx, capi.kmer_config(k=6, stride=1, prune=pr, ckthr=0),
                                          blocks, bounds, stream)
                         for pr in (capi.PRUNE_NONE, capi.PRUNE_EVEN_ODD))
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

    # warm-up: the first batch of each path once, untimed, with the timed loop's
    # result reductions (the first call of a torch kernel on a fresh machine
    # can compile it: 2.8 s inside the first timed batch, measured)
    for roff, coff, pb, m in batches():
        ctx.align_device(pb.data_ptr(), m, out.data_ptr(), stream.cuda_stream, roff, coff)
        capi.triples_device(pb.data_ptr(), out.data_ptr(), m, roff, coff, tr.data_ptr(),
                            tc.data_ptr(), tv.data_ptr(), stream.cuda_stream)
        res = out[:m * R].view(torch.int32).view(m, R // 4)
        int(res[:, 9].to(torch.int64).sum().item())
        torch.cat([res[:, 7].view(torch.float32) != 0])
        break

    # 2. plain path: alignment + triples per batch; per-pair pass mask kept for recall
    plain_pass = []
    batch_s = []
    cells = 0
    ntrip = 0
    sync()
    t0 = time.perf_counter()
    for roff, coff, pb, m in batches():
        tb = time.perf_counter()
        ctx.align_device(pb.data_ptr(), m, out.data_ptr(), stream.cuda_stream, roff, coff)
        ntrip += capi.triples_device(pb.data_ptr(), out.data_ptr(), m, roff, coff, tr.data_ptr(),
                                     tc.data_ptr(), tv.data_ptr(), stream.cuda_stream)
        res = out[:m * R].view(torch.int32).view(m, R // 4)
        cells += int(res[:, 9].to(torch.int64).sum().item())
        plain_pass.append(res[:, 7].view(torch.float32) != 0)
        batch_s.append(round(time.perf_counter() - tb, 4))
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
    counts = torch.tensor([ncand, cells, ntrip, ftrip, plain_trip, kept_trip, prod_nnz, sym_nnz],
                          dtype=torch.int64, device=f"cuda:{dev}")
    if dist is not None:
        dist.all_reduce(stats, op=dist.ReduceOp.MAX)
        dist.all_reduce(counts)
    gen_s, plain_s, filt_s = (float(x) for x in stats.tolist())
    ncand, cells, ntrip, ftrip, plain_trip, kept_trip, prod_nnz, sym_nnz = (
        int(x) for x in counts.tolist())
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
            "candidates": {"pairs": ncand, "seconds": gen_s, "pairs_per_s": ncand / gen_s,
                           "product_nnz": prod_nnz, "after_symmetric_prune": sym_nnz},
            "plain": {"seconds": plain_s, "alignments_per_s": ncand / plain_s,
                      "gcups": cells / plain_s / 1e9, "triples": ntrip,
                      "batch_seconds_rank0": batch_s},
            "tuned_filtered": {"seconds": filt_s, "alignments_per_s": ncand / filt_s,
                               "vs_plain_alignments_per_s": plain_s / filt_s, "triples": ftrip,
                               "recall_of_plain_triples": kept_trip / max(plain_trip, 1),
                               "training": {"pairs": fm["pairs"],
                                            "positive_fraction": fm["positive_fraction"],
                                            "val_recall": fm["val"]["recall"]}},
            "end_to_end_s": {"plain": gen_s + plain_s, "tuned_filtered": gen_s + filt_s},
        }
        if not args.no_cpu_baseline:
            p = oracle_params_for(capi.MODE_XDROP)
            sub = types.SimpleNamespace(pairs=allp[rng.permutation(len(allp))], ascii=w.ascii,
                                        offs=w.offs)
            c, n, dt, _ = cpu_sample(sub, capi.MODE_XDROP, p, args.cpu_seconds, host_cores())
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
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    from pastis_gb300 import build
    build.build()
    if args.workload == "manytomany":
        run_manytomany(args, rank, world, local_rank)
    else:
        run_gpu(args, rank, world, local_rank)


import numpy as np  # noqa: E402

if __name__ == "__main__":
    main()
