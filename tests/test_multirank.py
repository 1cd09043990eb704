"""Sharding of a batch over 2 ranks (gloo, CPU): each rank aligns its balanced
contiguous range with no data-path collective; gathering the per-rank results
in rank order reproduces the single-rank run bit for bit.  The aligner here is
the oracle (the GPU path is the same C ABI per rank, one GPU each)."""
import os

import numpy as np
import pytest


def test_balanced_ranges():
    from pastis_gb300.shard import balanced_ranges
    cost = np.array([1, 1, 1, 1, 100, 1, 1, 1], dtype=float)
    r = balanced_ranges(cost, 2)
    assert r[0][0] == 0 and r[-1][1] == len(cost) and r[0][1] == r[1][0]
    for parts in (1, 2, 3, 7, 20):
        rr = balanced_ranges(np.random.default_rng(parts).random(100), parts)
        assert len(rr) == parts and rr[0][0] == 0 and rr[-1][1] == 100
        assert all(a[1] == b[0] for a, b in zip(rr, rr[1:]))
    assert balanced_ranges(np.zeros(0), 3) == [(0, 0), (0, 0), (0, 0)]


def _worker(rank, world, port, path):
    import torch.distributed as dist
    import torch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from pastis_gb300 import synth
    from pastis_gb300.shard import pair_cost, my_range
    w = synth.generate("xdrop1m", seed=55, scale=0.0005)
    b, e = my_range(pair_cost(w.pairs, w.lengths()), rank, world)
    codes = O.encode(bytes(w.ascii))
    out = O.batch(1, codes, w.offs, codes, w.offs, w.pairs[b:e], O.make_params(-2, -11),
                  nthreads=1)
    blob = torch.from_numpy(out.view(np.uint8).copy())
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([blob.numel()]))
    mx = int(max(s.item() for s in sizes))
    padded = torch.zeros(mx, dtype=torch.uint8)
    padded[:blob.numel()] = blob
    parts = [torch.zeros(mx, dtype=torch.uint8) for _ in range(world)]
    dist.all_gather(parts, padded)
    if rank == 0:
        full = np.concatenate([p[:int(s.item())].numpy() for p, s in zip(parts, sizes)])
        np.save(path, full)
    dist.destroy_process_group()


def test_two_ranks_match_single(tmp_path, native, oracle_mod):
    import torch.multiprocessing as mp
    from pastis_gb300 import synth
    O = oracle_mod
    path = str(tmp_path / "gathered.npy")
    port = 29500 + (os.getpid() % 1000)
    mp.spawn(_worker, args=(2, port, path), nprocs=2, join=True)
    w = synth.generate("xdrop1m", seed=55, scale=0.0005)
    codes = O.encode(bytes(w.ascii))
    single = O.batch(1, codes, w.offs, codes, w.offs, w.pairs, O.make_params(-2, -11))
    gathered = np.load(path)
    assert gathered.tobytes() == single.view(np.uint8).tobytes()


def test_rank_failure_is_reported(tmp_path):
    """A rank that raises before the gather ends the job with an error on the
    host (no GPU involved): the failure surfaces through the launcher."""
    import torch.multiprocessing as mp
    with pytest.raises(Exception):
        mp.spawn(_fail_worker, args=(), nprocs=2, join=True)


def _fail_worker(rank):
    if rank == 1:
        raise RuntimeError("rank 1 failed between steps")
