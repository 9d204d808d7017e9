"""Multi-rank partition by Y-block ownership, exercised with gloo ranks on the
CPU: each rank evaluates its shard with the oracle into its own Y blocks, and
the union of the ranks' blocks equals the single-process result -- with no
reduction of Y across ranks."""
import os
import socket

import numpy as np
import pytest

from kronmult_gb300.shard import owner_of, plan_by_y_owner


def _case(seed=3, d=3, n=3, pool=8, nx=10, ny=9, ne=120):
    rng = np.random.default_rng(seed)
    N = n ** d
    return dict(d=d, n=n, pool=pool, Apool=rng.standard_normal((d, pool, n, n)),
                Xpool=rng.standard_normal((nx, N)), Y0=rng.standard_normal((ny, N)),
                y_idx=rng.geometric(0.25, ne) % ny, x_idx=rng.integers(0, nx, ne),
                a_idx=rng.integers(0, pool, (ne, d)))


def test_plan_is_a_partition_with_exclusive_y_blocks():
    rng = np.random.default_rng(0)
    y = rng.geometric(1 / 16, 5000) % 700
    for world in (1, 2, 3, 8):
        shards, ranges = plan_by_y_owner(y, world)
        allids = np.concatenate(shards)
        assert np.array_equal(np.sort(allids), np.arange(len(y)))
        owners = {}
        for r, ids in enumerate(shards):
            for yb in np.unique(y[ids]):
                assert owners.setdefault(int(yb), r) == r  # one owner per Y block
                assert owner_of(int(yb), ranges) == r
        sizes = [len(s) for s in shards]
        # balanced up to the largest Y block at each of the two cuts of a range
        assert max(sizes) - min(sizes) <= 2 * np.bincount(y).max() + 1


def _worker(rank, world, port, case, out):
    import torch.distributed as dist

    from oracle import pyoracle as po

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    shards, ranges = plan_by_y_owner(case["y_idx"], world)
    ids = shards[rank]
    Y = case["Y0"].copy()
    po.xbatched_idx(case["d"], case["n"], case["Apool"], case["n"], case["pool"], case["Xpool"], Y,
                    case["y_idx"][ids], case["x_idx"][ids], case["a_idx"][ids])
    lo, hi = ranges[rank]
    import torch

    # gather the owned blocks on rank 0 (test plumbing, not a data-path reduction)
    mine = torch.from_numpy(np.ascontiguousarray(Y[lo:hi]))
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([mine.numel()]))
    maxn = int(max(s.item() for s in sizes))
    buf = torch.zeros(maxn, dtype=torch.float64)
    buf[: mine.numel()] = mine.reshape(-1)
    got = [torch.zeros(maxn, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(got, buf)
    if rank == 0:
        N = case["n"] ** case["d"]
        Yfull = case["Y0"].copy()
        for r in range(world):
            a, b = ranges[r]
            Yfull[a:b] = got[r][: (b - a) * N].numpy().reshape(b - a, N)
        np.save(out, Yfull)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_match_single_process(oracle, tmp_path):
    import torch.multiprocessing as mp

    case = _case()
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "y.npy")
    mp.start_processes(_worker, args=(2, port, case, out), nprocs=2, join=True,
                       start_method="spawn")
    Yref = case["Y0"].copy()
    oracle.xbatched_idx(case["d"], case["n"], case["Apool"], case["n"], case["pool"],
                        case["Xpool"], Yref, case["y_idx"], case["x_idx"], case["a_idx"])
    got = np.load(out)
    # untouched blocks stay Y0; owned blocks equal the single-process sum
    assert np.allclose(got, Yref, rtol=1e-14, atol=1e-14)
