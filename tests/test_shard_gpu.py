"""Y-block ownership sharding with the CUDA library: two gloo ranks (CPU
process group), each running kmx_kronmult_xbatched_f64 on its shard of one
batch against its own range of Y blocks, on the visible GPU.  Nothing is
reduced across ranks on the data path; the ranks' Y ranges are gathered on
rank 0 over gloo only to compare their union with the oracle's
single-process result.  The ranks' kernels never wait on each other."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _case(seed=11, d=6, n=4, pool=32, nx=24, ny=40, ne=900):
    rng = np.random.default_rng(seed)
    N = n ** d
    return dict(d=d, n=n, pool=pool, Apool=rng.standard_normal((d, pool, n, n)) / 2,
                Xpool=rng.standard_normal((nx, N)), Y0=rng.standard_normal((ny, N)),
                y_idx=rng.geometric(1 / 16, ne) % ny, x_idx=rng.integers(0, nx, ne),
                a_idx=rng.integers(0, pool, (ne, d)))


def _worker(rank, world, port, case, out):
    import sys

    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import kronmult_gb300 as kmx
    from kronmult_gb300.shard import plan_by_y_owner

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    d, n, pool = case["d"], case["n"], case["pool"]
    N = n ** d
    shards, ranges = plan_by_y_owner(case["y_idx"], world)
    ids = np.sort(shards[rank])
    lo, hi = ranges[rank]
    Ad = torch.from_numpy(case["Apool"]).cuda()
    Xd = torch.from_numpy(case["Xpool"]).cuda()
    Yd = torch.from_numpy(np.ascontiguousarray(case["Y0"][lo:hi])).cuda()  # owned blocks only
    a_idx, x_idx, y_idx = case["a_idx"][ids], case["x_idx"][ids], case["y_idx"][ids] - lo
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    pY = kmx.pointer_array(Yd, y_idx * N)
    if len(ids):
        kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, len(ids))
    torch.cuda.synchronize()
    kmx.check_device_status()
    mine = Yd.cpu().reshape(-1)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([mine.numel()]))
    maxn = int(max(s.item() for s in sizes))
    buf = torch.zeros(maxn, dtype=torch.float64)
    buf[: mine.numel()] = mine
    got = [torch.zeros(maxn, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(got, buf)
    if rank == 0:
        Yfull = case["Y0"].copy()
        for r in range(world):
            a, b = ranges[r]
            Yfull[a:b] = got[r][: (b - a) * N].numpy().reshape(b - a, N)
        np.save(out, Yfull)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_run_their_y_shards_on_the_gpu(oracle, tmp_path):
    import torch.multiprocessing as mp

    from tests.common import blockwise_rel_err

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
    assert blockwise_rel_err(got - case["Y0"], Yref - case["Y0"]) <= 1e-13
