"""bench.py's multi-process path on CPU: two gloo ranks on 127.0.0.1.

The transport step does not exchange data between GPUs: `bench.py --gpus N`
runs N independent replicas, joined only by a barrier around the timed region
and the maximum of the ranks' times.  This checks that path (process-group
setup from the torchrun environment, barrier, max over ranks, whole-job rate)
without a GPU.
"""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.barrier(w)
    # each replica timed a different number of milliseconds; the job takes the slowest
    ms = bench.max_over_ranks(10.0 + rank, w)
    cells, nt = 1000, 2
    value = w * cells * nt / (ms / 1e3)
    out.put((rank, ms, value))
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, ms, value in res:
        assert ms == pytest.approx(11.0)
        assert value == pytest.approx(2 * 1000 * 2 / 0.011)
