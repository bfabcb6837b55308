"""The multi-GPU path of bench.py is replicas only (the SpMV / power-method
path does not shard on a single-GPU pool): N ranks each run the full
workload, the job time is the slowest rank's, and the value is all ranks'
bytes over that time.  Checked here with two gloo ranks on the CPU
(127.0.0.1 rendezvous), using the bench's own helpers."""
import os
import sys

import pytest

from conftest import ROOT


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 2.0 + rank  # rank 1 is the slow one
    bench.barrier(world)
    mx = bench.max_over_ranks(ms, world, device="cpu")
    q.put((rank, mx, bench.replica_gbs(1e9, mx, world)))
    dist.destroy_process_group()


def test_two_replicas_take_slowest_rank_and_sum_bytes():
    torch = pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [3.0, 3.0]
    # 2 ranks x 1e9 bytes in 3 ms
    assert all(abs(o[2] - 2e9 / 3e-3 / 1e9) < 1e-9 for o in out)
