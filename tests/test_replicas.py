"""Multi-GPU host logic on CPU: bench.py runs N independent replicas (the path
is not sharded across GPUs); the reported time is the maximum over ranks and
the throughput sums all ranks' work.  Exercised with 2 gloo ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 10.0 + 5.0 * rank                   # rank 1 is the slow one
    m = bench.reduce_max(ms, world, device="cpu")
    thr = bench.replica_throughput(1000.0, m * 1e-3, world)
    dist.barrier()
    q.put((rank, m, thr))
    dist.destroy_process_group()


def test_two_rank_replica_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert out[0][2] == pytest.approx(2 * 1000.0 / 0.015)


def test_single_rank_is_identity():
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.replica_throughput(10.0, 2.0, 1) == 5.0
