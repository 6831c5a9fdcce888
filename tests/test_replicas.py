"""Multi-GPU form of the benchmark: N independent replicas (the guiding step
has no exchange between GPUs in this build). Checked on CPU with two gloo
ranks: each replica gets its own inputs, and the job's time is the maximum
over the ranks, so the reported whole-job throughput is units of all ranks
over the slowest rank's time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    t = bench.barrier_max(1.0 + rank, ws)  # rank r "took" 1 + r seconds
    out.put((rank, t, bench.replica_seed(rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_time_is_max_and_inputs_differ():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in res] == [2.0, 2.0]
    assert res[0][2] != res[1][2]
