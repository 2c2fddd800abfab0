"""Multi-GPU is replicas only (each rank renders its own frames; no collective on the data path).
The host logic bench.py uses across ranks -- barrier, max-over-ranks time, whole-job throughput --
is exercised here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    t = bench.max_over_ranks(1.0 + rank, pg)     # rank 1 is the slowest
    frames_per_rank = 10
    fps = w * frames_per_rank / t
    q.put((r, w, t, fps))
    pg.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_replicas_take_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=100) for _ in procs]
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, world, t, fps in res:
        assert world == 2
        assert t == 2.0          # max over ranks
        assert fps == 10.0       # 2 ranks x 10 frames / 2 s
