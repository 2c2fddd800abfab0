"""Multi-GPU is replicas only (each rank renders its own frames; no collective on the data path).
The host logic bench.py uses across ranks -- barrier, max-over-ranks time, whole-job throughput --
is exercised here with two gloo ranks on the CPU, once with fixed times and once with each rank
rendering frames through the scene harness (the CPU checker library standing in for a rank's GPU)
and the ranks comparing digests of their images."""
import hashlib
import os
import socket
import sys
import time

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


def _render_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch
    import bench
    import oracle
    from helpers import render
    from softglrender_gb300 import scenes as S
    oracle.build()
    lib = oracle.restatement()
    w, r, local, pg = bench.dist_setup()
    scene = S.config_plain_small(width=96, height=64, lon=16, lat=8, tex=32)
    frames = 2
    bench.barrier(pg)
    t0 = time.perf_counter()
    for _ in range(frames):
        outs, _ = render(lib, scene)
    dt = time.perf_counter() - t0
    bench.barrier(pg)
    t = bench.max_over_ranks(dt, pg)
    h = hashlib.sha256()
    for o in outs:
        for k in sorted(o):
            h.update(o[k].tobytes())
    mine = torch.tensor(list(h.digest()), dtype=torch.int64)
    all_d = [torch.zeros_like(mine) for _ in range(w)]
    pg.all_gather(all_d, mine)
    same = all(torch.equal(d, all_d[0]) for d in all_d)
    drawn = any(bool((o["depth"] != o["depth"].flat[0]).any()) for o in outs)
    q.put((r, w, dt, t, w * frames / t, same, drawn))
    pg.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_replicas_render_identical_frames():
    """Each rank renders the same workload on its own; the images agree across ranks, and the
    whole-job rate counts every rank's frames against the slowest rank's time."""
    import oracle
    oracle.build()   # once, before the ranks load it
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_render_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=280) for _ in procs]
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    slowest = max(dt for _, _, dt, _, _, _, _ in res)
    for rank, world, dt, t, fps, same, drawn in res:
        assert world == 2 and same and drawn
        assert t == slowest
        assert abs(fps - 2 * 2 / slowest) < 1e-9
