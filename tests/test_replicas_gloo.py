"""Multi-GPU runs of bench.py are independent replicas (the reference's step has no
collective).  The host-side coordination (barrier, max-over-ranks time) is checked with
two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root), str(root / "l-game_gb300"), str(root / "tests")]
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    ws, r, lr = bench.dist_info()
    dist = bench.dist_init(ws)
    bench.barrier(dist)
    t = bench.reduce_max(dist, 1.0 + rank)
    bench.barrier(dist)
    q.put((r, ws, t))
    dist.destroy_process_group()


def test_two_rank_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res == [(0, 2, 2.0), (1, 2, 2.0)]
