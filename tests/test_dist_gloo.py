"""The N>1 path's host logic on two gloo ranks (CPU)."""
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
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from cuspfft_gb300 import dist as gd
    ws, rk, lr = gd.world()
    ms = gd.job_ms_per_fft(10.0 * (rank + 1), steps=5, world_size=ws)
    q.put((rk, ws, lr, ms))
    dist.destroy_process_group()


def test_two_rank_timing_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # slowest rank (20 ms for 5 steps) over 2 ranks x 5 steps
    assert [r[3] for r in res] == pytest.approx([2.0, 2.0])
    assert [(r[0], r[1], r[2]) for r in res] == [(0, 2, 0), (1, 2, 1)]


def test_single_process_defaults():
    from cuspfft_gb300 import dist as gd
    assert gd.job_ms_per_fft(12.0, steps=4, world_size=1) == pytest.approx(3.0)
