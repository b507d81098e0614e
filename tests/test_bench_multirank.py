"""The bench's multi-rank aggregation (one replica per GPU, scaling "weak") on CPU with gloo,
world size 2: every rank gets the slowest rank's time and the whole-job throughput; a rank that
fails to join makes the others' collective end with an error instead of hanging."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, times, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    t, v = bench.job_throughput(dist, times[rank], 1000, 10, world)
    q.put((rank, t, v))
    dist.barrier()
    dist.destroy_process_group()


def test_job_throughput_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [0.5, 2.0]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in out:
        assert t == 2.0
        assert v == 2 * 1000 * 10 / 2.0


def _lonely(port, q):
    import datetime
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=2,
                            timeout=datetime.timedelta(seconds=5))
    q.put("joined")


def test_missing_rank_ends_with_an_error():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_lonely, args=(_free_port(), q))
    p.start()
    p.join(timeout=120)
    assert p.exitcode not in (0, None)
    if p.is_alive():
        p.kill()


def test_fp64_roofline_arithmetic():
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r = bench.fp64_roofline(0.6, 199996)
    assert abs(r["peak"] - 629.28) < 1e-9
    assert abs(r["achieved"] - 1420 * 199996 / 0.6e-3 / 1e9) < 1e-9
    assert 0.7 < r["frac"] < 0.8


def test_each_rank_gets_its_own_gpu():
    """Under torchrun every rank sees one GPU as device 0: its own entry of an inherited device list
    (a launcher may export all of the node's GPUs), or the GPU with its local rank's number."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_visible_devices(3, None) == "3"
    assert bench.rank_visible_devices(3, "") == "3"
    assert bench.rank_visible_devices(3, "0,1,2,3,4,5,6,7") == "3"
    assert bench.rank_visible_devices(1, "4,5") == "5"
    assert bench.rank_visible_devices(0, "6") == "6"
    assert bench.rank_visible_devices(2, " 2, 3, 4 ") == "4"
