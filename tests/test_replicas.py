"""The multi-GPU mode of bench.py is "replicas only" (independent chains, no
collective on the data path). Its only cross-rank step is the max-over-ranks
timing; check it with world_size 2 over gloo on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, seconds, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(torch, dist, seconds[rank], "cpu")
    q.put((rank, t))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    seconds = [1.25, 3.5]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, seconds, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 3.5, 1: 3.5}


def test_single_process_needs_no_collective():
    import torch
    import bench
    assert bench.max_over_ranks(torch, None, 2.0, "cpu") == 2.0


def test_every_kernel_class_has_roofline_figures(pkg):
    """bench.py's algorithmic bytes and flops cover every kernel class the
    library times, except the catch-all class of starts and copies."""
    import bench
    from gaugefields_gb300 import _lib
    for k in _lib.KERNEL_CLASSES:
        if k == "other":
            continue
        assert bench.algorithmic_bytes_per_link(k) > 0 and bench.algorithmic_flops_per_link(k) > 0, k
        assert k in _lib.KERNEL_PRECISION, k
