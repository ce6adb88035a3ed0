"""Multi-rank host logic of the benchmark (frame sharding, max-over-ranks
timing) on two gloo ranks on the CPU: frames shard with no data-path
collective; the only collective is the MAX of the per-rank timings."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        f0, f1 = bench.shard(1000, r, w)
        slowest = bench.max_over_ranks(1.5 + r, w)
        q.put((r, w, local, f0, f1, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_time():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(2))
    (r0, w0, l0, a0, b0, s0), (r1, w1, l1, a1, b1, s1) = got
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert (a0, b0, a1, b1) == (0, 1000, 1000, 2000)  # weak scaling: disjoint, equal per-rank work
    assert s0 == s1 == 2.5                             # every rank reports the slowest rank's time
