"""Multi-rank host logic on gloo ranks on the CPU: the benchmark's frame
sharding and max-over-ranks timing (frames shard with no data-path
collective; the only collective is the MAX of the per-rank timings), and
the product's sharded md.rmsd (mdtraj_gb300.shard), whose gathered result
must equal one call over all frames bit for bit."""
import os
import socket

import numpy as np
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


def _oracle_score(t, r, frame, **kw):
    """md.rmsd's CPU path of the reference (compiled reference, or the C
    restatement) on one rank's frames; centres them in place like md.rmsd."""
    from oracle import cpu

    impl = cpu.best_available()
    return impl.md_rmsd(t.xyz, np.ascontiguousarray(r.xyz[frame]).copy())


class _Traj:
    def __init__(self, xyz):
        self.xyz = xyz
        self._rmsd_traces = None


def _shard_worker(rank, world, port, q):
    import torch.distributed as dist

    from mdtraj_gb300 import synth
    from mdtraj_gb300.shard import frame_range, rmsd_sharded

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _, x = synth.single_reference_frames(1001, 57, seed=11, sigma=np.geomspace(1e-3, 0.3, 1001),
                                             exact_fraction=0.02)
        t = _Traj(x)
        out = rmsd_sharded(t, _Traj(x.copy()), 3, score=_oracle_score)
        f0, f1 = frame_range(1001, rank, world)
        q.put((rank, out, f0, f1, t.xyz[f0:f1].copy()))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_rmsd_sharded_over_gloo_ranks_equals_one_call(world):
    """Each rank scores its own frame range, the (F,) results are gathered
    once, and the gathered array equals one md.rmsd over all frames bit for
    bit; each rank's in-place centring of its frames equals the one call's."""
    import torch.multiprocessing as mp

    from mdtraj_gb300 import synth
    from mdtraj_gb300.shard import frame_range

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=180) for _ in range(world)), key=lambda v: v[0])
    for p in procs:
        p.join(60)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    _, x = synth.single_reference_frames(1001, 57, seed=11, sigma=np.geomspace(1e-3, 0.3, 1001), exact_fraction=0.02)
    whole = _Traj(x)
    want = _oracle_score(whole, _Traj(x.copy()), 3)
    sizes = [f1 - f0 for _, _, f0, f1, _ in res]
    assert sum(sizes) == 1001 and max(sizes) - min(sizes) <= 1
    for rank, out, f0, f1, centred in res:
        assert (f0, f1) == frame_range(1001, rank, world)
        np.testing.assert_array_equal(out, want)
        np.testing.assert_array_equal(centred, whole.xyz[f0:f1])


def test_frame_range_covers_frames_once():
    from mdtraj_gb300.shard import frame_range

    for n in (0, 1, 7, 1000, 1001):
        for w in (1, 2, 3, 8):
            seen = np.zeros(n, int)
            for r in range(w):
                a, b = frame_range(n, r, w)
                seen[a:b] += 1
            assert np.all(seen == 1)
    with pytest.raises(ValueError):
        frame_range(10, 2, 2)


def test_row_requests_cover_the_upper_triangle_once():
    """The block partition of allpairs_sharded: over the ranks, every pair
    i <= j is in exactly one range, no range reaches below the diagonal's
    block, and each rank's ranges are disjoint block rows."""
    from mdtraj_gb300.shard import default_block, row_requests, triangle_blocks

    for F in (1, 2, 5, 64, 97, 300, 1001):
        for world in (1, 2, 3, 5, 8):
            for block in {default_block(F, world), 1, 7, 64, F}:
                cover = np.zeros((F, F), int)
                for r in range(world):
                    rows = set()
                    for i0, i1, j0, j1 in row_requests(F, block, r, world):
                        assert 0 <= i0 < i1 <= F and 0 <= j0 < j1 <= F and i0 <= j0
                        assert i0 not in rows
                        rows.add(i0)
                        cover[i0:i1, j0:j1] += 1
                iu = np.triu_indices(F)
                assert np.all(cover[iu] == 1), (F, world, block)
                assert len(triangle_blocks(F, block)) == (-(-F // block)) * (-(-F // block) + 1) // 2
    # default_block: at least four blocks per rank, unless blocks are already
    # one frame wide
    for F, world in ((20_000, 8), (4000, 3), (10, 16), (3, 2)):
        b = default_block(F, world)
        nb = -(-F // b)
        assert nb * (nb + 1) // 2 >= 4 * world or b == 1, (F, world, b)


def _fp64_rows(xyz, requests, precentered, method):
    """FP64 Kabsch RMSD of each range's frame pairs (the oracle), as the
    per-rank scorer of allpairs_sharded."""
    from oracle import fp64

    out = []
    for i0, i1, j0, j1 in requests:
        blk = np.empty((i1 - i0, j1 - j0), np.float32)
        for b, j in enumerate(range(j0, j1)):
            blk[:, b] = fp64.kabsch_rmsd(xyz[i0:i1], xyz[j])
        out.append(blk)
    return out


def _allpairs_worker(rank, world, port, q):
    import torch.distributed as dist

    from mdtraj_gb300 import synth
    from mdtraj_gb300.shard import allpairs_sharded

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _, x = synth.single_reference_frames(61, 17, seed=21, sigma=0.2)
        q.put((rank, allpairs_sharded(x, score=_fp64_rows)))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_allpairs_sharded_over_gloo_ranks_equals_the_whole_triangle(world):
    """Each rank computes its run of the upper triangle's blocks; after one
    all-gather every rank holds the same symmetric matrix, equal bit for bit
    to the whole triangle computed at once, diagonal 0."""
    import torch.multiprocessing as mp

    from mdtraj_gb300 import synth
    from mdtraj_gb300.shard import default_block, row_requests

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_allpairs_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=180) for _ in range(world)), key=lambda v: v[0])
    for p in procs:
        p.join(60)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    _, x = synth.single_reference_frames(61, 17, seed=21, sigma=0.2)
    (whole,) = _fp64_rows(x, [(0, 61, 0, 61)], False, "tensor")
    want = np.triu(whole, 1) + np.triu(whole, 1).T
    for _, out in res:
        np.testing.assert_array_equal(out, want)
    # the ranks' ranges cover the upper triangle once, a frame row at most once per rank
    B = default_block(61, world)
    cover = np.zeros((61, 61), int)
    for r in range(world):
        reqs = row_requests(61, B, r, world)
        assert len({i0 for i0, _, _, _ in reqs}) == len(reqs)
        for i0, i1, j0, j1 in reqs:
            cover[i0:i1, j0:j1] += 1
    iu = np.triu_indices(61, 1)
    assert cover.max() == 1 and np.all(cover[iu] == 1)
