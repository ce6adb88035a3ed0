"""md.rmsd over frame shards, one process per GPU.

Frames are independent in the reference's loop (mdtraj/rmsd/_rmsd.pyx:
217-224, a prange over frames), so the path shards by contiguous frame ranges
with nothing exchanged on the data path: every rank holds the reference frame,
scores its own range of the target on its own GPU, and the (F,) results are
gathered once at the end (the only collective).  The result equals one
md.rmsd call on all frames bit for bit, because each frame's RMSD depends on
that frame and the reference frame alone.

    import torch.distributed as dist
    dist.init_process_group("nccl")          # one rank per GPU
    out = rmsd_sharded(traj, traj, 0)         # full (F,) array on every rank

Each rank centres its own frames in place exactly as md.rmsd does for the
frames it is given (the in-place side effect of the reference); frames of
other ranks are not touched on this rank.

allpairs_sharded does the same for the all-pairs RMSD matrix of the
clustering workload: the upper triangle is cut into blocks, each rank
computes a contiguous run of them (one cross-RMSD launch on its own GPU)
and one all-gather assembles the symmetric matrix on every rank.
"""
from __future__ import annotations

import numpy as np


def frame_range(n_frames: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous range [f0, f1) of rank `rank` among `world`: sizes differ by
    at most one frame, lower ranks take the larger ones."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(int(n_frames), world)
    f0 = rank * base + min(rank, extra)
    return f0, f0 + base + (1 if rank < extra else 0)


class _Frames:
    """The target restricted to a frame range: a view of .xyz (so md.rmsd's
    in-place centring lands in the caller's array), traces sliced alike."""

    def __init__(self, target, f0: int, f1: int):
        self.xyz = target.xyz[f0:f1]
        tr = getattr(target, "_rmsd_traces", None)
        self._rmsd_traces = None if tr is None else tr[f0:f1]


def rmsd_sharded(target, reference, frame: int = 0, atom_indices=None, ref_atom_indices=None, parallel=True,
                 precentered: bool = False, superpose: bool = True, *, group=None, score=None) -> np.ndarray:
    """md.rmsd(target, reference, frame, ...) with the frames of `target`
    split over the ranks of `group` (default: the default process group; no
    process group or a world of one runs a single md.rmsd).  Every rank
    passes the whole trajectory objects (host arrays); each scores only its
    range and all ranks receive the gathered float32 (F,) result.

    `score(target_part, reference, frame, ...)` computes one rank's part; it
    defaults to this package's md.rmsd on the rank's current CUDA device."""
    import torch
    import torch.distributed as dist

    if score is None:
        from ._rmsd import rmsd as score
    kwargs = dict(atom_indices=atom_indices, ref_atom_indices=ref_atom_indices, parallel=parallel,
                  precentered=precentered, superpose=superpose)
    if not (dist.is_available() and dist.is_initialized()):
        return np.asarray(score(target, reference, frame, **kwargs), dtype=np.float32)
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    n_frames = int(target.xyz.shape[0])
    f0, f1 = frame_range(n_frames, rank, world)
    part = np.asarray(score(_Frames(target, f0, f1), reference, frame, **kwargs), dtype=np.float32)
    if part.shape != (f1 - f0,):
        raise RuntimeError(f"rank {rank}: scored {part.shape} for frames [{f0}, {f1})")
    if world == 1:
        return part
    # one all-gather of equal-sized blocks (the largest range), on the
    # device the backend works on
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    width = frame_range(n_frames, 0, world)[1]
    block = torch.zeros(width, dtype=torch.float32, device=dev)
    block[: f1 - f0] = torch.from_numpy(part).to(dev)
    blocks = [torch.empty_like(block) for _ in range(world)]
    dist.all_gather(blocks, block, group=group)
    out = np.empty(n_frames, dtype=np.float32)
    for r, b in enumerate(blocks):
        a, e = frame_range(n_frames, r, world)
        out[a:e] = b[: e - a].cpu().numpy()
    return out


# ---------------------------------------------------------------------------
# All-pairs RMSD matrix over ranks
# ---------------------------------------------------------------------------

def default_block(n_frames: int, world: int, per_rank: int = 4) -> int:
    """Frames per block edge such that the upper triangle of blocks holds at
    least `per_rank` blocks per rank (so that equal runs of blocks balance)."""
    n_frames = max(1, int(n_frames))
    nb = 1
    while nb * (nb + 1) // 2 < per_rank * world and nb < n_frames:
        nb += 1
    return -(-n_frames // nb)


def triangle_blocks(n_frames: int, block: int) -> list[tuple[int, int]]:
    """Blocks (I, J) with I <= J of the n_frames x n_frames matrix cut into
    blocks of `block` frames, in row-major order."""
    nb = -(-int(n_frames) // int(block))
    return [(i, j) for i in range(nb) for j in range(i, nb)]


def row_requests(n_frames: int, block: int, rank: int, world: int) -> list[tuple[int, int, int, int]]:
    """Rank `rank`'s part of the upper triangle: a contiguous run of
    triangle_blocks (sizes differ by at most one block), merged per block
    row into (i0, i1, j0, j1) frame ranges -- a run crosses a block row at
    most once, so each row of frames appears in at most one range."""
    blocks = triangle_blocks(n_frames, block)
    b0, b1 = frame_range(len(blocks), rank, world)
    out: list[tuple[int, int, int, int]] = []
    for bi, bj in blocks[b0:b1]:
        i0, i1 = bi * block, min(n_frames, (bi + 1) * block)
        j0, j1 = bj * block, min(n_frames, (bj + 1) * block)
        if out and out[-1][0] == i0 and out[-1][3] == j0:
            out[-1] = (i0, i1, out[-1][2], j1)
        else:
            out.append((i0, i1, j0, j1))
    return out


def _gpu_rows(xyz: np.ndarray, requests, precentered: bool, method: str) -> list[np.ndarray]:
    """One rank's ranges on its GPU in one cross launch: the trajectory is
    prepared once as both the database and the query set, and range
    (i0, i1, j0, j1) is the request "query frames [i0, i1) against database
    frames [j0, j1)" (gbrmsd_cross_rmsd)."""
    import torch

    from . import _device as D
    from . import cross

    dev = D.require_device()
    F = int(xyz.shape[0])
    fs = cross.FrameSet.from_frames(np.ascontiguousarray(xyz, dtype=np.float32), centre=not precentered, device=dev)
    outs = [torch.empty((i1 - i0, j1 - j0), dtype=torch.float32, device=dev) for i0, i1, j0, j1 in requests]
    table = cross.request_table([(o.data_ptr(), i0, i1 - i0, j0, j1) for o, (i0, i1, j0, j1) in zip(outs, requests)])
    ws = cross.CrossWorkspace(dev).get(F, F, len(requests))
    stream = D.stream_handle()
    cross.cross_launch(fs, F, fs, table, len(requests), method, ws, stream)
    cross.cross_status(ws, stream)
    return [o.cpu().numpy() for o in outs]


def allpairs_sharded(target, precentered: bool = False, method: str = "tensor", *, group=None,
                     block: int | None = None, score=None) -> np.ndarray:
    """The all-pairs RMSD matrix (allpairs.allpairs_rmsd) with the upper
    triangle's blocks split over the ranks of `group` (default: the default
    process group; no process group runs one allpairs_rmsd call).  Every rank
    passes the whole trajectory; each computes a contiguous run of the
    triangle's blocks on its own GPU (its frames prepared once, locally: no
    peer memory is read) and one all-gather returns the full symmetric
    float32 (F, F) matrix to every rank, diagonal 0.

    `score(xyz, requests, precentered, method)` computes one rank's ranges
    (see row_requests) and returns one (i1 - i0, j1 - j0) array per range;
    it defaults to this package's cross RMSD on the rank's current device."""
    import torch
    import torch.distributed as dist

    xyz = target.xyz if hasattr(target, "xyz") else target
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    if xyz.ndim != 3 or xyz.shape[2] != 3:
        raise ValueError("expected coordinates of shape (n_frames, n_atoms, 3)")
    F = int(xyz.shape[0])
    if not (dist.is_available() and dist.is_initialized()):
        from .allpairs import allpairs_rmsd

        return allpairs_rmsd(xyz, precentered=precentered, method=method)
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    out = np.zeros((F, F), dtype=np.float32)
    if F == 0:
        return out
    block = int(block) if block else default_block(F, world)
    score = score or _gpu_rows
    mine = row_requests(F, block, rank, world)
    parts = score(xyz, mine, precentered, method) if mine else []
    sizes = [sum((i1 - i0) * (j1 - j0) for i0, i1, j0, j1 in row_requests(F, block, r, world)) for r in range(world)]
    flat = np.zeros(max(sizes), dtype=np.float32)
    k = 0
    for p, (i0, i1, j0, j1) in zip(parts, mine):
        if p.shape != (i1 - i0, j1 - j0):
            raise RuntimeError(f"rank {rank}: scored {p.shape} for frames [{i0}, {i1}) x [{j0}, {j1})")
        flat[k:k + p.size] = p.ravel()
        k += p.size
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    buf = torch.from_numpy(flat).to(dev)
    bufs = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(bufs, buf, group=group)
    for r, b in enumerate(bufs):
        b = b.cpu().numpy()
        k = 0
        for i0, i1, j0, j1 in row_requests(F, block, r, world):
            n = (i1 - i0) * (j1 - j0)
            out[i0:i1, j0:j1] = b[k:k + n].reshape(i1 - i0, j1 - j0)
            k += n
    # each unordered pair once (the upper triangle), mirrored; diagonal 0
    upper = np.triu(out, 1)
    return upper + upper.T
