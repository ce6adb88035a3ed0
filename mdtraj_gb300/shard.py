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
