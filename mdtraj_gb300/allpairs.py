"""All-pairs RMSD matrix (the clustering workload of mdtraj's
examples/clustering.ipynb: ``D[i] = md.rmsd(traj, traj, i, precentered=True)``
for every i), computed as one symmetric matrix on the GB300.

``method="tensor"`` uses split-BF16 tcgen05 tensor-core tiles (hi + lo
planes, FP32 accumulation); ``method="fp32"`` uses plain FP32 CUDA-core
tiles.  Both solve QCP per pair in FP32 and recompute near-identical pairs
exactly.  Diagonal entries are exactly 0, like the reference's self-pair
shortcut.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _device as D
from . import _lib
from ._lib import check, lib

METHODS = {"fp32": 0, "tensor": 1}


def allpairs_device(x: torch.Tensor, n_frames: int, n_atoms: int, n_padded: int, layout: int, *,
                    centre: bool = True, method: str = "tensor", out: torch.Tensor | None = None,
                    ws: torch.Tensor | None = None) -> torch.Tensor:
    """Device-resident all-pairs RMSD; x is a padded frame buffer (see
    gbrmsd_allpairs).  Returns the (n_frames, n_frames) float32 tensor."""
    if method not in METHODS:
        raise ValueError(f"method must be one of {sorted(METHODS)}")
    device = x.device
    if out is None:
        out = torch.empty((n_frames, n_frames), dtype=torch.float32, device=device)
    need = lib.gbrmsd_allpairs_workspace_bytes(n_frames, n_atoms)
    if ws is None or ws.numel() < need:
        ws = D.empty_bytes(need, device)
    check(lib.gbrmsd_allpairs(x.data_ptr(), n_frames, n_atoms, n_padded, 3 * n_padded, layout, int(centre),
                              METHODS[method], out.data_ptr(), ws.data_ptr(), ws.numel(), D.stream_handle()))
    return out


def allpairs_rmsd(target, precentered: bool = False, method: str = "tensor") -> np.ndarray:
    """All-pairs RMSD matrix of a trajectory (object with ``.xyz`` or a
    (n_frames, n_atoms, 3) float32 array).  Returns float32 (F, F).

    precentered=True uses the coordinates as given (already centred, e.g.
    after ``center_coordinates()``); otherwise frames are centred first
    (without modifying the caller's coordinates)."""
    xyz = target.xyz if hasattr(target, "xyz") else target
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    if xyz.ndim != 3 or xyz.shape[2] != 3:
        raise ValueError("expected coordinates of shape (n_frames, n_atoms, 3)")
    F, A = xyz.shape[0], xyz.shape[1]
    if F == 0:
        return np.zeros((0, 0), dtype=np.float32)
    device = D.require_device()
    stream = D.stream_handle()
    x_dev, n_padded = D.frames_to_device(xyz, _lib.ATOM_MAJOR, device, stream)
    ws = D.empty_bytes(lib.gbrmsd_allpairs_workspace_bytes(F, A), device)
    out = allpairs_device(x_dev, F, A, n_padded, _lib.ATOM_MAJOR, centre=not precentered, method=method, ws=ws)
    result = D.to_host(out, stream)
    # raises when the device recorded an error (an expired wait)
    check(lib.gbrmsd_allpairs_status(ws.data_ptr(), None, stream))
    return result
