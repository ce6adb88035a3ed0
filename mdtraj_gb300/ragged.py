"""Ragged batches: many trajectories with different atom and frame counts,
each scored against its own frame 0 (``[md.rmsd(t, t, 0) for t in trajs]``,
the reference's per-trajectory loop over mdtraj/rmsd/_rmsd.pyx:64-243), in
one persistent launch that can be captured in a CUDA graph.

Trajectories are packed into one padded atom-major device buffer; the
launch configuration (warps, stage size, stages, largest work unit) comes
from the autotuner's cache for the batch's shape bucket, or is tuned on the
spot when ``autotune=True``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _device as D
from . import _lib
from ._lib import check, lib


def _pack_layout(atoms, frames):
    atoms = np.asarray(atoms, dtype=np.int32)
    frames = np.asarray(frames, dtype=np.int64)
    padded = ((atoms + 3) // 4 * 4).astype(np.int32)
    sizes = frames * 3 * padded.astype(np.int64)
    offsets = np.zeros(len(atoms), dtype=np.int64)
    offsets[1:] = np.cumsum(sizes)[:-1]
    return offsets, atoms, padded, frames, int(sizes.sum())


class RaggedBatch:
    """A packed batch on the device.

    Build from host arrays (``trajectories``: list of float32 (F_s, A_s, 3)) or
    from an already packed device buffer (``packed``: (x, atoms, frames) with
    x laid out by ``RaggedBatch.layout(atoms, frames)``).
    """

    def __init__(self, trajectories=None, *, packed=None, device=None, config=None, max_unit_quads=None,
                 autotune: bool = False):
        self.device = device if device is not None else D.require_device()
        if packed is not None:
            x, atoms, frames = packed
            self.offsets, self.atoms, self.padded, self.frames, total = _pack_layout(atoms, frames)
            if x.numel() < total:
                raise ValueError("packed buffer smaller than the layout of the given segments")
            self.x = x
        else:
            if not trajectories:
                raise ValueError("need at least one trajectory")
            arrs = [np.ascontiguousarray(t.xyz if hasattr(t, "xyz") else t, dtype=np.float32) for t in trajectories]
            for a in arrs:
                if a.ndim != 3 or a.shape[2] != 3 or a.shape[0] < 1 or a.shape[1] < 1:
                    raise ValueError("each trajectory must be (n_frames >= 1, n_atoms >= 1, 3)")
            self.offsets, self.atoms, self.padded, self.frames, total = _pack_layout(
                [a.shape[1] for a in arrs], [a.shape[0] for a in arrs])
            self.x = torch.zeros(max(total, 4), dtype=torch.float32, device=self.device)
            stream = D.stream_handle()
            for a, off, Ap in zip(arrs, self.offsets, self.padded):
                F, A = a.shape[0], a.shape[1]
                dst = self.x.data_ptr() + int(off) * 4
                if D.pageable_access():
                    check(lib.gbrmsd_copy_rows_kernel(dst, 3 * int(Ap), a.ctypes.data, 3 * A, 3 * A, 3 * int(Ap), F,
                                                      stream))
                else:
                    D.copy_rows(dst, 12 * int(Ap), a.ctypes.data, 12 * A, 12 * A, F, 1, stream)
            torch.cuda.current_stream().synchronize()
        self.n_seg = len(self.atoms)
        self.total_frames = int(self.frames.sum())
        self.bytes = int((12 * self.atoms.astype(np.int64) * self.frames).sum())
        if config is None and max_unit_quads is None:
            from .autotune import ragged_choice

            config, max_unit_quads = ragged_choice(self, autotune=autotune)
        self.configure(config if config is not None else 0, max_unit_quads if max_unit_quads is not None else 512)

    @staticmethod
    def layout(atoms, frames):
        """(float offsets, padded atom counts, total floats) of a packed buffer."""
        off, _, padded, _, total = _pack_layout(atoms, frames)
        return off, padded, total

    def _arrays(self):
        return (self.offsets.ctypes.data, self.atoms.ctypes.data, self.padded.ctypes.data, self.frames.ctypes.data)

    def configure(self, config: int, max_unit_quads: int) -> None:
        plan = _lib.RaggedPlan()
        check(lib.gbrmsd_ragged_plan(*self._arrays(), self.n_seg, int(config), int(max_unit_quads), C.addressof(plan)))
        self.plan = plan
        self.ws = D.empty_bytes(plan.ws_bytes, self.device)
        check(lib.gbrmsd_ragged_setup(self.x.data_ptr(), *self._arrays(), C.addressof(plan), self.ws.data_ptr(),
                                      self.ws.numel(), D.stream_handle()))
        self.out = torch.empty(self.total_frames, dtype=torch.float32, device=self.device)
        self.graph = None

    def run(self) -> torch.Tensor:
        """One persistent launch over the whole batch (current stream)."""
        check(lib.gbrmsd_ragged_rmsd(self.x.data_ptr(), self.out.data_ptr(), C.addressof(self.plan),
                                     self.ws.data_ptr(), self.ws.numel(), D.stream_handle()))
        return self.out

    def capture(self) -> "torch.cuda.CUDAGraph":
        """Captures run() in a CUDA graph (replayed by replay())."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run()  # warm-up outside the capture: sets kernel attributes
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def replay(self) -> torch.Tensor:
        if self.graph is None:
            self.capture()
        self.graph.replay()
        return self.out

    def results(self) -> list:
        """Per-trajectory float32 numpy arrays of the last run."""
        host = self.out.cpu().numpy()
        bounds = np.concatenate([[0], np.cumsum(self.frames)])
        return [host[bounds[i]:bounds[i + 1]] for i in range(self.n_seg)]


def ragged_rmsd(trajectories, *, autotune: bool = False) -> list:
    """``[md.rmsd(t, t, 0) for t in trajectories]`` in one launch: each
    trajectory (object with ``.xyz`` or a float32 (F, A, 3) array) is scored
    against its own frame 0.  Inputs are not modified."""
    b = RaggedBatch(trajectories, autotune=autotune)
    b.run()
    return b.results()
