"""XTC trajectories decoded on the GPU.

The reference reads XTC files on the host (mdtraj/formats/xtc/xtc.pyx over
xdrfile.c); here the file bytes go to the device as they are and one GPU
thread per frame decodes the compressed coordinates straight into the padded
layout the RMSD kernels read (gbrmsd_xtc_index / gbrmsd_xtc_decode).

    xyz, time, step, box = load_xtc(path)          # like XTCTrajectoryFile.read()
    for chunk in iter_xtc(path, chunk_bytes): ...   # device frames, chunk by chunk
    rmsd = rmsd_xtc(path, reference_xyz)            # md.rmsd(load(path), ref) streamed
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _device as D
from . import _lib
from ._lib import check, lib


@dataclass
class XtcChunk:
    """Frames decoded on the device: xyz is (n_frames, 3 * n_padded) float32,
    atom-major, padding atoms zero; step / time / box per frame."""

    xyz: torch.Tensor
    n_atoms: int
    n_padded: int
    step: torch.Tensor
    time: torch.Tensor
    box: torch.Tensor
    first_frame: int

    @property
    def n_frames(self) -> int:
        return int(self.xyz.shape[0])


def index_bytes(data: np.ndarray, capacity: int | None = None):
    """(frame offsets int64, n_atoms, bytes spanned by the complete frames) of
    an XTC byte buffer that starts at a frame boundary."""
    data = np.ascontiguousarray(data, dtype=np.uint8)
    n = C.c_int64()
    A = C.c_int32()
    used = C.c_int64()
    check(lib.gbrmsd_xtc_index(data.ctypes.data, data.size, None, 0, C.byref(n), C.byref(A), C.byref(used)))
    offsets = np.zeros(max(1, n.value if capacity is None else min(capacity, n.value)), dtype=np.int64)
    check(lib.gbrmsd_xtc_index(data.ctypes.data, data.size, offsets.ctypes.data, offsets.size, C.byref(n),
                               C.byref(A), C.byref(used)))
    return offsets[:n.value], int(A.value), int(used.value)


def decode_bytes(data: np.ndarray, offsets: np.ndarray, n_atoms: int, device=None, first_frame: int = 0) -> XtcChunk:
    """Decodes the frames at `offsets` of a host XTC byte buffer on the device."""
    device = device if device is not None else D.require_device()
    F = len(offsets)
    Ap = D.padded(n_atoms)
    d_data = torch.from_numpy(np.ascontiguousarray(data, dtype=np.uint8)).to(device)
    d_off = torch.from_numpy(np.ascontiguousarray(offsets, dtype=np.int64)).to(device)
    xyz = torch.zeros((F, 3 * Ap), dtype=torch.float32, device=device)
    step = torch.empty(F, dtype=torch.int32, device=device)
    time = torch.empty(F, dtype=torch.float32, device=device)
    box = torch.empty((F, 3, 3), dtype=torch.float32, device=device)
    status = torch.empty(F, dtype=torch.int32, device=device)
    if F:
        check(lib.gbrmsd_xtc_decode(d_data.data_ptr(), d_data.numel(), d_off.data_ptr(), F, n_atoms,
                                    xyz.data_ptr(), 3 * Ap, step.data_ptr(), time.data_ptr(), box.data_ptr(),
                                    status.data_ptr(), D.stream_handle()))
        bad = torch.nonzero(status).flatten()
        if bad.numel():
            i = int(bad[0])
            raise ValueError(f"XTC frame {first_frame + i} could not be decoded (status {int(status[i])})")
    return XtcChunk(xyz, n_atoms, Ap, step, time, box, first_frame)


def iter_xtc(path, chunk_bytes: int = 256 << 20, device=None):
    """Yields XtcChunk objects covering the file in order, each holding the
    complete frames of about `chunk_bytes` of the file."""
    device = device if device is not None else D.require_device()
    first = 0
    with open(path, "rb") as fh:
        carry = np.zeros(0, dtype=np.uint8)
        while True:
            block = np.empty(chunk_bytes, dtype=np.uint8)
            block = block[:fh.readinto(memoryview(block))]
            data = np.concatenate([carry, block]) if carry.size else block
            if data.size == 0:
                return
            offsets, A, used = index_bytes(data)
            if len(offsets) == 0:
                if block.size == 0:
                    raise ValueError("truncated XTC file: %d trailing bytes" % data.size)
                carry = data.copy()
                continue
            yield decode_bytes(data[:used], offsets, A, device, first)
            first += len(offsets)
            carry = data[used:].copy()
            if block.size == 0 and carry.size:
                raise ValueError("truncated XTC file: %d trailing bytes" % carry.size)


def load_xtc(path, device=None):
    """Coordinates (n_frames, n_atoms, 3) float32, time, step, box (n_frames,
    3, 3) as host arrays, like XTCTrajectoryFile(path).read()."""
    xs, ts, ss, bs = [], [], [], []
    A = 0
    for ch in iter_xtc(path, device=device):
        A = ch.n_atoms
        xs.append(ch.xyz.view(ch.n_frames, ch.n_padded, 3)[:, :A].contiguous().cpu().numpy())
        ts.append(ch.time.cpu().numpy())
        ss.append(ch.step.cpu().numpy())
        bs.append(ch.box.cpu().numpy())
    if not xs:
        return (np.zeros((0, 0, 3), np.float32), np.zeros(0, np.float32), np.zeros(0, np.int32),
                np.zeros((0, 3, 3), np.float32))
    return np.concatenate(xs), np.concatenate(ts), np.concatenate(ss), np.concatenate(bs)


def rmsd_xtc(path, reference, frame: int = 0, chunk_bytes: int = 256 << 20) -> np.ndarray:
    """md.rmsd(trajectory, reference, frame) for the trajectory stored in the
    XTC file at `path`, decoded and scored on the device chunk by chunk
    (the file's frames are not centred on the host; nothing but the bytes
    crosses the host link).  reference: object with .xyz or an array."""
    device = D.require_device()
    ref_xyz = reference.xyz if hasattr(reference, "xyz") else reference
    ref_frame = np.ascontiguousarray(np.asarray(ref_xyz, dtype=np.float32)[frame])
    dref = None
    outs = []
    for ch in iter_xtc(path, chunk_bytes, device):
        if dref is None:
            if ref_frame.shape[0] != ch.n_atoms:
                raise ValueError("Input trajectories must have same number of atoms. found %d and %d."
                                 % (ch.n_atoms, ref_frame.shape[0]))
            dref = D.DeviceReference(ref_frame, _lib.ATOM_MAJOR, centre=True, device=device)
        outs.append(D.rmsd_to_reference(ch.xyz, ch.n_frames, ch.n_atoms, ch.n_padded, _lib.ATOM_MAJOR,
                                        _lib.MODE_CENTER, dref).cpu().numpy())
    return np.concatenate(outs) if outs else np.zeros(0, np.float32)
