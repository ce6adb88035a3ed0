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
import os
import queue
import threading
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


_COPY_STREAMS: dict = {}


def _copy_stream(device) -> torch.cuda.Stream:
    key = (device.type, device.index)
    if key not in _COPY_STREAMS:
        _COPY_STREAMS[key] = torch.cuda.Stream(device=device)
    return _COPY_STREAMS[key]


def _decode_launch(data: np.ndarray, offsets: np.ndarray, n_atoms: int, device, first_frame: int):
    """Queues the decode of the frames at `offsets` on torch's current stream
    and returns (XtcChunk, per-frame status tensor) without waiting for it.
    The file bytes go up on a side stream (the host thread waits for that
    copy only, not for earlier kernels), then the decode waits for them."""
    F = len(offsets)
    Ap = D.padded(n_atoms)
    cur = torch.cuda.current_stream(device)
    side = _copy_stream(device)
    with torch.cuda.stream(side):
        d_data = torch.from_numpy(np.ascontiguousarray(data, dtype=np.uint8)).to(device)
        d_off = torch.from_numpy(np.ascontiguousarray(offsets, dtype=np.int64)).to(device)
    cur.wait_stream(side)
    d_data.record_stream(cur)
    d_off.record_stream(cur)
    xyz = torch.zeros((F, 3 * Ap), dtype=torch.float32, device=device)
    step = torch.empty(F, dtype=torch.int32, device=device)
    time = torch.empty(F, dtype=torch.float32, device=device)
    box = torch.empty((F, 3, 3), dtype=torch.float32, device=device)
    status = torch.zeros(F, dtype=torch.int32, device=device)
    if F:
        check(lib.gbrmsd_xtc_decode(d_data.data_ptr(), d_data.numel(), d_off.data_ptr(), F, n_atoms,
                                    xyz.data_ptr(), 3 * Ap, step.data_ptr(), time.data_ptr(), box.data_ptr(),
                                    status.data_ptr(), cur.cuda_stream))
    return XtcChunk(xyz, n_atoms, Ap, step, time, box, first_frame), status


def _raise_on_status(status: torch.Tensor, first_frame: int) -> None:
    bad = torch.nonzero(status).flatten()
    if bad.numel():
        i = int(bad[0])
        raise ValueError(f"XTC frame {first_frame + i} could not be decoded (status {int(status[i])})")


def decode_bytes(data: np.ndarray, offsets: np.ndarray, n_atoms: int, device=None, first_frame: int = 0) -> XtcChunk:
    """Decodes the frames at `offsets` of a host XTC byte buffer on the device
    (raises ValueError naming the first frame that could not be decoded)."""
    device = device if device is not None else D.require_device()
    ch, status = _decode_launch(data, offsets, n_atoms, device, first_frame)
    _raise_on_status(status, first_frame)
    return ch


def _read_chunks(path, chunk_bytes: int):
    """Host side of the stream: yields (bytes, frame offsets, n_atoms, first
    frame) for the complete frames of about `chunk_bytes` of the file at a
    time.  The file is memory-mapped, not read: the bytes of a chunk are a
    view of the mapping, so the only copy is the one to the device, and the
    host touches just the frame headers while indexing."""
    size = os.path.getsize(path)
    if size == 0:
        return
    mm = np.memmap(path, dtype=np.uint8, mode="c")  # private mapping: writable views, file untouched
    pos, first = 0, 0
    while pos < size:
        end = min(size, pos + chunk_bytes)
        offsets, A, used = index_bytes(mm[pos:end])
        while len(offsets) == 0 and end < size:  # a frame larger than chunk_bytes
            end = min(size, pos + 2 * (end - pos))
            offsets, A, used = index_bytes(mm[pos:end])
        if len(offsets) == 0:
            raise ValueError("truncated XTC file: %d trailing bytes" % (size - pos))
        yield mm[pos:pos + used], offsets, A, first
        first += len(offsets)
        pos += used


def _read_ahead(gen, depth: int = 2):
    """Runs a chunk generator on a reader thread, `depth` chunks ahead of the
    consumer: the file read and the host index of chunk k+1 (both release
    the GIL) overlap the device work on chunk k.  Exceptions are re-raised
    in the consumer."""
    q: queue.Queue = queue.Queue(maxsize=depth)
    done = object()
    stop = threading.Event()

    def run():
        try:
            for item in gen:
                while not stop.is_set():
                    try:
                        q.put(item, timeout=0.1)
                        break
                    except queue.Full:
                        continue
                if stop.is_set():
                    return
            q.put(done)
        except BaseException as e:  # handed to the consumer
            q.put(e)

    t = threading.Thread(target=run, name="xtc-reader", daemon=True)
    t.start()
    try:
        while True:
            item = q.get()
            if item is done:
                return
            if isinstance(item, BaseException):
                raise item
            yield item
    finally:
        stop.set()
        t.join(timeout=5.0)


def iter_xtc(path, chunk_bytes: int = 256 << 20, device=None):
    """Yields XtcChunk objects covering the file in order, each holding the
    complete frames of about `chunk_bytes` of the file (double-buffered: the
    next chunk is read and indexed while this one is decoded)."""
    device = device if device is not None else D.require_device()
    for data, offsets, A, first in _read_ahead(_read_chunks(path, chunk_bytes)):
        yield decode_bytes(data, offsets, A, device, first)


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
    outs, checks = [], []
    # the reader thread reads and indexes chunk k+1 while chunk k's bytes go
    # up, decode and score; statuses and RMSDs come back once, at the end
    for data, offsets, A, first in _read_ahead(_read_chunks(path, chunk_bytes)):
        if dref is None:
            if ref_frame.shape[0] != A:
                raise ValueError("Input trajectories must have same number of atoms. found %d and %d."
                                 % (A, ref_frame.shape[0]))
            dref = D.DeviceReference(ref_frame, _lib.ATOM_MAJOR, centre=True, device=device)
        ch, status = _decode_launch(data, offsets, A, device, first)
        checks.append((status, first))
        outs.append(D.rmsd_to_reference(ch.xyz, ch.n_frames, ch.n_atoms, ch.n_padded, _lib.ATOM_MAJOR,
                                        _lib.MODE_CENTER, dref))
    for status, first in checks:
        _raise_on_status(status, first)
    return torch.cat(outs).cpu().numpy() if outs else np.zeros(0, np.float32)
