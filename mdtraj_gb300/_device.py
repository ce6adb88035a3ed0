"""Device plumbing for the drop-in: torch owns device memory and streams,
libgbrmsd does the work.  Nothing here computes RMSDs."""
from __future__ import annotations

import os
import time
import warnings

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr


def require_device() -> torch.device:
    """The CUDA device the drop-in runs on; raises if there is none (there is
    no CPU implementation of the hot path)."""
    if not torch.cuda.is_available():
        raise RuntimeError(
            "mdtraj_gb300 needs a CUDA device (GB300, sm_103); no CPU fallback is provided"
        )
    dev = torch.device("cuda", torch.cuda.current_device())
    if not lib.gbrmsd_device_supported():
        raise RuntimeError(
            f"device {torch.cuda.get_device_name(dev)} is not sm_103: libgbrmsd.so is built for GB300 only"
        )
    return dev


def stream_handle(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def padded(n_atoms: int) -> int:
    """Atoms per frame in device memory: n_atoms rounded up to a multiple of 4
    (the reference's padding convention for its aligned paths)."""
    return (int(n_atoms) + 3) // 4 * 4


def empty_bytes(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=device)


def copy_rows(dst: int, dst_pitch: int, src: int, src_pitch: int, row_bytes: int, n_rows: int,
              kind: int, stream: int) -> None:
    check(lib.gbrmsd_copy_rows(dst, dst_pitch, src, src_pitch, row_bytes, n_rows, kind, stream))


_PAGEABLE = None

# A host array that fits one chunk but holds at least this many bytes is
# streamed as two halves when its centring is written back: the second
# half's copy to the device then runs beside the first half's write-back
# (10,000 x 1,000 atoms, 120 MB: 1.69 -> 1.59 ms per md.rmsd call on GB300;
# three or four chunks were slower than one).
TWO_CHUNK_MIN_BYTES = 64 << 20


def pageable_access() -> bool:
    """Kernels can read/write pageable host memory (Grace + NVLink-C2C)."""
    global _PAGEABLE
    if _PAGEABLE is None:
        _PAGEABLE = bool(lib.gbrmsd_pageable_access())
    return _PAGEABLE


def _rows(layout: int, F: int, A: int):
    """(rows, host row floats, device row floats) of a frame block."""
    Ap = padded(A)
    if layout == _lib.ATOM_MAJOR:
        return F, 3 * A, 3 * Ap
    return 3 * F, A, Ap


def frames_to_device(x: np.ndarray, layout: int, device, stream: int) -> tuple[torch.Tensor, int]:
    """Copies host frames (F, A, 3) atom-major or (F, 3, A) axis-major into a
    padded, 16-byte aligned device buffer (padding atoms zeroed).  Returns
    (buffer, n_padded).  With pageable host access a kernel reads the numpy
    memory directly; otherwise a strided cudaMemcpy2DAsync is used."""
    src = x
    x = np.ascontiguousarray(x, dtype=np.float32)
    F = x.shape[0]
    A = x.shape[1] if layout == _lib.ATOM_MAJOR else x.shape[2]
    Ap = padded(A)
    shape = (F, Ap * 3) if layout == _lib.ATOM_MAJOR else (F, 3, Ap)
    buf = torch.empty(shape, dtype=torch.float32, device=device)
    if F and A:
        rows, hrow, drow = _rows(layout, F, A)
        if pageable_access():
            check(lib.gbrmsd_copy_rows_kernel(buf.data_ptr(), drow, x.ctypes.data, hrow, hrow, drow, rows, stream))
            # the kernel reads the host pages asynchronously: wait for it, so
            # that the array (the caller's, or a converted copy made here) may
            # be dropped as soon as this returns -- a kernel reading pages
            # that were unmapped in the meantime faults the GPU
            torch.cuda.ExternalStream(stream, device=device).synchronize()
        else:
            copy_rows(buf.data_ptr(), drow * 4, x.ctypes.data, hrow * 4, hrow * 4, rows, 1, stream)
    return buf, Ap


def frames_to_host(buf: torch.Tensor, out: np.ndarray, layout: int, n_atoms: int, n_padded: int,
                   stream: int) -> None:
    """Inverse of frames_to_device, writing into the existing host array."""
    F = out.shape[0]
    A = int(n_atoms)
    if not F or not A:
        return
    rows, hrow, drow = _rows(layout, F, A)
    if pageable_access():
        check(lib.gbrmsd_copy_rows_kernel(out.ctypes.data, hrow, buf.data_ptr(), drow, hrow, hrow, rows, stream))
    else:
        copy_rows(out.ctypes.data, hrow * 4, buf.data_ptr(), drow * 4, hrow * 4, rows, 2, stream)


def to_host(t: torch.Tensor, stream: int) -> np.ndarray:
    """Device tensor -> new host numpy array (synchronises the stream)."""
    out = np.empty(tuple(t.shape), dtype=np.float32)
    if out.size:
        copy_rows(out.ctypes.data, out.nbytes, t.data_ptr(), out.nbytes, out.nbytes, 1, 2, stream)
    torch.cuda.current_stream().synchronize()
    return out


class DeviceReference:
    """A reference frame prepared on the device (centred or not), laid out
    for the streaming kernels.  Reusable across calls."""

    def __init__(self, ref_xyz: np.ndarray | torch.Tensor, layout: int, centre: bool, device=None):
        device = device if device is not None else require_device()
        stream = stream_handle()
        if isinstance(ref_xyz, torch.Tensor):
            raw = ref_xyz.to(device=device, dtype=torch.float32).contiguous().reshape(-1, 3)
        else:
            host = np.ascontiguousarray(ref_xyz, dtype=np.float32).reshape(-1, 3)
            raw = torch.empty(host.shape, dtype=torch.float32, device=device)
            if host.size:
                copy_rows(raw.data_ptr(), host.nbytes, host.ctypes.data, host.nbytes, host.nbytes, 1, 1, stream)
        self.n_atoms = int(raw.shape[0])
        self.n_padded = padded(self.n_atoms)
        self.layout = int(layout)
        self.centred = bool(centre)
        nbytes = lib.gbrmsd_reference_workspace_bytes(self.n_atoms, self.n_padded)
        self.ws = empty_bytes(nbytes, device)
        self._raw = raw  # keep alive until the preparation kernel has run
        check(lib.gbrmsd_prepare_reference(raw.data_ptr() if raw.numel() else None, self.n_atoms,
                                           self.n_padded, self.layout, int(centre),
                                           self.ws.data_ptr(), self.ws.numel(), stream))

    def info(self) -> tuple[float, np.ndarray]:
        """(trace as float32, float32 centroid that was subtracted);
        synchronises the current stream."""
        stream = stream_handle()
        g = _lib.C.c_float(0.0)
        cen = np.zeros(3, dtype=np.float32)
        check(lib.gbrmsd_reference_info(self.ws.data_ptr(), _lib.C.addressof(g), cen.ctypes.data, stream))
        return float(np.float32(g.value)), cen


def error_word(ws: torch.Tensor) -> torch.Tensor:
    """The device error word of a workspace (first int32 of its header) as a
    one-element device tensor view."""
    return ws[:4].view(torch.int32)


def raise_on_error_word(word: int, what: str) -> None:
    """Host side of the device error word (gbrmsd_workspace_error_word): an
    expired bounded wait raises; non-finite coordinates warn (their RMSD is
    0, the value the reference's clamp of a NaN msd returns)."""
    if word & _lib.ERR_TIMEOUT:
        raise _lib.GbrmsdError(_lib.E_DEVICE, f"{what}: a bounded wait on the GPU expired; the results are not valid")
    if word & _lib.ERR_NONFINITE:
        warnings.warn(f"{what}: some frames have non-finite coordinates; their RMSD is reported as 0, as "
                      "mdtraj's clamp of a NaN msd gives", RuntimeWarning, stacklevel=3)


def rmsd_to_reference(x: torch.Tensor, n_frames: int, n_atoms: int, n_padded: int, layout: int,
                      mode: int, ref: DeviceReference, *, g_target: torch.Tensor | None = None,
                      g_ref: float = 0.0, self_index: int = -1, out: torch.Tensor | None = None,
                      centroid_out: torch.Tensor | None = None,
                      trace_out: torch.Tensor | None = None, ws: torch.Tensor | None = None) -> torch.Tensor:
    """Device-resident RMSD of every frame of `x` to `ref` (see
    gbrmsd_rmsd_to_reference) on torch's current stream, which also orders
    the workspace's reuse.  Returns the float32 rmsd tensor.  Pass `ws`
    (gbrmsd_rmsd_workspace_bytes) to read its error word afterwards."""
    stream = stream_handle()
    device = x.device
    if out is None:
        out = torch.empty(n_frames, dtype=torch.float32, device=device)
    nbytes = lib.gbrmsd_rmsd_workspace_bytes(n_frames, n_atoms)
    if ws is None or ws.numel() < nbytes:
        ws = empty_bytes(nbytes, device)
    frame_stride = 3 * n_padded
    check(lib.gbrmsd_rmsd_to_reference(
        ptr(x), n_frames, n_atoms, n_padded, frame_stride, layout, mode, ref.ws.data_ptr(),
        ptr(g_target), float(g_ref), int(self_index), ptr(out), ptr(centroid_out), ptr(trace_out),
        ws.data_ptr(), ws.numel(), stream))
    return out


def center_inplace(x: torch.Tensor, n_frames: int, n_atoms: int, n_padded: int, layout: int,
                   traces_out: torch.Tensor | None = None,
                   centroid_out: torch.Tensor | None = None) -> torch.Tensor:
    """Centres device frames in place on torch's current stream; returns the
    float32 traces."""
    stream = stream_handle()
    device = x.device
    if traces_out is None:
        traces_out = torch.empty(n_frames, dtype=torch.float32, device=device)
    nbytes = lib.gbrmsd_rmsd_workspace_bytes(n_frames, n_atoms)
    ws = empty_bytes(nbytes, device)
    check(lib.gbrmsd_center_inplace(ptr(x), n_frames, n_atoms, n_padded, 3 * n_padded, layout,
                                    ptr(traces_out), ptr(centroid_out), ws.data_ptr(), ws.numel(), stream))
    return traces_out


# ---------------------------------------------------------------------------
# Pipelined host-buffer path
# ---------------------------------------------------------------------------

_STREAMS: dict = {}


def _side_streams(device) -> tuple[torch.cuda.Stream, torch.cuda.Stream]:
    key = (device.type, device.index)
    if key not in _STREAMS:
        _STREAMS[key] = (torch.cuda.Stream(device=device), torch.cuda.Stream(device=device))
    return _STREAMS[key]


class HostLocks:
    """Page-locks a host array range by range (gbrmsd_host_register), ahead
    of the kernels that stream it, and releases every range at the end.

    With the pages locked the GPU reaches them through its own page tables
    instead of translating each access through the host's: on GB300 a 24 GB
    md.rmsd took 186-200 ms locked and 400-1,000 ms unlocked once other
    processes had streamed pageable memory.  Locking costs ~1.5-4.5 ms per
    GB of host time, which runs while the GPU moves earlier chunks.  Ranges
    are page-aligned and disjoint; if a range cannot be locked (the caller
    locked the array already, or the driver refuses) the rest of the array
    stays pageable, which the kernels read just the same."""

    PAGE = os.sysconf("SC_PAGESIZE") if hasattr(os, "sysconf") else 4096

    def __init__(self, base: int, nbytes: int):
        page = self.PAGE
        self.done = base // page * page
        self.hi = (base + nbytes + page - 1) // page * page
        self.ranges: list[int] = []
        self.ok = nbytes > 0
        self.locked_bytes = 0
        self.lock_s = 0.0    # host time spent locking
        self.unlock_s = 0.0  # host time spent unlocking

    def cover(self, end: int) -> None:
        """Locks through the page holding byte end - 1."""
        if not self.ok:
            return
        page = self.PAGE
        target = min(self.hi, (end + page - 1) // page * page)
        if target <= self.done:
            return
        t = time.perf_counter()
        rc = lib.gbrmsd_host_register(self.done, target - self.done)
        self.lock_s += time.perf_counter() - t
        if rc != 0:
            self.ok = False
            return
        self.ranges.append(self.done)
        self.locked_bytes += target - self.done
        self.done = target

    def release(self) -> None:
        """Unlocks every range; call once no queued work touches the array."""
        t = time.perf_counter()
        for p in self.ranges:
            lib.gbrmsd_host_unregister(p)
        self.ranges = []
        self.unlock_s += time.perf_counter() - t


# Where the last rmsd_host_frames call spent its host time (for benchmarks):
# chunks, bytes page-locked and whether every range could be locked, seconds
# locking and unlocking, and the host's final wait for the GPU (small when
# the host loop, not the GPU, set the pace).
LAST_HOST_STREAM: dict = {}


def rmsd_host_frames(x: np.ndarray, ref: "DeviceReference", mode: int, *, g_target: np.ndarray | None = None,
                     g_ref: float = 0.0, self_index: int = -1, write_centred: bool = False,
                     chunk_bytes: int = 256 << 20, ring: int = 2) -> np.ndarray:
    """RMSD of every frame of a HOST atom-major array (F, A, 3) float32 to a
    prepared reference, streamed through the GPU in chunks.

    Chunk k+1's host->device copy (stream 1) runs together with chunk k's
    in-place centring write-back (stream 2), so both directions of the host
    link are busy at once; the RMSD kernels of chunk k run between the two
    phases, alone on the GPU (the persistent streaming kernel needs a whole
    SM's registers, which the copy kernels would otherwise hold until they
    end).  A ring of `ring` (>= 2) device chunk buffers bounds device memory.
    Returns float32 (F,).
    """
    device = require_device()
    F, A = x.shape[0], x.shape[1]
    if F == 0 or A == 0:
        # no atoms: the reference returns 0 for every frame (0/0 clamped)
        return np.zeros(F, dtype=np.float32)
    Ap = padded(A)
    frame_bytes = 12 * max(A, 1)
    C = max(1, min(F, chunk_bytes // frame_bytes))
    if write_centred and C == F and F >= 2 and F * frame_bytes >= TWO_CHUNK_MIN_BYTES:
        C = (F + 1) // 2
    n_chunks = (F + C - 1) // C
    s_in, s_work = _side_streams(device)
    cur = torch.cuda.current_stream(device)
    out = torch.empty(F, dtype=torch.float32, device=device)
    cent = torch.empty((F, 3), dtype=torch.float32, device=device) if write_centred else None
    g_dev = torch.from_numpy(np.ascontiguousarray(g_target, dtype=np.float32)).to(device) \
        if g_target is not None else None
    bufs = [torch.empty((C, 3 * Ap), dtype=torch.float32, device=device) for _ in range(min(ring, n_chunks))]
    ws = empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(C, A), device)
    # each chunk's call clears the workspace's error word: keep a copy per chunk
    words = torch.zeros(n_chunks, dtype=torch.int32, device=device)
    host_ok = pageable_access()
    in_done = [torch.cuda.Event() for _ in range(n_chunks)]
    rmsd_done = [torch.cuda.Event() for _ in range(n_chunks)]
    s_in.wait_stream(cur)
    s_work.wait_stream(cur)
    assert len(bufs) >= 2 or n_chunks == 1
    # lock the array chunk by chunk: chunk k+1 while the GPU moves chunk k
    # (only chunk 0's lock is in the open; with fewer than 3 chunks nothing
    # is locked, since the locks could not hide behind earlier work)
    locks = HostLocks(x.ctypes.data, F * 12 * A) if host_ok and n_chunks >= 3 else None
    try:
        for k in range(n_chunks):
            f0 = k * C
            n = min(C, F - f0)
            buf = bufs[k % len(bufs)]
            src = x.ctypes.data + f0 * 12 * A
            if locks is not None:
                locks.cover(x.ctypes.data + (f0 + n) * 12 * A)
            with torch.cuda.stream(s_in):
                if k >= 1:
                    # after chunk k-1's RMSD kernels (which follow chunk k-2's
                    # write-back on stream 2, so buffer k % ring is free again)
                    s_in.wait_event(rmsd_done[k - 1])
                if host_ok:
                    check(lib.gbrmsd_copy_rows_kernel(buf.data_ptr(), 3 * Ap, src, 3 * A, 3 * A, 3 * Ap, n,
                                                      s_in.cuda_stream))
                else:
                    copy_rows(buf.data_ptr(), 12 * Ap, src, 12 * A, 12 * A, n, 1, s_in.cuda_stream)
                in_done[k].record(s_in)
            with torch.cuda.stream(s_work):
                s_work.wait_event(in_done[k])
                si = self_index - f0 if 0 <= self_index - f0 < n else -1
                check(lib.gbrmsd_rmsd_to_reference(
                    buf.data_ptr(), n, A, Ap, 3 * Ap, _lib.ATOM_MAJOR, mode, ref.ws.data_ptr(),
                    ptr(g_dev[f0:f0 + n]) if g_dev is not None else None, float(g_ref), si,
                    out[f0:f0 + n].data_ptr(), cent[f0:f0 + n].data_ptr() if cent is not None else None, None,
                    ws.data_ptr(), ws.numel(), s_work.cuda_stream))
                words[k:k + 1].copy_(error_word(ws))
                rmsd_done[k].record(s_work)
                if write_centred:
                    dst = x.ctypes.data + f0 * 12 * A
                    if host_ok:
                        check(lib.gbrmsd_write_centred(dst, buf.data_ptr(), 3 * Ap, cent[f0:f0 + n].data_ptr(), n, A,
                                                       s_work.cuda_stream))
            if locks is not None:
                locks.cover(x.ctypes.data + min(F, f0 + n + C) * 12 * A)
    except BaseException:
        # kernels already queued read and write the caller's host array:
        # let them finish before the error leaves (and the array can go away)
        s_in.synchronize()
        s_work.synchronize()
        if locks is not None:
            locks.release()
        raise
    t_wait = time.perf_counter()
    s_work.synchronize()
    t_wait = time.perf_counter() - t_wait
    result = np.empty(F, dtype=np.float32)
    copy_rows(result.ctypes.data, 4 * F, out.data_ptr(), 4 * F, 4 * F, 1, 2, s_work.cuda_stream)
    word = np.zeros(n_chunks, dtype=np.int32)
    copy_rows(word.ctypes.data, word.nbytes, words.data_ptr(), word.nbytes, word.nbytes, 1, 2, s_work.cuda_stream)
    s_work.synchronize()
    s_in.synchronize()
    if locks is not None:
        locks.release()
    LAST_HOST_STREAM.clear()
    LAST_HOST_STREAM.update(chunks=n_chunks, wait_s=t_wait,
                            locked_bytes=locks.locked_bytes if locks is not None else 0,
                            all_locked=bool(locks is not None and locks.ok),
                            lock_s=locks.lock_s if locks is not None else 0.0,
                            unlock_s=locks.unlock_s if locks is not None else 0.0)
    raise_on_error_word(int(np.bitwise_or.reduce(word)), "rmsd")
    if write_centred and not host_ok:
        cent_h = np.empty((F, 3), dtype=np.float32)
        copy_rows(cent_h.ctypes.data, cent_h.nbytes, cent.data_ptr(), cent_h.nbytes, cent_h.nbytes, 1, 2,
                  s_work.cuda_stream)
        s_work.synchronize()
        check(lib.gbrmsd_host_subtract_centroids(x.ctypes.data, F, A, 3 * A, cent_h.ctypes.data, 0))
    # keep the device buffers alive until both streams are done
    del bufs, ws, out, cent, g_dev, words
    return result
