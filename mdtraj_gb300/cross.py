"""Cross RMSD: query frames against a set of database frames.

The work of ``[md.rmsd(db[a:b], queries, k) for k in range(len(queries))]``
(mdtraj/rmsd/_rmsd.pyx:64-243 once per query frame) as one call: every
query frame against every database frame of the range, optimal
superposition, float32 results shaped (n_query, b - a).  The reference has
no multi-reference call; this is the kernel behind the serving loop
(serving.py).

Frames are prepared once into a ``FrameSet`` on the device (centred float
rows, split BF16 planes and FP64 traces), so a database is prepared once and
scored against many query sets.  ``method="tensor"`` uses split-BF16
tcgen05 tiles, ``method="fp32"`` plain FP32 CUDA-core tiles; both recompute
near-identical pairs exactly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _device as D
from . import _lib
from ._lib import check, lib

METHODS = {"fp32": 0, "tensor": 1}


class FrameSet:
    """Device buffer of prepared frames with room for ``capacity`` frames of
    ``n_atoms`` atoms.  Rows are filled with ``prepare``."""

    def __init__(self, capacity: int, n_atoms: int, device=None):
        if capacity < 1 or n_atoms < 1:
            raise ValueError("FrameSet needs capacity >= 1 and n_atoms >= 1")
        self.device = device if device is not None else D.require_device()
        self.capacity = int(capacity)
        self.n_atoms = int(n_atoms)
        self.buf = D.empty_bytes(lib.gbrmsd_frameset_bytes(self.capacity, self.n_atoms), self.device)

    def prepare(self, x: torch.Tensor, first: int = 0, *, n_padded: int | None = None, centre: bool = True,
                stream: int | None = None) -> None:
        """Prepares device frames ``x`` (atom-major float32, (F, n_padded * 3)
        or (F, n_atoms, 3), contiguous) into rows [first, first + F)."""
        if x.dtype != torch.float32 or not x.is_cuda or not x.is_contiguous():
            raise ValueError("prepare expects a contiguous float32 CUDA tensor")
        F = int(x.shape[0])
        Ap = int(n_padded) if n_padded is not None else self.n_atoms
        if F and x.numel() // F != 3 * Ap:
            raise ValueError("frame size does not match n_padded * 3")
        check(lib.gbrmsd_frameset_prepare(x.data_ptr(), F, self.n_atoms, Ap, 3 * Ap, _lib.ATOM_MAJOR, int(centre),
                                          self.buf.data_ptr(), self.capacity, int(first),
                                          D.stream_handle() if stream is None else stream))

    @classmethod
    def from_frames(cls, xyz, *, centre: bool = True, chunk: int = 65536, device=None) -> "FrameSet":
        """A set holding all frames of ``xyz`` (host (F, A, 3) array or device
        tensor), prepared ``chunk`` frames at a time."""
        dev = device if device is not None else D.require_device()
        if isinstance(xyz, torch.Tensor) and xyz.is_cuda:
            F, A = int(xyz.shape[0]), int(xyz.shape[1])
            fs = cls(F, A, dev)
            x = xyz.reshape(F, 3 * A)
            for s in range(0, F, chunk):
                fs.prepare(x[s:s + chunk].contiguous(), s, centre=centre)
            return fs
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        if xyz.ndim != 3 or xyz.shape[2] != 3:
            raise ValueError("expected coordinates of shape (n_frames, n_atoms, 3)")
        F, A = xyz.shape[0], xyz.shape[1]
        fs = cls(F, A, dev)
        for s in range(0, F, chunk):
            part = torch.from_numpy(xyz[s:s + chunk].reshape(-1, 3 * A)).to(dev)
            fs.prepare(part, s, centre=centre)
        return fs


class CrossWorkspace:
    """Workspace of gbrmsd_cross_rmsd for a database size, query capacity and
    request count (grown on demand)."""

    def __init__(self, device):
        self.device = device
        self.buf = None

    def get(self, n_db: int, query_capacity: int, n_requests: int) -> torch.Tensor:
        need = lib.gbrmsd_cross_workspace_bytes(n_db, query_capacity, n_requests)
        if self.buf is None or self.buf.numel() < need:
            self.buf = D.empty_bytes(need, self.device)
        return self.buf


def request_table(requests) -> C.Array:
    """ctypes array of gbrmsd_cross_request_t from (out_ptr, pool0, n_query,
    db0, db1) tuples."""
    arr = (_lib.CrossRequest * max(1, len(requests)))()
    for k, (out, pool0, nq, db0, db1) in enumerate(requests):
        arr[k].out = out
        arr[k].pool0 = pool0
        arr[k].n_query = nq
        arr[k].db0 = db0
        arr[k].db1 = db1
    return arr


def cross_launch(db: FrameSet, n_db: int, queries: FrameSet, table: C.Array, n_requests: int, method: str,
                 ws: torch.Tensor, stream: int) -> None:
    if method not in METHODS:
        raise ValueError(f"method must be one of {sorted(METHODS)}")
    if db.n_atoms != queries.n_atoms:
        raise ValueError("database and query frames have different atom counts")
    check(lib.gbrmsd_cross_rmsd(db.buf.data_ptr(), db.capacity, n_db, queries.buf.data_ptr(), queries.capacity,
                                db.n_atoms, C.addressof(table), n_requests, METHODS[method], ws.data_ptr(),
                                ws.numel(), stream))


def cross_status(ws: torch.Tensor, stream: int | None = None) -> int:
    """Synchronises and returns the number of exactly refined pairs; raises
    if the device recorded an error."""
    n = C.c_int32(0)
    check(lib.gbrmsd_allpairs_status(ws.data_ptr(), C.byref(n), D.stream_handle() if stream is None else stream))
    return int(n.value)


def cross_rmsd(database, queries, *, db_range=None, method: str = "tensor") -> np.ndarray:
    """RMSD of every query frame against every database frame of
    ``db_range`` (default: all), optimal superposition (both centred first).
    ``database``: FrameSet or frames (object with ``.xyz``, host array or
    device tensor (F, A, 3)); ``queries``: frames.  Returns float32
    (n_query, n_db_range); row k equals ``md.rmsd(db[a:b], queries, k)``."""
    dev = D.require_device()
    db = database if isinstance(database, FrameSet) else FrameSet.from_frames(
        database.xyz if hasattr(database, "xyz") else database, device=dev)
    qx = queries.xyz if hasattr(queries, "xyz") else queries
    qs = FrameSet.from_frames(qx, device=dev)
    if qs.n_atoms != db.n_atoms:
        raise ValueError("database and query frames have different atom counts")
    a, b = (0, db.capacity) if db_range is None else (int(db_range[0]), int(db_range[1]))
    if not (0 <= a <= b <= db.capacity):
        raise ValueError("db_range outside the database")
    Q = qs.capacity
    out = torch.empty((Q, b - a), dtype=torch.float32, device=dev)
    if Q == 0 or b == a:
        return out.cpu().numpy()
    table = request_table([(out.data_ptr(), 0, Q, a, b)])
    ws = CrossWorkspace(dev).get(db.capacity, Q, 1)
    stream = D.stream_handle()
    cross_launch(db, db.capacity, qs, table, 1, method, ws, stream)
    cross_status(ws, stream)
    return out.cpu().numpy()
