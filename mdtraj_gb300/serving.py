"""Serving loop: a database of frames resident in HBM answering RMSD query
sets with continuous batching.

A request is a set of query frames scored against a contiguous range of the
database (``[md.rmsd(db[a:b], queries, k) for k]``, see cross.py).  The
server keeps the prepared database on the device and runs a host loop that

  * moves requests whose arrival time has passed into a FIFO queue;
  * admits queued requests while the query pool (prepared query frames on the
    device) has room for their frames and the HBM budget has room for their
    results;
  * whenever one of its stream slots is free, launches every admitted request
    as ONE batch on that slot: query upload, preparation into the pool, one
    cross-RMSD launch whose tiles mix the requests, and the copy of each
    result to pinned host memory;
  * completes batches whose events have fired, releasing pool rows and budget.

So requests that arrive while others are on the GPU join the next batch as
soon as a slot and memory free up, batches on different slots overlap on the
device (one batch's kernel with another's copies), and batches grow with the
load.  A request's results depend only on its own frames: the same alone and
in any mix.  ``slots=1, max_batch_requests=1`` gives one request per launch.
"""
from __future__ import annotations

import ctypes
import math
import time
import weakref
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _device as D
from . import _lib
from ._lib import lib
from .cross import CrossWorkspace, FrameSet, cross_launch, request_table

# bumped by Request.cancel(): the loop looks for withdrawn requests only when
# it has changed since its last look
_CANCELS = [0]


@dataclass
class Request:
    """Query frames (Q, A, 3) float32 against database frames [db0, db1)."""

    queries: np.ndarray
    db0: int
    db1: int
    arrival: float = 0.0  # seconds after the start of serve()
    rid: int = -1
    result: np.ndarray | None = None  # (Q, db1 - db0) float32 once done
    timeout: float | None = None  # seconds after arrival; None: no limit
    status: str = "pending"  # "done", "cancelled" or "timed_out" once finished
    t_admit: float = math.nan
    t_launch: float = math.nan
    t_done: float = math.nan
    batch: int = -1
    refined: int = 0
    _cancel: bool = field(default=False, repr=False)
    _p0: int = field(default=-1, repr=False)
    _out: torch.Tensor | None = field(default=None, repr=False)
    _host: torch.Tensor | None = field(default=None, repr=False)
    _hoff: int = field(default=-1, repr=False)  # result's page offset in the host result pool

    @property
    def n_query(self) -> int:
        return int(self.queries.shape[0])

    @property
    def result_bytes(self) -> int:
        return 4 * self.n_query * (self.db1 - self.db0)

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival

    def cancel(self) -> None:
        """Withdraws the request (from any thread).  While it is queued or
        admitted it is dropped before launch; once its batch is on the GPU
        the batch runs to the end and its result is discarded.  Either way
        it finishes with status "cancelled" and no result."""
        self._cancel = True
        _CANCELS[0] += 1

    def expired(self, now: float) -> bool:
        return self.timeout is not None and now > self.arrival + self.timeout


class PoolAllocator:
    """First-fit allocator of contiguous query-pool rows."""

    def __init__(self, capacity: int):
        self.capacity = int(capacity)
        self.free = [(0, self.capacity)]  # sorted, disjoint (start, length)

    def alloc(self, n: int):
        for k, (s, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    del self.free[k]
                else:
                    self.free[k] = (s + n, ln - n)
                return s
        return None

    def release(self, start: int, n: int) -> None:
        self.free.append((start, n))
        self.free.sort()
        merged = []
        for s, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == s:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((s, ln))
        self.free = merged

    @property
    def free_rows(self) -> int:
        return sum(ln for _, ln in self.free)


class HostResultPool:
    """Page-locked host memory for request results, handed out in 4 KB pages
    (first fit) and returned when a result array is dropped.

    Results copied into page-locked memory move by DMA without blocking the
    host; allocating page-locked memory per request costs far more than the
    copy (measured on the serving workload: 1,500 requests with ~73 MB
    results each took 2.9 s of host time in per-request allocations, against
    0.08 s for everything else).  One numpy buffer is locked once
    (gbrmsd_host_register) and results are views into it."""

    PAGE = 4096

    def __init__(self, nbytes: int):
        pages = max(1, int(nbytes) // self.PAGE)
        self.buf = np.empty(pages * self.PAGE, dtype=np.uint8)
        self.locked = lib.gbrmsd_host_register(self.buf.ctypes.data, self.buf.nbytes) == 0
        self.pages = PoolAllocator(pages)

    def take(self, nbytes: int):
        """Page offset of a free range of nbytes, or None (always None when
        the buffer could not be page-locked: copies into pageable memory
        would block the host, so such results get their own locked buffer)."""
        if not self.locked:
            return None
        return self.pages.alloc((int(nbytes) + self.PAGE - 1) // self.PAGE)

    def release(self, off: int, nbytes: int) -> None:
        self.pages.release(off, (int(nbytes) + self.PAGE - 1) // self.PAGE)

    def ptr(self, off: int) -> int:
        return self.buf.ctypes.data + off * self.PAGE

    def result(self, off: int, n_floats: int, nbytes: int) -> np.ndarray:
        """float32 array over the pages at `off`; the pages return to the pool
        once no array or view of it is left (the array's base is a ctypes
        object that every view keeps alive)."""
        holder = (ctypes.c_float * max(1, n_floats)).from_address(self.ptr(off))
        weakref.finalize(holder, self.release, off, nbytes)
        return np.frombuffer(holder, dtype=np.float32, count=n_floats)

    def close(self) -> None:
        if self.locked:
            lib.gbrmsd_host_unregister(self.buf.ctypes.data)
            self.locked = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class QueryStaging:
    """Page-locked host rows mirroring the device query pool: a request's
    query frames are copied (host memcpy) into the rows of its pool slot and
    go up with an asynchronous copy.  torch's copy from the caller's pageable
    array waits on the host until the copy engine has taken it, which behind
    a batch's result copies to the host took ~0.8 ms per request (a third of
    the loop's time in a 300-request burst)."""

    def __init__(self, rows: int, row_floats: int):
        self.arr = np.empty((int(rows), int(row_floats)), dtype=np.float32)
        self.locked = lib.gbrmsd_host_register(self.arr.ctypes.data, self.arr.nbytes) == 0

    def ptr(self, row: int) -> int:
        return self.arr.ctypes.data + int(row) * self.arr.strides[0]

    def close(self) -> None:
        if self.locked:
            lib.gbrmsd_host_unregister(self.arr.ctypes.data)
            self.locked = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Slot:
    timeline = None

    def __init__(self, device):
        self.stream = torch.cuda.Stream(device=device)
        self.ws = CrossWorkspace(device)
        self.event = None
        self.batch = None
        self.ws_buf = None
        # the batch's error word and refined-pair count, copied to the host
        # right after its kernels (read once its event has fired)
        self.hdr = torch.zeros(4, dtype=torch.int32, pin_memory=True)  # error word, list count, refined (int64)


class RmsdServer:
    """Resident database + continuous-batching request loop.

    database: FrameSet, or frames (host array / device tensor (F, A, 3)).
    method: "tensor" (split-BF16 tcgen05 tiles) or "fp32" (CUDA-core tiles).
    query_capacity: frames in the device query pool.
    hbm_budget_bytes: device bytes for results of admitted requests.
    slots: batches that may be in flight at once (one stream each).
    max_batch_requests: cap on requests per batch (None: no cap).
    result_to_host: copy each result to page-locked host memory (else results
    stay on the device as tensors).
    host_pool_bytes: page-locked host memory for results in flight or held by
    the caller (HostResultPool); a request whose result does not fit waits
    for space, or, when nothing is in flight, gets its own page-locked buffer.
    """

    def __init__(self, database, *, method: str = "tensor", query_capacity: int = 8192,
                 hbm_budget_bytes: int = 8 << 30, slots: int = 3, max_batch_requests: int | None = None,
                 result_to_host: bool = True, host_pool_bytes: int = 1 << 30, device=None):
        self.device = device if device is not None else D.require_device()
        self.db = database if isinstance(database, FrameSet) else FrameSet.from_frames(database, device=self.device)
        self.n_db = self.db.capacity
        self.n_atoms = self.db.n_atoms
        self.method = method
        self.qcap = int(query_capacity)
        self.qset = FrameSet(self.qcap, self.n_atoms, self.device)
        self.staging = torch.empty((self.qcap, 3 * self.n_atoms), dtype=torch.float32, device=self.device)
        self.qhost = QueryStaging(self.qcap, 3 * self.n_atoms)
        self.pool = PoolAllocator(self.qcap)
        self.budget = int(hbm_budget_bytes)
        self.used = 0
        self.slots = [_Slot(self.device) for _ in range(max(1, int(slots)))]
        self.max_batch = max_batch_requests
        self.result_to_host = result_to_host
        self.hpool = HostResultPool(host_pool_bytes) if result_to_host else None
        self.n_batches = 0
        self.batch_sizes = []
        self.batch_log = []  # per completed batch: requests, result bytes, host launch time, GPU kernels / copies

    # -- request checks ---------------------------------------------------
    def validate(self, r: Request) -> None:
        q = r.queries
        if q.ndim != 3 or q.shape[1] != self.n_atoms or q.shape[2] != 3 or q.dtype != np.float32:
            raise ValueError(f"request {r.rid}: queries must be float32 (Q, {self.n_atoms}, 3)")
        if not (1 <= q.shape[0] <= self.qcap):
            raise ValueError(f"request {r.rid}: 1 <= n_query <= query capacity ({self.qcap})")
        if not (0 <= r.db0 < r.db1 <= self.n_db):
            raise ValueError(f"request {r.rid}: database range must satisfy 0 <= db0 < db1 <= {self.n_db}")
        if r.result_bytes > self.budget:
            raise ValueError(f"request {r.rid}: result ({r.result_bytes} bytes) exceeds the HBM budget")

    # -- steps of the loop ----------------------------------------------------
    def _admit(self, r: Request, now: float, idle: bool = False) -> bool:
        if self.used + r.result_bytes > self.budget:
            return False
        hoff = -1
        if self.hpool is not None:
            hoff = self.hpool.take(r.result_bytes)
            if hoff is None:
                if self.hpool.locked and not idle:
                    return False  # wait for results in flight to free host space
                hoff = -1         # nothing in flight (or no pool): its own locked buffer
        p0 = self.pool.alloc(r.n_query)
        if p0 is None:
            if hoff >= 0:
                self.hpool.release(hoff, r.result_bytes)
            return False
        r._hoff = hoff
        r._p0 = p0
        r._out = torch.empty(r.n_query * (r.db1 - r.db0), dtype=torch.float32, device=self.device)
        self.used += r.result_bytes
        r.t_admit = now
        return True

    @staticmethod
    def _group_by_range(batch: list) -> None:
        """Lays the batch's queries out in the pool sorted by database range.

        A tile covers 80 query rows of the pool and, for those rows, every
        database row block that any of their requests needs; rows of a
        request whose range misses a block are computed and dropped.  When
        requests with similar ranges sit next to each other the blocks' unions
        shrink: on the serving mix (half full-database, half random slices)
        the share of computed pairs that are kept rises from ~0.83 to ~0.92.
        Only done when the batch owns one contiguous run of pool rows (the
        usual case); each request keeps its own contiguous rows."""
        spans = sorted((r._p0, r.n_query) for r in batch)
        for (a, n), (b, _) in zip(spans, spans[1:]):
            if a + n != b:
                return
        p = spans[0][0]
        for r in sorted(batch, key=lambda r: (r.db0, r.db1)):
            r._p0 = p
            p += r.n_query

    def _launch(self, slot: _Slot, batch: list, now: float) -> None:
        t_host = time.perf_counter()
        self._group_by_range(batch)
        s = slot.stream
        # per-batch timeline on the slot's stream: start, kernels done, copies done
        t_ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        with torch.cuda.stream(s):
            t_ev[0].record(s)
            for r in batch:
                rows = self.staging[r._p0:r._p0 + r.n_query]
                q = r.queries.reshape(r.n_query, -1)
                if self.qhost.locked:
                    # rows of a pool slot are not reused before the batch
                    # holding them completes, so the host rows are free too
                    self.qhost.arr[r._p0:r._p0 + r.n_query] = q
                    nb = q.nbytes
                    D.copy_rows(rows.data_ptr(), nb, self.qhost.ptr(r._p0), nb, nb, 1, 1, s.cuda_stream)
                else:
                    rows.copy_(torch.from_numpy(q), non_blocking=True)
                self.qset.prepare(rows, r._p0, stream=s.cuda_stream)
            table = request_table([(r._out.data_ptr(), r._p0, r.n_query, r.db0, r.db1) for r in batch])
            ws = slot.ws.get(self.n_db, self.qcap, len(batch))
            cross_launch(self.db, self.n_db, self.qset, table, len(batch), self.method, ws, s.cuda_stream)
            slot.hdr.copy_(ws[:16].view(torch.int32), non_blocking=True)
            t_ev[1].record(s)
            if self.result_to_host:
                for r in batch:
                    nb = 4 * r._out.numel()
                    if r._hoff >= 0:
                        D.copy_rows(self.hpool.ptr(r._hoff), nb, r._out.data_ptr(), nb, nb, 1, 2, s.cuda_stream)
                    else:
                        r._host = torch.empty(r._out.numel(), dtype=torch.float32, pin_memory=True)
                        r._host.copy_(r._out, non_blocking=True)
            t_ev[2].record(s)
        for r in batch:
            r.t_launch = now
            r.batch = self.n_batches
        self.n_batches += 1
        self.batch_sizes.append(len(batch))
        slot.event, slot.batch, slot.ws_buf = t_ev[2], batch, ws
        slot.timeline = (t_ev, time.perf_counter() - t_host, sum(r.result_bytes for r in batch))

    def _unadmit(self, r: Request) -> None:
        """Returns an admitted, not launched request's pool rows, budget and
        host result pages."""
        if r._hoff >= 0:
            self.hpool.release(r._hoff, r.result_bytes)
            r._hoff = -1
        self.pool.release(r._p0, r.n_query)
        self.used -= r.result_bytes
        r._out = None

    @staticmethod
    def _drop(r: Request, status: str, now: float) -> Request:
        r.status = status
        r.result = None
        r.t_done = now
        return r

    def _complete(self, slot: _Slot, now: float, keep_results: bool) -> list:
        err = int(slot.hdr[0])  # copied before the batch's event
        refined = int(slot.hdr[2:].view(torch.int64)[0])
        if err:
            raise _lib.GbrmsdError(_lib.E_DEVICE, "cross RMSD batch: device error word 0x%x (1 = wait expired)" % err)
        done = slot.batch
        t_ev, host_s, nbytes = slot.timeline
        self.batch_log.append({"requests": len(done), "result_bytes": nbytes, "launch_host_ms": host_s * 1e3,
                               "kernels_ms": t_ev[0].elapsed_time(t_ev[1]),
                               "copies_ms": t_ev[1].elapsed_time(t_ev[2])})
        for r in done:
            shape = (r.n_query, r.db1 - r.db0)
            # a request withdrawn or out of time while its batch ran: the
            # batch has finished, so its memory is released and the result
            # discarded
            late = "cancelled" if r._cancel else ("timed_out" if r.expired(now) else None)
            if late is not None:
                if r._hoff >= 0:
                    self.hpool.release(r._hoff, r.result_bytes)
                    r._hoff = -1
                self.pool.release(r._p0, r.n_query)
                self.used -= r.result_bytes
                r._out = None
                r._host = None
                r.refined = refined
                self._drop(r, late, now)
                continue
            r.status = "done"
            if self.result_to_host and r._hoff >= 0:
                if keep_results:
                    # an array over pool pages; they return when it is dropped
                    r.result = self.hpool.result(r._hoff, r.n_query * (r.db1 - r.db0), r.result_bytes).reshape(shape)
                else:
                    self.hpool.release(r._hoff, r.result_bytes)
                r._hoff = -1
            elif keep_results:
                r.result = (r._host.numpy() if self.result_to_host else r._out).reshape(shape)
            r.refined = refined
            r.t_done = now
            self.pool.release(r._p0, r.n_query)
            self.used -= r.result_bytes
            r._out = None if self.result_to_host or not keep_results else r._out
            if not keep_results:
                r._host = None
        slot.event, slot.batch, slot.ws_buf = None, None, None
        return done

    # -- the loop ------------------------------------------------------------
    def serve(self, requests, *, realtime: bool = True, keep_results: bool = True, poll_s: float = 50e-6) -> list:
        """Runs the loop over `requests` (arrival times in seconds from the
        start; realtime=False queues everything at once and resets the
        arrival times to 0).  Returns the requests with results and timings,
        in completion order."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            self.validate(r)
            if not realtime:
                r.arrival = 0.0
        n = len(reqs)
        queue, admitted, finished = deque(), [], []
        batch_bytes = 0
        batch_cap = (self.hpool.buf.nbytes // len(self.slots)) if self.hpool is not None and self.hpool.locked else 0
        nxt = 0
        has_timeouts = any(r.timeout is not None for r in reqs)
        cancels_seen, last_scan = -1, -1.0
        t0 = time.perf_counter()
        while len(finished) < n:
            now = time.perf_counter() - t0
            while nxt < n and (not realtime or reqs[nxt].arrival <= now):
                queue.append(reqs[nxt])
                nxt += 1
            for slot in self.slots:
                if slot.event is not None and slot.event.query():
                    finished.extend(self._complete(slot, time.perf_counter() - t0, keep_results))
            # requests withdrawn or out of time before their launch leave now
            # (looked for when a cancel happened, and every ms with timeouts)
            scan = _CANCELS[0] != cancels_seen or (has_timeouts and now - last_scan > 1e-3)
            if scan:
                cancels_seen, last_scan = _CANCELS[0], now
            if scan and any(r._cancel or r.expired(now) for r in queue):
                keep = deque()
                for r in queue:
                    if r._cancel or r.expired(now):
                        finished.append(self._drop(r, "cancelled" if r._cancel else "timed_out", now))
                    else:
                        keep.append(r)
                queue = keep
            if scan and any(r._cancel or r.expired(now) for r in admitted):
                keep = []
                for r in admitted:
                    if r._cancel or r.expired(now):
                        self._unadmit(r)
                        batch_bytes -= r.result_bytes
                        finished.append(self._drop(r, "cancelled" if r._cancel else "timed_out", now))
                    else:
                        keep.append(r)
                admitted = keep
            idle = not admitted and all(s.event is None for s in self.slots)
            while queue and (self.max_batch is None or len(admitted) < self.max_batch):
                # a batch holds at most 1/slots of the host result pool, so
                # the next batch's kernels can run while this one's results
                # copy out (one batch taking the whole pool serialised them)
                if admitted and batch_cap and batch_bytes + queue[0].result_bytes > batch_cap:
                    break
                if not self._admit(queue[0], now, idle=idle and not admitted):
                    break
                batch_bytes += queue[0].result_bytes
                admitted.append(queue.popleft())
            free = [s for s in self.slots if s.event is None]
            if admitted and free:
                self._launch(free[0], admitted, now)
                admitted = []
                batch_bytes = 0
                continue
            busy = any(s.event is not None for s in self.slots)
            if not busy and not admitted and not queue and nxt < n:
                wait = reqs[nxt].arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(min(wait, 0.01) if wait > 2e-3 else 0)
            elif busy:
                time.sleep(poll_s if poll_s > 0 else 0)
        return finished


def latency_summary(done: list, t_first: float | None = None) -> dict:
    """p50 / p99 / mean latency (ms) and completed queries per second, over
    the requests that finished with a result (status "done")."""
    done = [r for r in done if r.status == "done"]
    lat = np.array([r.latency for r in done]) * 1e3
    t0 = min(r.arrival for r in done) if t_first is None else t_first
    t1 = max(r.t_done for r in done)
    return {"requests": len(done), "p50_ms": round(float(np.percentile(lat, 50)), 3),
            "p99_ms": round(float(np.percentile(lat, 99)), 3), "mean_ms": round(float(lat.mean()), 3),
            "queries_per_s": round(len(done) / max(t1 - t0, 1e-9), 1),
            "query_frames_per_s": round(sum(r.n_query for r in done) / max(t1 - t0, 1e-9), 1),
            "pairs_per_s": round(sum(r.n_query * (r.db1 - r.db0) for r in done) / max(t1 - t0, 1e-9), 1)}


def batch_summary(log: list) -> dict:
    """Where a serving run's batches spent their time: mean requests per
    batch, host time to launch one, GPU time of its kernels (query upload,
    preparation, cross RMSD) and of its result copies to host memory, and the
    copies' rate."""
    if not log:
        return {"batches": 0}
    k = np.array([b["kernels_ms"] for b in log])
    c = np.array([b["copies_ms"] for b in log])
    nb = float(sum(b["result_bytes"] for b in log))
    return {"batches": len(log), "mean_requests": round(float(np.mean([b["requests"] for b in log])), 2),
            "launch_host_ms": round(float(np.mean([b["launch_host_ms"] for b in log])), 3),
            "kernels_ms": round(float(k.mean()), 3), "copies_ms": round(float(c.mean()), 3),
            "copies_gbs": round(nb / max(c.sum() / 1e3, 1e-9) / 1e9, 1),
            "gpu_ms_total": round(float(k.sum() + c.sum()), 1)}
