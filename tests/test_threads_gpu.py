"""Calls from several host threads at once.

mdtraj's kernels run with the GIL released (nogil / prange in _rmsd.pyx), so
callers may drive the library from several threads.  The C ABI holds no
per-call state outside the caller's workspace and stream; the lazily filled
process-wide caches (device attributes, the tensor-map encoder, the static
scratch address) are filled race-free.  Four threads, each on its own stream
and workspace, run single-reference RMSDs (both layouts, several shapes) and
a tensor-core all-pairs matrix three times over; every result must equal,
bit for bit, the same call made alone on one thread.
"""
import threading

import numpy as np
import pytest
import torch

from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, synth
from mdtraj_gb300.allpairs import allpairs_device

pytestmark = pytest.mark.gpu

CASES = [(2000, 301, _lib.ATOM_MAJOR), (1500, 1024, _lib.AXIS_MAJOR), (800, 4000, _lib.ATOM_MAJOR),
         (3000, 97, _lib.AXIS_MAJOR)]


def _setup(i, cuda, stream):
    F, A, layout = CASES[i]
    ref, x = synth.single_reference_frames(F, A, seed=40 + i, sigma=np.geomspace(1e-3, 0.4, F), exact_fraction=0.02)
    host = x if layout == _lib.ATOM_MAJOR else np.ascontiguousarray(x.transpose(0, 2, 1))
    xd, Ap = D.frames_to_device(host, layout, cuda, stream)
    r = D.DeviceReference(ref, layout, centre=True, device=cuda)
    _, xa = synth.single_reference_frames(300, 257, seed=60 + i, sigma=0.2)
    xad, Apa = D.frames_to_device(xa, _lib.ATOM_MAJOR, cuda, stream)
    # the host arrays stay referenced until the copies have run
    return dict(F=F, A=A, layout=layout, x=xd, Ap=Ap, ref=r, xa=xad, Apa=Apa, host=(host, xa))


def _run(c, cuda):
    """One single-reference call and one all-pairs call on the current stream."""
    lib = _lib.lib
    stream = D.stream_handle()
    F, A, Ap = c["F"], c["A"], c["Ap"]
    out = torch.empty(F, dtype=torch.float32, device=cuda)
    ws = D.empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(F, A), cuda)
    _lib.check(lib.gbrmsd_rmsd_to_reference(c["x"].data_ptr(), F, A, Ap, 3 * Ap, c["layout"], _lib.MODE_CENTER,
                                            c["ref"].ws.data_ptr(), None, 0.0, -1, out.data_ptr(), None, None,
                                            ws.data_ptr(), ws.numel(), stream))
    rm = D.to_host(out, stream)
    ap = allpairs_device(c["xa"], 300, 257, c["Apa"], _lib.ATOM_MAJOR, method="tensor")
    return rm, D.to_host(ap, stream)


def test_concurrent_threads_match_single_thread_results(cuda):
    stream = D.stream_handle()
    cases = [_setup(i, cuda, stream) for i in range(len(CASES))]
    torch.cuda.synchronize()
    want = [_run(c, cuda) for c in cases]

    streams = [torch.cuda.Stream(device=cuda) for _ in cases]
    got = [[] for _ in cases]
    errors = []
    start = threading.Barrier(len(cases))

    def work(i):
        try:
            torch.cuda.set_device(cuda)
            with torch.cuda.stream(streams[i]):
                start.wait()
                for _ in range(3):
                    got[i].append(_run(cases[i], cuda))
        except BaseException as e:  # re-raised on the main thread
            errors.append((i, e))

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    assert not any(t.is_alive() for t in threads), "a worker thread did not finish"
    assert not errors, errors
    for i, (rm, ap) in enumerate(want):
        assert len(got[i]) == 3
        for rm_i, ap_i in got[i]:
            np.testing.assert_array_equal(rm_i, rm, err_msg=f"case {CASES[i]}")
            np.testing.assert_array_equal(ap_i, ap, err_msg=f"all-pairs, thread {i}")
