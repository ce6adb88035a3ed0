"""The allocation-free entry point gbrmsd_rmsd_to_reference_noalloc.

Some callers cannot allocate device memory when they need RMSDs: code
inside another runtime's memory pool (the pool owns the device memory), a
plugin whose host application hands it buffers but no allocator, or a loop
that must not call cudaMalloc/cudaFree (they can synchronise the device).
For them the library keeps a fixed 16 MiB
scratch array on the device and this entry point takes no workspace.  The
test calls it through the C ABI, twice in a row (different shapes, then the
same shape again, so state left by one call cannot leak into the next), and
checks it against gbrmsd_rmsd_to_reference with a caller workspace: both
run the same kernels with the same split of the frames on the same inputs,
so the RMSDs and centroids must agree bit for bit.  Such callers read the
device error word through gbrmsd_noalloc_status (the scratch is not theirs to
read), which is checked after every call, and once after a bounded wait was
made to run out.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def _case(F, A, seed, cuda, stream):
    ref, x = synth.single_reference_frames(F, A, seed=seed, sigma=np.geomspace(1e-3, 0.5, F), exact_fraction=0.02)
    xd, Ap = D.frames_to_device(x, _lib.ATOM_MAJOR, cuda, stream)
    r = D.DeviceReference(ref, _lib.ATOM_MAJOR, centre=True)
    return xd, Ap, r


def _with_workspace(xd, F, A, Ap, r, cuda, stream):
    lib = _lib.lib
    out = torch.empty(F, dtype=torch.float32, device=cuda)
    cent = torch.empty((F, 3), dtype=torch.float32, device=cuda)
    ws = D.empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(F, A), cuda)
    _lib.check(lib.gbrmsd_rmsd_to_reference(xd.data_ptr(), F, A, Ap, 3 * Ap, _lib.ATOM_MAJOR, _lib.MODE_CENTER,
                                            r.ws.data_ptr(), None, 0.0, -1, out.data_ptr(), cent.data_ptr(), None,
                                            ws.data_ptr(), ws.numel(), stream))
    return D.to_host(out, stream), D.to_host(cent, stream)


def _no_alloc(xd, F, A, Ap, r, cuda, stream):
    lib = _lib.lib
    out = torch.empty(F, dtype=torch.float32, device=cuda)
    cent = torch.empty((F, 3), dtype=torch.float32, device=cuda)
    _lib.check(lib.gbrmsd_rmsd_to_reference_noalloc(xd.data_ptr(), F, A, Ap, 3 * Ap, _lib.ATOM_MAJOR,
                                                    _lib.MODE_CENTER, r.ws.data_ptr(), None, 0.0, -1,
                                                    out.data_ptr(), cent.data_ptr(), None, stream))
    return D.to_host(out, stream), D.to_host(cent, stream)


def _noalloc_word(stream) -> tuple[int, int]:
    word = C.c_int32(-1)
    rc = _lib.lib.gbrmsd_noalloc_status(C.addressof(word), stream)
    return rc, word.value


def test_no_alloc_entry_point_matches_workspace_entry_point_on_consecutive_calls(cuda):
    stream = D.stream_handle()
    for F, A, seed in [(3000, 777, 1), (700, 4096, 2), (700, 4096, 2)]:
        xd, Ap, r = _case(F, A, seed, cuda, stream)
        want, want_c = _with_workspace(xd, F, A, Ap, r, cuda, stream)
        got, got_c = _no_alloc(xd, F, A, Ap, r, cuda, stream)
        assert _noalloc_word(stream) == (_lib.GBRMSD_OK, 0)
        assert np.all(np.isfinite(got))
        np.testing.assert_array_equal(got, want, err_msg=f"rmsd {(F, A)}")
        np.testing.assert_array_equal(got_c, want_c, err_msg=f"centroids {(F, A)}")


def test_no_alloc_entry_point_rejects_requests_beyond_its_scratch(cuda):
    stream = D.stream_handle()
    A = Ap = 4
    F_max = int(_lib.lib.gbrmsd_noalloc_max_frames(A))
    assert 60_000 < F_max < 100_000
    assert _lib.lib.gbrmsd_rmsd_workspace_bytes(F_max + 1, A) > 16 << 20
    F = F_max + 1
    x = torch.zeros((F, 3 * Ap), dtype=torch.float32, device=cuda)  # real buffers: nothing is out of bounds
    out = torch.empty(F, dtype=torch.float32, device=cuda)
    r = D.DeviceReference(np.zeros((A, 3), np.float32), _lib.ATOM_MAJOR, centre=True)
    args = (A, Ap, 3 * Ap, _lib.ATOM_MAJOR, _lib.MODE_CENTER, r.ws.data_ptr(), None, 0.0, -1, out.data_ptr(), None,
            None, stream)
    rc = _lib.lib.gbrmsd_rmsd_to_reference_noalloc(x.data_ptr(), F, *args)
    assert rc == _lib.E_WORKSPACE
    assert f"at most {F_max} frames of {A} atoms" in _lib.last_error()
    # the largest accepted call runs
    _lib.check(_lib.lib.gbrmsd_rmsd_to_reference_noalloc(x.data_ptr(), F_max, *args))
    assert _noalloc_word(stream) == (_lib.GBRMSD_OK, 0)


def test_no_alloc_status_reports_an_expired_wait(cuda):
    """A bounded wait made to run out (the copy it waits for is never
    issued) is visible to a caller of the allocation-free entry point, and
    the next call is clean again."""
    lib = _lib.lib
    stream = D.stream_handle()
    F, A = 2000, 500
    xd, Ap, r = _case(F, A, 4, cuda, stream)
    want, _ = _no_alloc(xd, F, A, Ap, r, cuda, stream)
    try:
        _lib.check(lib.gbrmsd_set_wait_limit_ns(20_000_000))
        _lib.check(lib.gbrmsd_test_skip_copy(3))
        _no_alloc(xd, F, A, Ap, r, cuda, stream)
        rc, word = _noalloc_word(stream)
        assert rc == _lib.E_DEVICE and word & _lib.ERR_TIMEOUT, (rc, word)
    finally:
        lib.gbrmsd_test_skip_copy(-1)
        lib.gbrmsd_set_wait_limit_ns(0)
    got, _ = _no_alloc(xd, F, A, Ap, r, cuda, stream)
    assert _noalloc_word(stream) == (_lib.GBRMSD_OK, 0)
    np.testing.assert_array_equal(got, want)
