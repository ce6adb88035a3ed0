"""The allocation-free entry point gbrmsd_rmsd_to_reference_noalloc.

Some callers cannot allocate device memory when they need RMSDs: code
inside another runtime's memory pool (the pool owns the device memory), a
plugin whose host application hands it buffers but no allocator, or a loop
that must not call cudaMalloc/cudaFree (they can synchronise the device).
For them the library keeps a fixed 16 MiB
scratch array on the device and this entry point takes no workspace.  The
test calls it through the C ABI, twice in a row (different shapes, then the
same shape again, so state left by one call cannot leak into the next), and
checks it against gbrmsd_rmsd_to_reference with a caller workspace.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest
import torch

from conftest import ABS_TOL
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


def test_no_alloc_entry_point_matches_workspace_entry_point_on_consecutive_calls(cuda):
    stream = D.stream_handle()
    for F, A, seed in [(3000, 777, 1), (700, 4096, 2), (700, 4096, 2)]:
        xd, Ap, r = _case(F, A, seed, cuda, stream)
        want, want_c = _with_workspace(xd, F, A, Ap, r, cuda, stream)
        got, got_c = _no_alloc(xd, F, A, Ap, r, cuda, stream)
        assert np.all(np.isfinite(got))
        assert np.abs(got.astype(np.float64) - want).max() <= ABS_TOL, (F, A)
        assert np.abs(got_c.astype(np.float64) - want_c).max() <= 1e-6, (F, A)


def test_no_alloc_entry_point_rejects_requests_beyond_its_scratch(cuda):
    stream = D.stream_handle()
    F, A = 100_000, 4  # needs more than the 16 MiB scratch
    Ap = 4
    x = torch.zeros((F, 3 * Ap), dtype=torch.float32, device=cuda)  # real buffers: nothing is out of bounds
    out = torch.empty(F, dtype=torch.float32, device=cuda)
    r = D.DeviceReference(np.zeros((A, 3), np.float32), _lib.ATOM_MAJOR, centre=True)
    rc = _lib.lib.gbrmsd_rmsd_to_reference_noalloc(x.data_ptr(), F, A, Ap, 3 * Ap, _lib.ATOM_MAJOR,
                                                   _lib.MODE_CENTER, r.ws.data_ptr(), None, 0.0, -1,
                                                   out.data_ptr(), None, None, stream)
    assert rc == _lib.E_WORKSPACE
    assert "65536 frames" in _lib.last_error()
