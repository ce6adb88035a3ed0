"""Failure detection on the GPU without a GPU fault.

* A bounded wait that runs out: the failure-detection hook makes the
  streaming kernel never issue one bulk copy (nothing is put in flight for
  it), so the wait on that stage expires after a short limit.  The kernel
  records DEV_ERR_TIMEOUT, waits for its other copies and returns; the status
  calls report GBRMSD_E_DEVICE, the drop-in raises, and the next call on the
  same context gives the same bits as before.
* Non-finite coordinates: the reference clamps the NaN msd of such a frame to
  0 (mdtraj/rmsd/src/theobald_rmsd.cpp:275-277) and centres it in place to
  NaN / +-inf (src/center_generic.h); the GPU path returns the same values,
  records DEV_ERR_NONFINITE, and the drop-in warns.
"""
import ctypes as C
import time
import warnings

import numpy as np
import pytest
import torch

import mdtraj_gb300 as md
from conftest import assert_parity
from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, synth
from oracle import cpu, fp64

pytestmark = pytest.mark.gpu


@pytest.fixture
def hooks():
    lib = _lib.lib
    yield lib
    lib.gbrmsd_test_skip_copy(-1)
    lib.gbrmsd_set_wait_limit_ns(0)


class Obj:
    def __init__(self, xyz):
        self.xyz = xyz
        self._rmsd_traces = None


def _word(ws, stream) -> int:
    w = C.c_int32(-1)
    _lib.check(_lib.lib.gbrmsd_workspace_error_word(ws.data_ptr(), C.addressof(w), stream))
    return w.value


@pytest.mark.parametrize("layout", [_lib.ATOM_MAJOR, _lib.AXIS_MAJOR])
def test_expired_wait_is_reported_and_the_context_stays_usable(cuda, hooks, layout):
    lib = hooks
    F, A = 3000, 1000
    ref, x = synth.single_reference_frames(F, A, seed=5, sigma=0.05)
    stream = D.stream_handle()
    host = np.ascontiguousarray(x.transpose(0, 2, 1)) if layout == _lib.AXIS_MAJOR else x
    xd, Ap = D.frames_to_device(host, layout, cuda, stream)
    r = D.DeviceReference(ref, layout, centre=True)
    ws = D.empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(F, A), cuda)
    out = torch.empty(F, dtype=torch.float32, device=cuda)

    def run():
        _lib.check(lib.gbrmsd_rmsd_to_reference(xd.data_ptr(), F, A, Ap, 3 * Ap, layout, _lib.MODE_CENTER,
                                                r.ws.data_ptr(), None, 0.0, -1, out.data_ptr(), None, None,
                                                ws.data_ptr(), ws.numel(), stream))
        return D.to_host(out, stream)

    want = run()
    assert _word(ws, stream) == 0
    assert lib.gbrmsd_workspace_status(ws.data_ptr(), stream) == _lib.GBRMSD_OK
    # the hook is refused unless the wait limit is short
    assert lib.gbrmsd_test_skip_copy(5) == _lib.E_INVALID
    _lib.check(lib.gbrmsd_set_wait_limit_ns(20_000_000))  # 20 ms
    _lib.check(lib.gbrmsd_test_skip_copy(5))
    t0 = time.perf_counter()
    run()
    dt = time.perf_counter() - t0
    assert _word(ws, stream) & _lib.ERR_TIMEOUT
    assert lib.gbrmsd_workspace_status(ws.data_ptr(), stream) == _lib.E_DEVICE
    assert "bounded wait expired" in _lib.last_error()
    assert dt < 5.0, dt
    _lib.check(lib.gbrmsd_test_skip_copy(-1))
    _lib.check(lib.gbrmsd_set_wait_limit_ns(0))
    got = run()
    assert _word(ws, stream) == 0
    np.testing.assert_array_equal(got, want)


def test_drop_in_raises_when_a_wait_expires(cuda, hooks):
    lib = hooks
    ref, x = synth.single_reference_frames(500, 300, seed=6, sigma=0.05)
    _lib.check(lib.gbrmsd_set_wait_limit_ns(20_000_000))
    _lib.check(lib.gbrmsd_test_skip_copy(0))
    with pytest.raises(_lib.GbrmsdError, match="bounded wait"):
        md.rmsd(Obj(x.copy()), Obj(ref[None].copy()), 0)
    lib.gbrmsd_test_skip_copy(-1)
    lib.gbrmsd_set_wait_limit_ns(0)
    out = md.rmsd(Obj(x.copy()), Obj(ref[None].copy()), 0)
    assert_parity(out, fp64.kabsch_rmsd(x, ref), what="after an expired wait")


def test_wait_limit_is_validated():
    lib = _lib.lib
    assert lib.gbrmsd_set_wait_limit_ns(10) == _lib.E_INVALID
    assert lib.gbrmsd_set_wait_limit_ns(61_000_000_000) == _lib.E_INVALID
    assert lib.gbrmsd_test_skip_copy(-2) == _lib.E_INVALID
    _lib.check(lib.gbrmsd_set_wait_limit_ns(0))


def _nonfinite_case():
    ref, x = synth.single_reference_frames(64, 37, seed=3, sigma=0.1)
    x[2, 5, 0] = np.nan              # one NaN
    x[3, 7, 1] = np.inf              # one +inf: the reference's centroid is +inf
    x[4, 7, 1] = -np.inf             # +inf and -inf on one axis: NaN
    x[4, 9, 1] = np.inf
    x[5, :, 2] = np.inf              # a whole axis infinite
    x[9, 0] = np.nan                 # a whole atom NaN
    return ref, x


def test_nonfinite_frames_match_the_reference(cuda):
    ref, x = _nonfinite_case()
    bad = [2, 3, 4, 5, 9]
    ok = [f for f in range(len(x)) if f not in bad]
    impl = cpu.best_available()
    x_ref, r_ref = x.copy(), ref.copy()
    want = impl.md_rmsd(x_ref, r_ref)  # centres both in place
    t = Obj(x.copy())
    r = Obj(ref[None].copy())
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        got = md.rmsd(t, r, 0)
    assert any("non-finite" in str(w.message) for w in caught)
    np.testing.assert_array_equal(got[bad], np.zeros(len(bad), np.float32))
    np.testing.assert_array_equal(got[bad], want[bad])
    assert_parity(got[ok], fp64.kabsch_rmsd(x[ok], ref), want[ok], what="finite frames beside non-finite ones")
    # the in-place centring side effect: NaN and +-inf where the reference has them
    for f in range(len(x)):
        a, b = t.xyz[f], x_ref[f]
        assert np.array_equal(np.isnan(a), np.isnan(b)), f
        assert np.array_equal(np.isposinf(a), np.isposinf(b)) and np.array_equal(np.isneginf(a), np.isneginf(b)), f
        fin = np.isfinite(b)
        np.testing.assert_allclose(a[fin], b[fin], atol=5e-7, err_msg=str(f))


def test_nonfinite_input_sets_the_error_word(cuda):
    lib = _lib.lib
    ref, x = _nonfinite_case()
    F, A = x.shape[:2]
    stream = D.stream_handle()
    xd, Ap = D.frames_to_device(x, _lib.ATOM_MAJOR, cuda, stream)
    r = D.DeviceReference(ref, _lib.ATOM_MAJOR, centre=True)
    ws = D.empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(F, A), cuda)
    out = torch.empty(F, dtype=torch.float32, device=cuda)
    _lib.check(lib.gbrmsd_rmsd_to_reference(xd.data_ptr(), F, A, Ap, 3 * Ap, _lib.ATOM_MAJOR, _lib.MODE_CENTER,
                                            r.ws.data_ptr(), None, 0.0, -1, out.data_ptr(), None, None,
                                            ws.data_ptr(), ws.numel(), stream))
    assert _word(ws, stream) == _lib.ERR_NONFINITE
    assert lib.gbrmsd_workspace_status(ws.data_ptr(), stream) == _lib.E_DEVICE
    assert "non-finite" in _lib.last_error()
    # a clean call clears it
    xc = D.frames_to_device(synth.single_reference_frames(F, A, seed=1)[1], _lib.ATOM_MAJOR, cuda, stream)[0]
    _lib.check(lib.gbrmsd_rmsd_to_reference(xc.data_ptr(), F, A, Ap, 3 * Ap, _lib.ATOM_MAJOR, _lib.MODE_CENTER,
                                            r.ws.data_ptr(), None, 0.0, -1, out.data_ptr(), None, None,
                                            ws.data_ptr(), ws.numel(), stream))
    assert _word(ws, stream) == 0


def test_center_coordinates_of_nonfinite_frames_match_the_reference(cuda):
    _, x = _nonfinite_case()
    x_ref = x.copy()
    g_ref = cpu.best_available().center_inplace(x_ref)
    t = md.Trajectory(x.copy())
    t.center_coordinates()
    for f in range(len(x)):
        a, b = t.xyz[f], x_ref[f]
        assert np.array_equal(np.isnan(a), np.isnan(b)), f
        assert np.array_equal(np.isposinf(a), np.isposinf(b)) and np.array_equal(np.isneginf(a), np.isneginf(b)), f
        fin = np.isfinite(b)
        np.testing.assert_allclose(a[fin], b[fin], atol=5e-7, err_msg=str(f))
    assert np.array_equal(np.isnan(t._rmsd_traces), np.isnan(g_ref))
