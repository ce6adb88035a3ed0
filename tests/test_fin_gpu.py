"""The single-reference call's two finishes agree with the FP64 oracle.

With one unit per frame the streaming kernel finishes its own frames (float
pair records, QCP 32 frames per warp, CTA-wide refinement); otherwise, or
when the finish's few bytes of shared memory do not fit beside the
reference and the copy stages, a second kernel finishes from FP64 records.
Atom counts at the edge of the shared-memory budget take either path; a
forced 8-warp configuration always takes the second."""
import numpy as np
import pytest
import torch

from conftest import assert_parity
from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, synth
from oracle import fp64

pytestmark = pytest.mark.gpu


def _run(cuda, x, ref, layout, mode=_lib.MODE_CENTER):
    F, A = x.shape[0], x.shape[1]
    host = x if layout == _lib.ATOM_MAJOR else np.ascontiguousarray(x.transpose(0, 2, 1))
    stream = D.stream_handle()
    xd, Ap = D.frames_to_device(host, layout, cuda, stream)
    r = D.DeviceReference(ref, layout, centre=True)
    ws = D.empty_bytes(_lib.lib.gbrmsd_rmsd_workspace_bytes(F, A), cuda)
    cent = torch.empty((F, 3), dtype=torch.float32, device=cuda)
    out = D.rmsd_to_reference(xd, F, A, Ap, layout, mode, r, centroid_out=cent, ws=ws)
    _lib.check(_lib.lib.gbrmsd_workspace_status(ws.data_ptr(), stream))
    return D.to_host(out, stream), D.to_host(cent, stream)


@pytest.mark.parametrize("A", [2940, 2944, 2960, 2964, 7040, 7056, 11136, 11152])
def test_finish_paths_at_the_shared_memory_edge(cuda, A):
    F = 600
    ref, x = synth.single_reference_frames(F, A, seed=A, sigma=np.geomspace(1e-3, 0.3, F), exact_fraction=0.03)
    want = fp64.kabsch_rmsd(x, ref)
    got, cent = _run(cuda, x, ref, _lib.ATOM_MAJOR)
    assert_parity(got, want, what=f"A={A}")
    np.testing.assert_allclose(cent, x.astype(np.float64).mean(1), atol=5e-7)


@pytest.mark.parametrize("layout", [_lib.ATOM_MAJOR, _lib.AXIS_MAJOR])
def test_in_kernel_and_separate_finish_agree(cuda, layout):
    """The same frames through the default (in-kernel finish) and a forced
    8-warp configuration (separate finish): both within the bar of FP64 and
    within 2e-6 nm of each other."""
    F, A = 5000, 1000
    ref, x = synth.single_reference_frames(F, A, seed=9, sigma=np.geomspace(1e-3, 0.5, F), exact_fraction=0.02)
    want = fp64.kabsch_rmsd(x, ref)
    a, ca = _run(cuda, x, ref, layout)
    n_cfg = _lib.lib.gbrmsd_stream_config_count()
    try:
        _lib.check(_lib.lib.gbrmsd_stream_config_select(n_cfg - 3))  # first 8-warp configuration
        b, cb = _run(cuda, x, ref, layout)
    finally:
        _lib.lib.gbrmsd_stream_config_select(-1)
    assert_parity(a, want, what="in-kernel finish")
    assert_parity(b, want, what="separate finish")
    assert np.abs(a.astype(np.float64) - b).max() <= 2e-6
    np.testing.assert_allclose(ca, cb, atol=5e-7)
