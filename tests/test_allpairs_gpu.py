"""All-pairs RMSD matrix (tensor-core split-BF16 and FP32 CUDA-core paths)
against the FP64 Kabsch oracle and the reference's own per-row output
(md.rmsd(traj, traj, i, precentered=True) through the compiled reference)."""
import numpy as np
import pytest

import mdtraj_gb300 as md
from conftest import ABS_TOL, assert_parity
from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, cross, synth
from mdtraj_gb300._lib import check, lib
from mdtraj_gb300.allpairs import allpairs_device
from oracle import cpu, fp64

pytestmark = pytest.mark.gpu


def all_pairs_fp64(x):
    F = x.shape[0]
    iu = np.triu_indices(F, 1)
    pairs = np.stack(iu, 1)
    want = np.zeros((F, F))
    v = fp64.kabsch_rmsd_pairs(x, pairs)
    want[iu] = v
    want[(iu[1], iu[0])] = v
    return want


@pytest.mark.parametrize("method", ["tensor", "fp32"])
@pytest.mark.parametrize("F,A", [(300, 257), (43, 64), (81, 130), (1, 10), (2, 5), (97, 3)])
def test_allpairs_matches_fp64(cuda, method, F, A):
    labels, x = synth.metastable_walk(F, A, n_centres=7, seed=F + A)
    if F > 10:
        x[5] = x[4]                                   # exact duplicate frame
        x[7] = x[6] + np.random.default_rng(0).normal(0, 1e-3, x[6].shape).astype(np.float32)
    got = md.allpairs_rmsd(x, method=method)
    assert got.shape == (F, F) and got.dtype == np.float32
    assert np.all(np.diag(got) == 0.0)
    np.testing.assert_array_equal(got, got.T)
    want = all_pairs_fp64(x)
    assert_parity(got.ravel(), want.ravel(), what=f"{method} F={F} A={A}")


def test_allpairs_tensor_equals_fp32_and_reference_rows(cuda):
    labels, x = synth.metastable_walk(200, 500, n_centres=10, seed=3)
    t = md.allpairs_rmsd(x, method="tensor")
    f = md.allpairs_rmsd(x, method="fp32")
    assert np.abs(t - f).max() <= 2 * ABS_TOL
    ref = cpu.best_available()
    xc = x.copy()
    g = ref.center_inplace(xc)
    want = all_pairs_fp64(x)
    for i in (0, 17, 199):
        row = ref.multiple(xc, xc, g, g, i, axis_major=False)
        assert_parity(t[i], want[i], row, what=f"row {i} vs reference")


def test_allpairs_precentered_uses_coordinates_as_given(cuda):
    labels, x = synth.metastable_walk(60, 90, n_centres=4, seed=9)
    xc = x - x.astype(np.float64).mean(1, keepdims=True).astype(np.float32)
    a = md.allpairs_rmsd(xc, precentered=True, method="tensor")
    b = md.allpairs_rmsd(x, precentered=False, method="tensor")
    assert np.abs(a - b).max() < 1e-5


@pytest.mark.parametrize("method", ["tensor", "fp32"])
@pytest.mark.parametrize("A", [257, 1000])
def test_allpairs_rotated_copies_match_fp64(cuda, method, A):
    """Noisy rotated copies of one structure (0.001-0.4 nm noise, 3% exact
    copies): all 44,850 pairs, many of them just above the refinement
    threshold, where the split-BF16 inner products are least accurate."""
    F = 300
    _, x = synth.single_reference_frames(F, A, seed=F + A, sigma=np.geomspace(1e-3, 0.4, F), exact_fraction=0.03)
    got = md.allpairs_rmsd(x, method=method)
    np.testing.assert_array_equal(got, got.T)
    assert np.all(np.diag(got) == 0.0)
    assert_parity(got.ravel(), all_pairs_fp64(x).ravel(), what=f"{method} rotated copies A={A}")


def _near_identical(F=3000, A=64):
    """Every pair of these frames (~0.005 nm apart) lies below the refinement
    threshold (~0.37 nm here), and there are 4,498,500 of them: more than the
    workspace's refinement list of 2^22 entries."""
    _, x = synth.single_reference_frames(F, A, seed=5, sigma=2e-3)
    rng = np.random.default_rng(F)
    i = rng.integers(0, F, 20000)
    j = rng.integers(0, F, 20000)
    pairs = np.stack([np.minimum(i, j), np.maximum(i, j)], 1)
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    return x, pairs


@pytest.mark.parametrize("method", ["tensor", "fp32"])
def test_allpairs_refines_beyond_the_list_capacity(cuda, method):
    """Pairs that find the list full are marked in the output and refined by
    the refinement kernel's scan: every pair is refined, none is left NaN."""
    x, pairs = _near_identical()
    F, A = x.shape[0], x.shape[1]
    stream = D.stream_handle()
    xd, Ap = D.frames_to_device(x, _lib.ATOM_MAJOR, cuda, stream)
    ws = D.empty_bytes(lib.gbrmsd_allpairs_workspace_bytes(F, A), cuda)
    got = D.to_host(allpairs_device(xd, F, A, Ap, _lib.ATOM_MAJOR, method=method, ws=ws), stream)
    n = np.zeros(1, dtype=np.int32)
    check(lib.gbrmsd_allpairs_status(ws.data_ptr(), n.ctypes.data, stream))
    assert int(n[0]) == F * (F - 1) // 2 > (1 << 22)
    assert np.all(np.isfinite(got)) and np.all(np.diag(got) == 0.0)
    np.testing.assert_array_equal(got, got.T)
    want = fp64.kabsch_rmsd_pairs(x, pairs)
    assert_parity(got[pairs[:, 0], pairs[:, 1]], want, what=f"{method} beyond the list")


def test_cross_refines_beyond_the_list_capacity(cuda):
    """The same for the cross path: 3,000 queries against the 3,000 frames,
    9,000,000 pairs below the threshold."""
    x, pairs = _near_identical()
    got = cross.cross_rmsd(x, x, method="tensor")
    assert got.shape == (3000, 3000) and np.all(np.isfinite(got))
    want = fp64.kabsch_rmsd_pairs(x, pairs)
    assert_parity(got[pairs[:, 1], pairs[:, 0]], want, what="cross beyond the list")
    assert_parity(got[pairs[:, 0], pairs[:, 1]], want, what="cross beyond the list (transposed)")
