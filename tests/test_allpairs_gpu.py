"""All-pairs RMSD matrix (tensor-core split-BF16 and FP32 CUDA-core paths)
against the FP64 Kabsch oracle and the reference's own per-row output
(md.rmsd(traj, traj, i, precentered=True) through the compiled reference)."""
import numpy as np
import pytest

import mdtraj_gb300 as md
from conftest import ABS_TOL, assert_parity
from mdtraj_gb300 import synth
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
