"""Parity at the benchmark workloads' own sizes, against the reference's own
float32 md.rmsd (its CPU kernels compiled from its sources) as well as the
FP64 Kabsch oracle.

* md.rmsd on 10,000 frames x 1,000 atoms, host arrays, not precentered:
  the reference's benchmark class (md.rmsd over a trajectory, mdtraj/rmsd/
  _rmsd.pyx:211-224), generated as that workload is (reference uniform in a
  4 nm cube, sigma 0.05 nm, Haar rotations, translations in [-2, 2] nm).
  Every frame is checked, and so is the in-place centring side effect.
* The all-pairs matrix at 4,000 frames x 2,000 atoms (several row groups and
  fold units of the tensor tiles), random walk over 50 metastable centres:
  20,000 sampled pairs against FP64 and whole rows against the reference's
  precentered md.rmsd(traj, traj, i) (examples/clustering.ipynb, cell 6).
"""
import numpy as np
import pytest

import mdtraj_gb300 as md
from conftest import assert_parity
from mdtraj_gb300 import synth
from oracle import cpu, fp64

pytestmark = pytest.mark.gpu


class Obj:
    def __init__(self, xyz):
        self.xyz = xyz
        self._rmsd_traces = None


def test_md_rmsd_10000x1000_matches_the_reference_on_every_frame(cuda):
    ref_frame, x = synth.single_reference_frames(10_000, 1_000, seed=2024, sigma=0.05)
    impl = cpu.best_available()
    x_ref, r_ref = x.copy(), ref_frame.copy()
    want_ref = impl.md_rmsd(x_ref, r_ref)               # centres both in place
    want64 = fp64.kabsch_rmsd(x, ref_frame)
    t, r = Obj(x.copy()), Obj(ref_frame[None].copy())
    got = md.rmsd(t, r, 0)
    assert got.dtype == np.float32 and got.shape == (10_000,)
    err, rms = assert_parity(got, want64, want_ref, what="md.rmsd 10,000 x 1,000")
    assert err < 1e-5, err
    # the reference's in-place centring of the target and of the reference
    # frame: the same float subtraction of a centroid that can differ from
    # the reference's in its last bit (the reference sums raw coordinates in
    # double; the streaming pass sums float differences from a shift, whose
    # roundings move the mean by ~1e-9 nm), so a few percent of the centred
    # coordinates differ by one float ulp
    np.testing.assert_allclose(t.xyz, x_ref, rtol=0, atol=2e-6)
    np.testing.assert_allclose(r.xyz[0], r_ref, rtol=0, atol=2e-6)
    assert np.mean(t.xyz == x_ref) > 0.9


@pytest.mark.parametrize("method", ["tensor", "fp32"])
def test_allpairs_4000x2000_sampled_pairs_and_reference_rows(cuda, method):
    labels, x = synth.metastable_walk(4000, 2000, n_centres=50, seed=77, sigma=0.1, cube=5.0)
    got = md.allpairs_rmsd(x, method=method)
    assert got.shape == (4000, 4000)
    np.testing.assert_array_equal(got, got.T)
    assert not np.diag(got).any()
    rng = np.random.default_rng(1)
    pairs = rng.integers(0, 4000, (22_000, 2))
    pairs = pairs[pairs[:, 0] != pairs[:, 1]][:20_000]
    want = fp64.kabsch_rmsd_pairs(x, pairs)
    assert_parity(got[pairs[:, 0], pairs[:, 1]], want, what=f"{method} 20,000 sampled pairs")
    impl = cpu.best_available()
    xc = x.copy()
    g = impl.center_inplace(xc)
    for i in (0, 1234, 3999):
        row_ref = impl.multiple(xc, xc, g, g, i, axis_major=False)
        row64 = fp64.kabsch_rmsd(x, x[i])
        assert_parity(got[i], row64, row_ref, what=f"{method} row {i}")
