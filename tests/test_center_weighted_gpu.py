"""Trajectory.center_coordinates(mass_weighted=True) on the GPU
(gbrmsd_center_weighted_inplace) against the reference's own output
(tests/golden/center_mass.npz) and the FP64 restatement (oracle/fp64.py).

The reference subtracts a float64 centre of mass from float32 coordinates
(core/trajectory.py:2133-2134); the kernel forms the centre in float pairs and
rounds x - com once, so a coordinate may differ from the reference's only
where x - com lies within ~2^-40 of a float rounding midpoint: at most one
ulp, and in practice never on these inputs."""
import types

import numpy as np
import pytest

from mdtraj_gb300 import Trajectory
from oracle import fp64

pytestmark = pytest.mark.gpu


class _Top:
    """Topology stand-in: atoms carrying element masses."""

    def __init__(self, masses):
        self._atoms = [types.SimpleNamespace(element=types.SimpleNamespace(mass=float(m))) for m in masses]
        self.n_atoms = len(masses)

    @property
    def atoms(self):
        return iter(self._atoms)


def _assert_close_ulp(got, want, what):
    got = np.asarray(got)
    want = np.asarray(want)
    fin = np.isfinite(want)
    np.testing.assert_array_equal(got[~fin], want[~fin], err_msg=f"{what}: non-finite entries")
    g, w = got[fin], want[fin]
    assert np.all(np.isfinite(g)), what
    ulp = np.spacing(np.abs(w).astype(np.float32))
    diff = np.abs(g.astype(np.float64) - w.astype(np.float64))
    assert np.all(diff <= ulp), f"{what}: max {float((diff / ulp).max()):.2f} ulp"
    mism = int(np.count_nonzero(g != w))
    assert mism <= max(1, g.size // 100_000), f"{what}: {mism} of {g.size} coordinates differ by one ulp"


@pytest.mark.parametrize("name", ["mixed", "chunk", "hydrogen", "nonfinite"])
def test_mass_weighted_centring_matches_reference(cuda, golden, name):
    d = golden("center_mass.npz")
    x = d[f"{name}__xyz"].copy()
    t = Trajectory(x, _Top(d[f"{name}__masses"]))
    t.center_coordinates()  # cached traces, dropped by the mass-weighted call
    assert t._rmsd_traces is not None
    t.xyz = d[f"{name}__xyz"].copy()
    buf = t.xyz
    with np.errstate(invalid="ignore"):
        assert t.center_coordinates(mass_weighted=True) is t
    assert t.xyz is buf, "centred in place"
    assert t._rmsd_traces is None
    _assert_close_ulp(t.xyz, d[f"{name}__centred"], name)
    if name == "hydrogen":  # the reference's test_center: equal masses give a zero mean
        np.testing.assert_allclose(t.xyz.mean(1), 0.0, atol=1e-6)


@pytest.mark.parametrize("F,A,seed", [(2000, 1000, 1), (37, 5003, 2), (1, 1, 3), (9, 2, 4), (300, 2048, 5)])
def test_mass_weighted_centring_matches_oracle(cuda, F, A, seed):
    rng = np.random.default_rng(seed)
    masses = np.array([1.008, 12.011, 14.007, 15.999, 32.06])[rng.integers(0, 5, A)]
    x = (rng.uniform(-4, 4, size=(F, A, 3)) + rng.uniform(-30, 30, size=(F, 1, 3))).astype(np.float32)
    want = x.copy()
    com = fp64.center_of_mass_inplace(want, masses)
    t = Trajectory(x, _Top(masses))
    t.center_coordinates(mass_weighted=True)
    _assert_close_ulp(t.xyz, want, f"{F}x{A}")
    # the centred frames' own mass-weighted centres are ~0
    w = masses / masses.sum()
    resid = np.einsum("fkc,k->fc", t.xyz.astype(np.float64), w)
    assert np.abs(resid).max() <= 4 * np.spacing(np.float32(np.abs(com).max() + 4.0))


def test_mass_weighted_centring_empty_and_no_topology(cuda):
    t = Trajectory(np.zeros((0, 5, 3), np.float32), _Top(np.ones(5)))
    t.center_coordinates(mass_weighted=True)
    assert t.xyz.shape == (0, 5, 3)
    # without a topology the reference centres uniformly and caches the traces
    x = np.random.default_rng(0).normal(size=(4, 6, 3)).astype(np.float32)
    t = Trajectory(x.copy())
    t.center_coordinates(mass_weighted=True)
    assert t._rmsd_traces is not None
    np.testing.assert_allclose(t.xyz.mean(1), 0.0, atol=1e-6)
