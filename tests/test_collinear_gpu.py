"""md.rmsd and Trajectory.superpose on collinear structures (every 2-atom
selection, linear molecules) on the GPU, where K has a double largest
eigenvalue: exact rotated copies must come out at 0 (the reference returns
~1e-3 nm there), nearly collinear noisy frames within the parity bar of the
FP64 oracle, and superposed exact copies on the reference frame."""
import numpy as np
import pytest

import mdtraj_gb300 as md
from conftest import assert_parity
from oracle import fp64

pytestmark = pytest.mark.gpu


def _rotation(rng):
    q = rng.normal(size=4)
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _frames(A, F, seed, sigma):
    """Frame 0 collinear (A atoms on a line); frames 4k exact rotated and
    translated copies of it, the others with Gaussian noise sigma."""
    rng = np.random.default_rng(seed)
    base = np.outer(rng.uniform(-2, 2, A), rng.uniform(-1, 1, 3))
    x = np.empty((F, A, 3), np.float32)
    x[0] = base
    for f in range(1, F):
        noise = 0.0 if f % 4 == 0 else sigma * rng.normal(size=base.shape)
        x[f] = (base + noise) @ _rotation(rng).T + rng.uniform(-2, 2, 3)
    return x


@pytest.mark.parametrize("A", [2, 3, 40, 1001])
def test_collinear_exact_copies_and_noisy_frames(cuda, A):
    x = _frames(A, 400, seed=A, sigma=0.01)
    out = md.rmsd(md.Trajectory(x.copy()), md.Trajectory(x[:1].copy()), 0)
    want = fp64.kabsch_rmsd(x, x[0])
    assert_parity(out, want, what=f"collinear A={A}")
    assert np.abs(out[::4]).max() < 1e-5, out[::4].max()


def test_superpose_collinear_frames(cuda):
    # noise-free: every frame an exact rotated copy, so the superposed
    # coordinates are unique (the spin about the line moves no atom)
    x = _frames(40, 200, seed=9, sigma=0.0)
    t = md.Trajectory(x.copy())
    t.superpose(md.Trajectory(x[:1].copy()), frame=0)
    assert np.abs(t.xyz - x[0]).max() < 2e-5


def _pairs_fp64(x):
    F = x.shape[0]
    iu = np.triu_indices(F, 1)
    v = fp64.kabsch_rmsd_pairs(x, np.stack(iu, 1))
    want = np.zeros((F, F))
    want[iu] = v
    want[(iu[1], iu[0])] = v
    return want


@pytest.mark.parametrize("method", ["tensor", "fp32"])
@pytest.mark.parametrize("A", [2, 3, 40, 300])
def test_allpairs_tile_epilogue_at_double_roots(cuda, method, A):
    """Every 2-atom pair, and every pair with a collinear structure in it, has
    a double largest eigenvalue of K; the tiles' FP32 Newton cannot resolve it
    and hands the pair to the exact refinement."""
    x = _frames(A, 160, seed=100 + A, sigma=0.01)
    got = md.allpairs_rmsd(x, method=method)
    assert_parity(got.ravel(), _pairs_fp64(x).ravel(), what=f"all-pairs {method} collinear A={A}")
    sub = got[::4][:, ::4]  # exact rotated copies of frame 0, hence of each other
    assert np.abs(sub).max() < 1e-5, sub.max()


@pytest.mark.parametrize("method", ["tensor", "fp32"])
def test_allpairs_two_atom_random_frames(cuda, method):
    rng = np.random.default_rng(5)
    base = rng.uniform(0, 3, (2, 3))
    x = (base[None] + rng.normal(0, 0.1, (120, 2, 3))).astype(np.float32)
    got = md.allpairs_rmsd(x, method=method)
    assert_parity(got.ravel(), _pairs_fp64(x).ravel(), what=f"all-pairs {method} 2 atoms")


@pytest.mark.parametrize("method", ["tensor", "fp32"])
def test_cross_tile_epilogue_at_double_roots(cuda, method):
    from mdtraj_gb300 import serving

    for A in (2, 40):
        db = _frames(A, 300, seed=200 + A, sigma=0.01)
        queries = _frames(A, 24, seed=300 + A, sigma=0.01)
        queries[0] = db[0]  # an exact copy of a database frame
        server = serving.RmsdServer(db, method=method, query_capacity=64, slots=1)
        done = server.serve([serving.Request(queries=queries, db0=0, db1=300, rid=0)], realtime=False)
        got = done[0].result
        want = np.stack([fp64.kabsch_rmsd(db, q) for q in queries])
        assert_parity(got.ravel(), want.ravel(), what=f"cross {method} collinear A={A}")
        assert abs(got[0, 0]) < 1e-5
