"""The QCP solve of every finish (mdtraj_gb300/csrc/qcp.cuh, __host__
__device__) built for the host and checked on degenerate structures (CPU).

Collinear structures (and every 2-atom selection) give K a double largest
eigenvalue.  For exact rotated copies the Newton start, the upper bound
(G_a + G_b) / 2, is that double root: P and P' there are rounding noise, so
the solve must stop on P's rounding floor (not step to the negative double
root), and the rotation must come from the eigenspace (not from an adjugate
that is all rounding noise).  The reference itself returns ~1e-3 nm for
exact copies; here the finish must give < 1e-5 nm.  Nearly collinear and
general structures are checked against the eigenvalues of K (numpy) and
the FP64 Kabsch oracle.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ABS_TOL
from oracle import fp64

HERE = Path(__file__).resolve().parent


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return None


@pytest.fixture(scope="module")
def qcp_bin(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("qcp") / "qcp_host_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-ffp-contract=off", "-o", str(out),
                    str(HERE / "qcp_host_check.cu")], check=True, capture_output=True)
    return out


def _run(qcp_bin, pairs):
    lines = []
    for a, b in pairs:
        lines.append(str(len(a)))
        lines.extend(" ".join(f"{v:.9g}" for v in np.concatenate([a[k], b[k]])) for k in range(len(a)))
    r = subprocess.run([str(qcp_bin)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    return np.array([[float(v) for v in ln.split()] for ln in r.stdout.splitlines()])


def _rotation(rng):
    q = rng.normal(size=4)
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _case(kind, rng, sigma=0.0):
    if kind == "atoms2":
        b = rng.uniform(-2, 2, (2, 3))
    elif kind == "collinear":
        b = np.outer(rng.uniform(-2, 2, 40), rng.uniform(-1, 1, 3))
    else:  # general
        b = rng.uniform(-2, 2, (int(rng.integers(3, 200)), 3))
    b = b.astype(np.float32)
    a = (b.astype(np.float64) @ _rotation(rng).T + rng.uniform(-2, 2, 3) + sigma * rng.normal(size=b.shape))
    return a.astype(np.float32), b


def _finish_rmsd(res):
    """What the finish returns: the direct residual for flagged frames."""
    return np.where(res[:, 4] > 0, res[:, 5], np.sqrt(res[:, 3]))


@pytest.mark.parametrize("kind", ["atoms2", "collinear"])
def test_exact_copies_of_collinear_structures(qcp_bin, kind):
    rng = np.random.default_rng(5 if kind == "atoms2" else 6)
    res = _run(qcp_bin, [_case(kind, rng) for _ in range(400)])
    lam, lam64, lam0, lamdf = res[:, 0], res[:, 1], res[:, 2], res[:, 6]
    assert np.all(lam > 0) and np.all(lam64 > 0) and np.all(lamdf > 0), "converged to the negative double root"
    assert np.abs(lam - lam0).max() <= 1e-6 * lam0.max()
    assert np.abs(lamdf - lam0).max() <= 1e-6 * lam0.max()
    assert _finish_rmsd(res).max() < 1e-5
    assert res[:, 7].max() < 1e-5  # the refinement pass's rotation
    assert res[:, 8].max() < 1e-5  # the same from float-pair M and lambda (in-kernel finish)


def test_refinement_rotation_near_identical_frames(qcp_bin):
    """The FP32 rotation of the refinement pass gives the residual of the
    FP64 rotation on near-identical general frames (where it is used): the
    msd is second order in the rotation's ~1e-7 error, the rmsd first order,
    ~1e-7 x the structure's size (measured up to 4.5e-7 nm on exact copies
    of 4 nm structures, against 1e-7 with the FP64 rotation)."""
    rng = np.random.default_rng(11)
    pairs = [_case("general", rng, s) for s in (0.0, 1e-5, 1e-4, 1e-3) for _ in range(100)]
    res = _run(qcp_bin, pairs)
    np.testing.assert_allclose(res[:, 7], res[:, 5], rtol=0, atol=1e-6)
    # the in-kernel finish builds the same rotation from float-pair M and
    # lambda, without FP64
    np.testing.assert_allclose(res[:, 8], res[:, 5], rtol=0, atol=1e-6)


@pytest.mark.parametrize("kind,sigma", [("collinear", 0.01), ("atoms2", 0.05), ("general", 0.1), ("general", 1e-4)])
def test_noisy_structures_against_eigenvalues_and_fp64(qcp_bin, kind, sigma):
    rng = np.random.default_rng(int(sigma * 1e4) + len(kind))
    pairs = [_case(kind, rng, sigma) for _ in range(300)]
    res = _run(qcp_bin, pairs)
    true = []
    for a, b in pairs:
        x = a.astype(np.float64) - a.mean(0, dtype=np.float64)
        y = b.astype(np.float64) - b.mean(0, dtype=np.float64)
        m = x.T @ y
        k = np.array([[m[0, 0] + m[1, 1] + m[2, 2], m[1, 2] - m[2, 1], m[2, 0] - m[0, 2], m[0, 1] - m[1, 0]],
                      [m[1, 2] - m[2, 1], m[0, 0] - m[1, 1] - m[2, 2], m[0, 1] + m[1, 0], m[2, 0] + m[0, 2]],
                      [m[2, 0] - m[0, 2], m[0, 1] + m[1, 0], -m[0, 0] + m[1, 1] - m[2, 2], m[1, 2] + m[2, 1]],
                      [m[0, 1] - m[1, 0], m[2, 0] + m[0, 2], m[1, 2] + m[2, 1], -m[0, 0] - m[1, 1] + m[2, 2]]])
        true.append(np.linalg.eigvalsh(k)[-1])
    true = np.array(true)
    assert (np.abs(res[:, 0] - true) / res[:, 2]).max() <= 1e-6
    assert (np.abs(res[:, 1] - true) / res[:, 2]).max() <= 1e-6
    assert (np.abs(res[:, 6] - true) / res[:, 2]).max() <= 1e-6
    if kind == "general":
        # simple roots: the float-float solve agrees with the FP64 one to
        # ~2^-44 of the bound (at near double roots both stop on their
        # rounding floors, ~1e-7 apart)
        assert (np.abs(res[:, 6] - res[:, 1]) / res[:, 2]).max() <= 1e-12
    want = np.array([fp64.kabsch_rmsd(a[None], b)[0] for a, b in pairs])
    assert np.abs(_finish_rmsd(res) - want).max() <= ABS_TOL
