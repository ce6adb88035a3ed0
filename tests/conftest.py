"""Shared test setup.

Markers: ``gpu`` — needs a CUDA device (GB300); everything else runs on CPU.
Golden fixtures live in tests/golden/ (generated by tests/golden/make_golden.py
from the reference itself).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

# Parity bar (nm): every GPU result within ABS_TOL of the FP64 Kabsch oracle,
# and within ABS_TOL + |reference - fp64| of the reference's float32 output.
ABS_TOL = 1e-4


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / name)

    return load


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("this test needs a CUDA device")
    import mdtraj_gb300._device as D

    D.require_device()
    return torch.device("cuda", torch.cuda.current_device())


def assert_parity(gpu, fp64, ref=None, tol=ABS_TOL, what=""):
    """GPU vs FP64 oracle within tol; vs the reference within tol + ref error."""
    gpu = np.asarray(gpu, dtype=np.float64)
    fp64 = np.asarray(fp64, dtype=np.float64)
    err = np.abs(gpu - fp64)
    assert np.all(np.isfinite(gpu)), f"{what}: non-finite output"
    assert err.max(initial=0.0) <= tol, f"{what}: max |gpu - fp64| = {err.max():.3e} nm at {int(err.argmax())}"
    if ref is not None:
        ref = np.asarray(ref, dtype=np.float64)
        bound = tol + np.abs(ref - fp64)
        d = np.abs(gpu - ref)
        bad = d > bound
        assert not bad.any(), f"{what}: |gpu - ref| exceeds bound at {np.flatnonzero(bad)[:5]} ({d[bad][:5]})"
    return err.max(initial=0.0), float(np.sqrt(np.mean(err ** 2))) if err.size else 0.0
