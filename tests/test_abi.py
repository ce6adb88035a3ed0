"""The C-ABI library loads and exports every entry point declared in
include/gbrmsd.h; argument validation works without a GPU (CPU)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "gbrmsd.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(gbrmsd_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from mdtraj_gb300 import _lib

    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(_lib.lib, n), f"{n} declared in gbrmsd.h but not exported"
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"
    assert _lib.lib.gbrmsd_version() >= 1


def test_invalid_arguments_are_rejected_before_any_launch():
    from mdtraj_gb300 import _lib

    lib = _lib.lib
    # bad layout
    rc = lib.gbrmsd_rmsd_to_reference(16, 10, 8, 8, 24, 7, 0, 16, None, 0.0, -1, 16, None, None, 16, 1 << 20, None)
    assert rc == _lib.E_INVALID and "layout" in _lib.last_error()
    # n_padded not a multiple of 4
    rc = lib.gbrmsd_rmsd_to_reference(16, 10, 7, 7, 21, 0, 0, 16, None, 0.0, -1, 16, None, None, 16, 1 << 20, None)
    assert rc == _lib.E_INVALID and "n_padded" in _lib.last_error()
    # misaligned coordinates
    rc = lib.gbrmsd_rmsd_to_reference(20, 10, 8, 8, 24, 0, 0, 16, None, 0.0, -1, 16, None, None, 16, 1 << 20, None)
    assert rc == _lib.E_INVALID and "aligned" in _lib.last_error()
    # bad mode
    rc = lib.gbrmsd_rmsd_to_reference(16, 10, 8, 8, 24, 0, 9, 16, None, 0.0, -1, 16, None, None, 16, 1 << 20, None)
    assert rc == _lib.E_INVALID and "mode" in _lib.last_error()
    # precentered needs traces
    rc = lib.gbrmsd_rmsd_to_reference(16, 10, 8, 8, 24, 0, 1, 16, None, 0.0, -1, 16, None, None, 16, 1 << 20, None)
    assert rc == _lib.E_INVALID
    # workspace too small (validated before launching)
    rc = lib.gbrmsd_rmsd_to_reference(16, 10, 8, 8, 24, 0, 0, 16, None, 0.0, -1, 16, None, None, 16, 8, None)
    assert rc == _lib.E_WORKSPACE
    rc = lib.gbrmsd_prepare_reference(16, 5, 5, 0, 1, 16, 1 << 20, None)
    assert rc == _lib.E_INVALID
    with pytest.raises(ValueError):
        _lib.check(_lib.E_INVALID)


def test_workspace_sizes_scale_with_problem():
    from mdtraj_gb300 import _lib

    lib = _lib.lib
    a = lib.gbrmsd_reference_workspace_bytes(1000, 1000)
    b = lib.gbrmsd_reference_workspace_bytes(10000, 10000)
    assert 12 * 1000 < a < b
    assert lib.gbrmsd_reference_workspace_bytes(5, 3) == 0
    w1 = lib.gbrmsd_rmsd_workspace_bytes(1000, 100)
    w2 = lib.gbrmsd_rmsd_workspace_bytes(100000, 100)
    assert 0 < w1 < w2


def test_host_side_effect_helper_matches_numpy():
    from mdtraj_gb300 import _lib

    rng = np.random.default_rng(0)
    x = rng.normal(size=(37, 11, 3)).astype(np.float32)
    c = rng.normal(size=(37, 3)).astype(np.float32)
    want = x - c[:, None, :]
    _lib.check(_lib.lib.gbrmsd_host_subtract_centroids(x.ctypes.data, 37, 11, 33, c.ctypes.data, 4))
    np.testing.assert_array_equal(x, want)


def test_rmsd_workspace_is_monotone_in_frames():
    """A workspace sized for F frames must serve every call with fewer frames
    (the last chunk of a stream, a partial batch): the size never decreases
    as F grows."""
    from mdtraj_gb300 import _lib

    lib = _lib.lib
    for A in (1, 100, 1000, 4000, 10000, 100000):
        prev = 0
        for F in list(range(1, 3000, 7)) + [9728, 9729, 10**4, 10**5, 10**6]:
            w = lib.gbrmsd_rmsd_workspace_bytes(F, A)
            assert w >= prev, (A, F, w, prev)
            prev = w
