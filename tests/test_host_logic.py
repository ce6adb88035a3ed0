"""Boundary behaviour of the drop-in that needs no GPU: argument validation
and errors identical to mdtraj/rmsd/_rmsd.pyx:152-184 and the memmap tests
(tests/test_rmsd_memmap.py), ensure_type and Trajectory semantics (CPU)."""
import warnings

import numpy as np
import pytest

import mdtraj_gb300 as md
from mdtraj_gb300 import _rmsd
from mdtraj_gb300.utils import TypeCastPerformanceWarning, ensure_type


def traj(F=4, A=6, seed=0):
    return md.Trajectory(np.random.default_rng(seed).normal(size=(F, A, 3)).astype(np.float32))


def test_invalid_atom_indices_raise_value_error():
    t = traj()
    with pytest.raises(ValueError, match="atom_indices must be valid"):
        md.rmsd(t, t, 0, atom_indices=[0, 6])
    with pytest.raises(ValueError, match="atom_indices must be valid"):
        md.rmsd(t, t, 0, atom_indices=[-1, 2])
    with pytest.raises(ValueError, match="ref_atom_indices must be valid"):
        md.rmsd(t, t, 0, atom_indices=[0, 1], ref_atom_indices=[0, 9])
    with pytest.raises(ValueError, match="same number of atom indices"):
        md.rmsd(t, t, 0, atom_indices=[0, 1], ref_atom_indices=[0, 1, 2])


def test_frame_out_of_range_and_atom_mismatch():
    t = traj()
    with pytest.raises(ValueError, match="Cannot calculate RMSD of frame 4"):
        md.rmsd(t, t, 4)
    # different atom counts without indices: the reference evaluates
    # len(slice) and raises TypeError
    with pytest.raises(TypeError):
        md.rmsd(traj(A=6), traj(A=7), 0)


def test_wrong_ndim_is_an_assertion():
    class Obj:
        xyz = np.zeros((3, 4, 2), dtype=np.float32)
        _rmsd_traces = None

    with pytest.raises(AssertionError):
        md.rmsd(Obj(), Obj(), 0)


def test_read_only_target_raises_value_error():
    # tests/test_rmsd_memmap.py:11-56: read-only coordinates cannot be centred
    t = traj()
    t._xyz.setflags(write=False)
    with pytest.raises(ValueError):
        md.rmsd(t, t, 0)
    t2 = traj()
    t2._rmsd_traces = np.ones(4, dtype=np.float32)
    t2._xyz.setflags(write=False)
    with pytest.raises(ValueError):
        md.rmsd(t2, t2, 0, precentered=True)


def test_axis_major_argument_checks():
    x = np.zeros((3, 3, 5), dtype=np.float32)
    g = np.zeros(3, dtype=np.float32)
    with pytest.raises(ValueError, match="same number of atoms"):
        _rmsd.getMultipleRMSDs_axis_major(x, np.zeros((3, 3, 6), dtype=np.float32), g, g, 0)
    with pytest.raises(ValueError, match="Cannot calculate RMSD of frame 3"):
        _rmsd.getMultipleRMSDs_axis_major(x, x, g, g, 3)
    with pytest.raises(AssertionError):
        _rmsd.getMultipleRMSDs_axis_major(np.zeros((3, 4, 5), np.float32), np.zeros((3, 4, 5), np.float32), g, g, 0)
    with pytest.raises(ValueError, match="dtype mismatch"):
        _rmsd.getMultipleRMSDs_axis_major(x.astype(np.float64), x, g, g, 0)
    with pytest.raises(ValueError, match="C-contiguous"):
        _rmsd.getMultipleRMSDs_axis_major(np.zeros((3, 5, 3), np.float32).transpose(0, 2, 1), x, g, g, 0)
    with pytest.raises(TypeError):
        _rmsd.getMultipleRMSDs_atom_major(None, x, g, g, 0)


def test_no_device_means_loud_failure_not_cpu_fallback():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    t = traj()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        md.rmsd(t, t, 0)


def test_precentered_warning_paths_emit_runtime_warning():
    import torch

    if torch.cuda.is_available():
        pytest.skip("covered by the GPU tests")
    t = traj()
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        with pytest.raises(RuntimeError):
            md.rmsd(t, t, 0, precentered=True)  # no traces: warns, then needs the device
    assert any("precentered is ignored" in str(x.message) for x in w)


def test_ensure_type_semantics():
    with pytest.warns(TypeCastPerformanceWarning):
        a = ensure_type(np.arange(3, dtype=np.int32), dtype=np.int64, ndim=1, name="a")
    assert a.dtype == np.int64
    with pytest.raises(ValueError, match="must be ndim 2"):
        ensure_type(np.zeros(3), np.float32, 2, "b")
    v = ensure_type(np.zeros((4, 3)), np.float32, 3, "xyz", add_newaxis_on_deficient_ndim=True, warn_on_cast=False)
    assert v.shape == (1, 4, 3) and v.flags.c_contiguous
    with pytest.raises(ValueError, match="must be shape"):
        ensure_type(np.zeros((2, 4, 2)), np.float32, 3, "xyz", shape=(None, None, 3), warn_on_cast=False)
    with pytest.raises(TypeError):
        ensure_type(3.0, np.float32, 2, "c")
    assert ensure_type(None, np.float32, 1, "d", can_be_none=True) is None


def test_trajectory_contract():
    t = traj(F=5)
    assert t.xyz.dtype == np.float32 and t.xyz.flags.c_contiguous
    t._rmsd_traces = np.arange(5, dtype=np.float32)
    s = t[1:3]
    np.testing.assert_array_equal(s._rmsd_traces, [1, 2])
    np.testing.assert_array_equal(s.xyz, t.xyz[1:3])
    t.xyz = t.xyz * 2  # setting coordinates invalidates cached traces
    assert t._rmsd_traces is None
    one = md.Trajectory(np.zeros((4, 3)))
    assert one.n_frames == 1 and one.n_atoms == 4


def test_autotune_bucket_and_cache_roundtrip(tmp_path, monkeypatch):
    from mdtraj_gb300 import autotune

    monkeypatch.setenv("MDTRAJ_GB300_CACHE", str(tmp_path))
    b1 = autotune.shape_bucket([100, 2000, 50], [10, 20, 30])
    b2 = autotune.shape_bucket([101, 2005, 50], [10, 20, 30])
    assert b1 == b2 and b1.startswith("ragged:")
    assert autotune.load_cache() == {}
    autotune.save_cache({b1: {"config": 2, "max_unit_quads": 256}})
    assert autotune.load_cache()[b1]["config"] == 2


def test_autotune_cache_writers_do_not_collide(tmp_path, monkeypatch):
    """Eight threads saving different caches at once: every save succeeds,
    the file always parses as one complete cache, and no temporary file is
    left behind."""
    import threading

    from mdtraj_gb300 import autotune

    monkeypatch.setenv("MDTRAJ_GB300_CACHE", str(tmp_path))
    errors = []

    def writer(k):
        try:
            for i in range(50):
                autotune.save_cache({f"ragged:{k}": {"config": i, "pad": "x" * 4096}})
                got = autotune.load_cache()
                assert len(got) == 1 and next(iter(got.values()))["pad"] == "x" * 4096
        except BaseException as e:  # re-raised on the main thread
            errors.append(e)

    threads = [threading.Thread(target=writer, args=(k,)) for k in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:1]
    assert [p.name for p in tmp_path.iterdir()] == ["autotune.json"]


def test_ragged_layout_is_padded_and_aligned():
    from mdtraj_gb300 import RaggedBatch

    off, padded, total = RaggedBatch.layout([5, 8, 1], [2, 3, 4])
    assert list(padded) == [8, 8, 4]
    assert list(off) == [0, 2 * 3 * 8, 2 * 3 * 8 + 3 * 3 * 8]
    assert all(o % 4 == 0 for o in off) and total == off[-1] + 4 * 3 * 4


def test_pool_allocator_first_fit_and_merge():
    from mdtraj_gb300.serving import PoolAllocator

    p = PoolAllocator(100)
    a, b, c = p.alloc(30), p.alloc(50), p.alloc(20)
    assert (a, b, c) == (0, 30, 80) and p.alloc(1) is None
    p.release(b, 50)
    assert p.alloc(60) is None and p.alloc(40) == 30
    p.release(a, 30)
    p.release(30, 40)
    p.release(c, 20)
    assert p.free == [(0, 100)] and p.free_rows == 100


def test_host_result_pool_returns_pages_when_results_are_dropped():
    """Results are arrays over pool pages; the pages come back only when the
    result and every view of it are gone (no device needed: without one the
    pool is simply not page-locked)."""
    import gc

    from mdtraj_gb300.serving import HostResultPool

    pool = HostResultPool(16 * 4096)
    pool.locked = True  # (without a device the buffer is not locked; exercise the page bookkeeping)
    a = pool.take(3 * 4096 + 1)          # 4 pages
    b = pool.take(4096)                  # 1 page
    assert (a, b) == (0, 4) and pool.pages.free_rows == 11
    ra = pool.result(a, 10, 3 * 4096 + 1)
    ra[:] = np.arange(10, dtype=np.float32)
    view = ra.reshape(2, 5)[1]
    del ra
    gc.collect()
    assert pool.pages.free_rows == 11 and view.tolist() == [5, 6, 7, 8, 9]
    del view
    gc.collect()
    assert pool.pages.free_rows == 15
    pool.release(b, 4096)
    assert pool.pages.free == [(0, 16)]
    pool.locked = False


def test_batch_grouped_by_database_range():
    """A batch that owns one contiguous run of pool rows is laid out sorted
    by database range (each request contiguous, the run unchanged); a batch
    with gaps between its rows is left as admitted."""
    from mdtraj_gb300.serving import Request, RmsdServer

    def req(q, a, b, p0):
        r = Request(queries=np.zeros((q, 3, 3), np.float32), db0=a, db1=b)
        r._p0 = p0
        return r

    batch = [req(5, 300, 900, 10), req(3, 0, 1000, 15), req(4, 100, 200, 18), req(2, 0, 1000, 22)]
    RmsdServer._group_by_range(batch)
    order = sorted(batch, key=lambda r: r._p0)
    assert [(r.db0, r.db1) for r in order] == [(0, 1000), (0, 1000), (100, 200), (300, 900)]
    assert [(r._p0, r.n_query) for r in order] == [(10, 3), (13, 2), (15, 4), (19, 5)]
    gaps = [req(5, 300, 900, 10), req(3, 0, 1000, 40)]
    RmsdServer._group_by_range(gaps)
    assert [r._p0 for r in gaps] == [10, 40]


def test_cross_request_validation_in_library():
    """gbrmsd_cross_rmsd validates the request table before any device call."""
    import ctypes as C

    from mdtraj_gb300 import _lib
    from mdtraj_gb300.cross import request_table

    lib = _lib.lib
    fake = 1 << 20  # 16-byte aligned stand-in pointers: never dereferenced on these paths
    ws_bytes = lib.gbrmsd_cross_workspace_bytes(100, 16, 2)
    assert lib.gbrmsd_cross_workspace_bytes(100, 16, 100) > ws_bytes >= lib.gbrmsd_cross_workspace_bytes(100, 16, 1) > 0

    def call(reqs, method=1, n_db=100):
        t = request_table(reqs)
        return lib.gbrmsd_cross_rmsd(fake, 100, n_db, fake, 16, 8, C.addressof(t), len(reqs), method, fake, ws_bytes, None)

    assert call([(fake, 0, 4, 0, 10), (fake, 3, 2, 0, 10)]) == _lib.E_INVALID
    assert b"share query row" in lib.gbrmsd_last_error()
    assert call([(fake, 14, 4, 0, 10)]) == _lib.E_INVALID          # beyond the query capacity
    assert call([(fake, 0, 4, 5, 101)]) == _lib.E_INVALID          # beyond the database
    assert call([(None, 0, 4, 0, 10)]) == _lib.E_INVALID           # no output
    assert call([(fake, 0, 4, 0, 10)], method=2) == _lib.E_INVALID
    assert call([(fake, 0, 4, 0, 10)], n_db=101) == _lib.E_INVALID  # more frames than the set holds
    t = request_table([(fake, 0, 4, 0, 10)])
    assert lib.gbrmsd_cross_rmsd(fake, 100, 100, fake, 16, 8, C.addressof(t), 1, 1, fake, ws_bytes - 1,
                                 None) == _lib.E_WORKSPACE


def test_gaussian_chain_geometry():
    import math

    from mdtraj_gb300 import synth

    x = synth.gaussian_chain(3, 40, seed=2, sigma=0.0).double().numpy()
    d = np.diff(x, axis=1)
    np.testing.assert_allclose(np.linalg.norm(d, axis=2), 0.38, atol=1e-5)
    u, v = d[:, :-1], d[:, 1:]
    cosang = -(u * v).sum(2) / (np.linalg.norm(u, axis=2) * np.linalg.norm(v, axis=2))
    np.testing.assert_allclose(cosang, math.cos(math.radians(120.0)), atol=1e-4)
    q = synth.perturbed_queries(x.astype(np.float32), [1, 2], seed=0, sigma=0.0)
    from oracle import fp64

    assert fp64.kabsch_rmsd(q[:1], x[1])[0] < 1e-5
