"""Superposition on the GPU: Trajectory.superpose, superpose_atom_major, rmsf
and getMultipleAlignDisplaceRMSDs_atom_major against the reference's own
outputs (tests/golden/superpose_rmsf.npz) and the FP64 oracle.

Coordinates (nm) and RMSF values: |gpu - fp64| <= ABS_TOL and
|gpu - ref| <= ABS_TOL + |ref - fp64|."""
import numpy as np
import pytest

import mdtraj_gb300 as md
from conftest import ABS_TOL, assert_parity
from mdtraj_gb300 import _rmsd, synth
from oracle import fp64

pytestmark = pytest.mark.gpu


def test_superpose_matches_reference(cuda, golden):
    g = golden("superpose_rmsf.npz")
    x, rolled, sub, shifted = g["xyz"], g["rolled"], g["sub"], g["shifted"]
    cases = [
        ("all_f3", dict(frame=3), x, fp64.superpose(x, x[3])),
        ("sub_f0", dict(frame=0, atom_indices=sub), x, fp64.superpose(x, x[0], sub)),
        ("other_f2", dict(frame=2, atom_indices=sub, ref_atom_indices=shifted), rolled,
         fp64.superpose(x, rolled[2], sub, shifted)),
    ]
    for name, kw, refxyz, want in cases:
        t = md.Trajectory(x.copy())
        t._rmsd_traces = np.ones(len(x), np.float32)
        out = t.superpose(md.Trajectory(refxyz.copy()), **kw)
        assert out is t and t._rmsd_traces is None   # setting xyz resets the cached traces
        assert t.xyz.dtype == np.float32 and t.xyz.shape == x.shape
        assert_parity(t.xyz.ravel(), want.ravel(), g[f"sup_{name}"].ravel(), what=f"superpose {name}")


def test_superpose_large_and_exact_copies(cuda):
    ref, x = synth.single_reference_frames(1500, 1003, seed=5, sigma=0.1, exact_fraction=0.02)
    t = md.Trajectory(x.copy())
    t.superpose(md.Trajectory(x), frame=0)
    want = fp64.superpose(x, x[0])
    assert_parity(t.xyz.ravel(), want.ravel(), what="superpose 1500 x 1003")
    # exact rotated copies land on the reference
    exact = [i for i in range(len(x)) if fp64.kabsch_rmsd(x[i:i + 1], x[0])[0] < 1e-5]
    assert len(exact) >= 20
    assert np.abs(t.xyz[exact] - x[0]).max() < 2e-5


def test_superpose_argument_errors(cuda):
    t = md.Trajectory(np.zeros((2, 5, 3), np.float32) + np.arange(15, dtype=np.float32).reshape(5, 3))
    with pytest.raises(ValueError, match="greater than 0"):
        t.superpose(t, atom_indices=[])
    with pytest.raises(ValueError, match="consistent"):
        t.superpose(t, atom_indices=[0, 1, 2], ref_atom_indices=[0, 1])


def test_superpose_atom_major_rotates_in_place(cuda):
    ref, x = synth.single_reference_frames(64, 37, seed=9, sigma=0.1)
    align = np.ascontiguousarray(x - x.astype(np.float64).mean(1, keepdims=True), dtype=np.float32)
    target = align[:4].copy()
    g = np.einsum("ijk,ijk->i", align, align).astype(np.float32)
    gt = np.einsum("ijk,ijk->i", target, target).astype(np.float32)
    disp = align.copy()
    assert _rmsd.superpose_atom_major(target, align, gt, g, disp, 2) is None
    R = fp64.kabsch_rotations(align, target[2], centre=False)
    want = np.einsum("fij,fkj->fki", R, align.astype(np.float64))
    assert_parity(disp.ravel(), want.ravel(), what="superpose_atom_major")
    with pytest.raises(ValueError, match="same number of atoms"):
        _rmsd.superpose_atom_major(target[:, :10].copy(), align, gt, g, disp, 0)
    with pytest.raises(ValueError, match="same number of frames"):
        _rmsd.superpose_atom_major(target, align, gt, g, disp[:5].copy(), 0)


def test_rmsf_matches_reference(cuda, golden):
    g = golden("superpose_rmsf.npz")
    x, other, sub = g["xyz"], g["other"], g["sub"]
    t = md.Trajectory(x.copy())
    got = md.rmsf(t, t, 0)
    assert got.dtype == np.float32 and got.shape == (x.shape[1],)
    assert_parity(got, fp64.rmsf(x, x[0]), g["rmsf_self_f0"], what="rmsf self")
    # side effect: the target is centred in place (the reference's centring)
    assert np.abs(t.xyz - g["rmsf_self_f0_centred"]).max() < 1e-6
    t = md.Trajectory(x.copy())
    assert_parity(md.rmsf(t, None), fp64.rmsf(x, None), g["rmsf_none"], what="rmsf prealigned")
    t = md.Trajectory(x.copy())
    r = md.Trajectory(x.copy())
    got = md.rmsf(t, r, 5, atom_indices=sub)
    assert got.shape == (len(sub),)
    assert_parity(got, fp64.rmsf(x, x[5], atom_indices=sub), g["rmsf_sub_f5"], what="rmsf subset")
    np.testing.assert_array_equal(t.xyz, g["rmsf_sub_f5_xyz_after"])   # a selected copy is centred, not target
    t = md.Trajectory(x.copy())
    r = md.Trajectory(other.copy())
    assert_parity(md.rmsf(t, r, 1), fp64.rmsf(x, other[1]), g["rmsf_other_f1"], what="rmsf other reference")
    assert np.abs(r.xyz - g["rmsf_other_f1_ref_after"]).max() < 1e-6   # reference frame centred in place


def test_rmsf_precentered_and_errors(cuda):
    ref, x = synth.single_reference_frames(200, 64, seed=4, sigma=0.1)
    a = md.Trajectory(x.copy())
    b = md.Trajectory(x.copy())
    b.center_coordinates()
    want = md.rmsf(a, a, 3)
    got = md.rmsf(b, b, 3, precentered=True)
    assert np.abs(got - want).max() < 1e-5
    with pytest.warns(RuntimeWarning):
        md.rmsf(b, b, 3, atom_indices=np.arange(10), precentered=True)
    with pytest.raises(ValueError, match="Mode must be one of"):
        md.rmsf(a, a, 0, mode="chain")
    with pytest.raises(ValueError, match="Cannot calculate RMSF of frame"):
        md.rmsf(a, a, 500)
    with pytest.raises(ValueError, match="valid positive indices"):
        md.rmsf(a, a, 0, atom_indices=[0, 64])


class _Top:
    """Duck-typed topology: atoms 0-2 residue 0 (masses 1, 2, 3), 3-5 residue 1, residue 2 empty."""

    class _Atom:
        def __init__(self, i):
            self.residue = type("R", (), {"index": i // 3})()
            self.element = type("E", (), {"mass": float(i % 3 + 1)})()

    n_residues = 3

    def atom(self, i):
        return self._Atom(i)


def test_rmsf_residue_mode(cuda):
    ref, x = synth.single_reference_frames(50, 6, seed=8, sigma=0.2)
    t = md.Trajectory(x.copy())
    per_atom = md.rmsf(md.Trajectory(x.copy()), md.Trajectory(x.copy()), 0)
    t.topology = _Top()
    got = md.rmsf(t, md.Trajectory(x.copy()), 0, mode="residue")
    m = np.array([1, 2, 3, 1, 2, 3], np.float64)
    want0 = np.sqrt((per_atom[:3] ** 2 * m[:3]).sum() / m[:3].sum())
    want1 = np.sqrt((per_atom[3:] ** 2 * m[3:]).sum() / m[3:].sum())
    np.testing.assert_allclose(got[:2], [want0, want1], rtol=1e-5)
    assert got[2] == -1.0


def test_align_displace_matches_reference(cuda, golden):
    g = golden("superpose_rmsf.npz")
    al, di, gg = g["ad_align"], g["ad_displ"], g["ad_g"]
    d, rot = _rmsd.getMultipleAlignDisplaceRMSDs_atom_major(al, al, gg, gg, di, di, 21, 30, 4)
    want_d, want_r = fp64.align_displace(al[4, :21], al[:, :21], di[4, :30], di[:, :30])
    assert d.dtype == np.float32 and rot.shape == (len(al), 3, 3)
    assert_parity(d, want_d, g["ad_rmsd"], what="align-displace rmsd")
    assert np.abs(rot - want_r).max() < 1e-5 and np.abs(rot - g["ad_rot"]).max() < 1e-5
    with pytest.raises(ValueError, match="4\\*n"):
        _rmsd.getMultipleAlignDisplaceRMSDs_atom_major(al[:, :21].copy(), al, gg, gg, di, di, 21, 30, 4)
    with pytest.raises(ValueError, match="Cannot calculate RMSD of frame"):
        _rmsd.getMultipleAlignDisplaceRMSDs_atom_major(al, al, gg, gg, di, di, 21, 30, 99)
