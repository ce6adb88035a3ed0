"""GPU parity of the single-reference path against the reference's golden
vectors and the FP64 Kabsch oracle.  Bar: |gpu - fp64| <= 1e-4 nm and
|gpu - ref| <= 1e-4 + |ref - fp64| (conftest.assert_parity)."""
import numpy as np
import pytest
import torch

import mdtraj_gb300 as md
from conftest import ABS_TOL, assert_parity
from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, _rmsd, synth
from oracle import fp64

pytestmark = pytest.mark.gpu


class Obj:
    def __init__(self, xyz, traces=None):
        self.xyz = xyz
        self._rmsd_traces = traces


def test_frame0_xtc_md_rmsd_and_side_effect(cuda, golden):
    d = golden("frame0_xtc.npz")
    t = md.Trajectory(d["xyz"].copy())
    out = md.rmsd(t, t, 0)
    assert out.dtype == np.float32 and out.shape == (501,)
    assert out[0] == 0.0  # self pair: the reference's pointer-equality shortcut
    assert_parity(out, d["kabsch_fp64_frame0"], d["rmsd_frame0"], what="frame0.xtc")
    assert int(np.argmax(out)) == 44
    # md.rmsd centres the target in place, like the reference
    np.testing.assert_allclose(t.xyz, d["xyz_after_rmsd"], atol=5e-7)


def test_frame0_xtc_center_coordinates_and_precentered(cuda, golden):
    d = golden("frame0_xtc.npz")
    t = md.Trajectory(d["xyz"].copy())
    t.center_coordinates()
    np.testing.assert_allclose(t._rmsd_traces, d["traces"], rtol=2e-7)
    np.testing.assert_allclose(t.xyz, d["centred"], atol=5e-7)
    fp0 = fp64.kabsch_rmsd(d["xyz"], d["xyz"][0])
    fp10 = fp64.kabsch_rmsd(d["xyz"], d["xyz"][10])
    assert_parity(md.rmsd(t, t, 0, precentered=True), fp0, d["rmsd_precentered_frame0"], what="pre0")
    out10 = md.rmsd(t, t, 10, precentered=True)
    assert out10[10] == 0.0
    assert_parity(out10, fp10, d["rmsd_precentered_frame10"], what="pre10")


def test_frame0_xtc_axis_major_entry_point(cuda, golden):
    d = golden("frame0_xtc.npz")
    axis = np.ascontiguousarray(d["centred"].transpose(0, 2, 1))
    g = d["traces"].copy()
    out = _rmsd.getMultipleRMSDs_axis_major(axis, axis, g, g, 0)
    assert out[0] == 0.0
    assert_parity(out, d["kabsch_fp64_frame0"], d["rmsd_axis_major_frame0"], what="axis")
    atom = np.ascontiguousarray(d["centred"])
    out2 = _rmsd.getMultipleRMSDs_atom_major(atom, atom, g, g, 0)
    assert_parity(out2, d["kabsch_fp64_frame0"], d["rmsd_axis_major_frame0"], what="atom-major entry")


def test_frame0_xtc_nosuperpose_and_atom_indices(cuda, golden):
    d = golden("frame0_xtc.npz")
    t = md.Trajectory(d["xyz"].copy())
    ns = md.rmsd(t, t, 0, superpose=False)
    np.testing.assert_allclose(ns, fp64.msd_nosuperpose(d["xyz"], d["xyz"][0]), atol=1e-6)
    np.testing.assert_allclose(ns, d["rmsd_nosuperpose_frame0"], atol=1e-6)
    np.testing.assert_array_equal(t.xyz, d["xyz"])  # superpose=False does not centre
    sel = d["atom_indices"]
    t2 = md.Trajectory(d["xyz"].copy())
    out = md.rmsd(t2, t2, 0, atom_indices=sel)
    fp = fp64.kabsch_rmsd(d["xyz"][:, sel], d["xyz"][0, sel])
    assert_parity(out, fp, d["rmsd_atom_indices_frame0"], what="atom_indices")
    np.testing.assert_array_equal(t2.xyz, d["xyz"])  # a selection is a copy: no side effect


@pytest.mark.parametrize("case", ["cfg0_small", "copies", "atoms1", "atoms2", "atoms3", "atoms5", "cfg0_mid"])
def test_synthetic_golden_cases(cuda, golden, case):
    s = golden("synthetic.npz")
    x = s[f"{case}__xyz"]
    frame = int(s[f"{case}__frame"])
    t = md.Trajectory(x.copy())
    out = md.rmsd(t, t, frame)
    assert out[frame] == 0.0
    assert_parity(out, s[f"{case}__fp64"], s[f"{case}__ref"], what=case)
    # the same values when the reference frame is a separate object
    out2 = md.rmsd(md.Trajectory(x.copy()), md.Trajectory(x[frame:frame + 1].copy()), 0)
    assert_parity(out2, s[f"{case}__fp64"], what=case + " (separate reference)")
    ns = md.rmsd(md.Trajectory(x.copy()), md.Trajectory(x.copy()), frame, superpose=False)
    np.testing.assert_allclose(ns, s[f"{case}__nosup"], atol=2e-6, rtol=2e-6)


def test_ref_atom_indices_case(cuda, golden):
    s = golden("synthetic.npz")
    x, other = s["indices__xyz"], s["indices__other"]
    ai, rai = s["indices__ai"], s["indices__rai"]
    out = md.rmsd(Obj(x.copy()), Obj(other.copy()), 2, atom_indices=ai, ref_atom_indices=rai)
    fp = fp64.kabsch_rmsd(x[:, ai], other[2, rai])
    assert_parity(out, fp, s["indices__ref"], what="ref_atom_indices")


@pytest.mark.parametrize("A", [97, 7000, 12000])
@pytest.mark.parametrize("layout", [_lib.ATOM_MAJOR, _lib.AXIS_MAJOR])
def test_device_api_all_kernel_configs(cuda, A, layout):
    # A = 97: reference + 3 stages of 128 quads in shared memory;
    # A = 7000: 64-quad stages; A = 12000: reference read through L2.
    F = 96 if A > 5000 else 2000
    ref, x = synth.single_reference_frames(F, A, seed=A, sigma=np.geomspace(1e-3, 0.5, F), exact_fraction=0.05)
    want = fp64.kabsch_rmsd(x, ref)
    host = x if layout == _lib.ATOM_MAJOR else np.ascontiguousarray(x.transpose(0, 2, 1))
    stream = D.stream_handle()
    xd, Ap = D.frames_to_device(host, layout, cuda, stream)
    r = D.DeviceReference(ref, layout, centre=True)
    cent = torch.empty((F, 3), dtype=torch.float32, device=cuda)
    tr = torch.empty(F, dtype=torch.float32, device=cuda)
    out = D.rmsd_to_reference(xd, F, A, Ap, layout, _lib.MODE_CENTER, r, centroid_out=cent, trace_out=tr)
    got = D.to_host(out, stream)
    mx, rms = assert_parity(got, want, what=f"A={A} layout={layout}")
    c64 = x.astype(np.float64).mean(1)
    np.testing.assert_allclose(D.to_host(cent, stream), c64, atol=5e-7)
    a = x.astype(np.float64) - c64[:, None]
    np.testing.assert_allclose(D.to_host(tr, stream), (a * a).sum((1, 2)), rtol=1e-6)


@pytest.mark.parametrize("A", [1, 2, 3, 5, 7, 31, 33, 128, 129])
@pytest.mark.parametrize("F", [1, 2, 127])
def test_small_and_odd_shapes(cuda, A, F):
    ref, x = synth.single_reference_frames(F, A, seed=100 * A + F, sigma=0.1)
    out = md.rmsd(md.Trajectory(x.copy()), md.Trajectory(ref[None].copy()), 0)
    assert_parity(out, fp64.kabsch_rmsd(x, ref), what=f"A={A} F={F}")


def test_empty_atom_selection_and_empty_trajectory(cuda):
    ref, x = synth.single_reference_frames(5, 10, seed=1)
    t = md.Trajectory(x.copy())
    with pytest.warns(Warning):
        out = md.rmsd(t, t, 0, atom_indices=[])
    np.testing.assert_array_equal(out, np.zeros(5, np.float32))
    empty = Obj(np.zeros((0, 10, 3), np.float32))
    assert md.rmsd(empty, t, 0).shape == (0,)


def test_few_frames_many_atoms_uses_split_frames(cuda):
    # 3 frames x 50k atoms: each frame is split across warps and recombined
    ref, x = synth.single_reference_frames(3, 50000, seed=5, sigma=np.array([0.0, 0.01, 0.3]))
    out = md.rmsd(md.Trajectory(x.copy()), md.Trajectory(ref[None].copy()), 0)
    assert_parity(out, fp64.kabsch_rmsd(x, ref), what="split frames")


def test_exact_copies_are_refined_to_zero(cuda):
    ref, x = synth.single_reference_frames(200, 4000, seed=9, sigma=0.0)
    out = md.rmsd(md.Trajectory(x.copy()), md.Trajectory(ref[None].copy()), 0)
    want = fp64.kabsch_rmsd(x, ref)
    assert want.max() < 1e-5
    assert_parity(out, want, what="exact copies")
    assert out.max() < 5e-6


def test_precentered_atom_major_entry_with_separate_arrays(cuda):
    ref, x = synth.single_reference_frames(300, 301, seed=21, sigma=0.05)
    a = x.copy()
    g = _rmsd._center_inplace_atom_major(a)
    b = a[5:6].copy()
    gb = g[5:6].copy()
    out = _rmsd.getMultipleRMSDs_atom_major(b, a, gb, g, 0)
    assert_parity(out, fp64.kabsch_rmsd(x, x[5]), what="atom-major separate")
    assert out[5] < 1e-5


def test_workspace_reports_no_device_error(cuda):
    ref, x = synth.single_reference_frames(64, 100, seed=2)
    stream = D.stream_handle()
    xd, Ap = D.frames_to_device(x, _lib.ATOM_MAJOR, cuda, stream)
    r = D.DeviceReference(ref, _lib.ATOM_MAJOR, centre=True)
    ws = D.empty_bytes(_lib.lib.gbrmsd_rmsd_workspace_bytes(64, 100), cuda)
    out = torch.empty(64, dtype=torch.float32, device=cuda)
    _lib.check(_lib.lib.gbrmsd_rmsd_to_reference(xd.data_ptr(), 64, 100, Ap, 3 * Ap, 0, 0, r.ws.data_ptr(), None,
                                                 0.0, -1, out.data_ptr(), None, None, ws.data_ptr(), ws.numel(),
                                                 stream))
    _lib.check(_lib.lib.gbrmsd_workspace_status(ws.data_ptr(), stream))


def test_reference_info_matches_reference_centring(cuda, golden):
    d = golden("frame0_xtc.npz")
    r = D.DeviceReference(d["xyz"][3], _lib.ATOM_MAJOR, centre=True)
    g, cen = r.info()
    mu = (d["xyz"][3].astype(np.float64).sum(0) / 22).astype(np.float32)
    np.testing.assert_array_equal(cen, mu)
    c = d["xyz"][3] - mu
    assert abs(g - float((c.astype(np.float64) ** 2).sum())) < 1e-5 * g
