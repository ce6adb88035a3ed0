"""Superposition on the GB300: ``Trajectory.superpose``,
``superpose_atom_major``, ``rmsf`` and ``getMultipleAlignDisplaceRMSDs_atom_major``
with the reference's signatures, validation order, exceptions and in-place
effects (mdtraj/core/trajectory.py:1083-1170, mdtraj/rmsd/_rmsd.pyx:246-759).

Every per-frame computation runs in libgbrmsd.so: the optimal rotations come
from the streaming M pass plus a rotation-emitting QCP finish
(gbrmsd_rotations), and the coordinate work from gbrmsd_apply_rotations,
gbrmsd_rmsf and gbrmsd_rotated_rmsd.
"""
from __future__ import annotations

import ctypes as C
import warnings

import numpy as np
import torch

from . import _device as D
from . import _lib
from ._lib import check, lib
from ._rmsd import _memview1, _memview3, _writable_view
from .utils import ensure_type

OVERFLOW_MESSAGE = (
    "Encounted a potential overflow/underflow error during superpose() due to the magnitude of your `_xyz`"
    "coordinates. To circumvent this, (1) reload your trajectory and (2) divide and/or multiply your"
    "`_xyz` dataset by multiples of 10 before running superpose again. Then, (3) revert that "
    "multiplication/division after the calculations."
)


def _ptr(t):
    return None if t is None else t.data_ptr()


def _padded_device(x_dev: torch.Tensor, n_atoms: int) -> tuple[torch.Tensor, int]:
    """(F, n_atoms, 3) device tensor -> zero-padded (F, 3 * n_padded) buffer."""
    F = int(x_dev.shape[0])
    Ap = D.padded(n_atoms)
    if Ap == n_atoms and x_dev.is_contiguous():
        return x_dev.reshape(F, 3 * Ap), Ap
    buf = torch.zeros((F, Ap, 3), dtype=torch.float32, device=x_dev.device)
    buf[:, :n_atoms] = x_dev
    return buf.reshape(F, 3 * Ap), Ap


def _rotations(x_align: torch.Tensor, n_frames: int, n_align: int, n_padded: int, ref: D.DeviceReference, mode: int,
               g_target: torch.Tensor | None = None, g_ref: float = 0.0, want_mu: bool = False):
    """Per-frame rotations (F, 9) float32 [and FP64 centroids (F, 3)] of the
    alignment frames onto the prepared reference."""
    dev = x_align.device
    rot = torch.empty((n_frames, 9), dtype=torch.float32, device=dev)
    mu = torch.empty((n_frames, 3), dtype=torch.float64, device=dev) if want_mu else None
    ws = D.empty_bytes(lib.gbrmsd_rotations_workspace_bytes(n_frames, n_align), dev)
    check(lib.gbrmsd_rotations(x_align.data_ptr(), n_frames, n_align, n_padded, 3 * n_padded, _lib.ATOM_MAJOR, mode,
                               ref.ws.data_ptr(), _ptr(g_target), float(g_ref), rot.data_ptr(), _ptr(mu), None,
                               ws.data_ptr(), ws.numel(), D.stream_handle()))
    return rot, mu


# ---------------------------------------------------------------------------
# Trajectory.superpose
# ---------------------------------------------------------------------------


def superpose(traj, reference, frame=0, atom_indices=None, ref_atom_indices=None, parallel=True):
    """Superposes each conformation of ``traj`` upon frame ``frame`` of
    ``reference`` in place (the semantics of Trajectory.superpose,
    core/trajectory.py:1083-1170): every frame is centred on the centroid of
    its alignment atoms, rotated by the optimal rotation of those atoms onto
    the (centred) reference atoms, and translated onto the reference centroid.
    Returns ``traj``."""
    if atom_indices is None:
        atom_indices = slice(None)
    elif len(atom_indices) == 0:
        raise ValueError("Number of atom indices must be greater than 0")
    if ref_atom_indices is None:
        ref_atom_indices = atom_indices
    if not isinstance(ref_atom_indices, slice) and (len(ref_atom_indices) != len(atom_indices)):
        raise ValueError("Number of atoms must be consistent!")

    xyz = np.asarray(traj.xyz, order="c")
    n_frames, n_atoms = xyz.shape[0], xyz.shape[1]
    ref_align = np.array(reference.xyz[frame, ref_atom_indices, :], copy=True, order="c").reshape(1, -1, 3)
    n_align = ref_align.shape[1]
    sel = np.arange(n_atoms)[atom_indices]
    if len(sel) != n_align:
        raise ValueError("Number of atoms must be consistent!")
    ref_offset = ref_align[0].astype("float64").mean(0)
    ref_align[0] -= ref_offset
    if n_frames == 0:
        traj.xyz = xyz
        return traj

    device = D.require_device()
    stream = D.stream_handle()
    x_dev, Ap = D.frames_to_device(xyz, _lib.ATOM_MAJOR, device, stream)
    if len(sel) == n_atoms and np.array_equal(sel, np.arange(n_atoms)):
        x_align, Apa = x_dev, Ap
    else:
        idx = torch.from_numpy(sel.astype(np.int64)).to(device)
        x_align, Apa = _padded_device(x_dev.view(n_frames, Ap, 3).index_select(1, idx), n_align)
    ref = D.DeviceReference(ref_align[0], _lib.ATOM_MAJOR, centre=False, device=device)
    rot, mu = _rotations(x_align, n_frames, n_align, Apa, ref, _lib.MODE_CENTER, want_mu=True)
    flag = torch.zeros(1, dtype=torch.int32, device=device)
    off = (C.c_double * 3)(*[float(v) for v in ref_offset])
    check(lib.gbrmsd_apply_rotations(x_dev.data_ptr(), n_frames, n_atoms, 3 * Ap, rot.data_ptr(), mu.data_ptr(), off,
                                     flag.data_ptr(), stream))
    if not int(D.to_host(flag.view(torch.float32), stream).view(np.int32)[0]):
        raise OverflowError(OVERFLOW_MESSAGE)
    D.frames_to_host(x_dev, xyz, _lib.ATOM_MAJOR, n_atoms, Ap, stream)
    torch.cuda.current_stream().synchronize()
    traj.xyz = xyz
    return traj


# ---------------------------------------------------------------------------
# mdtraj._rmsd.superpose_atom_major
# ---------------------------------------------------------------------------


def superpose_atom_major(xyz_align_target, xyz_align_mobile, g_target, g_mobile, xyz_displace_mobile, target_frame,
                         parallel=True):
    """superpose_atom_major(xyz_target, xyz_mobile, g_target, g_mobile, xyz_mobile_displace)

    Rotates every frame of ``xyz_displace_mobile`` in place by the optimal
    rotation of the (pre-centred) ``xyz_align_mobile`` frame onto frame
    ``target_frame`` of ``xyz_align_target`` (_rmsd.pyx:618-674)."""
    xyz_align_target = _memview3(xyz_align_target, "xyz_align_target")
    xyz_align_mobile = _memview3(xyz_align_mobile, "xyz_align_mobile")
    g_target = _memview1(g_target, "g_target")
    g_mobile = _memview1(g_mobile, "g_mobile")
    xyz_displace_mobile = _memview3(xyz_displace_mobile, "xyz_displace_mobile")
    target_frame = int(target_frame)
    n_frames = xyz_align_mobile.shape[0]
    if not (xyz_align_target.shape[1] == xyz_align_mobile.shape[1]):
        raise ValueError("Input arrays must have same number of atoms. "
                         "found %d and %d." % (xyz_align_target.shape[1], xyz_align_mobile.shape[1]))
    if not xyz_align_mobile.shape[0] == xyz_displace_mobile.shape[0]:
        raise ValueError("xyz_align_mobile and xyz_displace_mobile must contain the same number of frames")
    if n_frames == 0:
        return
    if not (0 <= target_frame < xyz_align_target.shape[0]):
        raise IndexError("Out of bounds on buffer access (axis 0)")
    if g_mobile.shape[0] < n_frames:
        raise IndexError("Out of bounds on buffer access (axis 0)")
    n_align = xyz_align_mobile.shape[1]
    n_disp = xyz_displace_mobile.shape[1]
    device = D.require_device()
    stream = D.stream_handle()
    xa, Apa = D.frames_to_device(xyz_align_mobile, _lib.ATOM_MAJOR, device, stream)
    ref = D.DeviceReference(xyz_align_target[target_frame], _lib.ATOM_MAJOR, centre=False, device=device)
    g = torch.from_numpy(np.ascontiguousarray(g_mobile[:n_frames])).to(device)
    rot, _ = _rotations(xa, n_frames, n_align, Apa, ref, _lib.MODE_PRECENTERED, g, float(g_target[target_frame]))
    xd, Apd = D.frames_to_device(xyz_displace_mobile, _lib.ATOM_MAJOR, device, stream)
    check(lib.gbrmsd_apply_rotations(xd.data_ptr(), n_frames, n_disp, 3 * Apd, rot.data_ptr(), None, None, None,
                                     stream))
    D.frames_to_host(xd, xyz_displace_mobile, _lib.ATOM_MAJOR, n_disp, Apd, stream)
    torch.cuda.current_stream().synchronize()


# ---------------------------------------------------------------------------
# md.rmsf
# ---------------------------------------------------------------------------


def _centre_host_inplace(arr: np.ndarray, device, stream):
    """Centres float32 C-contiguous frames (F, A, 3) in place with the
    reference's rounding (inplace_center_and_trace_atom_major); returns
    (device copy of the centred frames, n_padded, float32 traces on device)."""
    F, A = arr.shape[0], arr.shape[1]
    x_dev, Ap = D.frames_to_device(arr, _lib.ATOM_MAJOR, device, stream)
    traces = D.center_inplace(x_dev, F, A, Ap, _lib.ATOM_MAJOR)
    D.frames_to_host(x_dev, arr, _lib.ATOM_MAJOR, A, Ap, stream)
    return x_dev, Ap, traces


def rmsf(target, reference, frame=0, atom_indices=None, ref_atom_indices=None, parallel=True, precentered=False,
         mode="atom"):
    """rmsf(target, reference, frame=0, atom_indices=None, parallel=True, precentered=False, mode='atom')

    Root-mean-square fluctuation of atom positions in ``target`` after
    superposing every frame onto frame ``frame`` of ``reference`` (or, with
    ``reference=None``, of the trajectory as it is).  Same arguments,
    validation, in-place centring of the target (and reference frame), and
    per-residue mode as mdtraj/rmsd/_rmsd.pyx:246-484."""
    frame = int(frame)
    trajectory_prealigned = False
    if reference is None:
        trajectory_prealigned = True
        reference = target

    atom_indices_is_none = False
    if atom_indices is None:
        atom_indices_is_none = True
        atom_indices = slice(None)
    else:
        atom_indices = ensure_type(np.asarray(atom_indices), dtype=int, ndim=1, name="atom_indices")
        if not np.all((atom_indices >= 0) * (atom_indices < target.xyz.shape[1]) *
                      (atom_indices < reference.xyz.shape[1])):
            raise ValueError("atom_indices must be valid positive indices")

    if ref_atom_indices is None:
        ref_atom_indices = atom_indices
    else:
        if len(ref_atom_indices) != len(atom_indices):
            raise ValueError("atom_indices and ref_atom_indices must have same number of atom indices. "
                             "found %d and %d." % (len(atom_indices), len(ref_atom_indices)))

    if not isinstance(ref_atom_indices, slice):
        ref_atom_indices = ensure_type(np.asarray(ref_atom_indices), dtype=int, ndim=1, name="ref_atom_indices")
        if not np.all((ref_atom_indices >= 0) * (ref_atom_indices < target.xyz.shape[1]) *
                      (ref_atom_indices < reference.xyz.shape[1])):
            raise ValueError("ref_atom_indices must be valid positive indices")

    if mode not in {"atom", "residue"}:
        raise ValueError('Mode must be one of "atom" or "residue". "%s" supplied.' % mode)

    assert (target.xyz.ndim == 3) and (reference.xyz.ndim == 3) and (target.xyz.shape[2]) == 3 and (
        reference.xyz.shape[2] == 3)
    if not ((target.xyz.shape[1] == reference.xyz.shape[1]) or (len(ref_atom_indices) == len(atom_indices))):
        raise ValueError("Input trajectories must have same number of atoms. "
                         "found %d and %d." % (target.xyz.shape[1], reference.xyz.shape[1]))
    if frame >= reference.xyz.shape[0]:
        raise ValueError("Cannot calculate RMSF of frame %d: reference has "
                         "only %d frames." % (frame, reference.xyz.shape[0]))

    n_frames = target.xyz.shape[0]
    target_xyz = np.asarray(target.xyz[:, atom_indices, :], order="C", dtype=np.float32)
    ref_xyz_frame = np.asarray(reference.xyz[frame, ref_atom_indices, :], order="C", dtype=np.float32)
    n_atoms = target_xyz.shape[1]
    _writable_view(target_xyz, "target")
    _writable_view(ref_xyz_frame, "reference")

    device = D.require_device()
    stream = D.stream_handle()
    if precentered and (reference._rmsd_traces is not None) and (target._rmsd_traces is not None) \
            and atom_indices_is_none:
        x_dev, Ap = D.frames_to_device(target_xyz, _lib.ATOM_MAJOR, device, stream)
        target_g = torch.from_numpy(np.ascontiguousarray(target._rmsd_traces, dtype=np.float32)).to(device)
        ref_g = float(np.float32(reference._rmsd_traces[frame]))
    else:
        if precentered:
            warnings.warn("in rmsd(), precentered is ignored when atom_indices != None", RuntimeWarning)
        x_dev, Ap, target_g = _centre_host_inplace(target_xyz, device, stream)
        rdev, rAp, rg = _centre_host_inplace(ref_xyz_frame.reshape(1, -1, 3), device, stream)
        ref_g = float(D.to_host(rg, stream)[0])

    if n_atoms == 0:
        return np.zeros(0, dtype=np.float32)
    # the displaced copy is taken after the centring: centred when the
    # centring went into target.xyz itself, the original coordinates otherwise
    disp_host = None
    if np.may_share_memory(target_xyz, target.xyz):
        disp, Apd = x_dev, Ap
    else:
        disp_host = np.ascontiguousarray(target.xyz[:, atom_indices, :], dtype=np.float32)  # read asynchronously
        disp, Apd = D.frames_to_device(disp_host, _lib.ATOM_MAJOR, device, stream)
    rot = None
    if not trajectory_prealigned:
        ref = D.DeviceReference(ref_xyz_frame, _lib.ATOM_MAJOR, centre=False, device=device)
        rot, _ = _rotations(x_dev, n_frames, n_atoms, Ap, ref, _lib.MODE_PRECENTERED, target_g, ref_g)
    out = torch.empty(n_atoms, dtype=torch.float32, device=device)
    ws = D.empty_bytes(lib.gbrmsd_rmsf_workspace_bytes(n_frames, n_atoms), device)
    check(lib.gbrmsd_rmsf(disp.data_ptr(), n_frames, n_atoms, 3 * Apd, _ptr(rot), out.data_ptr(), ws.data_ptr(),
                          ws.numel(), stream))
    fluctuations = D.to_host(out, stream)  # synchronises: disp_host no longer read
    del disp_host
    if mode == "atom":
        return fluctuations

    if atom_indices_is_none:
        atom_indices = np.arange(n_atoms)
    residue_indices = np.array([target.topology.atom(i).residue.index for i in atom_indices], dtype=np.int32)
    n_residues = target.topology.n_residues
    residue_fluctuations = np.zeros((n_residues,), dtype=np.float32)
    residue_masses = np.array([float(target.topology.atom(j).element.mass) for j in atom_indices], dtype=np.float32)
    residue_total_mass = np.zeros((n_residues,), dtype=np.float32)
    # the reference's float32 accumulation of the squared fluctuations
    sq = (fluctuations * fluctuations).astype(np.float32)
    for i in range(n_atoms):
        residue_fluctuations[residue_indices[i]] += np.float32(sq[i] * residue_masses[i])
        residue_total_mass[residue_indices[i]] += residue_masses[i]
    for i in range(n_residues):
        if residue_total_mass[i] > 0:
            residue_fluctuations[i] = np.sqrt(np.float32(residue_fluctuations[i] / residue_total_mass[i]))
        else:
            residue_fluctuations[i] = -1.0
    return residue_fluctuations


# ---------------------------------------------------------------------------
# mdtraj._rmsd.getMultipleAlignDisplaceRMSDs_atom_major
# ---------------------------------------------------------------------------


def getMultipleAlignDisplaceRMSDs_atom_major(xyz_align1, xyz_align2, g_align1, g_align2, xyz_displ1, xyz_displ2,
                                             n_atoms_align, n_atoms_displ, frame, parallel=True):
    """RMSD between frame ``frame`` of ``xyz_displ1`` and every frame of
    ``xyz_displ2`` after the rotation that best aligns frame ``frame`` of
    ``xyz_align1`` with each frame of ``xyz_align2`` (_rmsd.pyx:677-759).
    Returns (rmsds float32 (n_frames,), rotations float32 (n_frames, 3, 3))."""
    xyz_align1 = _memview3(xyz_align1, "xyz_align1")
    xyz_align2 = _memview3(xyz_align2, "xyz_align2")
    g_align1 = _memview1(g_align1, "g_align1")
    g_align2 = _memview1(g_align2, "g_align2")
    xyz_displ1 = _memview3(xyz_displ1, "xyz_displ1")
    xyz_displ2 = _memview3(xyz_displ2, "xyz_displ2")
    n_atoms_align, n_atoms_displ, frame = int(n_atoms_align), int(n_atoms_displ), int(frame)
    assert (xyz_align1.shape[2] == 3) and (xyz_align2.shape[2] == 3)
    assert (xyz_displ1.shape[2] == 3) and (xyz_displ2.shape[2] == 3)
    if not ((xyz_align1.shape[1] % 4 == 0) & (xyz_align2.shape[1] % 4 == 0)):
        raise ValueError("Input arrays must have middle dimension of 4*n, "
                         "found %d and %d." % (xyz_align1.shape[1], xyz_align2.shape[1]))
    if not ((xyz_displ1.shape[1] % 4 == 0) & (xyz_displ2.shape[1] % 4 == 0)):
        raise ValueError("Input arrays must have middle dimension of 4*n, "
                         "found %d and %d." % (xyz_displ1.shape[1], xyz_displ2.shape[1]))
    if not xyz_align1.shape[0] == xyz_displ1.shape[0]:
        raise ValueError("xyz_align1 and xyz_displ1 must contain the same number of frames")
    if not xyz_align2.shape[0] == xyz_displ2.shape[0]:
        raise ValueError("xyz_align2 and xyz_displ2 must contain the same number of frames")
    if frame >= xyz_align1.shape[0]:
        raise ValueError("Cannot calculate RMSD of frame %d: xyz1 has "
                         "only %d frames." % (frame, xyz_align1.shape[0]))
    n_frames = xyz_align2.shape[0]
    if n_frames == 0:
        return np.zeros(0, dtype=np.float32), np.zeros((0, 3, 3), dtype=np.float32)
    if not (0 < n_atoms_align <= xyz_align2.shape[1] and 0 <= n_atoms_displ <= xyz_displ2.shape[1]):
        raise ValueError("n_atoms_align / n_atoms_displ exceed the padded atom dimension")
    device = D.require_device()
    stream = D.stream_handle()
    Apa = xyz_align2.shape[1]
    xa = torch.from_numpy(xyz_align2.reshape(n_frames, -1)).to(device)
    # frames streamed, reference = align1[frame]: the rotation aligns each frame
    # onto the reference frame, which is the reference's own `rot` array for
    # its (reference frame, frame) call order
    ref = D.DeviceReference(xyz_align1[frame, :n_atoms_align], _lib.ATOM_MAJOR, centre=False, device=device)
    g = torch.from_numpy(np.ascontiguousarray(g_align2[:n_frames])).to(device)
    rot, _ = _rotations(xa, n_frames, n_atoms_align, Apa, ref, _lib.MODE_PRECENTERED, g, float(g_align1[frame]))
    xd = torch.from_numpy(xyz_displ2.reshape(n_frames, -1)).to(device)
    refd = torch.from_numpy(np.ascontiguousarray(xyz_displ1[frame, :n_atoms_displ]).reshape(-1)).to(device)
    out = torch.empty(n_frames, dtype=torch.float32, device=device)
    check(lib.gbrmsd_rotated_rmsd(xd.data_ptr(), n_frames, n_atoms_displ, 3 * xyz_displ2.shape[1], rot.data_ptr(),
                                  refd.data_ptr() if refd.numel() else None, out.data_ptr(), stream))
    return D.to_host(out, stream), D.to_host(rot, stream).reshape(n_frames, 3, 3)
