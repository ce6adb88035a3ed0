"""Drop-in replacement for the RMSD entry points of mdtraj._rmsd
(mdtraj/rmsd/_rmsd.pyx), backed by libgbrmsd on one GB300.

Same names, arguments, return values, warnings and exceptions as the
reference; the per-frame work runs in the CUDA library:

* ``rmsd``                          -> _rmsd.pyx:64-243
* ``getMultipleRMSDs_axis_major``   -> _rmsd.pyx:500-557
* ``getMultipleRMSDs_atom_major``   -> _rmsd.pyx:560-615
* ``_center_inplace_atom_major``    -> _rmsd.pyx:487-491

``parallel`` is accepted everywhere and has no effect (the reference uses it
to pick OpenMP vs a serial loop).  Results are float32 arrays on the host.
"""
from __future__ import annotations

import warnings

import numpy as np
import torch

from . import _device as D
from . import _lib
from ._lib import check, lib
from .utils import ensure_type

__all__ = [
    "rmsd",
    "getMultipleRMSDs_axis_major",
    "getMultipleRMSDs_atom_major",
    "_center_inplace_atom_major",
]


def _writable_view(arr: np.ndarray, what: str) -> None:
    # The reference binds these arrays to non-const Cython memoryviews, which
    # refuse read-only buffers with ValueError (tests/test_rmsd_memmap.py).
    if not arr.flags.writeable:
        raise ValueError(f"buffer source array is read-only ({what})")


def _alias_index(frames: np.ndarray, one: np.ndarray) -> int:
    """Index i with frames[i] starting at the same address as `one` (the
    reference's pointer-equality shortcut), or -1."""
    if frames.size == 0 or one.size == 0 or not np.may_share_memory(frames, one):
        return -1
    stride = frames.strides[0]
    off = one.ctypes.data - frames.ctypes.data
    if stride <= 0 or off < 0 or off % stride:
        return -1
    i = off // stride
    return int(i) if i < frames.shape[0] else -1


def _memview3(x, name: str) -> np.ndarray:
    """Coercion of a `float[:, :, ::1] not None` Cython argument."""
    if x is None:
        raise TypeError(f"Argument '{name}' must not be None")
    a = np.asarray(x)
    if a.dtype != np.float32:
        raise ValueError(f"Buffer dtype mismatch, expected 'float' but got '{a.dtype}'")
    if a.ndim != 3:
        raise ValueError(f"Buffer has wrong number of dimensions (expected 3, got {a.ndim})")
    if not a.flags.c_contiguous:
        raise ValueError("ndarray is not C-contiguous")
    _writable_view(a, name)
    return a


def _memview1(x, name: str) -> np.ndarray:
    if x is None:
        raise TypeError(f"Argument '{name}' must not be None")
    a = np.asarray(x)
    if a.dtype != np.float32:
        raise ValueError(f"Buffer dtype mismatch, expected 'float' but got '{a.dtype}'")
    if a.ndim != 1:
        raise ValueError(f"Buffer has wrong number of dimensions (expected 1, got {a.ndim})")
    if not a.flags.c_contiguous:
        raise ValueError("ndarray is not C-contiguous")
    return a


def rmsd(target, reference, frame=0, atom_indices=None, ref_atom_indices=None, parallel=True,
         precentered=False, superpose=True):
    """rmsd(target, reference, frame=0, atom_indices=None, ref_atom_indices=None,
            parallel=True, precentered=False, superpose=True)

    Compute RMSD of all conformations in target to a reference conformation.
    Note, this will center the conformations in place (exactly when the
    reference implementation would: float32 C-contiguous coordinates and
    ``atom_indices`` None).

    target, reference : objects with ``.xyz`` (n_frames, n_atoms, 3) and
        ``._rmsd_traces`` (e.g. mdtraj.Trajectory or mdtraj_gb300.Trajectory).
    Returns np.ndarray float32, shape (target.n_frames,).
    """
    frame = int(frame)
    atom_indices_is_none = False
    if atom_indices is None:
        atom_indices_is_none = True
        atom_indices = slice(None)
    else:
        atom_indices = ensure_type(np.asarray(atom_indices), dtype=int, ndim=1, name="atom_indices")
        if not np.all((atom_indices >= 0) * (atom_indices < target.xyz.shape[1])):
            raise ValueError("atom_indices must be valid positive indices")

    if ref_atom_indices is None:
        ref_atom_indices = atom_indices
    else:
        if len(ref_atom_indices) != len(atom_indices):
            raise ValueError(
                "atom_indices and ref_atom_indices must have same number of atom indices. "
                "found %d and %d." % (len(atom_indices), len(ref_atom_indices))
            )

    if not isinstance(ref_atom_indices, slice):
        ref_atom_indices = ensure_type(np.asarray(ref_atom_indices), dtype=int, ndim=1, name="ref_atom_indices")
        if not np.all((ref_atom_indices >= 0) * (ref_atom_indices < reference.xyz.shape[1])):
            raise ValueError("ref_atom_indices must be valid positive indices")

    assert (target.xyz.ndim == 3) and (reference.xyz.ndim == 3) and (target.xyz.shape[2] == 3) and (
        reference.xyz.shape[2] == 3
    )
    if not ((target.xyz.shape[1] == reference.xyz.shape[1]) or (len(ref_atom_indices) == len(atom_indices))):
        raise ValueError(
            "Input trajectories must have same number of atoms. "
            "found %d and %d." % (target.xyz.shape[1], reference.xyz.shape[1])
        )
    if frame >= reference.xyz.shape[0]:
        raise ValueError(
            "Cannot calculate RMSD of frame %d: reference has only %d frames." % (frame, reference.xyz.shape[0])
        )

    n_frames = target.xyz.shape[0]
    target_xyz = np.asarray(target.xyz[:, atom_indices, :], order="C", dtype=np.float32)
    ref_xyz_frame = np.asarray(reference.xyz[frame, ref_atom_indices, :], order="C", dtype=np.float32)
    _writable_view(target_xyz, "target")
    _writable_view(ref_xyz_frame, "reference")
    n_atoms = target_xyz.shape[1]
    if ref_xyz_frame.shape[0] != n_atoms:
        raise ValueError("Input trajectories must have same number of atoms. "
                         "found %d and %d." % (n_atoms, ref_xyz_frame.shape[0]))
    if n_frames == 0:
        return np.zeros(0, dtype=np.float32)

    # Mode selection and its warnings come first, as in the reference.
    if superpose:
        use_traces = (precentered and (reference._rmsd_traces is not None)
                      and (target._rmsd_traces is not None) and atom_indices_is_none)
        if not use_traces and precentered:
            warnings.warn("in rmsd(), precentered is ignored when atom_indices != None", RuntimeWarning)
        mode = _lib.MODE_PRECENTERED if use_traces else _lib.MODE_CENTER
    else:
        if precentered:
            warnings.warn("in rmsd(), precentered is ignored when superpose=False", RuntimeWarning)
        mode = _lib.MODE_NOSUPERPOSE

    device = D.require_device()
    self_index = _alias_index(target_xyz, ref_xyz_frame)

    if mode == _lib.MODE_PRECENTERED:
        target_g = np.ascontiguousarray(target._rmsd_traces, dtype=np.float32)
        ref_g = np.float32(reference._rmsd_traces[frame])
        ref = D.DeviceReference(ref_xyz_frame, _lib.ATOM_MAJOR, centre=False, device=device)
        return D.rmsd_host_frames(target_xyz, ref, _lib.MODE_PRECENTERED, g_target=target_g[:n_frames],
                                  g_ref=float(ref_g), self_index=self_index)

    if mode == _lib.MODE_CENTER:
        ref = D.DeviceReference(ref_xyz_frame, _lib.ATOM_MAJOR, centre=True, device=device)
        # the reference centres target.xyz in place when it is a view of it
        mutate_target = n_atoms > 0 and np.may_share_memory(target_xyz, target.xyz)
        mutate_ref = n_atoms > 0 and np.may_share_memory(ref_xyz_frame, reference.xyz)
        result = D.rmsd_host_frames(target_xyz, ref, _lib.MODE_CENTER, self_index=self_index,
                                    write_centred=mutate_target)
        if mutate_ref:
            _centre_frame_like_reference(ref_xyz_frame, ref)
        return result

    ref = D.DeviceReference(ref_xyz_frame, _lib.ATOM_MAJOR, centre=False, device=device)
    return D.rmsd_host_frames(target_xyz, ref, _lib.MODE_NOSUPERPOSE)


def _centre_frame_like_reference(frame_xyz: np.ndarray, ref: D.DeviceReference) -> None:
    """In-place centring of the (host) reference frame, as the reference does
    at _rmsd.pyx:213: mean accumulated in double, rounded to float,
    subtracted in float.  When the frame aliases the (already centred)
    target this is the reference's second, tiny centring of that frame."""
    mu = (frame_xyz.astype(np.float64).sum(axis=0) / frame_xyz.shape[0]).astype(np.float32)
    frame_xyz -= mu


def _multiple(xyz1, xyz2, g1, g2, frame, layout):
    xyz1 = _memview3(xyz1, "xyz1")
    xyz2 = _memview3(xyz2, "xyz2")
    g1 = _memview1(g1, "g1")
    g2 = _memview1(g2, "g2")
    frame = int(frame)
    n_frames = xyz2.shape[0]
    atoms_axis = 2 if layout == _lib.AXIS_MAJOR else 1
    dim_axis = 1 if layout == _lib.AXIS_MAJOR else 2
    n_atoms = xyz1.shape[atoms_axis]
    assert xyz1.ndim == 3 and xyz2.ndim == 3 and xyz1.shape[dim_axis] == 3 and xyz2.shape[dim_axis] == 3
    if not (xyz1.shape[atoms_axis] == xyz2.shape[atoms_axis]):
        raise ValueError("Input arrays must have same number of atoms. "
                         "found %d and %d." % (xyz1.shape[atoms_axis], xyz2.shape[atoms_axis]))
    if frame >= xyz1.shape[0]:
        raise ValueError("Cannot calculate RMSD of frame %d: xyz1 has only %d frames." % (frame, xyz1.shape[0]))
    if n_frames == 0:
        return np.zeros(0, dtype=np.float32)
    if g2.shape[0] < n_frames:
        raise IndexError("Out of bounds on buffer access (axis 0)")
    device = D.require_device()
    stream = D.stream_handle()
    ref_frame = xyz1[frame]
    ref_atom_major = ref_frame.T if layout == _lib.AXIS_MAJOR else ref_frame
    ref = D.DeviceReference(np.ascontiguousarray(ref_atom_major), layout, centre=False, device=device)
    x_dev, n_padded = D.frames_to_device(xyz2, layout, device, stream)
    g_dev = torch.from_numpy(np.ascontiguousarray(g2[:n_frames])).to(device)
    self_index = _alias_index(xyz2, ref_frame)
    out = torch.empty(n_frames, dtype=torch.float32, device=device)
    ws = D.empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(n_frames, n_atoms), device)
    D.rmsd_to_reference(x_dev, n_frames, n_atoms, n_padded, layout, _lib.MODE_PRECENTERED, ref,
                        g_target=g_dev, g_ref=float(g1[frame]), self_index=self_index, out=out, ws=ws)
    result = D.to_host(out, stream)
    word = _lib.C.c_int32(0)
    check(lib.gbrmsd_workspace_error_word(ws.data_ptr(), _lib.C.addressof(word), stream))
    D.raise_on_error_word(word.value, "getMultipleRMSDs")
    return result


def getMultipleRMSDs_axis_major(xyz1, xyz2, g1, g2, frame, parallel=True):
    """getMultipleRMSDs_axis_major(xyz1, xyz2, g1, g2, frame, parallel=True)

    RMSD of xyz1[frame] to every frame of xyz2, coordinates laid out axis-major
    (n_frames, 3, n_atoms), pre-centred, with traces g1, g2 supplied.
    Returns float32 (len(xyz2),).
    """
    return _multiple(xyz1, xyz2, g1, g2, frame, _lib.AXIS_MAJOR)


def getMultipleRMSDs_atom_major(xyz1, xyz2, g1, g2, frame, parallel=True):
    """getMultipleRMSDs_atom_major(xyz1, xyz2, g1, g2, frame, parallel=True)

    Same as getMultipleRMSDs_axis_major for atom-major (n_frames, n_atoms, 3).
    """
    return _multiple(xyz1, xyz2, g1, g2, frame, _lib.ATOM_MAJOR)


def _center_inplace_atom_major(xyz):
    """Centres every frame of a float32 C-contiguous (n_frames, n_atoms, 3)
    array in place and returns the float32 traces (sum of squared centred
    coordinates per frame)."""
    xyz = _memview3(xyz, "xyz")
    assert xyz.shape[2] == 3
    n_frames, n_atoms = xyz.shape[0], xyz.shape[1]
    if n_frames == 0:
        return np.zeros(0, dtype=np.float32)
    device = D.require_device()
    stream = D.stream_handle()
    x_dev, n_padded = D.frames_to_device(xyz, _lib.ATOM_MAJOR, device, stream)
    traces = D.center_inplace(x_dev, n_frames, n_atoms, n_padded, _lib.ATOM_MAJOR)
    D.frames_to_host(x_dev, xyz, _lib.ATOM_MAJOR, n_atoms, n_padded, stream)
    return D.to_host(traces, stream)


def _center_weighted_inplace_atom_major(xyz, weights) -> None:
    """Subtracts each frame's weighted centre sum_k w_k x_k from a float32
    C-contiguous (n_frames, n_atoms, 3) array in place: the work of
    ``xyz -= compute_center_of_mass(traj)[:, None, :]`` in
    Trajectory.center_coordinates(mass_weighted=True)
    (mdtraj/core/trajectory.py:2133-2134; mdtraj/geometry/distance.py:366-384),
    with ``weights`` the masses already normalised to sum 1."""
    xyz = _memview3(xyz, "xyz")
    assert xyz.shape[2] == 3
    n_frames, n_atoms = xyz.shape[0], xyz.shape[1]
    w = np.ascontiguousarray(weights, dtype=np.float64)
    if w.shape != (n_atoms,):
        raise ValueError(f"weights must have shape ({n_atoms},), got {w.shape}")
    if n_frames == 0 or n_atoms == 0:
        return
    device = D.require_device()
    stream = D.stream_handle()
    x_dev, n_padded = D.frames_to_device(xyz, _lib.ATOM_MAJOR, device, stream)
    w_dev = torch.from_numpy(w).to(device)
    check(lib.gbrmsd_center_weighted_inplace(x_dev.data_ptr(), n_frames, n_atoms, 3 * n_padded, w_dev.data_ptr(),
                                             None, stream))
    D.frames_to_host(x_dev, xyz, _lib.ATOM_MAJOR, n_atoms, n_padded, stream)
    torch.cuda.current_stream().synchronize()


# superposition entry points of the same module (_rmsd.pyx:246-759); imported
# last because they use the argument coercions above
from .superpose import getMultipleAlignDisplaceRMSDs_atom_major, rmsf, superpose_atom_major  # noqa: E402,F401
