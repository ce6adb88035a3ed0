"""Minimal trajectory container carrying the RMSD contract of
mdtraj.Trajectory (mdtraj/core/trajectory.py): float32 C-contiguous ``xyz``
whose setter drops cached traces (:1010-1029), ``_rmsd_traces`` filled by
``center_coordinates`` (:2114-2137) and carried through frame slicing
(:1325-1361).  Topology handling is out of scope; ``topology`` is stored
as given and only read for the atom masses of mass-weighted centring."""
from __future__ import annotations

import numpy as np

from .utils import ensure_type


class Trajectory:
    """Coordinates (nm) of ``n_frames`` conformations of ``n_atoms`` atoms."""

    def __init__(self, xyz, topology=None):
        self.topology = topology
        self.xyz = xyz
        # inner products of each centred conformation, set by center_coordinates
        self._rmsd_traces = None

    @property
    def top(self):
        return self.topology

    @property
    def xyz(self) -> np.ndarray:
        return self._xyz

    @xyz.setter
    def xyz(self, value):
        n_atoms = getattr(self.topology, "n_atoms", None) if self.topology is not None else None
        shape = (None, n_atoms, 3)
        value = ensure_type(value, np.float32, 3, "xyz", shape=shape, warn_on_cast=False,
                            add_newaxis_on_deficient_ndim=True)
        self._xyz = value
        self._rmsd_traces = None

    @property
    def n_frames(self) -> int:
        return int(self._xyz.shape[0])

    @property
    def n_atoms(self) -> int:
        return int(self._xyz.shape[1])

    def __len__(self) -> int:
        return self.n_frames

    def __getitem__(self, key):
        return self.slice(key)

    def slice(self, key, copy=True):
        xyz = self.xyz[key]
        if copy:
            xyz = xyz.copy()
        out = Trajectory(xyz, self.topology)
        if self._rmsd_traces is not None:
            traces = np.asarray(self._rmsd_traces)[key]
            out._rmsd_traces = np.array(traces, copy=True, ndmin=1)
        return out

    def center_coordinates(self, mass_weighted=False):
        """Centres each frame at the origin in place
        (core/trajectory.py:2114-2137).  Uniform weights cache the traces
        used by ``rmsd(..., precentered=True)``; with ``mass_weighted`` and a
        topology, each frame's centre of mass (masses ``atom.element.mass``
        of ``topology.atoms``, normalised to sum 1) is subtracted instead and
        the cached traces are dropped, as the reference's assignment to
        ``xyz`` drops them."""
        from ._rmsd import _center_inplace_atom_major, _center_weighted_inplace_atom_major

        if mass_weighted and self.topology is not None:
            masses = np.array([a.element.mass for a in self.topology.atoms])
            masses /= masses.sum()
            _center_weighted_inplace_atom_major(self._xyz, masses)
            self.xyz = self._xyz
        else:
            self._rmsd_traces = _center_inplace_atom_major(self._xyz)
        return self

    def superpose(self, reference, frame=0, atom_indices=None, ref_atom_indices=None, parallel=True):
        """Superposes each conformation upon frame ``frame`` of ``reference``
        in place (core/trajectory.py:1083-1170); returns self."""
        from .superpose import superpose

        return superpose(self, reference, frame, atom_indices, ref_atom_indices, parallel)
