"""mdtraj_gb300 — GB300-native RMSD hot path of mdtraj.

Drop-in entry points (same signatures and semantics as mdtraj):

    from mdtraj_gb300 import rmsd            # md.rmsd
    from mdtraj_gb300 import _rmsd           # mdtraj._rmsd axis/atom-major entry points
    from mdtraj_gb300 import rmsf            # md.rmsf
    from mdtraj_gb300 import Trajectory      # .xyz / ._rmsd_traces / center_coordinates / superpose

All per-frame work runs in libgbrmsd.so (hand-written sm_103a CUDA behind a
C ABI, include/gbrmsd.h) called through ctypes; PyTorch only owns device
buffers and streams.  There is no CPU fallback.
"""
from . import _lib  # loads libgbrmsd.so (raises ImportError if it was not built)
from . import _rmsd
from ._rmsd import rmsd, rmsf
from .allpairs import allpairs_rmsd
from .ragged import RaggedBatch, ragged_rmsd
from .trajectory import Trajectory

__all__ = ["rmsd", "rmsf", "allpairs_rmsd", "ragged_rmsd", "RaggedBatch", "Trajectory", "_rmsd"]
__version__ = "0.1.0"
