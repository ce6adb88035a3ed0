"""ORACLE — test infrastructure only (never used by mdtraj_gb300/).

FP64 restatement of mdtraj's Kabsch RMSD, mdtraj/geometry/alignment.py:117-181:
both structures are centred in float64, the optimal rotation comes from the
SVD of the correlation matrix with the reflection fix (:151-156), and the
RMSD is the direct residual of the transformed structure (:178-181).
Vectorised over frames; inputs are promoted from float32 to float64 exactly.
"""
from __future__ import annotations

import numpy as np


def kabsch_rmsd(frames: np.ndarray, ref: np.ndarray, chunk: int = 4096) -> np.ndarray:
    """RMSD (nm, float64) of each frame (F, A, 3) to ref (A, 3), atom-major."""
    frames = np.asarray(frames)
    ref64 = np.asarray(ref, dtype=np.float64)
    F, A = frames.shape[0], frames.shape[1]
    out = np.empty(F, dtype=np.float64)
    if A == 0:
        out[:] = 0.0
        return out
    b = ref64 - ref64.mean(0)
    for s in range(0, F, chunk):
        a = frames[s:s + chunk].astype(np.float64)
        a = a - a.mean(1, keepdims=True)
        corr = np.einsum("fki,kj->fij", a, b)              # mobile^T target
        V, S, Wt = np.linalg.svd(corr)
        refl = np.linalg.det(V) * np.linalg.det(Wt) < 0.0
        V[refl, :, -1] *= -1.0
        rot = V @ Wt                                        # mobile @ rot ~ target
        delta = np.einsum("fki,fij->fkj", a, rot) - b
        out[s:s + chunk] = np.sqrt((delta * delta).sum(axis=(1, 2)) / A)
    return out


def kabsch_rmsd_pairs(frames: np.ndarray, pairs: np.ndarray, chunk: int = 4096) -> np.ndarray:
    """RMSD of frames[i] to frames[j] for each row (i, j) of `pairs`."""
    frames = np.asarray(frames)
    pairs = np.asarray(pairs)
    out = np.empty(len(pairs), dtype=np.float64)
    A = frames.shape[1]
    for s in range(0, len(pairs), chunk):
        p = pairs[s:s + chunk]
        a = frames[p[:, 0]].astype(np.float64)
        b = frames[p[:, 1]].astype(np.float64)
        a = a - a.mean(1, keepdims=True)
        b = b - b.mean(1, keepdims=True)
        corr = np.einsum("fki,fkj->fij", a, b)
        V, S, Wt = np.linalg.svd(corr)
        refl = np.linalg.det(V) * np.linalg.det(Wt) < 0.0
        V[refl, :, -1] *= -1.0
        rot = V @ Wt
        delta = np.einsum("fki,fij->fkj", a, rot) - b
        out[s:s + chunk] = np.sqrt((delta * delta).sum(axis=(1, 2)) / A)
    return out


def msd_nosuperpose(frames: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """sqrt(mean |a - b|^2) in float64, no centring or rotation
    (mdtraj/rmsd/_rmsd.pyx:762-793)."""
    d = np.asarray(frames, dtype=np.float64) - np.asarray(ref, dtype=np.float64)[None]
    return np.sqrt((d * d).sum(axis=(1, 2)) / max(frames.shape[1], 1))
