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


def kabsch_rotations(frames: np.ndarray, ref: np.ndarray, centre: bool = True) -> np.ndarray:
    """Optimal rotations R (F, 3, 3), float64, with R (a - mean a) the frame
    aligned onto (ref - mean ref) (alignment.py:117-181 with the reflection
    fix).  centre=False uses the coordinates as given."""
    a = np.asarray(frames, dtype=np.float64)
    b = np.asarray(ref, dtype=np.float64)
    if centre:
        a = a - a.mean(1, keepdims=True)
        b = b - b.mean(0)
    corr = np.einsum("fki,kj->fij", a, b)                  # sum a b^T
    V, S, Wt = np.linalg.svd(corr)
    d = np.sign(np.linalg.det(V) * np.linalg.det(Wt))
    D = np.repeat(np.eye(3)[None], a.shape[0], 0)
    D[:, 2, 2] = d
    # maximise tr(R corr): R = W D V^T
    return np.einsum("fji,fjk,flk->fil", Wt, D, V)


def superpose(frames: np.ndarray, ref_frame: np.ndarray, align=None, ref_align=None) -> np.ndarray:
    """FP64 Trajectory.superpose (core/trajectory.py:1083-1170): every frame
    centred on the centroid of its alignment atoms, rotated onto the centred
    reference alignment atoms, translated onto the reference centroid."""
    x = np.asarray(frames, dtype=np.float64)
    ai = slice(None) if align is None else align
    ri = ai if ref_align is None else ref_align
    xa = x[:, ai]
    r = np.asarray(ref_frame, dtype=np.float64)[ri]
    mu = xa.mean(1, keepdims=True)
    rmu = r.mean(0)
    R = kabsch_rotations(xa - mu, r - rmu, centre=False)
    return np.einsum("fij,fkj->fki", R, x - mu) + rmu


def rmsf(target: np.ndarray, ref_frame: np.ndarray | None, atom_indices=None, ref_atom_indices=None) -> np.ndarray:
    """FP64 rmsf following the reference's data flow (_rmsd.pyx:246-484):
    rotations from the centred selection onto the centred reference frame; they
    are applied about the origin to the centred selection when atom_indices is
    None, to the original (uncentred) selection otherwise; ref_frame None
    means no rotation; the reference frame is restricted to ref_atom_indices
    (default atom_indices).  Then the per-atom RMS deviation from the mean."""
    x = np.asarray(target, dtype=np.float64)
    sel = x if atom_indices is None else x[:, atom_indices]
    c = sel - sel.mean(1, keepdims=True)
    disp = c if atom_indices is None else sel
    if ref_frame is not None:
        r = np.asarray(ref_frame, dtype=np.float64)
        ri = atom_indices if ref_atom_indices is None else ref_atom_indices
        if ri is not None:
            r = r[ri]
        R = kabsch_rotations(c, r - r.mean(0), centre=False)
        disp = np.einsum("fij,fkj->fki", R, disp)
    mean = disp.mean(0)
    return np.sqrt(((disp - mean) ** 2).sum(2).mean(0))


def align_displace(align_ref: np.ndarray, align: np.ndarray, displ_ref: np.ndarray, displ: np.ndarray):
    """FP64 getMultipleAlignDisplaceRMSDs_atom_major (_rmsd.pyx:677-759) on the
    real atoms: R aligns each frame's (pre-centred) alignment atoms onto the
    reference frame's, rmsd = sqrt(mean |R displ_k - displ_ref_k|^2).  Returns
    (rmsd (F,), R (F, 3, 3))."""
    R = kabsch_rotations(align, align_ref, centre=False)
    d = np.einsum("fij,fkj->fki", R, np.asarray(displ, dtype=np.float64)) - np.asarray(displ_ref, dtype=np.float64)
    n = max(displ.shape[1], 1)
    return np.sqrt((d * d).sum((1, 2)) / n), R


def center_of_mass_inplace(xyz: np.ndarray, masses: np.ndarray) -> np.ndarray:
    """Trajectory.center_coordinates(mass_weighted=True) restated: masses
    normalised to sum 1 (mdtraj/geometry/distance.py:369-370), each frame's
    centre of mass as a float64 dot product (:382-384), subtracted from the
    float32 coordinates through numpy's float64 loop
    (mdtraj/core/trajectory.py:2133-2134).  Modifies `xyz` in place and
    returns the (F, 3) centres."""
    w = np.array(masses, dtype=np.float64)
    w /= w.sum()
    com = np.empty((xyz.shape[0], 3))
    for i, x in enumerate(xyz):
        com[i, :] = x.astype("float64").T.dot(w)
    with np.errstate(invalid="ignore"):
        xyz -= com[:, np.newaxis, :]
    return com
