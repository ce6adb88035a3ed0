"""Seeded synthetic trajectories with the shapes and value distributions of
the benchmark workloads (there is no dataset: every input is generated).

Single reference (md.rmsd workloads):
    reference = n_atoms points i.i.d. uniform in a `cube` nm cube;
    frame i   = R_i (reference + N(0, sigma_i^2)) + t_i,
    R_i a Haar-random rotation (normalised Gaussian quaternion), t_i uniform
    in [-translate, translate]^3; frame 0 is the reference itself.

Host generators return numpy float32 atom-major arrays (small sizes, tests);
device generators fill torch CUDA tensors chunk by chunk (benchmark sizes).
"""
from __future__ import annotations

import math

import numpy as np


def _rot_from_quat_np(q: np.ndarray) -> np.ndarray:
    q = q / np.linalg.norm(q, axis=-1, keepdims=True)
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    r = np.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y),
    ], axis=-1)
    return r.reshape(q.shape[:-1] + (3, 3))


def haar_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    """n uniformly random rotation matrices (n, 3, 3), float64."""
    return _rot_from_quat_np(rng.normal(size=(n, 4)))


def single_reference_frames(n_frames: int, n_atoms: int, seed: int = 0, sigma=0.05, cube: float = 4.0,
                            translate: float = 2.0, exact_fraction: float = 0.0):
    """(reference (A, 3), frames (F, A, 3)) float32; frames[0] == reference.

    sigma: scalar or per-frame array of noise standard deviations (nm).
    exact_fraction: fraction of frames (chosen at random, excluding 0) that
    are exact rotated + translated copies (sigma forced to 0).
    """
    rng = np.random.default_rng(seed)
    ref = rng.uniform(0.0, cube, size=(n_atoms, 3))
    sig = np.broadcast_to(np.asarray(sigma, dtype=np.float64), (n_frames,)).copy()
    if exact_fraction > 0 and n_frames > 1:
        k = max(1, int(round(exact_fraction * n_frames)))
        sig[rng.choice(np.arange(1, n_frames), size=min(k, n_frames - 1), replace=False)] = 0.0
    rot = haar_rotations(n_frames, rng)
    t = rng.uniform(-translate, translate, size=(n_frames, 1, 3))
    noise = rng.normal(size=(n_frames, n_atoms, 3)) * sig[:, None, None]
    frames = np.einsum("fkj,fij->fki", ref[None] + noise, rot) + t
    frames[0] = ref
    return ref.astype(np.float32), np.ascontiguousarray(frames, dtype=np.float32)


def log_uniform(rng: np.random.Generator, lo: float, hi: float, size) -> np.ndarray:
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size=size))


# ---------------------------------------------------------------------------
# Device generators (torch, CUDA)
# ---------------------------------------------------------------------------


def _torch_rot_from_quat(q):
    import torch

    q = q / q.norm(dim=-1, keepdim=True)
    w, x, y, z = q.unbind(-1)
    r = torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y),
    ], dim=-1)
    return r.reshape(q.shape[:-1] + (3, 3))


def device_single_reference(n_frames: int, n_atoms: int, n_padded: int, layout: int, seed: int, device,
                            sigma_lo: float = 0.05, sigma_hi: float = 0.05, exact_fraction: float = 0.0,
                            cube: float = 4.0, translate: float = 2.0, chunk: int = 2048, out=None):
    """Fills a padded device buffer (new, or `out`) with single-reference frames.

    layout 0: (F, n_padded * 3) atom-major; layout 1: (F, 3, n_padded)
    axis-major.  sigma is log-uniform in [sigma_lo, sigma_hi] per frame;
    `exact_fraction` of the frames are exact copies.  Returns
    (reference float32 (A, 3) on device, frames tensor, per-frame sigma on
    host).  Padding atoms are zero.
    """
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    rng = np.random.default_rng(seed)
    ref = torch.rand((n_atoms, 3), generator=g, device=device, dtype=torch.float64) * cube
    if sigma_lo == sigma_hi:
        sig = np.full(n_frames, sigma_lo)
    else:
        sig = log_uniform(rng, sigma_lo, sigma_hi, n_frames)
    if exact_fraction > 0 and n_frames > 1:
        k = max(1, int(round(exact_fraction * n_frames)))
        sig[rng.choice(np.arange(1, n_frames), size=min(k, n_frames - 1), replace=False)] = 0.0
    if out is None:
        if layout == 0:
            out = torch.zeros((n_frames, n_padded * 3), dtype=torch.float32, device=device)
        else:
            out = torch.zeros((n_frames, 3, n_padded), dtype=torch.float32, device=device)
    else:
        out.zero_()
    sig_t = torch.from_numpy(sig).to(device)
    for s in range(0, n_frames, chunk):
        e = min(n_frames, s + chunk)
        n = e - s
        q = torch.randn((n, 4), generator=g, device=device, dtype=torch.float64)
        rot = _torch_rot_from_quat(q)
        t = (torch.rand((n, 1, 3), generator=g, device=device, dtype=torch.float64) * 2 - 1) * translate
        noise = torch.randn((n, n_atoms, 3), generator=g, device=device, dtype=torch.float64)
        noise *= sig_t[s:e, None, None]
        fr = torch.einsum("fkj,fij->fki", ref[None] + noise, rot) + t
        if s == 0:
            fr[0] = ref
        fr = fr.to(torch.float32)
        if layout == 0:
            out[s:e].view(n, n_padded, 3)[:, :n_atoms, :] = fr
        else:
            out[s:e, :, :n_atoms] = fr.transpose(1, 2)
        del fr, noise
    return ref.to(torch.float32), out, sig


def metastable_walk(n_frames: int, n_atoms: int, n_centres: int = 50, seed: int = 0, sigma: float = 0.1,
                    cube: float = 5.0, stay: float = 0.99):
    """All-pairs workload: a seeded Markov random walk over `n_centres`
    metastable structures (atoms uniform in a `cube` nm cube); frame =
    R (centre + N(0, sigma^2)), R Haar-random.  Returns (labels, frames)
    with frames float32 (F, A, 3)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, cube, size=(n_centres, n_atoms, 3))
    labels = np.empty(n_frames, dtype=np.int64)
    s = int(rng.integers(n_centres))
    for f in range(n_frames):
        if rng.random() > stay:
            s = int(rng.integers(n_centres))
        labels[f] = s
    frames = np.empty((n_frames, n_atoms, 3), dtype=np.float32)
    for s0 in range(0, n_frames, 1024):
        e = min(n_frames, s0 + 1024)
        rot = haar_rotations(e - s0, rng)
        pts = centres[labels[s0:e]] + rng.normal(size=(e - s0, n_atoms, 3)) * sigma
        frames[s0:e] = np.einsum("fkj,fij->fki", pts, rot)
    return labels, frames


def device_metastable_walk(n_frames: int, n_atoms: int, n_padded: int, seed: int, device, n_centres: int = 50,
                           sigma: float = 0.1, cube: float = 5.0, stay: float = 0.99, chunk: int = 1024):
    """Device version of metastable_walk into a padded atom-major buffer
    (F, n_padded * 3); padding atoms are zero."""
    import torch

    rng = np.random.default_rng(seed)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    centres = torch.rand((n_centres, n_atoms, 3), generator=g, device=device, dtype=torch.float64) * cube
    labels = np.empty(n_frames, dtype=np.int64)
    s = int(rng.integers(n_centres))
    for f in range(n_frames):
        if rng.random() > stay:
            s = int(rng.integers(n_centres))
        labels[f] = s
    lab = torch.from_numpy(labels).to(device)
    out = torch.zeros((n_frames, n_padded * 3), dtype=torch.float32, device=device)
    for s0 in range(0, n_frames, chunk):
        e = min(n_frames, s0 + chunk)
        q = torch.randn((e - s0, 4), generator=g, device=device, dtype=torch.float64)
        rot = _torch_rot_from_quat(q)
        pts = centres[lab[s0:e]] + torch.randn((e - s0, n_atoms, 3), generator=g, device=device,
                                               dtype=torch.float64) * sigma
        fr = torch.einsum("fkj,fij->fki", pts, rot).to(torch.float32)
        out[s0:e].view(e - s0, n_padded, 3)[:, :n_atoms, :] = fr
    return labels, out


def ragged_shapes(n_seg: int = 512, seed: int = 0, atoms=(50, 20000), frames=(100, 5000)):
    """Segment shapes of the ragged workload: atom counts log-uniform integers
    in `atoms`, frame counts uniform integers in `frames` (inclusive)."""
    rng = np.random.default_rng(seed)
    a = np.rint(np.exp(rng.uniform(math.log(atoms[0]), math.log(atoms[1]), n_seg))).astype(np.int32)
    f = rng.integers(frames[0], frames[1] + 1, n_seg).astype(np.int64)
    return a, f


def gaussian_chain(n_frames: int, n_atoms: int, seed: int = 0, device="cpu", bond: float = 0.38,
                   angle_deg: float = 120.0, sigma: float = 0.05, chunk: int = 131072):
    """Serving database frames: each frame is an independent backbone chain
    of `n_atoms` beads with fixed bond length `bond` (nm) and bond angle
    `angle_deg`, torsions uniform in [-pi, pi), plus i.i.d. N(0, sigma^2)
    noise per coordinate.  Built bead by bead (each new bead placed from the
    previous three), vectorised over frames.  Returns a float32 torch tensor
    (F, A, 3) on `device`."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    out = torch.empty((n_frames, n_atoms, 3), dtype=torch.float32, device=device)
    th = math.radians(angle_deg)
    ct, st = math.cos(th), math.sin(th)
    for s0 in range(0, n_frames, chunk):
        n = min(chunk, n_frames - s0)
        pos = torch.zeros((n, n_atoms, 3), dtype=torch.float32, device=device)
        if n_atoms > 1:
            pos[:, 1, 0] = bond
        if n_atoms > 2:
            pos[:, 2, 0] = bond - bond * ct
            pos[:, 2, 1] = bond * st
        tors = (torch.rand((n, n_atoms), generator=g, device=device) * 2 - 1) * math.pi
        for k in range(3, n_atoms):
            a, b, c = pos[:, k - 3], pos[:, k - 2], pos[:, k - 1]
            bc = c - b
            bc = bc / bc.norm(dim=1, keepdim=True)
            nrm = torch.cross(b - a, bc, dim=1)
            nrm = nrm / nrm.norm(dim=1, keepdim=True).clamp_min(1e-12)
            m = torch.cross(nrm, bc, dim=1)
            phi = tors[:, k:k + 1]
            pos[:, k] = c + bond * (-ct * bc + st * torch.cos(phi) * m + st * torch.sin(phi) * nrm)
        pos += torch.randn(pos.shape, generator=g, device=device) * sigma
        out[s0:s0 + n] = pos
    return out


def perturbed_queries(db, idx, seed: int = 0, sigma: float = 0.05, translate: float = 2.0) -> np.ndarray:
    """Query frames: database frames `idx` (host or device (F, A, 3)) plus
    N(0, sigma^2) noise, a Haar-random rotation and a uniform translation in
    [-translate, translate]^3.  Returns float32 numpy (len(idx), A, 3)."""
    rng = np.random.default_rng(seed)
    base = db[idx]
    base = base.cpu().numpy() if hasattr(base, "cpu") else np.asarray(base)
    base = base.astype(np.float64) + rng.normal(size=base.shape) * sigma
    rot = haar_rotations(len(idx), rng)
    t = rng.uniform(-translate, translate, size=(len(idx), 1, 3))
    return np.ascontiguousarray(np.einsum("fkj,fij->fki", base, rot) + t, dtype=np.float32)
