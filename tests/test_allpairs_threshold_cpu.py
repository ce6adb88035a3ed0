"""The refinement threshold of the all-pairs and cross tile epilogues
(pair_needs_refine in mdtraj_gb300/csrc/allpairs.cuh), checked on the CPU.

The tensor tiles form M from split BF16 planes (hi = bf16(x), lo = bf16(x -
hi); M ~ hi.hi^T + hi.lo^T + lo.hi^T).  Pairs whose rmsd lies below
c * scale / sqrt(n) (scale = (Ga + Gb) / 2n) are recomputed exactly; above
it the rmsd comes from the split M.  This emulation sums the three BF16
products exactly (FP64) and solves for lambda with numpy: on noisy rotated
copies of one structure (the class of input closest to the threshold) the
unrefined pairs must stay within 5e-5 nm of the exact rmsd, half the 1e-4
bar, because the tensor core's FP32 accumulation roughly doubles the error
on the GPU (measured 1.16e-4 nm there at c = 0.25)."""
import re
from pathlib import Path

import numpy as np
import pytest

from mdtraj_gb300 import synth

CUH = Path(__file__).resolve().parents[1] / "mdtraj_gb300" / "csrc" / "allpairs.cuh"


def _threshold_constant():
    src = CUH.read_text()
    body = src[src.index("bool pair_needs_refine("):]
    body = body[: body.index("}")]
    m = re.search(r"rn_mul\(([0-9.]+)f, scale\)", body)
    assert m, "pair_needs_refine no longer has the form r < rn_mul(c, scale) * sqrt(inv_n)"
    return float(m.group(1))


def _bf16(a):
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _lambda_max(M):
    S = M
    K = np.empty(M.shape[:-2] + (4, 4))
    K[..., 0, 0] = S[..., 0, 0] + S[..., 1, 1] + S[..., 2, 2]
    K[..., 1, 1] = S[..., 0, 0] - S[..., 1, 1] - S[..., 2, 2]
    K[..., 2, 2] = -S[..., 0, 0] + S[..., 1, 1] - S[..., 2, 2]
    K[..., 3, 3] = -S[..., 0, 0] - S[..., 1, 1] + S[..., 2, 2]
    K[..., 0, 1] = K[..., 1, 0] = S[..., 1, 2] - S[..., 2, 1]
    K[..., 0, 2] = K[..., 2, 0] = S[..., 2, 0] - S[..., 0, 2]
    K[..., 0, 3] = K[..., 3, 0] = S[..., 0, 1] - S[..., 1, 0]
    K[..., 1, 2] = K[..., 2, 1] = S[..., 0, 1] + S[..., 1, 0]
    K[..., 1, 3] = K[..., 3, 1] = S[..., 0, 2] + S[..., 2, 0]
    K[..., 2, 3] = K[..., 3, 2] = S[..., 1, 2] + S[..., 2, 1]
    return np.linalg.eigvalsh(K)[..., -1]


def _split_and_exact_rmsd(x, chunk=2048):
    """rmsd of every pair i < j from the exact M and from the split-BF16 M
    (the three products summed exactly), and the pairs' scale."""
    F, A = x.shape[0], x.shape[1]
    xc = x.astype(np.float64)
    xc = (xc - xc.mean(1, keepdims=True)).astype(np.float32)  # the prep's float-centred rows
    x64 = xc.astype(np.float64)
    hi = _bf16(xc)
    lo = _bf16((xc - hi.astype(np.float32)).astype(np.float32))
    G = (x64 ** 2).sum((1, 2))
    i, j = np.triu_indices(F, 1)
    r_ex = np.empty(i.size)
    r_bf = np.empty(i.size)
    for s in range(0, i.size, chunk):
        a, b = i[s:s + chunk], j[s:s + chunk]
        exact = np.einsum("pac,pad->pcd", x64[a], x64[b])
        split = (np.einsum("pac,pad->pcd", hi[a], hi[b]) + np.einsum("pac,pad->pcd", hi[a], lo[b])
                 + np.einsum("pac,pad->pcd", lo[a], hi[b]))
        r_ex[s:s + chunk] = np.sqrt(np.maximum((G[a] + G[b] - 2 * _lambda_max(exact)) / A, 0))
        r_bf[s:s + chunk] = np.sqrt(np.maximum((G[a] + G[b] - 2 * _lambda_max(split)) / A, 0))
    return r_ex, r_bf, (G[i] + G[j]) / (2 * A)


@pytest.mark.parametrize("A", [257, 1000])
def test_unrefined_pairs_of_the_split_bf16_m_stay_within_half_the_bar(A):
    c = _threshold_constant()
    F = 300
    _, x = synth.single_reference_frames(F, A, seed=F + A, sigma=np.geomspace(1e-3, 0.4, F), exact_fraction=0.03)
    r_ex, r_bf, scale = _split_and_exact_rmsd(x)
    kept = r_bf >= c * scale / np.sqrt(A)
    assert kept.sum() > 0.3 * kept.size  # the set exercises the tiles, not only the refinement
    err = np.abs(r_bf - r_ex)[kept]
    assert err.max() <= 5e-5, f"c={c}: unrefined split-BF16 error {err.max():.3e} nm"
