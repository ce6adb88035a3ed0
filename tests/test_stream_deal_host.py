"""The streaming kernel's dealing of units to warps and the in-kernel
finish's per-CTA frame order (mdtraj_gb300/csrc/stream_deal.cuh, __host__
__device__), built for the host and replayed over many sizes (CPU).

Every unit must be streamed exactly once, whatever the frame count, grid,
warps per CTA and splits; with one unit per frame each CTA's records and
finish must cover exactly the frames its warps streamed, in the local order
the kernel writes them, within the shared-memory slots the host sizes."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return None


@pytest.fixture(scope="module")
def deal_bin(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("deal") / "stream_deal_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-o", str(out), str(HERE / "stream_deal_check.cu")], check=True,
                   capture_output=True)
    return out


def _cases():
    for grid, warps in [(152, 16), (152, 8), (5, 16), (3, 8), (1, 4), (7, 3)]:
        W = grid * warps
        frames = set(range(0, 2 * W + 3, max(1, W // 97))) | {0, 1, W - 1, W, W + 1, 2 * W - 1, 4 * W + 17}
        if grid == 152:
            frames |= {10_000, 200_000}
        for F in sorted(frames):
            for S in (1, 2, 3):
                yield F, grid, warps, S


def test_every_unit_once_and_finish_order_matches(deal_bin):
    cases = list(_cases())
    text = "\n".join(f"{F} {g} {w} {S}" for F, g, w, S in cases) + "\n"
    r = subprocess.run([str(deal_bin)], input=text, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert r.stdout.strip() == f"ok {len(cases)}"
