"""The GPU's XTC frame decoder (mdtraj_gb300/csrc/xtc_dec.cuh, __host__
__device__) built for the host and checked bit for bit against the
reference reader's output on the reference-written fixtures (CPU), with the
file at a few byte offsets in memory (the stream's bytes are read
unaligned)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
GOLDEN = HERE / "golden"


@pytest.fixture(scope="module")
def xtc_bin(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("xtc") / "xtc_host_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-o", str(out), str(HERE / "xtc_host_check.cu")], check=True,
                   capture_output=True)
    return out


def _decode(xtc_bin, path, shift=0):
    raw = subprocess.run([str(xtc_bin), str(path), str(shift)], capture_output=True, check=True).stdout
    F, A = np.frombuffer(raw[:16], dtype=np.int64)
    rec = np.dtype([("status", "<i4"), ("step", "<i4"), ("time", "<f4"), ("box", "<f4", (3, 3)),
                    ("xyz", "<f4", (int(A), 3))])
    return np.frombuffer(raw[16:], dtype=rec, count=int(F))


@pytest.mark.parametrize("name", ["water", "tiny", "wide"])
@pytest.mark.parametrize("shift", [0, 1, 7])
def test_host_decoder_matches_reference_reader(xtc_bin, golden, name, shift):
    g = golden("xtc_cases.npz")
    out = _decode(xtc_bin, GOLDEN / f"xtc_{name}.xtc", shift)
    assert len(out) == len(g[f"{name}__xyz"])
    assert np.all(out["status"] == 0)
    np.testing.assert_array_equal(out["xyz"], g[f"{name}__xyz"])
    np.testing.assert_array_equal(out["step"], g[f"{name}__step"])
    np.testing.assert_array_equal(out["time"], g[f"{name}__time"])
    np.testing.assert_array_equal(out["box"], g[f"{name}__box"])
