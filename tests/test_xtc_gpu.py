"""GPU XTC decoding against the reference reader (tests/golden/xtc_cases.npz,
written and read back by the reference's formats/xtc): bit-exact coordinates,
time, step and box; chunked streaming; the fused decode + md.rmsd."""
from pathlib import Path

import numpy as np
import pytest

import mdtraj_gb300 as md
from conftest import assert_parity
from mdtraj_gb300 import xtc
from oracle import fp64

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden"


@pytest.mark.parametrize("name", ["water", "tiny", "wide"])
def test_decode_is_bit_exact(cuda, golden, name):
    g = golden("xtc_cases.npz")
    xyz, time, step, box = xtc.load_xtc(GOLDEN / f"xtc_{name}.xtc")
    np.testing.assert_array_equal(xyz, g[f"{name}__xyz"])
    np.testing.assert_array_equal(time, g[f"{name}__time"])
    np.testing.assert_array_equal(step, g[f"{name}__step"])
    np.testing.assert_array_equal(box, g[f"{name}__box"])


def test_chunked_streaming_matches_whole_file(cuda, golden):
    g = golden("xtc_cases.npz")
    chunks = list(xtc.iter_xtc(GOLDEN / "xtc_water.xtc", chunk_bytes=3000))
    assert len(chunks) > 10 and [c.first_frame for c in chunks] == list(np.cumsum([0] + [c.n_frames for c in chunks[:-1]]))
    got = np.concatenate([c.xyz.view(c.n_frames, c.n_padded, 3)[:, :c.n_atoms].cpu().numpy() for c in chunks])
    np.testing.assert_array_equal(got, g["water__xyz"])


def test_rmsd_straight_from_the_file(cuda, golden):
    g = golden("xtc_cases.npz")
    x = g["water__xyz"]
    got = xtc.rmsd_xtc(GOLDEN / "xtc_water.xtc", x, frame=3, chunk_bytes=20000)
    assert_parity(got, fp64.kabsch_rmsd(x, x[3]), what="xtc rmsd")
    assert np.abs(got - md.rmsd(md.Trajectory(x.copy()), md.Trajectory(x.copy()), 3)).max() < 1e-5


def test_malformed_frames_raise(cuda, tmp_path):
    data = np.fromfile(GOLDEN / "xtc_water.xtc", dtype=np.uint8)
    offsets, A, used = xtc.index_bytes(data)
    bad = data.copy()
    o = int(offsets[5]) + 56 + 32          # byte count of frame 5's bit stream
    bad[o:o + 4] = [0x7f, 0xff, 0xff, 0xf0]  # larger than the file
    with pytest.raises(ValueError, match="frame 5"):
        xtc.decode_bytes(bad, offsets, A)
    bad = data.copy()
    o = int(offsets[9]) + 56 + 28          # small-integer index of frame 9
    bad[o:o + 4] = [0, 0, 0, 99]
    with pytest.raises(ValueError, match="frame 9"):
        xtc.decode_bytes(bad, offsets, A)
    # flipped payload bits decode to other numbers but stay inside the frame
    bad = data.copy()
    bad[int(offsets[2]) + 200:int(offsets[2]) + 260] ^= 0x5A
    try:
        out = xtc.decode_bytes(bad, offsets, A)
        assert out.n_frames == len(offsets)
    except ValueError as e:
        assert "frame 2" in str(e)
