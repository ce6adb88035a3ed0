"""Host side of the GPU XTC reader: frame indexing (no device needed)."""
from pathlib import Path

import numpy as np
import pytest

from mdtraj_gb300 import xtc

GOLDEN = Path(__file__).parent / "golden"


@pytest.mark.parametrize("name,frames,atoms", [("water", 40, 1001), ("tiny", 12, 7), ("wide", 5, 50)])
def test_index_finds_every_frame(name, frames, atoms):
    data = np.fromfile(GOLDEN / f"xtc_{name}.xtc", dtype=np.uint8)
    offsets, A, used = xtc.index_bytes(data)
    assert len(offsets) == frames and A == atoms and used == data.size
    assert offsets[0] == 0 and np.all(np.diff(offsets) > 0) and np.all(offsets % 4 == 0)


def test_index_stops_before_a_truncated_frame_and_rejects_mixed_files():
    data = np.fromfile(GOLDEN / "xtc_water.xtc", dtype=np.uint8)
    offsets, A, used = xtc.index_bytes(data)
    cut = data[: offsets[7] + 100]
    o2, A2, used2 = xtc.index_bytes(cut)
    assert len(o2) == 7 and used2 == offsets[7] and A2 == A
    tiny = np.fromfile(GOLDEN / "xtc_tiny.xtc", dtype=np.uint8)
    with pytest.raises(ValueError, match="atoms"):
        xtc.index_bytes(np.concatenate([data, tiny]))
    with pytest.raises(ValueError, match="not an XTC"):
        xtc.index_bytes(np.arange(64, dtype=np.uint8))


@pytest.mark.parametrize("chunk", [3000, 20000, 1 << 20])
def test_read_ahead_chunks_cover_the_file_in_order(chunk):
    """The reader thread hands over every frame once, in order, whatever the
    chunk size (frames split across read blocks carry over)."""
    data = np.fromfile(GOLDEN / "xtc_water.xtc", dtype=np.uint8)
    offsets, A, used = xtc.index_bytes(data)
    starts = []
    for block, off, a, first in xtc._read_ahead(xtc._read_chunks(GOLDEN / "xtc_water.xtc", chunk)):
        assert a == A and first == len(starts)
        base = offsets[first]
        assert np.array_equal(block[: 64], data[base: base + 64])
        starts.extend(int(o) + int(base) for o in off)
    assert starts == [int(o) for o in offsets]


def test_read_ahead_reraises_reader_errors(tmp_path):
    data = np.fromfile(GOLDEN / "xtc_water.xtc", dtype=np.uint8)
    offsets, _, _ = xtc.index_bytes(data)
    bad = tmp_path / "cut.xtc"
    data[: offsets[3] + 50].tofile(bad)
    got = 0
    with pytest.raises(ValueError, match="truncated"):
        for _, off, _, _ in xtc._read_ahead(xtc._read_chunks(bad, 1 << 20)):
            got += len(off)
    assert got == 3
