"""The sharded all-pairs matrix on the GPU through a one-rank process group:
the block path (the rank's run of the triangle as one cross-RMSD launch,
the trajectory prepared once as database and queries) against one
allpairs_rmsd call and the FP64 oracle."""
import socket

import numpy as np
import pytest

from conftest import assert_parity
from oracle import fp64

pytestmark = pytest.mark.gpu


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("F,A,block", [(300, 257, 64), (257, 40, None), (97, 2, 50)])
def test_allpairs_sharded_block_path_on_one_gpu(cuda, F, A, block):
    import torch.distributed as dist

    from mdtraj_gb300 import synth
    from mdtraj_gb300.allpairs import allpairs_rmsd
    from mdtraj_gb300.shard import allpairs_sharded

    _, x = synth.single_reference_frames(F, A, seed=F + A, sigma=np.geomspace(1e-3, 0.4, F), exact_fraction=0.03)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{_port()}", rank=0, world_size=1)
    try:
        got = allpairs_sharded(x, block=block)
    finally:
        dist.destroy_process_group()
    one = allpairs_rmsd(x)
    np.testing.assert_array_equal(got, got.T)
    assert np.all(np.diag(got) == 0)
    rng = np.random.default_rng(F)
    i = rng.integers(0, F, 3000)
    j = rng.integers(0, F, 3000)
    keep = i != j
    pairs = np.stack([i[keep], j[keep]], 1)
    want = fp64.kabsch_rmsd_pairs(x, pairs)
    assert_parity(got[pairs[:, 0], pairs[:, 1]], want, what=f"sharded {F}x{A}")
    assert np.abs(got.astype(np.float64) - one).max() <= 5e-5
