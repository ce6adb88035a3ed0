"""Ragged batch (one persistent launch over many trajectories) against the
FP64 oracle, the reference's per-trajectory md.rmsd, and per-trajectory
launches of the single-reference path; CUDA-graph replay; autotuner."""
import numpy as np
import pytest
import torch

import mdtraj_gb300 as md
from conftest import assert_parity
from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, autotune, synth
from oracle import cpu, fp64

pytestmark = pytest.mark.gpu


def make_batch(n_seg=23, seed=0, max_atoms=900, max_frames=70):
    rng = np.random.default_rng(seed)
    trajs = []
    for s in range(n_seg):
        A = int(round(np.exp(rng.uniform(np.log(1), np.log(max_atoms)))))
        F = int(rng.integers(1, max_frames))
        ref, x = synth.single_reference_frames(F, A, seed=1000 + s, sigma=np.geomspace(1e-3, 0.3, F),
                                               exact_fraction=0.05)
        trajs.append(x)
    return trajs


def test_ragged_matches_fp64_and_reference(cuda):
    trajs = make_batch()
    out = md.ragged_rmsd(trajs)
    ref_impl = cpu.best_available()
    for x, got in zip(trajs, out):
        assert got.shape == (x.shape[0],)
        assert got[0] == 0.0
        want = fp64.kabsch_rmsd(x, x[0])
        xr = x.copy()
        ref = ref_impl.md_rmsd(xr, xr[0])
        assert_parity(got, want, ref, what=f"A={x.shape[1]} F={x.shape[0]}")


@pytest.mark.parametrize("config", range(5))
@pytest.mark.parametrize("muq", [32, 512])
def test_every_config_gives_the_same_answer(cuda, config, muq):
    trajs = make_batch(n_seg=9, seed=4, max_atoms=3000, max_frames=40)
    b = md.RaggedBatch(trajs, config=config, max_unit_quads=muq)
    got = b.run().cpu().numpy()
    want = np.concatenate([fp64.kabsch_rmsd(x, x[0]) for x in trajs])
    assert_parity(got, want, what=f"config {config} units {muq}")


def test_graph_replay_equals_direct_run_and_separate_launches(cuda):
    trajs = make_batch(n_seg=12, seed=7, max_atoms=2000, max_frames=50)
    b = md.RaggedBatch(trajs, config=0, max_unit_quads=256)
    direct = b.run().clone()
    b.capture()
    for _ in range(2):
        replayed = b.replay()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(direct.cpu().numpy(), replayed.cpu().numpy())
    # same frames through the single-reference path, one call per trajectory
    stream = D.stream_handle()
    sep = []
    for x in trajs:
        xd, Ap = D.frames_to_device(x, _lib.ATOM_MAJOR, cuda, stream)
        r = D.DeviceReference(x[0], _lib.ATOM_MAJOR, centre=True)
        sep.append(D.to_host(D.rmsd_to_reference(xd, x.shape[0], x.shape[1], Ap, _lib.ATOM_MAJOR,
                                                 _lib.MODE_CENTER, r, self_index=0), stream))
    assert np.abs(np.concatenate(sep) - direct.cpu().numpy()).max() < 1e-5


def test_invalid_segments_are_rejected(cuda):
    with pytest.raises(ValueError):
        md.ragged_rmsd([np.zeros((0, 5, 3), np.float32)])
    with pytest.raises(ValueError):
        md.ragged_rmsd([])


def test_autotuner_caches_a_choice(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("MDTRAJ_GB300_CACHE", str(tmp_path))
    trajs = make_batch(n_seg=6, seed=9, max_atoms=1500, max_frames=30)
    b = md.RaggedBatch(trajs, autotune=True)
    bucket = autotune.shape_bucket(b.atoms, b.frames)
    cache = autotune.load_cache()
    assert bucket in cache and len(cache[bucket]["timings"]) >= 5
    got = b.run().cpu().numpy()
    want = np.concatenate([fp64.kabsch_rmsd(x, x[0]) for x in trajs])
    assert_parity(got, want, what="autotuned")
    # a second batch of the same bucket reuses the cached choice without tuning
    c, m = autotune.ragged_choice(b)
    assert (c, m) == (cache[bucket]["config"], cache[bucket]["max_unit_quads"])
