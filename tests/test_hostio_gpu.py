"""Host-link copies (csrc/hostio.cu) and the chunked host-buffer path of
md.rmsd: the kernels that read the caller's pageable numpy memory into the
padded device layout and write the in-place centring back.

Copies are bit-exact; the centring write-back is the float32 subtraction
x - centroid, compared bit for bit with the same subtraction in numpy on the
centroids the kernel used; chunked RMSDs are within the parity bar of the
FP64 oracle whatever the chunk size."""
import numpy as np
import pytest
import torch

import mdtraj_gb300 as md
from conftest import assert_parity
from mdtraj_gb300 import _device as D
from mdtraj_gb300 import _lib, synth
from mdtraj_gb300._lib import check, lib
from oracle import fp64

pytestmark = pytest.mark.gpu


def _offset_view(shape, offset_floats, seed):
    """A float32 array of `shape` starting `offset_floats` floats into a
    larger buffer (16-byte alignment broken when offset_floats % 4 != 0)."""
    n = int(np.prod(shape))
    base = np.random.default_rng(seed).standard_normal(n + 8).astype(np.float32)
    return base[offset_floats:offset_floats + n].reshape(shape)


@pytest.mark.parametrize("A,offset", [(64, 0), (61, 0), (64, 1), (2, 0), (1, 3)])
def test_copy_in_and_out_atom_major(cuda, A, offset):
    F = 37
    x = _offset_view((F, A, 3), offset, seed=A + offset)
    buf, Ap = D.frames_to_device(x, _lib.ATOM_MAJOR, cuda, D.stream_handle())
    torch.cuda.synchronize()
    want = np.zeros((F, Ap, 3), np.float32)
    want[:, :A] = x
    np.testing.assert_array_equal(buf.view(F, Ap, 3).cpu().numpy(), want)
    out = _offset_view((F, A, 3), offset, seed=99)
    out[...] = 0
    D.frames_to_host(buf, out, _lib.ATOM_MAJOR, A, Ap, D.stream_handle())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out, x)


@pytest.mark.parametrize("A", [64, 62])
def test_copy_in_axis_major_zero_fills_padding(cuda, A):
    F = 9
    x = np.random.default_rng(A).standard_normal((F, 3, A)).astype(np.float32)
    buf, Ap = D.frames_to_device(x, _lib.AXIS_MAJOR, cuda, D.stream_handle())
    # garbage in the padding must be overwritten on every copy
    buf.fill_(7.0)
    buf, Ap = D.frames_to_device(x, _lib.AXIS_MAJOR, cuda, D.stream_handle())
    torch.cuda.synchronize()
    want = np.zeros((F, 3, Ap), np.float32)
    want[:, :, :A] = x
    np.testing.assert_array_equal(buf.cpu().numpy(), want)


@pytest.mark.parametrize("A,offset", [(40, 0), (41, 0), (40, 2)])
def test_write_centred_is_float32_subtraction(cuda, A, offset):
    F = 23
    Ap = D.padded(A)
    rng = np.random.default_rng(A)
    dev = torch.from_numpy(rng.standard_normal((F, Ap * 3)).astype(np.float32)).to(cuda)
    cent = torch.from_numpy(rng.standard_normal((F, 3)).astype(np.float32)).to(cuda)
    host = _offset_view((F, A, 3), offset, seed=3)
    check(lib.gbrmsd_write_centred(host.ctypes.data, dev.data_ptr(), 3 * Ap, cent.data_ptr(), F, A,
                                   D.stream_handle()))
    torch.cuda.synchronize()
    want = dev.view(F, Ap, 3)[:, :A].cpu().numpy() - cent.cpu().numpy()[:, None, :]
    np.testing.assert_array_equal(host, want)


@pytest.mark.parametrize("chunk_bytes", [12 * 24 * 5, 12 * 24 * 64, 1 << 28])
def test_chunked_host_path_matches_oracle(cuda, chunk_bytes):
    """md.rmsd on a host array streamed in chunks of a few frames (many
    chunks, both copy directions overlapping) and in one chunk: the same
    RMSDs (within the bar) and the same in-place centring."""
    A = 24
    ref, x = synth.single_reference_frames(301, A, seed=21, sigma=0.2, exact_fraction=0.02)
    want = fp64.kabsch_rmsd(x, x[7])
    ref_dev = D.DeviceReference(x[7], _lib.ATOM_MAJOR, centre=True, device=cuda)
    host = x.copy()
    got = D.rmsd_host_frames(host, ref_dev, _lib.MODE_CENTER, self_index=7, write_centred=True,
                             chunk_bytes=chunk_bytes)
    assert_parity(got, want, what=f"chunked host path ({chunk_bytes} B)")
    centred = x.astype(np.float64) - x.astype(np.float64).mean(1, keepdims=True)
    assert np.abs(host - centred).max() < 2e-6


def test_one_chunk_array_goes_as_two_halves(cuda, monkeypatch):
    """An array that fits one chunk but is above the two-halves threshold
    (lowered here) streams as two halves of 151 and 150 frames, self frame
    in the second half: the same RMSDs and the same in-place centring."""
    monkeypatch.setattr(D, "TWO_CHUNK_MIN_BYTES", 1)
    A = 24
    ref, x = synth.single_reference_frames(301, A, seed=22, sigma=0.2, exact_fraction=0.02)
    want = fp64.kabsch_rmsd(x, x[200])
    ref_dev = D.DeviceReference(x[200], _lib.ATOM_MAJOR, centre=True, device=cuda)
    host = x.copy()
    got = D.rmsd_host_frames(host, ref_dev, _lib.MODE_CENTER, self_index=200, write_centred=True)
    assert got[200] == 0.0
    assert_parity(got, want, what="two halves")
    centred = x.astype(np.float64) - x.astype(np.float64).mean(1, keepdims=True)
    assert np.abs(host - centred).max() < 2e-6


def test_drop_in_host_side_effect_unaligned_atoms(cuda):
    """The drop-in on an array whose rows are not a multiple of 16 bytes."""
    ref, x = synth.single_reference_frames(120, 33, seed=4, sigma=0.1)
    t = md.Trajectory(x.copy())
    got = md.rmsd(t, t, 5)
    assert_parity(got, fp64.kabsch_rmsd(x, x[5]), what="drop-in, 33 atoms")
    centred = x.astype(np.float64) - x.astype(np.float64).mean(1, keepdims=True)
    assert np.abs(t.xyz - centred).max() < 2e-6


def test_chunked_host_path_small_last_chunk(cuda):
    """Chunks of 300, 300 and 100 frames of 4,000 atoms: the last chunk uses
    more splits per frame than the first, inside the workspace sized for the
    first."""
    ref, x = synth.single_reference_frames(700, 4000, seed=6, sigma=0.1, exact_fraction=0.01)
    want = fp64.kabsch_rmsd(x, x[0])
    ref_dev = D.DeviceReference(x[0], _lib.ATOM_MAJOR, centre=True, device=cuda)
    host = x.copy()
    got = D.rmsd_host_frames(host, ref_dev, _lib.MODE_CENTER, self_index=0, write_centred=True,
                             chunk_bytes=12 * 4000 * 300)
    assert_parity(got, want, what="chunks of 300/300/100 frames")


def test_host_locks_are_released_and_tolerate_caller_locks(cuda):
    """The streaming path locks the array range by range and unlocks it
    before returning; an array the caller locked already is used as is."""
    A = 100
    ref, x = synth.single_reference_frames(900, A, seed=12, sigma=0.1)
    want = fp64.kabsch_rmsd(x, x[3])
    ref_dev = D.DeviceReference(x[3], _lib.ATOM_MAJOR, centre=True, device=cuda)
    chunk = 12 * A * 100  # 9 chunks: the array is locked chunk by chunk
    host = x.copy()
    got = D.rmsd_host_frames(host, ref_dev, _lib.MODE_CENTER, self_index=3, write_centred=True, chunk_bytes=chunk)
    assert_parity(got, want, what="locked chunks")
    # nothing is left locked: the caller can lock the whole array now
    assert lib.gbrmsd_host_register(host.ctypes.data, host.nbytes) == 0
    try:
        again = x.copy()
        np.copyto(host, again)
        got2 = D.rmsd_host_frames(host, ref_dev, _lib.MODE_CENTER, self_index=3, write_centred=True,
                                  chunk_bytes=chunk)
        assert_parity(got2, want, what="caller-locked array")
        centred = x.astype(np.float64) - x.astype(np.float64).mean(1, keepdims=True)
        assert np.abs(host - centred).max() < 2e-6
    finally:
        assert lib.gbrmsd_host_unregister(host.ctypes.data) == 0
