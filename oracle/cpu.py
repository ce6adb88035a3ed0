"""ORACLE — test infrastructure only (never used by mdtraj_gb300/).

ctypes access to the two CPU implementations built by oracle/Makefile:

* ``port``      — oracle/qcp_port.c, the C restatement of the reference
                  algorithm (always buildable: gcc + OpenMP);
* ``reference`` — mdtraj's own CPU kernels (center.cpp, theobald_rmsd.cpp)
                  compiled from the reference's sources, with a thin driver
                  (oracle/ref_driver.cpp) replaying the loops of _rmsd.pyx.

Both mutate their inputs exactly like the reference (in-place centring), so
callers pass copies.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "_build" / platform.machine() / "libqcp_port.so"
REF_SO = HERE / "_ref" / platform.machine() / "libref_rmsd.so"

_vp, _i64, _i32 = C.c_void_p, C.c_int64, C.c_int32


def build(ref: bool = True) -> None:
    """Builds the port (and, when its sources are available -- the checkout
    named by MDTRAJ_REF, or the copy staged under oracle/_ref/src -- the
    reference)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    if ref:
        root = os.environ.get("MDTRAJ_REF")
        extra = [f"REF_ROOT={root}"] if root else []
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", *extra], check=False,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def _load(path: Path, prefix: str):
    lib = C.CDLL(str(path))
    getattr(lib, f"{prefix}_md_rmsd").argtypes = [_vp, _i64, _i32, _vp, _vp]
    getattr(lib, f"{prefix}_multiple_axis_major").argtypes = [_vp, _vp, _vp, _vp, _i64, _i64, _i32, _vp]
    getattr(lib, f"{prefix}_multiple_atom_major").argtypes = [_vp, _vp, _vp, _vp, _i64, _i64, _i32, _vp]
    for fn in (f"{prefix}_md_rmsd", f"{prefix}_multiple_axis_major", f"{prefix}_multiple_atom_major"):
        getattr(lib, fn).restype = None
    return lib


class CpuRmsd:
    """One CPU implementation (``kind`` = "port" or "reference")."""

    def __init__(self, kind: str):
        self.kind = kind
        if kind == "port":
            if not PORT_SO.exists():
                build(ref=False)
            self.lib = _load(PORT_SO, "port")
            self.prefix = "port"
            self.lib.port_center_and_trace.argtypes = [_vp, _vp, _i64, _i32]
            self.lib.port_nosuperpose.argtypes = [_vp, _i64, _i32, _vp, _vp]
        elif kind == "reference":
            if not REF_SO.exists():
                build(ref=True)
            if not REF_SO.exists():
                raise FileNotFoundError("reference CPU kernels could not be built (no sources)")
            self.lib = _load(REF_SO, "ref")
            self.prefix = "ref"
            self.lib.ref_center_inplace.argtypes = [_vp, _i64, _i32, _vp]
            self.lib.ref_superpose_atom_major.argtypes = [_vp, _vp, C.c_float, _vp, _vp, _i64, _i32, _i32]
            self.lib.ref_rmsf_rotated.argtypes = [_vp, _vp, C.c_float, _vp, _vp, _i64, _i32, _i32, _vp]
        else:
            raise ValueError(kind)

    def md_rmsd(self, target: np.ndarray, ref_frame: np.ndarray) -> np.ndarray:
        """md.rmsd(target, ref) semantics; centres both arrays in place."""
        assert target.dtype == np.float32 and target.flags.c_contiguous
        assert ref_frame.dtype == np.float32 and ref_frame.flags.c_contiguous
        out = np.empty(target.shape[0], dtype=np.float32)
        getattr(self.lib, f"{self.prefix}_md_rmsd")(target.ctypes.data, target.shape[0], target.shape[1],
                                                     ref_frame.ctypes.data, out.ctypes.data)
        return out

    def multiple(self, xyz1, xyz2, g1, g2, frame: int, axis_major: bool) -> np.ndarray:
        n_atoms = xyz1.shape[2] if axis_major else xyz1.shape[1]
        out = np.empty(xyz2.shape[0], dtype=np.float32)
        fn = getattr(self.lib, f"{self.prefix}_multiple_{'axis' if axis_major else 'atom'}_major")
        fn(xyz1.ctypes.data, xyz2.ctypes.data, g1.ctypes.data, g2.ctypes.data, frame, xyz2.shape[0], n_atoms,
           out.ctypes.data)
        return out

    def center_inplace(self, xyz: np.ndarray) -> np.ndarray:
        traces = np.empty(xyz.shape[0], dtype=np.float32)
        if self.kind == "port":
            self.lib.port_center_and_trace(xyz.ctypes.data, traces.ctypes.data, xyz.shape[0], xyz.shape[1])
        else:
            self.lib.ref_center_inplace(xyz.ctypes.data, xyz.shape[0], xyz.shape[1], traces.ctypes.data)
        return traces

    def nosuperpose(self, target: np.ndarray, ref_frame: np.ndarray) -> np.ndarray:
        if self.kind != "port":
            raise NotImplementedError("the reference's msd_nosuperpose lives in Cython")
        out = np.empty(target.shape[0], dtype=np.float32)
        self.lib.port_nosuperpose(target.ctypes.data, target.shape[0], target.shape[1], ref_frame.ctypes.data,
                                  out.ctypes.data)
        return out


    def superpose(self, xyz: np.ndarray, ref_frame: np.ndarray) -> None:
        """Trajectory.superpose(t, ref, frame) on all atoms, in place on xyz
        (float32 C (F, A, 3)): the numpy steps of core/trajectory.py:1124-1165
        around the reference's compiled rotation loop."""
        if self.kind != "reference":
            raise NotImplementedError("superpose needs the reference's rotation kernels")
        n = xyz.shape[0]
        offset = np.mean(xyz, axis=1, dtype=np.float64).reshape(n, 1, 3)
        xyz -= offset
        ref_align = np.array(ref_frame, dtype=np.float32, copy=True, order="C").reshape(1, -1, 3)
        ref_offset = ref_align[0].astype(np.float64).mean(0)
        ref_align[0] -= ref_offset
        g = np.einsum("ijk,ijk->i", xyz, xyz)
        ref_g = np.einsum("ijk,ijk->i", ref_align, ref_align)
        self.lib.ref_superpose_atom_major(ref_align.ctypes.data, xyz.ctypes.data, float(ref_g[0]), g.ctypes.data,
                                          xyz.ctypes.data, n, xyz.shape[1], xyz.shape[1])
        xyz += ref_offset

    def rmsf(self, xyz: np.ndarray, ref_frame: np.ndarray) -> np.ndarray:
        """rmsf(t, ref, frame) on all atoms (_rmsd.pyx:389-456): centres xyz
        and a copy of the reference frame in place, rotates a copy, reduces."""
        if self.kind != "reference":
            raise NotImplementedError("rmsf needs the reference's rotation kernels")
        g = self.center_inplace(xyz)
        r = np.array(ref_frame, dtype=np.float32, copy=True, order="C").reshape(1, -1, 3)
        rg = self.center_inplace(r)
        disp = xyz.copy()
        out = np.empty(xyz.shape[1], dtype=np.float32)
        self.lib.ref_rmsf_rotated(xyz.ctypes.data, r.ctypes.data, float(rg[0]), g.ctypes.data, disp.ctypes.data,
                                  xyz.shape[0], xyz.shape[1], 1, out.ctypes.data)
        return out


def best_available() -> CpuRmsd:
    """The reference's own kernels when they can be built here, else the port."""
    try:
        return CpuRmsd("reference")
    except (FileNotFoundError, OSError):
        return CpuRmsd("port")


def n_threads() -> int:
    v = os.environ.get("OMP_NUM_THREADS")
    return int(v) if v else (os.cpu_count() or 1)


XTC_SO = HERE / "_ref" / platform.machine() / "libref_xtc.so"


def read_xtc_reference(path, n_atoms: int, max_frames: int):
    """(xyz (F, A, 3), step, time, box (F, 3, 3)) read by the reference's C XTC
    reader (oracle/ref_xtc_driver.c)."""
    if not XTC_SO.exists():
        build(ref=True)
    if not XTC_SO.exists():
        raise FileNotFoundError("reference XTC reader could not be built (no sources)")
    lib = C.CDLL(str(XTC_SO))
    lib.ref_xtc_read.restype = C.c_int
    lib.ref_xtc_read.argtypes = [C.c_char_p, C.c_int, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    xyz = np.zeros((max_frames, n_atoms, 3), np.float32)
    step = np.zeros(max_frames, np.int32)
    time = np.zeros(max_frames, np.float32)
    box = np.zeros((max_frames, 3, 3), np.float32)
    n = lib.ref_xtc_read(str(path).encode(), n_atoms, max_frames, xyz.ctypes.data, step.ctypes.data,
                         time.ctypes.data, box.ctypes.data)
    if n < 0:
        raise FileNotFoundError(str(path))
    return xyz[:n], step[:n], time[:n], box[:n]
