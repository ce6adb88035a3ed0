"""ctypes binding of libgbrmsd.so (declared in include/gbrmsd.h).

The library is loaded at import.  There is no CPU fallback: if the shared
library is missing the import fails with instructions to build it, and
every entry point raises when its status code is non-zero.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libgbrmsd.so"

GBRMSD_OK = 0
E_INVALID = -1
E_WORKSPACE = -2
E_CUDA = -3
E_DEVICE = -4
E_UNSUPPORTED = -5

ATOM_MAJOR = 0
AXIS_MAJOR = 1

MODE_CENTER = 0
MODE_PRECENTERED = 1
MODE_NOSUPERPOSE = 2

# device error word bits (gbrmsd_workspace_error_word)
ERR_TIMEOUT = 1
ERR_NONFINITE = 2

_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_sz = C.c_size_t
_f32 = C.c_float

# name -> (restype, argtypes); must match include/gbrmsd.h
SIGNATURES: dict[str, tuple] = {
    "gbrmsd_version": (C.c_int, []),
    "gbrmsd_last_error": (C.c_char_p, []),
    "gbrmsd_device_supported": (C.c_int, []),
    "gbrmsd_device_caps": (C.c_int, [_vp, _i32]),
    "gbrmsd_reference_workspace_bytes": (_sz, [_i32, _i32]),
    "gbrmsd_prepare_reference": (C.c_int, [_vp, _i32, _i32, _i32, _i32, _vp, _sz, _vp]),
    "gbrmsd_reference_info": (C.c_int, [_vp, _vp, _vp, _vp]),
    "gbrmsd_rmsd_workspace_bytes": (_sz, [_i64, _i32]),
    "gbrmsd_rmsd_to_reference": (
        C.c_int,
        [_vp, _i64, _i32, _i32, _i64, _i32, _i32, _vp, _vp, _f32, _i64, _vp, _vp, _vp, _vp, _sz, _vp],
    ),
    "gbrmsd_rmsd_to_reference_noalloc": (
        C.c_int,
        [_vp, _i64, _i32, _i32, _i64, _i32, _i32, _vp, _vp, _f32, _i64, _vp, _vp, _vp, _vp],
    ),
    "gbrmsd_allpairs_workspace_bytes": (_sz, [_i64, _i32]),
    "gbrmsd_allpairs": (C.c_int, [_vp, _i64, _i32, _i32, _i64, _i32, _i32, _i32, _vp, _vp, _sz, _vp]),
    "gbrmsd_allpairs_status": (C.c_int, [_vp, _vp, _vp]),
    "gbrmsd_rotations_workspace_bytes": (_sz, [_i64, _i32]),
    "gbrmsd_rotations": (C.c_int, [_vp, _i64, _i32, _i32, _i64, _i32, _i32, _vp, _vp, C.c_float, _vp, _vp, _vp, _vp,
                                   _sz, _vp]),
    "gbrmsd_apply_rotations": (C.c_int, [_vp, _i64, _i32, _i64, _vp, _vp, _vp, _vp, _vp]),
    "gbrmsd_rmsf_workspace_bytes": (_sz, [_i64, _i32]),
    "gbrmsd_rmsf": (C.c_int, [_vp, _i64, _i32, _i64, _vp, _vp, _vp, _sz, _vp]),
    "gbrmsd_rotated_rmsd": (C.c_int, [_vp, _i64, _i32, _i64, _vp, _vp, _vp, _vp]),
    "gbrmsd_xtc_index": (C.c_int, [_vp, _i64, _vp, _i64, _vp, _vp, _vp]),
    "gbrmsd_xtc_decode": (C.c_int, [_vp, _i64, _vp, _i64, _i32, _vp, _i64, _vp, _vp, _vp, _vp, _vp]),
    "gbrmsd_frameset_bytes": (_sz, [_i64, _i32]),
    "gbrmsd_frameset_prepare": (C.c_int, [_vp, _i64, _i32, _i32, _i64, _i32, _i32, _vp, _i64, _i64, _vp]),
    "gbrmsd_cross_workspace_bytes": (_sz, [_i64, _i64, _i32]),
    "gbrmsd_cross_rmsd": (C.c_int, [_vp, _i64, _i64, _vp, _i64, _i32, _vp, _i32, _i32, _vp, _sz, _vp]),
    "gbrmsd_ragged_config_count": (C.c_int, []),
    "gbrmsd_ragged_plan": (C.c_int, [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "gbrmsd_ragged_setup": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "gbrmsd_ragged_rmsd": (C.c_int, [_vp, _vp, _vp, _vp, _sz, _vp]),
    "gbrmsd_center_inplace": (C.c_int, [_vp, _i64, _i32, _i32, _i64, _i32, _vp, _vp, _vp, _sz, _vp]),
    "gbrmsd_center_weighted_inplace": (C.c_int, [_vp, _i64, _i32, _i64, _vp, _vp, _vp]),
    "gbrmsd_workspace_status": (C.c_int, [_vp, _vp]),
    "gbrmsd_workspace_error_word": (C.c_int, [_vp, _vp, _vp]),
    "gbrmsd_noalloc_status": (C.c_int, [_vp, _vp]),
    "gbrmsd_noalloc_max_frames": (_i64, [_i32]),
    "gbrmsd_set_wait_limit_ns": (C.c_int, [C.c_uint64]),
    "gbrmsd_test_skip_copy": (C.c_int, [_i64]),
    "gbrmsd_stream_config_count": (C.c_int, []),
    "gbrmsd_stream_config_select": (C.c_int, [_i32]),
    "gbrmsd_stream_config_describe": (C.c_int, [_i32, _i32, _vp]),
    "gbrmsd_profile_enable": (C.c_int, [_i32]),
    "gbrmsd_profile_read": (C.c_int, [_vp, _i32]),
    "gbrmsd_copy_rows": (C.c_int, [_vp, _sz, _vp, _sz, _sz, _sz, _i32, _vp]),
    "gbrmsd_host_subtract_centroids": (C.c_int, [_vp, _i64, _i32, _i64, _vp, _i32]),
    "gbrmsd_pageable_access": (C.c_int, []),
    "gbrmsd_host_register": (C.c_int, [_vp, _sz]),
    "gbrmsd_host_unregister": (C.c_int, [_vp]),
    "gbrmsd_copy_rows_kernel": (C.c_int, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp]),
    "gbrmsd_write_centred": (C.c_int, [_vp, _vp, _i64, _vp, _i64, _i32, _vp]),
}


class CrossRequest(C.Structure):
    """gbrmsd_cross_request_t (include/gbrmsd.h)."""

    _fields_ = [("out", C.c_void_p), ("pool0", C.c_int64), ("db0", C.c_int64), ("db1", C.c_int64),
                ("n_query", C.c_int32), ("reserved", C.c_int32)]


class RaggedPlan(C.Structure):
    """gbrmsd_ragged_plan_t (include/gbrmsd.h)."""

    _fields_ = [("n_seg", C.c_int32), ("config", C.c_int32), ("max_unit_quads", C.c_int32), ("grid", C.c_int32),
                ("total_frames", C.c_int64), ("total_units", C.c_int64), ("ws_bytes", C.c_size_t)]


class GbrmsdError(RuntimeError):
    """A libgbrmsd entry point returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"libgbrmsd error {code}: {message}")
        self.code = code


def _load() -> C.CDLL:
    if not _LIB_PATH.exists():
        raise ImportError(
            f"{_LIB_PATH} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python mdtraj_gb300/build.py)"
        )
    lib = C.CDLL(str(_LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def last_error() -> str:
    msg = lib.gbrmsd_last_error()
    return msg.decode() if msg else ""


def check(rc: int) -> None:
    """Raises on a non-zero status: ValueError for argument errors (the
    reference raises ValueError for bad shapes), GbrmsdError otherwise."""
    if rc == GBRMSD_OK:
        return
    msg = last_error()
    if rc == E_INVALID:
        raise ValueError(msg)
    raise GbrmsdError(rc, msg)


CAP_NAMES = ["cc_major", "cc_minor", "sms", "max_smem_optin", "pageable_memory_access",
             "pageable_uses_host_page_tables", "concurrent_managed_access", "host_register_supported",
             "direct_managed_access_from_host", "l2_bytes", "sm_clock_khz", "mem_clock_khz"]


def device_caps() -> dict:
    """Attributes of the current CUDA device (see gbrmsd_device_caps)."""
    import numpy as np

    buf = np.full(len(CAP_NAMES), -1, dtype=np.int32)
    n = lib.gbrmsd_device_caps(buf.ctypes.data, len(CAP_NAMES))
    if n < 0:
        check(n)
    return dict(zip(CAP_NAMES, buf.tolist()))


def ptr(obj) -> int | None:
    """Address of a torch tensor or numpy array (None for None)."""
    if obj is None:
        return None
    if hasattr(obj, "data_ptr"):
        return obj.data_ptr()
    return obj.ctypes.data
