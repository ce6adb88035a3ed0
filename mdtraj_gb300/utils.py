"""Boundary type coercion with the semantics of mdtraj.utils.ensure_type
(mdtraj/utils/validation.py:44-160): the drop-in validates its arguments the
way the reference does, so it raises the same exception types."""
from __future__ import annotations

import collections.abc
import warnings
from itertools import zip_longest

import numpy as np


class TypeCastPerformanceWarning(RuntimeWarning):
    """Emitted when an argument is cast to another dtype
    (mdtraj/utils/validation.py:40)."""


def ensure_type(val, dtype, ndim, name, length=None, can_be_none=False, shape=None,
                warn_on_cast=True, add_newaxis_on_deficient_ndim=False):
    """Checks ndim / shape / dtype of an array-like and returns a C-contiguous
    array of `dtype` (a copy only when needed).

    Raises TypeError for non-iterables, ValueError for ndim / length / shape
    mismatches; warns TypeCastPerformanceWarning on a dtype cast when
    `warn_on_cast`.  A None shape entry matches any extent.
    """
    if can_be_none and val is None:
        return None
    if not isinstance(val, np.ndarray):
        if isinstance(val, collections.abc.Iterable):
            if isinstance(val, collections.abc.Sequence):
                val = np.asarray(val, dtype=dtype)
            else:
                val = np.asarray(list(val), dtype=dtype)
        elif np.isscalar(val) and add_newaxis_on_deficient_ndim and ndim == 1:
            val = np.array([val])
        else:
            raise TypeError(f"{name} must be numpy array. You supplied type {type(val)}")
    if warn_on_cast and val.dtype != dtype:
        warnings.warn(f"Casting {name} dtype={val.dtype} to {dtype} ", TypeCastPerformanceWarning)
    if val.ndim != ndim:
        if add_newaxis_on_deficient_ndim and val.ndim + 1 == ndim:
            val = val[np.newaxis, ...]
        else:
            raise ValueError(f"{name} must be ndim {ndim}. You supplied {val.ndim}")
    val = np.ascontiguousarray(val, dtype=dtype)
    if length is not None and len(val) != length:
        raise ValueError(f"{name} must be length {length}. You supplied {len(val)}")
    if shape is not None:
        err = ValueError(
            "{} must be shape {}. You supplied  {}".format(name, str(shape).replace("None", "Any"), val.shape)
        )
        missing = object()
        for have, want in zip_longest(val.shape, shape, fillvalue=missing):
            if have is missing or want is missing:
                raise err
            if want is None:
                continue
            if have != want:
                raise err
    return val
