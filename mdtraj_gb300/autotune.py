"""Autotuner for the ragged batch kernel.

Candidates are the kernel's launch configurations (warps per CTA, quads per
shared-memory stage, stages per warp) crossed with the largest work unit
(quads per unit, which sets how large frames are split across warps).  Each
candidate is timed with CUDA events on the batch itself; the fastest is
cached per shape bucket in a JSON file ($MDTRAJ_GB300_CACHE/autotune.json,
default ~/.cache/mdtraj_gb300/autotune.json) and reused by later batches of
the same bucket.
"""
from __future__ import annotations

import json
import math
import os
import tempfile
from pathlib import Path

import numpy as np

UNIT_QUADS = (256, 512, 1024)


def cache_path() -> Path:
    root = os.environ.get("MDTRAJ_GB300_CACHE")
    base = Path(root) if root else Path.home() / ".cache" / "mdtraj_gb300"
    return base / "autotune.json"


def shape_bucket(atoms, frames) -> str:
    """Batches in one bucket share a tuned configuration: log2 buckets of the
    segment count, total bytes and the frame-weighted mean atom count."""
    atoms = np.asarray(atoms, dtype=np.float64)
    frames = np.asarray(frames, dtype=np.float64)
    total = float((12.0 * atoms * frames).sum())
    mean_atoms = float((atoms * frames).sum() / max(frames.sum(), 1.0))
    return "ragged:seg%d:bytes%d:atoms%d" % (round(math.log2(max(len(atoms), 1))), round(math.log2(max(total, 1.0))),
                                              round(math.log2(max(mean_atoms, 1.0))))


def load_cache() -> dict:
    p = cache_path()
    if p.exists():
        try:
            return json.loads(p.read_text())
        except (OSError, ValueError):
            return {}
    return {}


def save_cache(cache: dict) -> None:
    """Writes the cache atomically: a private temporary file in the same
    directory, then a rename, so processes or threads tuning at the same time
    never see (or leave) a partly written file; the last writer wins."""
    p = cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=p.name + ".", suffix=".tmp", dir=p.parent)
    try:
        with os.fdopen(fd, "w") as f:
            f.write(json.dumps(cache, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except BaseException:
        try:
            os.unlink(tmp)
        except OSError:
            pass
        raise


def tune_ragged(batch, reps: int = 3) -> dict:
    """Times every candidate on `batch` and caches the fastest.  Returns the
    cache entry {"config", "max_unit_quads", "ms", "timings"}."""
    import torch

    from ._lib import lib

    timings = []
    for cfg in range(lib.gbrmsd_ragged_config_count()):
        for muq in UNIT_QUADS:
            try:
                batch.configure(cfg, muq)
            except Exception:  # configuration does not fit this device
                continue
            batch.run()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ms = []
            for _ in range(reps):
                e0.record()
                batch.run()
                e1.record()
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            timings.append({"config": cfg, "max_unit_quads": muq, "ms": float(np.median(ms))})
    best = min(timings, key=lambda t: t["ms"])
    entry = {"config": best["config"], "max_unit_quads": best["max_unit_quads"], "ms": best["ms"],
             "timings": timings}
    cache = load_cache()
    cache[shape_bucket(batch.atoms, batch.frames)] = entry
    save_cache(cache)
    batch.configure(best["config"], best["max_unit_quads"])
    return entry


def ragged_choice(batch, autotune: bool = False):
    """(config, max_unit_quads) for a batch: the cached choice of its bucket,
    else a fresh tuning when `autotune`, else the defaults."""
    entry = load_cache().get(shape_bucket(batch.atoms, batch.frames))
    if entry:
        return int(entry["config"]), int(entry["max_unit_quads"])
    if autotune:
        batch.configure(0, 512)
        e = tune_ragged(batch)
        return e["config"], e["max_unit_quads"]
    return 0, 512
