"""Benchmark of the GB300 RMSD hot path; prints ONE JSON line (rank 0).

Workload (default, 1 GPU): single-reference RMSD of 200,000 frames x 10,000
atoms float32 (24 GB, axis-major on the device) to frame 0, not precentered:
frame = R (reference + N(0, sigma^2)) + t with sigma log-uniform in
[0.005, 0.5] nm, 1% exact rotated + translated copies; reference atoms
uniform in a 4 nm cube.  Synthetic, seeded (there is no dataset).

One step = one pass of md.rmsd's work (centre, trace, 3x3 inner product,
FP64 QCP, refinement of near-identical frames) over all frames with the
inputs resident in HBM; inputs are 24 GB >> L2 (129 MB), so no L2 flush is
needed between steps.  `e2e` is the same metric through the drop-in
md.rmsd (mdtraj_gb300.rmsd) with HOST numpy buffers: host->device copy of
the coordinates, the kernels, device->host of the results and the
reference's in-place centring side effect are all inside its timed region.

--impl reference times mdtraj's own CPU kernels (compiled from the
reference's sources by oracle/Makefile; the C restatement in oracle/ when
those sources are absent) with all host threads on a bounded frame sample.

Multi-GPU (torchrun, N > 1): frames are independent, so each rank processes
its own shard of the same per-GPU size (weak scaling, no collective on the
data path); timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_BYTES = 129 << 20        # GB300 L2
L2_FLUSH_BYTES = 256 << 20  # written between timed steps when the inputs fit in L2

class L2Flush:
    """Between timed steps: writes a 256 MB buffer (evicting everything the
    previous step left in L2), then reads a second one so that the lines left
    behind are clean and the next step's misses cause no write-backs of the
    flush's own dirty data."""

    def __init__(self, dev):
        import torch

        self.w = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
        self.r = torch.ones(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
        self.sink = torch.empty((), dtype=torch.float32, device=dev)

    def __call__(self, i):
        import torch

        self.w.fill_(i & 0xFF)
        torch.sum(self.r, dim=0, out=self.sink)


WORKLOADS = {
    # name: (n_frames, n_atoms, layout, sigma_lo, sigma_hi, exact_fraction)
    "single_reference_200000x10000": (200_000, 10_000, 1, 0.005, 0.5, 0.01),
    "single_reference_10000x1000": (10_000, 1_000, 0, 0.05, 0.05, 0.0),
    # all-pairs matrix: (n_frames, n_atoms, n_centres, sigma, cube, stay)
    "allpairs_20000x2000": (20_000, 2_000, 50, 0.1, 5.0, 0.99),
    # ragged batch: (segments, atoms lo, atoms hi, frames lo, frames hi, sigma)
    "ragged_512": (512, 50, 20_000, 100, 5_000, 0.05),
    # superposition / rmsf: (n_frames, n_atoms, sigma)
    "superpose_100000x1000": (100_000, 1_000, 0.05),
    # XTC decoding: (repetitions of the 40-frame x 1,001-atom fixture file)
    "xtc_decode_100000x1001": (2500,),
    # serving: (database frames, atoms, offered rates (requests/s), max query frames, slice lengths)
    "serving_500000x300": (500_000, 300, (100, 300, 1000, 3000, 10000), 256, (10_000, 500_000)),
}
DEFAULT_WORKLOAD = "single_reference_200000x10000"


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


def traffic_from_profiles(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` from a committed ncu summary
    (profiles/*.txt or *.md line: 'dram_bytes_per_launch <kernel> <workload> <bytes>')."""
    for f in sorted((ROOT / "profiles").glob("*.txt")) + sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            m = re.match(r"dram_bytes_per_launch\s+(\S+)\s+(\S+)\s+([0-9.eE+]+)", line.strip())
            if m and m.group(1) == kernel and m.group(2) == workload:
                return float(m.group(3))
    return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks / throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        mx = max(r[1] for r in rows)
        loaded = [r for r in rows if r[0] > 0.5 * mx] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in loaded for i, v in enumerate(r[2]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def shard(n_frames: int, rank: int, world: int) -> tuple[int, int]:
    """Weak scaling: every rank gets the full per-GPU workload; the global
    frame index range of rank r is [r * n, (r + 1) * n)."""
    return rank * n_frames, (rank + 1) * n_frames


def max_over_ranks(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU baseline (reference implementation on the host cores)
# ---------------------------------------------------------------------------


def _synth():
    """mdtraj_gb300/synth.py (numpy-only generators) loaded as a standalone
    module: importing it through the package would load libgbrmsd.so, and
    the reference arm must not map any of this project's libraries."""
    import importlib.util

    name = "_bench_synth"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, ROOT / "mdtraj_gb300" / "synth.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def _padded(n_atoms: int) -> int:
    return (int(n_atoms) + 3) // 4 * 4


def workload_config(workload: str, n_frames: int, world: int) -> dict:
    """The `config` object of both arms (this project's and the reference's):
    the same keys and values, so that the two lines name one workload.  How
    each arm runs it (device layout, OpenMP threads) is stated outside
    `config`."""
    spec = WORKLOADS[workload]
    if workload.startswith("allpairs"):
        _, A, C, sig, cube, stay = spec
        F = n_frames
        return {"workload": workload, "n_frames": F, "n_atoms": A, "centres": C, "sigma_nm": sig,
                "output": "full symmetric %d x %d float32" % (F, F),
                "l2": "operands (%.2f GB BF16 hi+lo) and output (%.2f GB) larger than L2; no flush"
                      % (3.0 * F * ((A + 63) // 64 * 64) * 2 * 2 / 1e9, 4.0 * F * F / 1e9),
                "parallelism": f"frame shards x{world}"}
    _, A, layout, s_lo, s_hi, exact = spec
    F = n_frames
    nbytes = 12.0 * _padded(A) * F
    small = nbytes < 4 * L2_BYTES
    return {"workload": workload, "n_frames": F, "n_atoms": A, "precentered": False,
            "sigma_nm": [s_lo, s_hi], "exact_copy_fraction": exact,
            "layout": ("%s float32 frames resident in HBM (value); host float32 (F, A, 3) atom-major arrays "
                       "(e2e and the reference's md.rmsd)" % ("axis-major" if layout == 1 else "atom-major")),
            "l2": ("inputs (%.3f GB) fit in L2: 256 MB write + 256 MB read between steps, each step timed alone, "
                   "launches replayed from a CUDA graph" % (nbytes / 1e9)) if small else
                  "inputs (%.1f GB) larger than L2; no flush" % (nbytes / 1e9),
            "parallelism": f"frame shards x{world}"}


def cpu_sample(n_atoms: int, n_sample: int, seed: int, sigma_lo: float, sigma_hi: float):
    synth = _synth()

    rng = np.random.default_rng(seed)
    sig = synth.log_uniform(rng, sigma_lo, sigma_hi, n_sample) if sigma_lo != sigma_hi else sigma_lo
    ref, x = synth.single_reference_frames(n_sample, n_atoms, seed=seed, sigma=sig)
    return ref, x


def time_cpu_reference(n_atoms: int, budget_s: float, sigma_lo: float, sigma_hi: float) -> dict:
    """Times md.rmsd's CPU path (reference kernels, OpenMP, all cores) on a
    bounded sample; returns frames/s and a description."""
    from oracle import cpu

    impl = cpu.best_available()
    n_sample = max(64, min(20_000, int(4e8 // max(n_atoms, 1) // 12)))  # <= ~400 MB sample
    ref, x = cpu_sample(n_atoms, n_sample, 1234, sigma_lo, sigma_hi)
    impl.md_rmsd(x[: min(256, n_sample)].copy(), ref.copy())  # warm up threads / pages
    frames = 0
    t_total = 0.0
    reps = 0
    # md.rmsd centres its inputs in place; repeating it on the same arrays
    # repeats the same work (both centring passes and the msd pass), as a
    # caller looping md.rmsd over a trajectory does.
    while t_total < budget_s or reps < 2:
        t0 = time.perf_counter()
        impl.md_rmsd(x, ref)
        t_total += time.perf_counter() - t0
        frames += n_sample
        reps += 1
        if reps >= 100000:
            break
    return {"value": frames / t_total, "unit": "frames/s", "cores": cpu.n_threads(), "kind": impl.kind,
            "sample": f"{reps} x md.rmsd over {n_sample} frames x {n_atoms} atoms (same generator, "
                      f"{t_total:.1f} s of CPU work, OpenMP threads={cpu.n_threads()})"}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------


def run_gpu(args) -> dict:
    import torch

    import mdtraj_gb300 as md
    from mdtraj_gb300 import _device as D
    from mdtraj_gb300 import _lib, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    # the other workloads run first, on a fresh process: the serving loop's
    # result copies to host memory slow down (measured 730-750 -> 200-530
    # queries/s on the same box) once the process has moved GBs through
    # pageable host memory (the accuracy checks, the host-array leg)
    workloads = None
    if rank == 0 and world == 1 and args.workload == DEFAULT_WORKLOAD and not args.skip_workloads:
        workloads = run_workloads(args)
    F, A, layout, s_lo, s_hi, exact = WORKLOADS[args.workload]
    if args.frames:
        F = args.frames
    Ap = D.padded(A)
    f0, f1 = shard(F, rank, world)
    # ---- device-resident inputs
    ref, x, sig = synth.device_single_reference(F, A, Ap, layout, seed=2024 + rank, device=dev,
                                                sigma_lo=s_lo, sigma_hi=s_hi, exact_fraction=exact)
    torch.cuda.synchronize()
    dref = D.DeviceReference(ref, layout, centre=True, device=dev)
    lib = _lib.lib
    ws = D.empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(F, A), dev)
    out = torch.empty(F, dtype=torch.float32, device=dev)
    stream = D.stream_handle()

    def step():
        _lib.check(lib.gbrmsd_rmsd_to_reference(x.data_ptr(), F, A, Ap, 3 * Ap, layout, _lib.MODE_CENTER,
                                                dref.ws.data_ptr(), None, 0.0, -1, out.data_ptr(), None, None,
                                                ws.data_ptr(), ws.numel(), D.stream_handle()))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    _lib.check(lib.gbrmsd_workspace_status(ws.data_ptr(), stream))
    # A working set that fits in L2 (120 MB at 10,000 x 1,000) is timed with
    # a 256 MB write between steps, each step between its own events, and the
    # step's launches replayed from a CUDA graph (the kernels take tens of
    # microseconds, so launch overhead would otherwise show).
    small = 12.0 * Ap * F < 4 * L2_BYTES
    flush = L2Flush(dev) if small else None
    graph = None
    if small:
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step()
        for _ in range(args.warmup):
            graph.replay()
        torch.cuda.synchronize()
    lib.gbrmsd_profile_enable(0 if small else args.steps)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record()
        for i in range(args.steps):
            if small:
                flush(i)
                ev[i][0].record()
                graph.replay()
                ev[i][1].record()
            else:
                step()
        e1.record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    if small:
        ms_total = float(sum(a.elapsed_time(b) for a, b in ev))
        # the streaming kernel alone, outside the graph, flushed the same way
        lib.gbrmsd_profile_enable(args.steps)
        for i in range(args.steps):
            flush(i + 7)
            step()
        torch.cuda.synchronize()
    else:
        ms_total = e0.elapsed_time(e1)
    kms = np.zeros(args.steps, dtype=np.float32)
    nk = lib.gbrmsd_profile_read(kms.ctypes.data, args.steps)
    lib.gbrmsd_profile_enable(0)
    _lib.check(lib.gbrmsd_workspace_status(ws.data_ptr(), stream))
    ms_step = max_over_ranks(ms_total / args.steps, world)
    value = world * F / (ms_step / 1e3)

    # ---- accuracy on the timed output (exact copies + random frames vs FP64)
    acc = accuracy_check(x, ref, out, F, A, Ap, layout, sig, rank)

    # ---- roofline of the streaming kernel
    peaks = measured_peaks()
    k_ms = float(np.mean(kms[:nk])) if nk > 0 else float("nan")
    alg_bytes = 12.0 * A * F
    achieved = alg_bytes / (k_ms / 1e3) / 1e9
    traffic = traffic_from_profiles("stream_kernel", args.workload)
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": traffic,
            "kernel": "stream_kernel", "kernel_ms": round(k_ms, 4),
            "algorithmic_bytes_per_launch": alg_bytes, "peak_src": peaks["src"]}

    del x
    torch.cuda.empty_cache()
    e2e = None
    if rank == 0 and not args.skip_e2e:
        e2e = run_e2e(args, F, A, s_lo, s_hi, exact, dev)
    cpu_base = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu_base = time_cpu_reference(A, args.cpu_budget, s_lo, s_hi)

    clocks = clk.summary()
    return {
        "metric": "rmsd_frames_per_s",
        "value": round(value, 1),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded, generated on device)",
        "config": workload_config(args.workload, F, world),
        "roofline": roof,
        "cpu_baseline": cpu_base,
        "e2e": e2e,
        # one streaming kernel per call: with one unit per frame (the cost
        # model's choice at both benchmark sizes) its finisher warp solves QCP
        # in the same launch
        "gpu_launches": args.steps,
        "clocks": clocks,
        "accuracy": acc,
        "workloads": workloads,
    }


def run_workloads(args) -> dict:
    """The other benchmark workloads, each shortened to a few seconds, run
    before the headline workload (whose timed region is device-only) so that
    one default run carries evidence for all of them (each entry has its own
    clock record; the serving loop runs first, while the process has moved
    nothing through host memory yet):
      cfg0 single_reference_10000x1000  md.rmsd's class of input: graph-replayed
           step, streaming-kernel roofline, accuracy vs FP64 and the reference;
      cfg2 allpairs_20000x2000  tensor-core matrix vs the FP32 CUDA-core tiles
           (ratio), 100,000 sampled pairs vs FP64;
      cfg3 ragged_512  one persistent graph launch vs 512 separate launches;
      cfg4 serving_500000x300  p50/p99 and queries/s at 100, 1,000 and 10,000
           offered requests/s beside one request per launch on FP32 tiles
           (fewer requests per rate than the full sweep of --workload
           serving_500000x300)."""
    import torch

    def sub(workload, fn, **kw):
        ns = argparse.Namespace(**vars(args))
        ns.workload, ns.frames, ns.skip_e2e, ns.skip_cpu, ns.warmup = workload, None, True, True, 3
        for k, v in kw.items():
            setattr(ns, k, v)
        t0 = time.perf_counter()
        try:
            r = fn(ns)
        except Exception as exc:  # one workload failing must not take the headline line with it
            r = {"error": f"{type(exc).__name__}: {exc}"[:400]}
        r["wall_s"] = round(time.perf_counter() - t0, 1)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        return r

    def keep(r, keys):
        return {k: r[k] for k in keys if k in r}

    out = {}
    r = sub("serving_500000x300", run_serving, rates=(100, 1000, 10000), serve_seconds=1.0, serve_max=400,
            baseline_max=100)
    serving_rec = keep(r, ["value", "unit", "sweep", "speedup_at_top_rate", "roofline", "kernel_compare", "accuracy",
                           "clocks", "config", "error", "wall_s"])
    r = sub("single_reference_10000x1000", run_gpu, steps=20)
    out["cfg0_single_reference_10000x1000"] = keep(r, ["value", "unit", "ms_per_step", "steps", "roofline", "accuracy",
                                                       "clocks", "config", "error", "wall_s"])
    r = sub("allpairs_20000x2000", run_allpairs, steps=3)
    out["cfg2_allpairs_20000x2000"] = keep(r, ["value", "unit", "ms_per_step", "steps", "roofline", "fp32_cuda_core",
                                               "refined_pairs", "accuracy", "clocks", "config", "error", "wall_s"])
    r = sub("ragged_512", run_ragged, steps=3)
    out["cfg3_ragged_512"] = keep(r, ["value", "unit", "ms_per_step", "steps", "roofline", "separate_launches",
                                      "accuracy", "clocks", "config", "error", "wall_s"])
    out["cfg4_serving_500000x300"] = serving_rec
    return out


def accuracy_check(x, ref, out, F, A, Ap, layout, sig, rank) -> dict:
    """max/RMS |gpu - FP64 Kabsch| on every exact copy plus random frames."""
    import torch

    from oracle import fp64

    rng = np.random.default_rng(7 + rank)
    exact_idx = np.flatnonzero(sig == 0.0)
    rand_idx = rng.choice(F, size=min(F, 2000 if A >= 5000 else 10000), replace=False)
    idx = np.unique(np.concatenate([exact_idx, rand_idx, [0]]))[:6000]
    sel = x[torch.from_numpy(idx).to(x.device)]
    if layout == 1:
        fr = sel[:, :, :A].transpose(1, 2).contiguous().cpu().numpy()
    else:
        fr = sel.view(len(idx), Ap, 3)[:, :A].contiguous().cpu().numpy()
    ref_h = ref.cpu().numpy()
    want = fp64.kabsch_rmsd(fr, ref_h)
    got = out[torch.from_numpy(idx).to(out.device)].cpu().numpy().astype(np.float64)
    err = np.abs(got - want)
    ex = np.isin(idx, exact_idx)
    res = {"checked_frames": int(len(idx)), "exact_copies": int(ex.sum()),
           "max_err_nm": float(err.max()), "rms_err_nm": float(np.sqrt((err ** 2).mean())),
           "max_err_exact_copies_nm": float(err[ex].max()) if ex.any() else None,
           "oracle": "FP64 Kabsch/SVD (oracle/fp64.py)"}
    # the same frames through the reference's own float32 md.rmsd (its CPU
    # kernels compiled from its sources): the second half of the parity bar,
    # |gpu - ref| <= 1e-4 + |ref - fp64|
    try:
        from oracle import cpu

        impl = cpu.best_available()
        r = impl.md_rmsd(np.ascontiguousarray(fr, dtype=np.float32), np.ascontiguousarray(ref_h, dtype=np.float32))
        r = r.astype(np.float64)
        ref_err = np.abs(r - want)
        bad = np.abs(got - r) > 1e-4 + ref_err
        res["vs_reference"] = {"kind": impl.kind, "frames_outside_bar": int(bad.sum()),
                               "max_abs_gpu_minus_ref_nm": float(np.abs(got - r).max()),
                               "reference_max_err_vs_fp64_nm": float(ref_err.max()),
                               "reference_frames_off_fp64_by_more_than_1e-4": int((ref_err > 1e-4).sum()),
                               "bar": "|gpu - ref| <= 1e-4 nm + |ref - fp64|"}
    except (OSError, FileNotFoundError) as exc:
        res["vs_reference"] = {"unavailable": str(exc)}
    return res


def run_e2e(args, F, A, s_lo, s_hi, exact, dev) -> dict:
    """md.rmsd through the drop-in on host numpy buffers (atom-major, the
    Trajectory.xyz layout).  Host data come from the device generator."""
    import torch

    import mdtraj_gb300 as md
    from mdtraj_gb300 import _device as D
    from mdtraj_gb300 import synth

    Fe = F if args.e2e_frames is None else min(F, args.e2e_frames)
    Ap = A  # host layout: unpadded (F, A, 3)
    ref, xd, _ = synth.device_single_reference(Fe, A, D.padded(A), 0, seed=99, device=dev,
                                               sigma_lo=s_lo, sigma_hi=s_hi, exact_fraction=exact)
    host = np.empty((Fe, A, 3), dtype=np.float32)
    host_t = torch.from_numpy(host)
    step = 8192
    for s in range(0, Fe, step):
        e = min(Fe, s + step)
        host_t[s:e].copy_(xd[s:e].view(e - s, D.padded(A), 3)[:, :A])
    ref_h = ref.cpu().numpy()
    del xd
    torch.cuda.empty_cache()

    class Obj:
        def __init__(self, xyz):
            self.xyz = xyz
            self._rmsd_traces = None

    target = Obj(host)
    reference = Obj(ref_h[None].copy())
    for _ in range(max(1, min(args.warmup, 2))):
        md.rmsd(target, reference, 0)
    torch.cuda.synchronize()
    times, host_steps = [], []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        md.rmsd(target, reference, 0)
        times.append(time.perf_counter() - t0)
        # where the call's host time went (page locking, unlocking, the wait
        # for the GPU at the end), per step
        st = D.LAST_HOST_STREAM
        host_steps.append({"lock_ms": round(st.get("lock_s", 0.0) * 1e3, 1), "unlock_ms": round(st.get("unlock_s", 0.0) * 1e3, 1),
                     "wait_ms": round(st.get("wait_s", 0.0) * 1e3, 1), "all_locked": st.get("all_locked")})
    t = float(np.mean(times))
    t_med = float(np.median(times))
    # inbound: every frame and the reference frame; outbound: one RMSD per
    # frame and the in-place centring of every frame written back
    h2d, d2h = int(Fe * A * 12 + A * 12), int(Fe * 4 + Fe * A * 12)
    link = host_link_peak(dev)
    res = {"value": round(Fe / t, 1), "unit": "frames/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": round(t * 1e3, 2),
           "median_ms_per_step": round(t_med * 1e3, 2), "median_value": round(Fe / t_med, 1),
           "frames": Fe, "api": "mdtraj_gb300.rmsd(target, reference, 0) on host float32 arrays",
           "steps": args.e2e_steps, "step_ms": [round(x * 1e3, 2) for x in times], "step_host": host_steps,
           "host_link": link}
    if link.get("both_gbs"):
        # the step's host traffic over the link's measured two-way rate
        res["host_link_frac"] = round((h2d + d2h) / t / 1e9 / link["both_gbs"], 4)
        res["host_link_frac_median"] = round((h2d + d2h) / t_med / 1e9 / link["both_gbs"], 4)
    return res


def host_link_peak(dev, nbytes: int = 4 << 30, chunk: int = 256 << 20, reps: int = 3) -> dict:
    """Measured host<->device rate of this machine with the copy engines:
    `nbytes` of page-locked host memory to the device, the device to a
    second page-locked buffer, each alone and both at once on two streams,
    one cudaMemcpyAsync (torch copy_) per `chunk`.  Best of `reps`."""
    import torch

    try:
        src = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        dst = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        d_in = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        d_out = torch.ones(nbytes, dtype=torch.uint8, device=dev)
    except RuntimeError as exc:
        return {"unavailable": str(exc).splitlines()[0]}
    s1, s2 = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    n = nbytes // chunk

    def run(h2d: bool, d2h: bool) -> float:
        best = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            for k in range(n):
                sl = slice(k * chunk, (k + 1) * chunk)
                if h2d:
                    with torch.cuda.stream(s1):
                        d_in[sl].copy_(src[sl], non_blocking=True)
                if d2h:
                    with torch.cuda.stream(s2):
                        dst[sl].copy_(d_out[sl], non_blocking=True)
            torch.cuda.synchronize(dev)
            best = min(best, time.perf_counter() - t0)
        return best

    t_in, t_out, t_both = run(True, False), run(False, True), run(True, True)
    res = {"h2d_gbs": round(nbytes / t_in / 1e9, 1), "d2h_gbs": round(nbytes / t_out / 1e9, 1),
           "both_gbs": round(2 * nbytes / t_both / 1e9, 1),
           "method": "%d MB page-locked each way, %d MB cudaMemcpyAsync chunks, copy engines, best of %d"
                     % (nbytes >> 20, chunk >> 20, reps)}
    del src, dst, d_in, d_out
    torch.cuda.empty_cache()
    return res


# ---------------------------------------------------------------------------
# All-pairs matrix workload
# ---------------------------------------------------------------------------


def run_allpairs(args) -> dict:
    """Symmetric RMSD matrix of 20,000 frames x 2,000 atoms (random walk over
    50 metastable centres, sigma 0.1 nm, random rotations).  One step = the
    full matrix with the split-BF16 tensor-core path; the plain FP32
    CUDA-core path is timed on the same input for comparison."""
    import torch

    from mdtraj_gb300 import _device as D
    from mdtraj_gb300 import _lib, synth
    from mdtraj_gb300.allpairs import METHODS

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    F, A, C, sig, cube, stay = WORKLOADS[args.workload]
    if args.frames:
        F = args.frames
    Ap = D.padded(A)
    labels, x = synth.device_metastable_walk(F, A, Ap, seed=77 + rank, device=dev, n_centres=C, sigma=sig,
                                             cube=cube, stay=stay)
    lib = _lib.lib
    ws = D.empty_bytes(lib.gbrmsd_allpairs_workspace_bytes(F, A), dev)
    out = torch.empty((F, F), dtype=torch.float32, device=dev)
    stream = D.stream_handle()

    def step(method):
        _lib.check(lib.gbrmsd_allpairs(x.data_ptr(), F, A, Ap, 3 * Ap, _lib.ATOM_MAJOR, 1, METHODS[method],
                                       out.data_ptr(), ws.data_ptr(), ws.numel(), stream))

    def timed(method, steps, warmup):
        for _ in range(warmup):
            step(method)
        torch.cuda.synchronize()
        lib.gbrmsd_profile_enable(steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            step(method)
        e1.record()
        torch.cuda.synchronize()
        k = np.zeros(steps, dtype=np.float32)
        n = lib.gbrmsd_profile_read(k.ctypes.data, steps)
        lib.gbrmsd_profile_enable(0)
        refined = np.zeros(1, dtype=np.int32)
        _lib.check(lib.gbrmsd_allpairs_status(ws.data_ptr(), refined.ctypes.data, stream))
        return e0.elapsed_time(e1) / steps, float(np.mean(k[:n])), int(refined[0])

    with ClockSampler(local) as clk:
        ms_step, k_ms, refined = timed("tensor", args.steps, args.warmup)
    out_t = out.clone()
    fp32_steps = max(1, min(2, args.steps))
    ms_fp32, k_fp32, _ = timed("fp32", fp32_steps, 1)
    pairs = F * (F - 1) / 2
    value = world * pairs / (ms_step / 1e3)
    peaks = measured_peaks()
    p = ROOT / "MEASURED_PEAKS.json"
    bf16_peak = json.loads(p.read_text())["bf16_tflops"] if p.exists() else 1900.0
    alg_flops = 3 * 18.0 * A * pairs            # three BF16 products of 9 MACs per atom per pair
    achieved = alg_flops / (k_ms / 1e3) / 1e12
    roof = {"bound": "tensor", "achieved": round(achieved, 1), "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": round(achieved / bf16_peak, 4), "traffic": traffic_from_profiles("allpairs_tc_kernel", args.workload),
            "kernel": "allpairs_tc_kernel", "kernel_ms": round(k_ms, 4),
            "algorithmic_flops_per_launch": alg_flops, "peak_src": "measured" if p.exists() else "fallback"}
    acc = allpairs_accuracy(x, out_t, F, A, Ap, rank)
    cpu_base = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu_base = time_cpu_allpairs(A, args.cpu_budget, C, sig, cube)
    e2e = None
    if rank == 0 and not args.skip_e2e:
        e2e = allpairs_e2e(x, F, A, Ap, args)
    return {
        "metric": "rmsd_pairs_per_s",
        "value": round(value, 1),
        "unit": "pairs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16x3 (split hi/lo, f32 accumulate)",
        "data": "synthetic (seeded, generated on device)",
        "config": workload_config(args.workload, F, world),
        "roofline": roof,
        "fp32_cuda_core": {"ms_per_step": round(ms_fp32, 3), "kernel_ms": round(k_fp32, 3),
                           "pairs_per_s": round(pairs / (ms_fp32 / 1e3), 1),
                           "tensor_speedup_kernel": round(k_fp32 / k_ms, 2),
                           "tensor_speedup_step": round(ms_fp32 / ms_step, 2)},
        "refined_pairs": refined,
        "cpu_baseline": cpu_base,
        "e2e": e2e,
        "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
        "accuracy": acc,
    }


def allpairs_accuracy(x, out, F, A, Ap, rank, n_pairs=100_000) -> dict:
    from oracle import fp64

    rng = np.random.default_rng(11 + rank)
    i = rng.integers(0, F, n_pairs)
    j = rng.integers(0, F, n_pairs)
    keep = i != j
    pairs = np.stack([i[keep], j[keep]], 1)
    frames = x.view(F, Ap, 3)[:, :A].cpu().numpy()
    want = fp64.kabsch_rmsd_pairs(frames, pairs)
    got = out[pairs[:, 0], pairs[:, 1]].cpu().numpy().astype(np.float64)
    err = np.abs(got - want)
    return {"checked_pairs": int(len(pairs)), "max_err_nm": float(err.max()), "rms_err_nm": float(np.sqrt((err ** 2).mean())),
            "oracle": "FP64 Kabsch/SVD (oracle/fp64.py)"}


def time_cpu_allpairs(A, budget_s, C, sig, cube) -> dict:
    """Reference CPU path of the clustering loop: precentered md.rmsd rows
    (getMultipleRMSDs_atom_major of the reference kernels) over a sample of
    rows of a 20,000-frame trajectory sample; pairs/s."""
    from oracle import cpu

    synth = _synth()
    impl = cpu.best_available()
    n_frames = 4000
    labels, x = synth.metastable_walk(n_frames, A, n_centres=C, seed=5, sigma=sig, cube=cube)
    g = impl.center_inplace(x)
    rows = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s and rows < n_frames:
        impl.multiple(x, x, g, g, rows, axis_major=False)
        rows += 1
    dt = time.perf_counter() - t0
    return {"value": rows * n_frames / dt, "unit": "pairs/s", "cores": cpu.n_threads(), "kind": impl.kind,
            "sample": f"{rows} rows x {n_frames} frames x {A} atoms of md.rmsd(traj, traj, i, precentered=True) "
                      f"({dt:.1f} s, OpenMP threads={cpu.n_threads()})"}


def allpairs_e2e(x, F, A, Ap, args) -> dict:
    """mdtraj_gb300.allpairs_rmsd on a host numpy trajectory: host->device
    coordinates, the matrix, device->host of the full F x F result."""
    import torch

    import mdtraj_gb300 as md

    host = x.view(F, Ap, 3)[:, :A].contiguous().cpu().numpy()
    md.allpairs_rmsd(host[:64], method="tensor")
    torch.cuda.synchronize()
    times = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        md.allpairs_rmsd(host, method="tensor")
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    return {"value": round(F * (F - 1) / 2 / t, 1), "unit": "pairs/s", "h2d_bytes_per_step": int(F * A * 12),
            "d2h_bytes_per_step": int(F * F * 4), "ms_per_step": round(t * 1e3, 2),
            "api": "mdtraj_gb300.allpairs_rmsd(host float32 (F, A, 3), method='tensor')", "steps": args.e2e_steps}


# ---------------------------------------------------------------------------
# Ragged batch workload
# ---------------------------------------------------------------------------


def ragged_setup(args, dev):
    from mdtraj_gb300 import RaggedBatch, synth

    nseg, alo, ahi, flo, fhi, sig = WORKLOADS[args.workload]
    if args.frames:
        nseg = min(nseg, args.frames)
    atoms, frames = synth.ragged_shapes(nseg, seed=3, atoms=(alo, ahi), frames=(flo, fhi))
    off, padded, total = RaggedBatch.layout(atoms, frames)
    import torch

    x = torch.empty(total, dtype=torch.float32, device=dev)
    for s in range(nseg):
        view = x[int(off[s]):int(off[s]) + int(frames[s]) * 3 * int(padded[s])].view(int(frames[s]),
                                                                                    3 * int(padded[s]))
        synth.device_single_reference(int(frames[s]), int(atoms[s]), int(padded[s]), 0, seed=50_000 + s, device=dev,
                                      sigma_lo=sig, sigma_hi=sig, out=view)
    return atoms, frames, off, padded, x


def run_ragged(args) -> dict:
    """512 trajectories (atoms log-uniform in [50, 20000], frames uniform in
    [100, 5000]), each md.rmsd'd against its own frame 0.  One step = one
    persistent ragged launch replayed from a CUDA graph; compared with one
    single-reference call per trajectory on the same GPU."""
    import torch

    from mdtraj_gb300 import RaggedBatch
    from mdtraj_gb300 import _device as D
    from mdtraj_gb300 import _lib, autotune

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    atoms, frames, off, padded, x = ragged_setup(args, dev)
    torch.cuda.synchronize()
    batch = RaggedBatch(packed=(x, atoms, frames), autotune=True)
    tune = autotune.load_cache().get(autotune.shape_bucket(atoms, frames), {})
    batch.capture()
    lib = _lib.lib
    for _ in range(args.warmup):
        batch.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            batch.replay()
        e1.record()
        torch.cuda.synchronize()
    ms_step = e0.elapsed_time(e1) / args.steps
    # events recorded inside a captured graph time nothing: the stream kernel's
    # own duration comes from the same launches issued directly
    lib.gbrmsd_profile_enable(args.steps)
    for _ in range(args.steps):
        batch.run()
    torch.cuda.synchronize()
    kms = np.zeros(args.steps, dtype=np.float32)
    nk = lib.gbrmsd_profile_read(kms.ctypes.data, args.steps)
    lib.gbrmsd_profile_enable(0)
    F_tot = int(frames.sum())
    value = world * F_tot / (ms_step / 1e3)
    k_ms = float(np.mean(kms[:nk])) if nk else float("nan")
    alg = float((12.0 * atoms.astype(np.float64) * frames).sum())
    peaks = measured_peaks()
    roof = {"bound": "hbm", "achieved": round(alg / (k_ms / 1e3) / 1e9, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(alg / (k_ms / 1e3) / 1e9 / peaks["hbm_gbs"], 4),
            "traffic": traffic_from_profiles("ragged_stream_kernel", args.workload), "kernel": "ragged_stream_kernel",
            "kernel_ms": round(k_ms, 4), "algorithmic_bytes_per_launch": alg, "peak_src": peaks["src"]}
    # the same work as one single-reference call per trajectory
    stream = D.stream_handle()
    refs, wss, outs = [], [], []
    for s in range(len(atoms)):
        A, Ap, F = int(atoms[s]), int(padded[s]), int(frames[s])
        seg = x[int(off[s]):int(off[s]) + F * 3 * Ap]
        refs.append(D.DeviceReference(seg[:3 * Ap].view(Ap, 3)[:A], _lib.ATOM_MAJOR, centre=True, device=dev))
        wss.append(D.empty_bytes(lib.gbrmsd_rmsd_workspace_bytes(F, A), dev))
        outs.append(torch.empty(F, dtype=torch.float32, device=dev))

    def separate():
        for s in range(len(atoms)):
            A, Ap, F = int(atoms[s]), int(padded[s]), int(frames[s])
            _lib.check(lib.gbrmsd_rmsd_to_reference(x.data_ptr() + int(off[s]) * 4, F, A, Ap, 3 * Ap, 0, 0,
                                                    refs[s].ws.data_ptr(), None, 0.0, 0, outs[s].data_ptr(), None,
                                                    None, wss[s].data_ptr(), wss[s].numel(), stream))

    separate()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(max(1, min(args.steps, 3))):
        separate()
    e1.record()
    torch.cuda.synchronize()
    ms_sep = e0.elapsed_time(e1) / max(1, min(args.steps, 3))
    got = batch.out.cpu().numpy()
    sep = np.concatenate([o.cpu().numpy() for o in outs])
    acc = ragged_accuracy(x, atoms, frames, off, padded, got)
    cpu_base = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu_base = ragged_cpu(x, atoms, frames, off, padded, args.cpu_budget)
    return {
        "metric": "rmsd_frames_per_s", "value": round(value, 1), "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, generated on device)",
        "config": {"workload": args.workload, "segments": int(len(atoms)), "frames": F_tot,
                   "atoms_range": [int(atoms.min()), int(atoms.max())], "bytes": alg,
                   "launch": "one persistent ragged launch replayed from a CUDA graph",
                   "tuned": {k: tune.get(k) for k in ("config", "max_unit_quads", "ms")},
                   "l2": "inputs (%.1f GB) larger than L2; no flush" % (alg / 1e9)},
        "roofline": roof,
        "separate_launches": {"launches": int(len(atoms)), "ms_per_step": round(ms_sep, 3),
                              "frames_per_s": round(F_tot / (ms_sep / 1e3), 1),
                              "ragged_speedup": round(ms_sep / ms_step, 3),
                              "max_abs_diff_vs_ragged": float(np.abs(sep - got).max())},
        "cpu_baseline": cpu_base, "e2e": None, "gpu_launches": 3 * args.steps, "clocks": clk.summary(),
        "accuracy": acc,
    }


def ragged_accuracy(x, atoms, frames, off, padded, got, n_seg=24, per_seg=64) -> dict:
    from oracle import fp64

    rng = np.random.default_rng(0)
    bounds = np.concatenate([[0], np.cumsum(frames)])
    errs = []
    for s in rng.choice(len(atoms), size=min(n_seg, len(atoms)), replace=False):
        A, Ap, F = int(atoms[s]), int(padded[s]), int(frames[s])
        fr = x[int(off[s]):int(off[s]) + F * 3 * Ap].view(F, Ap, 3)[:, :A]
        idx = np.unique(np.concatenate([[0], rng.choice(F, size=min(per_seg, F), replace=False)]))
        host = fr[idx].cpu().numpy()
        ref = fr[0].cpu().numpy()
        errs.append(np.abs(got[bounds[s] + idx] - fp64.kabsch_rmsd(host, ref)))
    e = np.concatenate(errs)
    return {"checked_frames": int(e.size), "max_err_nm": float(e.max()), "rms_err_nm": float(np.sqrt((e ** 2).mean())),
            "oracle": "FP64 Kabsch/SVD (oracle/fp64.py)"}


def ragged_cpu(x, atoms, frames, off, padded, budget_s) -> dict:
    """The reference's per-trajectory md.rmsd loop over a segment sample."""
    from oracle import cpu

    impl = cpu.best_available()
    rng = np.random.default_rng(1)
    order = rng.permutation(len(atoms))
    done_frames, done_atom_frames, t_total = 0, 0, 0.0
    for s in order:
        A, Ap, F = int(atoms[s]), int(padded[s]), int(frames[s])
        host = x[int(off[s]):int(off[s]) + F * 3 * Ap].view(F, Ap, 3)[:, :A].contiguous().cpu().numpy()
        t0 = time.perf_counter()
        impl.md_rmsd(host, host[0])
        t_total += time.perf_counter() - t0
        done_frames += F
        done_atom_frames += F * A
        if t_total > budget_s:
            break
    # scale to the whole batch by atom-frames (the work is linear in them)
    all_af = float((atoms.astype(np.float64) * frames).sum())
    frames_per_s = float(frames.sum()) / (t_total * all_af / done_atom_frames)
    return {"value": frames_per_s, "unit": "frames/s", "cores": cpu.n_threads(), "kind": impl.kind,
            "sample": f"md.rmsd(t, t, 0) on {done_frames} frames of a random segment sample "
                      f"({t_total:.1f} s), scaled to the batch by atom-frames"}


def run_reference(args) -> dict:
    rank, world, local = dist_env()
    if rank != 0:
        return None
    if args.workload.startswith("allpairs"):
        F, A, C, sig, cube, stay = WORKLOADS[args.workload]
        base = time_cpu_allpairs(A, args.cpu_budget, C, sig, cube)
        return {"impl": "reference", "metric": "rmsd_pairs_per_s", "value": round(base["value"], 1),
                "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(F * (F - 1) / 2 / base["value"] * 1e3, 2), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": workload_config(args.workload, args.frames or F, world),
                "how": "the reference's CPU kernels on all host cores; each step timed on a bounded row sample",
                "cpu_baseline": base,
                "e2e": {"value": round(base["value"], 1), "unit": "pairs/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
    F, A, layout, s_lo, s_hi, exact = WORKLOADS[args.workload]
    if args.frames:
        F = args.frames
    base = time_cpu_reference(A, args.cpu_budget, s_lo, s_hi)
    per_step_s = F / base["value"]
    return {
        "impl": "reference",
        "metric": "rmsd_frames_per_s",
        "value": round(base["value"], 1),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(per_step_s * 1e3, 2),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": workload_config(args.workload, F, world),
        "how": ("md.rmsd's CPU path (the reference's centring and msd kernels, OpenMP over all host cores) on "
                "host atom-major arrays; each step timed on a bounded frame sample"),
        "cpu_baseline": base,
        "e2e": {"value": round(base["value"], 1), "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# Serving workload
# ---------------------------------------------------------------------------


def serving_requests(db_host_frames, frame_ids, n, rate, seed, max_q, slice_range, n_db):
    """n requests: query frames log-uniform in [1, max_q]; half against the
    full database, half against a contiguous slice of uniform length in
    slice_range; Poisson arrivals at `rate` per second.  Queries are database
    frames (host copies in db_host_frames, indexed through frame_ids) plus
    0.05 nm noise, a random rotation and a translation."""
    from mdtraj_gb300 import serving, synth

    rng = np.random.default_rng(seed)
    reqs, t = [], 0.0
    lo, hi = slice_range[0], min(slice_range[1], n_db)
    for k in range(n):
        Q = int(np.clip(np.floor(synth.log_uniform(rng, 1, max_q + 1, 1)[0]), 1, max_q))
        if rng.random() < 0.5:
            a, b = 0, n_db
        else:
            ln = int(rng.integers(min(lo, n_db), hi + 1))
            a = int(rng.integers(0, n_db - ln + 1))
            b = a + ln
        pick = rng.integers(0, len(frame_ids), Q)
        q = synth.perturbed_queries(db_host_frames, pick, seed=int(rng.integers(1 << 30)))
        t += rng.exponential(1.0 / rate)
        reqs.append(serving.Request(queries=q, db0=a, db1=b, arrival=t, rid=k))
    return reqs


def run_serving(args) -> dict:
    """A 500,000-frame x 300-atom database resident in HBM (Gaussian-chain
    backbones) answering Poisson streams of query sets (1-256 frames each,
    full database or a slice) at offered rates from 100 to 10,000 requests/s.
    Continuous batching over split-BF16 tensor-core cross tiles is compared
    with one request per launch on the plain FP32 CUDA-core tiles, on the
    same requests and the same GPU.  Latency = arrival to results in host
    memory."""
    import torch

    from mdtraj_gb300 import _lib, cross, serving, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    F, A, rates, max_q, slice_range = WORKLOADS[args.workload]
    rates = getattr(args, "rates", None) or rates
    if args.frames:
        F = args.frames
    t_setup = time.perf_counter()
    db_x = synth.gaussian_chain(F, A, seed=2024 + rank, device=dev)
    dbs = cross.FrameSet.from_frames(db_x, device=dev)
    frame_ids = np.random.default_rng(99).integers(0, F, 4096)
    host_frames = db_x[torch.from_numpy(frame_ids).to(dev)].cpu().numpy()
    del db_x
    torch.cuda.empty_cache()
    setup_s = time.perf_counter() - t_setup
    lib = _lib.lib
    server = serving.RmsdServer(dbs, method="tensor", query_capacity=16384, hbm_budget_bytes=48 << 30, slots=3,
                                host_pool_bytes=4 << 30)
    base = serving.RmsdServer(dbs, method="fp32", query_capacity=1024, hbm_budget_bytes=48 << 30, slots=1,
                              max_batch_requests=1)
    # the rate of the result copies into the page-locked host result pool on this machine, now
    probe = torch.ones(256 << 20, dtype=torch.uint8, device=dev)
    from mdtraj_gb300 import _device as Dv
    s_probe = torch.cuda.current_stream().cuda_stream
    Dv.copy_rows(server.hpool.ptr(0), probe.numel(), probe.data_ptr(), probe.numel(), probe.numel(), 1, 2, s_probe)
    torch.cuda.synchronize()
    t_probe = time.perf_counter()
    for _ in range(4):
        Dv.copy_rows(server.hpool.ptr(0), probe.numel(), probe.data_ptr(), probe.numel(), probe.numel(), 1, 2, s_probe)
    torch.cuda.synchronize()
    pool_gbs = 4 * probe.numel() / (time.perf_counter() - t_probe) / 1e9
    del probe
    warm = serving_requests(host_frames, frame_ids, 24, 1e6, 1, max_q, slice_range, F)
    server.serve(warm, realtime=False, keep_results=False)
    base.serve(serving_requests(host_frames, frame_ids, 4, 1e6, 2, max_q, slice_range, F), realtime=False,
               keep_results=False)
    sweep = []
    with ClockSampler(local) as clk:
        for k, rate in enumerate(rates):
            n = max(20, min(int(rate * args.serve_seconds), args.serve_max))
            reqs = serving_requests(host_frames, frame_ids, n, rate, 1000 + k, max_q, slice_range, F)
            b0 = server.n_batches
            l0 = len(server.batch_log)
            t_serve = time.perf_counter()
            done = server.serve(reqs, realtime=True, keep_results=False)
            t_serve = time.perf_counter() - t_serve
            row = {"offered_rate": rate, "requests": n, "continuous": serving.latency_summary(done)}
            row["continuous"]["mean_batch_requests"] = round(n / max(1, server.n_batches - b0), 2)
            # where the time went: the batches' GPU time against the loop's wall time
            row["continuous"]["batches"] = serving.batch_summary(server.batch_log[l0:])
            row["continuous"]["batches"]["wall_s"] = round(t_serve, 3)
            nb = min(n, args.baseline_max)
            reqs_b = [serving.Request(queries=r.queries, db0=r.db0, db1=r.db1, arrival=r.arrival, rid=r.rid)
                      for r in reqs[:nb]]
            row["one_per_launch_fp32"] = serving.latency_summary(base.serve(reqs_b, realtime=True,
                                                                             keep_results=False))
            sweep.append(row)
            print(json.dumps(row), file=sys.stderr, flush=True)
    top = sweep[-1]
    # kernel-level: one fixed batch (32 requests x 80 query frames, full database)
    Qb, Rb = 80, 32
    qset = cross.FrameSet(Qb * Rb, A, dev)
    qx = torch.from_numpy(synth.perturbed_queries(host_frames, np.arange(Qb * Rb) % len(frame_ids), seed=5)
                          .reshape(Qb * Rb, -1)).to(dev)
    qset.prepare(qx, 0)
    outb = torch.empty((Rb, Qb, F), dtype=torch.float32, device=dev)
    table = cross.request_table([(outb[r].data_ptr(), r * Qb, Qb, 0, F) for r in range(Rb)])
    wsb = cross.CrossWorkspace(dev).get(F, Qb * Rb, Rb)
    stream = torch.cuda.current_stream().cuda_stream

    def kernel_ms(method, reps):
        # an NVTX range marks these launches for profilers (ncu --nvtx-include kernel_compare/)
        torch.cuda.nvtx.range_push("kernel_compare")
        try:
            return _kernel_ms(method, reps)
        finally:
            torch.cuda.nvtx.range_pop()

    def _kernel_ms(method, reps):
        cross.cross_launch(dbs, F, qset, table, Rb, method, wsb, stream)
        torch.cuda.synchronize()
        lib.gbrmsd_profile_enable(reps)
        for _ in range(reps):
            cross.cross_launch(dbs, F, qset, table, Rb, method, wsb, stream)
        torch.cuda.synchronize()
        kk = np.zeros(reps, dtype=np.float32)
        nn = lib.gbrmsd_profile_read(kk.ctypes.data, reps)
        lib.gbrmsd_profile_enable(0)
        return float(np.mean(kk[:nn]))

    k_tc = kernel_ms("tensor", 3)
    got_tc = outb.cpu().numpy()
    k_fp = kernel_ms("fp32", 1)
    pairs_b = float(Qb * Rb) * F
    p = ROOT / "MEASURED_PEAKS.json"
    bf16_peak = json.loads(p.read_text())["bf16_tflops"] if p.exists() else 1900.0
    alg = 3 * 18.0 * A * pairs_b
    ach = alg / (k_tc / 1e3) / 1e12
    roof = {"bound": "tensor", "achieved": round(ach, 1), "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": round(ach / bf16_peak, 4), "traffic": traffic_from_profiles("cross_tc_kernel", args.workload),
            "kernel": "allpairs_tc_kernel<cross>", "kernel_ms": round(k_tc, 4), "algorithmic_flops_per_launch": alg,
            "launch": "%d requests x %d query frames vs %d database frames" % (Rb, Qb, F),
            "peak_src": "measured" if p.exists() else "fallback"}
    # accuracy: sampled entries of the fixed batch against the FP64 oracle
    from oracle import fp64

    rng = np.random.default_rng(7)
    qh = qx.view(Qb * Rb, A, 3).cpu().numpy()
    errs = []
    for _ in range(40):
        qi = int(rng.integers(Qb * Rb))
        cols = rng.integers(0, F, 50)
        dbf = dbs_frames(dbs, cols, A)
        want = fp64.kabsch_rmsd(dbf, qh[qi])
        errs.append(np.abs(got_tc[qi // Qb, qi % Qb, cols] - want))
    e = np.concatenate(errs)
    cpu_base = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu_base = serving_cpu(dbs, F, A, qh[0], args.cpu_budget, top)
    h2d = float(np.mean([r.queries.nbytes for r in reqs]))
    d2h = float(np.mean([r.result_bytes for r in reqs]))
    return {
        "metric": "serving_queries_per_s", "value": top["continuous"]["queries_per_s"], "unit": "queries/s",
        "n_gpus": world, "steps": len(rates), "warmup": 1,
        "ms_per_step": round(1e3 / max(top["continuous"]["queries_per_s"], 1e-9), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 (split hi/lo, f32 accumulate)",
        "data": "synthetic (seeded Gaussian-chain database generated on device; perturbed database frames as queries)",
        "config": {"workload": args.workload, "db_frames": F, "n_atoms": A, "offered_rates": list(rates),
                   "query_frames": "log-uniform 1-%d" % max_q, "db_range": "full (50%%) or slice %d-%d" % slice_range,
                   "slots": len(server.slots), "query_capacity": server.qcap, "setup_s": round(setup_s, 1),
                   "latency": "arrival to results in pinned host memory",
                   "host_result_pool_gb": round(server.hpool.buf.nbytes / 1e9, 1),
                   "host_result_pool_locked": bool(server.hpool.locked),
                   "host_result_pool_copy_gbs": round(pool_gbs, 1),
                   "l2": "database (%.1f GB prepared) larger than L2; no flush" % (dbs.buf.numel() / 1e9)},
        "sweep": sweep,
        "speedup_at_top_rate": round(top["continuous"]["queries_per_s"] /
                                     max(1e-9, top["one_per_launch_fp32"]["queries_per_s"]), 2),
        "roofline": roof,
        "kernel_compare": {"tensor_ms": round(k_tc, 3), "fp32_ms": round(k_fp, 3),
                           "tensor_vs_fp32": round(k_fp / k_tc, 2), "pairs": pairs_b},
        "accuracy": {"checked_pairs": int(e.size), "max_err_nm": float(e.max()),
                     "rms_err_nm": float(np.sqrt((e ** 2).mean())), "oracle": "FP64 Kabsch/SVD (oracle/fp64.py)"},
        "cpu_baseline": cpu_base,
        "e2e": {"value": top["continuous"]["queries_per_s"], "unit": "queries/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "note": "per request: query frames in, RMSD rows out"},
        "gpu_launches": int(server.n_batches * 3),
        "clocks": clk.summary(),
    }


def dbs_frames(dbs, idx, A):
    """Centred float32 database frames idx (F_idx, A, 3) from a FrameSet."""
    import torch

    kpad = (A + 63) // 64 * 64
    x32 = dbs.buf[:3 * dbs.capacity * kpad * 4].view(torch.float32).view(dbs.capacity, 3, kpad)
    sel = x32[torch.from_numpy(np.asarray(idx)).to(x32.device)][:, :, :A]
    return sel.transpose(1, 2).contiguous().cpu().numpy()


def serving_cpu(dbs, F, A, q, budget_s, top) -> dict:
    """The reference's per-query-frame md.rmsd over database frames, on the
    host cores: frames/s on a bounded sample, converted to requests/s at the
    sweep's mean pairs per request."""
    from oracle import cpu

    impl = cpu.best_available()
    n = min(F, 100_000)
    target = np.ascontiguousarray(dbs_frames(dbs, np.arange(n), A))
    ref = np.ascontiguousarray(q)
    t0 = time.perf_counter()
    reps = 0
    while True:
        impl.md_rmsd(target.copy(), ref.copy())
        reps += 1
        if time.perf_counter() - t0 > budget_s or reps >= 50:
            break
    dt = time.perf_counter() - t0
    pairs_s = reps * n / dt
    mean_pairs = top["continuous"]["pairs_per_s"] / max(top["continuous"]["queries_per_s"], 1e-9)
    return {"value": round(pairs_s / mean_pairs, 3), "unit": "queries/s", "cores": cpu.n_threads(),
            "kind": impl.kind, "pairs_per_s": round(pairs_s, 1),
            "sample": "%d x md.rmsd(%d database frames, 1 query frame) in %.1f s; queries/s at the sweep's mean "
                      "pairs per request" % (reps, n, dt)}


# ---------------------------------------------------------------------------
# Superposition / RMSF workload
# ---------------------------------------------------------------------------


def run_superpose(args) -> dict:
    """Trajectory.superpose(t, t, 0) and md.rmsf(t, t, 0) on 100,000 frames x
    1,000 atoms generated as the single-reference workload (sigma 0.05 nm,
    random rotations and translations).  One step = superposing the
    device-resident frames onto frame 0: the rotation pass (streaming M + QCP
    rotations) and the fused centre/rotate/translate pass, in place."""
    import ctypes as C

    import torch

    import mdtraj_gb300 as md
    from mdtraj_gb300 import _device as D
    from mdtraj_gb300 import _lib, synth
    from mdtraj_gb300.superpose import _rotations

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    F, A, sig = WORKLOADS[args.workload]
    if args.frames:
        F = args.frames
    Ap = D.padded(A)
    ref, x, _ = synth.device_single_reference(F, A, Ap, 0, seed=7 + rank, device=dev, sigma_lo=sig, sigma_hi=sig)
    lib = _lib.lib
    stream = D.stream_handle()
    rng = np.random.default_rng(3)
    sample = np.sort(rng.choice(F, size=min(F, 2000), replace=False))
    before = x.view(F, Ap, 3)[torch.from_numpy(sample).to(dev), :A].cpu().numpy()
    frame0 = x.view(F, Ap, 3)[0, :A].cpu().numpy()
    ref_align = frame0.copy()
    ref_offset = ref_align.astype(np.float64).mean(0)
    ref_align -= ref_offset
    dref = D.DeviceReference(ref_align, _lib.ATOM_MAJOR, centre=False, device=dev)
    off = (C.c_double * 3)(*[float(v) for v in ref_offset])

    def step():
        rot, mu = _rotations(x, F, A, Ap, dref, _lib.MODE_CENTER, want_mu=True)
        _lib.check(lib.gbrmsd_apply_rotations(x.data_ptr(), F, A, 3 * Ap, rot.data_ptr(), mu.data_ptr(), off, None,
                                              stream))

    step()
    torch.cuda.synchronize()
    after = x.view(F, Ap, 3)[torch.from_numpy(sample).to(dev), :A].cpu().numpy()
    from oracle import fp64

    want = fp64.superpose(before, frame0)
    err = np.abs(after.astype(np.float64) - want)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    with ClockSampler(local) as clk:
        e[0].record()
        for _ in range(args.steps):
            step()
        e[1].record()
        torch.cuda.synchronize()
    ms_step = e[0].elapsed_time(e[1]) / args.steps
    # the two passes timed separately (same stream, events between them)
    e[0].record()
    rot, mu = _rotations(x, F, A, Ap, dref, _lib.MODE_CENTER, want_mu=True)
    e[1].record()
    _lib.check(lib.gbrmsd_apply_rotations(x.data_ptr(), F, A, 3 * Ap, rot.data_ptr(), mu.data_ptr(), off, None,
                                          stream))
    e[2].record()
    torch.cuda.synchronize()
    ms_rot, ms_apply = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    alg = 36.0 * A * F  # rotation pass reads 12 B/atom; the apply pass reads and writes 12 B/atom
    peaks = measured_peaks()
    ach = alg / (ms_step / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": round(ach, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(ach / peaks["hbm_gbs"], 4), "traffic": traffic_from_profiles("superpose_step", args.workload),
            "kernel": "stream_kernel + finish_kernel + apply_rotations_kernel (whole step)",
            "algorithmic_bytes_per_step": alg,
            "passes_ms": {"rotations": round(ms_rot, 4), "apply": round(ms_apply, 4)},
            "apply_GBs": round(24.0 * A * F / (ms_apply / 1e3) / 1e9, 1),
            "rotations_GBs": round(12.0 * A * F / (ms_rot / 1e3) / 1e9, 1), "peak_src": peaks["src"]}
    # rmsf on the device-resident frames: centring + rotations + reduction
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    traces = D.center_inplace(x, F, A, Ap, _lib.ATOM_MAJOR)
    rf = x.view(F, Ap, 3)[0, :A].cpu().numpy()
    rref = D.DeviceReference(rf, _lib.ATOM_MAJOR, centre=False, device=dev)
    rws = D.empty_bytes(lib.gbrmsd_rmsf_workspace_bytes(F, A), dev)
    rout = torch.empty(A, dtype=torch.float32, device=dev)

    def rmsf_step():
        tr = D.center_inplace(x, F, A, Ap, _lib.ATOM_MAJOR, traces_out=traces)
        rot2, _ = _rotations(x, F, A, Ap, rref, _lib.MODE_PRECENTERED, tr, float(np.float32((rf ** 2).sum())))
        _lib.check(lib.gbrmsd_rmsf(x.data_ptr(), F, A, 3 * Ap, rot2.data_ptr(), rout.data_ptr(), rws.data_ptr(),
                                   rws.numel(), stream))

    rmsf_step()
    torch.cuda.synchronize()
    t0.record()
    for _ in range(args.steps):
        rmsf_step()
    t1.record()
    torch.cuda.synchronize()
    ms_rmsf = t0.elapsed_time(t1) / args.steps
    rmsf_sec = {"ms_per_call": round(ms_rmsf, 4), "frames_per_s": round(F / (ms_rmsf / 1e3), 1),
                "algorithmic_bytes": 48.0 * A * F,
                "achieved_GBs": round(48.0 * A * F / (ms_rmsf / 1e3) / 1e9, 1),
                "note": "centring in place (read + write), rotation pass, rotated reduction (12 B/atom each read)"}
    e2e = None
    if rank == 0 and not args.skip_e2e:
        host = np.empty((F, A, 3), dtype=np.float32)
        D.frames_to_host(x, host, _lib.ATOM_MAJOR, A, Ap, stream)
        torch.cuda.synchronize()
        traj = md.Trajectory(host)
        traj.superpose(traj, 0)
        reps = max(1, min(3, args.steps))
        t_e = time.perf_counter()
        for _ in range(reps):
            traj.superpose(traj, 0)
        dt = (time.perf_counter() - t_e) / reps
        e2e = {"value": round(F / dt, 1), "unit": "frames/s", "h2d_bytes_per_step": 12 * A * F,
               "d2h_bytes_per_step": 12 * A * F, "note": "Trajectory.superpose on a host numpy array"}
        del host, traj
    cpu_base = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        from oracle import cpu

        impl = cpu.CpuRmsd("reference")
        n = min(F, 20000)
        xs = np.ascontiguousarray(before[: min(len(before), n)])
        xs = np.ascontiguousarray(np.concatenate([xs] * max(1, n // len(xs)))[:n])
        t_c = time.perf_counter()
        reps = 0
        while True:
            y = xs.copy()
            impl.superpose(y, frame0)
            reps += 1
            if time.perf_counter() - t_c > args.cpu_budget or reps >= 20:
                break
        dt = (time.perf_counter() - t_c) / reps
        cpu_base = {"value": round(n / dt, 1), "unit": "frames/s", "cores": cpu.n_threads(), "kind": "reference",
                    "sample": "Trajectory.superpose of %d frames x %d atoms (numpy steps + the reference's compiled "
                              "rotation loop), %d repetitions" % (n, A, reps)}
    return {
        "metric": "superpose_frames_per_s", "value": round(world * F / (ms_step / 1e3), 1), "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, generated on device)",
        "config": {"workload": args.workload, "n_frames": F, "n_atoms": A, "sigma_nm": sig,
                   "l2": "frames (%.1f GB) larger than L2; no flush" % (12.0 * A * F / 1e9)},
        "roofline": roof, "rmsf": rmsf_sec,
        "accuracy": {"checked_frames": int(len(sample)), "max_err_nm": float(err.max()),
                     "rms_err_nm": float(np.sqrt((err ** 2).mean())), "oracle": "FP64 superposition (oracle/fp64.py)"},
        "cpu_baseline": cpu_base, "e2e": e2e, "gpu_launches": 4 * args.steps, "clocks": clk.summary(),
    }


# ---------------------------------------------------------------------------
# XTC decoding workload
# ---------------------------------------------------------------------------


def run_xtc(args) -> dict:
    """Decoding an XTC trajectory of 100,000 frames x 1,001 atoms on the GPU
    (the fixture file tests/golden/xtc_water.xtc, written by the reference's
    XTC writer, repeated 2,500 times; 487 MB).  One step = decoding every frame
    from the file bytes resident in HBM into the padded coordinate layout.
    e2e = md.rmsd of the whole file against frame 0 straight from disk
    (read, upload, decode, score)."""
    import tempfile

    import torch

    from mdtraj_gb300 import _device as D
    from mdtraj_gb300 import _lib, xtc

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    (reps,) = WORKLOADS[args.workload]
    unit = np.fromfile(ROOT / "tests" / "golden" / "xtc_water.xtc", dtype=np.uint8)
    if args.frames:
        reps = max(1, args.frames // 40)
    data = np.tile(unit, reps)
    offsets, A, used = xtc.index_bytes(data)
    F = len(offsets)
    Ap = D.padded(A)
    lib = _lib.lib
    stream = D.stream_handle()
    d_data = torch.from_numpy(data).to(dev)
    d_off = torch.from_numpy(offsets).to(dev)
    out = torch.zeros((F, 3 * Ap), dtype=torch.float32, device=dev)
    status = torch.empty(F, dtype=torch.int32, device=dev)

    def step():
        _lib.check(lib.gbrmsd_xtc_decode(d_data.data_ptr(), d_data.numel(), d_off.data_ptr(), F, A, out.data_ptr(),
                                         3 * Ap, None, None, None, status.data_ptr(), stream))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    assert int(status.abs().sum()) == 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # every repetition of the fixture must decode to the reference reader's coordinates
    g = np.load(ROOT / "tests" / "golden" / "xtc_cases.npz")
    pick = np.random.default_rng(1).integers(0, F, 200)
    dec = out.view(F, Ap, 3)[torch.from_numpy(pick).to(dev), :A].cpu().numpy()
    exact = bool(np.array_equal(dec, g["water__xyz"][pick % 40]))
    moved = float(used + 12.0 * A * F)
    peaks = measured_peaks()
    roof = {"bound": "hbm", "achieved": round(moved / (ms / 1e3) / 1e9, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(moved / (ms / 1e3) / 1e9 / peaks["hbm_gbs"], 4),
            "traffic": traffic_from_profiles("xtc_decode_kernel", "xtc_decode_100000x1001") if F == 100_000 else None,
            "kernel": "xtc_decode_kernel", "kernel_ms": round(ms, 4),
            "algorithmic_bytes_per_launch": moved,
            "note": "compressed bytes read + decoded float32 written; one thread decodes one frame's bit stream "
                    "sequentially, so the kernel is bound by dependent integer work, not by HBM"}
    e2e = None
    if rank == 0 and not args.skip_e2e:
        with tempfile.TemporaryDirectory() as tmp:
            path = f"{tmp}/traj.xtc"
            data.tofile(path)
            ref = g["water__xyz"][:1]
            xtc.rmsd_xtc(path, ref)
            t0 = time.perf_counter()
            r = xtc.rmsd_xtc(path, ref)
            dt = time.perf_counter() - t0
        e2e = {"value": round(F / dt, 1), "unit": "frames/s", "h2d_bytes_per_step": int(used),
               "d2h_bytes_per_step": int(4 * F), "api": "mdtraj_gb300.xtc.rmsd_xtc(path, reference)",
               "note": "file read from a temporary file, decoded and scored on the GPU"}
    cpu_base = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        from oracle import cpu

        n = min(F, 20000)
        with tempfile.TemporaryDirectory() as tmp:
            path = f"{tmp}/sample.xtc"
            np.tile(unit, max(1, n // 40)).tofile(path)
            t0 = time.perf_counter()
            xyz, *_ = cpu.read_xtc_reference(path, A, n)
            dt = time.perf_counter() - t0
        cpu_base = {"value": round(len(xyz) / dt, 1), "unit": "frames/s", "cores": 1, "kind": "reference",
                    "sample": "%d frames read by the reference's C XTC reader (read_xtc, single-threaded as in "
                              "the reference)" % len(xyz)}
    return {
        "metric": "xtc_decode_frames_per_s", "value": round(world * F / (ms / 1e3), 1), "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32 bit stream -> f32",
        "data": "the reference-written 40-frame fixture repeated (synthetic water-like clusters)",
        "config": {"workload": args.workload, "n_frames": F, "n_atoms": A, "file_bytes": int(used),
                   "l2": "file (%.0f MB) larger than L2; no flush" % (used / 1e6)},
        "roofline": roof, "accuracy": {"checked_frames": 200, "bit_exact_vs_reference_reader": exact},
        "cpu_baseline": cpu_base, "e2e": e2e, "gpu_launches": args.steps, "clocks": clk.summary(),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--frames", type=int, default=None, help="override n_frames (smaller runs)")
    ap.add_argument("--e2e-frames", type=int, default=None)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU baseline work")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-workloads", action="store_true",
                    help="default workload only: leave out the shortened runs of the other workloads")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="offered load per rate (seconds of arrivals)")
    ap.add_argument("--serve-max", type=int, default=1500, help="max requests per rate")
    ap.add_argument("--baseline-max", type=int, default=300, help="max requests per rate for the one-per-launch baseline")
    ap.add_argument("--rates", type=lambda v: tuple(float(x) for x in v.split(",")), default=None,
                    help="serving: offered request rates (comma-separated requests/s)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        res = run_reference(args)
    elif args.workload.startswith("allpairs"):
        res = run_allpairs(args)
    elif args.workload.startswith("ragged"):
        res = run_ragged(args)
    elif args.workload.startswith("serving"):
        res = run_serving(args)
    elif args.workload.startswith("superpose"):
        res = run_superpose(args)
    elif args.workload.startswith("xtc"):
        res = run_xtc(args)
    else:
        res = run_gpu(args)
    rank = int(os.environ.get("RANK", "0"))
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
