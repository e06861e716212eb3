"""Benchmark: backward+forward transform pairs per second on one GB300.

Workload (default): the 192^3 R2C sparse transform of a spherical cutoff |k| <= 48 on the
hermitian half-space (231,391 frequency values, 3,607 z-sticks), FP64, external out-of-place real
space buffer. One step = one backward (frequency -> space) plus one forward (space -> frequency)
transform. Inputs are synthetic (seeded uniform values), resident in HBM for `value`; `e2e` runs
the same pair through the public API with pinned host buffers and the host<->device copies inside
the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs an independent replica (one transform does not shard; batches of
independent transforms would be split across ranks with no collective); the value is the total
pairs/s over all ranks, timed as the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "backward+forward pairs/s at 192^3: FP32-batched vs FP64-plain; % of HBM peak"
UNIT = "pairs/s"


# ---------------------------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------------------------
def sphere_indices(n: int, radius: float, r2c: bool) -> np.ndarray:
    """Centered triplets with x^2 + y^2 + z^2 <= radius^2 on an n^3 grid, in z-stick order (x, y, z
    ascending). R2C keeps x > 0, plus x = 0 with y > 0 or (y = 0, z >= 0). Built column by column:
    the z range of each (x, y) column comes from an integer-corrected square root."""
    lo, hi = n // 2 - n + 1, n // 2
    r = np.arange(lo, hi + 1, dtype=np.int64)
    x, y = np.meshgrid(r, r, indexing="ij")
    x, y = x.ravel(), y.ravel()
    r2 = radius * radius
    rest = r2 - (x * x + y * y)
    keep = rest >= 0
    if r2c:
        keep &= x >= 0
    x, y, rest = x[keep], y[keep], rest[keep]
    zm = np.floor(np.sqrt(np.maximum(rest, 0))).astype(np.int64)
    zm += ((zm + 1) ** 2 <= rest)  # correct the rounding of the square root both ways
    zm -= (zm * zm > rest)
    zlo = np.maximum(-zm, lo)
    zhi = np.minimum(zm, hi)
    if r2c:
        zlo = np.where((x == 0) & (y == 0), 0, zlo)
        drop = (x == 0) & (y < 0)
        zhi = np.where(drop, zlo - 1, zhi)
    cnt = np.maximum(zhi - zlo + 1, 0)
    total = int(cnt.sum())
    col = np.repeat(np.arange(len(x)), cnt)
    start = np.cumsum(cnt) - cnt
    z = zlo[col] + (np.arange(total) - start[col])
    return np.ascontiguousarray(np.stack([x[col], y[col], z], axis=1).astype(np.int32))


WORKLOADS = {
    # name: (n, radius, r2c)
    "r2c_192_sphere48": (192, 48, True),
    "c2c_64_sphere16": (64, 16, False),
    "c2c_96_sphere24": (96, 24, False),
}


# Batches of independent transforms: name -> (seed, builder). A builder returns one
# (n, radius, r2c) triple per transform.
def _uneven_128(rng):
    # 256 C2C transforms on 128^3, cutoff radius R ~ U[24, 40] each
    return [(128, float(r), False) for r in rng.uniform(24.0, 40.0, 256)]


def _mixed_512(rng):
    # 512 transforms on cubic grids from {48, 60, 72, 90, 108, 120, 150, 160}, half C2C and half
    # R2C, cutoff radius R = U(0.2, 0.3) * n
    sizes = np.array([48, 60, 72, 90, 108, 120, 150, 160])
    ns = rng.choice(sizes, 512)
    fr = rng.uniform(0.2, 0.3, 512)
    return [(int(n), float(f * n), bool(i % 2)) for i, (n, f) in enumerate(zip(ns, fr))]


BATCH_WORKLOADS = {
    "c2c_128_uneven256": (3, _uneven_128),
    "mixed_512": (5, _mixed_512),
}


def batch_specs(name: str) -> list:
    seed, builder = BATCH_WORKLOADS[name]
    return builder(np.random.default_rng(seed))


def make_values(idx: np.ndarray, r2c: bool, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
    if r2c:
        k0 = (idx == 0).all(axis=1)
        v[k0] = v[k0].real
    return v


def batch_pass_bytes(bt, geo: list) -> dict:
    """Algorithmic bytes of each pass slot of a batch (z, y, x per direction), summed over its
    transforms: a fused plane pass (path 2) moves sticks + space in the y slot and nothing in the x
    slot; split passes (path 1) and unbatched transforms (path 0) as in algorithmic_bytes."""
    out = {k: 0 for k in ("z_backward", "y_backward", "x_backward", "x_forward", "y_forward", "z_forward")}
    pair = 0
    for t, (n, npts, nsticks, ncols, r2c, tsize) in enumerate(geo):
        ab = algorithmic_bytes(n, npts, nsticks, ncols, r2c, tsize)
        k = ab["kernels"]
        pair += ab["pair"]
        if bt.transform_path(t) == 2:
            c = 2 * tsize
            fused = nsticks * n * c + n * n * n * (tsize if r2c else c)
            k = dict(k, y_backward=fused, y_forward=fused, x_backward=0, x_forward=0)
        for name in out:
            out[name] += k[name]
    return {"passes": out, "pair": pair}


def algorithmic_bytes(n: int, npts: int, nsticks: int, ncols: int, r2c: bool, tsize: int) -> dict:
    """Compulsory HBM bytes per launch of each kernel and per pair (compulsory-traffic accounting:
    sparse values + int32 value map + intermediates + dense space grid, each read or written once)."""
    c = 2 * tsize
    s = tsize if r2c else c
    vals = npts * (c + 4)
    sticks = nsticks * n * c
    planes = n * n * ncols * c
    space = n * n * n * s
    kern = {
        "z_backward": vals + sticks, "y_backward": sticks + planes, "x_backward": planes + space,
        "x_forward": space + planes, "y_forward": planes + sticks, "z_forward": sticks + vals,
    }
    pair = 2 * (npts * (c + 4) + space)
    return {"kernels": kern, "pair": pair}


def algorithmic_flops(n: int, nsticks: int, ncols: int, r2c: bool) -> dict:
    """Algorithmic flops per launch of each kernel and per pair: 5 n log2 n per complex 1D FFT of
    length n and 2.5 n log2 n per real one, over the z-sticks, the non-empty y columns of every plane
    and every x row (the pruned transform, not the dense 3D grid)."""
    c2c = 5.0 * n * np.log2(n)
    z = nsticks * c2c
    y = n * ncols * c2c
    x = n * n * (c2c / 2 if r2c else c2c)
    kern = {"z_backward": z, "y_backward": y, "x_backward": x, "x_forward": x, "y_forward": y, "z_forward": z}
    return {"kernels": kern, "pair": 2 * (z + y + x)}


def fp64_peak_tflops() -> float:
    """FP64 throughput of this GPU, measured here: best of five cuBLAS DGEMMs (torch.matmul, float64,
    4096^3, 2 n^3 flops each) timed with CUDA events after a warm-up."""
    import torch

    m = 4096
    a = torch.randn(m, m, dtype=torch.float64, device="cuda")
    b = torch.randn(m, m, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = float("inf")
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e))
    return 2.0 * m ** 3 / (best * 1e-3) / 1e12


# ---------------------------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
# multi-rank host logic (one process per GPU; covered by gloo tests on the CPU)
# ---------------------------------------------------------------------------------------------
def transform_cost(n: int, radius: float, r2c: bool, tsize: int = 4) -> int:
    """Algorithmic HBM bytes of one backward+forward pair of a batch transform (the sharding
    weight): sparse values + int32 value map + dense space grid, each once per direction."""
    npts = len(sphere_indices(n, radius, r2c))
    return algorithmic_bytes(n, npts, 0, 0, r2c, tsize)["pair"]


def shard(costs: list, rank: int, world: int) -> list:
    """Transforms of a batch owned by `rank`, balanced by cost (algorithmic bytes): greedy
    longest-processing-time assignment -- transforms in decreasing cost, each to the rank with the
    least cost so far (ties to the lower rank). Every transform has exactly one owner and no
    collective is needed on the data path."""
    order = sorted(range(len(costs)), key=lambda j: (-costs[j], j))
    load = [0] * world
    owner = [0] * len(costs)
    for j in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[j] = r
        load[r] += costs[j]
    return [j for j in range(len(costs)) if owner[j] == rank]


def max_over_ranks(value: float, world: int) -> float:
    """The largest `value` over all ranks (the job's time is its slowest rank's)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_window(step, stream, seconds: float = 0.2) -> None:
    """Run `step` untimed until about `seconds` of GPU work has passed (clock samples under load)."""
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for _ in range(8):
            step()
        stream.synchronize()


# ---------------------------------------------------------------------------------------------
# CPU baseline (the oracle port of the reference host pipeline)
# ---------------------------------------------------------------------------------------------
def cpu_pairs_per_s(workload: str, min_seconds: float, max_pairs: int, warmup: int = 1,
                    exact: bool = False) -> dict:
    """Pairs/s of the oracle port on all host threads: `max_pairs` pairs if `exact`, else pairs
    until `min_seconds` have passed (at most `max_pairs`)."""
    from oracle import pipeline

    n, radius, r2c = WORKLOADS[workload]
    idx = sphere_indices(n, radius, r2c)
    vals = make_values(idx, r2c)
    p = pipeline.HostPipeline(1 if r2c else 0, n, n, n, idx)
    cores = os.cpu_count() or 1
    for _ in range(warmup):
        p.forward(p.backward(vals, workers=cores), workers=cores)
    t0 = time.perf_counter()
    pairs = 0
    while pairs < max_pairs and (exact or pairs == 0 or time.perf_counter() - t0 < min_seconds):
        p.forward(p.backward(vals, workers=cores), workers=cores)
        pairs += 1
    dt = time.perf_counter() - t0
    return {"value": pairs / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{pairs} FP64 backward+forward pairs of {workload} (numpy/scipy.fft port of "
                      f"the reference host pipeline, {cores} threads), {dt:.2f} s"}


# ---------------------------------------------------------------------------------------------
# GPU measurement
# ---------------------------------------------------------------------------------------------
def load_traffic_table() -> dict:
    """DRAM bytes per launch measured by ncu (profiles/dram_traffic.txt), keyed by (kernel, workload)."""
    f = ROOT / "profiles" / "dram_traffic.txt"
    out = {}
    if f.exists():
        for line in f.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 4 and not line.startswith("#"):
                out[(parts[0], parts[1], parts[2])] = float(parts[3])
    return out


def load_instruction_table() -> dict:
    """Warp instructions per launch measured by ncu (smsp__inst_executed.sum,
    profiles/instructions.txt), keyed by (kernel, workload, dtype, split): the split is the
    kernel's radix split ("12x16", "12x4x4", ...)."""
    f = ROOT / "profiles" / "instructions.txt"
    out = {}
    if f.exists():
        for line in f.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 5 and not line.startswith("#"):
                out[(parts[0], parts[1], parts[2], parts[3])] = float(parts[4])
    return out


def issue_fractions(kern_ms: dict, workload: str, dtype: str, sm_mhz: float | None,
                    splits: dict | None = None) -> dict:
    """Instruction-issue roofline per kernel: its warp instructions (ncu count per launch, for the
    split the kernel ran with) over the issue slots of its CUDA-event time, 152 SMs x 4 schedulers
    x one instruction per clock at the SM clock sampled during the timed region (the maximum clock
    when no sample exists)."""
    table = load_instruction_table()
    mhz = sm_mhz or 2070.0
    out = {}
    for k, ms in kern_ms.items():
        split = (splits or {}).get(k)
        inst = table.get((k, workload, dtype, split)) if split else None
        if inst and ms > 0:
            slots = 152 * 4 * mhz * 1e6 * ms * 1e-3
            out[k] = {"split": split, "warp_instructions": int(inst), "issue_frac": round(inst / slots, 4)}
    return {"sm_mhz": mhz, "kernels": out,
            "source": "profiles/instructions.txt (ncu smsp__inst_executed.sum per launch)"} if out else {}


def oracle_errors(cases: list) -> dict:
    """Per-transform error of GPU results against the FP64 oracle (the restated reference host
    pipeline), computed after the timed regions. `cases` holds (label, n, r2c, idx, host_values,
    gpu_space, gpu_scaled_forward_of_gpu_space): the backward is compared with the oracle's FP64
    backward of the same values, the scaled forward with the oracle's scaled forward of the GPU's
    own space domain. Relative L2 and relative max-abs (over the largest reference magnitude)."""
    from oracle import pipeline

    rows = []
    for label, n, r2c, idx, host, space, fwd in cases:
        o = pipeline.HostPipeline(1 if r2c else 0, n, n, n, idx)
        want = o.backward(host)
        d = space.astype(want.dtype) - want
        b_l2 = float(np.linalg.norm(d.ravel()) / np.linalg.norm(want.ravel()))
        b_max = float(np.abs(d).max() / np.abs(want).max())
        want_f = o.forward(space.astype(np.float64 if r2c else np.complex128), scaled=True)
        d = fwd.astype(np.complex128) - want_f
        f_l2 = float(np.linalg.norm(d) / np.linalg.norm(want_f))
        f_max = float(np.abs(d).max() / np.abs(want_f).max())
        rows.append({"transform": label, "backward_rel_l2": float(f"{b_l2:.3g}"),
                     "backward_rel_maxabs": float(f"{b_max:.3g}"), "forward_rel_l2": float(f"{f_l2:.3g}"),
                     "forward_rel_maxabs": float(f"{f_max:.3g}")})
    keys = ("backward_rel_l2", "backward_rel_maxabs", "forward_rel_l2", "forward_rel_maxabs")
    return {"oracle": "FP64 numpy/scipy restatement of the reference host pipeline",
            "transforms_checked": len(rows),
            **{k + "_max": max(r[k] for r in rows) for k in keys},
            "per_transform": rows}


def measure_gpu(args, rank: int, world: int) -> dict:
    import torch

    import spfft_gb300 as sp

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    n, radius, r2c = WORKLOADS[args.workload]
    idx = sphere_indices(n, radius, r2c)
    npts = len(idx)
    ttype = sp.SPFFT_TRANS_R2C if r2c else sp.SPFFT_TRANS_C2C
    dtype = args.dtype
    ct = torch.complex128 if dtype == "float64" else torch.complex64
    rt = torch.float64 if dtype == "float64" else torch.float32
    tsize = 8 if dtype == "float64" else 4

    sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, npts, sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)  # warm
    torch.cuda.synchronize()
    # creation time with the host planner, then with the default (device) planner
    os.environ["SPFFT_GB300_PLANNER"] = "host"
    t_plan = time.perf_counter()
    sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, npts, sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
    plan_host_ms = (time.perf_counter() - t_plan) * 1e3
    del os.environ["SPFFT_GB300_PLANNER"]
    t_plan = time.perf_counter()
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, npts, sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
    plan_ms = (time.perf_counter() - t_plan) * 1e3
    vals_h = make_values(idx, r2c)
    values = torch.from_numpy(vals_h).to(ct).cuda()
    out_vals = torch.empty_like(values)
    space = torch.empty((n, n, n), dtype=rt if r2c else ct, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (126 MB)
    stream = torch.cuda.Stream()
    tuned = None
    if not args.no_autotune:  # plan-time autotuner (outside every timed region)
        tr.autotune(10)
        tuned = tr.tuning()
        tuned["splits"] = {k: None if v is None else "x".join(map(str, v)) for k, v in tr.splits().items()}
    tr.set_stream(stream)
    tr.set_execution_mode(sp.SPFFT_EXEC_ASYNCHRONOUS)

    def pair():
        tr.backward(values, space)
        tr.forward(space, out_vals, sp.SPFFT_NO_SCALING)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            pair()
    torch.cuda.synchronize()

    # ---- device-resident timed region -----------------------------------------------------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        # the sampler's first readings come from this untimed load window (about 0.2 s of the same
        # pairs), so a short timed region still has clock samples taken under load around it
        with torch.cuda.stream(stream):
            load_window(pair, stream)
        wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()  # L2 flush between timed iterations, outside the events
                starts[k].record(stream)
                pair()
                ends[k].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if world > 1:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    total_ms = max_over_ranks(total_ms, world)
    pairs_per_s = world * args.steps / (total_ms / 1e3)

    # ---- per-kernel times (stage events on the launching stream) ------------------------------
    nsticks = int(np.unique((idx[:, 0] % n) * n + idx[:, 1] % n).size)
    ncols = int(np.unique(idx[:, 0] % n).size)
    ab = algorithmic_bytes(n, npts, nsticks, ncols, r2c, tsize)
    names_b = ["z_backward", "y_backward", "x_backward"]
    names_f = ["x_forward", "y_forward", "z_forward"]
    acc = {k: [] for k in names_b + names_f}
    for _ in range(max(3, min(args.steps, 20))):
        flush.zero_()
        torch.cuda.synchronize()
        for nm, ms in zip(names_b, sp.stage_times(tr, 0, values, space, stream=stream)):
            acc[nm].append(ms)
        flush.zero_()
        torch.cuda.synchronize()
        for nm, ms in zip(names_f, sp.stage_times(tr, 1, space, out_vals, stream=stream)):
            acc[nm].append(ms)
    kern_ms = {k: statistics.median(v) for k, v in acc.items()}
    dominant = max(kern_ms, key=kern_ms.get)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = ab["kernels"][dominant] / (kern_ms[dominant] * 1e-3) / 1e9
    traffic = load_traffic_table().get((dominant, args.workload, dtype))
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_src,
                "traffic": traffic, "algorithmic_bytes": ab["kernels"][dominant],
                "kernel_ms": {k: round(v, 4) for k, v in kern_ms.items()},
                "kernel_gbs": {k: round(ab["kernels"][k] / (v * 1e-3) / 1e9, 1) for k, v in kern_ms.items()},
                "issue": issue_fractions(kern_ms, args.workload, dtype, clocks.summary().get("sm_mhz"),
                                         {k: None if v is None else "x".join(map(str, v))
                                          for k, v in tr.splits().items()}),
                "limiter": ("instruction issue: FP64 runs as double-float arithmetic on the FP32 pipes "
                            "(GB300's FP64 pipe is 57x slower), so the HBM fraction is not reachable"
                            if dtype == "float64" else "latency of a single small transform")}
    if dtype == "float64":
        # FP64 flop roofline: the pruned transform's algorithmic flops against this GPU's measured
        # FP64 rate. The double-float kernels run on the FP32 pipes, so the fraction exceeds 1.
        fl = algorithmic_flops(n, nsticks, ncols, r2c)
        fp64_peak = fp64_peak_tflops()
        achieved_tf = fl["pair"] * pairs_per_s / world / 1e12
        roofline["fp64_flops"] = {
            "algorithmic_flops_per_pair": int(fl["pair"]),
            "achieved_tflops": round(achieved_tf, 3),
            "fp64_peak_tflops": round(fp64_peak, 3),
            "peak_source": "cuBLAS DGEMM 4096^3 (torch.matmul float64), measured in this run",
            "frac": round(achieved_tf / fp64_peak, 3),
            "kernel_tflops": {k: round(fl["kernels"][k] / (v * 1e-3) / 1e12, 3) for k, v in kern_ms.items()},
        }
    pair_gbs = ab["pair"] * pairs_per_s / world / 1e9

    # ---- end to end through the public API with pinned host buffers ----------------------------
    tr.set_stream(None)
    tr.set_execution_mode(sp.SPFFT_EXEC_SYNCHRONOUS)
    hv = torch.from_numpy(vals_h).to(ct).pin_memory()
    hout = torch.empty_like(hv).pin_memory()
    hspace = torch.empty(tuple(space.shape), dtype=space.dtype).pin_memory()
    for _ in range(max(1, args.warmup)):
        tr.backward(hv, hspace)
        tr.forward(hspace, hout)
    e2e_steps = max(3, args.steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        tr.backward(hv, hspace)
        tr.forward(hspace, hout)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": round(e2e_steps / e2e_s * world, 3), "unit": UNIT,
           "h2d_bytes_per_step": int(hv.numel() * hv.element_size() + hspace.numel() * hspace.element_size()),
           "d2h_bytes_per_step": int(hspace.numel() * hspace.element_size() + hout.numel() * hout.element_size()),
           "host_access": os.environ.get("SPFFT_GB300_HOST_ACCESS", "direct"),
           "host_path": "space domain in host memory: plane-chunk copies overlapped with the chunks' y and x "
                        "passes in both directions; values read / written by the z pass over the host link "
                        "(copy mode: staged value copies)",
           "buffers": "pinned host (torch pin_memory), synchronous calls"}
    # the same pair with the reference's staged copies, for comparison
    if os.environ.get("SPFFT_GB300_HOST_ACCESS", "direct") != "copy":
        os.environ["SPFFT_GB300_HOST_ACCESS"] = "copy"
        tr2 = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, npts, sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
        del os.environ["SPFFT_GB300_HOST_ACCESS"]
        for _ in range(max(1, args.warmup)):
            tr2.backward(hv, hspace)
            tr2.forward(hspace, hout)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            tr2.backward(hv, hspace)
            tr2.forward(hspace, hout)
        torch.cuda.synchronize()
        e2e["staged_copies_value"] = round(e2e_steps / (time.perf_counter() - t0) * world, 3)
        del tr2

    # ---- comparison point: the same pair through dense 3D cuFFT (torch.fft) on the full grid ----
    cufft = measure_cufft_dense(args, idx, vals_h, n, r2c, ct, stream)

    # correctness guard on the timed output: forward(backward(v)) = N * v on C2C, and on R2C for
    # the values that are not on the x = 0 plane (those are folded by the hermitian fill)
    got = out_vals.cpu().numpy()
    want = vals_h * (n ** 3)
    sel = idx[:, 0] != 0 if r2c else slice(None)
    err = float(np.linalg.norm(got[sel] - want[sel]) / np.linalg.norm(want[sel]))

    # the reference's own GPU path on the same workload (and its backward next to ours)
    ours_space = None
    if dtype == "float64":
        tr.set_stream(None)
        tr.backward(torch.from_numpy(vals_h).to(ct).cuda(), space)
        torch.cuda.synchronize()
        ours_space = space.cpu().numpy()
    ref_gpu = (measure_reference_gpu(args, n, r2c, idx, vals_h, ours_space, args.batch)
               if ours_space is not None and not args.no_reference_gpu else None)

    batched = None if args.no_batched else measure_batched(args, args.workload, args.batch, "float32")
    grad = None if args.no_batched else measure_grad(args)

    return {
        "batched": batched, "grad": grad,
        "pairs_per_s": pairs_per_s, "ms_per_step": total_ms / args.steps, "wall_s": wall,
        "clocks": clocks.summary(), "roofline": roofline, "e2e": e2e,
        "pair_gbs": pair_gbs, "roundtrip_rel_l2": err, "cufft_dense": cufft, "reference_gpu": ref_gpu,
        "launches_per_step": 6 if tr.path_info()["split_plane"] else 4, "npts": npts, "nsticks": nsticks,
        "ncols": ncols, "tuning": tuned or tr.tuning(), "plan_ms": plan_ms,
        "plan_host_ms": plan_host_ms,
    }


def measure_plain_compact(args, workload: str, dtype: str = "float64") -> dict:
    """A single-transform configuration for the default line: pairs/s of the FP64 drop-in path on
    device buffers (autotuned plan, L2 flushed between timed steps, CUDA events), the dominant
    kernel's roofline, and one backward + scaled forward against the FP64 oracle."""
    import torch

    import spfft_gb300 as sp

    n, radius, r2c = WORKLOADS[workload]
    idx = sphere_indices(n, radius, r2c)
    ttype = sp.SPFFT_TRANS_R2C if r2c else sp.SPFFT_TRANS_C2C
    ct = torch.complex128 if dtype == "float64" else torch.complex64
    rt = torch.float64 if dtype == "float64" else torch.float32
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
    vals_h = make_values(idx, r2c)
    values = torch.from_numpy(vals_h).to(ct).cuda()
    out_vals = torch.empty_like(values)
    space = torch.empty((n, n, n), dtype=rt if r2c else ct, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    if not args.no_autotune:
        tr.autotune(3)
    tr.set_stream(stream)
    tr.set_execution_mode(sp.SPFFT_EXEC_ASYNCHRONOUS)

    def pair():
        tr.backward(values, space)
        tr.forward(space, out_vals, sp.SPFFT_NO_SCALING)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            pair()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            pair()
            ends[k].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    nsticks = int(np.unique((idx[:, 0] % n) * n + idx[:, 1] % n).size)
    ncols = int(np.unique(idx[:, 0] % n).size)
    ab = algorithmic_bytes(n, len(idx), nsticks, ncols, r2c, 8 if dtype == "float64" else 4)
    acc = {k: [] for k in ("z_backward", "y_backward", "x_backward", "x_forward", "y_forward", "z_forward")}
    for _ in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        for nm, t in zip(("z_backward", "y_backward", "x_backward"), sp.stage_times(tr, 0, values, space, stream=stream)):
            acc[nm].append(t)
        flush.zero_()
        torch.cuda.synchronize()
        for nm, t in zip(("x_forward", "y_forward", "z_forward"), sp.stage_times(tr, 1, space, out_vals, stream=stream)):
            acc[nm].append(t)
    kern_ms = {k: statistics.median(v) for k, v in acc.items() if v}
    dom = max(kern_ms, key=kern_ms.get)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = ab["kernels"][dom] / (kern_ms[dom] * 1e-3) / 1e9 if kern_ms[dom] > 0 else 0.0
    # accuracy: backward, then the scaled forward of the GPU's space domain, against the oracle
    tr.backward(values, space)
    tr.forward(space, out_vals, sp.SPFFT_FULL_SCALING)
    torch.cuda.synchronize()
    err = oracle_errors([(workload, n, r2c, idx, vals_h, space.cpu().numpy(), out_vals.cpu().numpy())])
    return {"workload": workload, "dtype": dtype, "value": round(args.steps / (ms / 1e3), 2), "unit": UNIT,
            "ms_per_step": round(ms / args.steps, 4), "frequency_values": len(idx),
            "l2": "flushed between timed steps (256 MB write)",
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "kernel_ms": {k: round(v, 4) for k, v in kern_ms.items()}},
            "vs_oracle": {k: v for k, v in err.items() if k != "per_transform"}}


def reference_source_dir() -> Path | None:
    """The reference source tree for the comparison build: $SPFFT_REFERENCE_SRC, else the staged
    copy baseline/_ref (git-ignored; see baseline/Makefile). None when neither exists."""
    for cand in (os.environ.get("SPFFT_REFERENCE_SRC"), str(ROOT / "baseline" / "_ref")):
        if cand and (Path(cand) / "src" / "execution" / "execution_gpu.cpp").exists():
            return Path(cand).resolve()
    return None


def measure_reference_gpu(args, n: int, r2c: bool, idx: np.ndarray, vals_h: np.ndarray, ours_space: np.ndarray,
                          batch: int) -> dict:
    """The reference's own GPU path (its CUDA kernels plus cuFFT; baseline/Makefile builds it from
    the reference's sources for sm_103a), timed by baseline/ref_gpu_bench on the same workload
    with the same protocol: FP64 plain (device buffers, external space buffer, L2 flushed, CUDA
    events) and FP32 over `batch` transforms through its multi-transform calls. The reference's
    backward result is compared with ours (`ours_space`) to show that both compute the same
    transform."""
    import tempfile

    src = reference_source_dir()
    if src is None:
        return {"unavailable": "the reference sources are not staged (baseline/_ref, or SPFFT_REFERENCE_SRC)"}
    t0 = time.perf_counter()
    build = subprocess.run(["make", "-s", "-j", str(os.cpu_count() or 4), "-C", str(ROOT / "baseline"),
                            f"REF={src}"], capture_output=True, text=True)
    build_s = time.perf_counter() - t0
    exe = ROOT / "baseline" / "_ref" / "build" / "ref_gpu_bench"
    if build.returncode != 0 or not exe.exists():
        tail = (build.stderr or build.stdout).strip().splitlines()[-1:] or ["?"]
        return {"unavailable": f"build of the reference GPU path failed: {tail[0][:200]}"}
    out = {"source": "the reference's own GPU path (execution_gpu.cpp, its CUDA kernels, cuFFT), built from "
                     "its sources for sm_103a by baseline/Makefile; driven through its public C++ API by "
                     "baseline/ref_gpu_bench.cpp", "build_s": round(build_s, 1)}
    with tempfile.TemporaryDirectory() as tmp:
        inp = Path(tmp) / "input.bin"
        with open(inp, "wb") as f:
            np.array([1 if r2c else 0, n, len(idx)], dtype=np.int32).tofile(f)
            np.ascontiguousarray(idx, dtype=np.int32).tofile(f)
            np.ascontiguousarray(vals_h, dtype=np.complex128).view(np.float64).tofile(f)
        space_out = Path(tmp) / "space.bin"
        runs = (("fp64_plain", "64", 1, str(space_out)), ("fp32_multi_transform", "32", batch, None))
        for key, prec, count, extra in runs:
            cmd = [str(exe), str(inp), prec, str(count), str(max(3, args.steps)), str(args.warmup)]
            if extra:
                cmd.append(extra)
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
            if r.returncode != 0:
                out[key] = {"unavailable": f"exit {r.returncode}: {(r.stderr or '').strip()[-200:]}"}
                continue
            res = json.loads(r.stdout.strip().splitlines()[-1])
            out[key] = {"value": round(res["pairs_per_s"], 2), "unit": UNIT, "ms_per_step": res["ms_per_step"],
                        "transforms_per_step": count}
        if space_out.exists():
            ref_space = np.fromfile(space_out, dtype=np.float64)
            ref_space = ref_space if r2c else ref_space.view(np.complex128)
            ours = ours_space.reshape(-1)
            out["fp64_backward_rel_l2_ours_vs_reference"] = float(
                np.linalg.norm(ours - ref_space) / np.linalg.norm(ref_space))
    out["protocol"] = ("device buffers, external out-of-place space domain (FP64) / multi-transform pointer "
                       "forms (FP32), asynchronous execution mode, CUDA events on the default stream, 256 MB "
                       "L2 flush between timed steps")
    return out


def measure_cufft_dense(args, idx: np.ndarray, vals_h: np.ndarray, n: int, r2c: bool, ct, stream) -> dict:
    """Pairs/s of the dense formulation with cuFFT (torch.fft): zero the full (half-)spectrum grid,
    scatter the values, inverse 3D FFT without scaling, forward 3D FFT, gather the values. Device
    buffers, CUDA events, L2 flushed between steps like the main measurement. A comparison point
    for the sparse kernels; its hermitian handling of the x = 0 plane is cuFFT's, not the
    reference's."""
    import torch

    nx = n // 2 + 1 if r2c else n
    wrapped = np.mod(idx.astype(np.int64), n)
    lin = torch.from_numpy((wrapped[:, 2] * n + wrapped[:, 1]) * nx + wrapped[:, 0]).cuda()
    values = torch.from_numpy(vals_h).to(ct).cuda()
    grid = torch.zeros((n, n, nx), dtype=ct, device="cuda")
    out = torch.empty_like(values)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def pair():
        grid.zero_()
        grid.view(-1)[lin] = values
        if r2c:
            space = torch.fft.irfftn(grid, s=(n, n, n), norm="forward")
            spec = torch.fft.rfftn(space, norm="backward")
        else:
            space = torch.fft.ifftn(grid, norm="forward")
            spec = torch.fft.fftn(space, norm="backward")
        out.copy_(spec.reshape(-1)[lin])

    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            pair()
        stream.synchronize()
        steps = max(3, min(args.steps, 20))
        ms = 0.0
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            pair()
            b.record(stream)
            b.synchronize()
            ms += a.elapsed_time(b)
    return {"value": round(steps / (ms / 1e3), 2), "unit": UNIT, "library": "cuFFT through torch.fft",
            "form": "dense 3D grid: zero, scatter, inverse FFT, forward FFT, gather"}


def measure_grad(args) -> dict:
    """Differentiation leg: one gradient step of L = sum V |psi|^2 with psi = backward(c) on 96^3
    C2C FP64 |k| <= 24 (c ~ N(0,1) complex, V ~ U(0,1) real), through the torch.autograd.Function
    of spfft_gb300.autograd: the backward transform, the loss, and the gradient by the hand-written
    adjoint (unnormalised forward transform + gather). Steps/s with CUDA events on the current
    stream; inputs resident on the device."""
    import torch

    import spfft_gb300 as sp
    from spfft_gb300 import autograd as ag

    n, radius = 96, 24
    idx = sphere_indices(n, radius, False)
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, sp.SPFFT_TRANS_C2C, n, n, n, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx)
    rng = np.random.default_rng(4)
    c = torch.from_numpy(rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))).cuda()
    c.requires_grad_(True)
    weight = torch.from_numpy(rng.uniform(0.0, 1.0, (n, n, n))).cuda()

    def step():
        psi = ag.backward(tr, c)
        loss = (weight * (psi.real ** 2 + psi.imag ** 2)).sum()
        (grad,) = torch.autograd.grad(loss, c)
        return grad

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    steps = max(5, args.steps)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        step()
    end.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / steps
    # the library's share of a step: the backward transform and the adjoint gradient kernels alone
    # (the loss's own gradient V * psi stands in as the adjoint's input)
    psi = torch.empty((n, n, n), dtype=torch.complex128, device="cuda")
    g_c = torch.empty(len(idx), dtype=torch.complex128, device="cuda")
    cs = c.detach()
    s = torch.cuda.current_stream().cuda_stream
    tr.backward_device(cs, psi, s)
    g_psi = (weight * 2.0).to(torch.complex128) * psi
    for _ in range(3):
        tr.backward_device(cs, psi, s)
        tr.adjoint_backward(g_psi, g_c, s)
    start.record()
    for _ in range(steps):
        tr.backward_device(cs, psi, s)
        tr.adjoint_backward(g_psi, g_c, s)
    end.record()
    torch.cuda.synchronize()
    ms_lib = start.elapsed_time(end) / steps
    return {"workload": "c2c_96_sphere24 (57,777 values), L = sum V |backward(c)|^2, FP64",
            "grad_steps_per_s": round(1e3 / ms, 1), "ms_per_step": round(ms, 4),
            "transform_and_adjoint_ms": round(ms_lib, 4),
            "step": "backward transform + loss + adjoint gradient (torch elementwise ops for the loss); "
                    "transform_and_adjoint_ms: the library's two kernel sequences of a step alone"}


def measure_batched(args, workload: str, batch: int, dtype: str, radii=None) -> dict:
    """Pairs/s of `batch` independent transforms run as one captured graph per step (backward and
    forward of every transform). The batch's working set exceeds L2, so no flush is needed."""
    import torch

    import spfft_gb300 as sp

    n, radius, r2c = WORKLOADS[workload] if workload in WORKLOADS else (None, None, None)
    if radii is None:
        radii = [radius] * batch
    ct = torch.complex128 if dtype == "float64" else torch.complex64
    rt = torch.float64 if dtype == "float64" else torch.float32
    ttype = sp.SPFFT_TRANS_R2C if r2c else sp.SPFFT_TRANS_C2C
    trs, vals, spaces, hosts, idxs = [], [], [], [], []
    cache = {}
    create_s = 0.0
    plans_before = sp.plan_cache_size()
    for b in range(batch):
        r = radii[b]
        if r not in cache:
            cache[r] = sphere_indices(n, r, r2c)
        idx = cache[r]
        idxs.append(idx)
        t0 = time.perf_counter()
        trs.append(sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype))
        create_s += time.perf_counter() - t0
        v = make_values(idx, r2c, seed=100 + b)
        if not r2c:
            v = v / np.sqrt(len(idx))
        hosts.append(v)
        vals.append(torch.from_numpy(v).to(ct).cuda())
        spaces.append(torch.empty((n, n, n), dtype=rt if r2c else ct, device="cuda"))
    bt = sp.Batch(trs)
    bt.bind(vals, spaces)
    stream = torch.cuda.Stream()
    if not args.no_autotune:
        bt.autotune(2, stream)
    for _ in range(args.warmup):
        bt.pair_graph(sp.SPFFT_FULL_SCALING, stream)  # scaled pairs keep the values bounded
    torch.cuda.synchronize()
    for b in range(batch):  # restore the inputs for the accuracy check after the timed steps
        vals[b].copy_(torch.from_numpy(hosts[b]).to(ct))
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for k in range(args.steps):
        starts[k].record(stream)
        bt.pair_graph(sp.SPFFT_FULL_SCALING, stream)
        ends[k].record(stream)
    torch.cuda.synchronize()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    # per-pass times and GB/s (events between the passes of a backward and of a forward)
    geo = []
    for idx in idxs:
        geo.append((n, len(idx), int(np.unique((idx[:, 0] % n) * n + idx[:, 1] % n).size),
                    int(np.unique(idx[:, 0] % n).size), r2c, 8 if dtype == "float64" else 4))
    pb = batch_pass_bytes(bt, geo)
    acc = {k: [] for k in pb["passes"]}
    for _ in range(5):
        for nm, t in zip(("z_backward", "y_backward", "x_backward"), bt.stage_times(0, sp.SPFFT_NO_SCALING, stream)):
            acc[nm].append(t)
        for nm, t in zip(("x_forward", "y_forward", "z_forward"), bt.stage_times(1, sp.SPFFT_FULL_SCALING, stream)):
            acc[nm].append(t)
    pass_ms = {k: statistics.median(v) for k, v in acc.items()}
    pass_gbs = {k: round(pb["passes"][k] / (pass_ms[k] * 1e-3) / 1e9, 1) for k in pass_ms if pb["passes"][k]}
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    dom = max(pass_ms, key=pass_ms.get)
    batch_roof = {"bound": "hbm", "kernel": dom + "_batch", "achieved": pass_gbs.get(dom), "peak": peak,
                  "unit": "GB/s", "frac": round(pass_gbs.get(dom, 0.0) / peak, 4),
                  "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                  "algorithmic_bytes": pb["passes"][dom]}
    for b in range(batch):  # the stage-timed passes changed the values: restore them
        vals[b].copy_(torch.from_numpy(hosts[b]).to(ct))
    bt.pair_graph(sp.SPFFT_FULL_SCALING, stream)
    torch.cuda.synchronize()
    # scaled backward+forward is the identity on C2C values and on R2C values off the x = 0 plane
    errs = []
    for b in (0, batch - 1):
        got = vals[b].cpu().numpy().astype(np.complex128)
        sel = idxs[b][:, 0] != 0 if r2c else slice(None)
        errs.append(float(np.linalg.norm(got[sel] - hosts[b][sel]) / np.linalg.norm(hosts[b][sel])))
    # FP32 against the FP64 oracle: backward and scaled forward of 8 transforms of the batch
    fp64_err = {}
    if dtype == "float32":
        for b in range(batch):
            vals[b].copy_(torch.from_numpy(hosts[b]).to(ct))
        bt.backward(stream)
        stream.synchronize()
        sample = sorted(set(np.linspace(0, batch - 1, min(8, batch)).astype(int).tolist()))
        spaces_h = {b: spaces[b].cpu().numpy() for b in sample}
        bt.forward(sp.SPFFT_FULL_SCALING, stream)
        stream.synchronize()
        fp64_err = oracle_errors([(f"{workload}[{b}]", n, r2c, idxs[b], hosts[b], spaces_h[b],
                                   vals[b].cpu().numpy()) for b in sample])
    info = bt.info()
    return {"value": round(batch * args.steps / (ms / 1e3), 2), "unit": UNIT, "dtype": dtype,
            "fp32_vs_fp64_oracle": fp64_err,
            "transforms_per_step": batch, "ms_per_step": round(ms / args.steps, 4),
            "graph_launches_per_step": 1, "kernel_launches_per_step": info["launches_per_pair"],
            "shape_groups": info["groups"], "roundtrip_rel_l2_max": max(errs),
            "plane_pass": "fused" if bt.transform_path(0) == 2 else "split",
            "row_groups": bt.row_groups(0),
            "pass_ms": {k: round(v, 4) for k, v in pass_ms.items()}, "pass_gbs": pass_gbs,
            "roofline": batch_roof,
            "hbm_gbs_per_pair_accounting": round(pb["pair"] / (ms / args.steps * 1e-3) / 1e9, 1),
            "workload": workload, "l2": "batch working set > L2 (no flush)",
            "creation": {"ms_total": round(create_s * 1e3, 2), "transforms": batch,
                         "index_plans": sp.plan_cache_size() - plans_before}}


def batch_values(idx: np.ndarray, r2c: bool, seed: int) -> np.ndarray:
    """complex N(0, 1) / sqrt(npts); real at k = 0 for R2C."""
    rng = np.random.default_rng(seed)
    v = (rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))) / np.sqrt(max(1, len(idx)))
    if r2c:
        k0 = (idx == 0).all(axis=1)
        v[k0] = v[k0].real
    return v


def oracle_sample(specs: list, mine: list, workload: str) -> list:
    """Positions (within `mine`) of the transforms whose FP32 results are checked against the FP64
    oracle: for c2c_128_uneven256 the smallest and the largest radius plus the first others (8 in
    all); otherwise the first transform of every (grid size, transform type) (16 for mixed_512)."""
    if workload == "c2c_128_uneven256":
        radii = [specs[j][1] for j in mine]
        pick = [int(np.argmin(radii)), int(np.argmax(radii))]
        pick += [i for i in range(len(mine)) if i not in pick][:6]
        return sorted(set(pick))
    first = {}
    for i, j in enumerate(mine):
        n, _, r2c = specs[j]
        first.setdefault((n, r2c), i)
    return sorted(first.values())


def measure_batch_workload(args, rank: int, world: int, workload: str | None = None,
                           compact: bool = False) -> dict:
    """A batch of independent transforms (sharded over the ranks by algorithmic bytes, no
    collective): FP32 pairs/s as one captured graph per step, the FP64 plain drop-in path over the
    same transforms one by one, the FP32 error against the FP64 oracle on a sample and against the
    FP64 GPU path on every transform, per-pass roofline, and (unless `compact`) an end-to-end leg
    with the frequency values in pinned host memory."""
    import torch

    import spfft_gb300 as sp

    workload = workload or args.workload
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    specs_all = batch_specs(workload)
    mine = shard([transform_cost(*sp_) for sp_ in specs_all], rank, world)
    idxs, hosts, geo = [], [], []
    for j in mine:
        n, radius, r2c = specs_all[j]
        idx = sphere_indices(n, radius, r2c)
        idxs.append(idx)
        hosts.append(batch_values(idx, r2c, seed=1000 + j))
        geo.append((n, len(idx), int(np.unique((idx[:, 0] % n) * n + idx[:, 1] % n).size),
                    int(np.unique(idx[:, 0] % n).size), r2c, 4))

    def make(dtype):
        ct = torch.complex128 if dtype == "float64" else torch.complex64
        rt = torch.float64 if dtype == "float64" else torch.float32
        trs, vals, spaces = [], [], []
        for j, idx, v in zip(mine, idxs, hosts):
            n, _, r2c = specs_all[j]
            ttype = sp.SPFFT_TRANS_R2C if r2c else sp.SPFFT_TRANS_C2C
            trs.append(sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, len(idx), sp.SPFFT_INDEX_TRIPLETS,
                                    idx, dtype=dtype))
            vals.append(torch.from_numpy(v).to(ct).cuda())
            spaces.append(torch.empty((n, n, n), dtype=rt if r2c else ct, device="cuda"))
        return trs, vals, spaces, ct

    stream = torch.cuda.Stream()
    # ---- FP32 batched -------------------------------------------------------------------------
    creation = {}
    if not compact:
        # creation of the whole set with the host planner (discarded), then the default planner
        os.environ["SPFFT_GB300_PLANNER"] = "host"
        t0 = time.perf_counter()
        discard = make("float32")
        creation["ms_total_host_planner"] = round((time.perf_counter() - t0) * 1e3, 1)
        del os.environ["SPFFT_GB300_PLANNER"], discard
    plans_before = sp.plan_cache_size()
    t0 = time.perf_counter()
    trs32, vals32, spaces32, ct32 = make("float32")
    create_s = time.perf_counter() - t0
    creation.update({"ms_total": round(create_s * 1e3, 1), "transforms": len(trs32),
                     "index_plans": sp.plan_cache_size() - plans_before,
                     "includes": "index planning, device tables, grid buffers, value and space buffers"})
    bt = sp.Batch(trs32)
    bt.bind(vals32, spaces32)
    if not args.no_autotune:
        bt.autotune(2, stream)
        for d, h in zip(vals32, hosts):  # the autotuner overwrote the bound buffers
            d.copy_(torch.from_numpy(h).to(ct32))
    for _ in range(args.warmup):
        bt.pair_graph(sp.SPFFT_FULL_SCALING, stream)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        load_window(lambda: bt.pair_graph(sp.SPFFT_FULL_SCALING, stream), stream)
        for k in range(args.steps):
            starts[k].record(stream)
            bt.pair_graph(sp.SPFFT_FULL_SCALING, stream)
            ends[k].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    total_ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    total_ms = max_over_ranks(total_ms, world)
    value = len(specs_all) * args.steps / (total_ms / 1e3)

    # per-pass roofline (groups run pass by pass for the events)
    names_b = ["z_backward", "y_backward", "x_backward"]
    names_f = ["x_forward", "y_forward", "z_forward"]
    acc = {k: [] for k in names_b + names_f}
    for _ in range(5):
        for nm, ms in zip(names_b, bt.stage_times(0, sp.SPFFT_NO_SCALING, stream)):
            acc[nm].append(ms)
        for nm, ms in zip(names_f, bt.stage_times(1, sp.SPFFT_FULL_SCALING, stream)):
            acc[nm].append(ms)
    pass_ms = {k: statistics.median(v) for k, v in acc.items()}
    pb = batch_pass_bytes(bt, geo)
    pass_bytes, pair_bytes = pb["passes"], pb["pair"]
    dominant = max(pass_ms, key=pass_ms.get)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = pass_bytes[dominant] / (pass_ms[dominant] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dominant + "_batch", "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "traffic": load_traffic_table().get((dominant + "_batch", workload, "float32")),
                "algorithmic_bytes": pass_bytes[dominant],
                "pass_ms": {k: round(v, 4) for k, v in pass_ms.items()},
                "pass_gbs": {k: round(pass_bytes[k] / (pass_ms[k] * 1e-3) / 1e9, 1) for k in pass_ms
                             if pass_bytes[k]}}

    # ---- end to end: values from / to pinned host memory around the captured pair ---------------
    e2e = None
    if not compact:
        hv = [torch.from_numpy(v).to(ct32).pin_memory() for v in hosts]
        ho = [torch.empty_like(h).pin_memory() for h in hv]
        e2e_steps = max(3, args.steps)

        def e2e_step():
            with torch.cuda.stream(stream):
                for d, h in zip(vals32, hv):
                    d.copy_(h, non_blocking=True)
                bt.pair_graph(sp.SPFFT_FULL_SCALING, stream)
                for h, d in zip(ho, vals32):
                    h.copy_(d, non_blocking=True)
            stream.synchronize()

        for _ in range(2):
            e2e_step()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        e2e_s = time.perf_counter() - t0
        vbytes = int(sum(h.numel() * h.element_size() for h in hv))
        e2e = {"value": round(len(specs_all) * e2e_steps / e2e_s, 2), "unit": UNIT,
               "h2d_bytes_per_step": vbytes * world, "d2h_bytes_per_step": vbytes * world,
               "buffers": "frequency values in pinned host memory, space domains on the device"}

    # ---- FP32 against the FP64 oracle on a sample (backward, then scaled forward) ---------------
    for d, h in zip(vals32, hosts):
        d.copy_(torch.from_numpy(h).to(ct32))
    bt.backward(stream)
    stream.synchronize()
    picked = oracle_sample(specs_all, mine, workload)
    space_h = {i: spaces32[i].cpu().numpy() for i in picked}
    bt.forward(sp.SPFFT_FULL_SCALING, stream)  # batched scaled forward of the FP32 space domains
    stream.synchronize()
    fwd32 = [v.clone() for v in vals32]
    vs_oracle = oracle_errors([(f"{workload}[{mine[i]}] {specs_all[mine[i]][0]}^3 "
                                f"{'R2C' if specs_all[mine[i]][2] else 'C2C'}",
                                specs_all[mine[i]][0], specs_all[mine[i]][2], idxs[i], hosts[i],
                                space_h[i], fwd32[i].cpu().numpy()) for i in picked])

    # ---- FP32 against the FP64 GPU path on every transform of this rank --------------------------
    trs64, vals64, spaces64, ct64 = make("float64")
    errs_b, errs_f, maxabs_b, maxabs_f = [], [], [], []
    for i in range(len(mine)):
        trs64[i].backward(vals64[i], spaces64[i])
        d = (spaces32[i].to(spaces64[i].dtype) - spaces64[i]).flatten()
        ref = spaces64[i].flatten()
        errs_b.append(float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref)))
        maxabs_b.append(float(d.abs().max() / ref.abs().max()))
        f64 = torch.empty_like(vals64[i])
        trs64[i].forward(spaces64[i], f64, sp.SPFFT_FULL_SCALING)
        d = (fwd32[i].to(ct64) - f64).flatten()
        errs_f.append(float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(f64.flatten())))
        maxabs_f.append(float(d.abs().max() / f64.abs().max()))

    # ---- FP64 plain: the drop-in API, one transform after another ------------------------------
    for t in trs64:
        t.set_stream(stream)
        t.set_execution_mode(sp.SPFFT_EXEC_ASYNCHRONOUS)

    def plain_step():
        for t, v, sp_ in zip(trs64, vals64, spaces64):
            t.backward(v, sp_)
            t.forward(sp_, v, sp.SPFFT_FULL_SCALING)

    with torch.cuda.stream(stream):
        plain_step()
    torch.cuda.synchronize()
    psteps = max(3, min(args.steps, 10))
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    with torch.cuda.stream(stream):
        for _ in range(psteps):
            plain_step()
    a1.record(stream)
    torch.cuda.synchronize()
    plain_ms = max_over_ranks(a0.elapsed_time(a1), world)
    plain = len(specs_all) * psteps / (plain_ms / 1e3)
    info = bt.info()
    del trs64, vals64, spaces64
    return {"value": value, "ms_per_step": total_ms / args.steps, "clocks": clocks.summary(),
            "roofline": roofline, "e2e": e2e, "pair_bytes": pair_bytes,
            "launches_per_step": info["launches_per_pair"], "groups": info["groups"],
            "creation": creation,
            "unbatched": info["unbatched"], "fp64_plain": plain,
            "vs_oracle": vs_oracle,
            "err_backward": max(errs_b), "err_forward": max(errs_f), "sampled": len(mine),
            "err_stats": {"backward_space_rel_l2": {"max": max(errs_b), "median": statistics.median(errs_b)},
                          "backward_space_rel_maxabs": {"max": max(maxabs_b), "median": statistics.median(maxabs_b)},
                          "forward_values_rel_l2": {"max": max(errs_f), "median": statistics.median(errs_f)},
                          "forward_values_rel_maxabs": {"max": max(maxabs_f), "median": statistics.median(maxabs_f)}},
            "transforms": len(specs_all)}


def batch_config_summary(res: dict) -> dict:
    """Compact form of measure_batch_workload's result for the default benchmark line."""
    return {"fp32_batched": {"value": round(res["value"], 2), "unit": UNIT,
                             "ms_per_step": round(res["ms_per_step"], 4),
                             "kernel_launches_per_pair": res["launches_per_step"],
                             "shape_groups": res["groups"]},
            "fp64_plain": {"value": round(res["fp64_plain"], 2), "unit": UNIT},
            "ratio_fp32_batched_vs_fp64_plain": round(res["value"] / res["fp64_plain"], 2),
            "roofline": {k: res["roofline"][k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac")},
            "fp32_vs_fp64_oracle": {k: v for k, v in res["vs_oracle"].items()},
            "clocks": res["clocks"]}


def cpu_batch_pairs_per_s(workload: str, min_seconds: float, max_pairs: int, exact: bool = False,
                          warmup: int = 1) -> dict:
    """Pairs/s of the oracle port over the batch's transforms in order (cycling), all host threads."""
    from oracle import pipeline

    specs = batch_specs(workload)
    cores = os.cpu_count() or 1
    cache = {}

    def get(j):
        if j not in cache:
            n, radius, r2c = specs[j]
            idx = sphere_indices(n, radius, r2c)
            cache[j] = (pipeline.HostPipeline(1 if r2c else 0, n, n, n, idx), batch_values(idx, r2c, 1000 + j))
        return cache[j]

    # size the sample from one timed pair, then plan every transform of it before timing
    p, v = get(0)
    for _ in range(max(1, warmup)):
        t0 = time.perf_counter()
        p.forward(p.backward(v, workers=cores), workers=cores)
        one = time.perf_counter() - t0
    count = max_pairs if exact else int(max(1, min(max_pairs, min_seconds / max(one, 1e-6))))
    for j in range(min(count, len(specs))):
        get(j)
    t0 = time.perf_counter()
    for k in range(count):
        p, v = get(k % len(specs))
        p.forward(p.backward(v, workers=cores), workers=cores)
    dt = time.perf_counter() - t0
    return {"value": count / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"the first {count} FP64 backward+forward pairs of {workload} (numpy/scipy.fft port "
                      f"of the reference host pipeline, {cores} threads, plans built before timing), {dt:.2f} s"}


def relaunch_ranks(n: int) -> int:
    """`--gpus N` (N > 1) without a launcher: start N ranks on this node, one process per GPU,
    through torch.distributed.run with the same arguments, and return its exit status."""
    import socket

    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS),
                    default="r2c_192_sphere48")
    ap.add_argument("--dtype", choices=["float64", "float32"], default="float64")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", type=int, default=64, help="transforms in the FP32-batched leg")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the plan-time default tile shapes instead of running the autotuner")
    ap.add_argument("--no-configs", action="store_true",
                    help="leave the other configurations' compact legs out of the default line")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="leave out the timing of the reference's own GPU path")
    ap.add_argument("--launch-check", action="store_true",
                    help="print this rank's place in the job as JSON and exit, before any GPU work")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    env_world = os.environ.get("WORLD_SIZE")
    if env_world is None and args.gpus > 1 and args.impl == "ours":
        return relaunch_ranks(args.gpus)
    world = int(env_world or "1")
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "ours" and world != args.gpus:
        print(f"bench.py: --gpus {args.gpus} does not match the launcher's WORLD_SIZE {world}", file=sys.stderr)
        return 2
    if args.launch_check:
        print(json.dumps({"rank": rank, "world_size": world,
                          "local_rank": int(os.environ.get("LOCAL_RANK", "0")), "gpus": args.gpus}), flush=True)
        return 0
    if args.workload in BATCH_WORKLOADS:
        return batch_main(args, rank, world)
    n, radius, r2c = WORKLOADS[args.workload]
    config = {"workload": args.workload, "grid": [n, n, n], "cutoff_radius": radius,
              "transform": "R2C" if r2c else "C2C", "precision": args.dtype,
              "space_buffer": "external out-of-place", "l2": "flushed between timed steps (256 MB write)",
              "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        # W untimed pairs, then exactly K timed pairs of the CPU port on all host threads
        res = cpu_pairs_per_s(args.workload, min_seconds=0.0, max_pairs=args.steps,
                              warmup=args.warmup, exact=True)
        value = res["value"]
        line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(1e3 / value, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {**res, "value": round(value, 3)},
                "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "note": "reference CPU path: FFTW is absent on this machine, so the oracle port "
                        "(numpy + scipy.fft restatement of the reference host pipeline) is timed"}
        print(json.dumps(line))
        return 0

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")

    from spfft_gb300 import build as _b
    _b.build()
    res = measure_gpu(args, rank, world)
    line = {
        "metric": METRIC, "value": round(res["pairs_per_s"], 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(res["ms_per_step"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.dtype == "float64" else "f32", "data": "synthetic",
        "config": config,
        "workload_stats": {"frequency_values": res["npts"], "z_sticks": res["nsticks"], "x_columns": res["ncols"]},
        "roofline": res["roofline"],
        "hbm_gbs_per_pair_accounting": round(res["pair_gbs"], 1),
        "e2e": res["e2e"], "clocks": res["clocks"],
        "gpu_launches": res["launches_per_step"] * args.steps,
        "roundtrip_rel_l2": res["roundtrip_rel_l2"], "tuning": res["tuning"],
        "cufft_dense_comparison": res["cufft_dense"],
        "reference_gpu": res["reference_gpu"],
        "transform_creation_ms": {"device_planner": round(res["plan_ms"], 2),
                                  "host_planner": round(res["plan_host_ms"], 2)},
    }
    if res["batched"]:
        line["fp32_batched"] = res["batched"]
        line["fp32_batched"]["ratio_vs_value"] = round(res["batched"]["value"] / res["pairs_per_s"], 2)
    if res["grad"]:
        line["differentiation"] = res["grad"]
    if world == 1 and not args.no_configs and args.workload == "r2c_192_sphere48":
        # the other configurations, compact: 64^3 C2C FP64 plain, and the two batched sets (FP32
        # batched against FP64 plain, FP32 error per transform against the FP64 oracle)
        line["configs"] = {
            "c2c_64_sphere16": measure_plain_compact(args, "c2c_64_sphere16"),
            "c2c_128_uneven256": batch_config_summary(
                measure_batch_workload(args, 0, 1, "c2c_128_uneven256", compact=True)),
            "mixed_512": batch_config_summary(measure_batch_workload(args, 0, 1, "mixed_512", compact=True)),
        }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_pairs_per_s(args.workload, args.cpu_seconds, 400)
        line["cpu_baseline"]["value"] = round(line["cpu_baseline"]["value"], 3)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))
    return 0


def batch_main(args, rank: int, world: int) -> int:
    specs = batch_specs(args.workload)
    sizes = sorted({n for n, _, _ in specs})
    config = {"workload": args.workload, "transforms": len(specs), "grids": [f"{n}^3" for n in sizes],
              "transform": "C2C" if not any(r for _, _, r in specs) else "C2C and R2C",
              "cutoff_radii": [round(min(r for _, r, _ in specs), 2), round(max(r for _, r, _ in specs), 2)],
              "precision": "float32 batched (one CUDA graph per step); float64 plain alongside",
              "space_buffer": "external out-of-place, one per transform",
              "l2": "batch working set > L2 (no flush)", "parallelism": f"transforms sharded x{world}"}
    if args.impl == "reference":
        if rank != 0:
            return 0
        res = cpu_batch_pairs_per_s(args.workload, 0.0, args.steps, exact=True, warmup=args.warmup)
        value = res["value"]
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 / value, 3), "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "cpu_baseline": {**res, "value": round(value, 3)},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference CPU path: the oracle port, one transform of the batch per step"}))
        return 0
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    from spfft_gb300 import build as _b
    _b.build()
    res = measure_batch_workload(args, rank, world)
    line = {
        "metric": METRIC, "value": round(res["value"], 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(res["ms_per_step"], 4),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config, "roofline": res["roofline"],
        "hbm_gbs_per_pair_accounting": round(res["pair_bytes"] / (res["ms_per_step"] * 1e-3) / 1e9, 1),
        "e2e": res["e2e"], "clocks": res["clocks"],
        "gpu_launches": res["launches_per_step"] * args.steps,
        "shape_groups": res["groups"], "unbatched_transforms": res["unbatched"],
        "transform_creation": res["creation"],
        "fp64_plain": {"value": round(res["fp64_plain"], 2), "unit": UNIT,
                       "ratio_fp32_batched_vs_fp64_plain": round(res["value"] / res["fp64_plain"], 2)},
        "fp32_vs_fp64_oracle": res["vs_oracle"],
        "fp32_vs_fp64_gpu_errors": res["err_stats"],
        "fp32_vs_fp64_gpu_rel_l2_max": {"backward_space": res["err_backward"], "forward_values": res["err_forward"],
                                        "transforms_checked": res["sampled"]},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_batch_pairs_per_s(args.workload, args.cpu_seconds, 2000)
        line["cpu_baseline"]["value"] = round(line["cpu_baseline"]["value"], 3)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
