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
    lo, hi = n // 2 - n + 1, n // 2
    r = np.arange(lo, hi + 1)
    x, y, z = np.meshgrid(r, r, r, indexing="ij")
    m = x * x + y * y + z * z <= radius * radius
    if r2c:
        m &= (x > 0) | ((x == 0) & ((y > 0) | ((y == 0) & (z >= 0))))
    return np.ascontiguousarray(np.stack([x[m], y[m], z[m]], axis=1).astype(np.int32))


WORKLOADS = {
    # name: (n, radius, r2c)
    "r2c_192_sphere48": (192, 48, True),
    "c2c_64_sphere16": (64, 16, False),
    "c2c_96_sphere24": (96, 24, False),
}


def make_values(idx: np.ndarray, r2c: bool, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
    if r2c:
        k0 = (idx == 0).all(axis=1)
        v[k0] = v[k0].real
    return v


def algorithmic_bytes(n: int, npts: int, nsticks: int, ncols: int, r2c: bool, tsize: int) -> dict:
    """Compulsory HBM bytes per launch of each kernel and per pair (SURVEY-style accounting:
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
                 "--format=csv,noheader,nounits", "-lms", "200"],
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

    tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, npts, sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
    vals_h = make_values(idx, r2c)
    values = torch.from_numpy(vals_h).to(ct).cuda()
    out_vals = torch.empty_like(values)
    space = torch.empty((n, n, n), dtype=rt if r2c else ct, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (126 MB)
    stream = torch.cuda.Stream()
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
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
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
                "kernel_ms": {k: round(v, 4) for k, v in kern_ms.items()}}
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

    # correctness guard on the timed output: forward(backward(v)) = N * v on C2C, and on R2C for
    # the values that are not on the x = 0 plane (those are folded by the hermitian fill)
    got = out_vals.cpu().numpy()
    want = vals_h * (n ** 3)
    sel = idx[:, 0] != 0 if r2c else slice(None)
    err = float(np.linalg.norm(got[sel] - want[sel]) / np.linalg.norm(want[sel]))

    batched = None if args.no_batched else measure_batched(args, args.workload, args.batch, "float32")

    return {
        "batched": batched,
        "pairs_per_s": pairs_per_s, "ms_per_step": total_ms / args.steps, "wall_s": wall,
        "clocks": clocks.summary(), "roofline": roofline, "e2e": e2e,
        "pair_gbs": pair_gbs, "roundtrip_rel_l2": err,
        "launches_per_step": 6, "npts": npts, "nsticks": nsticks, "ncols": ncols,
    }


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
    for b in range(batch):
        r = radii[b]
        if r not in cache:
            cache[r] = sphere_indices(n, r, r2c)
        idx = cache[r]
        idxs.append(idx)
        trs.append(sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype))
        v = make_values(idx, r2c, seed=100 + b)
        if not r2c:
            v = v / np.sqrt(len(idx))
        hosts.append(v)
        vals.append(torch.from_numpy(v).to(ct).cuda())
        spaces.append(torch.empty((n, n, n), dtype=rt if r2c else ct, device="cuda"))
    bt = sp.Batch(trs)
    bt.bind(vals, spaces)
    stream = torch.cuda.Stream()
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
    # scaled backward+forward is the identity on C2C values and on R2C values off the x = 0 plane
    errs = []
    for b in (0, batch - 1):
        got = vals[b].cpu().numpy().astype(np.complex128)
        sel = idxs[b][:, 0] != 0 if r2c else slice(None)
        errs.append(float(np.linalg.norm(got[sel] - hosts[b][sel]) / np.linalg.norm(hosts[b][sel])))
    info = bt.info()
    return {"value": round(batch * args.steps / (ms / 1e3), 2), "unit": UNIT, "dtype": dtype,
            "transforms_per_step": batch, "ms_per_step": round(ms / args.steps, 4),
            "graph_launches_per_step": 1, "kernel_launches_per_step": info["launches_per_pair"],
            "shape_groups": info["groups"], "roundtrip_rel_l2_max": max(errs),
            "workload": workload, "l2": "batch working set > L2 (no flush)"}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="r2c_192_sphere48")
    ap.add_argument("--dtype", choices=["float64", "float32"], default="float64")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", type=int, default=64, help="transforms in the FP32-batched leg")
    ap.add_argument("--no-batched", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
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
        "config": {**config, "frequency_values": res["npts"], "z_sticks": res["nsticks"],
                   "x_columns": res["ncols"]},
        "roofline": res["roofline"],
        "hbm_gbs_per_pair_accounting": round(res["pair_gbs"], 1),
        "e2e": res["e2e"], "clocks": res["clocks"],
        "gpu_launches": res["launches_per_step"] * args.steps,
        "roundtrip_rel_l2": res["roundtrip_rel_l2"],
    }
    if res["batched"]:
        line["fp32_batched"] = res["batched"]
        line["fp32_batched"]["ratio_vs_value"] = round(res["batched"]["value"] / res["pairs_per_s"], 2)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_pairs_per_s(args.workload, args.cpu_seconds, 400)
        line["cpu_baseline"]["value"] = round(line["cpu_baseline"]["value"], 3)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
