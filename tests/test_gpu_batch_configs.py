"""GPU parity of the two batched benchmark configurations on their actual seeded draws, against
the FP64 oracle (oracle/pipeline.py), transform by transform.

* 256 C2C transforms on 128^3 with cutoff radii R ~ U[24, 40] (bench.py workload
  c2c_128_uneven256): 8 of the seeded draws, the smallest and the largest radius among them.
* 512 transforms on cubic grids from {48, 60, 72, 90, 108, 120, 150, 160}, half C2C and half R2C,
  R = U(0.2, 0.3) * n (bench.py workload mixed_512): 16 draws, the first of every (size, type).

Each sample runs as one batch (the batched kernels, one launch per pass and shape group, replayed
from the captured pair graph) in FP32 and in FP64, and the FP64 drop-in path one transform at a
time; every backward (space domain) and scaled forward (values) is compared with the oracle.
Values are the benchmark's: complex N(0, 1) / sqrt(npts), real at k = 0 for R2C.
Tolerances (relative L2 per transform): FP64 <= 1e-12, FP32 <= 1e-5.
"""
from __future__ import annotations

import numpy as np
import pytest

import bench
import spfft_gb300 as sp
from oracle import pipeline
from util import rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

TOL = {"float64": 1e-12, "float32": 1e-5}


def _sample(workload):
    specs = bench.batch_specs(workload)
    if workload == "c2c_128_uneven256":
        radii = np.array([r for _, r, _ in specs])
        pick = [int(np.argmin(radii)), int(np.argmax(radii))]
        pick += [j for j in range(len(specs)) if j not in pick][:6]
        pick = sorted(pick)
    else:
        first = {}
        for j, (n, _, r2c) in enumerate(specs):
            first.setdefault((n, r2c), j)
        pick = sorted(first.values())
        assert len(pick) == 16
    return [(j, *specs[j]) for j in pick]


def _run(workload, dtype):
    sample = _sample(workload)
    ct = torch.complex128 if dtype == "float64" else torch.complex64
    rt = torch.float64 if dtype == "float64" else torch.float32
    items = []
    for j, n, radius, r2c in sample:
        idx = bench.sphere_indices(n, radius, r2c)
        ttype = sp.SPFFT_TRANS_R2C if r2c else sp.SPFFT_TRANS_C2C
        host = bench.batch_values(idx, r2c, seed=1000 + j)
        items.append(dict(
            j=j, n=n, r2c=r2c, idx=idx, host=host, ttype=ttype,
            tr=sp.Transform(1, sp.SPFFT_PU_GPU, ttype, n, n, n, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx,
                            dtype=dtype),
            vals=torch.from_numpy(host).to(ct).cuda(),
            space=torch.empty((n, n, n), dtype=rt if r2c else ct, device="cuda"),
            oracle=pipeline.HostPipeline(ttype, n, n, n, idx)))
    return items


@pytest.mark.parametrize("workload", ["c2c_128_uneven256", "mixed_512"])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_batched_draws_against_fp64_oracle(lib, workload, dtype):
    items = _run(workload, dtype)
    batch = sp.Batch([it["tr"] for it in items])
    batch.bind([it["vals"] for it in items], [it["space"] for it in items])
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        batch.backward(stream)
    stream.synchronize()
    worst_b = 0.0
    spaces = []
    for it in items:
        want = it["oracle"].backward(it["host"])
        got = it["space"].cpu().numpy()
        err = rel_l2(got, want)
        worst_b = max(worst_b, err)
        assert err <= TOL[dtype], (workload, it["j"], it["n"], it["r2c"], err)
        spaces.append(got.astype(np.complex128 if not it["r2c"] else np.float64))
    with torch.cuda.stream(stream):
        batch.forward(sp.SPFFT_FULL_SCALING, stream)
    stream.synchronize()
    for it, space in zip(items, spaces):
        want = it["oracle"].forward(space, scaled=True)
        err = rel_l2(it["vals"].cpu().numpy(), want)
        assert err <= TOL[dtype], (workload, it["j"], it["n"], it["r2c"], err)
    # the captured pair graph gives the same results as the direct calls
    for it in items:
        it["vals"].copy_(torch.from_numpy(it["host"]).to(it["vals"].dtype))
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        batch.pair_graph(sp.SPFFT_FULL_SCALING, stream)
    stream.synchronize()
    for it, space in zip(items, spaces):
        assert rel_l2(it["space"].cpu().numpy(), space) <= TOL[dtype]


@pytest.mark.parametrize("workload", ["c2c_128_uneven256", "mixed_512"])
def test_plain_fp64_draws_against_fp64_oracle(lib, workload):
    """The FP64 drop-in path (spfft_transform_backward / forward, one transform at a time) on the
    same draws."""
    for it in _run(workload, "float64"):
        it["tr"].backward(it["vals"], it["space"])
        want = it["oracle"].backward(it["host"])
        got = it["space"].cpu().numpy()
        assert rel_l2(got, want) <= TOL["float64"], (workload, it["j"])
        out = torch.empty_like(it["vals"])
        it["tr"].forward(it["space"], out, sp.SPFFT_FULL_SCALING)
        want_f = it["oracle"].forward(got, scaled=True)
        assert rel_l2(out.cpu().numpy(), want_f) <= TOL["float64"], (workload, it["j"])
