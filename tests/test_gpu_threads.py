"""Concurrent use from several host threads (ctypes releases the GIL during library calls):
transforms created at the same time, some with the same index set (the shared-plan cache and the
device planner under contention), each thread running backward / forward pairs on its own grid and
buffers. The reference makes creation thread-safe and execution thread-safe per grid
(docs/source/details.rst:77-88); every result must match the oracle."""
from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import pipeline
from util import rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)


def test_concurrent_creation_and_execution(lib):
    cases = [(0, 64, 20), (0, 64, 20), (1, 48, 12), (0, 60, 15), (1, 64, 20), (1, 48, 12)]
    rng = np.random.default_rng(91)
    prepared = []
    for t, n, r in cases:
        idx = sphere_indices(n, r, r2c=(t == 1))
        vals = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
        if t == 1:
            vals[(idx == 0).all(axis=1)] = vals[(idx == 0).all(axis=1)].real
        oracle = pipeline.HostPipeline(t, n, n, n, idx)
        want = oracle.backward(vals)
        prepared.append((t, n, idx, vals, want, oracle.forward(want)))
    torch.cuda.synchronize()

    def work(item):
        t, n, idx, vals, want, want_f = item
        torch.cuda.set_device(0)
        tr = sp.Transform(1, sp.SPFFT_PU_GPU, t, n, n, n, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx)
        v = torch.from_numpy(vals).cuda()
        space = torch.empty((n, n, n), dtype=torch.complex128 if t == 0 else torch.float64, device="cuda")
        f = torch.empty_like(v)
        errs = []
        for _ in range(5):
            tr.backward(v, space)
            tr.forward(space, f)
            torch.cuda.synchronize()
            errs.append(rel_l2(space.cpu().numpy(), want))
            errs.append(rel_l2(f.cpu().numpy(), want_f))
        return max(errs)

    with ThreadPoolExecutor(max_workers=len(prepared)) as pool:
        worst = list(pool.map(work, prepared))
    assert max(worst) <= 1e-12, worst
