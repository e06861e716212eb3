"""Failure paths without a GPU fault.

Allocation failures are injected on the host (spfft_gb300_inject_allocation_failure: the n-th next
device or pinned allocation raises the error a failing CUDA allocator raises, without calling it)
at every allocation of transform, grid and batch creation and of the pinned host space buffer.
Each failure must surface as its exact SpfftError code, or -- inside the device index planner --
fall back to the host planner. The library must stay usable afterwards. The validation errors of
the reference's transform and grid construction are checked with their codes alongside.
"""
from __future__ import annotations

import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import pipeline
from util import rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

E = sp.ErrorCode


def _works(tr, idx, dims, ttype=0):
    rng = np.random.default_rng(3)
    vals = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
    space = torch.empty(dims[::-1], dtype=torch.complex128 if ttype == 0 else torch.float64, device="cuda")
    tr.backward(torch.from_numpy(vals).cuda(), space)
    torch.cuda.synchronize()
    assert rel_l2(space.cpu().numpy(), pipeline.HostPipeline(ttype, *dims, idx).backward(vals)) <= 1e-12


@pytest.fixture(autouse=True)
def _disarm():
    yield
    sp.inject_allocation_failure(-1)


def test_transform_creation_allocation_failures(lib, monkeypatch):
    monkeypatch.setenv("SPFFT_GB300_PLAN_CACHE", "0")  # every creation plans (and allocates) anew
    dims = (64, 64, 64)
    idx = sphere_indices(64, 16)  # 17,077 values: planned on the device
    failed = fell_back = 0
    for k in range(64):
        sp.inject_allocation_failure(k)
        code = None
        try:
            tr = sp.Transform(1, sp.SPFFT_PU_GPU, 0, *dims, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx)
        except sp.SpfftError as e:
            code = e.error_code()
        pending = sp.inject_allocation_failure(-1)
        if code is not None:
            assert pending == -1, k  # the injected failure, nothing else
            assert code == E.SPFFT_GPU_ALLOCATION_ERROR, (k, code)
            failed += 1
            continue
        _works(tr, idx, dims)
        del tr
        if pending >= 0:
            break  # creation needed fewer than k + 1 allocations
        fell_back += 1  # the failure hit the device planner, which fell back to the host planner
    else:
        pytest.fail("transform creation never completed below the injection point")
    # the planner's three allocations fall back; the grid buffer, the plan tables and the scratch fail
    assert fell_back >= 1 and failed >= 3, (fell_back, failed)


def test_grid_and_batch_creation_allocation_failures(lib, monkeypatch):
    monkeypatch.setenv("SPFFT_GB300_PLAN_CACHE", "0")
    sp.inject_allocation_failure(0)
    with pytest.raises(sp.SpfftError) as e:
        sp.Grid(32, 32, 32, 32 * 32, sp.SPFFT_PU_GPU, 1)
    assert e.value.error_code() == E.SPFFT_GPU_ALLOCATION_ERROR
    assert sp.inject_allocation_failure(-1) == -1
    bidx = sphere_indices(64, 12)  # batched kernels exist for 64
    trs = [sp.Transform(1, sp.SPFFT_PU_GPU, 0, 64, 64, 64, len(bidx), sp.SPFFT_INDEX_TRIPLETS, bidx,
                        dtype="float32") for _ in range(3)]
    failed = 0
    for k in range(32):
        sp.inject_allocation_failure(k)
        try:
            batch = sp.Batch(trs)
        except sp.SpfftError as ex:
            assert ex.error_code() == E.SPFFT_GPU_ALLOCATION_ERROR
            assert sp.inject_allocation_failure(-1) == -1
            failed += 1
            continue
        pending = sp.inject_allocation_failure(-1)
        assert pending >= 0  # a batch has no fallback: success means no injected failure was met
        break
    assert failed >= 1 and batch.info()["groups"] == 1
    vals = [torch.zeros(len(bidx), dtype=torch.complex64, device="cuda") for _ in trs]
    spaces = [torch.zeros((64, 64, 64), dtype=torch.complex64, device="cuda") for _ in trs]
    batch.bind(vals, spaces)
    stream = torch.cuda.Stream()
    batch.pair_graph(sp.SPFFT_FULL_SCALING, stream)
    stream.synchronize()


def test_pinned_host_space_allocation_failure(lib):
    dims = (16, 16, 16)
    idx = sphere_indices(16, 5)
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, 0, *dims, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx)
    sp.inject_allocation_failure(0)
    with pytest.raises(sp.SpfftError) as e:
        tr.space_domain_data(sp.SPFFT_PU_HOST)
    assert e.value.error_code() == E.SPFFT_ALLOCATION_ERROR
    assert sp.inject_allocation_failure(-1) == -1
    assert tr.space_domain_data(sp.SPFFT_PU_HOST) != 0  # allocates now
    _works(tr, idx, dims)


def test_validation_errors(lib):
    """The checks of the reference's transform construction (transform_internal.cpp:52-77), in
    order, each with its code."""
    idx = sphere_indices(32, 8)
    nsticks = len(np.unique((idx[:, 0] % 32) * 32 + idx[:, 1] % 32))
    small = sp.Grid(32, 32, 32, nsticks - 1, sp.SPFFT_PU_GPU, 1)  # one z column too few
    with pytest.raises(sp.SpfftError) as e:
        small.create_transform(sp.SPFFT_PU_GPU, 0, 32, 32, 32, 32, len(idx), 0, idx)
    assert e.value.error_code() == E.SPFFT_INVALID_PARAMETER_ERROR
    grid = sp.Grid(24, 32, 32, 32 * 32, sp.SPFFT_PU_GPU, 1)  # x larger than the grid
    with pytest.raises(sp.SpfftError) as e:
        grid.create_transform(sp.SPFFT_PU_GPU, 0, 32, 32, 32, 32, len(idx), 0, idx)
    assert e.value.error_code() == E.SPFFT_INVALID_PARAMETER_ERROR
    ok = sp.Grid(32, 32, 32, nsticks, sp.SPFFT_PU_GPU, 1)
    with pytest.raises(sp.SpfftError) as e:  # this library executes on the GPU only
        ok.create_transform(sp.SPFFT_PU_HOST, 0, 32, 32, 32, 32, len(idx), 0, idx)
    assert e.value.error_code() == E.SPFFT_INVALID_PARAMETER_ERROR
    bad = idx.copy()
    bad[0] = (40, 0, 0)
    with pytest.raises(sp.SpfftError) as e:
        ok.create_transform(sp.SPFFT_PU_GPU, 0, 32, 32, 32, 32, len(bad), 0, bad)
    assert e.value.error_code() == E.SPFFT_INVALID_INDICES_ERROR
    tr = ok.create_transform(sp.SPFFT_PU_GPU, 0, 32, 32, 32, 32, len(idx), 0, idx)
    _works(tr, idx, (32, 32, 32))
