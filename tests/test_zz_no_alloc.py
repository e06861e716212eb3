"""GPU test of the allocation-free backward entry point (spfft_gb300_transform_backward_noalloc).

That entry point serves callers that cannot let the library call cudaMalloc: applications whose
device memory belongs to their own pool or arena allocator, latency-critical loops that cannot
afford an allocation's device synchronisation, plug-ins whose host application forbids them to
allocate. It keeps the transform's intermediates in a static 64 MiB device array. This test calls
it through the C ABI twice in a row, with different inputs, and compares each result with the
regular backward entry point (spfft_transform_backward_ptr) at the FP64 tolerance of the parity
suite; it also checks that sizes above the limit, a null handle and buffers that are not device
memory of the transform's GPU are rejected before any kernel runs.
It lives in its own file, collected last, and passes both alone and after the other tests.
"""
import ctypes

import numpy as np
import pytest

import spfft_gb300 as sp
from util import random_indices, rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)


def _noalloc(lib):
    fn = lib.spfft_gb300_transform_backward_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("case", ["c2c_64_sphere16", "r2c_24_20_18", "c2c_12_11_13"])
def test_noalloc_backward_matches_regular_backward(lib, case):
    rng = np.random.default_rng(42)
    if case == "c2c_64_sphere16":
        ttype, dims, idx = sp.SPFFT_TRANS_C2C, (64, 64, 64), sphere_indices(64, 16)
    elif case == "r2c_24_20_18":
        ttype, dims = sp.SPFFT_TRANS_R2C, (24, 20, 18)
        idx = random_indices(rng, *dims, r2c=True, stick_frac=0.8, fill_frac=0.8, centered=True)
    else:
        ttype, dims = sp.SPFFT_TRANS_C2C, (12, 11, 13)
        idx = random_indices(rng, *dims, r2c=False)
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, *dims, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx)
    fn = _noalloc(lib)
    shape = dims[::-1]
    st = torch.complex128 if ttype == sp.SPFFT_TRANS_C2C else torch.float64
    for call in range(2):  # two calls in a row share (and reuse) the static array
        vals = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
        v = torch.from_numpy(vals).cuda()
        want = torch.empty(shape, dtype=st, device="cuda")
        tr.backward(v, want)  # regular entry point
        got = torch.full(shape, float("nan"), dtype=st, device="cuda")
        torch.cuda.synchronize()
        assert fn(tr.handle, v.data_ptr(), got.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) <= 1e-12, (case, call)


def test_noalloc_rejects_intermediates_above_the_limit(lib):
    # 160^3 C2C with |k| <= 78: sticks (46.7 MiB) plus compact planes (61.3 MiB) exceed 64 MiB.
    idx = sphere_indices(160, 78)
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, sp.SPFFT_TRANS_C2C, 160, 160, 160, len(idx),
                      sp.SPFFT_INDEX_TRIPLETS, idx)
    v = torch.zeros(len(idx), dtype=torch.complex128, device="cuda")
    out = torch.empty((160, 160, 160), dtype=torch.complex128, device="cuda")
    fn = _noalloc(lib)
    assert fn(tr.handle, v.data_ptr(), out.data_ptr(), None) == sp.ErrorCode.SPFFT_INVALID_PARAMETER_ERROR
    assert fn(None, v.data_ptr(), out.data_ptr(), None) == sp.ErrorCode.SPFFT_INVALID_HANDLE_ERROR


def test_noalloc_rejects_buffers_that_are_not_device_memory(lib):
    # The kernels must never be handed a host address: a pageable numpy buffer, a pinned host
    # buffer and a null space pointer are refused with SPFFT_INVALID_PARAMETER_ERROR, and a
    # regular call afterwards still works (nothing was launched and no error is left pending).
    idx = sphere_indices(32, 8)
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, sp.SPFFT_TRANS_C2C, 32, 32, 32, len(idx),
                      sp.SPFFT_INDEX_TRIPLETS, idx)
    rng = np.random.default_rng(7)
    vals = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
    v = torch.from_numpy(vals).cuda()
    out = torch.empty((32, 32, 32), dtype=torch.complex128, device="cuda")
    host_vals = np.ascontiguousarray(vals)
    host_space = np.zeros((32, 32, 32), dtype=np.complex128)
    pinned_space = torch.zeros((32, 32, 32), dtype=torch.complex128).pin_memory()
    fn = _noalloc(lib)
    bad = sp.ErrorCode.SPFFT_INVALID_PARAMETER_ERROR
    torch.cuda.synchronize()
    assert fn(tr.handle, host_vals.ctypes.data, out.data_ptr(), None) == bad
    assert fn(tr.handle, v.data_ptr(), host_space.ctypes.data, None) == bad
    assert fn(tr.handle, v.data_ptr(), pinned_space.data_ptr(), None) == bad
    assert fn(tr.handle, v.data_ptr(), None, None) == bad
    assert not host_space.any() and not pinned_space.any()
    assert fn(tr.handle, v.data_ptr(), out.data_ptr(), None) == 0
    want = torch.empty_like(out)
    tr.backward(v, want)
    torch.cuda.synchronize()
    assert rel_l2(out.cpu().numpy(), want.cpu().numpy()) <= 1e-12
