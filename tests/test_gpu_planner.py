"""Device index planner and shared plans, on the GPU.

The device planner must give every table of the host planner bit for bit (the host planner is
pinned to the reference's own planner by the golden fixtures, tests/test_planner.py), raise the same
errors for the same invalid sets, and hand duplicate triplets back to the host planner. Transforms
planned on the device must give the same results as transforms planned on the host, and transforms
created with the same index set share one plan.
"""
from __future__ import annotations

import numpy as np
import pytest

import spfft_gb300 as sp
from util import load_npz_group, random_indices, rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)


def _same_tables(t, dims, idx, expect_device=True):
    host = sp.plan_tables(0, t, *dims, idx)
    dev = sp.plan_tables(1, t, *dims, idx)
    assert dev["used_device"] == (1 if expect_device else 0)
    for k in ("num_sticks", "num_columns", "zero_zero_stick", "identity_order"):
        assert dev[k] == host[k], (k, dims)
    for k in sp.PLAN_TABLE_FIELDS:
        np.testing.assert_array_equal(dev[k], host[k], err_msg=f"{k} {dims}")
    return dev


def test_device_planner_matches_reference_cases(lib):
    for key, c in load_npz_group("ref_cases.npz").items():
        t = sp.SPFFT_TRANS_R2C if key.startswith("r2c") else sp.SPFFT_TRANS_C2C
        _, _, dx, dy, dz = key.split("_")
        idx = c["indices"].astype(np.int32).reshape(-1, 3)
        if idx.shape[0] == 0:
            continue
        dev = _same_tables(t, (int(dx), int(dy), int(dz)), idx)
        np.testing.assert_array_equal(dev["value_indices"], c["value_indices"], err_msg=key)
        np.testing.assert_array_equal(dev["stick_keys"], c["stick_keys"], err_msg=key)
        assert dev["zero_zero_stick"] == int(c["zz"][0]), key


def test_device_planner_random_and_benchmark_sets(lib):
    rng = np.random.default_rng(21)
    cases = []
    for t, dims, centered in [(0, (64, 64, 64), True), (1, (96, 90, 80), False), (0, (100, 2, 13), False),
                              (1, (1, 100, 11), False), (0, (17, 31, 5), True), (1, (128, 128, 128), True)]:
        cases.append((t, dims, random_indices(rng, *dims, r2c=(t == 1), centered=centered)))
    cases.append((1, (192, 192, 192), sphere_indices(192, 48, True)))   # the headline set
    cases.append((0, (128, 128, 128), sphere_indices(128, 40, False)))
    cases.append((0, (64, 64, 64), sphere_indices(64, 16, False)))
    for t, dims, idx in cases:
        _same_tables(t, dims, idx)
        perm = rng.permutation(idx.shape[0])
        shuffled = _same_tables(t, dims, np.ascontiguousarray(idx[perm]))
        assert shuffled["identity_order"] == 0 or idx.shape[0] < 2


def test_device_planner_errors_and_fallbacks(lib):
    E = sp.ErrorCode
    rng = np.random.default_rng(4)
    plain = random_indices(rng, 64, 64, 64, r2c=False)          # no negative index
    centered = sphere_indices(64, 20, False)                     # negatives: centered ranges
    half = sphere_indices(64, 20, True)
    bad_cases = [
        (0, plain, [64, 0, 0]),        # x beyond the plain range [0, 63]
        (0, centered, [33, 0, 0]),     # beyond the centered range [-31, 32]
        (0, centered, [0, 0, -32]),
        (1, half, [33, 0, 0]),         # R2C x beyond dimX / 2
        (1, half, [-1, 0, 0]),         # R2C x is never negative
    ]
    for t, base, extra in bad_cases:
        idx = np.ascontiguousarray(np.concatenate([base, np.asarray([extra], dtype=np.int32)]))
        codes = []
        for planner in (0, 1):
            with pytest.raises(sp.SpfftError) as e:
                sp.plan_tables(planner, t, 64, 64, 64, idx)
            codes.append(e.value.error_code())
        assert codes[0] == codes[1] == E.SPFFT_INVALID_INDICES_ERROR, (extra, codes)
    # x = 40 is valid while no index is negative
    ok = np.ascontiguousarray(np.concatenate([plain, np.asarray([[40, 0, 0]], dtype=np.int32)]))
    ok = np.unique(ok, axis=0)
    _same_tables(0, (64, 64, 64), ok)
    # duplicate triplets: the host planner keeps user order; the device planner declines
    rng = np.random.default_rng(3)
    idx = random_indices(rng, 24, 24, 24, r2c=False)
    dup = np.ascontiguousarray(np.concatenate([idx, idx[::7]]))
    _same_tables(0, (24, 24, 24), dup, expect_device=False)


def _roundtrip(idx, dims, ttype, dtype="float64"):
    rng = np.random.default_rng(9)
    n = idx.shape[0]
    vals = torch.from_numpy(rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).cuda()
    if dtype == "float32":
        vals = vals.to(torch.complex64)
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, *dims, n, sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
    nz, ny, nx = dims[2], dims[1], dims[0]
    space = torch.empty((nz, ny, nx), dtype=(torch.complex128 if ttype == 0 else torch.float64)
                        if dtype == "float64" else (torch.complex64 if ttype == 0 else torch.float32),
                        device="cuda")
    out = torch.empty_like(vals)
    tr.backward(vals, space)
    tr.forward(space, out, sp.SPFFT_FULL_SCALING)
    torch.cuda.synchronize()
    return tr, space.cpu().numpy(), out.cpu().numpy()


def test_transforms_planned_on_device_match_host_planned(lib, monkeypatch):
    rng = np.random.default_rng(17)
    small = sphere_indices(64, 20, False)
    cases = [(1, (192, 192, 192), sphere_indices(192, 48, True)),
             (0, (64, 64, 64), np.ascontiguousarray(small[rng.permutation(small.shape[0])]))]
    monkeypatch.setenv("SPFFT_GB300_PLAN_CACHE", "0")
    for t, dims, idx in cases:
        for dtype in ("float64", "float32"):
            monkeypatch.setenv("SPFFT_GB300_PLANNER", "host")
            _, sh, vh = _roundtrip(idx, dims, t, dtype)
            monkeypatch.setenv("SPFFT_GB300_PLANNER", "device")
            _, sd, vd = _roundtrip(idx, dims, t, dtype)
            # same plan, same kernels: identical bits
            np.testing.assert_array_equal(sd, sh)
            np.testing.assert_array_equal(vd, vh)
            assert rel_l2(vd, vh) == 0.0


def test_transforms_share_plans(lib, monkeypatch):
    monkeypatch.delenv("SPFFT_GB300_PLAN_CACHE", raising=False)
    monkeypatch.delenv("SPFFT_GB300_PLANNER", raising=False)
    idx = sphere_indices(96, 23, False)
    before = sp.plan_cache_size()
    a, sa, va = _roundtrip(idx, (96, 96, 96), 0)
    assert sp.plan_cache_size() == before + 1
    b, sb, vb = _roundtrip(np.ascontiguousarray(idx.copy()), (96, 96, 96), 0)
    assert sp.plan_cache_size() == before + 1       # the second transform reused the plan
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(va, vb)
    other = np.ascontiguousarray(idx[::-1])
    c, _, _ = _roundtrip(other, (96, 96, 96), 0)     # another order is another plan
    assert sp.plan_cache_size() == before + 2
    del a, b, c
    import gc

    gc.collect()
    assert sp.plan_cache_size() == before
