"""CPU tests of the library's host planner against the reference's own planner output (golden
fixtures) -- bit-exact -- and of the C interface's error codes on paths that need no GPU."""
import ctypes

import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import ref
from util import load_npz_group, random_indices


def test_planner_matches_reference_test_cases(lib):
    for key, c in load_npz_group("ref_cases.npz").items():
        t = sp.SPFFT_TRANS_R2C if key.startswith("r2c") else sp.SPFFT_TRANS_C2C
        _, _, dx, dy, dz = key.split("_")
        vi, sk, zz = sp.plan_indices(t, int(dx), int(dy), int(dz), c["indices"])
        np.testing.assert_array_equal(vi, c["value_indices"], err_msg=key)
        np.testing.assert_array_equal(sk, c["stick_keys"], err_msg=key)
        assert zz == int(c["zz"][0]), key


def test_planner_edge_cases_and_error_codes(lib):
    for name, c in load_npz_group("ref_edges.npz").items():
        t, dx, dy, dz = map(int, c["args"])
        if "error" in c:
            with pytest.raises(sp.SpfftError) as e:
                sp.plan_indices(t, dx, dy, dz, c["indices"])
            assert e.value.error_code() == int(c["error"][0]), name
        else:
            vi, sk, zz = sp.plan_indices(t, dx, dy, dz, c["indices"])
            np.testing.assert_array_equal(vi, c["value_indices"], err_msg=name)
            np.testing.assert_array_equal(sk, c["stick_keys"], err_msg=name)
            assert zz == int(c["zz"][0]), name


def test_planner_matches_oracle_on_large_sets(lib):
    from oracle import indices as ix

    rng = np.random.default_rng(11)
    for t, dims in [(0, (64, 64, 64)), (1, (96, 90, 80)), (0, (100, 2, 13)), (1, (1, 100, 11))]:
        idx = random_indices(rng, *dims, r2c=(t == 1), centered=(dims[0] % 2 == 0))
        vi, sk, zz = sp.plan_indices(t, *dims, idx)
        p = ix.convert(t, *dims, idx)
        np.testing.assert_array_equal(vi, p["value_indices"])
        np.testing.assert_array_equal(sk, p["stick_keys"])
        assert zz == p["zero_zero_stick"]


def test_shuffled_value_order_keeps_mapping(lib):
    rng = np.random.default_rng(5)
    idx = random_indices(rng, 12, 11, 13, r2c=False)
    perm = rng.permutation(idx.shape[0])
    vi, sk, _ = sp.plan_indices(0, 12, 11, 13, idx)
    vi2, sk2, _ = sp.plan_indices(0, 12, 11, 13, idx[perm])
    np.testing.assert_array_equal(sk, sk2)
    np.testing.assert_array_equal(vi[perm], vi2)


def test_null_handles_and_bad_arguments(lib):
    E = sp.ErrorCode
    v = ctypes.c_int(0)
    assert lib.spfft_transform_dim_x(None, ctypes.byref(v)) == E.SPFFT_INVALID_HANDLE_ERROR
    assert lib.spfft_transform_destroy(None) == E.SPFFT_INVALID_HANDLE_ERROR
    assert lib.spfft_grid_destroy(None) == E.SPFFT_INVALID_HANDLE_ERROR
    assert lib.spfft_float_grid_max_dim_x(None, ctypes.byref(v)) == E.SPFFT_INVALID_HANDLE_ERROR
    assert lib.spfft_transform_backward(None, None, 2) == E.SPFFT_INVALID_HANDLE_ERROR
    h = ctypes.c_void_p()
    # negative sizes are rejected before any device work (transform.cpp:74-77)
    assert lib.spfft_transform_create_independent(ctypes.byref(h), 1, 2, 0, -1, 4, 4, 0, 0, None) == \
        E.SPFFT_INVALID_PARAMETER_ERROR
    # indices missing while elements are announced
    assert lib.spfft_transform_create_independent(ctypes.byref(h), 1, 2, 0, 4, 4, 4, 3, 0, None) == \
        E.SPFFT_INVALID_PARAMETER_ERROR
    # invalid indices are reported as such, before device allocation
    bad = (ctypes.c_int * 3)(9, 0, 0)
    assert lib.spfft_transform_create_independent(ctypes.byref(h), 1, 2, 0, 4, 4, 4, 1, 0, bad) == \
        E.SPFFT_INVALID_INDICES_ERROR
    # grid limits are validated first (grid_internal.cpp:61-67)
    assert lib.spfft_grid_create(ctypes.byref(h), 0, 4, 4, 1, 2, 1) == E.SPFFT_INVALID_PARAMETER_ERROR
    assert lib.spfft_grid_create(ctypes.byref(h), 4, 4, 4, 1, 4, 1) == E.SPFFT_INVALID_PARAMETER_ERROR


def test_plan_tables_are_consistent(lib):
    """The derived tables of the host planner (the ones the device planner must reproduce) agree
    with the reference-compatible value indices and stick keys."""
    rng = np.random.default_rng(8)
    for t, dims, centered in [(0, (12, 11, 13), False), (1, (16, 12, 10), True), (0, (20, 3, 7), True)]:
        idx = random_indices(rng, *dims, r2c=(t == 1), centered=centered)
        idx = np.ascontiguousarray(idx[rng.permutation(idx.shape[0])])
        tb = sp.plan_tables(0, t, *dims, idx)
        vi, sk, zz = sp.plan_indices(t, *dims, idx)
        assert tb["used_device"] == 0
        np.testing.assert_array_equal(tb["value_indices"], vi)
        np.testing.assert_array_equal(tb["stick_keys"], sk)
        assert tb["zero_zero_stick"] == zz and tb["num_sticks"] == len(sk)
        dy, dz = dims[1], dims[2]
        np.testing.assert_array_equal(tb["column_x"][tb["stick_column"]] * dy + tb["stick_y"], sk)
        np.testing.assert_array_equal(tb["stick_plane_pos"], tb["stick_y"] * tb["num_columns"] + tb["stick_column"])
        starts = tb["column_stick_start"]
        assert starts[0] == 0 and starts[-1] == len(sk) and np.all(np.diff(starts) > 0)
        assert np.all(np.diff(tb["entry_pos"]) > 0)
        np.testing.assert_array_equal(np.sort(tb["entry_user"]), np.arange(len(vi)))
        np.testing.assert_array_equal(vi[tb["entry_user"]], tb["entry_pos"])
        np.testing.assert_array_equal(
            tb["stick_entry_start"], np.searchsorted(tb["entry_pos"], np.arange(len(sk) + 1) * dz))
        assert len(tb["hermitian_weight"]) == (len(vi) if t == 1 else 0)
    assert sp.plan_cache_size() >= 0


def test_allocation_failure_hook_countdown(lib):
    """The fault-injection countdown arms and disarms without a GPU (nothing allocates here)."""
    assert sp.inject_allocation_failure(5) == -1
    assert sp.inject_allocation_failure(2) == 5
    assert sp.inject_allocation_failure(-1) == 2
    with pytest.raises(sp.SpfftError):
        sp.inject_allocation_failure(-2)


@pytest.mark.skipif(not ref.available(), reason="reference index code not built here")
def test_library_planner_matches_reference_planner_on_random_sets(lib):
    """The library's planner against the reference's own (spfft::Parameters, compiled from its
    sources into oracle/_ref) on random index sets: plain and centered, C2C and R2C, shuffled, with
    duplicated triplets and with out-of-range indices -- bit-exact, or the same error code."""
    rng = np.random.default_rng(29)
    checked = errors = 0
    for trial in range(160):
        t = trial % 2
        dx, dy, dz = (int(v) for v in rng.integers(1, 24, 3))
        idx = random_indices(rng, dx, dy, dz, t == 1, 0.5, 0.5, centered=bool((trial // 2) % 2))
        if len(idx) and trial % 5 == 0:
            idx = np.concatenate([idx, idx[rng.integers(0, len(idx), 3)]])
        if len(idx) and trial % 7 == 0:
            idx = idx.copy()
            idx[int(rng.integers(0, len(idx))), int(rng.integers(0, 3))] = int(rng.choice([dx, -dx, dy + 5]))
        idx = np.ascontiguousarray(idx[rng.permutation(len(idx))].astype(np.int32))
        r = ref.plan(t, dx, dy, dz, idx)
        if "error" in r:
            with pytest.raises(sp.SpfftError) as e:
                sp.plan_indices(t, dx, dy, dz, idx)
            assert e.value.error_code() == r["error"], (trial, dx, dy, dz)
            errors += 1
            continue
        vi, sk, zz = sp.plan_indices(t, dx, dy, dz, idx)
        np.testing.assert_array_equal(vi, r["value_indices"], err_msg=str(trial))
        np.testing.assert_array_equal(sk, r["stick_keys"], err_msg=str(trial))
        assert zz == r["zero_zero_stick"], trial
        checked += 1
    assert checked > 100 and errors > 5, (checked, errors)
