"""CPU checks of the oracle itself, against the reference's own outputs (golden fixtures generated
by the reference's index code) and the dense DFT definition."""
import numpy as np
import pytest

from oracle import dense, indices as ix, pipeline, ref
from util import load_npz_group, rel_l2


def test_oracle_indices_match_reference_test_cases():
    cases = load_npz_group("ref_cases.npz")
    assert len(cases) > 250
    for key, c in cases.items():
        t = 1 if key.startswith("r2c") else 0
        _, _, dx, dy, dz = key.split("_")
        p = ix.convert(t, int(dx), int(dy), int(dz), c["indices"].astype(np.int64))
        np.testing.assert_array_equal(p["value_indices"], c["value_indices"], err_msg=key)
        np.testing.assert_array_equal(p["stick_keys"], c["stick_keys"], err_msg=key)
        assert p["zero_zero_stick"] == int(c["zz"][0]), key


def test_oracle_indices_edge_cases():
    for name, c in load_npz_group("ref_edges.npz").items():
        t, dx, dy, dz = map(int, c["args"])
        if "error" in c:
            with pytest.raises(ix.IndexError_) as e:
                ix.convert(t, dx, dy, dz, c["indices"])
            assert e.value.code == int(c["error"][0]), name
        else:
            p = ix.convert(t, dx, dy, dz, c["indices"])
            np.testing.assert_array_equal(p["value_indices"], c["value_indices"], err_msg=name)
            np.testing.assert_array_equal(p["stick_keys"], c["stick_keys"], err_msg=name)
            assert p["zero_zero_stick"] == int(c["zz"][0]), name


def test_oracle_pipeline_matches_dense_golden():
    for name, c in load_npz_group("dense_small.npz").items():
        t, dx, dy, dz = map(int, c["args"])
        p = pipeline.HostPipeline(t, dx, dy, dz, c["indices"])
        assert rel_l2(p.backward(c["values"]), c["space"]) < 1e-13, name
        assert rel_l2(p.forward(c["forward_in"]), c["forward_out"]) < 1e-13, name
        # the dense oracle reproduces its own golden numbers
        assert rel_l2(dense.backward(t, dx, dy, dz, c["indices"], c["values"]), c["space"]) < 1e-13


@pytest.mark.parametrize("t", [0, 1])
def test_oracle_pipeline_matches_dense_on_reference_cases(t):
    rng = np.random.default_rng(7)
    cases = load_npz_group("ref_cases.npz")
    for key, c in cases.items():
        if (t == 1) != key.startswith("r2c"):
            continue
        _, _, dx, dy, dz = map(lambda s: int(s) if s.isdigit() else s, key.split("_"))
        idx = c["indices"].astype(np.int64)
        p = pipeline.HostPipeline(t, dx, dy, dz, idx)
        n = dx * dy * dz
        if t == 0:
            vals = rng.uniform(-1, 1, idx.size // 3) + 1j * rng.uniform(-1, 1, idx.size // 3)
            d = dense.backward(t, dx, dy, dz, idx, vals)
            np.testing.assert_allclose(p.backward(vals), d, atol=1e-9, err_msg=key)
            np.testing.assert_allclose(p.forward(d), dense.forward(t, dx, dy, dz, idx, d), atol=1e-8,
                                       err_msg=key)
        else:
            f = rng.uniform(-1, 1, (dz, dy, dx))
            vals = dense.forward(t, dx, dy, dz, idx, f)
            np.testing.assert_allclose(p.forward(f), vals, atol=1e-9, err_msg=key)
            np.testing.assert_allclose(p.backward(vals), f * n, atol=1e-8, err_msg=key)


@pytest.mark.skipif(not ref.available(), reason="reference sources not present (built by oracle/Makefile)")
@pytest.mark.skipif(not ref.available(), reason="reference index code not built here")
def test_oracle_indices_match_reference_binary_random():
    rng = np.random.default_rng(3)
    for trial in range(40):
        t = int(rng.integers(0, 2))
        dx, dy, dz = (int(v) for v in rng.integers(1, 20, 3))
        from util import random_indices
        idx = random_indices(rng, dx, dy, dz, t == 1, 0.5, 0.5, centered=bool(trial % 2))
        r = ref.plan(t, dx, dy, dz, idx)
        p = ix.convert(t, dx, dy, dz, idx)
        np.testing.assert_array_equal(p["value_indices"], r["value_indices"])
        np.testing.assert_array_equal(p["stick_keys"], r["stick_keys"])
        assert p["zero_zero_stick"] == r["zero_zero_stick"]


def test_oracle_pipeline_matches_reference_pipeline_golden():
    """The oracle against the reference's OWN host transform path (golden vectors it produced on
    the inputs of its local test suite; tests/golden/make_golden.py)."""
    cases = load_npz_group("ref_pipeline.npz")
    assert len(cases) >= 28
    for name, c in cases.items():
        t, dx, dy, dz = map(int, c["args"])
        p = pipeline.HostPipeline(t, dx, dy, dz, c["indices"].astype(np.int64))
        if t == 0:
            assert rel_l2(p.backward(c["values_in"]), c["space_out"]) < 1e-13, name
            assert rel_l2(p.forward(c["space_out"]), c["values_out"]) < 1e-13, name
        else:
            assert rel_l2(p.forward(c["space_in"]), c["values_out"]) < 1e-13, name
            assert rel_l2(p.backward(c["values_out"]), c["space_out"]) < 1e-13, name


@pytest.mark.skipif(not ref.pipeline_available(), reason="reference pipeline not built here")
@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_oracle_pipeline_matches_live_reference_pipeline(precision):
    """Where the reference's host path is built (oracle/_ref), the oracle against it live: the whole
    local suite of index sets, C2C and R2C, plain and centered, larger sphere sets, non-hermitian
    R2C values, and scaled forwards."""
    from util import sphere_indices

    tol = 1e-13 if precision == "float64" else 2e-6
    rng = np.random.default_rng(17)
    cases = [(1 if k.startswith("r2c") else 0, tuple(int(v) for v in k.split("_")[2:]),
              c["indices"].astype(np.int64)) for k, c in load_npz_group("ref_cases.npz").items()]
    cases += [(0, (64, 64, 64), sphere_indices(64, 16)), (1, (48, 48, 48), sphere_indices(48, 12, True)),
              (1, (30, 20, 18), sphere_indices(18, 6, True)), (0, (45, 50, 27), sphere_indices(27, 9))]
    for k, (t, dims, idx) in enumerate(cases):
        if idx.size == 0:
            continue
        n = idx.size // 3
        vals = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)  # non-hermitian for R2C too
        scaling = k % 2
        space, fwd = ref.pipeline_run(t, *dims, idx, values=vals, precision=precision, scaling=scaling)
        p = pipeline.HostPipeline(t, *dims, idx.reshape(-1, 3))
        want = p.backward(vals)
        assert rel_l2(space, want) < tol, (dims, t)
        want_f = p.forward(space.astype(np.complex128 if t == 0 else np.float64), scaled=bool(scaling))
        assert rel_l2(fwd, want_f) < tol, (dims, t)
