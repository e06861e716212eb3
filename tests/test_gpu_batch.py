"""GPU tests of batched execution (spfft_gb300_batch_*): mixed shapes, C2C and R2C, both
precisions, a shape without specialised kernels (run one by one inside the batch), and graph
replay with new data in the bound buffers. Each result is compared with the oracle."""
import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import pipeline
from util import random_indices, rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

TOL = {"float64": 1e-12, "float32": 1e-5}


def _make(dtype, specs, rng):
    ct = torch.complex128 if dtype == "float64" else torch.complex64
    rt = torch.float64 if dtype == "float64" else torch.float32
    items = []
    for (n, radius, ttype) in specs:
        if isinstance(n, tuple):
            dims = n
            idx = random_indices(rng, *dims, r2c=(ttype == 1), stick_frac=0.6, fill_frac=0.6)
        else:
            dims = (n, n, n)
            idx = sphere_indices(n, radius, r2c=(ttype == 1))
        tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, *dims, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
        vals = torch.zeros(len(idx), dtype=ct, device="cuda")
        space = torch.zeros(dims[::-1], dtype=ct if ttype == 0 else rt, device="cuda")
        items.append(dict(tr=tr, idx=idx, dims=dims, ttype=ttype, vals=vals, space=space,
                          oracle=pipeline.HostPipeline(ttype, *dims, idx)))
    return items


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batch_mixed_shapes_against_oracle(lib, dtype):
    rng = np.random.default_rng(3)
    specs = [(48, 12, 0), (48, 14, 0), (60, 15, 1), (64, 16, 1), (48, 10, 1), ((13, 12, 11), 0, 0),
             (64, 20, 0), (60, 12, 1)]
    items = _make(dtype, specs, rng)
    batch = sp.Batch([it["tr"] for it in items])
    info = batch.info()
    assert info["unbatched"] == 1 and info["groups"] >= 4, info
    batch.bind([it["vals"] for it in items], [it["space"] for it in items])
    stream = torch.cuda.Stream()
    for rep in range(2):  # second round reuses the captured graph with new data
        host_vals = []
        for it in items:
            v = rng.uniform(-1, 1, len(it["idx"])) + 1j * rng.uniform(-1, 1, len(it["idx"]))
            host_vals.append(v)
            it["vals"].copy_(torch.from_numpy(v).to(it["vals"].dtype))
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            batch.backward(stream)
        stream.synchronize()
        for it, v in zip(items, host_vals):
            want = it["oracle"].backward(v)
            assert rel_l2(it["space"].cpu().numpy(), want) <= TOL[dtype], (it["dims"], rep)
        with torch.cuda.stream(stream):
            batch.forward(sp.SPFFT_FULL_SCALING, stream)
        stream.synchronize()
        for it in items:
            want = it["oracle"].forward(it["space"].cpu().numpy().astype(
                np.complex128 if it["ttype"] == 0 else np.float64), scaled=True)
            assert rel_l2(it["vals"].cpu().numpy(), want) <= TOL[dtype], (it["dims"], rep)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batch_pair_graph_replay(lib, dtype):
    rng = np.random.default_rng(4)
    items = _make(dtype, [(64, 16, 0)] * 3 + [(48, 12, 1)] * 3, rng)
    batch = sp.Batch([it["tr"] for it in items])
    batch.bind([it["vals"] for it in items], [it["space"] for it in items])
    stream = torch.cuda.Stream()
    for rep in range(3):
        host_vals = []
        for it in items:
            v = rng.uniform(-1, 1, len(it["idx"])) + 1j * rng.uniform(-1, 1, len(it["idx"]))
            if it["ttype"] == 1:
                v[(it["idx"] == 0).all(axis=1)] = v[(it["idx"] == 0).all(axis=1)].real
            host_vals.append(v)
            it["vals"].copy_(torch.from_numpy(v).to(it["vals"].dtype))
        torch.cuda.synchronize()
        batch.pair_graph(sp.SPFFT_FULL_SCALING, stream)
        stream.synchronize()
        for it, v in zip(items, host_vals):
            o = it["oracle"]
            want = o.forward(o.backward(v), scaled=True)
            assert rel_l2(it["vals"].cpu().numpy(), want) <= 10 * TOL[dtype], (it["dims"], rep)
    with pytest.raises(sp.SpfftError):
        batch.pair_graph(sp.SPFFT_NO_SCALING, None)  # the default stream cannot be captured


def test_batch_rejects_shared_grids_and_mixed_precision(lib):
    grid = sp.Grid(32, 32, 32, 32 * 32, sp.SPFFT_PU_GPU, 1)
    idx = sphere_indices(32, 8)
    t1 = grid.create_transform(sp.SPFFT_PU_GPU, 0, 32, 32, 32, 32, len(idx), 0, idx)
    t2 = grid.create_transform(sp.SPFFT_PU_GPU, 0, 32, 32, 32, 32, len(idx), 0, idx)
    with pytest.raises(sp.SpfftError):
        sp.Batch([t1, t2])
    tf = sp.Transform(1, sp.SPFFT_PU_GPU, 0, 32, 32, 32, len(idx), 0, idx, dtype="float32")
    with pytest.raises(ValueError):
        sp.Batch([t1, tf])


@pytest.mark.parametrize("mode", ["split", "fused"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batch_plane_pass_modes(lib, dtype, mode, monkeypatch):
    """Both plane-pass forms of the batched kernels (split y and x passes with the compact planes
    in HBM; one fused kernel per plane), forced at batch creation, against the oracle, with the
    192^3 R2C shape of the benchmark among them."""
    monkeypatch.setenv("SPFFT_GB300_BATCH_PLANE", mode)
    rng = np.random.default_rng(5)
    specs = [(64, 16, 0), (64, 20, 0), (60, 15, 1), (192, 48, 1), ((13, 12, 11), 0, 0)]
    if dtype == "float64" and mode == "fused":
        specs = specs[:3] + specs[4:]  # the 192^3 compact plane in double-float exceeds one block
    items = _make(dtype, specs, rng)
    batch = sp.Batch([it["tr"] for it in items])
    want_path = 2 if mode == "fused" else 1
    assert [batch.transform_path(i) for i in range(len(items) - 1)] == [want_path] * (len(items) - 1)
    assert batch.transform_path(len(items) - 1) == 0
    batch.bind([it["vals"] for it in items], [it["space"] for it in items])
    host_vals = []
    for it in items:
        v = rng.uniform(-1, 1, len(it["idx"])) + 1j * rng.uniform(-1, 1, len(it["idx"]))
        if it["ttype"] == 1:
            v[(it["idx"] == 0).all(axis=1)] = v[(it["idx"] == 0).all(axis=1)].real
        host_vals.append(v)
        it["vals"].copy_(torch.from_numpy(v).to(it["vals"].dtype))
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    batch.backward(stream)
    stream.synchronize()
    for it, v in zip(items, host_vals):
        assert rel_l2(it["space"].cpu().numpy(), it["oracle"].backward(v)) <= TOL[dtype], it["dims"]
    batch.forward(sp.SPFFT_NO_SCALING, stream)
    stream.synchronize()
    for it in items:
        want = it["oracle"].forward(it["space"].cpu().numpy().astype(
            np.complex128 if it["ttype"] == 0 else np.float64))
        assert rel_l2(it["vals"].cpu().numpy(), want) <= TOL[dtype], it["dims"]
    ms_b = batch.stage_times(0, sp.SPFFT_NO_SCALING, stream)
    assert len(ms_b) == 3 and all(t >= 0 for t in ms_b)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batch_row_groups_give_identical_results(lib, dtype, monkeypatch):
    """The fused plane passes with the x pass split into independent row groups compute exactly
    what one group computes (same arithmetic per element), for every valid group count."""
    monkeypatch.setenv("SPFFT_GB300_BATCH_PLANE", "fused")
    specs = [(64, 16, 0), (60, 15, 1), (48, 12, 1), (64, 20, 0)]
    if dtype == "float32":
        specs.append((192, 48, 1))
    results = {}
    for groups in (1, 2, 3, 4):
        monkeypatch.setenv("SPFFT_GB300_BATCH_ROW_GROUPS", str(groups))
        rng = np.random.default_rng(7)
        items = _make(dtype, specs, rng)
        batch = sp.Batch([it["tr"] for it in items])
        got = batch.row_groups(0)
        if groups == 3 and dtype == "float64":
            assert got == 1  # 256 threads do not split into three groups of whole warps
            continue
        assert got == groups
        batch.bind([it["vals"] for it in items], [it["space"] for it in items])
        host_vals = []
        for it in items:
            v = rng.uniform(-1, 1, len(it["idx"])) + 1j * rng.uniform(-1, 1, len(it["idx"]))
            if it["ttype"] == 1:
                v[(it["idx"] == 0).all(axis=1)] = v[(it["idx"] == 0).all(axis=1)].real
            host_vals.append(v)
            it["vals"].copy_(torch.from_numpy(v).to(it["vals"].dtype))
        stream = torch.cuda.Stream()
        torch.cuda.synchronize()
        batch.backward(stream)
        stream.synchronize()
        spaces = [it["space"].cpu().numpy().copy() for it in items]
        for it, v, sp_ in zip(items, host_vals, spaces):
            assert rel_l2(sp_, it["oracle"].backward(v)) <= TOL[dtype], it["dims"]
        batch.forward(sp.SPFFT_NO_SCALING, stream)
        stream.synchronize()
        vals = [it["vals"].cpu().numpy().copy() for it in items]
        for it, sp_, got_v in zip(items, spaces, vals):
            want = it["oracle"].forward(sp_.astype(np.complex128 if it["ttype"] == 0 else np.float64))
            assert rel_l2(got_v, want) <= TOL[dtype], it["dims"]
        results[groups] = (spaces, vals)
    for groups, (spaces, vals) in results.items():
        for a, b in zip(spaces, results[1][0]):
            np.testing.assert_array_equal(a, b)
        for a, b in zip(vals, results[1][1]):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batch_autotune_then_graph(lib, dtype):
    """Autotuning a bound batch (per group: plane strategy and z block size), then a captured pair
    with new data against the oracle."""
    rng = np.random.default_rng(6)
    items = _make(dtype, [(64, 16, 0), (64, 16, 0), (60, 15, 1), (48, 12, 1), ((13, 12, 11), 0, 0)], rng)
    batch = sp.Batch([it["tr"] for it in items])
    batch.bind([it["vals"] for it in items], [it["space"] for it in items])
    stream = torch.cuda.Stream()
    batch.pair_graph(sp.SPFFT_FULL_SCALING, stream)  # a graph captured before tuning is dropped
    stream.synchronize()
    assert batch.autotune(2, stream) > 0
    host_vals = []
    for it in items:
        v = rng.uniform(-1, 1, len(it["idx"])) + 1j * rng.uniform(-1, 1, len(it["idx"]))
        if it["ttype"] == 1:
            v[(it["idx"] == 0).all(axis=1)] = v[(it["idx"] == 0).all(axis=1)].real
        host_vals.append(v)
        it["vals"].copy_(torch.from_numpy(v).to(it["vals"].dtype))
    torch.cuda.synchronize()
    batch.pair_graph(sp.SPFFT_FULL_SCALING, stream)
    stream.synchronize()
    for it, v in zip(items, host_vals):
        o = it["oracle"]
        assert rel_l2(it["vals"].cpu().numpy(), o.forward(o.backward(v), scaled=True)) <= 10 * TOL[dtype], it["dims"]
