"""GPU tests of the multi-transform functions (reference: src/spfft/multi_transform_internal.hpp:
63-174, tests through include/spfft/multi_transform.h) on their batched execution: mixed shapes
and types in one call, a length without specialised kernels inside the batch, repeated calls with
new buffers and with other transforms, pinned host buffers, asynchronous mode, and the calls that
must run one by one (mixed scalings, pageable host buffers, a user stream, a single transform).
Every result is compared with the oracle."""
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


def _values(rng, idx, r2c):
    v = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
    if r2c:
        k0 = (idx == 0).all(axis=1)
        v[k0] = v[k0].real
    return v


def _items(dtype, specs, rng):
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
        v = _values(rng, idx, ttype == 1)
        items.append(dict(tr=tr, idx=idx, dims=dims, ttype=ttype, host=v,
                          vals=torch.from_numpy(v).to(ct).cuda(),
                          space=torch.zeros(dims[::-1], dtype=ct if ttype == 0 else rt, device="cuda"),
                          out=torch.zeros(len(idx), dtype=ct, device="cuda"),
                          oracle=pipeline.HostPipeline(ttype, *dims, idx)))
    return items


def _check(items, dtype, scaled=False):
    for it in items:
        o = it["oracle"]
        want = o.backward(it["host"])
        assert rel_l2(it["space"].cpu().numpy(), want) <= TOL[dtype], it["dims"]
        assert rel_l2(it["out"].cpu().numpy(), o.forward(want, scaled=scaled)) <= 10 * TOL[dtype], it["dims"]


SPECS = [(48, 12, 0), (48, 14, 0), (60, 15, 1), (64, 16, 0), (60, 13, 1), ((11, 12, 13), 0, 0),
         ((12, 10, 9), 0, 1)]


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_multi_batched_mixed_against_oracle(lib, dtype):
    rng = np.random.default_rng(21)
    items = _items(dtype, SPECS, rng)
    trs = [it["tr"] for it in items]
    before = sp.multi_batched_calls()
    sp.multi_transform_backward(trs, [it["vals"] for it in items], [it["space"] for it in items])
    sp.multi_transform_forward(trs, [it["space"] for it in items], [it["out"] for it in items])
    assert sp.multi_batched_calls() == before + 2
    _check(items, dtype)

    # again with new data in the same buffers (cached plan, replayed graphs), scaled forward
    for it in items:
        it["host"] = _values(rng, it["idx"], it["ttype"] == 1)
        it["vals"].copy_(torch.from_numpy(it["host"]).to(it["vals"].dtype))
    torch.cuda.synchronize()
    sp.multi_transform_backward(trs, [it["vals"] for it in items], [it["space"] for it in items])
    sp.multi_transform_forward(trs, [it["space"] for it in items], [it["out"] for it in items],
                               [sp.SPFFT_FULL_SCALING] * len(items))
    assert sp.multi_batched_calls() == before + 4
    _check(items, dtype, scaled=True)

    # new buffers for the same transforms (rebinding in stream order)
    for it in items:
        it["vals"] = it["vals"].clone()
        it["space"] = torch.zeros_like(it["space"])
        it["out"] = torch.zeros_like(it["out"])
    sp.multi_transform_backward(trs, [it["vals"] for it in items], [it["space"] for it in items])
    sp.multi_transform_forward(trs, [it["space"] for it in items], [it["out"] for it in items])
    _check(items, dtype)

    # a subset (another set of transforms: the cached plan is replaced)
    sub = items[1:4]
    for it in sub:
        it["space"].zero_()
        it["out"].zero_()
    sp.multi_transform_backward([it["tr"] for it in sub], [it["vals"] for it in sub], [it["space"] for it in sub])
    sp.multi_transform_forward([it["tr"] for it in sub], [it["space"] for it in sub], [it["out"] for it in sub])
    _check(sub, dtype)


def test_multi_batched_after_transforms_are_destroyed(lib):
    """A new set of transforms that may reuse the addresses of destroyed ones gets a new plan."""
    rng = np.random.default_rng(22)
    for rep in range(3):
        items = _items("float64", [(48, 10 + rep, 0), (60, 12, 1), (64, 14 + rep, 0)], rng)
        trs = [it["tr"] for it in items]
        sp.multi_transform_backward(trs, [it["vals"] for it in items], [it["space"] for it in items])
        sp.multi_transform_forward(trs, [it["space"] for it in items], [it["out"] for it in items])
        _check(items, "float64")
        del items, trs


def test_multi_pinned_host_and_async(lib):
    rng = np.random.default_rng(23)
    items = _items("float64", [(48, 12, 0), (60, 14, 1), (64, 15, 0)], rng)
    trs = [it["tr"] for it in items]
    hv = [it["vals"].cpu().pin_memory() for it in items]
    hs = [torch.zeros(it["space"].shape, dtype=it["space"].dtype).pin_memory() for it in items]
    ho = [torch.zeros(it["out"].shape, dtype=it["out"].dtype).pin_memory() for it in items]
    before = sp.multi_batched_calls()
    sp.multi_transform_backward(trs, hv, hs)
    sp.multi_transform_forward(trs, hs, ho)
    assert sp.multi_batched_calls() == before + 2  # pinned host memory is device-addressable
    for it, s, o in zip(items, hs, ho):
        want = it["oracle"].backward(it["host"])
        assert rel_l2(s.numpy(), want) <= 1e-12
        assert rel_l2(o.numpy(), it["oracle"].forward(want)) <= 1e-11

    # asynchronous mode: completion is ordered before later work on the default stream
    for t in trs:
        t.set_execution_mode(sp.SPFFT_EXEC_ASYNCHRONOUS)
    for it in items:
        it["space"].zero_()
    torch.cuda.synchronize()
    sp.multi_transform_backward(trs, [it["vals"] for it in items], [it["space"] for it in items])
    for it in items:
        got = it["space"].cpu().numpy()  # a default-stream copy
        assert rel_l2(got, it["oracle"].backward(it["host"])) <= 1e-12


def test_multi_calls_that_run_one_by_one(lib):
    rng = np.random.default_rng(24)
    items = _items("float64", [(48, 12, 0), (60, 14, 1)], rng)
    trs = [it["tr"] for it in items]
    before = sp.multi_batched_calls()
    # mixed scalings
    sp.multi_transform_backward(trs, [it["vals"] for it in items], [it["space"] for it in items])
    sp.multi_transform_forward(trs, [it["space"] for it in items], [it["out"] for it in items],
                               [sp.SPFFT_NO_SCALING, sp.SPFFT_FULL_SCALING])
    assert sp.multi_batched_calls() == before + 1
    o0, o1 = items[0]["oracle"], items[1]["oracle"]
    assert rel_l2(items[0]["out"].cpu().numpy(), o0.forward(o0.backward(items[0]["host"]))) <= 1e-11
    assert rel_l2(items[1]["out"].cpu().numpy(),
                  o1.forward(o1.backward(items[1]["host"]), scaled=True)) <= 1e-11
    # pageable host buffers
    hv = [np.ascontiguousarray(it["host"]) for it in items]
    hs = [np.zeros(it["space"].shape, dtype=np.complex128 if it["ttype"] == 0 else np.float64) for it in items]
    sp.multi_transform_backward(trs, hv, hs)
    assert sp.multi_batched_calls() == before + 1
    for it, s in zip(items, hs):
        assert rel_l2(s, it["oracle"].backward(it["host"])) <= 1e-12
    # a transform with its own stream
    stream = torch.cuda.Stream()
    trs[0].set_stream(stream)
    sp.multi_transform_backward(trs, [it["vals"] for it in items], [it["space"] for it in items])
    torch.cuda.synchronize()
    assert sp.multi_batched_calls() == before + 1
    trs[0].set_stream(None)
    # one transform
    sp.multi_transform_backward(trs[:1], [items[0]["vals"]], [items[0]["space"]])
    assert sp.multi_batched_calls() == before + 1
    for it in items:
        assert rel_l2(it["space"].cpu().numpy(), it["oracle"].backward(it["host"])) <= 1e-12
